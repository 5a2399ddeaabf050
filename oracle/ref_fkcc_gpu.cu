// Device-side harness around pRRTC's own GPU collision checker.
//
// Test infrastructure only (the oracle's second verdict source): compiled by
// oracle/Makefile (`ref_gpu`) from the reference sources where they lie
// (src/planning/utils.cuh and the headers it includes), never copied, into a
// stand-alone sm_103a cubin under oracle/_ref/.  The tests load that cubin
// through the CUDA driver API; no product code links it.
//
// The reference's Environment<float> is built on the device from flat float
// arrays (ref_env_build.cuh).
//
// Each thread checks one configuration with ppln::collision::fkcc<Robot>
// (utils.cuh:326-327), as pRRTC's kernel does per interpolated point
// (pRRTC.cu:441,529): the configuration sits in a volatile array and the
// environment pointer is the global-memory struct.
#include "src/planning/utils.cuh"

using namespace ppln::collision;

#include "ref_env_build.cuh"

// out_free[i] = 1 when configuration i (row-major, `dim` floats) is free
// according to the reference checker.  Threads past n return at once.
template <class Robot>
__device__ void check(const float *q, long long n, int dim, unsigned char *scratch, unsigned char *out_free)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || dim != Robot::dimension) return;
    volatile float cfg[Robot::dimension];
    for (int d = 0; d < Robot::dimension; d++) cfg[d] = q[i * dim + d];
    Environment<float> *env = reinterpret_cast<Environment<float> *>(scratch);
    out_free[i] = fkcc<Robot>(cfg, env, (int)threadIdx.x) ? 1 : 0;
}

#define REF_CHECK_KERNEL(R)                                                                                    \
    extern "C" __global__ void ref_fkcc_gpu_##R(const float *q, long long n, int dim, unsigned char *scratch, \
                                                unsigned char *out_free)                                     \
    {                                                                                                          \
        check<ppln::robots::R>(q, n, dim, scratch, out_free);                                                  \
    }

#ifdef REF_ROBOT_PANDA
REF_CHECK_KERNEL(Panda)
#endif
#ifdef REF_ROBOT_FETCH
REF_CHECK_KERNEL(Fetch)
#endif
#ifdef REF_ROBOT_BAXTER
REF_CHECK_KERNEL(Baxter)
#endif
#ifdef REF_ROBOT_SPHERE
REF_CHECK_KERNEL(Sphere)
#endif
