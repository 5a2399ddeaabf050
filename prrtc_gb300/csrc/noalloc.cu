// prrtc_validate_configs_noalloc: collision checking for callers that must
// not allocate device memory.
//
// Some callers cannot call cudaMalloc: a control loop with a hard deadline
// (cudaMalloc and cudaFree can synchronise the whole device and take
// milliseconds), a process whose device memory is owned by another runtime's
// pool, or firmware-style code given a fixed memory budget up front.  This
// entry point needs no context and allocates nothing.  Its only device
// storage is the file-scope array below (kScratchBytes, reserved on every GPU
// that loads the library until the process exits): the packed obstacles of
// the call and the checker's two work counters.  The caller provides the
// configurations and the verdict buffer in device memory.  The obstacles are
// packed into a file-scope host array and copied from there; to stage a copy
// from pageable memory the driver may first wait for the work already queued
// on the stream.
//
// The array is shared by every call on a device and keeps the last call's
// contents; the counters are cleared at the start of each call.  Two calls
// whose work overlaps on the GPU (different streams, or different host
// threads) race on it: serialise them.  The first call on a device looks up
// the array's device address (cudaGetSymbolAddress) with that device current;
// make that first call before any stream capture.  A call made while its
// stream is being captured returns PRRTC_EINVAL and records nothing.
#include <cstring>
#include <mutex>

#include "context.h"
#include "prrtc_internal.h"

namespace {

// packed obstacle records (PRRTC_MAX_ENV_FLOATS floats) followed by two 64-bit counters
constexpr size_t kEnvBytes = (size_t)PRRTC_MAX_ENV_FLOATS * sizeof(float);
constexpr size_t kScratchBytes = kEnvBytes + 2 * sizeof(unsigned long long);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_ptr[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};

// Device address of the scratch array on the current device (set up once per device).
prrtc_status scratch_on_current_device(void **ptr, int *sms)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return PRRTC_ECUDA;
    }
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return PRRTC_ECUDA;
        }
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return PRRTC_ECUDA;
        }
        g_scratch_ptr[dev] = p;
        g_sms[dev] = n;
    }
    *ptr = g_scratch_ptr[dev];
    *sms = g_sms[dev];
    return PRRTC_OK;
}

// The packed obstacles of the call being made: a file-scope host array (no
// heap, nothing on the caller's stack), guarded while a call packs and
// copies it.  A copy from pageable memory returns once the data is staged,
// so the array is free again when cudaMemcpyAsync returns.
float4 g_packed[PRRTC_MAX_ENV_FLOATS / 4];
std::mutex g_pack_mu;

}  // namespace

extern "C" prrtc_status prrtc_validate_configs_noalloc(prrtc_robot robot, const prrtc_env_desc *env, const float *q,
                                                       int64_t n, uint8_t *out_free, void *stream)
{
    const prrtc::RobotOps *ops = prrtc::robot_ops(robot);
    if (!ops || !env || n < 0 || (n > 0 && (!q || !out_free))) return PRRTC_EINVAL;
    auto bad = [](const float *p, uint32_t c) { return c > 0 && !p; };
    if (bad(env->spheres, env->num_spheres) || bad(env->capsules, env->num_capsules) ||
        bad(env->z_aligned_capsules, env->num_z_aligned_capsules) || bad(env->cuboids, env->num_cuboids) ||
        bad(env->z_aligned_cuboids, env->num_z_aligned_cuboids))
        return PRRTC_EINVAL;
    const uint64_t floats = 4ull * env->num_spheres + 8ull * env->num_capsules + 8ull * env->num_z_aligned_capsules +
                            16ull * env->num_cuboids + 16ull * env->num_z_aligned_cuboids;
    if (floats > (uint64_t)PRRTC_MAX_ENV_FLOATS) return PRRTC_EINVAL;   // larger than the scratch array
    if (n == 0) return PRRTC_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // Not capturable into a graph: the obstacles are copied from the library's
    // host array at call time, and a replay would copy whatever that array
    // holds then.  Under stream capture the call refuses before it touches
    // the stream, so the caller's capture stays valid.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &capture) != cudaSuccess) {
        cudaGetLastError();
        return PRRTC_ECUDA;
    }
    if (capture != cudaStreamCaptureStatusNone) return PRRTC_EINVAL;
    void *scratch = nullptr;
    int sms = 0;
    prrtc_status s = scratch_on_current_device(&scratch, &sms);
    if (s) return s;
    unsigned long long *work = reinterpret_cast<unsigned long long *>(static_cast<unsigned char *>(scratch) + kEnvBytes);
    {
        std::lock_guard<std::mutex> g(g_pack_mu);
        size_t rec = 0;
        prrtc::pack_records(*env, [&](float4 r) { g_packed[rec++] = r; });   // rec <= PRRTC_MAX_ENV_FLOATS / 4
        if ((rec && cudaMemcpyAsync(scratch, g_packed, rec * sizeof(float4), cudaMemcpyHostToDevice, st) !=
                        cudaSuccess) ||
            cudaMemsetAsync(work, 0, 2 * sizeof(unsigned long long), st) != cudaSuccess) {
            cudaGetLastError();
            return PRRTC_ECUDA;
        }
    }
    const prrtc::EnvCounts counts{(int)env->num_spheres, (int)env->num_capsules, (int)env->num_z_aligned_capsules,
                                  (int)env->num_cuboids, (int)env->num_z_aligned_cuboids};
    const prrtc::LaunchEnv le{static_cast<const float4 *>(scratch), counts, sms, work};
    if (ops->validate_configs(le, q, n, out_free, st) != cudaSuccess) {
        cudaGetLastError();
        return PRRTC_ECUDA;
    }
    return PRRTC_OK;
}
