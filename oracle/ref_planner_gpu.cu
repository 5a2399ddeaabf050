// Device-side harness around pRRTC's own sampler (test infrastructure only).
//
// Compiled by oracle/Makefile (`ref_sampler`) from the reference sources where
// they lie: this file includes src/planning/pRRTC.cu unmodified (nothing is
// copied), and adds one kernel per robot that runs the reference's own
// halton_initialize (pRRTC.cu:58-79, bases shuffled with cuRAND by
// shuffle_array, pRRTC.cu:49-56), halton_next (pRRTC.cu:81-105) and
// Robot::scale_cfg (Robots.hh) for every sampling lane.  The lane's cuRAND
// state comes from the reference's own init_rng kernel (pRRTC.cu:107-111),
// which the tests launch by name with the seed pRRTC::solve passes (1,
// pRRTC.cu:666).  The product never links any of it.
//
// Output: bases[lane][dim] (the lane's shuffled primes), raw[lane][step][dim]
// (halton_next's values) and cfg[lane][step][dim] (after scale_cfg).
#include "src/planning/pRRTC.cu"

template <class Robot>
__device__ void ref_sequence(curandState *rng, float *bases, float *raw, float *cfg, int lanes, int steps)
{
    constexpr int D = Robot::dimension;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= lanes) return;
    pRRTC::HaltonState<Robot> h;
    curandState st = rng[idx];
    pRRTC::halton_initialize(h, 0, st, idx);
    for (int d = 0; d < D; d++) bases[(size_t)idx * D + d] = h.b[d];
    float r[D];
    for (int s = 0; s < steps; s++) {
        pRRTC::halton_next(h, r);
        const size_t o = ((size_t)idx * steps + s) * D;
        for (int d = 0; d < D; d++) raw[o + d] = r[d];
        Robot::scale_cfg(r);
        for (int d = 0; d < D; d++) cfg[o + d] = r[d];
    }
}

#define REF_SEQ_KERNEL(R)                                                                                 \
    extern "C" __global__ void ref_halton_##R(curandState *rng, float *bases, float *raw, float *cfg,     \
                                              int lanes, int steps)                                      \
    {                                                                                                     \
        ref_sequence<ppln::robots::R>(rng, bases, raw, cfg, lanes, steps);                                \
    }

REF_SEQ_KERNEL(Sphere)
REF_SEQ_KERNEL(Panda)
REF_SEQ_KERNEL(Fetch)
REF_SEQ_KERNEL(Baxter)

// sizeof(curandState) as this compilation sees it, for the host's allocation
extern "C" __global__ void ref_curand_state_bytes(unsigned long long *out) { out[0] = sizeof(curandState); }
