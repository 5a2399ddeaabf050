// Device-side harness around pRRTC's own planner kernels (test and
// measurement infrastructure only).
//
// Compiled by oracle/Makefile (`ref_sampler`) from the reference sources where
// they lie: this file includes src/planning/pRRTC.cu unmodified (nothing is
// copied), so the cubin holds pRRTC's own kernels (init_rng, init_halton,
// rrtc<Robot> for every robot) and file-scope device state, and adds:
//
// * ref_halton_<Robot>: the reference's own halton_initialize (pRRTC.cu:
//   58-79, bases shuffled with cuRAND by shuffle_array, pRRTC.cu:49-56),
//   halton_next (pRRTC.cu:81-105) and Robot::scale_cfg (Robots.hh) for every
//   sampling lane, whose cuRAND state comes from ref_init_rng (below) with
//   the seed pRRTC::solve passes (1, pRRTC.cu:666).  Output:
//   bases[lane][dim], raw[lane][step][dim] and cfg[lane][step][dim] (after
//   scale_cfg).
// * ref_init_rng: the body of pRRTC's init_rng kernel (pRRTC.cu:107-111), one
//   curand_init per state.  The cubin does not hold init_rng itself (the
//   compiler keeps no entry for it here), so this is its one line again.
// * ref_reset / ref_read: what pRRTC::solve writes into and reads from its
//   file-scope state around a launch (pRRTC.cu:673-674,711-747 and
//   reset_device_variables), so a host driver can run rrtc<Robot> the way
//   pRRTC::solve does; the Environment<float> comes from ref_env_build.cuh.
// The product never links any of it.
#include "src/planning/pRRTC.cu"

using namespace ppln::collision;

#include "ref_env_build.cuh"

extern "C" __global__ void ref_init_rng(curandState *states, unsigned long seed, int n)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    curand_init(seed + idx, idx, 0, &states[idx]);
}

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

// sizes as this compilation sees them, for the host's allocations:
// curandState, HaltonState<Sphere/Panda/Fetch/Baxter>
extern "C" __global__ void ref_curand_state_bytes(unsigned long long *out)
{
    out[0] = sizeof(curandState);
    out[1] = sizeof(pRRTC::HaltonState<ppln::robots::Sphere>);
    out[2] = sizeof(pRRTC::HaltonState<ppln::robots::Panda>);
    out[3] = sizeof(pRRTC::HaltonState<ppln::robots::Fetch>);
    out[4] = sizeof(pRRTC::HaltonState<ppln::robots::Baxter>);
}

// One thread: the file-scope state pRRTC::solve sets before a launch (the
// free indices and tree sizes, pRRTC.cu:673-674) and clears after one
// (solved, path sizes, cost, goal index, iterations).
extern "C" __global__ void ref_reset(int free0, int free1)
{
    pRRTC::solved = 0;
    pRRTC::atomic_free_index[0] = free0;
    pRRTC::atomic_free_index[1] = free1;
    pRRTC::nodes_size[0] = free0;
    pRRTC::nodes_size[1] = free1;
    pRRTC::path_size[0] = 0;
    pRRTC::path_size[1] = 0;
    pRRTC::cost = 0.0f;
    pRRTC::reached_goal_idx = 0;
    pRRTC::solved_iters = 0;
}

// One thread: what pRRTC::solve reads back after a launch (pRRTC.cu:711-747).
// ints: solved, free index 0, free index 1, path size 0, path size 1,
// reached goal, solved iterations; cost; path[2][MAX_PATH_SIZE].
extern "C" __global__ void ref_read(int *ints, float *cost, float *path)
{
    ints[0] = pRRTC::solved;
    ints[1] = pRRTC::atomic_free_index[0];
    ints[2] = pRRTC::atomic_free_index[1];
    ints[3] = pRRTC::path_size[0];
    ints[4] = pRRTC::path_size[1];
    ints[5] = pRRTC::reached_goal_idx;
    ints[6] = pRRTC::solved_iters;
    cost[0] = pRRTC::cost;
    for (int t = 0; t < 2; t++)
        for (int i = 0; i < pRRTC::MAX_PATH_SIZE; i++) path[t * pRRTC::MAX_PATH_SIZE + i] = pRRTC::path[t][i];
}
