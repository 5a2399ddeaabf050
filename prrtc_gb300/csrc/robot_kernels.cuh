// Per-robot kernels.  Included by one translation unit per robot after that
// robot's generated checker; GEN names the generated namespace.
#pragma once

#include "clearance_kernel.cuh"
#include "device_common.cuh"
#include "planner_device.cuh"
#include "prrtc_internal.h"

namespace prrtc {

// Configurations are read row-major; every thread owns one configuration.
template <int D>
__device__ __forceinline__ void load_cfg(const float *__restrict__ q, int64_t i, float (&out)[D])
{
#pragma unroll
    for (int d = 0; d < D; d++) out[d] = __ldg(q + i * D + d);
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// work[0] += algorithmic FLOPs, work[1] += configurations (one atomic per warp)
__device__ __forceinline__ void add_work(unsigned long long *work, unsigned long long flops, unsigned long long cfgs)
{
    flops = warp_sum(flops);
    cfgs = warp_sum(cfgs);
    if ((threadIdx.x & 31) == 0 && work) {
        atomicAdd(work, flops);
        atomicAdd(work + 1, cfgs);
    }
}

// Launch bounds of the stand-alone configuration checker, per robot: by
// default at most 64 registers (128-thread blocks, 8 per SM), where the
// straight-line checker spills a little but 32 resident warps per SM instead
// of 16 hide its dependency waits better (2^20 random configurations: Panda
// 1.23 vs 1.27 ms on the tabletop scene and 1.81 vs 1.97 ms on the shelf,
// Baxter 3.70 ms against 4.50 ms unconstrained and 4.53 ms at 122 registers
// on a shelf scene; Fetch, table form, 5.28 ms against 5.56 ms
// unconstrained); a robot file may specialise it.
template <class Gen>
struct ValidateLaunch {
    static constexpr int kMaxThreads = 128, kMinBlocks = 8;
};

template <class Gen>
__global__ void __launch_bounds__(ValidateLaunch<Gen>::kMaxThreads, ValidateLaunch<Gen>::kMinBlocks)
    k_validate_configs(const float4 *__restrict__ env, EnvCounts nc,
                                                          const float *__restrict__ q, int64_t n,
                                                          uint8_t *__restrict__ out, unsigned long long *work)
{
    extern __shared__ float4 s_env[];
    __shared__ unsigned long long s_bar;
    stage_env_bulk(s_env, env, nc.records(), &s_bar);
    CheckCtx ctx{{s_env, nc}, 0.0f, nullptr};
    unsigned long long flops = 0, cfgs = 0;
    // The warp steps through the grid-stride loop together (a warp-uniform
    // trip count) and meets at __syncwarp after every configuration: lanes
    // whose check ended early wait there instead of starting their next
    // configuration out of step with the rest.  Blocks are whole warps (128
    // threads).  Baxter's table-form walk on 2^20 random configurations: 4.7
    // instead of 17.2 ms, 13.7 instead of 3.7 lanes active per instruction.
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w < n; w += stride) {
        const int64_t i = w + (threadIdx.x & 31u);
        if (i < n) {
            float cfg[Gen::kDof];
            load_cfg<Gen::kDof>(q, i, cfg);
            ctx.work = 0;
            out[i] = Gen::fkcc_validate(cfg, ctx) ? 1 : 0;
            flops += ctx.work + Gen::kFkFlops;
            cfgs++;
        }
        __syncwarp();
    }
    add_work(work, flops, cfgs);
}

// One block per edge (grid-stride): thread t checks points k = t+1, t+1+blockDim, ...
// MinBlocks > 0 builds it for that many resident 128-thread blocks per SM: 8
// (at most 64 registers) is faster for 128-point edges (the Panda shelf
// scene at g = 128: 1.79 vs 1.91 ms for 2^14 edges) and slower for the
// 32-thread blocks of short edges, which keep the unconstrained build (0).
template <class Gen, int MinBlocks>
__global__ void __launch_bounds__(128, MinBlocks) k_validate_edges(const float4 *__restrict__ env, EnvCounts nc,
                                                        const float *__restrict__ a, const float *__restrict__ b,
                                                        int64_t n, int g, uint8_t *__restrict__ out,
                                                        unsigned long long *work)
{
    unsigned long long flops = 0, cfgs = 0;
    constexpr int D = Gen::kDof;
    extern __shared__ float4 s_env[];
    __shared__ float s_a[D], s_step[D];
    __shared__ int s_bad;
    __shared__ unsigned long long s_bar;
    stage_env_bulk(s_env, env, nc.records(), &s_bar);
    CheckCtx ctx{{s_env, nc}, 0.0f, &s_bad};
    const float fg = (float)g;
    for (int64_t e = blockIdx.x; e < n; e += gridDim.x) {
        __syncthreads();
        if (threadIdx.x == 0) s_bad = 0;
        if (threadIdx.x < D) {
            const float av = __ldg(a + e * D + threadIdx.x);
            s_a[threadIdx.x] = av;
            s_step[threadIdx.x] = __fdiv_rn(__fsub_rn(__ldg(b + e * D + threadIdx.x), av), fg);
        }
        __syncthreads();
        for (int k = threadIdx.x + 1; k <= g; k += blockDim.x) {
            if (s_bad) break;
            float cfg[D];
#pragma unroll
            for (int d = 0; d < D; d++) cfg[d] = __fadd_rn(s_a[d], __fmul_rn((float)k, s_step[d]));
            ctx.work = 0;
            if (!Gen::fkcc(cfg, ctx)) s_bad = 1;
            flops += ctx.work + Gen::kFkFlops;
            cfgs++;
        }
        __syncthreads();
        if (threadIdx.x == 0) out[e] = s_bad ? 0 : 1;
    }
    add_work(work, flops, cfgs);
}

// Goal-region candidates: flags[t] = 1 when candidate t (goal_candidate)
// puts the chosen sphere's centre in the box and the checker finds it free.
template <class Gen>
__global__ void __launch_bounds__(128) k_goal_flags(const float4 *__restrict__ env, EnvCounts nc, const GoalQuery g,
                                                    uint8_t *__restrict__ flags)
{
    extern __shared__ float4 s_env[];
    __shared__ unsigned long long s_bar;
    stage_env_bulk(s_env, env, nc.records(), &s_bar);
    CheckCtx ctx{{s_env, nc}, 0.0f, nullptr};
    // warp-uniform trip count, lanes meeting after every candidate (as in k_validate_configs)
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long tw = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); tw < g.tries; tw += stride) {
        const long long t = tw + (threadIdx.x & 31u);
        if (t < g.tries) {
            float q[Gen::kDof];
            goal_candidate(g.seed, t, Gen::kDof, g.scale, g.offset, q);
            float4 s[Gen::kNumSpheres];
            Gen::fk_spheres(q, s);
            const float4 c = s[g.sphere];
            bool ok = c.x >= g.lo[0] && c.x <= g.hi[0] && c.y >= g.lo[1] && c.y <= g.hi[1] && c.z >= g.lo[2] &&
                      c.z <= g.hi[2];
            if (ok) {
                ctx.work = 0;
                ok = Gen::fkcc_validate(q, ctx);
            }
            flags[t] = ok ? 1 : 0;
        }
        __syncwarp();
    }
}

template <class Gen>
__global__ void __launch_bounds__(128) k_fk_spheres(const float *__restrict__ q, int64_t n, float4 *__restrict__ out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float cfg[Gen::kDof];
        load_cfg<Gen::kDof>(q, i, cfg);
        Gen::fk_spheres(cfg, out + i * Gen::kNumSpheres);
    }
}


// ---------------------------------------------------------------------------
// Plain form: the reference's persistent RRT-Connect kernel (rrtc<Robot>,
// pRRTC.cu:305-602) with one block per sampling lane.  Per pass a block
// samples (Halton, per-lane bases), scans its tree for the nearest node,
// steers by `range`, validates the edge at `granularity` points with all of
// its threads, appends the node, then scans the other tree and tries to
// connect in ceil(d / range) validated sub-edges.  The first block to connect
// wins a CAS on ctl->solved and traces the path.
//
// Departures from the reference, all deliberate:
//  * sub-edge points are a + k * ((b - a) / g) with b the node about to be
//    appended (the reference uses vec / g; the two differ only in rounding),
//    so every point a revalidation of the returned path checks is a point the
//    planner checked;
//  * edge validation stops early once any thread of the block has found a
//    collision (block flag polled between checker groups);
//  * nodes past max_samples are never written (the reference writes them
//    before failing, pRRTC.cu:451-454,535-537), the traceback is bounded by
//    the path buffer, and the DD CAS loops are bounded;
//  * an optional device time budget ends the search with solved = -2.
template <class Gen>
__global__ void __launch_bounds__(256) k_rrtc_plain(const PlainParams P)
{
    constexpr int D = Gen::kDof;
    extern __shared__ float4 s_env[];
    __shared__ float s_cfg[D], s_nn[D], s_step[D], s_vec[D], s_next[D];
    __shared__ float s_hb[D], s_hn[D], s_hd[D];
    __shared__ float s_red_d[8];
    __shared__ int s_red_i[8];
    __shared__ float s_dsq, s_scale;
    __shared__ int s_nn_idx, s_index, s_t, s_o, s_bad, s_skip, s_exit;
    __shared__ unsigned s_next_ext;
    const int tid = threadIdx.x, bid = blockIdx.x;
    volatile QueryCtl *ctl = P.ctl;

    __shared__ unsigned long long s_bar;
    if (tid < D) {
        s_hb[tid] = P.halton_bases[bid * 16 + tid];
        s_hn[tid] = 0.0f;
        s_hd[tid] = 1.0f;
    }
    stage_env_bulk(s_env, P.env, P.env_n.records(), &s_bar);   // synchronises the block
    CheckCtx ctx{{s_env, P.env_n}, P.pad, &s_bad};
    const float fg = (float)P.granularity;
    const unsigned long long t0 = P.budget_ns ? global_ns() : 0ull;
    int iter = 0;
    unsigned long long my_flops = 0, my_cfgs = 0;

    while (true) {
        if (tid == 0) {
            iter++;
            if (iter > P.max_iters) atomicCAS((int *)&ctl->solved, 0, -1);
            if (P.budget_ns && global_ns() - t0 > P.budget_ns) atomicCAS((int *)&ctl->solved, 0, -2);
            // tree choice (pRRTC.cu:348-371)
            const int f0 = ctl->free_index[0], f1 = ctl->free_index[1];
            if (P.balance == 0 || iter == 1) {
                s_t = (bid < (P.num_new_configs / 2)) ? 0 : 1;
            } else if (P.balance == 1 && 2 * abs(f0 - f1) < 3 * P.num_new_configs) {
                const float ratio = f0 / (float)(f0 + f1);
                s_t = ((float)bid < P.num_new_configs * (1.0f - ratio)) ? 0 : 1;
            } else if (P.balance == 1) {
                const float ratio = f0 / (float)(f0 + f1);
                s_t = ratio < P.tree_ratio ? 0 : 1;
            } else if (P.balance == 2) {
                const int ft = s_t == 0 ? f0 : f1, fo = s_t == 0 ? f1 : f0;
                const float ratio = abs(ft - fo) / (float)ft;
                if (ratio < P.tree_ratio) s_t = 1 - s_t;
            }
            s_o = 1 - s_t;
            halton_next<D>(s_hb, s_hn, s_hd, s_cfg);
            scale_sample<D>(s_cfg, P.scale, P.offset);
        }
        __syncthreads();
        const int t = s_t, o = s_o;

        // nearest node of this tree (pRRTC.cu:384-412)
        block_nn<D>(P.nodes[t], P.cap, ctl->free_index[t], s_cfg, s_red_d, s_red_i, &s_dsq, &s_nn_idx);
        if (tid == 0) {
            const float dist = sqrtf(s_dsq);
            s_scale = fminf(1.0f, P.range / dist);
            s_skip = P.dynamic_domain && __ldcg(P.radii[t] + s_nn_idx) < dist;
            s_exit = ctl->solved != 0;
            s_bad = 0;
        }
        if (tid < D) s_nn[tid] = __ldcg(P.nodes[t] + (size_t)tid * P.cap + s_nn_idx);
        __syncthreads();
        if (s_skip) {
            if (s_exit) break;
            continue;
        }
        // steer and validate the extension edge (pRRTC.cu:430-444)
        if (tid < D) {
            const float nn = s_nn[tid];
            const float c = fmaf(s_cfg[tid] - nn, s_scale, nn);
            s_cfg[tid] = c;
            s_step[tid] = __fdiv_rn(__fsub_rn(c, nn), fg);
        }
        __syncthreads();
        for (int k = tid + 1; k <= P.granularity; k += blockDim.x) {
            if (s_bad) break;
            float q[D];
#pragma unroll
            for (int d = 0; d < D; d++) q[d] = __fadd_rn(s_nn[d], __fmul_rn((float)k, s_step[d]));
            ctx.work = 0;
            if (!Gen::fkcc(q, ctx)) s_bad = 1;
            my_flops += ctx.work + Gen::kFkFlops;
            my_cfgs++;
        }
        __syncthreads();

        if (!s_bad) {
            // append (pRRTC.cu:447-476)
            if (tid == 0) {
                const int idx = atomicAdd((int *)&ctl->free_index[t], 1);
                if (idx >= P.max_samples || idx >= P.cap) {
                    atomicCAS((int *)&ctl->solved, 0, -1);
                    s_index = -1;
                } else {
                    P.parents[t][idx] = s_nn_idx;
                    if (P.dynamic_domain) {
                        P.radii[t][idx] = FLT_MAX;
                        dd_grow(P.radii[t] + s_nn_idx, P.dd_alpha);
                    }
                    s_index = idx;
                }
            }
            __syncthreads();
            const int index = s_index;
            if (index >= 0) {
                if (tid < D) P.nodes[t][(size_t)tid * P.cap + index] = s_cfg[tid];
                __threadfence();
                __syncthreads();
                // connect (pRRTC.cu:478-551)
                block_nn<D>(P.nodes[o], P.cap, ctl->free_index[o], s_cfg, s_red_d, s_red_i, &s_dsq, &s_nn_idx);
                if (tid == 0) {
                    s_next_ext = (unsigned)ceilf(sqrtf(s_dsq) / P.range);
                    s_bad = 0;
                }
                __syncthreads();
                const unsigned n_ext = s_next_ext;
                if (tid < D) s_vec[tid] = (__ldcg(P.nodes[o] + (size_t)tid * P.cap + s_nn_idx) - s_cfg[tid]) / (float)n_ext;
                __syncthreads();
                unsigned i_ext = 0;
                int parent = index;
                while (i_ext < n_ext) {
                    if (tid < D) {
                        const float a = s_cfg[tid];
                        const float b = a + s_vec[tid];
                        s_next[tid] = b;
                        s_step[tid] = __fdiv_rn(__fsub_rn(b, a), fg);
                    }
                    __syncthreads();
                    for (int k = tid + 1; k <= P.granularity; k += blockDim.x) {
                        if (s_bad) break;
                        float q[D];
#pragma unroll
                        for (int d = 0; d < D; d++) q[d] = __fadd_rn(s_cfg[d], __fmul_rn((float)k, s_step[d]));
                        ctx.work = 0;
                        if (!Gen::fkcc(q, ctx)) s_bad = 1;
                        my_flops += ctx.work + Gen::kFkFlops;
                        my_cfgs++;
                    }
                    __syncthreads();
                    if (s_bad) break;
                    if (tid == 0) {
                        const int idx = atomicAdd((int *)&ctl->free_index[t], 1);
                        if (idx >= P.max_samples || idx >= P.cap) {
                            atomicCAS((int *)&ctl->solved, 0, -1);
                            s_index = -1;
                        } else {
                            P.parents[t][idx] = parent;
                            P.radii[t][idx] = FLT_MAX;
                            s_index = idx;
                        }
                    }
                    __syncthreads();
                    if (s_index < 0) break;
                    if (tid < D) {
                        s_cfg[tid] = s_next[tid];
                        P.nodes[t][(size_t)tid * P.cap + s_index] = s_next[tid];
                    }
                    __threadfence();
                    parent = s_index;
                    i_ext++;
                    __syncthreads();
                }
                if (i_ext == n_ext && s_index >= 0) {
                    // connected: the first block wins and traces both trees (pRRTC.cu:552-582)
                    if (tid == 0 && atomicCAS((int *)&ctl->solved, 0, 1) == 0) {
                        __threadfence();
                        float cost = 0.0f;
                        int root_t = 0, root_o = 0;
                        const int nt = trace_to_root<D>(P.nodes[t], P.parents[t], P.cap, s_index,
                                                        P.path + (size_t)t * P.path_cap * D, P.path_cap, &cost, &root_t);
                        const int no = trace_to_root<D>(P.nodes[o], P.parents[o], P.cap, s_nn_idx,
                                                        P.path + (size_t)o * P.path_cap * D, P.path_cap, &cost, &root_o);
                        if (nt < 0 || no < 0) ctl->error |= 1;
                        ctl->path_size[t] = nt < 0 ? 0 : nt;
                        ctl->path_size[o] = no < 0 ? 0 : no;
                        ctl->reached_goal = t == 1 ? root_t : root_o;
                        ctl->cost = cost;
                        ctl->solved_iters = iter;
                        __threadfence();
                    }
                    __syncthreads();
                }
            }
        } else if (P.dynamic_domain && tid == 0) {
            dd_shrink(P.radii[t] + s_nn_idx, P.dd_alpha, P.dd_radius, P.dd_min_radius);
        }
        __syncthreads();
        if (tid == 0) s_exit = ctl->solved != 0;
        __syncthreads();
        if (s_exit) break;
    }
    add_work(P.work, my_flops, my_cfgs);
}

}  // namespace prrtc

#include "batch_kernel.cuh"

namespace prrtc {

inline int grid_for(int64_t work, int threads, int sms, int per_sm)
{
    int64_t blocks = (work + threads - 1) / threads;
    int64_t cap = (int64_t)sms * per_sm;
    if (blocks > cap) blocks = cap;
    return blocks < 1 ? 1 : (int)blocks;
}

template <class Gen>
struct RobotKernels {
    static cudaError_t validate_configs(const LaunchEnv &le, const float *q, int64_t n, uint8_t *out,
                                        cudaStream_t st)
    {
        if (n <= 0) return cudaSuccess;
        const int threads = 128;
        const size_t smem = (size_t)le.counts.records() * sizeof(float4);
        k_validate_configs<Gen><<<grid_for(n, threads, le.sms, 16), threads, smem, st>>>(le.rec, le.counts, q, n, out, le.work);
        return cudaGetLastError();
    }
    static cudaError_t validate_edges(const LaunchEnv &le, const float *a, const float *b, int64_t n, int g,
                                      uint8_t *out, cudaStream_t st)
    {
        if (n <= 0) return cudaSuccess;
        const int threads = g >= 128 ? 128 : ((g + 31) / 32) * 32;
        const size_t smem = (size_t)le.counts.records() * sizeof(float4);
        int64_t blocks = n;
        const int64_t cap = (int64_t)le.sms * (2048 / threads);
        if (blocks > cap) blocks = cap;
        if (threads == 128)
            k_validate_edges<Gen, 8><<<(int)blocks, threads, smem, st>>>(le.rec, le.counts, a, b, n, g, out, le.work);
        else
            k_validate_edges<Gen, 0><<<(int)blocks, threads, smem, st>>>(le.rec, le.counts, a, b, n, g, out, le.work);
        return cudaGetLastError();
    }
    static cudaError_t fk_spheres(const float *q, int64_t n, float *out, int sms, cudaStream_t st)
    {
        if (n <= 0) return cudaSuccess;
        k_fk_spheres<Gen><<<grid_for(n, 128, sms, 8), 128, 0, st>>>(q, n, reinterpret_cast<float4 *>(out));
        return cudaGetLastError();
    }
    static cudaError_t solve_plain(const PlainParams &P, int threads, cudaStream_t st)
    {
        const size_t smem = (size_t)P.env_n.records() * sizeof(float4);
        k_rrtc_plain<Gen><<<P.num_new_configs, threads, smem, st>>>(P);
        return cudaGetLastError();
    }
    static cudaError_t solve_batch(const BatchParams &P, int blocks, int wpb, cudaStream_t st)
    {
        // (batch_occupancy, called when the batch is created, set the kernel's
        // dynamic shared-memory limit for this size)
        const size_t smem = warp_scratch_bytes<Gen>(P.env_records, P.shared_frames) * wpb;
        k_rrtc_batch<Gen><<<blocks, 32 * wpb, smem, st>>>(P);
        return cudaGetLastError();
    }
    static int batch_occupancy(int wpb, int env_records, int shared_frames)
    {
        int n = 0;
        const size_t smem = warp_scratch_bytes<Gen>(env_records, shared_frames != 0) * wpb;
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(k_rrtc_batch<Gen>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_rrtc_batch<Gen>, 32 * wpb, smem) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return n;
    }
    static cudaError_t goal_flags(const LaunchEnv &le, const GoalQuery &g, uint8_t *flags, cudaStream_t st)
    {
        if (g.tries <= 0) return cudaSuccess;
        const size_t smem = (size_t)le.counts.records() * sizeof(float4);
        k_goal_flags<Gen><<<grid_for(g.tries, 128, le.sms, 16), 128, smem, st>>>(le.rec, le.counts, g, flags);
        return cudaGetLastError();
    }
    static cudaError_t smooth_paths(const ClrLaunch &P, size_t env_bytes, cudaStream_t st)
    {
        if (P.n_paths <= 0) return cudaSuccess;
        const size_t smem = env_bytes + 2 * sizeof(float) * (size_t)P.waypoints * Gen::kDof;
        cudaError_t e = cudaFuncSetAttribute(k_smooth_paths<Gen>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        const int threads = P.waypoints <= 64 ? 64 : 128;
        k_smooth_paths<Gen><<<P.n_paths, threads, smem, st>>>(P);
        return cudaGetLastError();
    }
    static RobotOps ops(int dof_check)
    {
        RobotOps o{};
        o.dof = Gen::kDof;
        o.num_spheres = Gen::kNumSpheres;
        o.validate_configs = &validate_configs;
        o.validate_edges = &validate_edges;
        o.fk_spheres = &fk_spheres;
        o.solve_plain = &solve_plain;
        o.solve_batch = &solve_batch;
        o.batch_occupancy = &batch_occupancy;
        o.smooth_paths = &smooth_paths;
        o.goal_flags = &goal_flags;
        (void)dof_check;
        return o;
    }
};

}  // namespace prrtc

// Wraps a generated namespace into the Gen interface the kernels expect.
#define PRRTC_GEN_ADAPTER(NAME, NS)                                                                 \
    namespace prrtc {                                                                               \
    struct NAME {                                                                                   \
        static constexpr int kDof = NS::kDof;                                                       \
        static constexpr int kNumSpheres = NS::kNumSpheres;                                         \
        static constexpr int kFrames = NS::kFrames;                                                 \
        static constexpr unsigned kFkFlops = NS::kFkFlops;                                          \
        template <class Ctx>                                                                        \
        static __device__ __forceinline__ bool fkcc(const float *q, Ctx &ctx)                       \
        {                                                                                           \
            return NS::fkcc(q, ctx);                                                                \
        }                                                                                           \
        template <class Ctx>                                                                        \
        static __device__ __forceinline__ bool fkcc_validate(const float *q, Ctx &ctx)              \
        {                                                                                           \
            return NS::fkcc_validate(q, ctx);                                                       \
        }                                                                                           \
        static __device__ __forceinline__ void fk_spheres(const float *q, float4 *out)              \
        {                                                                                           \
            NS::fk_spheres(q, out);                                                                 \
        }                                                                                           \
    };                                                                                              \
    }
