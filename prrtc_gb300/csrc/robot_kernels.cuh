// Per-robot kernels.  Included by one translation unit per robot after that
// robot's generated checker; GEN names the generated namespace.
#pragma once

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

template <class Gen>
__global__ void __launch_bounds__(256) k_validate_configs(const float4 *__restrict__ env, EnvCounts nc,
                                                          const float *__restrict__ q, int64_t n,
                                                          uint8_t *__restrict__ out, unsigned long long *work)
{
    extern __shared__ float4 s_env[];
    stage_env(s_env, env, nc.records());
    __syncthreads();
    CheckCtx ctx{{s_env, nc}, 0.0f, nullptr};
    unsigned long long flops = 0, cfgs = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float cfg[Gen::kDof];
        load_cfg<Gen::kDof>(q, i, cfg);
        ctx.work = 0;
        out[i] = Gen::fkcc(cfg, ctx) ? 1 : 0;
        flops += ctx.work + Gen::kFkFlops;
        cfgs++;
    }
    add_work(work, flops, cfgs);
}

// One block per edge (grid-stride): thread t checks points k = t+1, t+1+blockDim, ...
template <class Gen>
__global__ void __launch_bounds__(128) k_validate_edges(const float4 *__restrict__ env, EnvCounts nc,
                                                        const float *__restrict__ a, const float *__restrict__ b,
                                                        int64_t n, int g, uint8_t *__restrict__ out,
                                                        unsigned long long *work)
{
    unsigned long long flops = 0, cfgs = 0;
    constexpr int D = Gen::kDof;
    extern __shared__ float4 s_env[];
    __shared__ float s_a[D], s_step[D];
    __shared__ int s_bad;
    stage_env(s_env, env, nc.records());
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

    stage_env(s_env, P.env, P.env_n.records());
    if (tid < D) {
        s_hb[tid] = P.halton_bases[bid * 16 + tid];
        s_hn[tid] = 0.0f;
        s_hd[tid] = 1.0f;
    }
    __syncthreads();
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
#pragma unroll
            for (int d = 0; d < D; d++) s_cfg[d] = fmaf(s_cfg[d], P.scale[d], P.offset[d]);
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

// ---------------------------------------------------------------------------
// Batched form: many queries, one persistent launch.  Every warp is an
// independent worker.  Queries occupy slots (trees in a slot-indexed arena);
// a worker joins a running slot, runs one RRT-Connect iteration there, and
// keeps iterating until the slot's query is finished; then it moves on to the
// next running slot (round-robin cursor), so the warps of finished queries are
// stolen by the unfinished ones.  The last warp to leave a finished slot
// restores its arena region to NaN and admits the next pending query into it.
//
// Sampling follows the reference's lanes virtually: sample k of a query is
// Halton point k / L + 1 of virtual lane k % L, whose prime bases are that
// lane's (the reference's per-block shuffled bases); balance modes use the
// virtual lane as the reference uses blockIdx.

struct WarpScratch {
    float from[16], step[16], cfg[16], nn[16], vec[16], next[16];
    int bad;
    int pad_[3];
};

// Whole warp: check the g points of the edge in W (from + k * step),
// k = 1..g, in ceil(g / 32) rounds of one point per lane.  Contiguous order
// gives round r the points 32 r + lane + 1; interleaved order gives it
// lane * R + r + 1, so the first round already samples the whole edge at
// stride R and a collision usually ends the edge after one round.  Adds the
// work done to work[0] (FLOPs) and work[1] (points).
template <class Gen>
__device__ __forceinline__ bool warp_validate(const WarpScratch &W, int g, int interleave, CheckCtx &ctx,
                                              unsigned long long *work)
{
    constexpr int D = Gen::kDof;
    const int lane = lane_id();
    volatile int *flag = ctx.stop_flag;
    if (lane == 0) *flag = 0;
    __syncwarp();
    bool bad = false;
    int n = 0;
    unsigned long long flops = 0;
    const int R = (g + 31) >> 5;
    for (int r = 0; r < R; r++) {
        const int k = interleave ? lane * R + r + 1 : 32 * r + lane + 1;
        const bool run = k <= g && !*flag;
        if (run) {
            float q[D];
#pragma unroll
            for (int d = 0; d < D; d++) q[d] = __fadd_rn(W.from[d], __fmul_rn((float)k, W.step[d]));
            ctx.work = 0;
            if (!Gen::fkcc(q, ctx)) {
                bad = true;
                *flag = 1;
            }
            flops += ctx.work + Gen::kFkFlops;
        }
        n += __popc(__ballot_sync(0xffffffffu, run));
        if (__any_sync(0xffffffffu, bad)) break;
    }
    flops = warp_sum(flops);
    if (lane == 0) {
        atomicAdd(work, flops);
        atomicAdd(work + 1, (unsigned long long)n);
    }
    return !__any_sync(0xffffffffu, bad);
}

// lane 0 only: finish an unsolved query (first caller wins)
__device__ __forceinline__ void batch_finish(const BatchParams &P, SlotState *S, int q, int status)
{
    if (atomicCAS(&S->state, SLOT_RUNNING, SLOT_DONE) != SLOT_RUNNING) return;
    BatchOut &o = P.out[q];
    volatile SlotState *vs = S;
    o.solved = 0;
    o.status = status;
    o.start_tree_size = min(vs->free_index[0], P.cap);
    o.goal_tree_size = min(vs->free_index[1], P.cap);
    o.path_length = 0;
    o.iters = -1;
    o.cost = 0.0f;
    o.path_rows = 0;
    o.samples = vs->ticket;
    o.t_done = global_ns();
    __threadfence();
    atomicAdd(&P.ctr->done, 1);
}

// lane 0 only: walk a tree from `start` to its root; returns the node count
// (root excluded) or -1 on a broken chain.
template <int D>
__device__ int chain_length(const int *parents, int cap, int start, int *root)
{
    const volatile int *vp = parents;
    int cur = start;
    for (int n = 0; n <= cap; n++) {
        const int par = vp[cur];
        if (par == cur) {
            *root = cur;
            return n;
        }
        if (par < 0 || par >= cap) return -1;
        cur = par;
    }
    return -1;
}

// lane 0 only: trace the solution into the path pool in the reference's
// order (goal, goal-tree segment toward the junction, start-tree segment,
// start; pRRTC.cu:731-741) and publish the query's result.
template <int D>
__device__ void batch_trace(const BatchParams &P, SlotState *S, int s, int q, int t, int jt, int jo, int iter)
{
    const float *nodes_s = P.nodes + (size_t)s * 2 * D * P.cap;
    const int *par_s = P.parents + (size_t)s * 2 * P.cap;
    const int o = 1 - t;
    const int j0 = t == 0 ? jt : jo, j1 = t == 0 ? jo : jt;
    int r0 = 0, r1 = 0;
    const int n0 = chain_length<D>(par_s, P.cap, j0, &r0);
    const int n1 = chain_length<D>(par_s + P.cap, P.cap, j1, &r1);
    BatchOut &out = P.out[q];
    out.solved = 1;
    out.iters = iter;
    out.reached_goal = r1;
    volatile SlotState *vs = S;
    out.start_tree_size = min(vs->free_index[0], P.cap);
    out.goal_tree_size = min(vs->free_index[1], P.cap);
    out.samples = vs->ticket;
    if (n0 < 0 || n1 < 0) {
        out.status = PRRTC_ENOMEM;
        out.path_rows = 0;
    } else {
        const int rows = n0 + n1 + 2;
        const int off = atomicAdd(&P.ctr->path_next, rows);
        // cost in the reference's order: the connecting tree first, then the other
        float cost = 0.0f;
        for (int pass = 0; pass < 2; pass++) {
            const int tree = pass == 0 ? t : o;
            const float *nd = nodes_s + (size_t)tree * D * P.cap;
            const int *pr = par_s + (size_t)tree * P.cap;
            int cur = tree == 0 ? j0 : j1;
            const int n = tree == 0 ? n0 : n1;
            for (int i = 0; i < n; i++) {
                const int par = ((const volatile int *)pr)[cur];
                float acc = 0.0f;
                const bool write = off + rows <= P.path_pool_rows;
                const int row = tree == 0 ? off + n1 + 1 + i : off + n1 - i;
#pragma unroll
                for (int d = 0; d < D; d++) {
                    const float a = __ldcg(nd + (size_t)d * P.cap + cur);
                    const float b = __ldcg(nd + (size_t)d * P.cap + par);
                    const float df = a - b;
                    acc = fmaf(df, df, acc);
                    if (write) P.path_pool[(size_t)row * D + d] = a;
                }
                cost += sqrtf(acc);
                cur = par;
            }
        }
        out.cost = cost;
        out.path_length = n0 + n1;
        if (off + rows <= P.path_pool_rows) {
            const BatchQueryDesc &Q = P.queries[q];
            const float *start = P.cfg_pool + Q.cfg_off;
            const float *goal = start + D + (size_t)r1 * D;
#pragma unroll
            for (int d = 0; d < D; d++) {
                P.path_pool[(size_t)off * D + d] = goal[d];
                P.path_pool[(size_t)(off + rows - 1) * D + d] = start[d];
            }
            out.path_off = off;
            out.path_rows = rows;
            out.status = 0;
        } else {
            out.path_rows = 0;
            out.status = PRRTC_ENOMEM;
        }
    }
    out.t_done = global_ns();
    __threadfence();
    atomicAdd(&P.ctr->done, 1);
}

// whole warp: write query qa's roots into slot s and start it
template <int D>
__device__ void batch_admit(const BatchParams &P, int s, int qa)
{
    const int lane = lane_id();
    const BatchQueryDesc Q = P.queries[qa];
    float *nodes_s = P.nodes + (size_t)s * 2 * D * P.cap;
    int *par_s = P.parents + (size_t)s * 2 * P.cap;
    float *rad_s = P.radii + (size_t)s * 2 * P.cap;
    const float *cfg = P.cfg_pool + Q.cfg_off;
    if (lane < D) nodes_s[(size_t)lane * P.cap] = cfg[lane];
    for (int i = lane; i < Q.num_goals * D; i += 32) {
        const int g = i / D, d = i % D;
        nodes_s[(size_t)D * P.cap + (size_t)d * P.cap + g] = cfg[D + i];
    }
    for (int g = lane; g < Q.num_goals; g += 32) {
        par_s[P.cap + g] = g;
        rad_s[P.cap + g] = FLT_MAX;
    }
    if (lane == 0) {
        par_s[0] = 0;
        rad_s[0] = FLT_MAX;
    }
    if (P.balance == 2)
        for (int l = lane; l < P.lanes; l += 32) P.tsel[(size_t)s * P.lanes + l] = 0;
    if (lane == 0) {
        SlotState *S = &P.slots[s];
        S->query = qa;
        S->free_index[0] = 1;
        S->free_index[1] = Q.num_goals;
        S->ticket = 0;
        P.out[qa].t_admit = global_ns();
    }
    __threadfence();
    __syncwarp();
    if (lane == 0) atomicExch(&P.slots[s].state, SLOT_RUNNING);
}

// whole warp: restore slot s's used arena prefix to NaN
template <int D>
__device__ void batch_scrub(const BatchParams &P, int s)
{
    const volatile SlotState *vs = &P.slots[s];
    float *nodes_s = P.nodes + (size_t)s * 2 * D * P.cap;
    for (int t = 0; t < 2; t++) {
        const int n = min(vs->free_index[t], P.cap);
        float *nd = nodes_s + (size_t)t * D * P.cap;
        for (int d = 0; d < D; d++)
            for (int i = lane_id(); i < n; i += 32) nd[(size_t)d * P.cap + i] = __int_as_float(0xFFFFFFFF);
    }
    __threadfence();
    __syncwarp();
}

// whole warp: leave slot s; the last warp out of a finished slot scrubs it
// and admits the next pending query (returns true if this warp now works on
// that newly admitted query).
template <int D>
__device__ bool batch_leave(const BatchParams &P, int s, bool allow_admit)
{
    const int lane = lane_id();
    int recycle = 0;
    if (lane == 0) {
        __threadfence();
        SlotState *S = &P.slots[s];
        const int left = atomicSub(&S->workers, 1) - 1;
        recycle = left == 0 && atomicCAS(&S->state, SLOT_DONE, SLOT_BUSY) == SLOT_DONE;
    }
    recycle = __shfl_sync(0xffffffffu, recycle, 0);
    if (!recycle) return false;
    batch_scrub<D>(P, s);
    int qa = -1;
    if (lane == 0 && allow_admit) {
        if (*(volatile int *)&P.ctr->admit_next < P.num_queries) qa = atomicAdd(&P.ctr->admit_next, 1);
        if (qa >= P.num_queries) qa = -1;
        if (qa >= 0) atomicAdd(&P.slots[s].workers, 1);
    }
    qa = __shfl_sync(0xffffffffu, qa, 0);
    if (qa >= 0) {
        batch_admit<D>(P, s, qa);
        return true;
    }
    if (lane == 0) atomicExch(&P.slots[s].state, SLOT_FREE);
    return false;
}

template <class Gen>
__global__ void __launch_bounds__(128) k_rrtc_batch(const BatchParams P)
{
    constexpr int D = Gen::kDof;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ float4 s_raw[];
    WarpScratch &W = reinterpret_cast<WarpScratch *>(s_raw)[threadIdx.x >> 5];
    const int lane = lane_id();
    BatchCounters *C = P.ctr;
    const float fg = (float)P.granularity;
    if (lane == 0) atomicCAS(&C->t0, 0ull, global_ns());
    int slot = -1;
    unsigned idle = 0;

    while (true) {
        // ---- time budget
        int timed_out = 0;
        if (lane == 0 && P.budget_ns) timed_out = global_ns() - *(volatile unsigned long long *)&C->t0 > P.budget_ns;
        timed_out = __shfl_sync(FULL, timed_out, 0);
        if (timed_out) {
            if (slot >= 0) {
                if (lane == 0) batch_finish(P, &P.slots[slot], P.slots[slot].query, PRRTC_ETIMEDOUT);
                __syncwarp();
                batch_leave<D>(P, slot, false);
            }
            return;
        }
        // ---- find work
        if (slot < 0) {
            int found = -1, admit = -1, rec = -1;
            if (lane == 0) {
                const unsigned s0 = atomicAdd((unsigned *)&C->cursor, 1u);
                for (int tries = 0; tries < P.num_slots && found < 0 && rec < 0; tries++) {
                    const int s = (int)((s0 + (unsigned)tries) % (unsigned)P.num_slots);
                    SlotState *S = &P.slots[s];
                    const int st = *(volatile int *)&S->state;
                    if (st == SLOT_RUNNING) {
                        atomicAdd(&S->workers, 1);
                        if (*(volatile int *)&S->state == SLOT_RUNNING) {
                            found = s;
                        } else {
                            rec = s;      // leave it again (possibly recycling it)
                        }
                    } else if (st == SLOT_FREE && *(volatile int *)&C->admit_next < P.num_queries) {
                        if (atomicCAS(&S->state, SLOT_FREE, SLOT_BUSY) == SLOT_FREE) {
                            const int qa = atomicAdd(&C->admit_next, 1);
                            if (qa < P.num_queries) {
                                atomicAdd(&S->workers, 1);
                                found = s;
                                admit = qa;
                            } else {
                                atomicExch(&S->state, SLOT_FREE);
                            }
                        }
                    }
                }
            }
            found = __shfl_sync(FULL, found, 0);
            admit = __shfl_sync(FULL, admit, 0);
            rec = __shfl_sync(FULL, rec, 0);
            if (rec >= 0) {
                if (batch_leave<D>(P, rec, true)) {
                    slot = rec;
                    idle = 0;
                }
                continue;
            }
            if (found < 0) {
                int all_done = 0;
                if (lane == 0) all_done = *(volatile int *)&C->done >= P.num_queries;
                if (__shfl_sync(FULL, all_done, 0)) return;
                if (++idle > (1u << 22)) {
                    if (lane == 0) atomicOr(&C->error, 1);
                    return;
                }
                __nanosleep(256);
                continue;
            }
            if (admit >= 0) batch_admit<D>(P, found, admit);
            slot = found;
            idle = 0;
        }

        // ---- one RRT-Connect iteration on `slot`
        SlotState *S = &P.slots[slot];
        const int q = *(volatile int *)&S->query;
        const BatchQueryDesc Qd = P.queries[q];
        CheckCtx ctx{{Qd.env, Qd.env_n}, P.pad, &W.bad};
        float *nodes_s = P.nodes + (size_t)slot * 2 * D * P.cap;
        int *par_s = P.parents + (size_t)slot * 2 * P.cap;
        float *rad_s = P.radii + (size_t)slot * 2 * P.cap;

        int k = 0;
        if (lane == 0) k = atomicAdd(&S->ticket, 1);
        k = __shfl_sync(FULL, k, 0);
        const int vl = k % P.lanes;
        const int iter = k / P.lanes + 1;
        if ((long long)k >= P.max_samples_drawn) {
            if (lane == 0) batch_finish(P, S, q, 0);
        } else {
            int t = 0;
            if (lane == 0) {
                volatile SlotState *vs = S;
                const int f0 = vs->free_index[0], f1 = vs->free_index[1];
                const int L = P.lanes;
                if (P.balance == 0 || iter == 1) {
                    t = (vl < (L / 2)) ? 0 : 1;
                } else if (P.balance == 1 && 2 * abs(f0 - f1) < 3 * L) {
                    const float ratio = f0 / (float)(f0 + f1);
                    t = ((float)vl < L * (1.0f - ratio)) ? 0 : 1;
                } else if (P.balance == 1) {
                    const float ratio = f0 / (float)(f0 + f1);
                    t = ratio < P.tree_ratio ? 0 : 1;
                } else {
                    int *ts = P.tsel + (size_t)slot * L + vl;
                    t = *(volatile int *)ts;
                    const int ft = t == 0 ? f0 : f1, fo = t == 0 ? f1 : f0;
                    const float ratio = abs(ft - fo) / (float)ft;
                    if (ratio < P.tree_ratio) t = 1 - t;
                    *ts = t;
                }
                if (P.balance == 2 && iter == 1) P.tsel[(size_t)slot * L + vl] = t;
            }
            t = __shfl_sync(FULL, t, 0);
            const int o = 1 - t;
            float *nd_t = nodes_s + (size_t)t * D * P.cap, *nd_o = nodes_s + (size_t)o * D * P.cap;
            int *pr_t = par_s + (size_t)t * P.cap;
            float *rd_t = rad_s + (size_t)t * P.cap;
            if (lane < D) {
                const float h = radical_inverse((unsigned)iter, (unsigned)P.halton_bases[vl * 16 + lane]);
                W.cfg[lane] = fmaf(h, P.scale[lane], P.offset[lane]);
            }
            __syncwarp();
            float qv[D];
#pragma unroll
            for (int d = 0; d < D; d++) qv[d] = W.cfg[d];
            float dsq;
            int ni;
            const int cnt_t = *(volatile int *)&S->free_index[t];
            warp_nn<D>(nd_t, P.cap, cnt_t, qv, dsq, ni);
            if (lane == 0) atomicAdd(&C->nn_nodes, (unsigned long long)min(cnt_t, P.cap));
            const float dist = sqrtf(dsq);
            const float scale = fminf(1.0f, P.range / dist);
            int skip = 0;
            if (lane == 0) skip = P.dynamic_domain && __ldcg(rd_t + ni) < dist;
            skip = __shfl_sync(FULL, skip, 0);
            if (!skip) {
                if (lane < D) {
                    const float nn = __ldcg(nd_t + (size_t)lane * P.cap + ni);
                    const float c = fmaf(W.cfg[lane] - nn, scale, nn);
                    W.nn[lane] = nn;
                    W.from[lane] = nn;
                    W.cfg[lane] = c;
                    W.step[lane] = __fdiv_rn(__fsub_rn(c, nn), fg);
                }
                __syncwarp();
                if (!warp_validate<Gen>(W, P.granularity, P.edge_order, ctx, C->work)) {
                    if (lane == 0 && P.dynamic_domain) dd_shrink(rd_t + ni, P.dd_alpha, P.dd_radius, P.dd_min_radius);
                } else {
                    int idx = -1;
                    if (lane == 0) {
                        idx = atomicAdd(&S->free_index[t], 1);
                        if (idx >= P.max_samples || idx >= P.cap) {
                            batch_finish(P, S, q, idx >= P.max_samples ? 0 : PRRTC_ENOMEM);
                            idx = -1;
                        } else {
                            pr_t[idx] = ni;
                            if (P.dynamic_domain) {
                                rd_t[idx] = FLT_MAX;
                                dd_grow(rd_t + ni, P.dd_alpha);
                            }
                        }
                    }
                    idx = __shfl_sync(FULL, idx, 0);
                    if (idx >= 0) {
                        if (lane < D) nd_t[(size_t)lane * P.cap + idx] = W.cfg[lane];
                        __threadfence();
                        __syncwarp();
                        // connect toward the other tree
#pragma unroll
                        for (int d = 0; d < D; d++) qv[d] = W.cfg[d];
                        int oi;
                        const int cnt_o = *(volatile int *)&S->free_index[o];
                        warp_nn<D>(nd_o, P.cap, cnt_o, qv, dsq, oi);
                        if (lane == 0) atomicAdd(&C->nn_nodes, (unsigned long long)min(cnt_o, P.cap));
                        const unsigned n_ext = (unsigned)ceilf(sqrtf(dsq) / P.range);
                        if (lane < D) W.vec[lane] = (__ldcg(nd_o + (size_t)lane * P.cap + oi) - W.cfg[lane]) / (float)n_ext;
                        __syncwarp();
                        unsigned i_ext = 0;
                        int parent = idx;
                        while (i_ext < n_ext) {
                            if (lane < D) {
                                const float a = W.cfg[lane];
                                const float b = a + W.vec[lane];
                                W.next[lane] = b;
                                W.from[lane] = a;
                                W.step[lane] = __fdiv_rn(__fsub_rn(b, a), fg);
                            }
                            __syncwarp();
                            if (!warp_validate<Gen>(W, P.granularity, P.edge_order, ctx, C->work)) break;
                            int idx2 = -1;
                            if (lane == 0) {
                                idx2 = atomicAdd(&S->free_index[t], 1);
                                if (idx2 >= P.max_samples || idx2 >= P.cap) {
                                    batch_finish(P, S, q, idx2 >= P.max_samples ? 0 : PRRTC_ENOMEM);
                                    idx2 = -1;
                                } else {
                                    pr_t[idx2] = parent;
                                    rd_t[idx2] = FLT_MAX;
                                }
                            }
                            idx2 = __shfl_sync(FULL, idx2, 0);
                            if (idx2 < 0) {
                                parent = -1;
                                break;
                            }
                            if (lane < D) {
                                W.cfg[lane] = W.next[lane];
                                nd_t[(size_t)lane * P.cap + idx2] = W.next[lane];
                            }
                            __threadfence();
                            __syncwarp();
                            parent = idx2;
                            i_ext++;
                        }
                        if (i_ext == n_ext && parent >= 0 && lane == 0) {
                            if (atomicCAS(&S->state, SLOT_RUNNING, SLOT_DONE) == SLOT_RUNNING) {
                                __threadfence();
                                batch_trace<D>(P, S, slot, q, t, parent, oi, iter);
                            }
                        }
                        __syncwarp();
                    }
                }
            }
        }
        // ---- leave a finished slot
        int st = 0;
        if (lane == 0) st = *(volatile int *)&S->state;
        st = __shfl_sync(FULL, st, 0);
        if (st != SLOT_RUNNING) {
            if (!batch_leave<D>(P, slot, true)) slot = -1;
        }
    }
}

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
        k_validate_edges<Gen><<<(int)blocks, threads, smem, st>>>(le.rec, le.counts, a, b, n, g, out, le.work);
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
        const size_t smem = sizeof(WarpScratch) * wpb;
        k_rrtc_batch<Gen><<<blocks, 32 * wpb, smem, st>>>(P);
        return cudaGetLastError();
    }
    static int batch_occupancy(int wpb)
    {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_rrtc_batch<Gen>, 32 * wpb, sizeof(WarpScratch) * wpb) !=
            cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return n;
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
        static constexpr unsigned kFkFlops = NS::kFkFlops;                                          \
        template <class Ctx>                                                                        \
        static __device__ __forceinline__ bool fkcc(const float *q, Ctx &ctx)                       \
        {                                                                                           \
            return NS::fkcc(q, ctx);                                                                \
        }                                                                                           \
        static __device__ __forceinline__ void fk_spheres(const float *q, float4 *out)              \
        {                                                                                           \
            NS::fk_spheres(q, out);                                                                 \
        }                                                                                           \
    };                                                                                              \
    }
