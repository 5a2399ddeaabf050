// Batched form of the planner: many queries, one persistent launch.
//
// Every warp is an independent worker.  A slot holds one *attempt* at a query:
// its own pair of trees in the arena and its own sample stream.  A worker
// joins a running slot and runs RRT-Connect iterations there until the slot
// ends, then moves to the next running slot (round-robin cursor), so the warps
// of finished queries are stolen by unfinished ones.  The last warp to leave
// an ended slot scrubs its arena region back to NaN and reuses the slot:
// restarting the query (if its only attempt ran out of samples or arena) or
// admitting the next pending query.  When no query is pending, idle warps open
// extra attempts of long-running queries in free slots: RRT-Connect's run
// time is heavy-tailed in narrow passages, and the first of several
// independent attempts to connect ends the query (the others are cancelled).
//
// Sampling follows the reference's lanes virtually: sample k of an attempt is
// Halton point k / L + 1 of virtual lane k % L (pRRTC.cu:81-105), with that
// lane's prime bases (sampler 0: the reference's per-block shuffled bases,
// offset by L lanes per attempt) or per-(query, attempt) digit-scrambled bases
// (sampler 1).  The balance modes see the virtual lane as pRRTC sees
// blockIdx.x.
#pragma once

#include "device_common.cuh"
#include "planner_device.cuh"
#include "prrtc_internal.h"

namespace prrtc {

// Per-warp shared scratch of the batched planner, followed in shared memory
// by the obstacle records of the query the warp works on: room for the
// batch's largest environment (BatchParams::env_records, at most
// kWarpEnvRecords); queries with larger scenes read theirs from global
// memory through L1.
template <int D>
struct alignas(16) WarpScratch {
    static constexpr int kPairQuads = (D + 1) / 2;              // float4 holding a staged node pair
    static constexpr int kPairStride = kPairQuads | 1;         // odd: staging stores conflict at most 2-way
    static constexpr int kTreeQuads = 16 * kPairStride + 1;    // per tree (+1: the trees' pairs in other banks)
    union {
        // early rejection: the first coordinates of the staged nodes (+1: bank skew)
        float chunk[D][33];
        // the nearest-node pass: 32 nodes of each tree as 16 node pairs, pair p
        // of tree t at nnp[t * kTreeQuads + p * kPairStride + k], k < kPairQuads,
        // holding (x_2k of node 2p, of node 2p + 1, x_2k+1 of node 2p, of node 2p + 1)
        float4 nnp[2 * kTreeQuads];
    };
    float from[D], step[D], cfg[D], nn[D], vec[D], next[D];
    float rad2[32];        // early rejection: the staged nodes' squared widened domain radii
    float box_lo[8], box_hi[8];   // and the box around all their domains
    unsigned hsh[16];      // scrambled sampler: the hash of (query, attempt, dimension)
    // the round's samples that survive the dynamic-domain test, per lane:
    // coordinates, tree, nearest node, Halton iteration and distance (kept
    // here rather than in registers across the edge checks)
    float pend_q[D][32];
    int pend_t[32], pend_i[32], pend_it[32];
    float pend_d[32];
    unsigned long long env_bar;   // mbarrier of the bulk copies that stage the obstacle records
    int bad;
};

// A warp's shared memory: its WarpScratch, then room for env_records
// obstacle records, then (with shared frames) the checker's frame area.
template <class Gen>
__host__ __device__ constexpr size_t warp_scratch_bytes(int env_records, bool shared_frames)
{
    return sizeof(WarpScratch<Gen::kDof>) + (size_t)env_records * sizeof(float4) +
           (shared_frames ? shared_frame_bytes(Gen::kFrames) : 0);
}

// Exact early rejection of dynamic-domain samples.  When every lane of a
// round samples the same tree and it has at most 32 nodes (a trapped tree
// rejects all but ~1e-4 of its samples), the nodes are staged with their
// domain radii widened by kEarlyRel and kEarlyAbs (float rounding of the
// full test stays far inside that), and the digit loops stop after
// kEarlyTrips trips: each coordinate of the first dimension group is then
// known to an interval.  A lane whose interval box is outside every widened
// domain would be rejected by the full test whatever its remaining digits
// are; when that holds for every lane, the warp skips the rest of the
// round.  Otherwise the digit loops continue from where they stopped, so
// samples and decisions are the same as without the test.  The nodes are
// staged every round, as the full test reads them; a tree of more than
// kEarlyBox nodes also gets the box around all its domains as a first test.
constexpr int kEarlyTrips = 4;
constexpr float kEarlyRel = 1.0f / 1024.0f, kEarlyAbs = 1.0f / 65536.0f;
constexpr int kEarlyBox = 8;

// warps an attempt admits: kJoinBase for its first kJoinYoungNs, then up to
// max_workers
constexpr int kJoinBase = 4;
constexpr unsigned long long kJoinYoungNs = 200000;

// whole warp: stage the first G coordinates and the widened radii of the
// tree's first cnt (<= 32) nodes and, above kEarlyBox nodes, the box around
// their domains.  A node with a NaN coordinate or radius (an insertion in
// flight) makes the box unbounded in that dimension.
template <int G, class WS>
__device__ __forceinline__ void stage_domains(WS &W, const float *nd, const float *rd, int cap, int cnt)
{
    const int lane = lane_id();
    const bool have = lane < cnt;
    const float r = have ? __ldcg(rd + lane) : 0.0f;
    const float m = fmaf(r, 1.0f + kEarlyRel, kEarlyAbs);
    W.rad2[lane] = m * m;
#pragma unroll
    for (int j = 0; j < G; j++) {
        const float c = have ? __ldcg(nd + (size_t)j * cap + lane) : 0.0f;
        W.chunk[j][lane] = c;
        if (cnt <= kEarlyBox) continue;
        float lo = c - m, hi = c + m;
        if (!have) {
            lo = INFINITY;
            hi = -INFINITY;
        } else if (!(lo == lo) || !(hi == hi)) {
            lo = -INFINITY;
            hi = INFINITY;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, off));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, off));
        }
        if (lane == 0) {
            W.box_lo[j] = lo;
            W.box_hi[j] = hi;
        }
    }
    __syncwarp();
}

// one lane: can the sample whose first G coordinates are being digitised in
// r still land in a staged domain?  The digits to come add less than
// f * b to h (nothing once idx is 0), plus at most 2^-20 of rounding over
// the remaining fmaf steps; the scrambled sampler's rotation keeps an
// interval unless it wraps past 1.  Coordinates are fmaf(v, scale, offset),
// monotone in v.  A NaN anywhere answers yes.
template <int G, bool SCRAMBLE, class WS>
__device__ __forceinline__ bool early_near(const RadicalDigits<G, SCRAMBLE> &r, const unsigned (&hsh)[G],
                                           const BatchParams &P, const WS &W, int cnt)
{
    float lo[G], hi[G];
    bool in_box = true;
#pragma unroll
    for (int j = 0; j < G; j++) {
        const float w = r.idx[j] ? fmaf(r.f[j] * (float)r.b[j], 1.0f + kEarlyRel, 1.0f / 1048576.0f) : 0.0f;
        float vlo = r.h[j], vhi = r.h[j] + w;
        if (SCRAMBLE) {
            const float rot = (float)(hsh[j] >> 8) * (1.0f / 16777216.0f);
            vlo += rot;
            vhi += rot;
            if (vlo >= 1.0f) {
                vlo -= 1.0f;
                vhi -= 1.0f;
            } else if (vhi >= 1.0f) {
                vlo = 0.0f;
                vhi = 1.0f;
            }
        }
        const float qa = fmaf(vlo, P.scale[j], P.offset[j]), qb = fmaf(vhi, P.scale[j], P.offset[j]);
        lo[j] = fminf(qa, qb);
        hi[j] = fmaxf(qa, qb);
        if (cnt > kEarlyBox) in_box = in_box && !(hi[j] < W.box_lo[j] || lo[j] > W.box_hi[j]);
    }
    bool near = false;
    if (in_box) {
        for (int n = 0; n < cnt && !near; n++) {
            float acc = 0.0f;
#pragma unroll
            for (int j = 0; j < G; j++) {
                const float c = W.chunk[j][n];
                const float g = fmaxf(fmaxf(c - hi[j], lo[j] - c), 0.0f);
                acc = fmaf(g, g, acc);
            }
            near = !(acc > W.rad2[n]);
        }
    }
    return near;
}

// whole warp: the coordinates d0 .. d0 + G - 1 of every lane's sample into
// qv.  With `early` (first group only), returns true when the early test
// rejected every lane's sample; qv is then incomplete.
template <int D, int G, bool SCRAMBLE>
__device__ __forceinline__ bool sample_group(const BatchParams &P, const WarpScratch<D> &W, unsigned iter, int d0,
                                             const unsigned (&bs)[G], const unsigned (&as)[G],
                                             const unsigned (&hsh)[G], bool early, int cnt, bool valid, float (&qv)[D])
{
    RadicalDigits<G, SCRAMBLE> r(iter, bs, as);
    if (early) {
        r.run(kEarlyTrips);
        const bool near = valid && early_near<G, SCRAMBLE, WarpScratch<D>>(r, hsh, P, W, cnt);
        if (!__any_sync(0xffffffffu, near)) return true;
    }
    r.finish();
#pragma unroll
    for (int j = 0; j < G; j++) {
        const int d = d0 + j;
        if (d < D) {
            float h = r.h[j];
            if (SCRAMBLE) {
                h += (float)(hsh[j] >> 8) * (1.0f / 16777216.0f);
                h -= floorf(h);
            }
            qv[d] = fmaf(h, P.scale[d], P.offset[d]);
        }
    }
    return false;
}

// Whole warp: check the g points of the edge in W (from + k * step),
// k = 1..g, in ceil(g / 32) rounds of one point per lane.  Contiguous order
// gives round r the points 32 r + lane + 1; interleaved order gives it
// lane * R + r + 1, so the first round already samples the whole edge at
// stride R.  Adds the work done to work[0] (FLOPs) and work[1] (points).
template <class Gen, class Ctx>
__device__ __forceinline__ bool warp_validate(const WarpScratch<Gen::kDof> &W, int g, int interleave, Ctx &ctx,
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

__device__ __forceinline__ int vload(const int *p) { return *(const volatile int *)p; }

// lane 0: count a finished query.  The one that completes 99 % of the batch
// records the time and the work counters at that moment, so the host can
// report the launch's bulk apart from its tail.
__device__ __forceinline__ void count_done(const BatchParams &P, unsigned long long t)
{
    const int k = atomicAdd(&P.ctr->done, 1) + 1;
    if (k == (P.num_queries * 99 + 99) / 100) {
        P.ctr->t99 = t;
        P.ctr->work99[0] = *(volatile unsigned long long *)&P.ctr->work[0];
        P.ctr->work99[1] = *(volatile unsigned long long *)&P.ctr->work[1];
    }
}

// lane 0: publish an unsolved query's result (first caller wins)
__device__ __forceinline__ void finish_query_unsolved(const BatchParams &P, const SlotState *S, int q, int status)
{
    if (atomicCAS(&P.qstate[q].state, 1, 2) != 1) return;
    BatchOut &o = P.out[q];
    const volatile SlotState *vs = S;
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
    count_done(P, o.t_done);
}

// lane 0: end the attempt in slot S unsolved (first caller wins).  The last
// live attempt of a query either asks for a restart in this slot or, when the
// query has used its attempts (or on timeout), publishes it as unsolved.
__device__ __forceinline__ void finish_attempt(const BatchParams &P, SlotState *S, int q, int status)
{
    if (atomicCAS(&S->state, SLOT_RUNNING, SLOT_DONE) != SLOT_RUNNING) return;
    const int live = atomicSub(&P.qstate[q].live, 1) - 1;
    if (status == PRRTC_ETIMEDOUT) {
        finish_query_unsolved(P, S, q, status);
        return;
    }
    if (live == 0 && vload(&P.qstate[q].state) == 1) {
        if (vload(&P.qstate[q].attempts) < P.max_attempts)
            S->restart = 1;
        else
            finish_query_unsolved(P, S, q, status);
    }
}

// lane 0: walk a tree from `start` to its root; returns the node count
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

// lane 0, after winning the query: trace the solution into the path pool in
// the reference's order (goal, goal-tree segment toward the junction,
// start-tree segment, start; pRRTC.cu:731-741) and publish the result.
template <int D>
__device__ void batch_trace(const BatchParams &P, const SlotState *S, int s, int q, int t, int jt, int jo, int iter)
{
    const float *nodes_s = P.nodes + (size_t)s * 2 * D * P.cap;
    const int *par_s = P.parents + (size_t)s * 2 * P.cap;
    const int o = 1 - t;
    const int j0 = t == 0 ? jt : jo, j1 = t == 0 ? jo : jt;
    int r0 = 0, r1 = 0;
    const int n0 = chain_length<D>(par_s, P.cap, j0, &r0);
    const int n1 = chain_length<D>(par_s + P.cap, P.cap, j1, &r1);
    BatchOut &out = P.out[q];
    const volatile SlotState *vs = S;
    out.solved = 1;
    out.iters = iter;
    out.reached_goal = r1;
    out.start_tree_size = min(vs->free_index[0], P.cap);
    out.goal_tree_size = min(vs->free_index[1], P.cap);
    out.samples = vs->ticket;
    out.path_rows = 0;
    out.status = PRRTC_ENOMEM;
    if (n0 >= 0 && n1 >= 0) {
        const int rows = n0 + n1 + 2;
        const int off = atomicAdd(&P.ctr->path_next, rows);
        const bool fits = off + rows <= P.path_pool_rows;
        // cost in the reference's order: the connecting tree first, then the other
        float cost = 0.0f;
        for (int pass = 0; pass < 2; pass++) {
            const int tree = pass == 0 ? t : o;
            const float *nd = nodes_s + (size_t)tree * D * P.cap;
            const int *pr = par_s + (size_t)tree * P.cap;
            int cur = tree == 0 ? j0 : j1;
            const int n = tree == 0 ? n0 : n1;
            for (int i = 0; i < n; i++) {
                const int par = vload(pr + cur);
                float acc = 0.0f;
                const int row = tree == 0 ? off + n1 + 1 + i : off + n1 - i;
#pragma unroll
                for (int d = 0; d < D; d++) {
                    const float a = __ldcg(nd + (size_t)d * P.cap + cur);
                    const float b = __ldcg(nd + (size_t)d * P.cap + par);
                    const float df = a - b;
                    acc = fmaf(df, df, acc);
                    if (fits) P.path_pool[(size_t)row * D + d] = a;
                }
                cost += sqrtf(acc);
                cur = par;
            }
        }
        out.cost = cost;
        out.path_length = n0 + n1;
        if (fits) {
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
        }
    }
    out.t_done = global_ns();
    __threadfence();
    count_done(P, out.t_done);
}

// whole warp: write query qa's roots into slot s as attempt `attempt` and start it
template <int D>
__device__ void batch_admit(const BatchParams &P, int s, int qa, int attempt)
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
        SlotState *S = &P.slots[s];
        S->query = qa;
        S->attempt = attempt;
        S->restart = 0;
        S->t_start = global_ns();
        S->free_index[0] = 1;
        S->free_index[1] = Q.num_goals;
        S->ticket = 0;
    }
    __threadfence();
    __syncwarp();
    if (lane == 0) atomicExch(&P.slots[s].state, SLOT_RUNNING);
}

// lane 0: a new query's first attempt
__device__ __forceinline__ void open_query(const BatchParams &P, int qa)
{
    QueryState &qs = P.qstate[qa];
    qs.attempts = 1;
    qs.live = 1;
    qs.t_first = global_ns();
    P.out[qa].t_admit = qs.t_first;
    __threadfence();
    atomicExch(&qs.state, 1);
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

// whole warp: leave slot s.  The last warp out of an ended slot scrubs it and
// reuses it: a restart of its query if one was asked for, else the next
// pending query.  Returns true when this warp now works on the reused slot.
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
    int qa = -1, att = 0;
    if (lane == 0 && allow_admit) {
        SlotState *S = &P.slots[s];
        const int q = S->query;
        if (S->restart && vload(&P.qstate[q].state) == 1) {
            att = atomicAdd(&P.qstate[q].attempts, 1);
            if (att < P.max_attempts) {
                atomicAdd(&P.qstate[q].live, 1);
                atomicAdd(&P.ctr->attempts, 1);
                qa = q;
            } else if (vload(&P.qstate[q].live) == 0) {
                finish_query_unsolved(P, S, q, 0);
            }
        }
        if (qa < 0 && s < P.admit_slots && vload(&P.ctr->admit_next) < P.num_queries) {
            qa = atomicAdd(&P.ctr->admit_next, 1);
            if (qa >= P.num_queries) {
                qa = -1;
            } else {
                if (P.order) qa = P.order[qa];
                att = 0;
                open_query(P, qa);
            }
        }
        if (qa >= 0) atomicAdd(&S->workers, 1);
    }
    qa = __shfl_sync(0xffffffffu, qa, 0);
    att = __shfl_sync(0xffffffffu, att, 0);
    if (qa >= 0) {
        batch_admit<D>(P, s, qa, att);
        return true;
    }
    if (lane == 0) atomicExch(&P.slots[s].state, SLOT_FREE);
    return false;
}

// whole warp: a running query that may get one more attempt, scanning from
// `from`; -1 if none.  A query qualifies after running k x restart_after_ns
// with k attempts, or at once when `forced` (every running attempt is at its
// worker cap, so an idle warp would otherwise wait).
__device__ __forceinline__ int spawn_candidate(const BatchParams &P, unsigned from, unsigned long long now,
                                               bool forced)
{
    for (int base = 0; base < P.num_queries; base += 32) {
        const int q = (int)((from + (unsigned)base + (unsigned)lane_id()) % (unsigned)P.num_queries);
        bool ok = false;
        if (base + lane_id() < P.num_queries) {
            const QueryState &qs = P.qstate[q];
            const int a = vload(&qs.attempts);
            ok = vload(&qs.state) == 1 && a < P.max_attempts &&
                 (forced ||
                  now - *(const volatile unsigned long long *)&qs.t_first > P.restart_after_ns * (unsigned long long)a);
        }
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (m) return __shfl_sync(0xffffffffu, q, __ffs(m) - 1);
    }
    return -1;
}

template <class Gen>
__global__ void __launch_bounds__(128) k_rrtc_batch(const BatchParams P)
{
    constexpr int D = Gen::kDof;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ float4 s_raw[];
    char *const warp_smem =
        reinterpret_cast<char *>(s_raw) + (threadIdx.x >> 5) * warp_scratch_bytes<Gen>(P.env_records, P.shared_frames);
    WarpScratch<D> &W = *reinterpret_cast<WarpScratch<D> *>(warp_smem);
    float4 *const W_env = reinterpret_cast<float4 *>(warp_smem + sizeof(WarpScratch<D>));
    float4 *const W_frames = W_env + P.env_records;   // the checker's frames (shared_frames)
    const int lane = lane_id();
    BatchCounters *C = P.ctr;
    const float fg = (float)P.granularity;
    unsigned long long t_launch = 0;   // lane 0: the launch's start (the first warp's clock)
    if (lane == 0) {
        const unsigned long long now = global_ns();
        const unsigned long long first = atomicCAS(&C->t0, 0ull, now);
        t_launch = first ? first : now;
    }
    int slot = -1;
    int cq = 0, catt = 0;   // the slot's query and attempt, read when this warp takes the slot
    bool fresh = true;
    bool trapped = false;   // this warp's last round on its slot was rejected early in full
    unsigned idle = 0;
    const float4 *staged = nullptr;   // the global records now in W_env
    const unsigned env_bar = (unsigned)__cvta_generic_to_shared(&W.env_bar);
    unsigned env_phase = 0;           // parity of W.env_bar's next phase
    if (lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(env_bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    unsigned long long nn_visits = 0;   // flushed once per warp (a shared counter would serialise)
    auto flush = [&]() {
        if (lane == 0 && nn_visits) atomicAdd(&C->nn_nodes, nn_visits);
        nn_visits = 0;
    };

    while (true) {
        // ---- time budget
        int timed_out = 0;
        if (lane == 0 && P.budget_ns) timed_out = global_ns() - t_launch > P.budget_ns;
        timed_out = __shfl_sync(FULL, timed_out, 0);
        if (timed_out) {
            if (slot >= 0) {
                if (lane == 0) finish_attempt(P, &P.slots[slot], P.slots[slot].query, PRRTC_ETIMEDOUT);
                __syncwarp();
                batch_leave<D>(P, slot, false);
            }
            flush();
            return;
        }
        // ---- find work: a pending query, else a running attempt with room for
        // another warp; in the tail, free slots become extra attempts
        if (slot < 0) {
            int found = -1, admit = -1, rec = -1, free_slot = -1, free_cand = -1, joinable = 0;
            unsigned s0 = 0;
            if (lane == 0) {
                s0 = atomicAdd((unsigned *)&C->cursor, 1u);
                const bool pending = vload(&C->admit_next) < P.num_queries;
                const unsigned long long now = global_ns();
                for (int tries = 0; tries < P.num_slots; tries++) {
                    const int s = (int)((s0 + (unsigned)tries) % (unsigned)P.num_slots);
                    SlotState *S = &P.slots[s];
                    const int st = vload(&S->state);
                    if (st == SLOT_FREE && pending && s < P.admit_slots) {
                        if (atomicCAS(&S->state, SLOT_FREE, SLOT_BUSY) != SLOT_FREE) continue;
                        int qa = atomicAdd(&C->admit_next, 1);
                        if (qa < P.num_queries) {
                            if (P.order) qa = P.order[qa];
                            open_query(P, qa);
                            atomicAdd(&S->workers, 1);
                            found = s;
                            admit = qa;
                            break;
                        }
                        atomicExch(&S->state, SLOT_FREE);
                    } else if (st == SLOT_FREE && free_cand < 0 && P.max_attempts > 1 && !pending) {
                        free_cand = s;   // claimed below, only if there is nothing to join
                    } else if (st == SLOT_RUNNING) {
                        const int w = vload(&S->workers);
                        if (w >= P.max_workers) continue;
                        // a young attempt takes few warps: idle warps that all join
                        // it at once (the tail of a stream) see two small trees,
                        // send half their samples to the free one, and its connect
                        // steps fill the arena.  It counts as joinable all the same
                        // (the warp waits for it instead of forcing another attempt).
                        if (w >= kJoinBase &&
                            now - *(const volatile unsigned long long *)&S->t_start < kJoinYoungNs) {
                            joinable = 1;
                            continue;
                        }
                        joinable = 1;
                        atomicAdd(&S->workers, 1);
                        if (vload(&S->state) == SLOT_RUNNING)
                            found = s;
                        else
                            rec = s;        // leave it again (possibly recycling it)
                        break;
                    }
                }
                if (free_cand >= 0 && found < 0 && rec < 0 &&
                    atomicCAS(&P.slots[free_cand].state, SLOT_FREE, SLOT_BUSY) == SLOT_FREE)
                    free_slot = free_cand;
            }
            found = __shfl_sync(FULL, found, 0);
            admit = __shfl_sync(FULL, admit, 0);
            rec = __shfl_sync(FULL, rec, 0);
            free_slot = __shfl_sync(FULL, free_slot, 0);
            joinable = __shfl_sync(FULL, joinable, 0);
            s0 = __shfl_sync(FULL, s0, 0);
            if (free_slot >= 0) {
                // nothing to join: an extra attempt of a running query
                const int qc = spawn_candidate(P, s0 * 7919u, global_ns(), !joinable);
                int att = -1;
                if (lane == 0) {
                    if (qc >= 0) {
                        att = atomicAdd(&P.qstate[qc].attempts, 1);
                        if (att < P.max_attempts && vload(&P.qstate[qc].state) == 1) {
                            atomicAdd(&P.qstate[qc].live, 1);
                            atomicAdd(&C->attempts, 1);
                            atomicAdd(&P.slots[free_slot].workers, 1);
                        } else {
                            att = -1;
                        }
                    }
                    if (att < 0) atomicExch(&P.slots[free_slot].state, SLOT_FREE);
                }
                att = __shfl_sync(FULL, att, 0);
                if (att >= 0) {
                    batch_admit<D>(P, free_slot, qc, att);
                    slot = free_slot;
                    fresh = true;
                    idle = 0;
                    continue;
                }
            }
            if (rec >= 0) {
                if (batch_leave<D>(P, rec, true)) {
                    slot = rec;
                    fresh = true;
                    idle = 0;
                }
                continue;
            }
            if (found < 0) {
                int all_done = 0;
                if (lane == 0) all_done = vload(&C->done) >= P.num_queries;
                if (__shfl_sync(FULL, all_done, 0)) {
                    flush();
                    return;
                }
                if (++idle > P.idle_limit) {
                    if (lane == 0) atomicOr(&C->error, 1);
                    flush();
                    return;
                }
                __nanosleep(256);
                continue;
            }
            if (admit >= 0) batch_admit<D>(P, found, admit, 0);
            slot = found;
            fresh = true;
            idle = 0;
        }

        // ---- one round of up to 32 samples on `slot`: every lane draws a
        // sample, one shared pass over each tree finds all their nearest
        // nodes, and the samples that pass the dynamic-domain test are then
        // extended one at a time by the whole warp (32 of pRRTC's lanes
        // reading one tree snapshot, pRRTC.cu:378-427)
        // The slot's query and attempt stay fixed while this warp works on it (a
        // slot is reused only after its last worker has left).
        SlotState *S = &P.slots[slot];
        if (fresh) {
            if (lane == 0) {
                cq = vload(&S->query);
                catt = vload(&S->attempt);
            }
            cq = __shfl_sync(FULL, cq, 0);
            catt = __shfl_sync(FULL, catt, 0);
            // scrambled Halton: digit multiplier and rotation per (query, attempt, dimension)
            if (lane < 16)
                W.hsh[lane] = hash32((unsigned)cq * 0x9E3779B1u + (unsigned)catt * 0xC2B2AE35u +
                                     (unsigned)lane * 0x85EBCA77u + 0x165667B1u);
            __syncwarp();
            fresh = false;
            trapped = false;
        }
        const int q = cq, attempt = catt;
        const BatchQueryDesc Qd = P.queries[q];
        const float4 *envp = Qd.env;
        if (Qd.env_n.records() <= P.env_records) {
            if (staged != Qd.env) {   // the records are read-only for the whole launch
                // one bulk copy by the TMA engine into the warp's area, completed
                // on the warp's mbarrier (after a proxy fence: the area was last
                // read by the checker's ordinary loads); the wait is bounded, a
                // plain copy of the same bytes behind it
                __syncwarp();
                const unsigned bytes = (unsigned)Qd.env_n.records() * 16u;
                if (bytes) {
                    if (lane == 0) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(env_bar),
                                     "r"(bytes)
                                     : "memory");
                        asm volatile(
                            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                                (unsigned)__cvta_generic_to_shared(W_env)),
                            "l"(Qd.env), "r"(bytes), "r"(env_bar)
                            : "memory");
                    }
                    bool done = false;
                    for (int i = 0; i < kBulkPolls && !done; i++) done = bulk_phase_done(env_bar, env_phase);
                    env_phase ^= 1u;
                    if (!__all_sync(FULL, done))
                        for (int i = lane; i < Qd.env_n.records(); i += 32) W_env[i] = __ldg(Qd.env + i);
                }
                __syncwarp();
                staged = Qd.env;
            }
            envp = W_env;
        }
        CheckCtx ctx{{envp, Qd.env_n}, P.pad, &W.bad};
        SharedCheckCtx sctx{ctx, W_frames + lane};
        // every point of an edge through the robot's checker, frames where P says
        auto validate = [&]() {
            return P.shared_frames ? warp_validate<Gen>(W, P.granularity, P.edge_order, sctx, C->work)
                                   : warp_validate<Gen>(W, P.granularity, P.edge_order, ctx, C->work);
        };
        float *nodes_s = P.nodes + (size_t)slot * 2 * D * P.cap;
        int *par_s = P.parents + (size_t)slot * 2 * P.cap;
        float *rad_s = P.radii + (size_t)slot * 2 * P.cap;

        // the round's shared state in one batch of independent loads: the slot's
        // and the query's states, the tree sizes and the round's sample
        // tickets (taken even when the attempt turns out to have ended: a
        // ticket is only a count).  A warp whose last round here was rejected
        // early in full takes tickets for P.sub_rounds batches at once, so the
        // warps sampling a trapped attempt share one atomic per sub_rounds x 32
        // samples; tickets a round does not use are skipped samples.
        const int take = trapped ? 32 * P.sub_rounds : 32;
        int k0 = 0, sst = 0, qst = 0, f0 = 0, f1 = 0;
        if (lane == 0) {
            sst = vload(&S->state);
            qst = vload(&P.qstate[q].state);
            f0 = vload(&S->free_index[0]);
            f1 = vload(&S->free_index[1]);
            k0 = atomicAdd(&S->ticket, take);
        }
        sst = __shfl_sync(FULL, sst, 0);
        qst = __shfl_sync(FULL, qst, 0);
        k0 = __shfl_sync(FULL, k0, 0);
        f0 = __shfl_sync(FULL, f0, 0);
        f1 = __shfl_sync(FULL, f1, 0);
        if (sst != SLOT_RUNNING) {
            // the attempt has ended (solved, failed or cancelled): leave the
            // slot, possibly taking it over for a restart or the next query
            if (batch_leave<D>(P, slot, true))
                fresh = true;
            else
                slot = -1;
            continue;
        }
        if (qst == 2) {
            // another attempt finished the query: cancel this one
            if (lane == 0 && atomicCAS(&S->state, SLOT_RUNNING, SLOT_DONE) == SLOT_RUNNING)
                atomicSub(&P.qstate[q].live, 1);
            continue;
        }
        if ((long long)k0 >= P.max_samples_drawn) {
            if (lane == 0) finish_attempt(P, S, q, 0);
            continue;
        }
        {
            // -- this lane's sample.  While every lane's sample is rejected by
            // the early test, the warp draws up to P.sub_rounds batches of 32
            // under one round header: the next 32 tickets, the same tree sizes
            // and, while the lanes keep choosing the same tree, the same
            // staged domains (32 more of pRRTC's lanes reading one snapshot)
            int k, vl, iter, t, t0, cnt0;
            bool valid, early, rejected = false;
            float qv[D];
            constexpr int NG = (D + 6) / 7, G = (D + NG - 1) / NG;
            static_assert(G <= 7, "dimension groups of at most 7");
            int staged_t = -1;
            // a lane count that is a power of two divides by a shift
            const int lshift = (P.lanes & (P.lanes - 1)) == 0 ? __ffs(P.lanes) - 1 : -1;
            for (int sub = 0;; sub++) {
                k = k0 + lane;
                valid = (long long)k < P.max_samples_drawn;
                if (lshift >= 0) {
                    vl = k & (P.lanes - 1);
                    iter = (k >> lshift) + 1;
                } else {
                    vl = k % P.lanes;
                    iter = k / P.lanes + 1;
                }
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
                    // vamp balance (pRRTC.cu:364-371): a lane swaps trees unless the
                    // other is much larger.  The lane's previous tree is taken as
                    // alternating from its first choice, so no per-lane state is
                    // shared by the warps working on the attempt.
                    const int prev = ((iter - 1) + (vl < (L / 2) ? 0 : 1)) & 1;
                    const int ft = prev == 0 ? f0 : f1, fo = prev == 0 ? f1 : f0;
                    const float ratio = abs(ft - fo) / (float)ft;
                    t = ratio < P.tree_ratio ? 1 - prev : prev;
                }
                // dimensions in ceil(D / 7) equal groups, each group's digit chains interleaved
                t0 = __shfl_sync(FULL, t, 0);
                cnt0 = min(t0 == 0 ? f0 : f1, P.cap);
                early = P.dynamic_domain && cnt0 <= 32 && __all_sync(FULL, t == t0);
                if (early && staged_t != t0) {
                    stage_domains<G>(W, nodes_s + (size_t)t0 * D * P.cap, rad_s + (size_t)t0 * P.cap, P.cap, cnt0);
                    staged_t = t0;
                }
                rejected = false;
#pragma unroll
                for (int d0 = 0; d0 < D; d0 += G) {
                    unsigned bs[G], as[G], hsh[G];
                    const int row = P.sampler == 0 ? (vl + attempt * P.lanes) % P.bases_lanes : vl % P.bases_lanes;
#pragma unroll
                    for (int j = 0; j < G; j++) {
                        const int d = d0 + j < D ? d0 + j : D - 1;   // a short last group repeats a dimension
                        bs[j] = (unsigned)P.halton_bases[row * 16 + d];
                        hsh[j] = P.sampler == 0 ? 0u : W.hsh[d];
                        as[j] = 1u + hsh[j] - div_by(hsh[j], kDivTable.magic[bs[j] - 1u]) * (bs[j] - 1u);
                    }
                    const bool e = early && d0 == 0;
                    const unsigned it = (unsigned)iter;
                    rejected = P.sampler == 0 ? sample_group<D, G, false>(P, W, it, d0, bs, as, hsh, e, cnt0, valid, qv)
                                              : sample_group<D, G, true>(P, W, it, d0, bs, as, hsh, e, cnt0, valid, qv);
                    if (rejected) break;
                }
                if (!rejected || sub + 1 >= P.sub_rounds) break;
                int k1 = k0 + 32;
                if (take == 32) {   // the first trapped round: the next tickets one batch at a time
                    if (lane == 0) k1 = atomicAdd(&S->ticket, 32);
                    k1 = __shfl_sync(FULL, k1, 0);
                }
                if ((long long)k1 >= P.max_samples_drawn) break;   // the next header ends the attempt
                k0 = k1;
            }
            trapped = rejected && P.sub_rounds > 1;
            if (!rejected) {
                // -- nearest node of every lane's sample: both trees in one pass,
                // 32 nodes of each staged per step in shared memory as node pairs;
                // a lane scans its own tree's chunk, two nodes per packed FP32
                // instruction (__fadd2_rn / __ffma2_rn: each half computes the
                // same operations as the scalar form, fsub then fmaf over the
                // dimensions in order), nodes in index order, so the nearest
                // node and its distance are the scalar scan's
                float best = FLT_MAX;
                int bi = 0;
                {
                    constexpr int PQ = WarpScratch<D>::kPairQuads, PS = WarpScratch<D>::kPairStride,
                                  TQ = WarpScratch<D>::kTreeQuads;
                    const bool act0 = __any_sync(FULL, valid && t == 0), act1 = __any_sync(FULL, valid && t == 1);
                    const int cnt0 = act0 ? min(f0, P.cap) : 0, cnt1 = act1 ? min(f1, P.cap) : 0;
                    const int cmax = max(cnt0, cnt1);
                    float2 nq[2 * PQ];   // -q twice per dimension (x - q == x + (-q) exactly)
#pragma unroll
                    for (int d = 0; d < 2 * PQ; d++) nq[d] = d < D ? make_float2(-qv[d], -qv[d]) : make_float2(0.0f, 0.0f);
                    const float4 *mine = W.nnp + (t == 0 ? 0 : TQ);
                    float *stage = reinterpret_cast<float *>(W.nnp + (lane >> 1) * PS) + (lane & 1);
                    const float qnan = __int_as_float(0x7FFFFFFF);
                    for (int base = 0; base < cmax; base += 32) {
                        const int i = base + lane;
#pragma unroll
                        for (int d = 0; d < D; d++) {
                            const int o = (d >> 1) * 4 + (d & 1) * 2;
                            stage[o] = i < cnt0 ? __ldcg(nodes_s + (size_t)d * P.cap + i) : qnan;
                            stage[4 * TQ + o] = i < cnt1 ? __ldcg(nodes_s + (size_t)(D + d) * P.cap + i) : qnan;
                        }
                        __syncwarp();
                        const int pairs = (min(32, cmax - base) + 1) >> 1;
                        for (int pr = 0; pr < pairs; pr++) {
                            const float4 *r = mine + pr * PS;
                            float2 a = make_float2(0.0f, 0.0f);
#pragma unroll
                            for (int k = 0; k < PQ; k++) {
                                const float4 v = r[k];
                                const float2 x0 = __fadd2_rn(make_float2(v.x, v.y), nq[2 * k]);
                                a = __ffma2_rn(x0, x0, a);
                                if (2 * k + 1 < D) {
                                    const float2 x1 = __fadd2_rn(make_float2(v.z, v.w), nq[2 * k + 1]);
                                    a = __ffma2_rn(x1, x1, a);
                                }
                            }
                            if (a.x < best) {
                                best = a.x;
                                bi = base + 2 * pr;
                            }
                            if (a.y < best) {
                                best = a.y;
                                bi = base + 2 * pr + 1;
                            }
                        }
                        __syncwarp();
                    }
                    nn_visits += (unsigned long long)cnt0 * __popc(__ballot_sync(FULL, valid && t == 0)) +
                                 (unsigned long long)cnt1 * __popc(__ballot_sync(FULL, valid && t == 1));
                }
                const float dist = sqrtf(best);
                bool go = valid;
                if (go && P.dynamic_domain) go = !(__ldcg(rad_s + (size_t)t * P.cap + bi) < dist);
                unsigned todo = __ballot_sync(FULL, go);
                if (go) {
#pragma unroll
                    for (int d = 0; d < D; d++) W.pend_q[d][lane] = qv[d];
                    W.pend_t[lane] = t;
                    W.pend_i[lane] = bi;
                    W.pend_it[lane] = iter;
                    W.pend_d[lane] = dist;
                }
                __syncwarp();

                // -- extend (and connect) each surviving sample, in lane order
                while (todo) {
                    const int j = __ffs(todo) - 1;
                    todo &= todo - 1;
                    const int tj = W.pend_t[j];
                    const int ni = W.pend_i[j];
                    const int iterj = W.pend_it[j];
                    const float distj = W.pend_d[j];
                    if (lane < D) W.cfg[lane] = W.pend_q[lane][j];
                    const int o = 1 - tj;
                    float *nd_t = nodes_s + (size_t)tj * D * P.cap, *nd_o = nodes_s + (size_t)o * D * P.cap;
                    int *pr_t = par_s + (size_t)tj * P.cap;
                    float *rd_t = rad_s + (size_t)tj * P.cap;
                    const float scale = fminf(1.0f, P.range / distj);
                    if (lane < D) {
                        const float nn = __ldcg(nd_t + (size_t)lane * P.cap + ni);
                        const float c = fmaf(W.cfg[lane] - nn, scale, nn);
                        W.nn[lane] = nn;
                        W.from[lane] = nn;
                        W.cfg[lane] = c;
                        W.step[lane] = __fdiv_rn(__fsub_rn(c, nn), fg);
                    }
                    __syncwarp();
                    if (!validate()) {
                        if (lane == 0 && P.dynamic_domain)
                            dd_shrink(rd_t + ni, P.dd_alpha, P.dd_radius, P.dd_min_radius);
                        continue;
                    }
                    int idx = -1;
                    if (lane == 0) {
                        idx = atomicAdd(&S->free_index[tj], 1);
                        if (idx >= P.max_samples || idx >= P.cap) {
                            finish_attempt(P, S, q, idx >= P.max_samples ? 0 : PRRTC_ENOMEM);
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
                    if (idx < 0) break;
                    if (lane < D) nd_t[(size_t)lane * P.cap + idx] = W.cfg[lane];
                    __threadfence();
                    __syncwarp();
                    // connect toward the other tree (pRRTC.cu:478-551)
                    float cq[D];
#pragma unroll
                    for (int d = 0; d < D; d++) cq[d] = W.cfg[d];
                    float dsq;
                    int oi;
                    const int cnt_o = vload(&S->free_index[o]);
                    warp_nn<D>(nd_o, P.cap, cnt_o, cq, dsq, oi);
                    nn_visits += (unsigned long long)min(cnt_o, P.cap);
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
                        if (!validate()) break;
                        int idx2 = -1;
                        if (lane == 0) {
                            idx2 = atomicAdd(&S->free_index[tj], 1);
                            if (idx2 >= P.max_samples || idx2 >= P.cap) {
                                finish_attempt(P, S, q, idx2 >= P.max_samples ? 0 : PRRTC_ENOMEM);
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
                        // connected: end the attempt, then the first attempt to
                        // win the query traces the path
                        if (atomicCAS(&S->state, SLOT_RUNNING, SLOT_DONE) == SLOT_RUNNING) {
                            atomicSub(&P.qstate[q].live, 1);
                            if (atomicCAS(&P.qstate[q].state, 1, 2) == 1) {
                                __threadfence();
                                batch_trace<D>(P, S, slot, q, tj, parent, oi, iterj);
                            }
                        }
                    }
                    __syncwarp();
                    // stop once the attempt has ended (solved here, or elsewhere)
                    int ended = 0;
                    if (lane == 0) ended = vload(&S->state) != SLOT_RUNNING;
                    if (__shfl_sync(FULL, ended, 0)) break;
                }
            }
        }
        // an attempt that ended in this round is left at the next round's start
    }
}

}  // namespace prrtc
