// Per-robot path smoothing by gradient descent on the clearance cost, judged
// by the robot's own collision checker.  Included from robot_kernels.cuh.
#pragma once

#include "clearance_device.cuh"
#include "planner_device.cuh"

namespace prrtc {

// Deterministic block sum (fixed blockDim, fixed order); every thread gets it.
__device__ __forceinline__ float block_sum(float v, float *s_red)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    float t = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_red[w];
    return t;
}

// One block per path.  First `shortcut_rounds` shortcut attempts: a span
// (i, j) of the path, chosen by a hash of (path, round), is replaced by evenly
// spaced points on the straight segment q_i -> q_j when every one of those
// sub-edges is free at granularity / 4 points (a quick filter; the judge below
// checks at full resolution).  Then the path stays in shared memory for all
// `steps` iterations of
//     q_w <- clamp(q_w - step * (cost_weight * dC/dq(q_w) + smooth_weight * (2 q_w - q_{w-1} - q_{w+1})))
// over the interior waypoints (the end points stay where they are).  The
// result is then checked edge by edge with the robot's checker at
// `granularity` points per edge (a + k ((b - a) / g), k = 1..g, as the
// planner interpolates); it is written back only if every point is free, so a
// rejected path is left exactly as it came in.
template <class Gen>
__global__ void __launch_bounds__(128) k_smooth_paths(const ClrLaunch P)
{
    constexpr int D = Gen::kDof;
    extern __shared__ float4 s_dyn[];
    __shared__ int s_bad;
    __shared__ float s_red[4];
    __shared__ unsigned long long s_bar;
    const int path = blockIdx.x;
    const int W = P.waypoints;
    const ClrEnv pe = P.envs[path];
    const int R = pe.n.records();
    float *s_q = reinterpret_cast<float *>(s_dyn + R);
    float *s_g = s_q + W * D;
    float *gq = P.q + (size_t)path * W * D;
    for (int i = threadIdx.x; i < W * D; i += blockDim.x) s_q[i] = gq[i];
    stage_env_bulk(s_dyn, pe.rec, R, &s_bar);   // synchronises the block
    const ClrEnv e{s_dyn, pe.n};
    const ClrSmooth s = P.s;
    CheckCtx ctx{EnvView{e.rec, e.n}, 0.0f, &s_bad};
    if (P.cost_before) {   // the cost of the path as given
        float cost = 0.0f;
        for (int w = threadIdx.x; w < W; w += blockDim.x) {
            float g[kClrMaxJoints];
            cost += clr::cost_grad(P.M, e, s_q + w * D, s.margin, s.cost_weight, g);
        }
        const float total = block_sum(cost, s_red);
        if (threadIdx.x == 0) P.cost_before[path] = total;
    }
    const int gs = max(1, s.granularity / 4);
    for (int r = 0; r < s.shortcut_rounds && W > 2; r++) {
        const unsigned h = hash32((unsigned)path * 0x9E3779B1u + (unsigned)r * 0x85EBCA77u + 0x27D4EB2Fu);
        const int span = 2 + (int)(h % (unsigned)min(W - 2, 31));   // 2 .. min(W - 1, 32) segments
        const int i0 = (int)((h >> 8) % (unsigned)(W - span));
        const float *qa = s_q + i0 * D, *qb = s_q + (i0 + span) * D;
        if (threadIdx.x == 0) s_bad = 0;
        __syncthreads();
        // sub-edge m runs from p_m to p_{m+1}, p_m = qa + (m / span) (qb - qa)
        for (int idx = threadIdx.x; idx < span * gs; idx += blockDim.x) {
            if (*(volatile int *)&s_bad) break;
            const int m = idx / gs, k = idx - m * gs + 1;
            float cfg[D];
#pragma unroll
            for (int d = 0; d < D; d++) {
                const float delta = qb[d] - qa[d];
                const float a = qa[d] + ((float)m / (float)span) * delta, b = qa[d] + ((float)(m + 1) / (float)span) * delta;
                cfg[d] = __fadd_rn(a, __fmul_rn((float)k, __fdiv_rn(__fsub_rn(b, a), (float)gs)));
            }
            ctx.work = 0;
            if (!Gen::fkcc(cfg, ctx)) s_bad = 1;
        }
        __syncthreads();
        if (s_bad == 0)
            for (int i = threadIdx.x; i < (span - 1) * D; i += blockDim.x) {
                const int m = i / D + 1, d = i - (m - 1) * D;
                s_q[(i0 + m) * D + d] = qa[d] + ((float)m / (float)span) * (qb[d] - qa[d]);
            }
        __syncthreads();
    }
    for (int it = 0; it <= s.steps; it++) {
        float cost = 0.0f;
        for (int w = threadIdx.x; w < W; w += blockDim.x) {
            float g[kClrMaxJoints];
            cost += clr::cost_grad(P.M, e, s_q + w * D, s.margin, s.cost_weight, g);
            if (w > 0 && w < W - 1)
#pragma unroll
                for (int d = 0; d < D; d++)
                    s_g[w * D + d] =
                        g[d] + s.smooth_weight * (2.0f * s_q[w * D + d] - s_q[(w - 1) * D + d] - s_q[(w + 1) * D + d]);
        }
        if (it == s.steps) {
            const float total = block_sum(cost, s_red);
            if (threadIdx.x == 0 && P.cost_after) P.cost_after[path] = total;
        }
        __syncthreads();
        if (it == s.steps) break;
        for (int i = threadIdx.x + D; i < (W - 1) * D; i += blockDim.x) {
            const int d = i % D;
            s_q[i] = fminf(fmaxf(s_q[i] - s.step * s_g[i], P.lo[d]), P.hi[d]);
        }
        __syncthreads();
    }
    // the judge: every edge at the planner's interpolation points
    if (threadIdx.x == 0) s_bad = 0;
    __syncthreads();
    const float fg = (float)s.granularity;
    const int total = (W - 1) * s.granularity;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        if (*(volatile int *)&s_bad) break;
        const int ed = idx / s.granularity, k = idx - ed * s.granularity + 1;
        const float *a = s_q + ed * D, *b = a + D;
        float cfg[D];
#pragma unroll
        for (int d = 0; d < D; d++) cfg[d] = __fadd_rn(a[d], __fmul_rn((float)k, __fdiv_rn(__fsub_rn(b[d], a[d]), fg)));
        ctx.work = 0;
        if (!Gen::fkcc(cfg, ctx)) s_bad = 1;
    }
    __syncthreads();
    const bool ok = s_bad == 0;
    if (ok)
        for (int i = threadIdx.x; i < W * D; i += blockDim.x) gq[i] = s_q[i];
    if (threadIdx.x == 0) P.accepted[path] = ok ? 1 : 0;
}

}  // namespace prrtc
