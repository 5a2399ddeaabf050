// Device pieces of the RRT-Connect planner shared by the plain (single-query,
// drop-in) form and the batched form: Halton sampling, the nearest-neighbour
// scan, dynamic-domain radius updates and path traceback.
//
// Trees are structure-of-arrays: coordinate d of node i of a tree lives at
// nodes[d * cap + i] (cap a multiple of 4, so a thread reads four nodes per
// 16-byte load).  Unwritten nodes hold NaN (the arena is filled with 0xFF
// bytes), so a node whose coordinates are not all visible yet yields a NaN
// distance, which never compares below the running minimum: the scan skips it
// without the reference's explicit sentinel test (pRRTC.cu:297-303,390).
#pragma once

#include <cfloat>
#include <cstdint>

#include "device_common.cuh"
#include "prrtc_internal.h"

namespace prrtc {

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// One step of the reference's incremental Halton recurrence for dimension
// count D (halton_next, pRRTC.cu:81-105), float32 exactly as written there.
template <int D>
__device__ __forceinline__ void halton_next(float *b, float *n, float *d, float *out)
{
#pragma unroll 1
    for (int i = 0; i < D; i++) {
        const float xf = d[i] - n[i];
        if (xf == 1.0f) {
            d[i] = floorf(d[i] * b[i]);
            n[i] = 1.0f;
        } else {
            float y = floorf(d[i] / b[i]);
            while (xf <= y) y = floorf(y / b[i]);
            n[i] = floorf((b[i] + 1.0f) * y) - xf;
        }
        out[i] = n[i] / d[i];
    }
}

// A raw Halton point scaled into the joint box as Robot::scale_cfg does
// (Robots.hh: q * s_m + s_a, one fused multiply-add per joint, as nvcc
// contracts it).
template <int D>
__device__ __forceinline__ void scale_sample(float *q, const float *scale, const float *offset)
{
#pragma unroll
    for (int d = 0; d < D; d++) q[d] = fmaf(q[d], scale[d], offset[d]);
}

// Block-wide nearest neighbour of s_q among the first `count` nodes of a tree.
// Squared L2 accumulated as the reference does (sq_l2_dist, utils.cuh:100-109).
// Ties resolve to the lowest node index.  Result in (s_out_d, s_out_i).
template <int D>
__device__ __forceinline__ void block_nn(const float *__restrict__ nodes, int cap, int count, const float *s_q,
                                         float *s_red_d, int *s_red_i, float *s_out_d, int *s_out_i)
{
    float q[D];
#pragma unroll
    for (int d = 0; d < D; d++) q[d] = s_q[d];
    float bd = FLT_MAX;
    int bi = 0x7fffffff;
    if (count > cap) count = cap;
    const int n4 = (count + 3) >> 2;
    const float4 *base = reinterpret_cast<const float4 *>(nodes);
    const int cap4 = cap >> 2;
    for (int c = threadIdx.x; c < n4; c += blockDim.x) {
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
#pragma unroll
        for (int d = 0; d < D; d++) {
            const float4 v = __ldcg(base + (size_t)d * cap4 + c);
            const float x0 = v.x - q[d], x1 = v.y - q[d], x2 = v.z - q[d], x3 = v.w - q[d];
            a0 = fmaf(x0, x0, a0);
            a1 = fmaf(x1, x1, a1);
            a2 = fmaf(x2, x2, a2);
            a3 = fmaf(x3, x3, a3);
        }
        const int i0 = 4 * c;
        if (a0 < bd) { bd = a0; bi = i0; }
        if (a1 < bd) { bd = a1; bi = i0 + 1; }
        if (a2 < bd) { bd = a2; bi = i0 + 2; }
        if (a3 < bd) { bd = a3; bi = i0 + 3; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float od = __shfl_xor_sync(0xffffffffu, bd, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (od < bd || (od == bd && oi < bi)) { bd = od; bi = oi; }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
        s_red_d[warp] = bd;
        s_red_i[warp] = bi;
    }
    __syncthreads();
    if (warp == 0) {
        bd = lane < nw ? s_red_d[lane] : FLT_MAX;
        bi = lane < nw ? s_red_i[lane] : 0x7fffffff;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float od = __shfl_xor_sync(0xffffffffu, bd, off);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (od < bd || (od == bd && oi < bi)) { bd = od; bi = oi; }
        }
        if (lane == 0) {
            *s_out_d = bd;
            *s_out_i = (bi == 0x7fffffff) ? 0 : bi;
        }
    }
    __syncthreads();
}

// Dynamic-domain updates with the reference's CAS loops (pRRTC.cu:456-468,
// 584-598): each update is computed from the radius it replaces.  A failed
// CAS returns the radius another update just wrote, which the next try
// starts from (no second read).  A shrink of a radius already at the floor
// (rmin) changes nothing and issues no CAS (trapped trees sit there).  A
// failed CAS means another update landed, so every update ends after at most
// as many retries as there are concurrent updaters; the loop is still
// bounded (kDdTries, far above any block or warp count the planners launch)
// so that no wait can be endless.
constexpr int kDdTries = 1 << 16;

__device__ __forceinline__ void dd_grow(float *r, float alpha)
{
    int *ri = reinterpret_cast<int *>(r);
    int cur = *(volatile int *)ri;
    for (int tries = 0; tries < kDdTries; tries++) {
        const float old = __int_as_float(cur);
        if (old == FLT_MAX) return;
        const float nw = old * (1.0f + alpha);
        const int seen = atomicCAS(ri, cur, __float_as_int(nw));
        if (seen == cur) return;
        cur = seen;
    }
}

__device__ __forceinline__ void dd_shrink(float *r, float alpha, float radius0, float rmin)
{
    int *ri = reinterpret_cast<int *>(r);
    int cur = *(volatile int *)ri;
    for (int tries = 0; tries < kDdTries; tries++) {
        const float old = __int_as_float(cur);
        const float nw = (old == FLT_MAX) ? radius0 : fmaxf(old * (1.0f - alpha), rmin);
        if (__float_as_int(nw) == cur) return;   // at the floor already: the update writes nothing new
        const int seen = atomicCAS(ri, cur, __float_as_int(nw));
        if (seen == cur) return;
        cur = seen;
    }
}

// Walk parents from `start` to the root, recording node coordinates and adding
// edge lengths (l2_dist, utils.cuh:89-98) to *cost.  Returns the number of
// nodes recorded (root excluded) and the root in *root; -1 if out exceeds cap.
template <int D>
__device__ int trace_to_root(const float *nodes, const int *parents, int cap, int start, float *out, int out_cap,
                             float *cost, int *root)
{
    int cur = start, n = 0;
    const volatile int *vp = parents;
    for (int steps = 0; steps <= cap; steps++) {
        const int par = vp[cur];
        if (par == cur) {
            *root = cur;
            return n;
        }
        if (n >= out_cap || par < 0 || par >= cap) return -1;
        float acc = 0.0f;
#pragma unroll
        for (int d = 0; d < D; d++) {
            const float a = __ldcg(nodes + (size_t)d * cap + cur);
            const float b = __ldcg(nodes + (size_t)d * cap + par);
            const float df = a - b;
            acc = fmaf(df, df, acc);
            out[n * D + d] = a;
        }
        *cost += sqrtf(acc);
        n++;
        cur = par;
    }
    return -1;
}

}  // namespace prrtc

namespace prrtc {

// ---------------------------------------------------------------------------
// Warp-level pieces for the batched planner: every warp is an independent
// worker, so nothing here synchronises more than one warp.

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// Warp argmin of squared distance from q (all lanes hold the full q) over the
// first `count` nodes of a SoA tree; ties -> lowest index.  All lanes return
// the result.
template <int D>
__device__ __forceinline__ void warp_nn(const float *__restrict__ nodes, int cap, int count, const float (&q)[D],
                                        float &out_d, int &out_i)
{
    float bd = FLT_MAX;
    int bi = 0x7fffffff;
    if (count > cap) count = cap;
    const int n4 = (count + 3) >> 2;
    const float4 *base = reinterpret_cast<const float4 *>(nodes);
    const int cap4 = cap >> 2;
    for (int c = lane_id(); c < n4; c += 32) {
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
#pragma unroll
        for (int d = 0; d < D; d++) {
            const float4 v = __ldcg(base + (size_t)d * cap4 + c);
            const float x0 = v.x - q[d], x1 = v.y - q[d], x2 = v.z - q[d], x3 = v.w - q[d];
            a0 = fmaf(x0, x0, a0);
            a1 = fmaf(x1, x1, a1);
            a2 = fmaf(x2, x2, a2);
            a3 = fmaf(x3, x3, a3);
        }
        const int i0 = 4 * c;
        if (a0 < bd) { bd = a0; bi = i0; }
        if (a1 < bd) { bd = a1; bi = i0 + 1; }
        if (a2 < bd) { bd = a2; bi = i0 + 2; }
        if (a3 < bd) { bd = a3; bi = i0 + 3; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float od = __shfl_xor_sync(0xffffffffu, bd, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (od < bd || (od == bd && oi < bi)) { bd = od; bi = oi; }
    }
    out_d = bd;
    out_i = bi == 0x7fffffff ? 0 : bi;
}

// Exact unsigned division by a small divisor b (2..64) without a divide
// instruction: q = floor(i * M / 2^k) with k = 32 + ceil(log2 b) and
// M = floor(2^k / b) + 1, which equals floor(i / b) for every 32-bit i
// because 2^k < M * b <= 2^k + b <= 2^k + 2^(k-32) (Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994).
// magic[b] holds M * 2^(64-k), so q is the high word of one 64-bit product.
// The sampler's digit loops divide by the Halton bases; a rejected sample of
// a dynamic-domain query is almost nothing but those loops.  They use the
// 31-bit form: for i < 2^31, q = floor(i * m / 2^(31 + l)) with
// l = ceil(log2 b) and m = ceil(2^(31 + l) / b) < 2^32, exact because
// 0 <= m * b - 2^(31 + l) < b <= 2^l (the same theorem with N = 31), so q is
// one 32-bit multiply-high and a shift by l - 1.
struct DivTable {
    unsigned long long magic[65];
    unsigned m31[65];
    unsigned s31[65];
    float inv[65];   // 1 / b, correctly rounded
    constexpr DivTable() : magic(), m31(), s31(), inv()
    {
        for (unsigned b = 2; b <= 64; b++) {
            unsigned ell = 0;
            while ((1u << ell) < b) ell++;
            const unsigned k = 32 + ell;
            magic[b] = ((1ull << k) / b + 1) << (64 - k);
            m31[b] = (unsigned)(((1ull << (31 + ell)) + b - 1) / b);
            s31[b] = ell - 1;
            inv[b] = 1.0f / (float)b;
        }
    }
};
__constant__ const DivTable kDivTable = DivTable();

__device__ __forceinline__ unsigned div_by(unsigned i, unsigned long long magic)
{
    return (unsigned)__umul64hi((unsigned long long)i, magic);
}

// floor(i / b) for i < 2^31 (m = m31[b], s = s31[b])
__device__ __forceinline__ unsigned div31(unsigned i, unsigned m, unsigned s)
{
    return __umulhi(i, m) >> s;
}

// Radical inverses of one index iter < 2^31 in N bases at once, float32: the
// closed form of the reference's incremental Halton recurrence.  h[d] =
// sum over the digits of iter in base b[d], least significant first, of
// digit * b^-k, accumulated by fmaf in that order with the weight f = b^-k
// kept as a running float product; with SCRAMBLE every digit is first
// multiplied by a[d] mod b[d] (a linear digit scrambling that breaks the
// correlations between large prime bases while keeping each dimension's
// low-discrepancy structure).  The digit chains of the N dimensions advance
// together, one digit of every dimension per trip, for as many trips as the
// smallest base needs: N independent dependency chains instead of N loops in
// a row, and the same trip count on every lane.  A dimension whose index is
// exhausted adds fmaf(f, 0, h) = h, so its value is the same as from its own
// loop.
//
// The state can stop between trips: after any trip, h[d] holds the digits so
// far and the digits still to come add less than f[d] * b[d] (each at most
// b - 1 times a weight f, f / b, ...), nothing at all once idx[d] is 0.
template <int N, bool SCRAMBLE>
struct RadicalDigits {
    unsigned idx[N], m[N], s[N], b[N], a[N];
    float f[N], inv[N], h[N];
    unsigned rem, mmin, smin;

    __device__ __forceinline__ RadicalDigits(unsigned iter, const unsigned (&bs)[N], const unsigned (&as)[N])
    {
        unsigned bmin = bs[0];
#pragma unroll
        for (int d = 0; d < N; d++) {
            b[d] = bs[d];
            a[d] = as[d];
            idx[d] = iter;
            m[d] = kDivTable.m31[b[d]];
            s[d] = kDivTable.s31[b[d]];
            inv[d] = kDivTable.inv[b[d]];
            f[d] = inv[d];
            h[d] = 0.0f;
            bmin = min(bmin, b[d]);
        }
        mmin = kDivTable.m31[bmin];
        smin = kDivTable.s31[bmin];
        rem = iter;
    }
    __device__ __forceinline__ void trip()
    {
#pragma unroll
        for (int d = 0; d < N; d++) {
            const unsigned q = div31(idx[d], m[d], s[d]);
            unsigned dig = idx[d] - q * b[d];
            if (SCRAMBLE) {
                const unsigned t = a[d] * dig;   // < 64 * 64
                dig = t - div31(t, m[d], s[d]) * b[d];
            }
            h[d] = fmaf(f[d], (float)dig, h[d]);
            idx[d] = q;
            f[d] *= inv[d];
        }
        rem = div31(rem, mmin, smin);
    }
    __device__ __forceinline__ void run(int trips)
    {
        for (int k = 0; k < trips && rem > 0; k++) trip();
    }
    __device__ __forceinline__ void finish()
    {
        while (rem > 0) trip();
    }
};

__device__ __forceinline__ unsigned hash32(unsigned x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

}  // namespace prrtc
