// Device-side building blocks shared by every robot's kernels: the packed
// environment, the reference's sphere-vs-primitive tests, and the three
// routines the generated checkers call for leaf spheres.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace prrtc {

// 3x4 row-major rigid transform: r00 r01 r02 tx | r10 r11 r12 ty | r20 r21 r22 tz
struct Frame {
    float m[12];
};

// A self-collision leaf pair: sphere a in frame A, sphere b in frame B.
struct LeafPair {
    float4 a;
    float4 b;
};

// Packed environment, float4 records, in this order (all 16-byte aligned):
//   spheres  ns  x 1   (x, y, z, r)
//   capsules nc  x 2   (x1, y1, z1, r) (xv, yv, zv, rdv)
//   zcaps    nzc x 2   same
//   cuboids  ncb x 4   (x, y, z, r1) (a1x, a1y, a1z, r2) (a2x, a2y, a2z, r3) (a3x, a3y, a3z, 0)
//   zcuboids nzb x 4   same
// The reference's cylinders array is never read by its checker and is not packed.
struct EnvCounts {
    int ns, nc, nzc, ncb, nzb;
    __host__ __device__ int records() const { return ns + 2 * nc + 2 * nzc + 4 * ncb + 4 * nzb; }
};

struct EnvView {
    const float4 *rec;   // records (shared memory once staged)
    EnvCounts n;
};

// Copy a packed environment into shared memory (all threads of the block
// participate; caller synchronises).
__device__ __forceinline__ void stage_env(float4 *smem, const float4 *__restrict__ g, int records)
{
    for (int i = threadIdx.x; i < records; i += blockDim.x) smem[i] = __ldg(g + i);
}

// The same copy as one bulk asynchronous copy by the SM's TMA engine
// (cp.async.bulk global -> shared, no tensor map), completed on the
// shared-memory mbarrier `bar`: thread 0 arms the barrier with the byte count
// and issues the copy, every thread waits for the barrier's phase 0.  Both
// addresses are 16-byte aligned (float4 records) and the size is a multiple
// of 16 bytes, as the bulk copy requires.  All threads of the block call it,
// once per kernel (the barrier's first phase); it returns with the records in
// shared memory and the block synchronised.  The wait is bounded: should the
// copy not complete within kBulkPolls polls, the block copies the records
// itself (the same bytes) and, before it returns, polls once more so that no
// copy can still be landing while the block goes on.
constexpr int kBulkPolls = 1 << 20;

// has the mbarrier at shared address `bar` completed its phase of parity `parity`?
__device__ __forceinline__ bool bulk_phase_done(unsigned bar, unsigned parity)
{
    unsigned done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return done != 0;
}

__device__ __forceinline__ void stage_env_bulk(float4 *smem, const float4 *__restrict__ g, int records,
                                               unsigned long long *mbar)
{
    if (records <= 0) {
        __syncthreads();
        return;
    }
    const unsigned bytes = (unsigned)records * 16u;
    const unsigned bar = (unsigned)__cvta_generic_to_shared(mbar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(g), "r"(bytes), "r"(bar)
                     : "memory");
    }
    __syncthreads();   // the barrier is armed before anyone polls it
    bool done = false;
    for (int i = 0; i < kBulkPolls && !done; i++) done = bulk_phase_done(bar, 0u);
    if (!__syncthreads_and(done)) {
        stage_env(smem, g, records);
        for (int i = 0; i < kBulkPolls && !done; i++) done = bulk_phase_done(bar, 0u);
        __syncthreads();
    }
}

// ---- the reference's primitive tests (src/planning/utils.cuh:58-209) ------
// Each returns true when the sphere (x, y, z, r) intersects the primitive,
// i.e. the reference's "< 0" on squared distance minus squared radius.

__device__ __forceinline__ bool hit_sphere(float4 s, float x, float y, float z, float r)
{
    const float dx = x - s.x, dy = y - s.y, dz = z - s.z;
    const float rs = r + s.w;
    return dx * dx + dy * dy + dz * dz - rs * rs < 0.0f;
}

__device__ __forceinline__ bool hit_capsule(float4 a, float4 v, float x, float y, float z, float r)
{
    const float dot = (x - a.x) * v.x + (y - a.y) * v.y + (z - a.z) * v.z;
    const float cdf = fmaxf(fminf(dot * v.w, 1.0f), 0.0f);
    const float dx = x - (a.x + v.x * cdf), dy = y - (a.y + v.y * cdf), dz = z - (a.z + v.z * cdf);
    const float rs = r + a.w;
    return dx * dx + dy * dy + dz * dz - rs * rs < 0.0f;
}

__device__ __forceinline__ bool hit_z_capsule(float4 a, float4 v, float x, float y, float z, float r)
{
    const float dot = (z - a.z) * v.z;
    const float cdf = fmaxf(fminf(dot * v.w, 1.0f), 0.0f);
    const float dx = x - a.x, dy = y - a.y, dz = z - (a.z + v.z * cdf);
    const float rs = r + a.w;
    return dx * dx + dy * dy + dz * dz - rs * rs < 0.0f;
}

__device__ __forceinline__ bool hit_cuboid(float4 c0, float4 c1, float4 c2, float4 c3, float x, float y,
                                           float z, float rsq)
{
    const float xs = x - c0.x, ys = y - c0.y, zs = z - c0.z;
    const float a1 = fmaxf(0.0f, fabsf(c1.x * xs + c1.y * ys + c1.z * zs) - c0.w);
    const float a2 = fmaxf(0.0f, fabsf(c2.x * xs + c2.y * ys + c2.z * zs) - c1.w);
    const float a3 = fmaxf(0.0f, fabsf(c3.x * xs + c3.y * ys + c3.z * zs) - c2.w);
    return a1 * a1 + a2 * a2 + a3 * a3 - rsq < 0.0f;
}

__device__ __forceinline__ bool hit_z_cuboid(float4 c0, float4 c1, float4 c2, float x, float y, float z,
                                             float rsq)
{
    const float xs = x - c0.x, ys = y - c0.y, zs = z - c0.z;
    const float a1 = fmaxf(0.0f, fabsf(c1.x * xs + c1.y * ys) - c0.w);
    const float a2 = fmaxf(0.0f, fabsf(c2.x * xs + c2.y * ys) - c1.w);
    const float a3 = fmaxf(0.0f, fabsf(zs) - c2.w);
    return a1 * a1 + a2 * a2 + a3 * a3 - rsq < 0.0f;
}

// Algorithmic FLOPs of one primitive test (FMA = 2; min/max/abs not counted),
// the weights the roofline uses for the reference checker's work.
constexpr int kFlopSphere = 11, kFlopCapsule = 26, kFlopZCapsule = 16, kFlopCuboid = 27, kFlopZCuboid = 18,
              kFlopPair = 11;

// Sphere against every obstacle with early exit
// (sphere_environment_in_collision, utils.cuh:211-242).  Not inlined: every
// generated call site shares one copy of the obstacle loops.  Returns
// 2 * (FLOPs of the tests executed) + (1 if hit).
//
// Spheres, capsules and cuboids are tested two at a time (independent
// dependency chains, one branch); on a hit the count stops at the first
// hitting test, so verdicts and counts are the reference's, in its order.
static __device__ __noinline__ int env_hit(const EnvView e, float x, float y, float z, float r)
{
    const float4 *p = e.rec;
    int w = 0, i = 0;
    for (; i + 2 <= e.n.ns; i += 2) {
        const bool h0 = hit_sphere(p[i], x, y, z, r), h1 = hit_sphere(p[i + 1], x, y, z, r);
        if (h0 | h1) return 2 * (w + (h0 ? 1 : 2) * kFlopSphere) + 1;
        w += 2 * kFlopSphere;
    }
    if (i < e.n.ns) {
        w += kFlopSphere;
        if (hit_sphere(p[i], x, y, z, r)) return 2 * w + 1;
    }
    p += e.n.ns;
    for (i = 0; i + 2 <= e.n.nc; i += 2) {
        const float4 *c = p + 2 * i;
        const bool h0 = hit_capsule(c[0], c[1], x, y, z, r), h1 = hit_capsule(c[2], c[3], x, y, z, r);
        if (h0 | h1) return 2 * (w + (h0 ? 1 : 2) * kFlopCapsule) + 1;
        w += 2 * kFlopCapsule;
    }
    if (i < e.n.nc) {
        w += kFlopCapsule;
        if (hit_capsule(p[2 * i], p[2 * i + 1], x, y, z, r)) return 2 * w + 1;
    }
    p += 2 * e.n.nc;
    for (i = 0; i < e.n.nzc; i++) {
        w += kFlopZCapsule;
        if (hit_z_capsule(p[2 * i], p[2 * i + 1], x, y, z, r)) return 2 * w + 1;
    }
    p += 2 * e.n.nzc;
    const float rsq = r * r;
    for (i = 0; i + 2 <= e.n.ncb; i += 2) {
        const float4 *c = p + 4 * i;
        const bool h0 = hit_cuboid(c[0], c[1], c[2], c[3], x, y, z, rsq),
                   h1 = hit_cuboid(c[4], c[5], c[6], c[7], x, y, z, rsq);
        if (h0 | h1) return 2 * (w + (h0 ? 1 : 2) * kFlopCuboid) + 1;
        w += 2 * kFlopCuboid;
    }
    if (i < e.n.ncb) {
        w += kFlopCuboid;
        if (hit_cuboid(p[4 * i], p[4 * i + 1], p[4 * i + 2], p[4 * i + 3], x, y, z, rsq)) return 2 * w + 1;
    }
    p += 4 * e.n.ncb;
    for (i = 0; i < e.n.nzb; i++) {
        w += kFlopZCuboid;
        if (hit_z_cuboid(p[4 * i], p[4 * i + 1], p[4 * i + 2], x, y, z, rsq)) return 2 * w + 1;
    }
    return 2 * w;
}

__device__ __forceinline__ void xform(const Frame &T, float4 c, float &x, float &y, float &z)
{
    x = T.m[0] * c.x + T.m[1] * c.y + T.m[2] * c.z + T.m[3];
    y = T.m[4] * c.x + T.m[5] * c.y + T.m[6] * c.z + T.m[7];
    z = T.m[8] * c.x + T.m[9] * c.y + T.m[10] * c.z + T.m[11];
}

// Leaf spheres (given in frame T) against the environment; pad inflates every
// radius (0 reproduces the reference exactly).  Returns 2 * FLOPs + (1 if any hit).
static __device__ __noinline__ int env_leaves(const EnvView e, const Frame T, const float4 *__restrict__ leaves, int n,
                                              float pad)
{
    int w = 0;
    for (int i = 0; i < n; i++) {
        const float4 c = leaves[i];
        float x, y, z;
        xform(T, c, x, y, z);
        const int h = env_hit(e, x, y, z, c.w + pad);
        w += h >> 1;
        if (h & 1) return 2 * w + 1;
    }
    return 2 * w;
}

// Leaf pairs: a in frame A, b in frame B, Tab = inv(T_A) * T_B
// (sphere_sphere_self_collision, utils.cuh:83-86).  pad2 is the added
// inflation of a pair (twice the per-sphere pad).  Returns 2 * FLOPs + hit.
static __device__ __noinline__ int self_pairs(const Frame Tab, const LeafPair *__restrict__ pairs, int n, float pad2)
{
    auto hit = [&](const LeafPair &pr) {
        float x, y, z;
        xform(Tab, pr.b, x, y, z);
        const float dx = pr.a.x - x, dy = pr.a.y - y, dz = pr.a.z - z;
        const float rs = pr.a.w + pr.b.w + pad2;
        return dx * dx + dy * dy + dz * dz - rs * rs < 0.0f;
    };
    int i = 0;
    for (; i + 2 <= n; i += 2) {   // two at a time, counted up to the first hit
        const bool h0 = hit(pairs[i]), h1 = hit(pairs[i + 1]);
        if (h0 | h1) return 2 * kFlopPair * (i + (h0 ? 1 : 2)) + 1;
    }
    if (i < n && hit(pairs[i])) return 2 * kFlopPair * (i + 1) + 1;
    return 2 * kFlopPair * n;
}

// ---- table-driven checker (robots with many groups) -----------------------
// A generated checker for a robot with hundreds of groups (Baxter: 388) as
// straight-line code does not fit the instruction cache; its table form
// computes every frame first and then walks the same schedule through these
// tables, making the same ctx calls in the same order (same verdicts, same
// counts).  Frames are indexed by joint config index + 1; F[0] is the world.

struct GenSched {
    int kind;    // 0 environment group, 1 self group
    int index;
};
struct GenEnvGroup {
    int gate;             // gating sphere: index into the gate centres, -1 none
    int first_block, nblocks, pad_;
};
struct GenLeafBlock {
    int frame, first, n, pad_;
};
struct GenSelfGroup {
    int ga, gb;           // gating pair: indices into the gate centres
    int first_block, nblocks;
};
struct GenPairBlock {
    int fa, fb, first, n;
};

// Tab = inv(A) * B for rigid transforms A and B.
__device__ __forceinline__ Frame relative_frame(const Frame &A, const Frame &B)
{
    Frame R;
    const float d0 = B.m[3] - A.m[3], d1 = B.m[7] - A.m[7], d2 = B.m[11] - A.m[11];
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int k = 0; k < 3; k++) R.m[4 * i + k] = A.m[i] * B.m[k] + A.m[4 + i] * B.m[4 + k] + A.m[8 + i] * B.m[8 + k];
        R.m[4 * i + 3] = A.m[i] * d0 + A.m[4 + i] * d1 + A.m[8 + i] * d2;
    }
    return R;
}

// Where a table-form checker keeps its frames (F[0] the world, F[q + 1] the
// frame of joint q) while it walks the schedule.
//
// LocalFrames: an array per thread (frames 1 .. N-1; the world frame is a
// constant).  The schedule indexes it with table values, so it lives in
// local memory, cached by L1 while it fits there.
//
// SharedFrames: one column per lane in a warp's shared-memory area, float4
// k (0..2) of frame i (i >= 1) at p[(3 (i - 1) + k) * 32], p = area + lane.
// A warp's 32 lanes touch 32 consecutive float4 per access (no bank
// conflicts), every read hits, and nothing competes with it for L1.  The
// world frame is not stored.  shared_frame_bytes(N) is a warp's area.
template <int N>
struct LocalFrames {
    Frame F[N > 1 ? N - 1 : 1];   // the world frame is not stored
    __device__ __forceinline__ void set(int i, const Frame &f)
    {
        if (i > 0) F[i - 1] = f;
    }
    __device__ __forceinline__ const Frame *view() const { return F; }
};

struct SharedFrames {
    float4 *p;
    __device__ __forceinline__ void set(int i, const Frame &f)
    {
        if (i == 0) return;
        float4 *q = p + 3 * (i - 1) * 32;
        q[0] = make_float4(f.m[0], f.m[1], f.m[2], f.m[3]);
        q[32] = make_float4(f.m[4], f.m[5], f.m[6], f.m[7]);
        q[64] = make_float4(f.m[8], f.m[9], f.m[10], f.m[11]);
    }
    __device__ __forceinline__ SharedFrames view() const { return *this; }
};

__host__ __device__ constexpr size_t shared_frame_bytes(int frames)
{
    return (size_t)(frames > 1 ? frames - 1 : 0) * 3 * 32 * sizeof(float4);
}

__device__ __forceinline__ Frame world_frame()
{
    return Frame{{1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f}};
}

// frame i of a local array holding frames 1 .. N-1 (LocalFrames::view)
__device__ __forceinline__ Frame frame_at(const Frame *F, int i) { return i == 0 ? world_frame() : F[i - 1]; }

__device__ __forceinline__ Frame frame_at(const SharedFrames F, int i)
{
    if (i == 0) return world_frame();
    const float4 *q = F.p + 3 * (i - 1) * 32;
    const float4 a = q[0], b = q[32], c = q[64];
    return Frame{{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w}};
}

// What the generated checkers call.  pad = 0 and stop_flag = nullptr give the
// reference checker's verdicts; planners may inflate every sphere by pad
// (a certified margin) and share a flag through which any lane's collision
// ends the other lanes' work on the same edge.  `work` accumulates the
// algorithmic FLOPs of the primitive tests executed (reference weights).
struct CheckCtx {
    static constexpr bool kSharedFrames = false;   // table-form frames in a local array
    EnvView env;
    float pad;
    volatile int *stop_flag;
    unsigned work = 0;
    __device__ __forceinline__ bool take(int h)
    {
        work += (unsigned)(h >> 1);
        return h & 1;
    }
    __device__ __forceinline__ bool env_hit(float x, float y, float z, float r)
    {
        return take(prrtc::env_hit(env, x, y, z, r + pad));
    }
    __device__ __forceinline__ bool env_leaves(const Frame &T, const float4 *l, int n)
    {
        return take(prrtc::env_leaves(env, T, l, n, pad));
    }
    __device__ __forceinline__ bool self_pairs(const Frame &T, const LeafPair *p, int n)
    {
        return take(prrtc::self_pairs(T, p, n, 2.0f * pad));
    }
    __device__ __forceinline__ bool pair_hit(float dx, float dy, float dz, float rs)
    {
        work += kFlopPair;
        rs += 2.0f * pad;
        return dx * dx + dy * dy + dz * dz - rs * rs < 0.0f;
    }
    __device__ __forceinline__ bool stop() const { return stop_flag != nullptr && *stop_flag != 0; }
};

// The same checks with the table-form frames in the warp's shared-memory
// area (frames: the area's base + lane, see SharedFrames).
struct SharedCheckCtx : CheckCtx {
    static constexpr bool kSharedFrames = true;
    float4 *frames;
};

// The frame store a generated checker uses with context type Ctx.
template <class Ctx, int N, bool = Ctx::kSharedFrames>
struct FrameStore : LocalFrames<N> {
    __device__ __forceinline__ explicit FrameStore(const Ctx &) {}
};
template <class Ctx, int N>
struct FrameStore<Ctx, N, true> : SharedFrames {
    __device__ __forceinline__ explicit FrameStore(const Ctx &c) : SharedFrames{c.frames} {}
};

// The schedule of a table-form checker (see GenSched); returns true when free.
// F is a frame view: a local array (const Frame *) or SharedFrames.
// A gate sphere (x, y, z, r in frame T) in world coordinates, radius kept.
__device__ __forceinline__ float4 gate_centre(const Frame &T, float4 c)
{
    float x, y, z;
    xform(T, c, x, y, z);
    return make_float4(x, y, z, c.w);
}

// G: the world centres of the gate spheres, computed with the frames (the
// same xform as a leaf's, so verdicts do not change).
template <class Frames, class Ctx>
__device__ __noinline__ bool run_schedule(const Frames F, const float4 *__restrict__ G, const GenSched *__restrict__ sched,
                                          int nsched,
                                          const GenEnvGroup *__restrict__ eg, const GenLeafBlock *__restrict__ lb,
                                          const float4 *__restrict__ leaves, const GenSelfGroup *__restrict__ sg,
                                          const GenPairBlock *__restrict__ pb, const LeafPair *__restrict__ pairs,
                                          Ctx &ctx)
{
    for (int s = 0; s < nsched; s++) {
        const GenSched e = sched[s];
        if (e.kind == 0) {
            const GenEnvGroup g = eg[e.index];
            bool go = true;
            if (g.gate >= 0) {
                const float4 c = G[g.gate];
                go = ctx.env_hit(c.x, c.y, c.z, c.w);
            }
            if (go)
                for (int k = g.first_block; k < g.first_block + g.nblocks; k++) {
                    const GenLeafBlock b = lb[k];
                    if (ctx.env_leaves(frame_at(F, b.frame + 1), leaves + b.first, b.n)) return false;
                }
        } else {
            const GenSelfGroup g = sg[e.index];
            const float4 a = G[g.ga], b = G[g.gb];
            if (ctx.pair_hit(a.x - b.x, a.y - b.y, a.z - b.z, a.w + b.w))
                for (int k = g.first_block; k < g.first_block + g.nblocks; k++) {
                    const GenPairBlock b = pb[k];
                    if (ctx.self_pairs(relative_frame(frame_at(F, b.fa + 1), frame_at(F, b.fb + 1)), pairs + b.first, b.n))
                        return false;
                }
        }
        if (ctx.stop()) return true;
    }
    return true;
}

}  // namespace prrtc
