// Straight-line CUDA collision checker for pRRTC's sphere model.  Generated by
// prrtc_gb300/robots/codegen.py from the fitted model; do not edit.
// Semantics follow the reference checker fkcc<Robot> (src/planning/utils.cuh):
// a leaf counts only when its group's gate (bounding sphere or bounding pair)
// is hit; a config is free when no counted leaf is hit.
#pragma once

namespace prrtc { namespace gen_sphere {

constexpr int kDof = 3;
constexpr int kFrames = 4;   // the world and one frame per joint
constexpr int kNumSpheres = 1;
constexpr int kNumLeaves = 1;
constexpr int kNumPairs = 1;
// canonical algorithmic FLOPs of one forward kinematics: 2 * (12 * dof + 9 * spheres)
constexpr unsigned kFkFlops = 90u;

// leaf spheres in their frame: (x, y, z, r)
__device__ const float4 kSphereLeaf[kNumLeaves] = {
    {0.0f, 0.0f, 0.0f, 1.0f},
};
// sphere pairs: a = (x, y, z, r) in frame A, b = (x, y, z, r) in frame B
__device__ const LeafPair kSpherePair[kNumPairs] = {
    {{0.0f, 0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f, 0.0f}},
};

// Returns true when configuration q is collision-free.
template <class Ctx>
__device__ __forceinline__ bool fkcc(const float *__restrict__ q, Ctx &ctx)
{
    // environment group 0: sphere
    const float t0_0 = q[0];
    const float a1_1 = t0_0;
    const float t1_2 = a1_1;
    const float t1_3 = q[1];
    const float a2_4 = t1_2;
    const float a2_5 = t1_3;
    const float t2_6 = a2_4;
    const float t2_7 = a2_5;
    const float t2_8 = q[2];
    const float p9 = t2_6;
    const float p10 = t2_7;
    const float p11 = t2_8;
    if (ctx.env_hit(p9, p10, p11, 1.0f)) return false;
    if (ctx.stop()) return true;
    return true;
}

// The same verdicts for the stand-alone checker of single configurations.
template <class Ctx>
__device__ __forceinline__ bool fkcc_validate(const float *__restrict__ q, Ctx &ctx)
{
    return fkcc(q, ctx);
}

// World centre and radius of every model sphere (model sphere order).
__device__ __forceinline__ void fk_spheres(const float *__restrict__ q, float4 *__restrict__ out)
{
    const float t0_0 = q[0];
    const float a1_1 = t0_0;
    const float t1_2 = a1_1;
    const float t1_3 = q[1];
    const float a2_4 = t1_2;
    const float a2_5 = t1_3;
    const float t2_6 = a2_4;
    const float t2_7 = a2_5;
    const float t2_8 = q[2];
    const float p9 = t2_6;
    const float p10 = t2_7;
    const float p11 = t2_8;
    out[0] = make_float4(p9, p10, p11, 1.0f);
}

} }  // namespace prrtc::gen_sphere
