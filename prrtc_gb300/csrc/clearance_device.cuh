// Differentiable clearance: device side.  No reference counterpart (pRRTC
// returns raw RRT-Connect paths); this is the cost used to repair and smooth
// them.
//
// For one configuration q the cost is
//     C(q) = 1/2 sum over env leaf spheres s, obstacles o of max(0, m - sd(s, o))^2
//          + 1/2 sum over self-collision leaf pairs (a, b) of max(0, m - sd(a, b))^2
// with sd the signed distance in metres (negative inside) and m the margin:
// a squared hinge, continuous with a continuous gradient.  The leaf spheres
// and pairs are exactly the ones the reference checker tests at its leaves
// (fkcc<Robot>, utils.cuh), so C(q) = 0 with m >= 0 means every leaf test is
// clear.  Box distances are true signed distances with the interior included:
// the reference's box test (utils.cuh:158-176) is flat inside a box, which has
// no gradient to follow out of it.
//
// Precision: every sphere-obstacle and sphere-sphere term is first screened
// in float32 (the bulk of the work); the few terms the screen keeps, the
// forward kinematics and the adjoint sweep run in float64, so the result
// matches a float64 evaluation to ~1e-7 even for terms a fraction of a
// millimetre inside the margin (float32 coordinates near 1 m are only good
// to 6e-8 m, a 4e-4 relative error on such a term).
//
// The adjoint recomputes forward kinematics rather than keeping per-link
// transforms from a forward pass.  Each active term becomes a force
// g = dC/dc on a sphere centre c; per joint j the forces G_j and the moments
// M_j = sum (c - o_j) x g about the joint's origin o_j are summed, then
// accumulated from the tips toward the base (a child's moment shifted to its
// parent's origin by (o_child - o_parent) x G_child), and each joint's
// derivative is axis . M_j for a revolute joint or axis . G_j for a
// prismatic one.  Lever arms stay link-sized.
#pragma once

#include "device_common.cuh"
#include "robots/model_types.h"

namespace prrtc {

constexpr int kClrMaxJoints = 14;

// A robot's collision model in the layout the clearance kernels read: every
// index is a position in these tables (joints in chain order, parents first).
struct ClrModel {
    int dof, nj, n_leaf, n_pair;
    const prrtc_joint_def *joints;
    const int *joint_parent;   // table position of each joint's parent, -1 = world
    const float4 *leaf;        // env leaf spheres (x, y, z, r) in their joint's frame
    const int *leaf_joint;     // table position of each leaf's joint, -1 = world
    const float4 *pair_a, *pair_b;
    const int2 *pair_joint;
};

// One path's obstacles (device records, layout of device_common.cuh).
struct ClrEnv {
    const float4 *rec;
    EnvCounts n;
};

// Smoothing settings as the kernels read them (prrtc_smooth_settings).
struct ClrSmooth {
    float margin, step, cost_weight, smooth_weight;
    int steps, granularity, shortcut_rounds;
};

// One launch of the smoothing kernel over n_paths paths of `waypoints` rows.
struct ClrLaunch {
    ClrModel M;
    const ClrEnv *envs;       // [n_paths]
    int n_paths, waypoints;
    float *q;                 // [n_paths][waypoints][dof], rewritten for accepted paths
    float lo[kClrMaxJoints], hi[kClrMaxJoints];   // joint limits
    ClrSmooth s;
    uint8_t *accepted;        // [n_paths]
    float *cost_before, *cost_after;              // [n_paths], may be null
};

namespace clr {

// Every function here is also built for the host, so the same code can be
// run and compared on a CPU.
#define CLR_FN __host__ __device__ __forceinline__

// Slack of the float32 screen: a term is evaluated in float64 when its
// float32 hinge argument m - sd exceeds -kScreen.  Float32 centres are within
// ~1e-6 m of the float64 ones and sd is 1-Lipschitz in the centre, so no
// active term is screened out.
constexpr float kScreen = 1e-4f;

CLR_FN float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
CLR_FN float3 sub(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
CLR_FN float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
CLR_FN double3 d3(double x, double y, double z) { return make_double3(x, y, z); }
CLR_FN double3 d3(float3 a) { return d3(a.x, a.y, a.z); }
CLR_FN double3 sub(double3 a, double3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
CLR_FN double3 add(double3 a, double3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
CLR_FN double3 scale(double s, double3 a) { return d3(s * a.x, s * a.y, s * a.z); }
CLR_FN double dot(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
CLR_FN double3 cross(double3 a, double3 b)
{
    return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// ---- float32 screen: signed distances only -------------------------------

CLR_FN float sd_point_f(float3 d, float rsum) { return sqrtf(dot(d, d)) - rsum; }

CLR_FN float sd_capsule_f(float3 c, float r, float4 a, float4 v, bool z)
{
    const float s = z ? (c.z - a.z) * v.z : (c.x - a.x) * v.x + (c.y - a.y) * v.y + (c.z - a.z) * v.z;
    const float t = fminf(fmaxf(s * v.w, 0.0f), 1.0f);
    const float3 d = z ? f3(c.x - a.x, c.y - a.y, c.z - (a.z + v.z * t))
                       : f3(c.x - (a.x + v.x * t), c.y - (a.y + v.y * t), c.z - (a.z + v.z * t));
    return sd_point_f(d, r + a.w);
}

// Box with centre ce, unit axes a1..a3, half extents h (true signed distance).
CLR_FN float sd_box_f(float3 c, float r, float3 ce, float3 a1, float3 a2, float3 a3, float3 h)
{
    const float3 d = sub(c, ce);
    const float q1 = fabsf(dot(a1, d)) - h.x, q2 = fabsf(dot(a2, d)) - h.y, q3 = fabsf(dot(a3, d)) - h.z;
    const float p1 = fmaxf(q1, 0.0f), p2 = fmaxf(q2, 0.0f), p3 = fmaxf(q3, 0.0f);
    const float out = sqrtf(p1 * p1 + p2 * p2 + p3 * p3);
    return (out > 0.0f ? out : fmaxf(q1, fmaxf(q2, q3))) - r;
}

// ---- float64 terms: cost and force -------------------------------------

// Adds 1/2 max(0, m - sd)^2 to *cost and -phi * dsd/dc to *g.
CLR_FN void hinge(double sd, double3 gsd, double m, double *cost, double3 *g)
{
    const double phi = m - sd;
    if (phi > 0.0) {
        *cost += 0.5 * phi * phi;
        *g = sub(*g, scale(phi, gsd));
    }
}

// Distance term for centre offset d from the closest point of a primitive.
CLR_FN void point_term(double3 d, double rsum, double m, double *cost, double3 *g)
{
    const double len = sqrt(dot(d, d));
    const double inv = len > 0.0 ? 1.0 / len : 0.0;
    hinge(len - rsum, scale(inv, d), m, cost, g);
}

CLR_FN void capsule_term(double3 c, double r, float4 a, float4 v, bool z, double m, double *cost, double3 *g)
{
    const double s = z ? (c.z - a.z) * (double)v.z
                       : (c.x - a.x) * (double)v.x + (c.y - a.y) * (double)v.y + (c.z - a.z) * (double)v.z;
    double t = s * (double)v.w;
    t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
    const double3 d = z ? d3(c.x - a.x, c.y - a.y, c.z - (a.z + v.z * t))
                        : d3(c.x - (a.x + v.x * t), c.y - (a.y + v.y * t), c.z - (a.z + v.z * t));
    point_term(d, r + (double)a.w, m, cost, g);
}

CLR_FN void box_term(double3 c, double r, float3 ce, float3 a1f, float3 a2f, float3 a3f, float3 h, double m,
                     double *cost, double3 *g)
{
    const double3 d = sub(c, d3(ce)), a1 = d3(a1f), a2 = d3(a2f), a3 = d3(a3f);
    const double u1 = dot(a1, d), u2 = dot(a2, d), u3 = dot(a3, d);
    const double s1 = u1 < 0.0 ? -1.0 : 1.0, s2 = u2 < 0.0 ? -1.0 : 1.0, s3 = u3 < 0.0 ? -1.0 : 1.0;
    const double q1 = fabs(u1) - h.x, q2 = fabs(u2) - h.y, q3 = fabs(u3) - h.z;
    double sd;
    double3 gsd;
    if (q1 > 0.0 || q2 > 0.0 || q3 > 0.0) {
        const double p1 = (q1 > 0.0 ? q1 : 0.0) * s1, p2 = (q2 > 0.0 ? q2 : 0.0) * s2, p3 = (q3 > 0.0 ? q3 : 0.0) * s3;
        const double o = sqrt(p1 * p1 + p2 * p2 + p3 * p3);
        sd = o - r;
        gsd = scale(1.0 / o, add(add(scale(p1, a1), scale(p2, a2)), scale(p3, a3)));
    } else if (q1 >= q2 && q1 >= q3) {   // inside: the nearest face
        sd = q1 - r;
        gsd = scale(s1, a1);
    } else if (q2 >= q3) {
        sd = q2 - r;
        gsd = scale(s2, a2);
    } else {
        sd = q3 - r;
        gsd = scale(s3, a3);
    }
    hinge(sd, gsd, m, cost, g);
}

// ---- kinematics --------------------------------------------------------

// World frames of every joint (3x4 row-major, by table position), float64.
CLR_FN void fk(const ClrModel &M, const float *q, double (*T)[12])
{
    for (int j = 0; j < M.nj; j++) {
        const prrtc_joint_def &J = M.joints[j];
        const int p = M.joint_parent[j];
        double A[12];
        for (int i = 0; i < 3; i++) {
            const double p0 = p < 0 ? (i == 0 ? 1.0 : 0.0) : T[p][4 * i];
            const double p1 = p < 0 ? (i == 1 ? 1.0 : 0.0) : T[p][4 * i + 1];
            const double p2 = p < 0 ? (i == 2 ? 1.0 : 0.0) : T[p][4 * i + 2];
            const double p3 = p < 0 ? 0.0 : T[p][4 * i + 3];
            for (int k = 0; k < 3; k++) A[4 * i + k] = p0 * J.F[k] + p1 * J.F[4 + k] + p2 * J.F[8 + k];
            A[4 * i + 3] = p0 * J.F[3] + p1 * J.F[7] + p2 * J.F[11] + p3;
        }
        const double th = q[J.q];
        double *Tj = T[j];
        if (J.revolute) {   // rotation by th about local z
            double s, c;
            sincos(th, &s, &c);
            for (int i = 0; i < 3; i++) {
                Tj[4 * i] = c * A[4 * i] + s * A[4 * i + 1];
                Tj[4 * i + 1] = c * A[4 * i + 1] - s * A[4 * i];
                Tj[4 * i + 2] = A[4 * i + 2];
                Tj[4 * i + 3] = A[4 * i + 3];
            }
        } else {            // translation by th along local z
            for (int i = 0; i < 3; i++) {
                Tj[4 * i] = A[4 * i];
                Tj[4 * i + 1] = A[4 * i + 1];
                Tj[4 * i + 2] = A[4 * i + 2];
                Tj[4 * i + 3] = A[4 * i + 3] + th * A[4 * i + 2];
            }
        }
    }
}

// Rotated local offset of a sphere (its lever arm about the joint's origin).
CLR_FN double3 lever(const double (*T)[12], int j, float4 p)
{
    const double *t = T[j];
    return d3(t[0] * p.x + t[1] * p.y + t[2] * p.z, t[4] * p.x + t[5] * p.y + t[6] * p.z,
              t[8] * p.x + t[9] * p.y + t[10] * p.z);
}

CLR_FN double3 place(const double (*T)[12], int j, float4 p)
{
    if (j < 0) return d3(p.x, p.y, p.z);
    const double *t = T[j];
    return add(lever(T, j, p), d3(t[3], t[7], t[11]));
}

CLR_FN float3 place(const float (*T)[12], int j, float4 p)
{
    if (j < 0) return f3(p.x, p.y, p.z);
    const float *t = T[j];
    return f3(t[0] * p.x + t[1] * p.y + t[2] * p.z + t[3], t[4] * p.x + t[5] * p.y + t[6] * p.z + t[7],
              t[8] * p.x + t[9] * p.y + t[10] * p.z + t[11]);
}

// ---- one configuration -------------------------------------------------

// Every obstacle against leaf sphere l on joint j: float32 screen at cf,
// float64 terms at the exact centre.  Adds the cost, returns dC/dc.
static __host__ __device__ double3 env_force(const ClrEnv e, const double (*T)[12], int j, float4 l, float3 cf,
                                             double m, double *cost)
{
    double3 g = d3(0.0, 0.0, 0.0), c = g;
    bool have = false;
    const float r = l.w, keep = -kScreen - (float)m;   // kept when sd_f < m + kScreen
    auto centre = [&]() {
        if (!have) {
            c = place(T, j, l);
            have = true;
        }
        return c;
    };
    const float4 *p = e.rec;
    for (int i = 0; i < e.n.ns; i++) {
        const float4 s = p[i];
        if (-sd_point_f(sub(cf, f3(s.x, s.y, s.z)), r + s.w) > keep)
            point_term(sub(centre(), d3(s.x, s.y, s.z)), (double)r + s.w, m, cost, &g);
    }
    p += e.n.ns;
    for (int k = 0; k < 2; k++) {
        const int n = k ? e.n.nzc : e.n.nc;
        for (int i = 0; i < n; i++) {
            const float4 a = p[2 * i], v = p[2 * i + 1];   // (x1, y1, z1, r) (xv, yv, zv, 1/|v|^2)
            if (-sd_capsule_f(cf, r, a, v, k) > keep) capsule_term(centre(), r, a, v, k, m, cost, &g);
        }
        p += 2 * n;
    }
    for (int k = 0; k < 2; k++) {
        const int n = k ? e.n.nzb : e.n.ncb;
        for (int i = 0; i < n; i++) {
            const float4 c0 = p[4 * i], c1 = p[4 * i + 1], c2 = p[4 * i + 2], c3 = p[4 * i + 3];
            // z-aligned: the reference reads the xy parts of axes 1 and 2 and world z
            const float3 a1 = f3(c1.x, c1.y, k ? 0.0f : c1.z), a2 = f3(c2.x, c2.y, k ? 0.0f : c2.z),
                         a3 = k ? f3(0.0f, 0.0f, 1.0f) : f3(c3.x, c3.y, c3.z), ce = f3(c0.x, c0.y, c0.z),
                         h = f3(c0.w, c1.w, c2.w);
            if (-sd_box_f(cf, r, ce, a1, a2, a3, h) > keep) box_term(centre(), r, ce, a1, a2, a3, h, m, cost, &g);
        }
        p += 4 * n;
    }
    return g;
}

// Smallest float32 signed distance of sphere (cf, r) to any obstacle.
static __host__ __device__ float env_min_sd(const ClrEnv e, float3 cf, float r)
{
    float best = 3.4e38f;
    const float4 *p = e.rec;
    for (int i = 0; i < e.n.ns; i++) best = fminf(best, sd_point_f(sub(cf, f3(p[i].x, p[i].y, p[i].z)), r + p[i].w));
    p += e.n.ns;
    for (int k = 0; k < 2; k++) {
        const int n = k ? e.n.nzc : e.n.nc;
        for (int i = 0; i < n; i++) best = fminf(best, sd_capsule_f(cf, r, p[2 * i], p[2 * i + 1], k));
        p += 2 * n;
    }
    for (int k = 0; k < 2; k++) {
        const int n = k ? e.n.nzb : e.n.ncb;
        for (int i = 0; i < n; i++) {
            const float4 c0 = p[4 * i], c1 = p[4 * i + 1], c2 = p[4 * i + 2], c3 = p[4 * i + 3];
            best = fminf(best, sd_box_f(cf, r, f3(c0.x, c0.y, c0.z), f3(c1.x, c1.y, k ? 0.0f : c1.z),
                                        f3(c2.x, c2.y, k ? 0.0f : c2.z), k ? f3(0.0f, 0.0f, 1.0f) : f3(c3.x, c3.y, c3.z),
                                        f3(c0.w, c1.w, c2.w)));
        }
        p += 4 * n;
    }
    return best;
}

// Smallest signed distance of configuration q's env leaf spheres to the obstacles.
static __host__ __device__ float min_clearance(const ClrModel &M, const ClrEnv e, const float *q)
{
    double T[kClrMaxJoints][12];
    float Tf[kClrMaxJoints][12];
    fk(M, q, T);
    for (int j = 0; j < M.nj; j++)
        for (int k = 0; k < 12; k++) Tf[j][k] = (float)T[j][k];
    float best = 3.4e38f;
    for (int i = 0; i < M.n_leaf; i++) {
        const float4 l = M.leaf[i];
        best = fminf(best, env_min_sd(e, place(Tf, M.leaf_joint[i], l), l.w));
    }
    return best;
}

// Cost of configuration q (dof floats); grad[d] = scale * dC/dq[d] for every dof.
static __host__ __device__ __noinline__ float cost_grad(const ClrModel &M, const ClrEnv e, const float *q, float mf,
                                                        float scale_f, float *grad)
{
    double T[kClrMaxJoints][12];
    float Tf[kClrMaxJoints][12];   // float32 copy for the screen
    fk(M, q, T);
    for (int j = 0; j < M.nj; j++)
        for (int k = 0; k < 12; k++) Tf[j][k] = (float)T[j][k];
    // per joint: summed force (0..2) and moment about the joint's own origin (3..5)
    double F[kClrMaxJoints][6];
    for (int j = 0; j < M.nj; j++)
        for (int k = 0; k < 6; k++) F[j][k] = 0.0;
    const double m = mf;
    double cost = 0.0;
    auto push = [&](int j, float4 s, double3 g) {   // force g on the sphere at s in joint j's frame
        if (j < 0) return;
        const double3 mo = cross(lever(T, j, s), g);
        F[j][0] += g.x;
        F[j][1] += g.y;
        F[j][2] += g.z;
        F[j][3] += mo.x;
        F[j][4] += mo.y;
        F[j][5] += mo.z;
    };
    for (int i = 0; i < M.n_leaf; i++) {
        const float4 l = M.leaf[i];
        const int j = M.leaf_joint[i];
        const double3 g = env_force(e, T, j, l, place(Tf, j, l), m, &cost);
        if (g.x != 0.0 || g.y != 0.0 || g.z != 0.0) push(j, l, g);
    }
    for (int i = 0; i < M.n_pair; i++) {
        const float4 a = M.pair_a[i], b = M.pair_b[i];
        const int2 j = M.pair_joint[i];
        if (-sd_point_f(sub(place(Tf, j.x, a), place(Tf, j.y, b)), a.w + b.w) <= -kScreen - mf) continue;
        double3 g = d3(0.0, 0.0, 0.0);
        point_term(sub(place(T, j.x, a), place(T, j.y, b)), (double)a.w + b.w, m, &cost, &g);
        push(j.x, a, g);
        push(j.y, b, scale(-1.0, g));
    }
    // tips to base: each joint moves everything it carries
    for (int j = M.nj - 1; j >= 0; j--) {
        const prrtc_joint_def &J = M.joints[j];
        const double *t = T[j];
        const double3 axis = d3(t[2], t[6], t[10]);
        const double3 G = d3(F[j][0], F[j][1], F[j][2]), Mo = d3(F[j][3], F[j][4], F[j][5]);
        grad[J.q] = (float)(scale_f * dot(axis, J.revolute ? Mo : G));
        const int p = M.joint_parent[j];
        if (p >= 0) {   // shift the moment to the parent's origin
            const double *tp = T[p];
            const double3 mo = cross(d3(t[3] - tp[3], t[7] - tp[7], t[11] - tp[11]), G);
            F[p][0] += G.x;
            F[p][1] += G.y;
            F[p][2] += G.z;
            F[p][3] += Mo.x + mo.x;
            F[p][4] += Mo.y + mo.y;
            F[p][5] += Mo.z + mo.z;
        }
    }
    return (float)cost;
}

}  // namespace clr
}  // namespace prrtc
