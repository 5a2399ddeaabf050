/*
 * Oracle: CPU restatement of pRRTC's collision checker and planner.
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Compiled with -ffp-contract=off
 * so float expressions round the same way on x86-64 and aarch64; fused
 * operations appear only where written as fmaf(), mirroring the GPU code
 * (pRRTC compiled by nvcc contracts a*b+c into fused multiply-adds).
 *
 * Robot models come from the generated C tables in
 * prrtc_gb300/csrc/robots/<robot>_model.h (fitted to the reference's
 * generated checkers by prrtc_gb300/robots/extract.py); the float64 FK here
 * walks those tables generically and shares no code with the CUDA path.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <time.h>
#include <stdlib.h>
#include <string.h>

#include "../prrtc_gb300/csrc/robots/sphere_model.h"
#include "../prrtc_gb300/csrc/robots/panda_model.h"
#include "../prrtc_gb300/csrc/robots/fetch_model.h"
#include "../prrtc_gb300/csrc/robots/baxter_model.h"

typedef struct {
    int dof, nj, ns, neg, nsg, nsched;
    const prrtc_joint_def *joints;
    const prrtc_sphere_def *spheres;
    const prrtc_group_def *env_groups;
    const short *env_leaves;
    const prrtc_group_def *self_groups;
    const short (*self_pairs)[2];
    const prrtc_sched_def *sched;
    float scale[14], offset[14];   /* Robots.hh get_s_m / get_s_a */
} robot_t;

#define ROBOT_ENTRY(R)                                                                                  \
    {k##R##Dof, k##R##NumJoints, k##R##NumSpheres, k##R##NumEnvGroups, k##R##NumSelfGroups,           \
     k##R##NumSchedule, k##R##Joints, k##R##Spheres, k##R##EnvGroups, k##R##EnvLeaves, k##R##SelfGroups, \
     k##R##SelfPairs, k##R##Schedule, {0}, {0}}

static robot_t g_robots[4] = {ROBOT_ENTRY(Sphere), ROBOT_ENTRY(Panda), ROBOT_ENTRY(Fetch), ROBOT_ENTRY(Baxter)};
static const float k_scale[4][14] = {
    {10.0f, 10.0f, 10.0f},
    {5.9342f, 3.6652f, 5.9342f, 3.2289f, 5.9342f, 3.9095999999999997f, 5.9342f},
    {0.38615f, 3.2112f, 2.739f, 6.28318f, 4.502f, 6.28318f, 4.32f, 6.28318f},
    {3.40335987756f, 3.194f, 6.10835987756f, 2.6679999999999997f, 6.118f, 3.66479632679f, 6.118f,
     3.40335987756f, 3.194f, 6.10835987756f, 2.6679999999999997f, 6.118f, 3.66479632679f, 6.118f}};
static const float k_offset[4][14] = {
    {-5.0f, -5.0f, -5.0f},
    {-2.9671f, -1.8326f, -2.9671f, -3.1416f, -2.9671f, -0.0873f, -2.9671f},
    {0.0f, -1.6056f, -1.221f, -3.14159f, -2.251f, -3.14159f, -2.16f, -3.14159f},
    {-1.70167993878f, -2.147f, -3.05417993878f, -0.05f, -3.059f, -1.57079632679f, -3.059f,
     -1.70167993878f, -2.147f, -3.05417993878f, -0.05f, -3.059f, -1.57079632679f, -3.059f}};

static const robot_t *robot_get(int r)
{
    if (r < 0 || r > 3) return NULL;
    robot_t *R = &g_robots[r];
    if (R->scale[0] == 0.0f) {
        memcpy(R->scale, k_scale[r], sizeof R->scale);
        memcpy(R->offset, k_offset[r], sizeof R->offset);
    }
    return R;
}

int oracle_dof(int robot)
{
    const robot_t *R = robot_get(robot);
    return R ? R->dof : -1;
}

int oracle_num_spheres(int robot)
{
    const robot_t *R = robot_get(robot);
    return R ? R->ns : -1;
}

int oracle_limits(int robot, float *scale, float *offset)
{
    const robot_t *R = robot_get(robot);
    if (!R) return -1;
    memcpy(scale, R->scale, sizeof(float) * R->dof);
    memcpy(offset, R->offset, sizeof(float) * R->dof);
    return 0;
}

/* ------------------------------------------------------------ float64 FK */

typedef struct {
    double T[14][12];     /* world frame of each joint, by config index */
} frames_t;

static void compose(const double *P, const float *F, double *A)
{
    for (int i = 0; i < 3; i++) {
        for (int k = 0; k < 3; k++)
            A[4 * i + k] = P[4 * i] * F[k] + P[4 * i + 1] * F[4 + k] + P[4 * i + 2] * F[8 + k];
        A[4 * i + 3] = P[4 * i] * F[3] + P[4 * i + 1] * F[7] + P[4 * i + 2] * F[11] + P[4 * i + 3];
    }
}

static void fk_frames(const robot_t *R, const double *q, frames_t *fr)
{
    static const double I[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    for (int j = 0; j < R->nj; j++) {
        const prrtc_joint_def *J = &R->joints[j];
        const double *P = J->parent < 0 ? I : fr->T[J->parent];
        double A[12];
        compose(P, J->F, A);
        double *T = fr->T[J->q];
        const double th = q[J->q];
        if (J->revolute) {
            const double c = cos(th), s = sin(th);
            for (int i = 0; i < 3; i++) {
                T[4 * i] = c * A[4 * i] + s * A[4 * i + 1];
                T[4 * i + 1] = c * A[4 * i + 1] - s * A[4 * i];
                T[4 * i + 2] = A[4 * i + 2];
                T[4 * i + 3] = A[4 * i + 3];
            }
        } else {
            for (int i = 0; i < 3; i++) {
                T[4 * i] = A[4 * i];
                T[4 * i + 1] = A[4 * i + 1];
                T[4 * i + 2] = A[4 * i + 2];
                T[4 * i + 3] = A[4 * i + 3] + th * A[4 * i + 2];
            }
        }
    }
}

static void sphere_centre(const robot_t *R, const frames_t *fr, int s, double *c)
{
    const prrtc_sphere_def *S = &R->spheres[s];
    if (S->frame < 0) {
        c[0] = S->x;
        c[1] = S->y;
        c[2] = S->z;
        return;
    }
    const double *T = fr->T[S->frame];
    for (int i = 0; i < 3; i++) c[i] = T[4 * i] * S->x + T[4 * i + 1] * S->y + T[4 * i + 2] * S->z + T[4 * i + 3];
}

int oracle_fk_spheres(int robot, const double *q, long n, double *out)
{
    const robot_t *R = robot_get(robot);
    if (!R) return -1;
#pragma omp parallel for schedule(static, 256)
    for (long i = 0; i < n; i++) {
        frames_t fr;
        fk_frames(R, q + i * R->dof, &fr);
        for (int s = 0; s < R->ns; s++) {
            double *o = out + (i * R->ns + s) * 4;
            sphere_centre(R, &fr, s, o);
            o[3] = R->spheres[s].r;
        }
    }
    return 0;
}

/* ------------------------------------------- reference primitive tests (float) */
/* Written exactly as src/planning/utils.cuh:58-242 evaluates them. */

static int env_hit_f(const oracle_env *e, float x, float y, float z, float r, int64_t *cnt)
{
    for (int i = 0; i < e->ns; i++) {
        const float *s = e->spheres + 4 * i;
        const float xs = s[0] - x, ys = s[1] - y, zs = s[2] - z;
        const float sum = xs * xs + ys * ys + zs * zs;
        const float rs = s[3] + r;
        if (cnt) cnt[ORC_SPHERE]++;
        if (sum - rs * rs < 0) return 1;
    }
    for (int i = 0; i < e->nc; i++) {
        const float *c = e->capsules + 8 * i;
        const float dot = (x - c[0]) * c[3] + (y - c[1]) * c[4] + (z - c[2]) * c[5];
        const float cdf = fmaxf(fminf(dot * c[7], 1.0f), 0.0f);
        const float xs = x - (c[0] + c[3] * cdf), ys = y - (c[1] + c[4] * cdf), zs = z - (c[2] + c[5] * cdf);
        const float sum = xs * xs + ys * ys + zs * zs;
        const float rs = r + c[6];
        if (cnt) cnt[ORC_CAPSULE]++;
        if (sum - rs * rs < 0) return 1;
    }
    for (int i = 0; i < e->nzc; i++) {
        const float *c = e->zcapsules + 8 * i;
        const float dot = (z - c[2]) * c[5];
        const float cdf = fmaxf(fminf(dot * c[7], 1.0f), 0.0f);
        const float xs = x - c[0], ys = y - c[1], zs = z - (c[2] + c[5] * cdf);
        const float sum = xs * xs + ys * ys + zs * zs;
        const float rs = r + c[6];
        if (cnt) cnt[ORC_ZCAPSULE]++;
        if (sum - rs * rs < 0) return 1;
    }
    const float rsq = r * r;
    for (int i = 0; i < e->ncb; i++) {
        const float *c = e->cuboids + 15 * i;
        const float xs = x - c[0], ys = y - c[1], zs = z - c[2];
        const float a1 = fmaxf(0.0f, fabsf(c[3] * xs + c[4] * ys + c[5] * zs) - c[12]);
        const float a2 = fmaxf(0.0f, fabsf(c[6] * xs + c[7] * ys + c[8] * zs) - c[13]);
        const float a3 = fmaxf(0.0f, fabsf(c[9] * xs + c[10] * ys + c[11] * zs) - c[14]);
        const float sum = a1 * a1 + a2 * a2 + a3 * a3;
        if (cnt) cnt[ORC_CUBOID]++;
        if (sum - rsq < 0) return 1;
    }
    for (int i = 0; i < e->nzb; i++) {
        const float *c = e->zcuboids + 15 * i;
        const float xs = x - c[0], ys = y - c[1], zs = z - c[2];
        const float a1 = fmaxf(0.0f, fabsf(c[3] * xs + c[4] * ys) - c[12]);
        const float a2 = fmaxf(0.0f, fabsf(c[6] * xs + c[7] * ys) - c[13]);
        const float a3 = fmaxf(0.0f, fabsf(zs) - c[14]);
        const float sum = a1 * a1 + a2 * a2 + a3 * a3;
        if (cnt) cnt[ORC_ZCUBOID]++;
        if (sum - rsq < 0) return 1;
    }
    return 0;
}

static int pair_hit_f(const float *a, const float *b, int64_t *cnt)
{
    const float xs = a[0] - b[0], ys = a[1] - b[1], zs = a[2] - b[2];
    const float sum = xs * xs + ys * ys + zs * zs;
    const float rs = a[3] + b[3];
    if (cnt) cnt[ORC_SELF]++;
    return sum - rs * rs < 0;
}

/* ----------------------------------------------- float64 signed distances */

static double sd_env(const oracle_env *e, const double *p, double r, double *min_abs)
{
    double best = DBL_MAX;
#define ACC(v)                                  \
    do {                                        \
        const double v_ = (v);                  \
        if (v_ < best) best = v_;               \
        if (min_abs && fabs(v_) < *min_abs) *min_abs = fabs(v_); \
    } while (0)
    for (int i = 0; i < e->ns; i++) {
        const float *s = e->spheres + 4 * i;
        const double dx = p[0] - s[0], dy = p[1] - s[1], dz = p[2] - s[2];
        ACC(sqrt(dx * dx + dy * dy + dz * dz) - (r + s[3]));
    }
    for (int k = 0; k < 2; k++) {
        const float *base = k ? e->zcapsules : e->capsules;
        const int n = k ? e->nzc : e->nc;
        for (int i = 0; i < n; i++) {
            const float *c = base + 8 * i;
            double t = k ? (p[2] - c[2]) * c[5] * (double)c[7]
                         : ((p[0] - c[0]) * c[3] + (p[1] - c[1]) * c[4] + (p[2] - c[2]) * c[5]) * (double)c[7];
            t = t < 0 ? 0 : (t > 1 ? 1 : t);
            const double qx = k ? c[0] : c[0] + c[3] * t, qy = k ? c[1] : c[1] + c[4] * t, qz = c[2] + c[5] * t;
            const double dx = p[0] - qx, dy = p[1] - qy, dz = p[2] - qz;
            ACC(sqrt(dx * dx + dy * dy + dz * dz) - (r + c[6]));
        }
    }
    for (int k = 0; k < 2; k++) {
        const float *base = k ? e->zcuboids : e->cuboids;
        const int n = k ? e->nzb : e->ncb;
        for (int i = 0; i < n; i++) {
            const float *c = base + 15 * i;
            const double xs = p[0] - c[0], ys = p[1] - c[1], zs = p[2] - c[2];
            double a1, a2, a3;
            if (k) {
                a1 = fabs(c[3] * xs + c[4] * ys) - c[12];
                a2 = fabs(c[6] * xs + c[7] * ys) - c[13];
                a3 = fabs(zs) - c[14];
            } else {
                a1 = fabs(c[3] * xs + c[4] * ys + c[5] * zs) - c[12];
                a2 = fabs(c[6] * xs + c[7] * ys + c[8] * zs) - c[13];
                a3 = fabs(c[9] * xs + c[10] * ys + c[11] * zs) - c[14];
            }
            a1 = a1 > 0 ? a1 : 0;
            a2 = a2 > 0 ? a2 : 0;
            a3 = a3 > 0 ? a3 : 0;
            ACC(sqrt(a1 * a1 + a2 * a2 + a3 * a3) - r);
        }
    }
#undef ACC
    return best;
}

static double sd_pair(const double *a, double ra, const double *b, double rb)
{
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return sqrt(dx * dx + dy * dy + dz * dz) - (ra + rb);
}

/* ------------------------------------------------------------- the checker */

typedef struct {
    double c[128][3];
    float f[128][4];
    unsigned char have[128];
} centres_t;

static const float *centre_f(const robot_t *R, const frames_t *fr, centres_t *C, int s)
{
    if (!C->have[s]) {
        sphere_centre(R, fr, s, C->c[s]);
        C->f[s][0] = (float)C->c[s][0];
        C->f[s][1] = (float)C->c[s][1];
        C->f[s][2] = (float)C->c[s][2];
        C->f[s][3] = R->spheres[s].r;
        C->have[s] = 1;
    }
    return C->f[s];
}

/* 1 when free (reference semantics); counts executed tests */
static int check_one(const robot_t *R, const float *qf, const oracle_env *e, int64_t *cnt)
{
    double q[14];
    for (int d = 0; d < R->dof; d++) q[d] = qf[d];
    frames_t fr;
    fk_frames(R, q, &fr);
    centres_t C;
    memset(C.have, 0, sizeof C.have);
    for (int k = 0; k < R->nsched; k++) {
        const prrtc_sched_def *it = &R->sched[k];
        if (it->kind == 0) {
            const prrtc_group_def *G = &R->env_groups[it->index];
            if (G->gate_a >= 0) {
                const float *s = centre_f(R, &fr, &C, G->gate_a);
                if (!env_hit_f(e, s[0], s[1], s[2], s[3], cnt)) continue;
            }
            for (int l = 0; l < G->count; l++) {
                const float *s = centre_f(R, &fr, &C, R->env_leaves[G->first + l]);
                if (env_hit_f(e, s[0], s[1], s[2], s[3], cnt)) return 0;
            }
        } else {
            const prrtc_group_def *G = &R->self_groups[it->index];
            const float *a = centre_f(R, &fr, &C, G->gate_a);
            const float *b = centre_f(R, &fr, &C, G->gate_b);
            if (!pair_hit_f(a, b, cnt)) continue;
            for (int l = 0; l < G->count; l++) {
                const short *pr = R->self_pairs[G->first + l];
                const float *x = centre_f(R, &fr, &C, pr[0]);
                const float *y = centre_f(R, &fr, &C, pr[1]);
                if (pair_hit_f(x, y, cnt)) return 0;
            }
        }
    }
    return 1;
}

/* min |signed distance| over every test the hierarchy contains */
static double margin_one(const robot_t *R, const float *qf, const oracle_env *e)
{
    double q[14];
    for (int d = 0; d < R->dof; d++) q[d] = qf[d];
    frames_t fr;
    fk_frames(R, q, &fr);
    double c[128][3];
    for (int s = 0; s < R->ns; s++) sphere_centre(R, &fr, s, c[s]);
    double m = DBL_MAX;
    for (int g = 0; g < R->neg; g++) {
        const prrtc_group_def *G = &R->env_groups[g];
        if (G->gate_a >= 0) sd_env(e, c[G->gate_a], R->spheres[G->gate_a].r, &m);
        for (int l = 0; l < G->count; l++) {
            const int s = R->env_leaves[G->first + l];
            sd_env(e, c[s], R->spheres[s].r, &m);
        }
    }
    for (int g = 0; g < R->nsg; g++) {
        const prrtc_group_def *G = &R->self_groups[g];
        double v = fabs(sd_pair(c[G->gate_a], R->spheres[G->gate_a].r, c[G->gate_b], R->spheres[G->gate_b].r));
        if (v < m) m = v;
        for (int l = 0; l < G->count; l++) {
            const short *pr = R->self_pairs[G->first + l];
            v = fabs(sd_pair(c[pr[0]], R->spheres[pr[0]].r, c[pr[1]], R->spheres[pr[1]].r));
            if (v < m) m = v;
        }
    }
    return m;
}

int oracle_check(int robot, const float *q, long n, const oracle_env *env, uint8_t *out_free, double *margin,
                 int64_t *counts)
{
    const robot_t *R = robot_get(robot);
    if (!R || !env) return -1;
    int64_t tot[ORC_NCOUNT] = {0};
#pragma omp parallel
    {
        int64_t loc[ORC_NCOUNT] = {0};
#pragma omp for schedule(static, 256)
        for (long i = 0; i < n; i++) {
            out_free[i] = (uint8_t)check_one(R, q + i * R->dof, env, counts ? loc : NULL);
            if (margin) margin[i] = margin_one(R, q + i * R->dof, env);
        }
        if (counts) {
#pragma omp critical
            for (int k = 0; k < ORC_NCOUNT; k++) tot[k] += loc[k];
        }
    }
    if (counts)
        for (int k = 0; k < ORC_NCOUNT; k++) counts[k] += tot[k];
    return 0;
}

static int edge_free(const robot_t *R, const float *a, const float *b, int g, const oracle_env *e, int64_t *nchk)
{
    float step[14], p[14];
    const float fg = (float)g;
    for (int d = 0; d < R->dof; d++) step[d] = (b[d] - a[d]) / fg;
    for (int k = 1; k <= g; k++) {
        for (int d = 0; d < R->dof; d++) p[d] = a[d] + (float)k * step[d];
        if (nchk) (*nchk)++;
        if (!check_one(R, p, e, NULL)) return 0;
    }
    return 1;
}

int oracle_check_edges(int robot, const float *a, const float *b, long n, int g, const oracle_env *env,
                       uint8_t *out_free)
{
    const robot_t *R = robot_get(robot);
    if (!R || !env || g < 1) return -1;
#pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < n; i++) out_free[i] = (uint8_t)edge_free(R, a + i * R->dof, b + i * R->dof, g, env, NULL);
    return 0;
}

int oracle_clearance(int robot, const float *qf, long n, const oracle_env *e, double *out)
{
    const robot_t *R = robot_get(robot);
    if (!R || !e) return -1;
#pragma omp parallel for schedule(static, 256)
    for (long i = 0; i < n; i++) {
        double q[14];
        for (int d = 0; d < R->dof; d++) q[d] = qf[i * R->dof + d];
        frames_t fr;
        fk_frames(R, q, &fr);
        double c[128][3];
        for (int s = 0; s < R->ns; s++) sphere_centre(R, &fr, s, c[s]);
        double m = DBL_MAX;
        for (int g = 0; g < R->neg; g++) {
            const prrtc_group_def *G = &R->env_groups[g];
            for (int l = 0; l < G->count; l++) {
                const int s = R->env_leaves[G->first + l];
                const double v = sd_env(e, c[s], R->spheres[s].r, NULL);
                if (v < m) m = v;
            }
        }
        for (int g = 0; g < R->nsg; g++) {
            const prrtc_group_def *G = &R->self_groups[g];
            for (int l = 0; l < G->count; l++) {
                const short *pr = R->self_pairs[G->first + l];
                const double v = sd_pair(c[pr[0]], R->spheres[pr[0]].r, c[pr[1]], R->spheres[pr[1]].r);
                if (v < m) m = v;
            }
        }
        out[i] = m;
    }
    return 0;
}

/* ------------------------------------------ float64 clearance cost + gradient */

/* Adds 1/2 max(0, m - sd)^2 and its gradient in the centre (-phi * dsd/dc). */
static void hinge64(double sd, const double *gsd, double m, double *cost, double *g)
{
    const double phi = m - sd;
    if (phi <= 0) return;
    *cost += 0.5 * phi * phi;
    for (int k = 0; k < 3; k++) g[k] -= phi * gsd[k];
}

static void point64(const double *d, double rsum, double m, double *cost, double *g)
{
    const double len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double u[3] = {len > 0 ? d[0] / len : 0, len > 0 ? d[1] / len : 0, len > 0 ? d[2] / len : 0};
    hinge64(len - rsum, u, m, cost, g);
}

/* Signed distance of a sphere to a box: centre ce, unit axes ax[3][3], half extents h. */
static void box64(const double *p, double r, const double *ce, const double ax[3][3], const double *h, double m,
                  double *cost, double *g)
{
    double u[3], q[3], s[3];
    for (int a = 0; a < 3; a++) {
        u[a] = ax[a][0] * (p[0] - ce[0]) + ax[a][1] * (p[1] - ce[1]) + ax[a][2] * (p[2] - ce[2]);
        s[a] = u[a] < 0 ? -1.0 : 1.0;
        q[a] = fabs(u[a]) - h[a];
    }
    double sd, gsd[3] = {0, 0, 0};
    if (q[0] > 0 || q[1] > 0 || q[2] > 0) {
        double o2 = 0, w[3];
        for (int a = 0; a < 3; a++) {
            w[a] = (q[a] > 0 ? q[a] : 0) * s[a];
            o2 += w[a] * w[a];
        }
        const double o = sqrt(o2);
        sd = o - r;
        for (int a = 0; a < 3; a++)
            for (int k = 0; k < 3; k++) gsd[k] += w[a] * ax[a][k] / o;
    } else {
        int a = 0;
        if (q[1] > q[a]) a = 1;
        if (q[2] > q[a]) a = 2;
        sd = q[a] - r;
        for (int k = 0; k < 3; k++) gsd[k] = s[a] * ax[a][k];
    }
    hinge64(sd, gsd, m, cost, g);
}

static void env_cost64(const oracle_env *e, const double *p, double r, double m, double *cost, double *g)
{
    for (int i = 0; i < e->ns; i++) {
        const float *s = e->spheres + 4 * i;
        const double d[3] = {p[0] - s[0], p[1] - s[1], p[2] - s[2]};
        point64(d, r + s[3], m, cost, g);
    }
    for (int k = 0; k < 2; k++) {
        const float *base = k ? e->zcapsules : e->capsules;
        const int n = k ? e->nzc : e->nc;
        for (int i = 0; i < n; i++) {
            const float *c = base + 8 * i;   /* p1 (0..2), v (3..5), r (6), 1/|v|^2 (7) */
            double t = k ? (p[2] - c[2]) * c[5] * (double)c[7]
                         : ((p[0] - c[0]) * c[3] + (p[1] - c[1]) * c[4] + (p[2] - c[2]) * c[5]) * (double)c[7];
            t = t < 0 ? 0 : (t > 1 ? 1 : t);
            const double d[3] = {p[0] - (k ? c[0] : c[0] + c[3] * t), p[1] - (k ? c[1] : c[1] + c[4] * t),
                                 p[2] - (c[2] + c[5] * t)};
            point64(d, r + c[6], m, cost, g);
        }
    }
    for (int k = 0; k < 2; k++) {
        const float *base = k ? e->zcuboids : e->cuboids;
        const int n = k ? e->nzb : e->ncb;
        for (int i = 0; i < n; i++) {
            const float *c = base + 15 * i;  /* centre (0..2), axes (3..11), half extents (12..14) */
            const double ce[3] = {c[0], c[1], c[2]}, h[3] = {c[12], c[13], c[14]};
            double ax[3][3];
            if (k) {
                const double z[3][3] = {{c[3], c[4], 0}, {c[6], c[7], 0}, {0, 0, 1}};
                memcpy(ax, z, sizeof ax);
            } else {
                for (int a = 0; a < 3; a++)
                    for (int j = 0; j < 3; j++) ax[a][j] = c[3 + 3 * a + j];
            }
            box64(p, r, ce, ax, h, m, cost, g);
        }
    }
}

/* grad[q] += g . dc/dq over every joint that moves the sphere on `frame`. */
static void jacobian_t(const robot_t *R, const frames_t *fr, const int *pos, int frame, const double *c,
                       const double *g, double *grad)
{
    for (int f = frame; f >= 0; f = R->joints[pos[f]].parent) {
        const prrtc_joint_def *J = &R->joints[pos[f]];
        const double *T = fr->T[f];
        const double z[3] = {T[2], T[6], T[10]};
        if (J->revolute) {
            const double v[3] = {c[0] - T[3], c[1] - T[7], c[2] - T[11]};
            const double dc[3] = {z[1] * v[2] - z[2] * v[1], z[2] * v[0] - z[0] * v[2], z[0] * v[1] - z[1] * v[0]};
            grad[f] += g[0] * dc[0] + g[1] * dc[1] + g[2] * dc[2];
        } else {
            grad[f] += g[0] * z[0] + g[1] * z[1] + g[2] * z[2];
        }
    }
}

int oracle_cost_grad(int robot, const double *q, long n, const oracle_env *e, double margin, double *cost,
                     double *grad)
{
    const robot_t *R = robot_get(robot);
    if (!R || !e) return -1;
    int pos[14];
    for (int j = 0; j < R->nj; j++) pos[R->joints[j].q] = j;
#pragma omp parallel for schedule(static, 16)
    for (long i = 0; i < n; i++) {
        const double *qi = q + i * R->dof;
        double *gi = grad + i * R->dof;
        frames_t fr;
        fk_frames(R, qi, &fr);
        double c[128][3];
        for (int s = 0; s < R->ns; s++) sphere_centre(R, &fr, s, c[s]);
        for (int d = 0; d < R->dof; d++) gi[d] = 0;
        double C = 0;
        for (int gr = 0; gr < R->neg; gr++) {
            const prrtc_group_def *G = &R->env_groups[gr];
            for (int l = 0; l < G->count; l++) {
                const int s = R->env_leaves[G->first + l];
                double g[3] = {0, 0, 0};
                env_cost64(e, c[s], R->spheres[s].r, margin, &C, g);
                jacobian_t(R, &fr, pos, R->spheres[s].frame, c[s], g, gi);
            }
        }
        for (int gr = 0; gr < R->nsg; gr++) {
            const prrtc_group_def *G = &R->self_groups[gr];
            for (int l = 0; l < G->count; l++) {
                const int a = R->self_pairs[G->first + l][0], b = R->self_pairs[G->first + l][1];
                const double d[3] = {c[a][0] - c[b][0], c[a][1] - c[b][1], c[a][2] - c[b][2]};
                double g[3] = {0, 0, 0};
                point64(d, (double)R->spheres[a].r + R->spheres[b].r, margin, &C, g);
                const double ng[3] = {-g[0], -g[1], -g[2]};
                jacobian_t(R, &fr, pos, R->spheres[a].frame, c[a], g, gi);
                jacobian_t(R, &fr, pos, R->spheres[b].frame, c[b], ng, gi);
            }
        }
        cost[i] = C;
    }
    return 0;
}

/* ------------------------------------------------------------- the planner */

typedef struct {
    float *nodes;    /* [cap][dof] */
    int *parents;
    float *radii;
    int count, cap;
} tree_t;

static int tree_push(tree_t *t, int dof)
{
    if (t->count == t->cap) {
        const int nc = t->cap ? 2 * t->cap : 1024;
        float *nn = realloc(t->nodes, sizeof(float) * (size_t)nc * dof);
        int *np = realloc(t->parents, sizeof(int) * (size_t)nc);
        float *nr = realloc(t->radii, sizeof(float) * (size_t)nc);
        if (!nn || !np || !nr) {
            /* keep whichever blocks moved so they are freed later */
            if (nn) t->nodes = nn;
            if (np) t->parents = np;
            if (nr) t->radii = nr;
            return -1;
        }
        t->nodes = nn;
        t->parents = np;
        t->radii = nr;
        t->cap = nc;
    }
    return t->count++;
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static uint64_t splitmix64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* halton_next (pRRTC.cu:81-105), float32 as written there */
static void halton_next(int D, const float *b, float *n, float *d, float *out)
{
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

static int nearest(const tree_t *t, int D, const float *q, float *dsq)
{
    float best = FLT_MAX;
    int bi = 0;
    for (int i = 0; i < t->count; i++) {
        const float *x = t->nodes + (size_t)i * D;
        float a = 0.0f;
        for (int d = 0; d < D; d++) {
            const float df = x[d] - q[d];
            a = fmaf(df, df, a);
        }
        if (a < best) {
            best = a;
            bi = i;
        }
    }
    *dsq = best;
    return bi;
}

/* dynamic-domain radius updates (pRRTC.cu:456-468 grow, 584-598 shrink) */
static void dd_grow_one(float *r, float alpha)
{
    if (*r != FLT_MAX) *r = *r * (1.0f + alpha);
}

static void dd_shrink_one(float *r, float alpha, float radius0, float rmin)
{
    *r = (*r == FLT_MAX) ? radius0 : fmaxf(*r * (1.0f - alpha), rmin);
}

int oracle_halton(int dof, const float *bases16, int lanes, int steps, const float *scale, const float *offset,
                  float *raw, float *cfg)
{
    if (dof < 1 || dof > 16 || lanes < 0 || steps < 0 || !bases16 || !scale || !offset || !raw || !cfg) return -1;
    for (int l = 0; l < lanes; l++) {
        float b[16], n[16], d[16], out[16];
        for (int i = 0; i < dof; i++) {
            b[i] = bases16[16 * l + i];
            n[i] = 0.0f;
            d[i] = 1.0f;
        }
        for (int s = 0; s < steps; s++) {
            halton_next(dof, b, n, d, out);
            const size_t o = ((size_t)l * steps + s) * dof;
            for (int i = 0; i < dof; i++) {
                raw[o + i] = out[i];
                cfg[o + i] = fmaf(out[i], scale[i], offset[i]);
            }
        }
    }
    return 0;
}

int oracle_nearest(int dof, const float *nodes, int count, const float *q, int nq, int *out_i, float *out_d)
{
    if (dof < 1 || count < 0 || nq < 0 || (count && !nodes) || (nq && (!q || !out_i || !out_d))) return -1;
    tree_t t;
    memset(&t, 0, sizeof t);
    t.nodes = (float *)nodes;
    t.count = t.cap = count;
    for (int k = 0; k < nq; k++) out_i[k] = nearest(&t, dof, q + (size_t)k * dof, &out_d[k]);
    return 0;
}

int oracle_dd_apply(float *radii, int n, const uint8_t *ops, int nops, float alpha, float radius0, float rmin)
{
    if (n < 0 || nops < 0 || (n && (!radii || (nops && !ops)))) return -1;
    for (int i = 0; i < n; i++)
        for (int k = 0; k < nops; k++) {
            if (ops[(size_t)i * nops + k])
                dd_shrink_one(&radii[i], alpha, radius0, rmin);
            else
                dd_grow_one(&radii[i], alpha);
        }
    return 0;
}

static float trace(const tree_t *t, int D, int start, float *seg, int seg_cap, int *nseg, int *root)
{
    float cost = 0.0f;
    int cur = start, n = 0;
    while (t->parents[cur] != cur) {
        const int par = t->parents[cur];
        float acc = 0.0f;
        for (int d = 0; d < D; d++) {
            const float df = t->nodes[(size_t)cur * D + d] - t->nodes[(size_t)par * D + d];
            acc = fmaf(df, df, acc);
        }
        cost += sqrtf(acc);
        if (n < seg_cap) memcpy(seg + (size_t)n * D, t->nodes + (size_t)cur * D, sizeof(float) * D);
        n++;
        cur = par;
    }
    *nseg = n;
    *root = cur;
    return cost;
}

int oracle_solve(int robot, const float *start, const float *goals, int num_goals, const oracle_env *env,
                 const oracle_settings *S, const float *bases, float *path, int path_cap, oracle_result *res)
{
    const robot_t *R = robot_get(robot);
    if (!R || !start || !goals || num_goals < 1 || !env || !S || !res || S->num_new_configs < 1 ||
        S->granularity < 1)
        return -1;
    const int D = R->dof, L = S->num_new_configs, g = S->granularity;
    memset(res, 0, sizeof *res);
    tree_t T[2];
    memset(T, 0, sizeof T);
    float *hb = malloc(sizeof(float) * (size_t)L * D), *hn = malloc(sizeof(float) * (size_t)L * D),
          *hd = malloc(sizeof(float) * (size_t)L * D);
    int *tsel = calloc((size_t)L, sizeof(int)), *iters = calloc((size_t)L, sizeof(int));
    int rc = 0;
    if (!hb || !hn || !hd || !tsel || !iters) {
        rc = -2;
        goto done;
    }
    for (int l = 0; l < L; l++) {
        float pr[16] = {3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59};
        if (bases) {
            memcpy(pr, bases + 16 * l, sizeof pr);
        } else if (l != 0) {
            uint64_t st = 0x5eed0000ull + (uint64_t)l;
            for (int i = 15; i > 0; i--) {
                const int j = (int)(splitmix64(&st) % (uint64_t)(i + 1));
                const float tmp = pr[i];
                pr[i] = pr[j];
                pr[j] = tmp;
            }
        }
        for (int d = 0; d < D; d++) {
            hb[l * D + d] = pr[d];
            hn[l * D + d] = 0.0f;
            hd[l * D + d] = 1.0f;
        }
    }
    {
        const int i0 = tree_push(&T[0], D);
        if (i0 < 0) {
            rc = -2;
            goto done;
        }
        memcpy(T[0].nodes, start, sizeof(float) * D);
        T[0].parents[0] = 0;
        T[0].radii[0] = FLT_MAX;
        for (int k = 0; k < num_goals; k++) {
            const int ik = tree_push(&T[1], D);
            if (ik < 0) {
                rc = -2;
                goto done;
            }
            memcpy(T[1].nodes + (size_t)ik * D, goals + (size_t)k * D, sizeof(float) * D);
            T[1].parents[ik] = ik;
            T[1].radii[ik] = FLT_MAX;
        }
    }
    int solved = 0, win_iter = -1, junction_t = -1, junction_o = -1, win_t = 0;
    const float fg = (float)g;
    const double deadline = S->budget_s > 0 ? now_s() + S->budget_s : 0;
    while (!solved) {
        if (deadline > 0 && now_s() > deadline) {
            solved = -2;
            break;
        }
        for (int bid = 0; bid < L && !solved; bid++) {
            int iter = ++iters[bid];
            if (iter > S->max_iters) {
                solved = -1;
                break;
            }
            const int f0 = T[0].count, f1 = T[1].count;
            int t = tsel[bid];
            if (S->balance == 0 || iter == 1) {
                t = (bid < (L / 2)) ? 0 : 1;
            } else if (S->balance == 1 && 2 * abs(f0 - f1) < 3 * L) {
                const float ratio = f0 / (float)(f0 + f1);
                t = ((float)bid < L * (1.0f - ratio)) ? 0 : 1;
            } else if (S->balance == 1) {
                const float ratio = f0 / (float)(f0 + f1);
                t = ratio < S->tree_ratio ? 0 : 1;
            } else if (S->balance == 2) {
                const int ft = t == 0 ? f0 : f1, fo = t == 0 ? f1 : f0;
                const float ratio = abs(ft - fo) / (float)ft;
                if (ratio < S->tree_ratio) t = 1 - t;
            }
            tsel[bid] = t;
            const int o = 1 - t;
            float cfg[14], nn[14], step[14], p[14], vec[14], next[14];
            halton_next(D, hb + bid * D, hn + bid * D, hd + bid * D, cfg);
            for (int d = 0; d < D; d++) cfg[d] = fmaf(cfg[d], R->scale[d], R->offset[d]);
            float dsq;
            const int ni = nearest(&T[t], D, cfg, &dsq);
            const float dist = sqrtf(dsq);
            const float scale = fminf(1.0f, S->range / dist);
            if (S->dynamic_domain && T[t].radii[ni] < dist) continue;
            memcpy(nn, T[t].nodes + (size_t)ni * D, sizeof(float) * D);
            for (int d = 0; d < D; d++) {
                cfg[d] = fmaf(cfg[d] - nn[d], scale, nn[d]);
                step[d] = (cfg[d] - nn[d]) / fg;
            }
            int ok = 1;
            for (int k = 1; k <= g && ok; k++) {
                for (int d = 0; d < D; d++) p[d] = nn[d] + (float)k * step[d];
                res->checks++;
                ok = check_one(R, p, env, NULL);
            }
            if (!ok) {
                if (S->dynamic_domain) dd_shrink_one(&T[t].radii[ni], S->dd_alpha, S->dd_radius, S->dd_min_radius);
                continue;
            }
            int idx = tree_push(&T[t], D);
            if (idx < 0 || idx >= S->max_samples) {
                solved = -1;
                break;
            }
            T[t].parents[idx] = ni;
            T[t].radii[idx] = FLT_MAX;
            if (S->dynamic_domain) dd_grow_one(&T[t].radii[ni], S->dd_alpha);
            memcpy(T[t].nodes + (size_t)idx * D, cfg, sizeof(float) * D);
            /* connect */
            const int oi = nearest(&T[o], D, cfg, &dsq);
            const unsigned n_ext = (unsigned)ceilf(sqrtf(dsq) / S->range);
            for (int d = 0; d < D; d++) vec[d] = (T[o].nodes[(size_t)oi * D + d] - cfg[d]) / (float)n_ext;
            unsigned i_ext = 0;
            int parent = idx;
            while (i_ext < n_ext) {
                for (int d = 0; d < D; d++) {
                    next[d] = cfg[d] + vec[d];
                    step[d] = (next[d] - cfg[d]) / fg;
                }
                ok = 1;
                for (int k = 1; k <= g && ok; k++) {
                    for (int d = 0; d < D; d++) p[d] = cfg[d] + (float)k * step[d];
                    res->checks++;
                    ok = check_one(R, p, env, NULL);
                }
                if (!ok) break;
                idx = tree_push(&T[t], D);
                if (idx < 0 || idx >= S->max_samples) {
                    solved = -1;
                    break;
                }
                T[t].parents[idx] = parent;
                T[t].radii[idx] = FLT_MAX;
                memcpy(T[t].nodes + (size_t)idx * D, next, sizeof(float) * D);
                memcpy(cfg, next, sizeof(float) * D);
                parent = idx;
                i_ext++;
            }
            if (solved) break;
            if (i_ext == n_ext) {
                solved = 1;
                win_iter = iter;
                junction_t = idx;
                junction_o = oi;
                win_t = t;
            }
        }
    }
    res->start_tree_size = T[0].count;
    res->goal_tree_size = T[1].count;
    if (solved == 1) {
        const int t = win_t, o = 1 - t;
        float *seg[2];
        int nseg[2], root[2];
        seg[0] = malloc(sizeof(float) * (size_t)T[0].count * D);
        seg[1] = malloc(sizeof(float) * (size_t)T[1].count * D);
        if (!seg[0] || !seg[1]) {
            free(seg[0]);
            free(seg[1]);
            rc = -2;
            goto done;
        }
        float cost = trace(&T[t], D, junction_t, seg[t], T[t].count, &nseg[t], &root[t]);
        cost += trace(&T[o], D, junction_o, seg[o], T[o].count, &nseg[o], &root[o]);
        res->solved = 1;
        res->iters = win_iter;
        res->cost = cost;
        res->path_length = nseg[0] + nseg[1];
        res->path_rows = nseg[0] + nseg[1] + 2;
        if (path && path_cap >= res->path_rows) {
            float *w = path;
            memcpy(w, goals + (size_t)root[1] * D, sizeof(float) * D);
            w += D;
            for (int i = nseg[1] - 1; i >= 0; i--, w += D) memcpy(w, seg[1] + (size_t)i * D, sizeof(float) * D);
            for (int i = 0; i < nseg[0]; i++, w += D) memcpy(w, seg[0] + (size_t)i * D, sizeof(float) * D);
            memcpy(w, start, sizeof(float) * D);
        }
        free(seg[0]);
        free(seg[1]);
    } else {
        res->iters = -1;
    }
done:
    for (int k = 0; k < 2; k++) {
        free(T[k].nodes);
        free(T[k].parents);
        free(T[k].radii);
    }
    free(hb);
    free(hn);
    free(hd);
    free(tsel);
    free(iters);
    return rc;
}

int oracle_solve_many(int robot, int nq, const float *starts, const float *goals, const oracle_env *envs,
                      const oracle_settings *s, float *paths, int path_cap, oracle_result *res, int threads)
{
    const int D = oracle_dof(robot);
    if (D < 0) return -1;
    int rc = 0;
    if (threads > 0) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(| : rc)
        for (int i = 0; i < nq; i++)
            rc |= oracle_solve(robot, starts + (size_t)i * D, goals + (size_t)i * D, 1, envs + i, s, NULL,
                               paths ? paths + (size_t)i * path_cap * D : NULL, path_cap, res + i);
    } else {
#pragma omp parallel for schedule(dynamic, 1) reduction(| : rc)
        for (int i = 0; i < nq; i++)
            rc |= oracle_solve(robot, starts + (size_t)i * D, goals + (size_t)i * D, 1, envs + i, s, NULL,
                               paths ? paths + (size_t)i * path_cap * D : NULL, path_cap, res + i);
    }
    return rc;
}
