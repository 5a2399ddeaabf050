/*
 * Oracle: CPU restatement of pRRTC's collision checker and RRT-Connect
 * planner.  TEST INFRASTRUCTURE ONLY — used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU baseline as the checker; the
 * library never links or calls it.
 *
 * Pinned against the reference itself: tests/test_oracle_ref.py compares it
 * with pRRTC's own checker compiled from its sources (oracle/_ref, built by
 * `make -C oracle ref`) and with the float64 evaluation of the reference's
 * generated code, and tests/golden/ holds fixtures made from those.
 *
 * Obstacle arrays use the flat layouts of include/prrtc/prrtc.h.
 */
#ifndef PRRTC_ORACLE_H
#define PRRTC_ORACLE_H

#include <stdint.h>

typedef struct oracle_env {
    const float *spheres;    int ns;    /* 4 floats each */
    const float *capsules;   int nc;    /* 8 */
    const float *zcapsules;  int nzc;   /* 8 */
    const float *cuboids;    int ncb;   /* 15 */
    const float *zcuboids;   int nzb;   /* 15 */
} oracle_env;

/* primitive tests counted by oracle_check (executed, with the reference's early exits) */
enum { ORC_SPHERE = 0, ORC_CAPSULE, ORC_ZCAPSULE, ORC_CUBOID, ORC_ZCUBOID, ORC_SELF, ORC_NCOUNT };

int oracle_dof(int robot);
int oracle_num_spheres(int robot);
int oracle_limits(int robot, float *scale, float *offset);

/* Float64 forward kinematics of every model sphere: out [n][S][4] (x y z r). */
int oracle_fk_spheres(int robot, const double *q, long n, double *out);

/*
 * Reference-semantics verdicts (fkcc<Robot>, utils.cuh:326-33131): sphere
 * centres from the float64 FK rounded to float, every primitive test in
 * float32 as the reference writes it, the gate/leaf hierarchy and group
 * order of the reference.  out_free[i] = 1 when free.  Optional outputs:
 * margin[i] = min over every test of the hierarchy of |signed distance| in
 * float64 (metres; the near-contact measure), counts[ORC_NCOUNT] += tests
 * executed.  Threads: OpenMP over configurations.
 */
int oracle_check(int robot, const float *q, long n, const oracle_env *env, uint8_t *out_free,
                 double *margin, int64_t *counts);

/* Edges a[i] -> b[i]: free when a + k * ((b - a) / g), k = 1..g, are all free
 * (float32 interpolation without fused multiply-add). */
int oracle_check_edges(int robot, const float *a, const float *b, long n, int g, const oracle_env *env,
                       uint8_t *out_free);

/* Float64 clearance: min signed distance over leaf spheres vs obstacles and
 * leaf self pairs (negative = penetrating). */
int oracle_clearance(int robot, const float *q, long n, const oracle_env *env, double *out);

/*
 * Float64 clearance cost and its gradient (the differentiable clearance of
 * prrtc_path_cost_grad; no reference counterpart).  Per configuration:
 *   C = 1/2 sum over leaf spheres x obstacles and leaf self pairs of max(0, m - sd)^2
 * with sd the float64 signed distance (boxes: true distance, interior
 * included).  grad[i][d] = dC/dq_d, assembled with the geometric Jacobian of
 * each sphere centre (z_j x (c - o_j) per revolute ancestor joint j, z_j per
 * prismatic one) -- a different route from the library's tip-to-base sweep.
 */
int oracle_cost_grad(int robot, const double *q, long n, const oracle_env *env, double margin, double *cost,
                     double *grad);

/*
 * RRT-Connect as pRRTC runs it (rrtc<Robot>, pRRTC.cu:305-602), with its
 * `num_new_configs` lanes emulated in round-robin order on one thread.
 * Settings are pRRTC_settings fields.  bases: [lanes][16] Halton prime bases
 * (NULL: lane 0 natural order, others shuffled with a SplitMix64 stream).
 * Path (goal first, as pRRTC) goes to path[path_cap][dof].
 */
typedef struct oracle_settings {
    int max_samples, max_iters, num_new_configs, granularity;
    float range;
    int balance;
    float tree_ratio;
    int dynamic_domain;
    float dd_alpha, dd_radius, dd_min_radius;
    double budget_s;         /* wall-clock budget per query, 0 = none (then unsolved) */
} oracle_settings;

typedef struct oracle_result {
    int solved;
    int start_tree_size, goal_tree_size;
    int path_length, path_rows, iters;
    float cost;
    int64_t checks;          /* configurations checked */
} oracle_result;

/* Units of the planner, for the device-side parity tests:
 *   oracle_halton    lanes x steps points of halton_next (pRRTC.cu:81-105) from
 *                    bases16[lane][16] (the lane's primes), raw and scaled by
 *                    fmaf(raw, scale, offset) (Robot::scale_cfg, Robots.hh);
 *   oracle_nearest   argmin of squared L2 (sq_l2_dist, utils.cuh:100-109) over
 *                    nodes[count][dof], first index on ties, NaN nodes never win;
 *   oracle_dd_apply  ops[i][k] (0 grow, 1 shrink) applied in order to radii[i]
 *                    (pRRTC.cu:456-468, 584-598). */
int oracle_halton(int dof, const float *bases16, int lanes, int steps, const float *scale, const float *offset,
                  float *raw, float *cfg);
int oracle_nearest(int dof, const float *nodes, int count, const float *q, int nq, int *out_i, float *out_d);
int oracle_dd_apply(float *radii, int n, const uint8_t *ops, int nops, float alpha, float radius0, float rmin);

int oracle_solve(int robot, const float *start, const float *goals, int num_goals, const oracle_env *env,
                 const oracle_settings *s, const float *bases, float *path, int path_cap, oracle_result *res);

/* Many independent queries (OpenMP over queries, `threads` <= 0: all). */
int oracle_solve_many(int robot, int nq, const float *starts, const float *goals, const oracle_env *envs,
                      const oracle_settings *s, float *paths, int path_cap, oracle_result *res, int threads);

#endif
