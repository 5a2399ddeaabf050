/*
 * prrtc_gb300 — C ABI of a GB300-native (sm_103a) implementation of pRRTC's
 * GPU RRT-Connect hot path.
 *
 * The reference exports only C++ templates:
 *   - pRRTC::solve<Robot>(start, goals, env, settings)      src/planning/Planners.hh:75-78
 *     (defined src/planning/pRRTC.cu:607-766, instantiated :768-771)
 *   - ppln::collision::fkcc<Robot>(q, env, tid)              src/planning/utils.cuh:326-327
 * This header is the C boundary that replaces both; include/prrtc/compat.hh
 * rebuilds the reference's C++ signatures on top of it.
 *
 * Conventions
 *   - Every array argument may be host memory or CUDA device memory of the
 *     context's device; the library detects which (cudaPointerGetAttributes)
 *     and copies host data itself.  Outputs follow the same rule.
 *   - Configurations are row-major float32 [n][dof] in the reference's joint
 *     order (Robots.hh).
 *   - Calls on one context are serialised by an internal mutex; different
 *     contexts are independent (no global device state, unlike the reference's
 *     file-scope __device__ variables, pRRTC.cu:26-35).
 *   - No call resets the device (the reference ends solve() with
 *     cudaDeviceReset(), pRRTC.cu:764).
 */
#ifndef PRRTC_PRRTC_H
#define PRRTC_PRRTC_H

#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum prrtc_status {
    PRRTC_OK = 0,
    PRRTC_EINVAL = 1,        /* bad argument (null, size, unknown robot, env too large) */
    PRRTC_ENOMEM = 2,        /* device allocation failed, or a tree arena is full */
    PRRTC_ETIMEDOUT = 3,     /* a device-side time budget ran out */
    PRRTC_ECUDA = 4,         /* CUDA runtime error (see prrtc_last_error) */
    PRRTC_EUNSUPPORTED = 5
} prrtc_status;

/* Robots of the reference (src/planning/Robots.hh:10-237). */
typedef enum prrtc_robot {
    PRRTC_ROBOT_SPHERE = 0,  /* toy 3-DoF point robot, radius 1 */
    PRRTC_ROBOT_PANDA = 1,   /* 7-DoF */
    PRRTC_ROBOT_FETCH = 2,   /* 8-DoF (q0 = prismatic torso) */
    PRRTC_ROBOT_BAXTER = 3   /* 14-DoF, both arms */
} prrtc_robot;

typedef struct prrtc_ctx prrtc_ctx;
typedef struct prrtc_env prrtc_env;

/*
 * Obstacles (replaces ppln::collision::Environment<float>,
 * src/collision/environment.hh:11-44).  Flat float arrays in host memory;
 * floats per obstacle:
 *   spheres            4   x y z r                               (shapes.hh:271-290)
 *   capsules           8   x1 y1 z1 xv yv zv r rdv               (shapes.hh:176-267)
 *   z_aligned_capsules 8   same layout, axis along z
 *   cylinders          8   accepted and ignored, like the reference checker,
 *                          which never reads them (utils.cuh:211-242)
 *   cuboids           15   x y z, axis_1 xyz, axis_2 xyz, axis_3 xyz,
 *                          axis_1_r axis_2_r axis_3_r            (shapes.hh:75-171)
 *   z_aligned_cuboids 15   same layout
 * rdv is 1 / |(xv, yv, zv)|^2 as in the reference's factory.
 */
typedef struct prrtc_env_desc {
    const float *spheres;
    uint32_t num_spheres;
    const float *capsules;
    uint32_t num_capsules;
    const float *z_aligned_capsules;
    uint32_t num_z_aligned_capsules;
    const float *cylinders;
    uint32_t num_cylinders;
    const float *cuboids;
    uint32_t num_cuboids;
    const float *z_aligned_cuboids;
    uint32_t num_z_aligned_cuboids;
} prrtc_env_desc;

/* Largest environment one kernel stages in shared memory (obstacle floats
 * after packing: 4 per sphere, 8 per capsule, 16 per cuboid). */
#define PRRTC_MAX_ENV_FLOATS 11264

/*
 * Planner settings, byte-identical to pRRTC_settings
 * (src/planning/pRRTC_settings.hh:3-16), same defaults via
 * prrtc_settings_default().
 */
typedef struct prrtc_settings {
    int max_samples;
    int max_iters;
    int num_new_configs;
    int granularity;
    float range;
    int balance;
    float tree_ratio;
    bool dynamic_domain;
    float dd_alpha;
    float dd_radius;
    float dd_min_radius;
} prrtc_settings;

/*
 * Result of one query (replaces PlannerResult<Robot>, Planners.hh:11-23).
 * The caller provides path storage: path_capacity rows of dof floats.  The
 * path is written in the reference's order: goal first, then the goal-tree
 * segment, the start-tree segment and the start (pRRTC.cu:731-741).
 */
typedef struct prrtc_result {
    int solved;              /* 1 solved, 0 not */
    int status;              /* prrtc_status of this query */
    int start_tree_size;
    int goal_tree_size;
    int path_length;         /* nodes traced from both trees (pRRTC.cu:743) */
    int iters;               /* iterations of the winning lane (-1 if unsolved) */
    float cost;              /* sum of edge lengths traced (pRRTC.cu:561,571) */
    int path_rows;           /* rows written to path */
    int path_capacity;       /* in: rows available in path */
    float *path;             /* in: [path_capacity][dof] host buffer, may be NULL */
    uint64_t wall_ns;        /* whole call, host clock */
    uint64_t kernel_ns;      /* planner kernel(s), device clock */
    uint64_t copy_ns;        /* host<->device copies of the query */
    uint64_t finish_ns;      /* batched form: from the launch's start to this query's end
                                (device clock; 0 if it never started) */
    int64_t samples;         /* batched form: samples drawn for this query, all attempts */
} prrtc_result;

/* ---- context ------------------------------------------------------------ */
prrtc_status prrtc_create(prrtc_ctx **out, int device);
prrtc_status prrtc_destroy(prrtc_ctx *ctx);
const char *prrtc_status_string(prrtc_status s);
/* Text of the last error on this context (empty if none). */
const char *prrtc_last_error(const prrtc_ctx *ctx);
/* Total kernel launches this context has issued (for accounting). */
uint64_t prrtc_launch_count(const prrtc_ctx *ctx);
/* Planning margin: every robot sphere is inflated by pad metres while
 * planning (default 0 = the reference's semantics).  A positive pad makes
 * every returned path free under any checker whose sphere centres are within
 * pad of this one's. */
prrtc_status prrtc_set_planning_margin(prrtc_ctx *ctx, float pad);
/* Device time budget of one planner launch in ns (0 = none, the default).
 * When it runs out the query ends unsolved with status PRRTC_ETIMEDOUT. */
prrtc_status prrtc_set_time_budget(prrtc_ctx *ctx, uint64_t ns);

/* ---- robots ------------------------------------------------------------- */
int prrtc_robot_dof(prrtc_robot robot);             /* -1 for an unknown robot */
int prrtc_robot_num_spheres(prrtc_robot robot);     /* spheres of fk_spheres */
/* Joint scaling of the reference sampler: q = u * scale + offset, u in [0,1)
 * (Robots.hh scale_cfg).  Writes dof floats to each (host memory). */
prrtc_status prrtc_robot_limits(prrtc_robot robot, float *scale, float *offset);

/* ---- environments ------------------------------------------------------- */
prrtc_status prrtc_env_upload(prrtc_ctx *ctx, const prrtc_env_desc *desc, prrtc_env **out);
prrtc_status prrtc_env_free(prrtc_ctx *ctx, prrtc_env *env);

/* ---- collision checking (replaces fkcc<Robot>, utils.cuh:326-33131) ----- */
/* out_free[i] = 1 when configuration i is collision-free. */
prrtc_status prrtc_validate_configs(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_env *env,
                                    const float *q, int64_t n, uint8_t *out_free);
/*
 * Edge i from a[i] to b[i] is free when every point
 *     a + k * ((b - a) / granularity),  k = 1 .. granularity
 * is free (the reference's extend interpolation, pRRTC.cu:430-442, evaluated
 * in float32 without fused multiply-add).  granularity in [1, 1024].
 */
prrtc_status prrtc_validate_edges(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_env *env,
                                  const float *a, const float *b, int64_t n, int granularity,
                                  uint8_t *out_free);
/*
 * prrtc_validate_configs without allocating anything (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc or cudaFree: a control
 * loop with a hard deadline (those calls can synchronise the device), a
 * process whose device memory belongs to another runtime's pool, or code with
 * a fixed memory budget.  No context is needed; verdicts are the same as
 * prrtc_validate_configs'.
 *   env        host arrays; at most PRRTC_MAX_ENV_FLOATS packed floats, else
 *              PRRTC_EINVAL (the limit of the library's fixed device array)
 *   q, out_free  device memory of the current device ([n][dof] floats, n bytes)
 *   stream     cudaStream_t to run on (NULL: the default stream).  The
 *              obstacles are copied from a host array inside the library
 *              (pageable memory); to stage that copy the driver may first
 *              wait for the work already queued on `stream`.  The call
 *              returns once the copy is staged and the check is queued.
 * The library keeps one fixed array of PRRTC_MAX_ENV_FLOATS floats plus two
 * counters on every GPU that loads it, for the life of the process.  Every
 * call on a device shares it, so calls whose GPU work overlaps (other
 * streams, other threads) race: serialise them.  The first call on a device
 * looks up the array's address with that device current; make it before any
 * stream capture.  The call cannot be captured into a CUDA graph (a replay
 * would copy whatever the host array holds at that time): while `stream` is
 * being captured it returns PRRTC_EINVAL without touching the stream, and the
 * capture stays valid.
 */
prrtc_status prrtc_validate_configs_noalloc(prrtc_robot robot, const prrtc_env_desc *env, const float *q,
                                            int64_t n, uint8_t *out_free, void *stream);
/*
 * Goal regions (no counterpart in pRRTC, whose goals are configurations,
 * pRRTC.cu:690-693): up to max_goals collision-free configurations whose model
 * sphere `sphere` (e.g. the hand's bounding sphere) has its centre inside the
 * box [box_lo, box_hi] (world, metres).  Candidates t = 0 .. tries-1 of a
 * seeded sequence spanning the joint box are tested on the GPU; the first
 * accepted ones in sequence order are returned, so the result depends only
 * on the arguments.  goals: host [max_goals][dof]; *num_found receives the
 * count.  Pass them as a query's goals (num_goals > 1 is a goal set).
 */
prrtc_status prrtc_sample_goals(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_env *env, int sphere,
                                const float *box_lo, const float *box_hi, uint64_t seed, int64_t tries,
                                int max_goals, float *goals, int *num_found);
/* World centre and radius of every model sphere: out is [n][num_spheres][4]. */
prrtc_status prrtc_fk_spheres(prrtc_ctx *ctx, prrtc_robot robot, const float *q, int64_t n,
                              float *out);

/* Device time of the context's last prrtc_validate_configs or
 * prrtc_validate_edges launch (CUDA events on the context's stream around the
 * kernel alone), in ns.  No counterpart in the reference. */
prrtc_status prrtc_last_kernel_ns(prrtc_ctx *ctx, uint64_t *ns);
/* Work counters: algorithmic FLOPs (weights as prrtc_batch_stats.flops) and
 * configurations checked by validate_configs / validate_edges / solve since
 * the last reset. */
prrtc_status prrtc_work_counters(prrtc_ctx *ctx, uint64_t *flops, uint64_t *configs, int reset);
/* Diagnostic: FP32 FMA throughput of the device in TFLOP/s, measured with a
 * chain-of-FMA kernel over every SM (the roofline denominator of the
 * validator, which runs on the FP32 pipe). */
prrtc_status prrtc_measure_fp32_peak(prrtc_ctx *ctx, double *tflops);

/* ---- planning (replaces pRRTC::solve<Robot>, pRRTC.cu:607-766) ---------- */
void prrtc_settings_default(prrtc_settings *s);
/* goals: [num_goals][dof].  start/goals/path are host memory. */
prrtc_status prrtc_solve(prrtc_ctx *ctx, prrtc_robot robot, const float *start, const float *goals,
                         int num_goals, const prrtc_env *env, const prrtc_settings *settings,
                         prrtc_result *result);

/* ---- batched planning (no reference counterpart: pRRTC solves one query per
 * call; its only callers loop over problems, scripts/evaluate_mbm.cpp:126-151) */

/* One query of a batch.  The environment is either an uploaded prrtc_env or
 * host arrays (env = NULL), which the batch packs and uploads itself. */
typedef struct prrtc_query {
    const prrtc_env *env;
    const prrtc_env_desc *env_desc;
    const float *start;              /* [dof], host */
    const float *goals;              /* [num_goals][dof], host */
    int num_goals;
} prrtc_query;

typedef struct prrtc_batch_settings {
    prrtc_settings plan;             /* applied to every query; a query gives up after
                                        max_iters x num_new_configs samples, pRRTC's total */
    int lanes;                       /* virtual sampling lanes per query: sample k of a query is
                                        Halton point k / lanes + 1 of lane k % lanes, and the balance
                                        modes see the lane as pRRTC sees blockIdx.x.  0: 2.  pRRTC's
                                        own count (plan.num_new_configs) reproduces its sample set,
                                        whose first points cluster near the lower joint limits */
    int max_nodes_per_tree;          /* arena capacity per tree (0: min(max_samples, 65536)) */
    int max_active;                  /* queries in flight at once (0: all queries, within the arena
                                        budget); with max_attempts > 1 further slots hold only
                                        restarts and extra attempts */
    int warps_per_block;             /* 0: 4 */
    int edge_order;                  /* order a warp checks an edge's points in: 0 contiguous
                                        rounds, 1 interleaved (every round spans the edge) */
    int sampler;                     /* 0: pRRTC's Halton lanes; 1: Halton with per-query digit
                                        scrambling and rotation (decorrelates large bases) */
    int max_attempts;                /* independent attempts per query (0: 4; 1: none).  An attempt
                                        that runs out of samples or arena restarts the query; once
                                        no query is pending, idle warps open extra attempts of
                                        queries running longer than k x restart_after_ns; the first
                                        attempt to connect wins */
    uint64_t restart_after_ns;       /* 0: 10 ms */
    int max_workers_per_attempt;     /* warps working one attempt at once (0: unlimited; an attempt
                                        younger than 200 us takes at most 4); when every running
                                        attempt is full, an idle warp opens a new attempt */
    int blocks_per_sm;               /* 0: occupancy maximum */
    int use_graph;                   /* replay each run as a captured CUDA graph */
    float margin;                    /* sphere inflation while planning, metres (>= 0) */
    uint64_t time_budget_ns;         /* 0: none */
    int admission;                   /* order queries start in when slots are fewer than queries:
                                        0 tightest first (smallest clearance of start or goal to an
                                        obstacle, computed on the GPU at create: the hard queries
                                        start early and no longer set the batch's end); 1 as given */
    uint32_t idle_wait_limit;        /* polls (about 256 ns each) a warp with no work to take makes
                                        before it gives up and the run ends with PRRTC_ECUDA and
                                        stats.error = 1 (0: 2^22, about a second) */
    int shared_frames;               /* 1: the checker keeps its forward-kinematics frames in each
                                        warp's shared memory; 0: in local memory (cached by L1) */
    int rounds_per_header;           /* batches of 32 samples a warp may draw under one read of the
                                        attempt's shared state while the early dynamic-domain test
                                        rejects all of them (0: 4, at most 64; 1: one batch per read) */
} prrtc_batch_settings;

typedef struct prrtc_batch prrtc_batch;

/* Totals of the last run of a batch. */
typedef struct prrtc_batch_stats {
    uint64_t kernel_ns;              /* planner launch, device clock */
    int64_t samples;                 /* samples drawn over all queries */
    int solved;                      /* queries solved */
    int blocks, warps_per_block;     /* launch shape used */
    int slots;                       /* resident query slots */
    int error;                       /* nonzero: a worker gave up waiting for work */
    int extra_attempts;              /* attempts opened beyond each query's first */
    uint64_t configs_checked;        /* configurations validated (edge points examined) */
    uint64_t flops;                  /* algorithmic FLOPs of those checks: forward kinematics
                                        2 (12 dof + 9 spheres) per config, plus the primitive
                                        tests executed x {sphere 11, capsule 26, z-capsule 16,
                                        cuboid 27, z-cuboid 18, sphere pair 11} */
    uint64_t nn_nodes;               /* tree nodes visited by nearest-neighbour scans */
    uint64_t bulk_ns;                /* device time from the launch's start until 99 % of the queries
                                        had finished (the launch without its tail) */
    uint64_t bulk_flops;             /* flops counted by then */
    uint64_t bulk_configs;           /* configurations checked by then */
} prrtc_batch_stats;

void prrtc_batch_settings_default(prrtc_batch_settings *s);
/* Packs and uploads the queries and allocates the batch's device state. */
prrtc_status prrtc_batch_create(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_query *queries, int n,
                                const prrtc_batch_settings *settings, prrtc_batch **out);
/* Solves every query of the batch in one persistent launch; inputs and
 * results stay on the device.  A batch may be run again (same answers). */
prrtc_status prrtc_batch_run(prrtc_ctx *ctx, prrtc_batch *batch);
/* Copies the last run's results (and paths into each result's buffer). */
prrtc_status prrtc_batch_results(prrtc_ctx *ctx, prrtc_batch *batch, prrtc_result *results);
prrtc_status prrtc_batch_stats_get(prrtc_ctx *ctx, const prrtc_batch *batch, prrtc_batch_stats *stats);
prrtc_status prrtc_batch_free(prrtc_ctx *ctx, prrtc_batch *batch);
/* create + run + results + free. */
prrtc_status prrtc_solve_batch(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_query *queries, int n,
                               const prrtc_batch_settings *settings, prrtc_result *results);

/* ---- differentiable clearance (no reference counterpart: pRRTC returns raw
 * RRT-Connect paths, pRRTC.cu:568-602, and never post-processes them) ------
 *
 * Cost of one configuration, margin m (metres):
 *   C(q) = 1/2 sum over env leaf spheres x obstacles of max(0, m - sd)^2
 *        + 1/2 sum over self-collision leaf pairs of max(0, m - sd)^2
 * sd = signed distance (negative inside; true box distance, interior
 * included).  The leaf spheres and pairs are those the checker tests, so
 * C(q) = 0 means every leaf test of fkcc<Robot> clears by at least m. */

/* Cost and joint gradient of every waypoint of n_paths paths, path i in
 * envs[i].  q: [n_paths][waypoints][dof]; cost: [n_paths][waypoints];
 * grad: [n_paths][waypoints][dof] = dC/dq.  Host or device pointers.  The
 * gradient is a hand-written adjoint that recomputes forward kinematics. */
prrtc_status prrtc_path_cost_grad(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_env *const *envs, int n_paths,
                                  int waypoints, const float *q, float margin, float *cost, float *grad);

typedef struct prrtc_smooth_settings {
    float margin;          /* hinge margin, metres (0.02) */
    int steps;             /* gradient steps (50) */
    float step;            /* step size (0.05) */
    float cost_weight;     /* weight of dC/dq (100) */
    float smooth_weight;   /* weight of the discrete path Laplacian (1) */
    int granularity;       /* checker points per edge for the final judgement (128) */
    int shortcut_rounds;   /* shortcut attempts before smoothing (8): a span (i, j) is replaced by
                              evenly spaced points on the segment q_i -> q_j when its sub-edges
                              are free at granularity / 4 points */
} prrtc_smooth_settings;
void prrtc_smooth_settings_default(prrtc_smooth_settings *s);

/* Shortens and smooths paths in place: `shortcut_rounds` shortcut attempts,
 * then `steps` iterations of
 *   q_w -= step * (cost_weight * dC/dq(q_w) + smooth_weight * (2 q_w - q_{w-1} - q_{w+1}))
 * on the interior waypoints (end points fixed, joint limits clamped), then
 * checks every edge with the collision checker at `granularity` points
 * (a + k ((b - a) / g), k = 1..g).  A path is written back only if all its
 * points are free: accepted[i] = 1; otherwise it is left exactly as given
 * and accepted[i] = 0.  2 <= waypoints <= 256.  cost_before / cost_after
 * (optional) receive each path's summed cost before and after. */
prrtc_status prrtc_smooth_paths(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_env *const *envs, int n_paths,
                                int waypoints, float *q, const prrtc_smooth_settings *settings, uint8_t *accepted,
                                float *cost_before, float *cost_after);

#ifdef __cplusplus
}
#endif
#endif /* PRRTC_PRRTC_H */
