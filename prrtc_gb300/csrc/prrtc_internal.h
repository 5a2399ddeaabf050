// Internal host-side declarations shared by the C ABI and the per-robot
// kernel translation units.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "prrtc/prrtc.h"
#include "device_common.cuh"

namespace prrtc {

// A packed environment as the kernels see it.
struct LaunchEnv {
    const float4 *rec;   // device records
    EnvCounts counts;
    int sms;             // SM count of the device
    unsigned long long *work;   // [2]: FLOPs, configurations (device, accumulated)
};

// Device control block of one query (replaces the reference's file-scope
// __device__ globals solved, atomic_free_index, path_size, cost,
// reached_goal_idx, solved_iters, pRRTC.cu:26-34).
struct QueryCtl {
    int solved;          // 0 running, 1 solved, -1 exhausted (iters or samples), -2 time budget
    int free_index[2];   // next free node of each tree
    int path_size[2];    // nodes traced from each tree
    float cost;
    int reached_goal;
    int solved_iters;
    int error;           // bit 0: path buffer too small
    int pad_;
};

// Everything the plain-form planner kernel needs (passed by value).
struct PlainParams {
    // pRRTC_settings (pRRTC_settings.hh:3-16)
    int max_samples, max_iters, num_new_configs, granularity;
    float range;
    int balance;
    float tree_ratio;
    int dynamic_domain;
    float dd_alpha, dd_radius, dd_min_radius;
    float pad;                         // collision margin added to every sphere (0 = reference)
    unsigned long long budget_ns;      // device time budget (0 = none)
    // two trees, nodes SoA: nodes[t][d * cap + i]
    float *nodes[2];
    int *parents[2];
    float *radii[2];
    int cap;
    const float *halton_bases;         // [lanes][16] shuffled prime bases per lane
    float scale[16], offset[16];       // joint scaling (Robots.hh scale_cfg)
    const float4 *env;
    EnvCounts env_n;
    QueryCtl *ctl;
    float *path;                       // [2][path_cap][dof]
    int path_cap;
    unsigned long long *work;          // [2]: FLOPs, configurations (device, accumulated)
};

// ---- batched planner ------------------------------------------------------
struct BatchQueryDesc {
    const float4 *env;   // packed obstacle records (device)
    EnvCounts env_n;
    int cfg_off;         // float offset of start (dof floats) then goals in the config pool
    int num_goals;
};

enum SlotStateCode { SLOT_FREE = 0, SLOT_RUNNING = 1, SLOT_DONE = 2, SLOT_BUSY = 3 };

// One resident slot: an attempt at a query (its trees live in the arena at
// the slot's index).
// Each slot owns two 128-byte lines: the sample ticket, taken by an atomic
// in every round header of every warp working the slot, on the second, so
// that those atomics neither queue the reads of the slot's state nor touch
// the lines of other slots.
struct alignas(128) SlotState {
    int query;
    int attempt;         // attempt number of the query (selects its sample stream)
    int state;           // SlotStateCode
    int free_index[2];
    int workers;         // warps registered on the slot
    int restart;         // 1: the warp that recycles the slot restarts the query here
    unsigned long long t_start;   // device ns when the slot's attempt was admitted
    alignas(128) int ticket;      // samples drawn so far
};

// Per-query state shared by its attempts.
struct QueryState {
    int state;           // 0 pending, 1 running, 2 finished
    int attempts;        // attempts started
    int live;            // attempts running
    int pad_;
    unsigned long long t_first;   // first admission, device ns
};

// Per-query result, written by the warp that finishes the query.
struct BatchOut {
    int solved;          // 1 solved, 0 not
    int status;          // 0 ok, prrtc_status otherwise
    int start_tree_size, goal_tree_size;
    int path_length;
    int iters;
    float cost;
    int path_off, path_rows;
    int reached_goal;
    int samples;
    int pad_;
    unsigned long long t_admit, t_done;   // device globaltimer, ns
};

struct BatchCounters {
    int admit_next;      // next query to admit
    int cursor;          // round-robin slot cursor
    int done;            // queries finished
    int path_next;       // rows used in the path pool
    int error;           // bit 0: a worker gave up waiting for work
    int attempts;        // attempts started beyond each query's first
    int pad_[2];
    unsigned long long t0;
    unsigned long long work[2];      // algorithmic FLOPs of the checks, configurations checked
    unsigned long long nn_nodes;     // tree nodes visited by nearest-neighbour scans
    unsigned long long t99;          // device clock when 99 % of the queries had finished
    unsigned long long work99[2];    // work[] at that moment
};

// cap on a batch query's samples: 2^31 - 2^24, so that tickets taken past it
// by every resident warp (32 each) still fit an int
constexpr long long kMaxSamplesDrawn = 0x7f000000LL;
// obstacle records a planner warp stages in shared memory (larger
// environments are read from global memory)
constexpr int kWarpEnvRecords = 256;

struct BatchParams {
    int max_samples, max_iters, lanes, granularity;
    int env_records;     // records each warp can stage: the batch's largest environment, <= kWarpEnvRecords
    float range;
    int balance;
    float tree_ratio;
    int dynamic_domain;
    float dd_alpha, dd_radius, dd_min_radius;
    float pad;
    unsigned long long budget_ns;
    int num_queries, num_slots, cap, path_pool_rows;
    int admit_slots;     // slots [0, admit_slots) take new queries (max_active); the rest only extra attempts
    int edge_order;      // 0 contiguous, 1 interleaved (see warp_validate)
    long long max_samples_drawn;   // per query: max_iters x num_new_configs, pRRTC's total budget
    int sampler;         // 0 Halton lanes as pRRTC, 1 scrambled Halton per query
    int max_attempts;    // attempts per query (restarts and parallel attempts), >= 1
    int max_workers;     // warps per attempt
    int bases_lanes;     // rows of halton_bases
    unsigned long long restart_after_ns;   // a query may get its k-th extra attempt after k x this
    unsigned idle_limit;                   // polls before an idle warp gives up (error flag)
    int shared_frames;                     // the checker's frames in the warp's shared memory (else local)
    int sub_rounds;                        // 32-sample batches a round may draw while all are rejected early
    const float *cfg_pool;
    const BatchQueryDesc *queries;
    const int *order;    // admission order (query ids), null: index order
    QueryState *qstate;
    SlotState *slots;
    BatchOut *out;
    BatchCounters *ctr;
    float *nodes;        // [slot][2][dof][cap], NaN where unwritten
    int *parents;        // [slot][2][cap]
    float *radii;        // [slot][2][cap]
    float *path_pool;    // [path_pool_rows][dof]
    const float *halton_bases;   // [lanes][16]
    float scale[16], offset[16];
};

// Goal-region sampling (prrtc_sample_goals): candidate t of a seed, the same
// on the host and the device (integer hash, then one correctly rounded fmaf
// per joint), so the host can rebuild the candidates the device accepted.
__host__ __device__ inline unsigned goal_hash(unsigned x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__host__ __device__ inline void goal_candidate(unsigned long long seed, long long t, int dof, const float *scale,
                                               const float *offset, float *q)
{
    for (int d = 0; d < dof; d++) {
        unsigned h = goal_hash((unsigned)seed ^ goal_hash((unsigned)(seed >> 32) + 0x9E3779B9u * (unsigned)d));
        h = goal_hash(h ^ (unsigned)t);
        h = goal_hash(h ^ (unsigned)((unsigned long long)t >> 32) ^ 0x85EBCA6Bu);
        const float u = (float)(h >> 8) * (1.0f / 16777216.0f);   // [0, 1), 24 bits, exact
        q[d] = fmaf(u, scale[d], offset[d]);
    }
}

struct GoalQuery {
    unsigned long long seed;
    long long tries;
    int sphere;                   // model sphere whose centre must lie in the box
    float lo[3], hi[3];
    float scale[16], offset[16];  // the robot's joint box
};

struct ClrLaunch;   // clearance_device.cuh
struct Ctx;         // context.h

// score[i] = smallest clearance (metres, float32 screen) of query i's start or
// goals to its obstacles, over the robot's env leaf spheres (clearance.cu).
prrtc_status query_clearance(Ctx *c, prrtc_robot robot, const BatchQueryDesc *queries, const float *cfg_pool, int n,
                             float *score);

struct RobotOps {
    int dof;
    int num_spheres;
    cudaError_t (*validate_configs)(const LaunchEnv &, const float *q, int64_t n, uint8_t *out, cudaStream_t);
    cudaError_t (*validate_edges)(const LaunchEnv &, const float *a, const float *b, int64_t n, int g,
                                  uint8_t *out, cudaStream_t);
    cudaError_t (*fk_spheres)(const float *q, int64_t n, float *out, int sms, cudaStream_t);
    cudaError_t (*solve_plain)(const PlainParams &, int threads, cudaStream_t);
    cudaError_t (*solve_batch)(const BatchParams &, int blocks, int warps_per_block, cudaStream_t);
    int (*batch_occupancy)(int warps_per_block, int env_records, int shared_frames);   // resident blocks per SM
    cudaError_t (*smooth_paths)(const ClrLaunch &, size_t env_bytes, cudaStream_t);
    cudaError_t (*goal_flags)(const LaunchEnv &, const GoalQuery &, uint8_t *flags, cudaStream_t);
};

// Shuffled Halton prime bases per sampling lane, as the reference seeds them
// (pRRTC.cu:49-79,107-121): lane 0 keeps {3,5,...,59}; lane i > 0 shuffles
// them with cuRAND XORWOW (seed 1 + i, subsequence i).
cudaError_t launch_halton_bases(float *out, int lanes, cudaStream_t st);

RobotOps robot_ops_sphere();
RobotOps robot_ops_panda();
RobotOps robot_ops_fetch();
RobotOps robot_ops_baxter();

}  // namespace prrtc
