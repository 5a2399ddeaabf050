// Host side of the batched planner (prrtc_batch_*, prrtc_solve_batch).
//
// A batch packs its queries once (obstacle records, start/goal configs,
// descriptors) and owns its device state: slot table, per-query results and
// a path pool.  The node arena (slots x 2 trees x cap nodes) is NaN wherever
// no node is written, an invariant the kernel restores as it recycles slots,
// so a run needs no arena reset; the context keeps the arena between batches.
// A run is four stream operations (three small memsets and the persistent
// launch), optionally captured once as a CUDA graph and replayed.
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cstring>
#include <vector>

#include "context.h"
#include "prrtc_internal.h"

namespace prrtc {

struct Arena {
    int dof = 0, cap = 0, slots = 0;
    float *nodes = nullptr;
    int *parents = nullptr;
    float *radii = nullptr;
    bool in_use = false;
};

static void arena_free(Arena *a)
{
    if (!a) return;
    cudaFree(a->nodes);
    cudaFree(a->parents);
    cudaFree(a->radii);
    delete a;
}

void release_arena(Ctx *c)
{
    arena_free(c->arena);
    c->arena = nullptr;
}

// An arena of at least (slots, cap) for dof, NaN-filled; reuses the context's.
static prrtc_status take_arena(Ctx *c, int dof, int cap, int slots, Arena **out)
{
    Arena *a = c->arena;
    if (a && !a->in_use && a->dof == dof && a->cap == cap && a->slots >= slots) {
        a->in_use = true;
        *out = a;
        return PRRTC_OK;
    }
    if (a && !a->in_use) {
        arena_free(a);
        c->arena = nullptr;
    }
    a = new Arena();
    a->dof = dof;
    a->cap = cap;
    a->slots = slots;
    const size_t nn = (size_t)slots * 2 * dof * cap, np = (size_t)slots * 2 * cap;
    if (cudaMalloc(&a->nodes, nn * sizeof(float)) != cudaSuccess || cudaMalloc(&a->parents, np * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&a->radii, np * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        arena_free(a);
        return c->fail(PRRTC_ENOMEM, "batch: cannot allocate an arena of %d slots x %d nodes", slots, cap);
    }
    prrtc_status s = c->cuda(cudaMemsetAsync(a->nodes, 0xFF, nn * sizeof(float), c->stream), "arena fill");
    if (s) {
        arena_free(a);
        return s;
    }
    a->in_use = true;
    if (!c->arena) c->arena = a;
    *out = a;
    return PRRTC_OK;
}

static void give_back_arena(Ctx *c, Arena *a)
{
    if (!a) return;
    a->in_use = false;
    if (c->arena == a) return;
    if (!c->arena) {
        c->arena = a;
        return;
    }
    // keep the larger one
    if ((size_t)a->slots * a->cap > (size_t)c->arena->slots * c->arena->cap && !c->arena->in_use) {
        arena_free(c->arena);
        c->arena = a;
    } else {
        arena_free(a);
    }
}

}  // namespace prrtc

using namespace prrtc;

struct prrtc_batch {
    prrtc_robot robot;
    int n = 0, dof = 0, slots = 0, cap = 0, lanes = 0, blocks = 0, wpb = 4, path_rows = 0;
    bool use_graph = false;
    BatchParams P{};
    std::vector<int> num_goals;
    // device
    void *blob = nullptr;          // cfg pool | env pool | descs | slots | outs | counters | path pool
    Arena *arena = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // last run
    prrtc_batch_stats stats{};
    unsigned long long t0 = 0;     // device clock at the last run's start (first warp)
    bool ran = false;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

extern "C" void prrtc_batch_settings_default(prrtc_batch_settings *s)
{
    if (!s) return;
    std::memset(s, 0, sizeof *s);
    prrtc_settings_default(&s->plan);
}

extern "C" prrtc_status prrtc_batch_create(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_query *queries, int n,
                                           const prrtc_batch_settings *settings, prrtc_batch **out)
{
    Ctx *c = Ctx::of(ctx);
    const RobotOps *ops = robot_ops(robot);
    if (!c) return PRRTC_EINVAL;
    if (!ops || !queries || n < 1 || !settings || !out) return c->fail(PRRTC_EINVAL, "batch_create: bad argument");
    const prrtc_settings &S = settings->plan;
    if (S.num_new_configs < 1 || S.granularity < 1 || S.granularity > 1024 || !(S.range > 0.0f) || S.max_iters < 0 ||
        !(settings->margin >= 0.0f) || settings->warps_per_block < 0 || settings->warps_per_block > 4 ||
        settings->lanes < 0 || settings->lanes > 4096)
        return c->fail(PRRTC_EINVAL, "batch_create: bad settings");
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    *out = nullptr;
    const int D = ops->dof;
    int cap = settings->max_nodes_per_tree > 0 ? settings->max_nodes_per_tree : std::min(S.max_samples, 65536);
    cap = std::max(4, (std::min(cap, S.max_samples) + 3) & ~3);
    // pack queries: sizes first (every query checked), so that the packed
    // configurations and obstacle records are allocated once and written in
    // place, with no per-query temporaries
    size_t cfg_floats = 0, env_records = 0;
    for (int i = 0; i < n; i++) {
        const prrtc_query &q = queries[i];
        if (!q.start || !q.goals || q.num_goals < 1 || q.num_goals >= cap || (!q.env && !q.env_desc))
            return c->fail(PRRTC_EINVAL, "batch_create: bad query %d", i);
        cfg_floats += (size_t)(1 + q.num_goals) * D;
        if (!q.env) {
            const prrtc_env_desc &e = *q.env_desc;
            const uint64_t recs = (uint64_t)e.num_spheres + 2ull * e.num_capsules + 2ull * e.num_z_aligned_capsules +
                                  4ull * e.num_cuboids + 4ull * e.num_z_aligned_cuboids;
            if (recs * 4 > (uint64_t)PRRTC_MAX_ENV_FLOATS) return c->fail(PRRTC_EINVAL, "batch_create: env %d too large", i);
            env_records += recs;
        }
    }
    std::vector<float> cfg;
    std::vector<float4> envs;
    cfg.reserve(cfg_floats);
    envs.reserve(env_records);
    std::vector<BatchQueryDesc> descs(n);
    std::vector<int> env_rec_off(n, -1);
    for (int i = 0; i < n; i++) {
        const prrtc_query &q = queries[i];
        descs[i].cfg_off = (int)cfg.size();
        descs[i].num_goals = q.num_goals;
        cfg.insert(cfg.end(), q.start, q.start + D);
        cfg.insert(cfg.end(), q.goals, q.goals + (size_t)q.num_goals * D);
        if (q.env) {
            const Env *e = reinterpret_cast<const Env *>(q.env);
            descs[i].env = e->dev;
            descs[i].env_n = e->counts;
        } else {
            const prrtc_env_desc &e = *q.env_desc;
            env_rec_off[i] = (int)envs.size();
            descs[i].env_n = EnvCounts{(int)e.num_spheres, (int)e.num_capsules, (int)e.num_z_aligned_capsules,
                                       (int)e.num_cuboids, (int)e.num_z_aligned_cuboids};
            pack_records(e, [&](float4 r) { envs.push_back(r); });
        }
    }
    prrtc_batch *b = new prrtc_batch();
    b->robot = robot;
    b->n = n;
    b->dof = D;
    b->cap = cap;
    b->lanes = settings->lanes > 0 ? settings->lanes : 2;
    b->use_graph = settings->use_graph != 0;
    b->wpb = settings->warps_per_block > 0 ? settings->warps_per_block : 4;
    const size_t slot_bytes = (size_t)2 * cap * (D + 2) * sizeof(float);
    const size_t arena_budget = (size_t)32 << 30;
    const int max_attempts = settings->max_attempts > 0 ? settings->max_attempts : 4;
    const int active = settings->max_active > 0 ? std::min(settings->max_active, n) : n;
    int slots = active;
    if (max_attempts > 1) slots += std::max(64, n / 4);   // room for restarts and extra attempts
    slots = (int)std::max<size_t>(1, std::min<size_t>(slots, arena_budget / slot_bytes));
    b->slots = slots;
    b->path_rows = std::max(4096, n * 512);
    for (int i = 0; i < n; i++) b->num_goals.push_back(queries[i].num_goals);

    // one device blob for everything small
    size_t off = 0;
    const size_t o_cfg = off;
    off = align256(off + cfg.size() * sizeof(float));
    const size_t o_env = off;
    off = align256(off + std::max<size_t>(1, envs.size()) * sizeof(float4));
    const size_t o_desc = off;
    off = align256(off + n * sizeof(BatchQueryDesc));
    const size_t o_order = off;
    off = align256(off + n * sizeof(int));
    const size_t o_qstate = off;
    off = align256(off + n * sizeof(QueryState));
    const size_t o_slots = off;
    off = align256(off + slots * sizeof(SlotState));
    const size_t o_out = off;
    off = align256(off + n * sizeof(BatchOut));
    const size_t o_ctr = off;
    off = align256(off + sizeof(BatchCounters));
    const size_t o_path = off;
    off = align256(off + (size_t)b->path_rows * D * sizeof(float));
    prrtc_status s;
    if (cudaMalloc(&b->blob, off) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return c->fail(PRRTC_ENOMEM, "batch_create: cannot allocate %zu bytes", off);
    }
    char *base = static_cast<char *>(b->blob);
    float4 *env_dev = reinterpret_cast<float4 *>(base + o_env);
    for (int i = 0; i < n; i++)
        if (env_rec_off[i] >= 0) descs[i].env = env_dev + env_rec_off[i];
    if ((s = ensure_halton_bases(c, b->lanes * max_attempts)) ||
        (s = c->cuda(cudaMemcpyAsync(base + o_cfg, cfg.data(), cfg.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream), "batch upload")) ||
        (!envs.empty() && (s = c->cuda(cudaMemcpyAsync(env_dev, envs.data(), envs.size() * sizeof(float4), cudaMemcpyHostToDevice, c->stream), "batch upload"))) ||
        (s = c->cuda(cudaMemcpyAsync(base + o_desc, descs.data(), n * sizeof(BatchQueryDesc), cudaMemcpyHostToDevice, c->stream), "batch upload")) ||
        (s = take_arena(c, D, cap, slots, &b->arena)) ||
        (s = c->cuda(cudaEventCreate(&b->ev0), "event")) || (s = c->cuda(cudaEventCreate(&b->ev1), "event")) ||
        (s = c->cuda(cudaStreamSynchronize(c->stream), "batch upload"))) {
        prrtc_batch_free(ctx, b);
        return s;
    }
    // admission order: tightest start/goal clearance first (longest expected
    // solve first), so the hard queries do not start last and end the batch
    int *order_dev = nullptr;
    if (settings->admission == 0 && n > 1) {
        std::vector<float> score(n);
        if ((s = query_clearance(c, robot, reinterpret_cast<const BatchQueryDesc *>(base + o_desc),
                                 reinterpret_cast<const float *>(base + o_cfg), n, score.data()))) {
            prrtc_batch_free(ctx, b);
            return s;
        }
        std::vector<int> order(n);
        for (int i = 0; i < n; i++) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return score[x] < score[y]; });
        order_dev = reinterpret_cast<int *>(base + o_order);
        if ((s = c->cuda(cudaMemcpy(order_dev, order.data(), n * sizeof(int), cudaMemcpyHostToDevice), "batch order"))) {
            prrtc_batch_free(ctx, b);
            return s;
        }
    }
    BatchParams &P = b->P;
    P.order = order_dev;
    P.max_samples = S.max_samples;
    P.max_iters = S.max_iters;
    P.lanes = b->lanes;
    P.granularity = S.granularity;
    int max_records = 0;
    for (int i = 0; i < n; i++) max_records = std::max(max_records, descs[i].env_n.records());
    P.env_records = std::min(max_records, kWarpEnvRecords);
    P.range = S.range;
    P.balance = S.balance;
    P.tree_ratio = S.tree_ratio;
    P.dynamic_domain = S.dynamic_domain ? 1 : 0;
    P.dd_alpha = S.dd_alpha;
    P.dd_radius = S.dd_radius;
    P.dd_min_radius = S.dd_min_radius;
    P.pad = settings->margin;
    P.budget_ns = settings->time_budget_ns;
    P.num_queries = n;
    P.num_slots = slots;
    P.admit_slots = std::min(active, slots);
    P.cap = cap;
    P.path_pool_rows = b->path_rows;
    P.edge_order = settings->edge_order ? 1 : 0;
    P.sampler = settings->sampler ? 1 : 0;
    P.max_attempts = max_attempts;
    P.max_workers = settings->max_workers_per_attempt > 0 ? settings->max_workers_per_attempt : 1 << 30;
    P.bases_lanes = c->bases_lanes;
    P.restart_after_ns = settings->restart_after_ns ? settings->restart_after_ns : 10000000ull;
    P.idle_limit = settings->idle_wait_limit ? settings->idle_wait_limit : (1u << 22);
    P.shared_frames = settings->shared_frames ? 1 : 0;
    P.sub_rounds = settings->rounds_per_header > 0 ? std::min(settings->rounds_per_header, 64) : 4;
    // pRRTC stops a query when any of its num_new_configs lanes passes max_iters
    // (pRRTC.cu:343-346), i.e. after about max_iters x num_new_configs samples
    // below 2^31 with room for the tickets that warps take after the last one
    // (32 per warp per round): sample indices and Halton indices stay int
    P.max_samples_drawn = std::min<long long>((long long)S.max_iters * S.num_new_configs, kMaxSamplesDrawn);
    P.cfg_pool = reinterpret_cast<const float *>(base + o_cfg);
    P.queries = reinterpret_cast<const BatchQueryDesc *>(base + o_desc);
    P.qstate = reinterpret_cast<QueryState *>(base + o_qstate);
    P.slots = reinterpret_cast<SlotState *>(base + o_slots);
    P.out = reinterpret_cast<BatchOut *>(base + o_out);
    P.ctr = reinterpret_cast<BatchCounters *>(base + o_ctr);
    P.nodes = b->arena->nodes;
    P.parents = b->arena->parents;
    P.radii = b->arena->radii;
    P.path_pool = reinterpret_cast<float *>(base + o_path);
    P.halton_bases = c->bases;
    prrtc_robot_limits(robot, P.scale, P.offset);
    // launch shape
    const int occ = ops->batch_occupancy(b->wpb, P.env_records, P.shared_frames);
    int per_sm = settings->blocks_per_sm > 0 ? std::min(settings->blocks_per_sm, std::max(occ, 1)) : std::max(occ, 1);
    b->blocks = c->sms * per_sm;
    b->stats.blocks = b->blocks;
    b->stats.warps_per_block = b->wpb;
    b->stats.slots = slots;
    *out = b;
    return PRRTC_OK;
}

// The run sequence: reset slots, results and counters, then the launch.
static prrtc_status enqueue_run(Ctx *c, prrtc_batch *b, const RobotOps *ops)
{
    prrtc_status s;
    if ((s = c->cuda(cudaMemsetAsync(b->P.slots, 0, b->slots * sizeof(SlotState), c->stream), "batch reset")) ||
        (s = c->cuda(cudaMemsetAsync(b->P.qstate, 0, b->n * sizeof(QueryState), c->stream), "batch reset")) ||
        (s = c->cuda(cudaMemsetAsync(b->P.out, 0, b->n * sizeof(BatchOut), c->stream), "batch reset")) ||
        (s = c->cuda(cudaMemsetAsync(b->P.ctr, 0, sizeof(BatchCounters), c->stream), "batch reset")) ||
        (s = c->cuda(ops->solve_batch(b->P, b->blocks, b->wpb, c->stream), "batch launch")))
        return s;
    return PRRTC_OK;
}

extern "C" prrtc_status prrtc_batch_run(prrtc_ctx *ctx, prrtc_batch *b)
{
    Ctx *c = Ctx::of(ctx);
    if (!c || !b) return PRRTC_EINVAL;
    const RobotOps *ops = robot_ops(b->robot);
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    prrtc_status s;
    if (b->use_graph && !b->graph) {
        cudaGraph_t graph;
        if ((s = c->cuda(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "graph capture"))) return s;
        s = enqueue_run(c, b, ops);
        cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
        if (s) return s;
        if ((s = c->cuda(e, "graph capture"))) return s;
        e = cudaGraphInstantiate(&b->graph, graph, 0);
        cudaGraphDestroy(graph);
        if ((s = c->cuda(e, "graph instantiate"))) return s;
    }
    cudaEventRecord(b->ev0, c->stream);
    if (b->graph) {
        if ((s = c->cuda(cudaGraphLaunch(b->graph, c->stream), "graph launch"))) return s;
    } else if ((s = enqueue_run(c, b, ops))) {
        return s;
    }
    c->launches++;
    cudaEventRecord(b->ev1, c->stream);
    BatchCounters ctr;
    if ((s = c->cuda(cudaMemcpyAsync(&ctr, b->P.ctr, sizeof ctr, cudaMemcpyDeviceToHost, c->stream), "batch counters")) ||
        (s = c->cuda(cudaStreamSynchronize(c->stream), "batch run")))
        return s;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->stats.kernel_ns = (uint64_t)(ms * 1e6);
    b->stats.error = ctr.error;
    b->t0 = ctr.t0;
    b->stats.configs_checked = ctr.work[1];
    b->stats.extra_attempts = ctr.attempts;
    b->stats.flops = ctr.work[0];
    b->stats.nn_nodes = ctr.nn_nodes;
    b->stats.bulk_ns = ctr.t99 > ctr.t0 ? ctr.t99 - ctr.t0 : 0;
    b->stats.bulk_flops = ctr.work99[0];
    b->stats.bulk_configs = ctr.work99[1];
    b->ran = true;
    // every slot must be free again, i.e. its arena region back to NaN
    std::vector<SlotState> sl(b->slots);
    if ((s = c->cuda(cudaMemcpyAsync(sl.data(), b->P.slots, b->slots * sizeof(SlotState), cudaMemcpyDeviceToHost, c->stream), "batch slots")) ||
        (s = c->cuda(cudaStreamSynchronize(c->stream), "batch slots")))
        return s;
    bool clean = true;
    for (const SlotState &x : sl) clean = clean && x.state == SLOT_FREE;
    if (!clean || ctr.error) {
        const size_t nn = (size_t)b->arena->slots * 2 * b->dof * b->cap;
        if ((s = c->cuda(cudaMemsetAsync(b->arena->nodes, 0xFF, nn * sizeof(float), c->stream), "arena refill")) ||
            (s = c->cuda(cudaStreamSynchronize(c->stream), "arena refill")))
            return s;
        b->stats.error |= clean ? 0 : 2;
    }
    if (ctr.error) return c->fail(PRRTC_ECUDA, "batch: a worker gave up waiting for work");
    return PRRTC_OK;
}

extern "C" prrtc_status prrtc_batch_results(prrtc_ctx *ctx, prrtc_batch *b, prrtc_result *res)
{
    Ctx *c = Ctx::of(ctx);
    if (!c || !b || !res) return PRRTC_EINVAL;
    if (!b->ran) return c->fail(PRRTC_EINVAL, "batch_results: the batch has not run");
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    std::vector<BatchOut> outs(b->n);
    BatchCounters ctr;
    prrtc_status s;
    if ((s = c->cuda(cudaMemcpyAsync(outs.data(), b->P.out, b->n * sizeof(BatchOut), cudaMemcpyDeviceToHost, c->stream), "batch results")) ||
        (s = c->cuda(cudaMemcpyAsync(&ctr, b->P.ctr, sizeof ctr, cudaMemcpyDeviceToHost, c->stream), "batch results")) ||
        (s = c->cuda(cudaStreamSynchronize(c->stream), "batch results")))
        return s;
    const int rows = std::min(ctr.path_next, b->path_rows);
    std::vector<float> paths((size_t)std::max(rows, 1) * b->dof);
    if (rows > 0 &&
        ((s = c->cuda(cudaMemcpyAsync(paths.data(), b->P.path_pool, (size_t)rows * b->dof * sizeof(float), cudaMemcpyDeviceToHost, c->stream), "batch paths")) ||
         (s = c->cuda(cudaStreamSynchronize(c->stream), "batch paths"))))
        return s;
    int solved = 0;
    int64_t samples = 0;
    for (int i = 0; i < b->n; i++) {
        const BatchOut &o = outs[i];
        prrtc_result &r = res[i];
        r.solved = o.solved;
        r.status = o.t_admit == 0 ? (b->P.budget_ns ? PRRTC_ETIMEDOUT : PRRTC_ECUDA) : o.status;
        r.start_tree_size = o.start_tree_size;
        r.goal_tree_size = o.goal_tree_size;
        r.path_length = o.path_length;
        r.iters = o.solved ? o.iters : -1;
        r.cost = o.cost;
        r.kernel_ns = o.t_done > o.t_admit ? o.t_done - o.t_admit : 0;
        r.finish_ns = (o.t_done > b->t0 && b->t0) ? o.t_done - b->t0 : 0;
        r.samples = o.samples;
        r.wall_ns = b->stats.kernel_ns;
        r.copy_ns = 0;
        r.path_rows = 0;
        solved += o.solved;
        samples += o.samples;
        if (o.solved && o.path_rows > 0 && o.path_off + o.path_rows <= rows) {
            r.path_rows = o.path_rows;
            if (r.path && r.path_capacity >= o.path_rows)
                std::memcpy(r.path, paths.data() + (size_t)o.path_off * b->dof, sizeof(float) * o.path_rows * b->dof);
            else if (r.path)
                r.status = PRRTC_EINVAL;
        }
    }
    b->stats.solved = solved;
    b->stats.samples = samples;
    return PRRTC_OK;
}

extern "C" prrtc_status prrtc_batch_stats_get(prrtc_ctx *ctx, const prrtc_batch *b, prrtc_batch_stats *st)
{
    if (!ctx || !b || !st) return PRRTC_EINVAL;
    *st = b->stats;
    return PRRTC_OK;
}

extern "C" prrtc_status prrtc_batch_free(prrtc_ctx *ctx, prrtc_batch *b)
{
    Ctx *c = Ctx::of(ctx);
    if (!c || !b) return PRRTC_EINVAL;
    {
        std::lock_guard<std::mutex> g(c->mu);
        cudaSetDevice(c->device);
        cudaStreamSynchronize(c->stream);
        if (b->graph) cudaGraphExecDestroy(b->graph);
        if (b->ev0) cudaEventDestroy(b->ev0);
        if (b->ev1) cudaEventDestroy(b->ev1);
        cudaFree(b->blob);
        give_back_arena(c, b->arena);
    }
    delete b;
    return PRRTC_OK;
}

extern "C" prrtc_status prrtc_solve_batch(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_query *queries, int n,
                                          const prrtc_batch_settings *settings, prrtc_result *results)
{
    const auto t0 = std::chrono::steady_clock::now();
    prrtc_batch *b = nullptr;
    prrtc_status s = prrtc_batch_create(ctx, robot, queries, n, settings, &b);
    if (s) return s;
    const auto t1 = std::chrono::steady_clock::now();
    if (!(s = prrtc_batch_run(ctx, b))) s = prrtc_batch_results(ctx, b, results);
    const auto t2 = std::chrono::steady_clock::now();
    const uint64_t up = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0).count();
    const uint64_t all = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t2 - t0).count();
    if (!s)
        for (int i = 0; i < n; i++) {
            results[i].wall_ns = all;
            results[i].copy_ns = up;
        }
    prrtc_batch_free(ctx, b);
    return s;
}
