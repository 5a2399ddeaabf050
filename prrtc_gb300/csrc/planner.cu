// Host side of the plain-form planner: prrtc_solve (replaces
// pRRTC::solve<Robot>, src/planning/pRRTC.cu:607-766).
//
// Differences from the reference's host code, all deliberate:
//  * device buffers live in the context and are reused across calls (the
//    reference mallocs and frees every array per query and finishes with
//    cudaDeviceReset, pRRTC.cu:629-665,748-764);
//  * the node arena is filled with NaN by one cudaMemsetAsync instead of a
//    host-built -9999 array copied over PCIe (pRRTC.cu:644-646);
//  * every per-query value sits in a QueryCtl block, not in file-scope
//    __device__ globals, so contexts are independent.
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cstring>
#include <vector>

#include <curand_kernel.h>

#include "context.h"
#include "prrtc_internal.h"

namespace prrtc {

struct PlannerState {
    int dof = 0, cap = 0, path_cap = 0;
    float *nodes = nullptr;     // [2][dof][cap]
    int *parents = nullptr;     // [2][cap]
    float *radii = nullptr;     // [2][cap]
    float *path = nullptr;      // [2][path_cap][dof]
    QueryCtl *ctl = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

__global__ void k_halton_bases(float *out, int lanes)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= lanes) return;
    float primes[16] = {3.f, 5.f, 7.f, 11.f, 13.f, 17.f, 19.f, 23.f, 29.f, 31.f, 37.f, 41.f, 43.f, 47.f, 53.f, 59.f};
    if (idx != 0) {
        curandState st;
        curand_init(1ull + idx, idx, 0, &st);
        for (int i = 15; i > 0; i--) {  // Fisher-Yates, as shuffle_array (pRRTC.cu:49-56)
            const int j = curand(&st) % (i + 1);
            const float tmp = primes[i];
            primes[i] = primes[j];
            primes[j] = tmp;
        }
    }
    for (int i = 0; i < 16; i++) out[idx * 16 + i] = primes[i];
}

cudaError_t launch_halton_bases(float *out, int lanes, cudaStream_t st)
{
    k_halton_bases<<<(lanes + 63) / 64, 64, 0, st>>>(out, lanes);
    return cudaGetLastError();
}

static void free_state(PlannerState *p)
{
    if (!p) return;
    cudaFree(p->nodes);
    cudaFree(p->parents);
    cudaFree(p->radii);
    cudaFree(p->path);
    cudaFree(p->ctl);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
}

prrtc_status ensure_halton_bases(Ctx *c, int lanes)
{
    if (c->bases_lanes >= lanes) return PRRTC_OK;
    cudaFree(c->bases);
    c->bases = nullptr;
    c->bases_lanes = 0;
    const int want = std::max(lanes, 1024);
    if (cudaMalloc(&c->bases, sizeof(float) * 16 * want) != cudaSuccess) {
        cudaGetLastError();
        return c->fail(PRRTC_ENOMEM, "cannot allocate Halton bases");
    }
    prrtc_status s = c->cuda(launch_halton_bases(c->bases, want, c->stream), "halton bases");
    if (s) return s;
    c->launches++;
    c->bases_lanes = want;
    return PRRTC_OK;
}

void Ctx::release_planner_state()
{
    cudaFree(bases);
    bases = nullptr;
    bases_lanes = 0;
    if (planner) {
        free_state(planner);
        delete planner;
        planner = nullptr;
    }
}

static constexpr int kPathCap = 65536;

// Make sure trees of `cap` nodes, `lanes` Halton lanes and the path buffer exist.
static prrtc_status ensure_state(Ctx *c, int dof, int cap, int lanes)
{
    if (!c->planner) {
        c->planner = new PlannerState();
        if (cudaEventCreate(&c->planner->ev0) != cudaSuccess || cudaEventCreate(&c->planner->ev1) != cudaSuccess)
            return c->cuda(cudaGetLastError(), "event create");
    }
    PlannerState *p = c->planner;
    if (p->dof != dof || p->cap < cap) {
        cudaFree(p->nodes);
        cudaFree(p->parents);
        cudaFree(p->radii);
        cudaFree(p->path);
        p->nodes = nullptr;
        p->parents = nullptr;
        p->radii = nullptr;
        p->path = nullptr;
        p->dof = 0;
        p->cap = 0;
        const int path_cap = std::min(cap, kPathCap);
        if (cudaMalloc(&p->nodes, sizeof(float) * 2 * (size_t)dof * cap) != cudaSuccess ||
            cudaMalloc(&p->parents, sizeof(int) * 2 * (size_t)cap) != cudaSuccess ||
            cudaMalloc(&p->radii, sizeof(float) * 2 * (size_t)cap) != cudaSuccess ||
            cudaMalloc(&p->path, sizeof(float) * 2 * (size_t)path_cap * dof) != cudaSuccess) {
            cudaGetLastError();
            return c->fail(PRRTC_ENOMEM, "solve: cannot allocate trees of %d nodes", cap);
        }
        p->dof = dof;
        p->cap = cap;
        p->path_cap = path_cap;
    }
    if (!p->ctl && cudaMalloc(&p->ctl, sizeof(QueryCtl)) != cudaSuccess) {
        cudaGetLastError();
        return c->fail(PRRTC_ENOMEM, "solve: cannot allocate control block");
    }
    return PRRTC_OK;
}

}  // namespace prrtc

using namespace prrtc;

static uint64_t ns_since(std::chrono::steady_clock::time_point t0)
{
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
}

extern "C" prrtc_status prrtc_solve(prrtc_ctx *ctx, prrtc_robot robot, const float *start, const float *goals,
                                    int num_goals, const prrtc_env *env, const prrtc_settings *settings,
                                    prrtc_result *res)
{
    const auto wall0 = std::chrono::steady_clock::now();
    Ctx *c = Ctx::of(ctx);
    const RobotOps *ops = robot_ops(robot);
    const Env *e = reinterpret_cast<const Env *>(env);
    if (!c) return PRRTC_EINVAL;
    if (!ops || !e || !start || !goals || num_goals < 1 || !settings || !res)
        return c->fail(PRRTC_EINVAL, "solve: bad argument");
    const prrtc_settings &S = *settings;
    if (S.num_new_configs < 1 || S.granularity < 1 || S.granularity > 1024 || S.max_samples < num_goals + 1 ||
        S.max_iters < 0 || !(S.range > 0.0f))
        return c->fail(PRRTC_EINVAL, "solve: bad settings");
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    const int D = ops->dof;
    const int cap = (S.max_samples + 3) & ~3;
    prrtc_status s = ensure_state(c, D, cap, S.num_new_configs);
    if (s) return s;
    if ((s = ensure_halton_bases(c, S.num_new_configs))) return s;
    PlannerState *p = c->planner;
    cudaStream_t st = c->stream;

    // reset the arena: NaN nodes, control block, roots (pRRTC.cu:643-693)
    if ((s = c->cuda(cudaMemsetAsync(p->nodes, 0xFF, sizeof(float) * 2 * (size_t)D * p->cap, st), "arena reset"))) return s;
    if ((s = c->cuda(cudaMemsetAsync(p->ctl, 0, sizeof(QueryCtl), st), "ctl reset"))) return s;
    std::vector<float> roots((size_t)D * num_goals);
    std::vector<int> root_par(num_goals);
    std::vector<float> root_rad(num_goals, FLT_MAX);
    for (int i = 0; i < num_goals; i++) {
        root_par[i] = i;
        for (int d = 0; d < D; d++) roots[(size_t)d * num_goals + i] = goals[(size_t)i * D + d];
    }
    const auto copy0 = std::chrono::steady_clock::now();
    float *tree0 = p->nodes, *tree1 = p->nodes + (size_t)D * p->cap;
    int *par0 = p->parents, *par1 = p->parents + p->cap;
    float *rad0 = p->radii, *rad1 = p->radii + p->cap;
    const int zero = 0, one = 1;
    QueryCtl init{};
    init.free_index[0] = 1;
    init.free_index[1] = num_goals;
    init.solved_iters = -1;
    if ((s = c->cuda(cudaMemcpy2DAsync(tree0, sizeof(float) * p->cap, start, sizeof(float), sizeof(float), D,
                                       cudaMemcpyHostToDevice, st), "start upload")) ||
        (s = c->cuda(cudaMemcpy2DAsync(tree1, sizeof(float) * p->cap, roots.data(), sizeof(float) * num_goals,
                                       sizeof(float) * num_goals, D, cudaMemcpyHostToDevice, st), "goal upload")) ||
        (s = c->cuda(cudaMemcpyAsync(par0, &zero, sizeof(int), cudaMemcpyHostToDevice, st), "root parent")) ||
        (s = c->cuda(cudaMemcpyAsync(par1, root_par.data(), sizeof(int) * num_goals, cudaMemcpyHostToDevice, st), "goal parents")) ||
        (s = c->cuda(cudaMemcpyAsync(rad0, root_rad.data(), sizeof(float), cudaMemcpyHostToDevice, st), "root radius")) ||
        (s = c->cuda(cudaMemcpyAsync(rad1, root_rad.data(), sizeof(float) * num_goals, cudaMemcpyHostToDevice, st), "goal radii")) ||
        (s = c->cuda(cudaMemcpyAsync(p->ctl, &init, sizeof(QueryCtl), cudaMemcpyHostToDevice, st), "ctl init")))
        return s;
    (void)one;
    if ((s = c->cuda(cudaStreamSynchronize(st), "upload"))) return s;
    uint64_t copy_ns = ns_since(copy0);

    PlainParams P{};
    P.max_samples = S.max_samples;
    P.max_iters = S.max_iters;
    P.num_new_configs = S.num_new_configs;
    P.granularity = S.granularity;
    P.range = S.range;
    P.balance = S.balance;
    P.tree_ratio = S.tree_ratio;
    P.dynamic_domain = S.dynamic_domain ? 1 : 0;
    P.dd_alpha = S.dd_alpha;
    P.dd_radius = S.dd_radius;
    P.dd_min_radius = S.dd_min_radius;
    P.pad = c->plan_pad;
    P.budget_ns = c->budget_ns;
    P.nodes[0] = tree0;
    P.nodes[1] = tree1;
    P.parents[0] = par0;
    P.parents[1] = par1;
    P.radii[0] = rad0;
    P.radii[1] = rad1;
    P.cap = p->cap;
    P.halton_bases = c->bases;
    prrtc_robot_limits(robot, P.scale, P.offset);
    P.env = e->dev;
    P.env_n = e->counts;
    P.ctl = p->ctl;
    P.path = p->path;
    P.path_cap = p->path_cap;
    P.work = c->work_dev;
    int threads = ((S.granularity + 31) / 32) * 32;
    if (threads > 256) threads = 256;

    cudaEventRecord(p->ev0, st);
    if ((s = c->cuda(ops->solve_plain(P, threads, st), "planner launch"))) return s;
    c->launches++;
    cudaEventRecord(p->ev1, st);
    QueryCtl out{};
    if ((s = c->cuda(cudaMemcpyAsync(&out, p->ctl, sizeof(QueryCtl), cudaMemcpyDeviceToHost, st), "ctl read")) ||
        (s = c->cuda(cudaStreamSynchronize(st), "planner")))
        return s;
    float kms = 0.0f;
    cudaEventElapsedTime(&kms, p->ev0, p->ev1);

    const auto copy1 = std::chrono::steady_clock::now();
    res->solved = out.solved == 1 ? 1 : 0;
    res->status = out.solved == -2 ? PRRTC_ETIMEDOUT : PRRTC_OK;
    res->start_tree_size = out.free_index[0];
    res->goal_tree_size = out.free_index[1];
    res->iters = out.solved == 1 ? out.solved_iters : -1;
    res->cost = 0.0f;
    res->path_length = 0;
    res->path_rows = 0;
    if (res->solved) {
        if (out.error & 1) return c->fail(PRRTC_ENOMEM, "solve: path longer than %d nodes", p->path_cap);
        const int n1 = out.path_size[1], n0 = out.path_size[0];
        std::vector<float> seg((size_t)(n0 + n1) * D);
        if (n0 && (s = c->cuda(cudaMemcpyAsync(seg.data(), p->path, sizeof(float) * n0 * D, cudaMemcpyDeviceToHost, st), "path read")))
            return s;
        if (n1 && (s = c->cuda(cudaMemcpyAsync(seg.data() + (size_t)n0 * D, p->path + (size_t)p->path_cap * D,
                                               sizeof(float) * n1 * D, cudaMemcpyDeviceToHost, st), "path read")))
            return s;
        if ((s = c->cuda(cudaStreamSynchronize(st), "path read"))) return s;
        res->cost = out.cost;
        res->path_length = n0 + n1;
        // goal, goal-tree segment reversed, start-tree segment, start (pRRTC.cu:731-741)
        const int rows = n0 + n1 + 2;
        res->path_rows = rows;
        if (res->path && res->path_capacity >= rows) {
            float *w = res->path;
            const int gi = std::min(std::max(out.reached_goal, 0), num_goals - 1);
            std::memcpy(w, goals + (size_t)gi * D, sizeof(float) * D);
            w += D;
            for (int i = n1 - 1; i >= 0; i--, w += D) std::memcpy(w, seg.data() + (size_t)(n0 + i) * D, sizeof(float) * D);
            for (int i = 0; i < n0; i++, w += D) std::memcpy(w, seg.data() + (size_t)i * D, sizeof(float) * D);
            std::memcpy(w, start, sizeof(float) * D);
        } else if (res->path) {
            res->status = PRRTC_EINVAL;
            c->fail(PRRTC_EINVAL, "solve: path needs %d rows, capacity %d", rows, res->path_capacity);
        }
    }
    copy_ns += ns_since(copy1);
    res->kernel_ns = (uint64_t)(kms * 1e6);
    res->copy_ns = copy_ns;
    res->finish_ns = res->kernel_ns;
    res->samples = 0;
    res->wall_ns = ns_since(wall0);
    return (prrtc_status)res->status;
}
