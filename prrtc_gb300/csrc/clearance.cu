// Differentiable clearance, host side: prrtc_path_cost_grad (cost and joint
// gradient of every waypoint) and prrtc_smooth_paths (gradient smoothing
// judged by the checker).  The cost and its adjoint are in
// clearance_device.cuh; the smoothing kernel, which needs each robot's own
// checker, is in clearance_kernel.cuh.  No reference counterpart.
#include <algorithm>
#include <cstring>
#include <vector>

#include "clearance_device.cuh"
#include "clearance_model.h"
#include "context.h"
#include "prrtc_internal.h"

namespace prrtc {

// Every waypoint of every path: one thread per waypoint, blocks of 64
// waypoints of one path, the path's obstacles staged in shared memory.
__global__ void __launch_bounds__(64) k_path_cost_grad(ClrModel M, const ClrEnv *__restrict__ envs, int waypoints,
                                                      const float *__restrict__ q, float margin,
                                                      float *__restrict__ cost, float *__restrict__ grad)
{
    extern __shared__ float4 s_env[];
    __shared__ unsigned long long s_bar;
    const int path = blockIdx.y;
    const ClrEnv pe = envs[path];
    stage_env_bulk(s_env, pe.rec, pe.n.records(), &s_bar);
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= waypoints) return;
    const size_t row = (size_t)path * waypoints + w;
    float g[kClrMaxJoints];
    cost[row] = clr::cost_grad(M, ClrEnv{s_env, pe.n}, q + row * M.dof, margin, 1.0f, g);
    for (int d = 0; d < M.dof; d++) grad[row * M.dof + d] = g[d];
}

// One thread per query: the smallest clearance of its start and goals.
__global__ void __launch_bounds__(64) k_query_clearance(ClrModel M, const BatchQueryDesc *__restrict__ queries,
                                                       const float *__restrict__ cfg, int n, float *__restrict__ score)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const BatchQueryDesc d = queries[i];
    const ClrEnv e{d.env, d.env_n};
    float best = 3.4e38f;
    for (int c = 0; c <= d.num_goals; c++) best = fminf(best, clr::min_clearance(M, e, cfg + d.cfg_off + c * M.dof));
    score[i] = best;
}

namespace {

size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

}  // namespace

struct ClearanceState {
    void *tables[4] = {};
    ClrModel model[4] = {};
    ClrEnv *envs = nullptr;   // per-path obstacle table on the device
    int envs_cap = 0;
};

void release_clearance_state(Ctx *c)
{
    if (!c->clearance) return;
    for (void *p : c->clearance->tables) cudaFree(p);
    cudaFree(c->clearance->envs);
    delete c->clearance;
    c->clearance = nullptr;
}

// The robot's tables on the device, uploaded on first use.  Caller holds
// c->mu with the device current.
static prrtc_status model_on_device(Ctx *c, prrtc_robot robot, ClrModel *model)
{
    if (!c->clearance) c->clearance = new ClearanceState();
    ClearanceState *cs = c->clearance;
    if (!cs->tables[robot]) {
        const ClrHostModel &h = clr_host_model(robot);
        const void *src[7] = {h.joints.data(), h.parent.data(), h.leaf.data(),     h.leaf_joint.data(),
                              h.pa.data(),     h.pb.data(),     h.pair_joint.data()};
        const size_t bytes[7] = {h.joints.size() * sizeof(prrtc_joint_def), h.parent.size() * sizeof(int),
                                 h.leaf.size() * sizeof(float4),            h.leaf_joint.size() * sizeof(int),
                                 h.pa.size() * sizeof(float4),              h.pb.size() * sizeof(float4),
                                 h.pair_joint.size() * sizeof(int2)};
        size_t off[7], total = 0;
        for (int k = 0; k < 7; k++) {
            off[k] = total;
            total += al16(std::max<size_t>(bytes[k], 16));
        }
        std::vector<char> blob(total, 0);
        for (int k = 0; k < 7; k++)
            if (bytes[k]) memcpy(blob.data() + off[k], src[k], bytes[k]);
        char *d = nullptr;
        if (cudaMalloc(&d, total) != cudaSuccess) {
            cudaGetLastError();
            return c->fail(PRRTC_ENOMEM, "clearance: robot tables (%zu bytes)", total);
        }
        const cudaError_t e = cudaMemcpy(d, blob.data(), total, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(d);
            return c->cuda(e, "clearance: robot tables");
        }
        ClrModel &m = cs->model[robot];
        m.dof = h.dof;
        m.nj = (int)h.joints.size();
        m.n_leaf = (int)h.leaf.size();
        m.n_pair = (int)h.pa.size();
        m.joints = (const prrtc_joint_def *)(d + off[0]);
        m.joint_parent = (const int *)(d + off[1]);
        m.leaf = (const float4 *)(d + off[2]);
        m.leaf_joint = (const int *)(d + off[3]);
        m.pair_a = (const float4 *)(d + off[4]);
        m.pair_b = (const float4 *)(d + off[5]);
        m.pair_joint = (const int2 *)(d + off[6]);
        cs->tables[robot] = d;
    }
    *model = cs->model[robot];
    return PRRTC_OK;
}

// The robot's tables and the per-path obstacle table of this call.  Caller
// holds c->mu with the device current.
static prrtc_status prepare(Ctx *c, prrtc_robot robot, const prrtc_env *const *envs, int n_paths, ClrModel *model,
                            int *max_records)
{
    prrtc_status s = model_on_device(c, robot, model);
    if (s) return s;
    ClearanceState *cs = c->clearance;
    std::vector<ClrEnv> table(n_paths);
    int mr = 0;
    for (int i = 0; i < n_paths; i++) {
        const Env *e = reinterpret_cast<const Env *>(envs[i]);
        if (!e) return c->fail(PRRTC_EINVAL, "clearance: environment of path %d is null", i);
        table[i] = ClrEnv{e->dev, e->counts};
        mr = std::max(mr, e->counts.records());
    }
    // earlier work on the context's stream may still read the old table
    if ((s = c->cuda(cudaStreamSynchronize(c->stream), "clearance: stream"))) return s;
    if (cs->envs_cap < n_paths) {
        cudaFree(cs->envs);
        cs->envs = nullptr;
        cs->envs_cap = 0;
        if (cudaMalloc(&cs->envs, sizeof(ClrEnv) * n_paths) != cudaSuccess) {
            cudaGetLastError();
            return c->fail(PRRTC_ENOMEM, "clearance: obstacle table for %d paths", n_paths);
        }
        cs->envs_cap = n_paths;
    }
    *max_records = mr;
    // `table` is pageable and local: a synchronous copy
    return c->cuda(cudaMemcpy(cs->envs, table.data(), sizeof(ClrEnv) * n_paths, cudaMemcpyHostToDevice),
                   "clearance: obstacle table");
}

prrtc_status query_clearance(Ctx *c, prrtc_robot robot, const BatchQueryDesc *queries, const float *cfg_pool, int n,
                             float *score)
{
    ClrModel M;
    prrtc_status s = model_on_device(c, robot, &M);
    if (s) return s;
    float *d = static_cast<float *>(c->scratch(3, (size_t)n * sizeof(float)));
    if (!d) return c->fail(PRRTC_ENOMEM, "query_clearance: scratch");
    k_query_clearance<<<(n + 63) / 64, 64, 0, c->stream>>>(M, queries, cfg_pool, n, d);
    if ((s = c->cuda(cudaGetLastError(), "query_clearance: launch"))) return s;
    c->launches++;
    if ((s = c->cuda(cudaMemcpyAsync(score, d, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, c->stream),
                     "query_clearance: copy")))
        return s;
    return c->cuda(cudaStreamSynchronize(c->stream), "query_clearance");
}

}  // namespace prrtc

using namespace prrtc;

extern "C" prrtc_status prrtc_path_cost_grad(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_env *const *envs,
                                             int n_paths, int waypoints, const float *q, float margin, float *cost,
                                             float *grad)
{
    Ctx *c = Ctx::of(ctx);
    if (!c) return PRRTC_EINVAL;
    const RobotOps *ops = robot_ops(robot);
    if (!ops || n_paths < 0 || waypoints < 1 || !(margin >= 0.0f) || (n_paths > 0 && (!envs || !q || !cost || !grad)))
        return c->fail(PRRTC_EINVAL, "path_cost_grad: bad argument");
    if (n_paths > 65535) return c->fail(PRRTC_EINVAL, "path_cost_grad: at most 65535 paths per call");
    if (n_paths == 0) return PRRTC_OK;
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    ClrModel M;
    int max_rec = 0;
    prrtc_status s;
    if ((s = prepare(c, robot, envs, n_paths, &M, &max_rec))) return s;
    const size_t rows = (size_t)n_paths * waypoints;
    void *dq, *dcost, *dgrad;
    if ((s = c->device_view(q, rows * M.dof * sizeof(float), 0, true, &dq)) ||
        (s = c->device_view(cost, rows * sizeof(float), 1, false, &dcost)) ||
        (s = c->device_view(grad, rows * M.dof * sizeof(float), 2, false, &dgrad)))
        return s;
    const dim3 grid((waypoints + 63) / 64, n_paths);
    k_path_cost_grad<<<grid, 64, (size_t)max_rec * sizeof(float4), c->stream>>>(
        M, c->clearance->envs, waypoints, (const float *)dq, margin, (float *)dcost, (float *)dgrad);
    if ((s = c->cuda(cudaGetLastError(), "path_cost_grad: launch"))) return s;
    c->launches++;
    if (dcost != cost && (s = c->cuda(cudaMemcpyAsync(cost, dcost, rows * sizeof(float), cudaMemcpyDeviceToHost,
                                                      c->stream),
                                      "path_cost_grad: copy")))
        return s;
    if (dgrad != grad && (s = c->cuda(cudaMemcpyAsync(grad, dgrad, rows * M.dof * sizeof(float),
                                                      cudaMemcpyDeviceToHost, c->stream),
                                      "path_cost_grad: copy")))
        return s;
    return c->cuda(cudaStreamSynchronize(c->stream), "path_cost_grad");
}

extern "C" void prrtc_smooth_settings_default(prrtc_smooth_settings *s)
{
    if (!s) return;
    s->margin = 0.02f;
    s->steps = 50;
    s->step = 0.05f;
    s->cost_weight = 100.0f;
    s->smooth_weight = 1.0f;
    s->granularity = 128;
    s->shortcut_rounds = 8;
}

extern "C" prrtc_status prrtc_smooth_paths(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_env *const *envs,
                                           int n_paths, int waypoints, float *q, const prrtc_smooth_settings *settings,
                                           uint8_t *accepted, float *cost_before, float *cost_after)
{
    Ctx *c = Ctx::of(ctx);
    if (!c) return PRRTC_EINVAL;
    const RobotOps *ops = robot_ops(robot);
    if (!ops || !settings || n_paths < 0 || waypoints < 2 || waypoints > 256 ||
        (n_paths > 0 && (!envs || !q || !accepted)))
        return c->fail(PRRTC_EINVAL, "smooth_paths: bad argument (2 <= waypoints <= 256)");
    const prrtc_smooth_settings &st = *settings;
    if (!(st.margin >= 0.0f) || st.steps < 0 || !(st.step >= 0.0f) || !(st.cost_weight >= 0.0f) ||
        !(st.smooth_weight >= 0.0f) || st.granularity < 1 || st.granularity > (1 << 20) || st.shortcut_rounds < 0)
        return c->fail(PRRTC_EINVAL, "smooth_paths: bad settings");
    if (n_paths == 0) return PRRTC_OK;
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    ClrLaunch P{};
    int max_rec = 0;
    prrtc_status s;
    if ((s = prepare(c, robot, envs, n_paths, &P.M, &max_rec))) return s;
    float scale[kClrMaxJoints], offset[kClrMaxJoints];
    if ((s = prrtc_robot_limits(robot, scale, offset))) return c->fail(s, "smooth_paths: limits");
    for (int d = 0; d < P.M.dof; d++) {
        P.lo[d] = offset[d];
        P.hi[d] = offset[d] + scale[d];
    }
    const size_t rows = (size_t)n_paths * waypoints;
    void *dq, *dacc, *dcb = nullptr, *dca = nullptr;
    if ((s = c->device_view(q, rows * P.M.dof * sizeof(float), 0, true, &dq)) ||
        (s = c->device_view(accepted, (size_t)n_paths, 1, false, &dacc)) ||
        (cost_before && (s = c->device_view(cost_before, n_paths * sizeof(float), 2, false, &dcb))) ||
        (cost_after && (s = c->device_view(cost_after, n_paths * sizeof(float), 3, false, &dca))))
        return s;
    P.envs = c->clearance->envs;
    P.n_paths = n_paths;
    P.waypoints = waypoints;
    P.q = (float *)dq;
    P.s = ClrSmooth{st.margin, st.step, st.cost_weight, st.smooth_weight, st.steps, st.granularity, st.shortcut_rounds};
    P.accepted = (uint8_t *)dacc;
    P.cost_before = (float *)dcb;
    P.cost_after = (float *)dca;
    if ((s = c->cuda(ops->smooth_paths(P, (size_t)max_rec * sizeof(float4), c->stream), "smooth_paths: launch")))
        return s;
    c->launches++;
    auto back = [&](void *host, void *dev, size_t bytes) -> prrtc_status {
        if (!host || host == dev) return PRRTC_OK;
        return c->cuda(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->stream), "smooth_paths: copy");
    };
    if ((s = back(q, dq, rows * P.M.dof * sizeof(float))) || (s = back(accepted, dacc, n_paths)) ||
        (s = back(cost_before, dcb, n_paths * sizeof(float))) || (s = back(cost_after, dca, n_paths * sizeof(float))))
        return s;
    return c->cuda(cudaStreamSynchronize(c->stream), "smooth_paths");
}
