// C ABI: contexts, environments, collision checking (include/prrtc/prrtc.h).
#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "prrtc_internal.h"
#include "context.h"

using namespace prrtc;

namespace prrtc {

const RobotOps *robot_ops(prrtc_robot r)
{
    static const RobotOps ops[4] = {robot_ops_sphere(), robot_ops_panda(), robot_ops_fetch(), robot_ops_baxter()};
    if ((int)r < 0 || (int)r > 3) return nullptr;
    return &ops[(int)r];
}

// Joint scaling of the reference sampler (Robots.hh get_s_m / get_s_a).
struct Limits {
    int dof;
    float scale[14];
    float offset[14];
};

const Limits *robot_limits(prrtc_robot r)
{
    static const Limits sphere = {3, {10.0f, 10.0f, 10.0f}, {-5.0f, -5.0f, -5.0f}};                // Robots.hh:190-237
    static const Limits panda = {7,                                                                 // Robots.hh:10-64
                                 {5.9342f, 3.6652f, 5.9342f, 3.2289f, 5.9342f, 3.9095999999999997f, 5.9342f},
                                 {-2.9671f, -1.8326f, -2.9671f, -3.1416f, -2.9671f, -0.0873f, -2.9671f}};
    static const Limits fetch = {8,                                                                 // Robots.hh:66-120
                                 {0.38615f, 3.2112f, 2.739f, 6.28318f, 4.502f, 6.28318f, 4.32f, 6.28318f},
                                 {0.0f, -1.6056f, -1.221f, -3.14159f, -2.251f, -3.14159f, -2.16f, -3.14159f}};
    static const Limits baxter = {14,                                                               // Robots.hh:122-188
                                  {3.40335987756f, 3.194f, 6.10835987756f, 2.6679999999999997f, 6.118f,
                                   3.66479632679f, 6.118f, 3.40335987756f, 3.194f, 6.10835987756f,
                                   2.6679999999999997f, 6.118f, 3.66479632679f, 6.118f},
                                  {-1.70167993878f, -2.147f, -3.05417993878f, -0.05f, -3.059f, -1.57079632679f,
                                   -3.059f, -1.70167993878f, -2.147f, -3.05417993878f, -0.05f, -3.059f,
                                   -1.57079632679f, -3.059f}};
    switch (r) {
    case PRRTC_ROBOT_SPHERE: return &sphere;
    case PRRTC_ROBOT_PANDA: return &panda;
    case PRRTC_ROBOT_FETCH: return &fetch;
    case PRRTC_ROBOT_BAXTER: return &baxter;
    }
    return nullptr;
}

prrtc_status Ctx::fail(prrtc_status s, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    last_error = buf;
    return s;
}

prrtc_status Ctx::cuda(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return PRRTC_OK;
    cudaGetLastError();
    return fail(PRRTC_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

bool Ctx::is_device_ptr(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

void *Ctx::scratch(int slot, size_t bytes)
{
    Buf &b = bufs[slot];
    if (b.bytes >= bytes) return b.ptr;
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    size_t want = std::max<size_t>(bytes, 1 << 20);
    if (cudaMalloc(&b.ptr, want) != cudaSuccess) {
        cudaGetLastError();
        b.ptr = nullptr;
        return nullptr;
    }
    b.bytes = want;
    return b.ptr;
}

// Device view of a caller array: the array itself if it is device memory,
// else a scratch copy (copied in when `in` is true).
prrtc_status Ctx::device_view(const void *p, size_t bytes, int slot, bool in, void **out)
{
    if (is_device_ptr(p)) {
        *out = const_cast<void *>(p);
        return PRRTC_OK;
    }
    void *d = scratch(slot, bytes);
    if (!d) return fail(PRRTC_ENOMEM, "cannot allocate %zu bytes of scratch", bytes);
    if (in && bytes) {
        prrtc_status s = cuda(cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, stream), "copy in");
        if (s) return s;
    }
    *out = d;
    return PRRTC_OK;
}

}  // namespace prrtc

// ---------------------------------------------------------------- C ABI

// 8 independent FMA chains per thread: enough ILP to fill the FP32 pipe.
__global__ void k_fma_peak(float *out, int iters, float a, float b)
{
    float x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-7f + i;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = fmaf(x[i], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    if (s == 12345.0f) out[0] = s;   // keeps the chains live
}

extern "C" {

const char *prrtc_status_string(prrtc_status s)
{
    switch (s) {
    case PRRTC_OK: return "ok";
    case PRRTC_EINVAL: return "invalid argument";
    case PRRTC_ENOMEM: return "out of memory";
    case PRRTC_ETIMEDOUT: return "device time budget exhausted";
    case PRRTC_ECUDA: return "CUDA error";
    case PRRTC_EUNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

prrtc_status prrtc_create(prrtc_ctx **out, int device)
{
    if (!out) return PRRTC_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return PRRTC_ECUDA;
    }
    Ctx *c = new Ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaMalloc(&c->work_dev, 2 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(c->work_dev, 0, 2 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaEventCreate(&c->kev[0]) != cudaSuccess || cudaEventCreate(&c->kev[1]) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return PRRTC_ECUDA;
    }
    *out = reinterpret_cast<prrtc_ctx *>(c);
    return PRRTC_OK;
}

prrtc_status prrtc_destroy(prrtc_ctx *ctx)
{
    Ctx *c = Ctx::of(ctx);
    if (!c) return PRRTC_EINVAL;
    {
        std::lock_guard<std::mutex> g(c->mu);
        cudaSetDevice(c->device);
        cudaStreamSynchronize(c->stream);
        for (auto &b : c->bufs)
            if (b.ptr) cudaFree(b.ptr);
        c->release_planner_state();
        release_arena(c);
        release_clearance_state(c);
        cudaFree(c->work_dev);
        for (cudaEvent_t ev : c->kev)
            if (ev) cudaEventDestroy(ev);
        cudaStreamDestroy(c->stream);
    }
    delete c;
    return PRRTC_OK;
}

prrtc_status prrtc_last_kernel_ns(prrtc_ctx *ctx, uint64_t *ns)
{
    Ctx *c = Ctx::of(ctx);
    if (!c || !ns) return PRRTC_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    *ns = c->last_kernel_ns;
    return PRRTC_OK;
}

const char *prrtc_last_error(const prrtc_ctx *ctx)
{
    const Ctx *c = reinterpret_cast<const Ctx *>(ctx);
    return c ? c->last_error.c_str() : "";
}

uint64_t prrtc_launch_count(const prrtc_ctx *ctx)
{
    const Ctx *c = reinterpret_cast<const Ctx *>(ctx);
    return c ? c->launches : 0;
}

prrtc_status prrtc_set_planning_margin(prrtc_ctx *ctx, float pad)
{
    Ctx *c = Ctx::of(ctx);
    if (!c || !(pad >= 0.0f) || pad > 0.1f) return PRRTC_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    c->plan_pad = pad;
    return PRRTC_OK;
}

prrtc_status prrtc_set_time_budget(prrtc_ctx *ctx, uint64_t ns)
{
    Ctx *c = Ctx::of(ctx);
    if (!c) return PRRTC_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    c->budget_ns = ns;
    return PRRTC_OK;
}

int prrtc_robot_dof(prrtc_robot robot)
{
    const RobotOps *o = robot_ops(robot);
    return o ? o->dof : -1;
}

int prrtc_robot_num_spheres(prrtc_robot robot)
{
    const RobotOps *o = robot_ops(robot);
    return o ? o->num_spheres : -1;
}

prrtc_status prrtc_robot_limits(prrtc_robot robot, float *scale, float *offset)
{
    const Limits *l = robot_limits(robot);
    if (!l || !scale || !offset) return PRRTC_EINVAL;
    std::memcpy(scale, l->scale, sizeof(float) * l->dof);
    std::memcpy(offset, l->offset, sizeof(float) * l->dof);
    return PRRTC_OK;
}

prrtc_status prrtc_env_upload(prrtc_ctx *ctx, const prrtc_env_desc *d, prrtc_env **out)
{
    Ctx *c = Ctx::of(ctx);
    if (!c || !d || !out) return PRRTC_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    *out = nullptr;
    auto bad = [](const float *p, uint32_t n) { return n > 0 && !p; };
    if (bad(d->spheres, d->num_spheres) || bad(d->capsules, d->num_capsules) ||
        bad(d->z_aligned_capsules, d->num_z_aligned_capsules) || bad(d->cuboids, d->num_cuboids) ||
        bad(d->z_aligned_cuboids, d->num_z_aligned_cuboids))
        return c->fail(PRRTC_EINVAL, "env_upload: null array with a non-zero count");
    Env *e = new Env();
    e->counts = EnvCounts{(int)d->num_spheres, (int)d->num_capsules, (int)d->num_z_aligned_capsules,
                          (int)d->num_cuboids, (int)d->num_z_aligned_cuboids};
    const int64_t rec = (int64_t)d->num_spheres + 2ll * d->num_capsules + 2ll * d->num_z_aligned_capsules +
                        4ll * d->num_cuboids + 4ll * d->num_z_aligned_cuboids;
    if (rec * 4 > PRRTC_MAX_ENV_FLOATS) {
        delete e;
        return c->fail(PRRTC_EINVAL, "env_upload: %lld packed floats exceed PRRTC_MAX_ENV_FLOATS (%d)",
                       (long long)(rec * 4), PRRTC_MAX_ENV_FLOATS);
    }
    pack_env(*d, e->host);
    e->num_cylinders = d->num_cylinders;
    if (!e->host.empty()) {
        cudaSetDevice(c->device);
        if (cudaMalloc(&e->dev, e->host.size() * sizeof(float4)) != cudaSuccess) {
            cudaGetLastError();
            delete e;
            return c->fail(PRRTC_ENOMEM, "env_upload: cudaMalloc failed");
        }
        prrtc_status s = c->cuda(cudaMemcpy(e->dev, e->host.data(), e->host.size() * sizeof(float4), cudaMemcpyHostToDevice),
                                 "env_upload copy");
        if (s) {
            cudaFree(e->dev);
            delete e;
            return s;
        }
    }
    *out = reinterpret_cast<prrtc_env *>(e);
    return PRRTC_OK;
}

prrtc_status prrtc_env_free(prrtc_ctx *ctx, prrtc_env *env)
{
    Ctx *c = Ctx::of(ctx);
    Env *e = reinterpret_cast<Env *>(env);
    if (!c || !e) return PRRTC_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (e->dev) cudaFree(e->dev);
    delete e;
    return PRRTC_OK;
}

prrtc_status prrtc_validate_configs(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_env *env, const float *q,
                                    int64_t n, uint8_t *out_free)
{
    Ctx *c = Ctx::of(ctx);
    const RobotOps *ops = robot_ops(robot);
    const Env *e = reinterpret_cast<const Env *>(env);
    if (!c || !ops || !e || n < 0 || (n > 0 && (!q || !out_free))) return c ? c->fail(PRRTC_EINVAL, "validate_configs: bad argument") : PRRTC_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    if (n == 0) return PRRTC_OK;
    cudaSetDevice(c->device);
    void *dq, *dout;
    prrtc_status s;
    if ((s = c->device_view(q, sizeof(float) * ops->dof * n, 0, true, &dq))) return s;
    if ((s = c->device_view(out_free, n, 1, false, &dout))) return s;
    LaunchEnv le{e->dev, e->counts, c->sms, c->work_dev};
    cudaEventRecord(c->kev[0], c->stream);
    if ((s = c->cuda(ops->validate_configs(le, (const float *)dq, n, (uint8_t *)dout, c->stream), "validate_configs launch"))) return s;
    cudaEventRecord(c->kev[1], c->stream);
    c->launches++;
    if (dout != out_free && (s = c->cuda(cudaMemcpyAsync(out_free, dout, n, cudaMemcpyDeviceToHost, c->stream), "copy out"))) return s;
    if ((s = c->cuda(cudaStreamSynchronize(c->stream), "validate_configs"))) return s;
    c->note_kernel_time();
    return PRRTC_OK;
}

prrtc_status prrtc_sample_goals(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_env *env, int sphere,
                                const float *box_lo, const float *box_hi, uint64_t seed, int64_t tries, int max_goals,
                                float *goals, int *num_found)
{
    Ctx *c = Ctx::of(ctx);
    const RobotOps *ops = robot_ops(robot);
    const Env *e = reinterpret_cast<const Env *>(env);
    if (!c) return PRRTC_EINVAL;
    if (!ops || !e || !box_lo || !box_hi || !num_found || tries < 0 || max_goals < 0 || (max_goals > 0 && !goals) ||
        sphere < 0 || sphere >= ops->num_spheres)
        return c->fail(PRRTC_EINVAL, "sample_goals: bad argument");
    if (tries > (int64_t)1 << 30) return c->fail(PRRTC_EINVAL, "sample_goals: at most 2^30 tries per call");
    *num_found = 0;
    if (tries == 0 || max_goals == 0) return PRRTC_OK;
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    GoalQuery gq{};
    gq.seed = seed;
    gq.tries = tries;
    gq.sphere = sphere;
    for (int k = 0; k < 3; k++) {
        gq.lo[k] = box_lo[k];
        gq.hi[k] = box_hi[k];
    }
    prrtc_robot_limits(robot, gq.scale, gq.offset);
    uint8_t *flags = static_cast<uint8_t *>(c->scratch(1, (size_t)tries));
    if (!flags) return c->fail(PRRTC_ENOMEM, "sample_goals: %lld flags", (long long)tries);
    LaunchEnv le{e->dev, e->counts, c->sms, nullptr};
    prrtc_status s;
    if ((s = c->cuda(ops->goal_flags(le, gq, flags, c->stream), "sample_goals launch"))) return s;
    c->launches++;
    std::vector<uint8_t> h((size_t)tries);
    if ((s = c->cuda(cudaMemcpyAsync(h.data(), flags, (size_t)tries, cudaMemcpyDeviceToHost, c->stream), "sample_goals copy")) ||
        (s = c->cuda(cudaStreamSynchronize(c->stream), "sample_goals")))
        return s;
    // the first max_goals accepted candidates, in candidate order (deterministic)
    int found = 0;
    for (int64_t t = 0; t < tries && found < max_goals; t++)
        if (h[(size_t)t]) goal_candidate(seed, t, ops->dof, gq.scale, gq.offset, goals + (size_t)found++ * ops->dof);
    *num_found = found;
    return PRRTC_OK;
}

prrtc_status prrtc_validate_edges(prrtc_ctx *ctx, prrtc_robot robot, const prrtc_env *env, const float *a,
                                  const float *b, int64_t n, int granularity, uint8_t *out_free)
{
    Ctx *c = Ctx::of(ctx);
    const RobotOps *ops = robot_ops(robot);
    const Env *e = reinterpret_cast<const Env *>(env);
    if (!c || !ops || !e || n < 0 || granularity < 1 || granularity > 1024 || (n > 0 && (!a || !b || !out_free)))
        return c ? c->fail(PRRTC_EINVAL, "validate_edges: bad argument") : PRRTC_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    if (n == 0) return PRRTC_OK;
    cudaSetDevice(c->device);
    void *da, *db, *dout;
    prrtc_status s;
    const size_t cb = sizeof(float) * ops->dof * n;
    if ((s = c->device_view(a, cb, 0, true, &da))) return s;
    if ((s = c->device_view(b, cb, 2, true, &db))) return s;
    if ((s = c->device_view(out_free, n, 1, false, &dout))) return s;
    LaunchEnv le{e->dev, e->counts, c->sms, c->work_dev};
    cudaEventRecord(c->kev[0], c->stream);
    if ((s = c->cuda(ops->validate_edges(le, (const float *)da, (const float *)db, n, granularity, (uint8_t *)dout, c->stream),
                     "validate_edges launch")))
        return s;
    cudaEventRecord(c->kev[1], c->stream);
    c->launches++;
    if (dout != out_free && (s = c->cuda(cudaMemcpyAsync(out_free, dout, n, cudaMemcpyDeviceToHost, c->stream), "copy out"))) return s;
    if ((s = c->cuda(cudaStreamSynchronize(c->stream), "validate_edges"))) return s;
    c->note_kernel_time();
    return PRRTC_OK;
}

prrtc_status prrtc_fk_spheres(prrtc_ctx *ctx, prrtc_robot robot, const float *q, int64_t n, float *out)
{
    Ctx *c = Ctx::of(ctx);
    const RobotOps *ops = robot_ops(robot);
    if (!c || !ops || n < 0 || (n > 0 && (!q || !out))) return c ? c->fail(PRRTC_EINVAL, "fk_spheres: bad argument") : PRRTC_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    if (n == 0) return PRRTC_OK;
    cudaSetDevice(c->device);
    void *dq, *dout;
    prrtc_status s;
    const size_t ob = sizeof(float) * 4 * ops->num_spheres * n;
    if ((s = c->device_view(q, sizeof(float) * ops->dof * n, 0, true, &dq))) return s;
    if ((s = c->device_view(out, ob, 1, false, &dout))) return s;
    if ((s = c->cuda(ops->fk_spheres((const float *)dq, n, (float *)dout, c->sms, c->stream), "fk_spheres launch"))) return s;
    c->launches++;
    if (dout != out && (s = c->cuda(cudaMemcpyAsync(out, dout, ob, cudaMemcpyDeviceToHost, c->stream), "copy out"))) return s;
    return c->cuda(cudaStreamSynchronize(c->stream), "fk_spheres");
}

prrtc_status prrtc_work_counters(prrtc_ctx *ctx, uint64_t *flops, uint64_t *configs, int reset)
{
    Ctx *c = Ctx::of(ctx);
    if (!c) return PRRTC_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    unsigned long long h[2];
    prrtc_status s;
    if ((s = c->cuda(cudaMemcpyAsync(h, c->work_dev, sizeof h, cudaMemcpyDeviceToHost, c->stream), "work counters")) ||
        (reset && (s = c->cuda(cudaMemsetAsync(c->work_dev, 0, sizeof h, c->stream), "work counters"))) ||
        (s = c->cuda(cudaStreamSynchronize(c->stream), "work counters")))
        return s;
    if (flops) *flops = h[0];
    if (configs) *configs = h[1];
    return PRRTC_OK;
}

prrtc_status prrtc_measure_fp32_peak(prrtc_ctx *ctx, double *tflops)
{
    Ctx *c = Ctx::of(ctx);
    if (!c || !tflops) return PRRTC_EINVAL;
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    float *sink = (float *)c->scratch(3, 64);
    if (!sink) return c->fail(PRRTC_ENOMEM, "fp32 peak: scratch");
    const int threads = 256, blocks = c->sms * 8, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_peak<<<blocks, threads, 0, c->stream>>>(sink, iters, 0.999999f, 1e-6f);   // warm-up
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < 5; r++) k_fma_peak<<<blocks, threads, 0, c->stream>>>(sink, iters, 0.999999f, 1e-6f);
    cudaEventRecord(e1, c->stream);
    prrtc_status s = c->cuda(cudaEventSynchronize(e1), "fp32 peak");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s) return s;
    c->launches += 6;
    const double flops = 5.0 * blocks * threads * (double)iters * 8 * 2;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return PRRTC_OK;
}

void prrtc_settings_default(prrtc_settings *s)
{
    if (!s) return;
    // pRRTC_settings.hh:3-16
    s->max_samples = 1000000;
    s->max_iters = 1000000;
    s->num_new_configs = 600;
    s->granularity = 64;
    s->range = 0.5f;
    s->balance = 1;
    s->tree_ratio = 0.5f;
    s->dynamic_domain = true;
    s->dd_alpha = 0.0001f;
    s->dd_radius = 4.0f;
    s->dd_min_radius = 1.0f;
}

}  // extern "C"
