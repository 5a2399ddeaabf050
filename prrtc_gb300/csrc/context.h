// Host-side context and environment objects behind the opaque C handles.
#pragma once

#include <mutex>
#include <string>
#include <vector>

#include "prrtc_internal.h"

namespace prrtc {

struct Env {
    EnvCounts counts{};
    float4 *dev = nullptr;           // packed records on the device
    std::vector<float4> host;        // the same records on the host
    uint32_t num_cylinders = 0;      // accepted, never checked (as the reference)
};

// Pack a flat obstacle description into float4 records (layout in
// device_common.cuh), handing each record to emit(float4) in order.
template <class Emit>
inline void pack_records(const prrtc_env_desc &d, Emit &&emit)
{
    for (uint32_t i = 0; i < d.num_spheres; i++) {
        const float *s = d.spheres + 4 * i;
        emit(make_float4(s[0], s[1], s[2], s[3]));
    }
    auto caps = [&](const float *p, uint32_t n) {
        for (uint32_t i = 0; i < n; i++) {
            const float *c = p + 8 * i;
            emit(make_float4(c[0], c[1], c[2], c[6]));
            emit(make_float4(c[3], c[4], c[5], c[7]));
        }
    };
    caps(d.capsules, d.num_capsules);
    caps(d.z_aligned_capsules, d.num_z_aligned_capsules);
    auto cubs = [&](const float *p, uint32_t n) {
        for (uint32_t i = 0; i < n; i++) {
            const float *c = p + 15 * i;
            emit(make_float4(c[0], c[1], c[2], c[12]));
            emit(make_float4(c[3], c[4], c[5], c[13]));
            emit(make_float4(c[6], c[7], c[8], c[14]));
            emit(make_float4(c[9], c[10], c[11], 0.0f));
        }
    };
    cubs(d.cuboids, d.num_cuboids);
    cubs(d.z_aligned_cuboids, d.num_z_aligned_cuboids);
}

inline void pack_env(const prrtc_env_desc &d, std::vector<float4> &out)
{
    out.clear();
    pack_records(d, [&](float4 r) { out.push_back(r); });
}

struct PlannerState;    // planner.cu
struct ClearanceState;  // clearance.cu

struct Ctx {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::string last_error;
    uint64_t launches = 0;
    struct Buf {
        void *ptr = nullptr;
        size_t bytes = 0;
    };
    Buf bufs[4];
    PlannerState *planner = nullptr;
    float *bases = nullptr;                 // Halton prime bases per sampling lane [lanes][16]
    int bases_lanes = 0;
    struct Arena *arena = nullptr;          // batched-planner arena kept between batches
    unsigned long long *work_dev = nullptr; // [2] FLOPs, configurations (prrtc_work_counters)
    float plan_pad = 0.0f;                  // prrtc_set_planning_margin
    unsigned long long budget_ns = 0;       // prrtc_set_time_budget
    ClearanceState *clearance = nullptr;    // robot tables for the clearance cost
    cudaEvent_t kev[2] = {nullptr, nullptr};   // around the last checker launch (prrtc_last_kernel_ns)
    uint64_t last_kernel_ns = 0;

    static Ctx *of(prrtc_ctx *c) { return reinterpret_cast<Ctx *>(c); }
    prrtc_status fail(prrtc_status s, const char *fmt, ...);
    prrtc_status cuda(cudaError_t e, const char *what);
    static bool is_device_ptr(const void *p);
    void *scratch(int slot, size_t bytes);
    prrtc_status device_view(const void *p, size_t bytes, int slot, bool in, void **out);
    void release_planner_state();
    // after a synchronised checker launch bracketed by kev: its device time
    void note_kernel_time()
    {
        float ms = 0.0f;
        last_kernel_ns = cudaEventElapsedTime(&ms, kev[0], kev[1]) == cudaSuccess ? (uint64_t)(ms * 1e6) : 0;
        cudaGetLastError();
    }
};

const RobotOps *robot_ops(prrtc_robot r);
prrtc_status ensure_halton_bases(Ctx *c, int lanes);
void release_arena(Ctx *c);
void release_clearance_state(Ctx *c);

struct Limits;
const Limits *robot_limits(prrtc_robot r);

}  // namespace prrtc
