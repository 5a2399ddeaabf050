// Drop-in definition of pRRTC's planner entry point on top of the C ABI.
//
// pRRTC declares (src/planning/Planners.hh:75-78)
//
//     namespace pRRTC {
//     template <typename Robot>
//     PlannerResult<Robot> solve(typename Robot::Configuration &start,
//                                std::vector<typename Robot::Configuration> &goals,
//                                ppln::collision::Environment<float> &environment,
//                                pRRTC_settings &settings);
//     }
//
// and defines it in src/planning/pRRTC.cu:607-766.  A program built against
// pRRTC's headers switches to this library by compiling, instead of
// pRRTC.cu, one translation unit that includes pRRTC's Planners.hh and then
// this header, and linking libprrtc_gb300.so:
//
//     #include "src/planning/Planners.hh"
//     #include "prrtc/compat.hh"
//     PRRTC_GB300_INSTANTIATE_SOLVE()     // Sphere, Panda, Fetch, Baxter
//
// Behaviour kept: the signature, PlannerResult fields, goal-first path order,
// solved = false on exhaustion of max_iters / max_samples.  Changed: no
// cudaDeviceReset() at the end (pRRTC.cu:764), device state is kept in one
// process-wide context on device 0, and CUDA errors throw std::runtime_error
// instead of exit() (utils.cuh:249-255).
#pragma once

#include <array>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "prrtc/prrtc.h"

namespace prrtc_gb300 {

inline prrtc_ctx *shared_context()
{
    static std::once_flag once;
    static prrtc_ctx *ctx = nullptr;
    std::call_once(once, [] {
        if (prrtc_create(&ctx, 0) != PRRTC_OK) throw std::runtime_error("prrtc_create failed");
    });
    return ctx;
}

template <class Robot>
inline prrtc_robot robot_of()
{
    const std::string n = Robot::name;   // Robots.hh: "sphere", "panda", "fetch", "baxter"
    if (n == "sphere") return PRRTC_ROBOT_SPHERE;
    if (n == "panda") return PRRTC_ROBOT_PANDA;
    if (n == "fetch") return PRRTC_ROBOT_FETCH;
    if (n == "baxter") return PRRTC_ROBOT_BAXTER;
    throw std::runtime_error("unsupported robot " + n);
}

// Flat obstacle arrays read field by field from the reference's shape structs
// (shapes.hh), so the std::string header of each shape never matters.
template <class Env>
struct FlatEnv {
    std::vector<float> s, c, zc, cy, cb, zcb;
    prrtc_env_desc desc{};

    explicit FlatEnv(const Env &e)
    {
        for (unsigned i = 0; i < e.num_spheres; i++) {
            const auto &o = e.spheres[i];
            s.insert(s.end(), {o.x, o.y, o.z, o.r});
        }
        auto caps = [](std::vector<float> &out, const auto *a, unsigned n) {
            for (unsigned i = 0; i < n; i++) {
                const auto &o = a[i];
                out.insert(out.end(), {o.x1, o.y1, o.z1, o.xv, o.yv, o.zv, o.r, o.rdv});
            }
        };
        caps(c, e.capsules, e.num_capsules);
        caps(zc, e.z_aligned_capsules, e.num_z_aligned_capsules);
        caps(cy, e.cylinders, e.num_cylinders);
        auto cubs = [](std::vector<float> &out, const auto *a, unsigned n) {
            for (unsigned i = 0; i < n; i++) {
                const auto &o = a[i];
                out.insert(out.end(), {o.x, o.y, o.z, o.axis_1_x, o.axis_1_y, o.axis_1_z, o.axis_2_x, o.axis_2_y,
                                       o.axis_2_z, o.axis_3_x, o.axis_3_y, o.axis_3_z, o.axis_1_r, o.axis_2_r,
                                       o.axis_3_r});
            }
        };
        cubs(cb, e.cuboids, e.num_cuboids);
        cubs(zcb, e.z_aligned_cuboids, e.num_z_aligned_cuboids);
        desc = prrtc_env_desc{s.data(), (uint32_t)(s.size() / 4), c.data(), (uint32_t)(c.size() / 8),
                              zc.data(), (uint32_t)(zc.size() / 8), cy.data(), (uint32_t)(cy.size() / 8),
                              cb.data(), (uint32_t)(cb.size() / 15), zcb.data(), (uint32_t)(zcb.size() / 15)};
    }
};

template <class Settings>
inline prrtc_settings settings_of(const Settings &s)
{
    prrtc_settings o;
    o.max_samples = s.max_samples;
    o.max_iters = s.max_iters;
    o.num_new_configs = s.num_new_configs;
    o.granularity = s.granularity;
    o.range = s.range;
    o.balance = s.balance;
    o.tree_ratio = s.tree_ratio;
    o.dynamic_domain = s.dynamic_domain;
    o.dd_alpha = s.dd_alpha;
    o.dd_radius = s.dd_radius;
    o.dd_min_radius = s.dd_min_radius;
    return o;
}

template <class Robot, class Result, class Env, class Settings>
Result solve_impl(typename Robot::Configuration &start, std::vector<typename Robot::Configuration> &goals,
                  Env &environment, Settings &settings)
{
    constexpr int D = Robot::dimension;
    prrtc_ctx *ctx = shared_context();
    FlatEnv<Env> flat(environment);
    prrtc_env *env = nullptr;
    if (prrtc_env_upload(ctx, &flat.desc, &env) != PRRTC_OK) throw std::runtime_error(prrtc_last_error(ctx));
    std::vector<float> g;
    for (auto &q : goals) g.insert(g.end(), q.begin(), q.end());
    const prrtc_settings S = settings_of(settings);
    std::vector<float> path((size_t)(S.max_samples < 65536 ? S.max_samples : 65536) * 2 * D + 2 * D);
    prrtc_result r{};
    r.path = path.data();
    r.path_capacity = (int)(path.size() / D);
    const prrtc_status st = prrtc_solve(ctx, robot_of<Robot>(), start.data(), g.data(), (int)goals.size(), env, &S, &r);
    prrtc_env_free(ctx, env);
    if (st != PRRTC_OK && st != PRRTC_ETIMEDOUT) throw std::runtime_error(prrtc_last_error(ctx));
    Result res;
    res.solved = r.solved != 0;
    res.start_tree_size = r.start_tree_size;
    res.goal_tree_size = r.goal_tree_size;
    res.path_length = r.path_length;
    res.iters = r.iters;
    res.cost = r.cost;
    res.wall_ns = r.wall_ns;
    res.kernel_ns = r.kernel_ns;
    res.copy_ns = r.copy_ns;
    for (int i = 0; i < r.path_rows; i++) {
        typename Robot::Configuration q;
        std::memcpy(q.data(), path.data() + (size_t)i * D, sizeof(float) * D);
        res.path.emplace_back(q);
    }
    return res;
}

}  // namespace prrtc_gb300

// The reference's declaration is a template; this defines it for every Robot.
namespace pRRTC {
template <typename Robot>
PlannerResult<Robot> solve(typename Robot::Configuration &start, std::vector<typename Robot::Configuration> &goals,
                           ppln::collision::Environment<float> &environment, pRRTC_settings &settings)
{
    return prrtc_gb300::solve_impl<Robot, PlannerResult<Robot>>(start, goals, environment, settings);
}
}  // namespace pRRTC

// Explicit instantiations matching pRRTC.cu:768-771.
#define PRRTC_GB300_INSTANTIATE_SOLVE()                                                                        \
    template PlannerResult<ppln::robots::Sphere> pRRTC::solve<ppln::robots::Sphere>(                          \
        std::array<float, 3> &, std::vector<std::array<float, 3>> &, ppln::collision::Environment<float> &,    \
        pRRTC_settings &);                                                                                     \
    template PlannerResult<ppln::robots::Panda> pRRTC::solve<ppln::robots::Panda>(                            \
        std::array<float, 7> &, std::vector<std::array<float, 7>> &, ppln::collision::Environment<float> &,    \
        pRRTC_settings &);                                                                                     \
    template PlannerResult<ppln::robots::Fetch> pRRTC::solve<ppln::robots::Fetch>(                            \
        std::array<float, 8> &, std::vector<std::array<float, 8>> &, ppln::collision::Environment<float> &,    \
        pRRTC_settings &);                                                                                     \
    template PlannerResult<ppln::robots::Baxter> pRRTC::solve<ppln::robots::Baxter>(                          \
        std::array<float, 14> &, std::vector<std::array<float, 14>> &, ppln::collision::Environment<float> &,  \
        pRRTC_settings &);
