// Test stand-ins for the reference types the drop-in shim binds to, declared
// with the reference's names and fields (src/planning/Planners.hh:11-23,
// src/planning/pRRTC_settings.hh:3-16, src/planning/Robots.hh name/dimension/
// Configuration, src/collision/environment.hh:11-44, src/collision/shapes.hh
// field names).  Used where the reference's own headers are not available;
// tests/test_compat.py also compiles the shim against the real headers.
#pragma once
#include <array>
#include <chrono>
#include <cstddef>
#include <string>
#include <vector>

struct pRRTC_settings {
    int max_samples = 1000000;
    int max_iters = 1000000;
    int num_new_configs = 600;
    int granularity = 64;
    float range = 0.5;
    int balance = 1;
    float tree_ratio = 0.5;
    bool dynamic_domain = true;
    float dd_alpha = 0.0001;
    float dd_radius = 4.0;
    float dd_min_radius = 1.0;
};

namespace ppln::robots {
struct Panda {
    static constexpr auto name = "panda";
    static constexpr auto dimension = 7;
    using Configuration = std::array<float, dimension>;
};
}  // namespace ppln::robots

template <typename Robot>
struct PlannerResult {
    bool solved = false;
    std::vector<typename Robot::Configuration> path;
    int start_tree_size = 0;
    int goal_tree_size = 0;
    int path_length = 0;
    int iters = 0;
    float cost = 0.0;
    std::size_t wall_ns = 0;
    std::size_t kernel_ns = 0;
    std::size_t copy_ns = 0;
};

namespace ppln::collision {
template <typename T> struct Shape { std::string name; T min_distance; };
template <typename T> struct Sphere : Shape<T> { T x, y, z, r; };
template <typename T> struct Cylinder : Shape<T> { T x1, y1, z1, xv, yv, zv, r, rdv; };
template <typename T> using Capsule = Cylinder<T>;
template <typename T> struct Cuboid : Shape<T> {
    T x, y, z, axis_1_x, axis_1_y, axis_1_z, axis_2_x, axis_2_y, axis_2_z, axis_3_x, axis_3_y, axis_3_z, axis_1_r,
        axis_2_r, axis_3_r;
};
template <typename T> struct Environment {
    Sphere<T> *spheres = nullptr; unsigned int num_spheres = 0;
    Capsule<T> *capsules = nullptr; unsigned int num_capsules = 0;
    Capsule<T> *z_aligned_capsules = nullptr; unsigned int num_z_aligned_capsules = 0;
    Cylinder<T> *cylinders = nullptr; unsigned int num_cylinders = 0;
    Cuboid<T> *cuboids = nullptr; unsigned int num_cuboids = 0;
    Cuboid<T> *z_aligned_cuboids = nullptr; unsigned int num_z_aligned_cuboids = 0;
    ~Environment() { delete[] spheres; delete[] capsules; delete[] cuboids; delete[] z_aligned_capsules; delete[] cylinders; delete[] z_aligned_cuboids; }
};
}  // namespace ppln::collision

namespace pRRTC {
template <typename Robot>
PlannerResult<Robot> solve(typename Robot::Configuration &start, std::vector<typename Robot::Configuration> &goals,
                           ppln::collision::Environment<float> &environment, pRRTC_settings &settings);
}
