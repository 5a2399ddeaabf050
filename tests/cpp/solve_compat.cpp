// Calls pRRTC::solve<Panda> through the drop-in shim (include/prrtc/compat.hh).
// Reads a query from stdin: ns then ns*4 floats (spheres), nb then nb*15
// floats (cuboids), start[7], goal[7]; prints solved, cost, rows, then the
// path rows (goal first).
#include <cstdio>
#include <iostream>

#ifdef USE_REFERENCE_HEADERS
#include "src/planning/Planners.hh"
#else
#include "standin_types.hh"
#endif
#include "prrtc/compat.hh"

template PlannerResult<ppln::robots::Panda> pRRTC::solve<ppln::robots::Panda>(
    std::array<float, 7> &, std::vector<std::array<float, 7>> &, ppln::collision::Environment<float> &,
    pRRTC_settings &);

int main()
{
    using namespace ppln::collision;
    Environment<float> env{};
    unsigned ns, nb;
    std::cin >> ns;
    env.spheres = new Sphere<float>[ns];
    env.num_spheres = ns;
    for (unsigned i = 0; i < ns; i++) std::cin >> env.spheres[i].x >> env.spheres[i].y >> env.spheres[i].z >> env.spheres[i].r;
    std::cin >> nb;
    env.cuboids = new Cuboid<float>[nb];
    env.num_cuboids = nb;
    for (unsigned i = 0; i < nb; i++) {
        auto &c = env.cuboids[i];
        std::cin >> c.x >> c.y >> c.z >> c.axis_1_x >> c.axis_1_y >> c.axis_1_z >> c.axis_2_x >> c.axis_2_y >> c.axis_2_z >>
            c.axis_3_x >> c.axis_3_y >> c.axis_3_z >> c.axis_1_r >> c.axis_2_r >> c.axis_3_r;
    }
    std::array<float, 7> start, goal;
    for (auto &v : start) std::cin >> v;
    for (auto &v : goal) std::cin >> v;
    std::vector<std::array<float, 7>> goals{goal};
    pRRTC_settings s;
    s.max_samples = 100000;
    s.num_new_configs = 256;
    s.granularity = 32;
    s.range = 1.0f;
    s.balance = 0;
    s.dynamic_domain = false;
    auto res = pRRTC::solve<ppln::robots::Panda>(start, goals, env, s);
    std::printf("%d %.9g %zu\n", res.solved ? 1 : 0, res.cost, res.path.size());
    for (auto &q : res.path) {
        for (float v : q) std::printf("%.9g ", v);
        std::printf("\n");
    }
    return 0;
}
