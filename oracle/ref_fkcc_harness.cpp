// Host-side harness around pRRTC's own collision checker.
//
// Test infrastructure only (the oracle): compiled by oracle/Makefile from the
// reference sources where they lie (src/planning/utils.cuh, which includes
// Robots.hh, collision/environment.hh and collision/shapes.hh), never copied.
// It builds a ppln::collision::Environment<float> from flat obstacle arrays
// and calls ppln::collision::fkcc<Robot> (utils.cuh:326-327) on each config,
// exactly as the reference kernel does per thread (pRRTC.cu:441,529).
//
// Flat layouts (floats per obstacle): sphere 4 (x y z r); capsule 8
// (x1 y1 z1 xv yv zv r rdv); cuboid 15 (x y z, axis1 xyz, axis2 xyz,
// axis3 xyz, r1 r2 r3).  Cylinders are accepted by the reference but never
// read by its checker (utils.cuh:211-242), so the harness does not take them.
#include "src/planning/utils.cuh"

#ifndef REF_ROBOT
#error "define REF_ROBOT (Panda, Fetch, Baxter or Sphere)"
#endif
#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)

using ppln::collision::Environment;

static void fill_env(Environment<float> &env, const float *sph, int ns, const float *cap, int nc,
                     const float *zcap, int nzc, const float *cub, int ncb, const float *zcub, int nzcb)
{
    env.spheres = ns ? new ppln::collision::Sphere<float>[ns] : nullptr;
    env.num_spheres = ns;
    for (int i = 0; i < ns; i++) {
        const float *s = sph + 4 * i;
        env.spheres[i] = ppln::collision::Sphere<float>(s[0], s[1], s[2], s[3]);
    }
    auto caps = [](const float *src, int n) {
        auto *dst = n ? new ppln::collision::Capsule<float>[n] : nullptr;
        for (int i = 0; i < n; i++) {
            const float *c = src + 8 * i;
            dst[i] = ppln::collision::Capsule<float>(c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7]);
        }
        return dst;
    };
    env.capsules = caps(cap, nc);
    env.num_capsules = nc;
    env.z_aligned_capsules = caps(zcap, nzc);
    env.num_z_aligned_capsules = nzc;
    env.cylinders = nullptr;
    env.num_cylinders = 0;
    auto cubs = [](const float *src, int n) {
        auto *dst = n ? new ppln::collision::Cuboid<float>[n] : nullptr;
        for (int i = 0; i < n; i++) {
            const float *c = src + 15 * i;
            dst[i] = ppln::collision::Cuboid<float>(c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], c[8],
                                                    c[9], c[10], c[11], c[12], c[13], c[14]);
        }
        return dst;
    };
    env.cuboids = cubs(cub, ncb);
    env.num_cuboids = ncb;
    env.z_aligned_cuboids = cubs(zcub, nzcb);
    env.num_z_aligned_cuboids = nzcb;
}

// out_free[i] = 1 when config i is collision-free per the reference checker.
extern "C" int CAT(ref_fkcc_, REF_ROBOT)(const float *q, long n, int dim, const float *sph, int ns,
                                          const float *cap, int nc, const float *zcap, int nzc,
                                          const float *cub, int ncb, const float *zcub, int nzcb,
                                          unsigned char *out_free)
{
    using Robot = ppln::robots::REF_ROBOT;
    if (dim != Robot::dimension) return -1;
    Environment<float> env;
    fill_env(env, sph, ns, cap, nc, zcap, nzc, cub, ncb, zcub, nzcb);
    #pragma omp parallel for schedule(static, 1024)
    for (long i = 0; i < n; i++) {
        volatile float cfg[Robot::dimension];
        for (int d = 0; d < Robot::dimension; d++) cfg[d] = q[i * dim + d];
        out_free[i] = ppln::collision::fkcc<Robot>(cfg, &env, 0) ? 1 : 0;
    }
    return 0;
}
