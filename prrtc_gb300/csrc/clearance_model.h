// A robot's collision model rearranged for the clearance kernels (host
// side): the generated tables of robots/<robot>_model.h reindexed by table
// position, env leaf spheres and self-collision leaf pairs expanded.
#pragma once

#include <vector>

#include "clearance_device.cuh"
#include "prrtc/prrtc.h"
#include "robots/baxter_model.h"
#include "robots/fetch_model.h"
#include "robots/panda_model.h"
#include "robots/sphere_model.h"

namespace prrtc {

struct ClrHostModel {
    int dof = 0;
    std::vector<prrtc_joint_def> joints;
    std::vector<int> parent, leaf_joint;
    std::vector<float4> leaf, pa, pb;
    std::vector<int2> pair_joint;

    // A ClrModel whose pointers are this object's own arrays (host memory).
    ClrModel host_view() const
    {
        return ClrModel{dof, (int)joints.size(), (int)leaf.size(), (int)pa.size(), joints.data(), parent.data(),
                        leaf.data(), leaf_joint.data(), pa.data(), pb.data(), pair_joint.data()};
    }
};

template <int NJ, int NS, int NL, int NP>
inline ClrHostModel make_clr_model(int dof, const prrtc_joint_def (&J)[NJ], const prrtc_sphere_def (&S)[NS],
                                   const short (&L)[NL], const short (&P)[NP][2], int num_pairs)
{
    ClrHostModel h;
    h.dof = dof;
    int pos_of_q[kClrMaxJoints] = {};
    for (int j = 0; j < NJ; j++) pos_of_q[J[j].q] = j;
    auto pos = [&](int q) { return q < 0 ? -1 : pos_of_q[q]; };
    for (int j = 0; j < NJ; j++) {
        h.joints.push_back(J[j]);
        h.parent.push_back(pos(J[j].parent));
    }
    for (int i = 0; i < NL; i++) {
        const prrtc_sphere_def &s = S[L[i]];
        h.leaf.push_back(make_float4(s.x, s.y, s.z, s.r));
        h.leaf_joint.push_back(pos(s.frame));
    }
    for (int i = 0; i < num_pairs; i++) {
        const prrtc_sphere_def &a = S[P[i][0]], &b = S[P[i][1]];
        h.pa.push_back(make_float4(a.x, a.y, a.z, a.r));
        h.pb.push_back(make_float4(b.x, b.y, b.z, b.r));
        h.pair_joint.push_back(make_int2(pos(a.frame), pos(b.frame)));
    }
    return h;
}

#define PRRTC_CLR_MODEL(R) \
    make_clr_model(k##R##Dof, k##R##Joints, k##R##Spheres, k##R##EnvLeaves, k##R##SelfPairs, k##R##NumSelfPairs)

inline const ClrHostModel &clr_host_model(prrtc_robot r)
{
    static const ClrHostModel m[4] = {PRRTC_CLR_MODEL(Sphere), PRRTC_CLR_MODEL(Panda), PRRTC_CLR_MODEL(Fetch),
                                      PRRTC_CLR_MODEL(Baxter)};
    return m[(int)r];
}

}  // namespace prrtc
