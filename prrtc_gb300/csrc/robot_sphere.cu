// Kernels for pRRTC's sphere robot (model: robots/sphere_fkcc.cuh).
#include "device_common.cuh"
#include "robots/sphere_fkcc.cuh"
#include "robot_kernels.cuh"

PRRTC_GEN_ADAPTER(GenSphere, gen_sphere)

namespace prrtc {
RobotOps robot_ops_sphere() { return RobotKernels<GenSphere>::ops(GenSphere::kDof); }
}  // namespace prrtc
