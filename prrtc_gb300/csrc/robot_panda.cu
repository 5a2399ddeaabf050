// Kernels for pRRTC's panda robot (model: robots/panda_fkcc.cuh).
#include "device_common.cuh"
#include "robots/panda_fkcc.cuh"
#include "robot_kernels.cuh"

PRRTC_GEN_ADAPTER(GenPanda, gen_panda)

namespace prrtc {
RobotOps robot_ops_panda() { return RobotKernels<GenPanda>::ops(GenPanda::kDof); }
}  // namespace prrtc
