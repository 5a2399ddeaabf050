// Kernels for pRRTC's baxter robot (model: robots/baxter_fkcc.cuh).
#include "device_common.cuh"
#include "robots/baxter_fkcc.cuh"
#include "robot_kernels.cuh"

PRRTC_GEN_ADAPTER(GenBaxter, gen_baxter)

namespace prrtc {
RobotOps robot_ops_baxter() { return RobotKernels<GenBaxter>::ops(GenBaxter::kDof); }
}  // namespace prrtc
