// Kernels for pRRTC's fetch robot (model: robots/fetch_fkcc.cuh).
#include "device_common.cuh"
#include "robots/fetch_fkcc.cuh"
#include "robot_kernels.cuh"

PRRTC_GEN_ADAPTER(GenFetch, gen_fetch)

namespace prrtc {
RobotOps robot_ops_fetch() { return RobotKernels<GenFetch>::ops(GenFetch::kDof); }
}  // namespace prrtc
