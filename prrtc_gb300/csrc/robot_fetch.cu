// Kernels for pRRTC's fetch robot (model: robots/fetch_fkcc.cuh).
#include "device_common.cuh"
#include "robots/fetch_fkcc.cuh"
#include "robot_kernels.cuh"

PRRTC_GEN_ADAPTER(GenFetch, gen_fetch)

namespace prrtc {
// Fetch's stand-alone checker runs faster unconstrained (104 registers;
// a minimum of 0 blocks per SM sets no register target)
template <>
struct ValidateLaunch<GenFetch> {
    static constexpr int kMaxThreads = 256, kMinBlocks = 0;
};
}  // namespace prrtc

namespace prrtc {
RobotOps robot_ops_fetch() { return RobotKernels<GenFetch>::ops(GenFetch::kDof); }
}  // namespace prrtc
