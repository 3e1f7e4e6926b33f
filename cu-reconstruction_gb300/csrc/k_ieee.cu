// Compat mode in IEEE arithmetic (the CPU oracle's operations) and the fixed
// mode.  Compiled without fast math; every floating-point operation on the
// data path is an explicit round-to-nearest intrinsic.
#define GBT_ARITH_NS ieeearith
#include "gbt_kernels.cuh"

namespace gbt {

using namespace ieeearith;

cudaError_t launch_integrate_compat_ieee(const IntegrateArgs& a, int brick, int grid, cudaStream_t s) {
    return launch_integrate_mode<kCompat>(a, brick, grid, s);
}

cudaError_t launch_integrate_fixed(const IntegrateArgs& a, int brick, int grid, cudaStream_t s) {
    return launch_integrate_mode<kFixed>(a, brick, grid, s);
}

cudaError_t launch_batch_compat_ieee(const BatchArgs& a, int brick, int grid, cudaStream_t s) {
    return launch_batch_mode<kCompat>(a, brick, grid, s);
}

cudaError_t launch_batch_fixed(const BatchArgs& a, int brick, int grid, cudaStream_t s) {
    return launch_batch_mode<kFixed>(a, brick, grid, s);
}

cudaError_t launch_mc_compat_ieee(const McArgs& a, cudaStream_t s) { return launch_mc_mode<kCompat>(a, s); }

cudaError_t launch_mc_fixed(const McArgs& a, cudaStream_t s) { return launch_mc_mode<kFixed>(a, s); }

}  // namespace gbt
