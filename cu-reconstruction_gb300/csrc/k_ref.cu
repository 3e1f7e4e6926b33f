// Compat-mode kernels in the reference's arithmetic.  This translation unit
// is compiled with -use_fast_math, the flag the reference's CUDA sources are
// built with (modules/CMakeLists.txt:17-22), so that its divisions and
// multiply-add contractions come out as the reference's do.
#define GBT_REF_ARITH 1
#define GBT_ARITH_NS refarith
#include "gbt_kernels.cuh"

namespace gbt {

cudaError_t launch_integrate_compat_ref(const IntegrateArgs& a, int brick, int grid, cudaStream_t s) {
    return refarith::launch_integrate_mode<refarith::kCompat>(a, brick, grid, s);
}

cudaError_t launch_stream_compat_ref(const IntegrateArgs& a, const VolumeMaps& m, int grid, cudaStream_t s) {
    return refarith::launch_stream_mode<refarith::kCompat>(a, m, grid, s);
}

cudaError_t launch_batch_compat_ref(const BatchArgs& a, int brick, int grid, cudaStream_t s) {
    return refarith::launch_batch_mode<refarith::kCompat>(a, brick, grid, s);
}

int integrate_resident_ctas_compat_ref(int kind, int brick) {
    return refarith::resident_ctas_mode<refarith::kCompat>(kind, brick);
}

cudaError_t launch_mc_compat_ref(const McArgs& a, cudaStream_t s) {
    return refarith::launch_mc_mode<refarith::kCompat>(a, s);
}

}  // namespace gbt
