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

cudaError_t launch_stream_compat_ieee(const IntegrateArgs& a, const VolumeMaps& m, int grid, cudaStream_t s) {
    return launch_stream_mode<kCompat>(a, m, grid, s);
}

cudaError_t launch_stream_fixed(const IntegrateArgs& a, const VolumeMaps& m, int grid, cudaStream_t s) {
    return launch_stream_mode<kFixed>(a, m, grid, s);
}

cudaError_t launch_batch_compat_ieee(const BatchArgs& a, int brick, int grid, cudaStream_t s) {
    return launch_batch_mode<kCompat>(a, brick, grid, s);
}

cudaError_t launch_batch_fixed(const BatchArgs& a, int brick, int grid, cudaStream_t s) {
    return launch_batch_mode<kFixed>(a, brick, grid, s);
}

int integrate_resident_ctas_compat_ieee(int kind, int brick) { return resident_ctas_mode<kCompat>(kind, brick); }

int integrate_resident_ctas_fixed(int kind, int brick) { return resident_ctas_mode<kFixed>(kind, brick); }

cudaError_t launch_mc_compat_ieee(const McArgs& a, cudaStream_t s) { return launch_mc_mode<kCompat>(a, s); }

cudaError_t launch_mc_fixed(const McArgs& a, cudaStream_t s) { return launch_mc_mode<kFixed>(a, s); }

namespace {
unsigned weld_grid(int64_t n) {
    static const int sms = [] {
        int dev = 0, m = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev);
        return m > 0 ? m : 1;
    }();
    const int64_t want = (n + 255) / 256;
    const int64_t cap = (int64_t)sms * 16;
    return (unsigned)(want < 1 ? 1 : (want < cap ? want : cap));
}
}  // namespace

cudaError_t launch_weld_fixed(const WeldArgs& w, cudaStream_t s) {
    ieeearith::weld_mark_kernel<<<weld_grid(w.mc.ncubes), 256, 0, s>>>(w.mc, w.bits);
    ieeearith::weld_count_kernel<<<(unsigned)w.nblocks, 256, 0, s>>>(w.bits, w.nwords, w.block_sums);
    ieeearith::weld_scan_blocks_kernel<<<1, 1024, 0, s>>>(w.block_sums, w.nblocks, w.nverts);
    ieeearith::weld_offsets_kernel<<<(unsigned)w.nblocks, 256, 0, s>>>(w.bits, w.nwords, w.block_sums, w.word_offset);
    return cudaGetLastError();
}

cudaError_t launch_weld_vertices_fixed(const WeldArgs& w, cudaStream_t s) {
    ieeearith::weld_vertices_kernel<<<weld_grid(w.nwords), 256, 0, s>>>(w);
    return cudaGetLastError();
}

}  // namespace gbt
