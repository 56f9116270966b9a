// Clipping kernels of the mixed-precision engine (64- and 128-vertex warp engines,
// single containers and batches); one translation unit per precision keeps
// each compile small.
#include "vgpu_engine.cuh"

namespace vgpu {

cudaError_t launch_cells_mixed(const CellParams &cp, int big, int sms, cudaStream_t s, int warps) {
    if (warps > kMaxCtaWarps) warps = kMaxCtaWarps;
    return big ? launch_one<VGPU_MIXED, 4>(cp, warps, sms, s) : launch_one<VGPU_MIXED, 2>(cp, warps, sms, s);
}

cudaError_t launch_cells_batch_mixed(const BatchParams &bp, int big, int sms, cudaStream_t s) {
    return big ? launch_batch_one<VGPU_MIXED, 4>(bp, sms, s) : launch_batch_one<VGPU_MIXED, 2>(bp, sms, s);
}

}  // namespace vgpu
