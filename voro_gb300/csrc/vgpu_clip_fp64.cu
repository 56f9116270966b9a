// Clipping kernels of the plain FP64 engine (64- and 128-vertex warp engines,
// single containers and batches); one translation unit per precision keeps
// each compile small.
#include "vgpu_engine.cuh"

namespace vgpu {

cudaError_t launch_cells_fp64(const CellParams &cp, int big, int sms, cudaStream_t s, int warps) {
    if (warps > kMaxCtaWarps) warps = kMaxCtaWarps;
    return big ? launch_one<VGPU_FP64, 4>(cp, warps, sms, s) : launch_one<VGPU_FP64, 2>(cp, warps, sms, s);
}

cudaError_t launch_cells_batch_fp64(const BatchParams &bp, int big, int sms, cudaStream_t s) {
    return big ? launch_batch_one<VGPU_FP64, 4>(bp, sms, s) : launch_batch_one<VGPU_FP64, 2>(bp, sms, s);
}

}  // namespace vgpu
