// Clipping kernels of the plain FP64 engine (64- and 128-vertex warp engines,
// single containers and batches); one translation unit per precision keeps
// each compile small.
#include "vgpu_engine.cuh"

namespace vgpu {

cudaError_t launch_cells_fp64(const CellParams &cp, int pass, int sms, cudaStream_t s, int warps) {
    if (warps > kMaxCtaWarps) warps = kMaxCtaWarps;
    // pass 0: 64 slots; later passes: 128 slots
    return pass ? launch_one<VGPU_FP64, 4, false>(cp, warps, sms, s) : launch_one<VGPU_FP64, 2, false>(cp, warps, sms, s);
}

cudaError_t launch_cells_batch_fp64(const BatchParams &bp, int pass, int sms, cudaStream_t s) {
    return pass ? launch_batch_one<VGPU_FP64, 4, false>(bp, sms, s) : launch_batch_one<VGPU_FP64, 2, false>(bp, sms, s);
}

}  // namespace vgpu
