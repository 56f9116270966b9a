// Clipping kernels of the mixed-precision engine (64- and 128-vertex warp engines,
// single containers and batches); one translation unit per precision keeps
// each compile small.
#include "vgpu_engine.cuh"

namespace vgpu {

cudaError_t launch_cells_mixed(const CellParams &cp, int pass, int sms, cudaStream_t s, int warps) {
    if (warps > kMaxCtaWarps) warps = kMaxCtaWarps;
    // pass 0: the FP64-free first pass; 1: the full 64-slot engine; 2: 128 slots
    return pass == 0   ? launch_one<VGPU_MIXED, 2, true>(cp, warps, sms, s)
           : pass == 1 ? launch_one<VGPU_MIXED, 2, false>(cp, warps, sms, s)
                       : launch_one<VGPU_MIXED, 4, false>(cp, warps, sms, s);
}

cudaError_t launch_cells_batch_mixed(const BatchParams &bp, int pass, int sms, cudaStream_t s) {
    return pass == 0   ? launch_batch_one<VGPU_MIXED, 2, true>(bp, sms, s)
           : pass == 1 ? launch_batch_one<VGPU_MIXED, 2, false>(bp, sms, s)
                       : launch_batch_one<VGPU_MIXED, 4, false>(bp, sms, s);
}

}  // namespace vgpu
