// screen_comp_any.cu -- FP32 screen kernel of any other composite cutter.
#include "screen.cuh"

namespace oclg {

void screen_launch_comp_any(const DropCtx& h, unsigned blocks, cudaStream_t stream) {
    k_drop_screen<2, -1><<<blocks, dim3(SCREEN_WARPS * 32), 0, stream>>>(h);
}

}  // namespace oclg
