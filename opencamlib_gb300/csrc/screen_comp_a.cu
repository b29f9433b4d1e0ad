// screen_comp_a.cu -- FP32 screen kernels of BallConeCutter and BullConeCutter.
#include "screen.cuh"

namespace oclg {

bool screen_launch_comp_a(const DropCtx& h, int sig, unsigned blocks, cudaStream_t stream) {
    const dim3 tb(SCREEN_WARPS * 32);
    if (sig == SIG_BALLCONE) k_drop_screen<2, SIG_BALLCONE, false><<<blocks, tb, 0, stream>>>(h);
    else if (sig == SIG_BULLCONE) k_drop_screen<2, SIG_BULLCONE, false><<<blocks, tb, 0, stream>>>(h);
    else return false;
    return true;
}


bool screen_launch_comp_a_dense_b(const BatchView& bv, int sig, unsigned blocks, cudaStream_t stream) {
    const dim3 tb(SCREEN_WARPS * 32);
    if (sig == SIG_BALLCONE) k_drop_screen_b<2, SIG_BALLCONE><<<blocks, tb, 0, stream>>>(bv);
    else if (sig == SIG_BULLCONE) k_drop_screen_b<2, SIG_BULLCONE><<<blocks, tb, 0, stream>>>(bv);
    else return false;
    return true;
}

}  // namespace oclg
