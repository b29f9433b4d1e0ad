// screen_comp_a_sparse.cu -- seeding and FP32 screen kernels of BallConeCutter and BullConeCutter for spread-out warps.
#include "screen.cuh"

namespace oclg {

bool screen_launch_comp_a_sparse(const DropCtx& h, int sig, unsigned blocks, cudaStream_t stream, int stage) {
    const dim3 tb(SCREEN_WARPS * 32);
    if (sig == SIG_BALLCONE) {
        if (stage == 0) k_drop_seed<2, SIG_BALLCONE><<<blocks, tb, 0, stream>>>(h);
        else k_drop_screen<2, SIG_BALLCONE, true><<<blocks, tb, 0, stream>>>(h);
    } else if (sig == SIG_BULLCONE) {
        if (stage == 0) k_drop_seed<2, SIG_BULLCONE><<<blocks, tb, 0, stream>>>(h);
        else k_drop_screen<2, SIG_BULLCONE, true><<<blocks, tb, 0, stream>>>(h);
    } else {
        return false;
    }
    return true;
}


bool screen_launch_comp_a_b(const BatchView& bv, int sig, unsigned blocks, cudaStream_t stream, int stage) {
    const dim3 tb(SCREEN_WARPS * 32);
    if (sig == SIG_BALLCONE) {
        if (stage == 0) k_drop_seed_b<2, SIG_BALLCONE><<<blocks, tb, 0, stream>>>(bv);
        else k_drop_screen_sparse_b<2, SIG_BALLCONE><<<blocks, tb, 0, stream>>>(bv);
    } else if (sig == SIG_BULLCONE) {
        if (stage == 0) k_drop_seed_b<2, SIG_BULLCONE><<<blocks, tb, 0, stream>>>(bv);
        else k_drop_screen_sparse_b<2, SIG_BULLCONE><<<blocks, tb, 0, stream>>>(bv);
    } else {
        return false;
    }
    return true;
}

}  // namespace oclg
