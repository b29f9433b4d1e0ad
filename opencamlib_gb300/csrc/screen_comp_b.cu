// screen_comp_b.cu -- FP32 screen kernels of CylConeCutter and ConeConeCutter.
#include "screen.cuh"

namespace oclg {

bool screen_launch_comp_b(const DropCtx& h, int sig, unsigned blocks, cudaStream_t stream) {
    const dim3 tb(SCREEN_WARPS * 32);
    if (sig == SIG_CYLCONE) k_drop_screen<2, SIG_CYLCONE, false><<<blocks, tb, 0, stream>>>(h);
    else if (sig == SIG_CONECONE) k_drop_screen<2, SIG_CONECONE, false><<<blocks, tb, 0, stream>>>(h);
    else return false;
    return true;
}


bool screen_launch_comp_b_dense_b(const BatchView& bv, int sig, unsigned blocks, cudaStream_t stream) {
    const dim3 tb(SCREEN_WARPS * 32);
    if (sig == SIG_CYLCONE) k_drop_screen_b<2, SIG_CYLCONE><<<blocks, tb, 0, stream>>>(bv);
    else if (sig == SIG_CONECONE) k_drop_screen_b<2, SIG_CONECONE><<<blocks, tb, 0, stream>>>(bv);
    else return false;
    return true;
}

}  // namespace oclg
