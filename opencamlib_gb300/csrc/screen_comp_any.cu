// screen_comp_any.cu -- FP32 screen kernels of any other composite cutter (dense and spread-out warps).
#include "screen.cuh"

namespace oclg {

void screen_launch_comp_any(const DropCtx& h, unsigned blocks, cudaStream_t stream) {
    k_drop_screen<2, -1, false><<<blocks, dim3(SCREEN_WARPS * 32), 0, stream>>>(h);
}

void screen_launch_comp_any_sparse(const DropCtx& h, unsigned blocks, cudaStream_t stream, int stage) {
    if (stage == 0) k_drop_seed<2, -1><<<blocks, dim3(SCREEN_WARPS * 32), 0, stream>>>(h);
    else k_drop_screen<2, -1, true><<<blocks, dim3(SCREEN_WARPS * 32), 0, stream>>>(h);
}

void screen_launch_comp_any_dense_b(const BatchView& bv, unsigned blocks, cudaStream_t stream) {
    k_drop_screen_b<2, -1><<<blocks, dim3(SCREEN_WARPS * 32), 0, stream>>>(bv);
}

void screen_launch_comp_any_b(const BatchView& bv, unsigned blocks, cudaStream_t stream, int stage) {
    if (stage == 0) k_drop_seed_b<2, -1><<<blocks, dim3(SCREEN_WARPS * 32), 0, stream>>>(bv);
    else k_drop_screen_sparse_b<2, -1><<<blocks, dim3(SCREEN_WARPS * 32), 0, stream>>>(bv);
}

}  // namespace oclg
