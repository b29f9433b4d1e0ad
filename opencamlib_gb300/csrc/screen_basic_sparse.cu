// screen_basic_sparse.cu -- seeding and FP32 screen kernels of the cyl, ball, bull and cone for spread-out warps.
#include "screen.cuh"

namespace oclg {

void screen_launch_basic_sparse(const DropCtx& h, int kind, unsigned blocks, cudaStream_t stream, int stage) {
    const dim3 tb(SCREEN_WARPS * 32);
    switch (kind) {
    case OCL_CUTTER_CONE:
        if (stage == 0) k_drop_seed<1, OCL_CUTTER_CONE><<<blocks, tb, 0, stream>>>(h);
        else k_drop_screen<1, OCL_CUTTER_CONE, true><<<blocks, tb, 0, stream>>>(h);
        break;
    case OCL_CUTTER_CYL:
        if (stage == 0) k_drop_seed<0, OCL_CUTTER_CYL><<<blocks, tb, 0, stream>>>(h);
        else k_drop_screen<0, OCL_CUTTER_CYL, true><<<blocks, tb, 0, stream>>>(h);
        break;
    case OCL_CUTTER_BALL:
        if (stage == 0) k_drop_seed<0, OCL_CUTTER_BALL><<<blocks, tb, 0, stream>>>(h);
        else k_drop_screen<0, OCL_CUTTER_BALL, true><<<blocks, tb, 0, stream>>>(h);
        break;
    default:
        if (stage == 0) k_drop_seed<0, OCL_CUTTER_BULL><<<blocks, tb, 0, stream>>>(h);
        else k_drop_screen<0, OCL_CUTTER_BULL, true><<<blocks, tb, 0, stream>>>(h);
        break;
    }
}


void screen_launch_basic_b(const BatchView& bv, int kind, unsigned blocks, cudaStream_t stream, int stage) {
    const dim3 tb(SCREEN_WARPS * 32);
    switch (kind) {
    case OCL_CUTTER_CONE:
        if (stage == 0) k_drop_seed_b<1, OCL_CUTTER_CONE><<<blocks, tb, 0, stream>>>(bv);
        else k_drop_screen_sparse_b<1, OCL_CUTTER_CONE><<<blocks, tb, 0, stream>>>(bv);
        break;
    case OCL_CUTTER_CYL:
        if (stage == 0) k_drop_seed_b<0, OCL_CUTTER_CYL><<<blocks, tb, 0, stream>>>(bv);
        else k_drop_screen_sparse_b<0, OCL_CUTTER_CYL><<<blocks, tb, 0, stream>>>(bv);
        break;
    case OCL_CUTTER_BALL:
        if (stage == 0) k_drop_seed_b<0, OCL_CUTTER_BALL><<<blocks, tb, 0, stream>>>(bv);
        else k_drop_screen_sparse_b<0, OCL_CUTTER_BALL><<<blocks, tb, 0, stream>>>(bv);
        break;
    default:
        if (stage == 0) k_drop_seed_b<0, OCL_CUTTER_BULL><<<blocks, tb, 0, stream>>>(bv);
        else k_drop_screen_sparse_b<0, OCL_CUTTER_BULL><<<blocks, tb, 0, stream>>>(bv);
        break;
    }
}

}  // namespace oclg
