// screen_basic.cu -- FP32 screen kernels of the cyl, ball, bull and cone.
#include "screen.cuh"

namespace oclg {

void screen_launch_basic(const DropCtx& h, int kind, unsigned blocks, cudaStream_t stream) {
    const dim3 tb(SCREEN_WARPS * 32);
    switch (kind) {
    case OCL_CUTTER_CONE: k_drop_screen<1, OCL_CUTTER_CONE, false><<<blocks, tb, 0, stream>>>(h); break;
    case OCL_CUTTER_CYL: k_drop_screen<0, OCL_CUTTER_CYL, false><<<blocks, tb, 0, stream>>>(h); break;
    case OCL_CUTTER_BALL: k_drop_screen<0, OCL_CUTTER_BALL, false><<<blocks, tb, 0, stream>>>(h); break;
    default: k_drop_screen<0, OCL_CUTTER_BULL, false><<<blocks, tb, 0, stream>>>(h); break;
    }
}


void screen_launch_basic_dense_b(const BatchView& bv, int kind, unsigned blocks, cudaStream_t stream) {
    const dim3 tb(SCREEN_WARPS * 32);
    switch (kind) {
    case OCL_CUTTER_CONE: k_drop_screen_b<1, OCL_CUTTER_CONE><<<blocks, tb, 0, stream>>>(bv); break;
    case OCL_CUTTER_CYL: k_drop_screen_b<0, OCL_CUTTER_CYL><<<blocks, tb, 0, stream>>>(bv); break;
    case OCL_CUTTER_BALL: k_drop_screen_b<0, OCL_CUTTER_BALL><<<blocks, tb, 0, stream>>>(bv); break;
    default: k_drop_screen_b<0, OCL_CUTTER_BULL><<<blocks, tb, 0, stream>>>(bv); break;
    }
}

}  // namespace oclg
