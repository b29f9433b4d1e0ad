// drop_util.cuh -- warp helpers and grid queries shared by the drop kernels.
#pragma once
#include "drop.cuh"

namespace oclg {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float warp_min(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_mind(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_maxd(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// k-th element of the centre-out sequence over [lo, hi] starting at c.
__device__ __forceinline__ int centre_out(int k, int c, int lo, int hi) {
    // sequence c, c+1, c-1, c+2, c-2, ... skipping values outside [lo, hi]
    int up = hi - c, dn = c - lo;
    int m = min(up, dn);
    if (k <= 2 * m) {
        if (k == 0) return c;
        int s = (k + 1) / 2;
        return (k & 1) ? c + s : c - s;
    }
    int rest = k - 2 * m;
    return (up > dn) ? c + m + rest : c - m - rest;
}

// Query rectangle of a warp at grid level L in cell coordinates, widened by
// one cell to the left and below (a triangle's home cell is its min corner's
// and its extent is at most one cell); returns false if empty.
__device__ __forceinline__ bool warp_rect(const GridP& g, int L, double xmin, double xmax, double ymin, double ymax,
                                          double reach, int& c0, int& c1, int& r0, int& r1) {
    const double inv = g.inv_cs[L];
    double a0 = floor((xmin - reach - g.x0) * inv) - 1.0, a1 = floor((xmax + reach - g.x0) * inv);
    double b0 = floor((ymin - reach - g.y0) * inv) - 1.0, b1 = floor((ymax + reach - g.y0) * inv);
    if (a1 < 0 || b1 < 0 || a0 > g.ncol[L] - 1 || b0 > g.nrow[L] - 1) return false;
    c0 = (int)fmax(a0, 0.0);
    c1 = (int)fmin(a1, (double)(g.ncol[L] - 1));
    r0 = (int)fmax(b0, 0.0);
    r1 = (int)fmin(b1, (double)(g.nrow[L] - 1));
    return true;
}

// ---------------------------------------------------------------------------
// Batch tiles (BatchView): one persistent block takes (job, block) tiles in
// turn; the job's context lives in shared memory while the block works on it.
// ---------------------------------------------------------------------------
struct TileState {
    uint2 tile;    // the block's current tile
    uint32_t job;  // job whose context is in shared memory (~0u: none yet)
};
static_assert(sizeof(DropCtx) % 8 == 0, "DropCtx is copied in 8-byte words");

__device__ __forceinline__ void batch_copy_ctx(const DropCtx* __restrict__ src, DropCtx& dst) {
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(&dst);
    for (int k = threadIdx.x; k < (int)(sizeof(DropCtx) / 8); k += blockDim.x) d[k] = s[k];
}

// Next tile of a persistent block; every thread of the block calls it.
// Returns 0 when the launch's tiles are used up, 1 for a tile of the job
// already in `ctx`, 2 for a tile of another job (its context copied in).
// `ts.job` must be set to ~0u by one thread before the first call.
__device__ __forceinline__ int batch_next_tile(const BatchView& bv, TileState& ts, DropCtx& ctx, uint2& tile) {
    __syncthreads();  // the block is done with the previous tile
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(bv.next, 1u);
        ts.tile = t < bv.ntiles ? bv.tiles[t] : make_uint2(0xFFFFFFFFu, 0u);
    }
    __syncthreads();
    tile = ts.tile;
    if (tile.x == 0xFFFFFFFFu) return 0;
    if (tile.x == ts.job) return 1;
    batch_copy_ctx(bv.ctxs + tile.x, ctx);
    __syncthreads();
    if (threadIdx.x == 0) ts.job = tile.x;  // read again only after the next call's first barrier
    return 2;
}

__device__ __forceinline__ float hlb_at(const float* hlb, float d, float inv_step) {
    int k = (int)(fmaxf(d, 0.0f) * inv_step);
    k = min(k, HLB_N - 1);
    return hlb[k];
}


}  // namespace oclg
