// Operand-tile layout of the tensor-core Hankel transform (hankel_tc.cu), shared with the kernels
// that write its A operand directly (k_hankel_tc_prep, and the spectral update k_spec_point, which
// forms the next inverse transform's operand from the stage estimate it has just computed).
//
// A tile of 64 frequencies becomes 128 MMA rows (row 2j = Re A(w0 + j, .), row 2j + 1 = Im A(w0 + j,
// .)) by 64 reduction elements, bf16, in the K-major no-swizzle core-matrix layout: 8x8 core matrices
// of 128 contiguous bytes (8 rows of 16 bytes), core matrices adjacent in K 128 bytes apart, adjacent
// in M 1024 bytes apart.  Each FP32 value x is stored as x_hi = bf16(x) in the first 16 KB of the
// 32 KB tile pair and x_lo = bf16(x - x_hi) in the second.  Tiles of azimuthal mode m are ordered
// [m][w / 64][k / 64].
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"
#include "uppe_internal.h"

#define TC_ROWS 128  // MMA rows per tile (64 frequencies x re/im)
#define TC_W 64      // frequencies per tile
#define TC_N 128     // output columns per tile
#define TC_K 64      // reduction elements per shared tile (four K=16 MMAs)
#define TC_TILE_BYTES (TC_ROWS * TC_K * 2)  // 16 KB per bf16 operand tile

// Byte offset of element (row, k) of a 128 x 64 bf16 tile.
__device__ __forceinline__ uint32_t core_off(int row, int k) {
    return (uint32_t)((row >> 3) * 1024 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
    hi = __float2bfloat16_rn(x);
    lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

// Element (w, k) of azimuthal mode m of the A operand: v split into its four bf16 parts.
__device__ __forceinline__ void tc_store_split(uint8_t* __restrict__ Atc, int nwt, int nkt, int m, int w, int k,
                                               float2 v) {
    __nv_bfloat16 rh, rl, ih, il;
    split_bf16(v.x, rh, rl);
    split_bf16(v.y, ih, il);
    const unsigned uw = (unsigned)w, uk = (unsigned)k;  // both >= 0: shifts and masks
    const int wl = (int)(uw % TC_W), kk = (int)(uk % TC_K);
    uint8_t* tile = Atc + (((size_t)m * nwt + uw / TC_W) * nkt + uk / TC_K) * (size_t)(2 * TC_TILE_BYTES);
    const uint32_t ore = core_off(2 * wl, kk), oim = core_off(2 * wl + 1, kk);
    *reinterpret_cast<__nv_bfloat16*>(tile + ore) = rh;
    *reinterpret_cast<__nv_bfloat16*>(tile + oim) = ih;
    *reinterpret_cast<__nv_bfloat16*>(tile + TC_TILE_BYTES + ore) = rl;
    *reinterpret_cast<__nv_bfloat16*>(tile + TC_TILE_BYTES + oim) = il;
}

// The next inverse transform's operand, written by the spectral update of the stage before it:
// Atc NULL when not asked.
struct TcNext {
    uint8_t* Atc;
    int nwt, nkt, Nk;  // tile counts of the inverse transform (reduction over the Nk radial modes)
    StepArgs z;        // the next evaluation's z
};
