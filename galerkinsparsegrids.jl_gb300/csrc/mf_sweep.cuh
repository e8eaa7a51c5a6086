// mf_sweep.cuh -- the pencil sweep of the matrix-free form: the stage
// kernel (mf.cu) applies a pencil's 1D operator to a tile gathered into
// shared memory, a row block's stored k x k blocks in table order, each
// entry's hi and lo halves in the two lanes of a paired FMA.
#pragma once
#include <cuda_runtime.h>

namespace sgdg {

// 1-based level of row block rb of a 1D prefix (block 0: level 1; blocks
// 2^(l-2) .. 2^(l-1)-1: level l)
__device__ __forceinline__ int block_level(int rb) { return rb == 0 ? 1 : (32 - __clz(rb)) + 1; }

// A 1D operator table: block CSR over row blocks, each stored block as
// (column block << 12 | distinct block id), distinct blocks as k rows of
// (hi, lo) FP32 pairs padded to RS floats.
struct OpTable {
    const int* rowptr;
    const int* ent;
    const float* val;
};

// The accumulation of one stored block: acc[i][c] += S[i][jj] * x[jj][c] with
// S = hi + lo carried in the two halves of a paired FMA.
template <int K, int CPT>
__device__ __forceinline__ void block_fma(const float* __restrict__ blk, const float (&x)[K][CPT],
                                          float2 (&acc)[K][CPT]) {
    constexpr int RS = ((2 * K + 3) / 4) * 4;
    const float4* sv = reinterpret_cast<const float4*>(blk);
#pragma unroll
    for (int i = 0; i < K; i++) {
        float srow[RS];
#pragma unroll
        for (int v = 0; v < RS / 4; v++) {
            const float4 f = sv[i * (RS / 4) + v];
            srow[4 * v] = f.x;
            srow[4 * v + 1] = f.y;
            srow[4 * v + 2] = f.z;
            srow[4 * v + 3] = f.w;
        }
#pragma unroll
        for (int jj = 0; jj < K; jj++) {
            const float2 s = make_float2(srow[2 * jj], srow[2 * jj + 1]);
#pragma unroll
            for (int c = 0; c < CPT; c++) acc[i][c] = __ffma2_rn(s, make_float2(x[jj][c], x[jj][c]), acc[i][c]);
        }
    }
}

// out[i][c] = sum over the stored blocks p0, p0 + pstep, ... of row block rb
// with column block < nrb of S(rb, cb)[i][jj] * src[cb*K + jj][jq*CPT + c]:
// src is a row-major tile of W columns.
template <int K, int CPT>
__device__ __forceinline__ void sweep(const OpTable& T, const float* __restrict__ src, int W, int nrb, int rb, int jq,
                                      int p0, int pstep, float (&out)[K][CPT]) {
    constexpr int RS = ((2 * K + 3) / 4) * 4;
    float2 acc[K][CPT];
#pragma unroll
    for (int i = 0; i < K; i++)
#pragma unroll
        for (int c = 0; c < CPT; c++) acc[i][c] = make_float2(0.f, 0.f);
    const int pb = T.rowptr[rb], pe = T.rowptr[rb + 1];
    for (int p = pb + p0; p < pe; p += pstep) {
        const int e = T.ent[p];
        const int cb = e >> 12;
        if (cb >= nrb) break;
        float x[K][CPT];
#pragma unroll
        for (int jj = 0; jj < K; jj++) {
            const float* xp = src + (cb * K + jj) * W + jq * CPT;
            if constexpr (CPT == 4) {
                const float4 v = *reinterpret_cast<const float4*>(xp);
                x[jj][0] = v.x;
                x[jj][1] = v.y;
                x[jj][2] = v.z;
                x[jj][3] = v.w;
            } else {
                const float2 v = *reinterpret_cast<const float2*>(xp);
                x[jj][0] = v.x;
                x[jj][1] = v.y;
            }
        }
        block_fma<K, CPT>(T.val + (e & 4095) * (K * RS), x, acc);
    }
#pragma unroll
    for (int i = 0; i < K; i++)
#pragma unroll
        for (int c = 0; c < CPT; c++) out[i][c] = acc[i][c].x + acc[i][c].y;
}

// The shuffle tree that sums a warp-cooperative row's lane partials.
template <int K, int CPT>
__device__ __forceinline__ void warp_sum(float (&o)[K][CPT]) {
#pragma unroll
    for (int i = 0; i < K; i++)
#pragma unroll
        for (int c = 0; c < CPT; c++)
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) o[i][c] += __shfl_xor_sync(0xffffffffu, o[i][c], off);
}

}  // namespace sgdg
