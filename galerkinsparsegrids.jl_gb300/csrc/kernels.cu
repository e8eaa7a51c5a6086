// kernels.cu -- sm_103a kernels of libsgdg.
//
//  * k_csr_spmv / k_csr_rk4: the plain form.  FP64 CSR mat-vec (the closure
//    body *(RHS, x) of src/pdes.jl:63) with VS lanes per row; the RK4 variant
//    fuses the classical stage combination into the row epilogue.
//  * k_mf_pass: the chosen form.  One launch applies D_d for one dimension d
//    to every pencil tile of every solve in a batch, matrix-free: the 1D
//    operator's k x k blocks (FP32, read through the read-only path) are
//    swept over a pencil staged in shared memory, accumulating over
//    dimensions in an FP32 partial-sum vector; the tile that completes an
//    element applies the FP64 RK4 stage update.
#include <cuda_runtime.h>

#include "engine.h"

namespace sgdg {

// ------------------------------------------------------------------ RK4 ----
// Same stage formulas as the FP64 oracle: acc collects k1 + 2k2 + 2k3, the
// stage input is y + c dt k, and y += dt/6 (acc + k4) at stage 4.
__device__ __forceinline__ void rk_stage(int stage, double dt, double k, double& y, double& acc, double& un) {
    switch (stage) {
        case 1: acc = k; un = y + (0.5 * dt) * k; break;
        case 2: acc = acc + 2.0 * k; un = y + (0.5 * dt) * k; break;
        case 3: acc = acc + 2.0 * k; un = y + dt * k; break;
        default: y = y + (dt / 6.0) * (acc + k); un = y; break;
    }
}

// ------------------------------------------------------------ plain form ----
template <int VS>
__device__ __forceinline__ double csr_row(const DevCSR& A, int64_t row, const double* __restrict__ x, int lane) {
    double s = 0.0;
    if (row < A.m) {
        const int64_t b = A.rowptr[row], e = A.rowptr[row + 1];
        for (int64_t p = b + lane; p < e; p += VS) s = fma(__ldg(A.val + p), __ldg(x + __ldg(A.col + p)), s);
    }
#pragma unroll
    for (int o = VS / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

template <int VS>
__global__ void __launch_bounds__(256) k_csr_spmv(DevCSR A, const double* __restrict__ x, double* __restrict__ y) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t row = t / VS;
    const int lane = int(t % VS);
    double s = csr_row<VS>(A, row, x, lane);
    if (row < A.m && lane == 0) y[row] = s;
}

template <int VS>
__global__ void __launch_bounds__(256) k_csr_rk4(DevCSR A, const double* uin, double* y, double* __restrict__ acc,
                                                 double* __restrict__ uout, double dt, int stage) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t row = t / VS;
    const int lane = int(t % VS);
    double k = csr_row<VS>(A, row, uin, lane);
    if (row < A.m && lane == 0) {
        double yy = y[row], aa = stage == 1 ? 0.0 : acc[row], un;
        rk_stage(stage, dt, k, yy, aa, un);
        if (stage == 4)
            y[row] = yy;
        else {
            acc[row] = aa;
            uout[row] = un;
        }
    }
}

// ----------------------------------------------------------- chosen form ----
__device__ __forceinline__ int block_level(int rb) { return rb == 0 ? 1 : (32 - __clz(rb)) + 1; }

struct TileGeom {
    const int64_t* boff;
    const int* colA;
    const int* colB;
    int kD, lp, kd1;
    __device__ __forceinline__ int64_t addr(int rb, int i, int c) const {
        const int l = block_level(rb);
        const int lc = l > 2 ? l - 2 : 0;
        const int cd0 = l >= 2 ? rb - (1 << (l - 2)) : 0;
        return boff[l - 1] + colA[c] + ((int64_t)colB[c] << lc) + (int64_t)kD * ((int64_t)cd0 << lp) +
               (int64_t)i * kd1;
    }
};

// y[rb*K+i][c] = sum over stored blocks (rb, cb < nrb) of S_blk[i][j] * x[cb*K+j][c]
template <int K>
__device__ __forceinline__ void sweep_pair(const MFSolve& s, const float* __restrict__ X, int wc, int nrb, int rb,
                                           int c, float (&out)[K]) {
#pragma unroll
    for (int i = 0; i < K; i++) out[i] = 0.f;
    const int pb = __ldg(s.s_rowptr + rb), pe = __ldg(s.s_rowptr + rb + 1);
    for (int q = pb; q < pe; q++) {
        const int cb = __ldg(s.s_colblk + q);
        if (cb >= nrb) break;
        float xk[K];
#pragma unroll
        for (int j = 0; j < K; j++) xk[j] = X[(cb * K + j) * wc + c];
        constexpr int KK4 = (K * K + 3) / 4;
        float sb[KK4 * 4];
        const float4* sv = reinterpret_cast<const float4*>(s.s_val + (size_t)q * (KK4 * 4));
#pragma unroll
        for (int v = 0; v < KK4; v++) {
            float4 f = __ldg(sv + v);
            sb[4 * v] = f.x;
            sb[4 * v + 1] = f.y;
            sb[4 * v + 2] = f.z;
            sb[4 * v + 3] = f.w;
        }
#pragma unroll
        for (int i = 0; i < K; i++)
#pragma unroll
            for (int j = 0; j < K; j++) out[i] = fmaf(sb[i * K + j], xk[j], out[i]);
    }
}

template <int K, bool WAVE>
__device__ void mf_tile(const MFTile& t, const MFSolve& s, int stage, int in_sel, int rk, float* smem) {
    const int tid = threadIdx.x, nth = blockDim.x;
    const int nrb = 1 << (t.lmax - 1);
    const int m = nrb * K;
    const int wc = t.wc;
    int* colA = reinterpret_cast<int*>(smem);
    int* colB = colA + wc;
    float* X = reinterpret_cast<float*>(colB + wc);
    float* Y = X + m * wc;
    const int kD = s.kD, kd1 = t.kd1;
    for (int c = tid; c < wc; c += nth) {
        const int r = t.r0 + c;
        const int mr = r % t.kDm1, cr = r / t.kDm1;
        const int Pd = 1 << t.lp;
        colA[c] = kD * (cr & (Pd - 1)) + (mr % kd1) + (mr / kd1) * kd1 * K;
        colB[c] = kD * ((cr >> t.lp) << t.lp);
    }
    __syncthreads();
    const TileGeom g{s.blockoff + t.boff, colA, colB, kD, t.lp, kd1};
    const float* __restrict__ uin = s.u[in_sel];
    // stage the pencil chunk; the memory-contiguous index runs fastest
    const int ne = m * wc;
    for (int e = tid; e < ne; e += nth) {
        int c, i, rb;
        if (kd1 == 1) {
            i = e % K;
            const int q = e / K;
            c = q % wc;
            rb = q / wc;
        } else {
            c = e % wc;
            const int q = e / wc;
            i = q % K;
            rb = q / K;
        }
        X[(rb * K + i) * wc + c] = __ldg(uin + g.addr(rb, i, c));
    }
    __syncthreads();
    const int np = nrb * wc;
    if (WAVE) {
        for (int p = tid; p < np; p += nth) {
            const int c = p % wc, rb = p / wc;
            float o[K];
            sweep_pair<K>(s, X, wc, nrb, rb, c, o);
#pragma unroll
            for (int i = 0; i < K; i++) Y[(rb * K + i) * wc + c] = o[i];
        }
        __syncthreads();
    }
    const float coef = s.coef[t.d];
    const bool last = (t.flags & TILE_LAST) != 0, first = (t.flags & TILE_FIRST) != 0;
    for (int p = tid; p < np; p += nth) {
        const int c = p % wc, rb = p / wc;
        float o[K];
        sweep_pair<K>(s, WAVE ? Y : X, wc, nrb, rb, c, o);
#pragma unroll
        for (int i = 0; i < K; i++) {
            const int64_t a = g.addr(rb, i, c);
            const float z = coef * o[i];
            if (!(rk && last)) {
                s.rhs[a] = first ? z : s.rhs[a] + z;
                continue;
            }
            const float kv = first ? z : s.rhs[a] + z;
            float* uout = s.u[in_sel ^ 1];
            if (WAVE) {
                // u' = v (stage input of the velocity field), v' = L u
                const int64_t av = s.N + a;
                double yu = s.y[a], au = s.acc[a], un;
                rk_stage(stage, s.dt, (double)uin[av], yu, au, un);
                if (stage == 4) s.y[a] = yu; else s.acc[a] = au;
                uout[a] = (float)un;
                double yv = s.y[av], av_ = s.acc[av], vn;
                rk_stage(stage, s.dt, (double)kv, yv, av_, vn);
                if (stage == 4) s.y[av] = yv; else s.acc[av] = av_;
                uout[av] = (float)vn;
            } else {
                double yy = s.y[a], aa = s.acc[a], un;
                rk_stage(stage, s.dt, (double)kv, yy, aa, un);
                if (stage == 4) s.y[a] = yy; else s.acc[a] = aa;
                uout[a] = (float)un;
            }
        }
    }
}

__global__ void __launch_bounds__(kMFThreads) k_mf_pass(const MFTile* __restrict__ tiles, int ntiles,
                                                        const MFSolve* __restrict__ solves, int stage, int in_sel,
                                                        int rk) {
    extern __shared__ __align__(16) float smem[];
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
        const MFTile t = tiles[ti];
        const MFSolve s = solves[t.solve];
        if (s.status == 0) {
            switch (s.k * 2 + s.kind) {
                case 2: mf_tile<1, false>(t, s, stage, in_sel, rk, smem); break;
                case 3: mf_tile<1, true>(t, s, stage, in_sel, rk, smem); break;
                case 4: mf_tile<2, false>(t, s, stage, in_sel, rk, smem); break;
                case 5: mf_tile<2, true>(t, s, stage, in_sel, rk, smem); break;
                case 6: mf_tile<3, false>(t, s, stage, in_sel, rk, smem); break;
                case 7: mf_tile<3, true>(t, s, stage, in_sel, rk, smem); break;
                case 8: mf_tile<4, false>(t, s, stage, in_sel, rk, smem); break;
                case 9: mf_tile<4, true>(t, s, stage, in_sel, rk, smem); break;
                case 10: mf_tile<5, false>(t, s, stage, in_sel, rk, smem); break;
                case 11: mf_tile<5, true>(t, s, stage, in_sel, rk, smem); break;
                default: break;
            }
        }
        __syncthreads();
    }
}

__global__ void k_f64_to_f32(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void k_f32_to_f64(const float* __restrict__ a, double* __restrict__ b, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

// stage input of every live solve from its FP64 state: u[0] = fp32(y)
__global__ void k_restage(const MFSolve* __restrict__ solves, int nsolves) {
    const int si = blockIdx.y;
    if (si >= nsolves) return;
    const MFSolve& s = solves[si];
    if (s.status != 0) return;
    const int64_t n = s.kind == MF_KIND_WAVE ? 2 * s.N : s.N;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s.u[0][i] = (float)s.y[i];
}

// ------------------------------------------------------------ launchers ----
cudaError_t launch_restage(const MFSolve* solves, int nsolves, cudaStream_t st) {
    if (nsolves <= 0) return cudaSuccess;
    for (int s0 = 0; s0 < nsolves; s0 += 65535) {
        int cnt = nsolves - s0 < 65535 ? nsolves - s0 : 65535;
        k_restage<<<dim3(64, cnt), 256, 0, st>>>(solves + s0, cnt);
    }
    return cudaGetLastError();
}

static int grid_for(int64_t threads) {
    int64_t b = (threads + 255) / 256;
    return (int)(b > (1LL << 30) ? (1LL << 30) : (b < 1 ? 1 : b));
}

cudaError_t launch_csr_spmv(const DevCSR& A, const double* x, double* y, cudaStream_t st) {
    const int64_t th = A.m * A.vs;
    switch (A.vs) {
        case 1: k_csr_spmv<1><<<grid_for(th), 256, 0, st>>>(A, x, y); break;
        case 2: k_csr_spmv<2><<<grid_for(th), 256, 0, st>>>(A, x, y); break;
        case 4: k_csr_spmv<4><<<grid_for(th), 256, 0, st>>>(A, x, y); break;
        case 8: k_csr_spmv<8><<<grid_for(th), 256, 0, st>>>(A, x, y); break;
        case 16: k_csr_spmv<16><<<grid_for(th), 256, 0, st>>>(A, x, y); break;
        default: k_csr_spmv<32><<<grid_for(th), 256, 0, st>>>(A, x, y); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_csr_rk4(const DevCSR& A, const double* uin, double* y, double* acc, double* uout, double dt,
                           int stage, cudaStream_t st) {
    const int64_t th = A.m * A.vs;
    switch (A.vs) {
        case 1: k_csr_rk4<1><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, stage); break;
        case 2: k_csr_rk4<2><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, stage); break;
        case 4: k_csr_rk4<4><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, stage); break;
        case 8: k_csr_rk4<8><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, stage); break;
        case 16: k_csr_rk4<16><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, stage); break;
        default: k_csr_rk4<32><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, stage); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_mf_pass(const MFTile* tiles, int ntiles, const MFSolve* solves, int stage, int in_sel, int rk,
                           size_t smem, int grid, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_mf_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    int g = grid > 0 ? (grid < ntiles ? grid : ntiles) : ntiles;
    k_mf_pass<<<g, kMFThreads, smem, st>>>(tiles, ntiles, solves, stage, in_sel, rk);
    return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(const double* a, float* b, int64_t n, cudaStream_t st) {
    k_f64_to_f32<<<grid_for(n) > 4096 ? 4096 : grid_for(n), 256, 0, st>>>(a, b, n);
    return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const float* a, double* b, int64_t n, cudaStream_t st) {
    k_f32_to_f64<<<grid_for(n) > 4096 ? 4096 : grid_for(n), 256, 0, st>>>(a, b, n);
    return cudaGetLastError();
}

}  // namespace sgdg
