// kernels.cu -- the plain form and small helpers.
//
//  * k_csr_spmv / k_csr_rk4: FP64 CSR mat-vec (the closure body *(RHS, x) of
//    src/pdes.jl:63) with VS lanes per row; the RK4 variant fuses the
//    classical stage combination into the row epilogue.  Rows longer than
//    A.split are skipped there and summed by k_csr_segments (one warp per
//    segment) and k_csr_long_rows (segment partials in order, then the same
//    epilogue).
//  * k_f64_to_f32 / k_f32_to_f64: precision conversions of whole vectors.
#include <cuda_runtime.h>

#include "engine.h"
#include "rk.cuh"

namespace sgdg {

template <int VS>
__device__ __forceinline__ double csr_row(const DevCSR& A, int64_t row, const double* __restrict__ x, int lane,
                                          bool& long_row) {
    double s = 0.0;
    long_row = false;
    if (row < A.m) {
        const int64_t b = A.rowptr[row], e = A.rowptr[row + 1];
        long_row = e - b > A.split;
        if (!long_row) {
            // four entries per lane in flight: the column loads, then the gathers of x
            int64_t p = b + lane;
            for (; p + 3 * VS < e; p += 4 * VS) {
                const int c0 = __ldg(A.col + p), c1 = __ldg(A.col + p + VS), c2 = __ldg(A.col + p + 2 * VS),
                          c3 = __ldg(A.col + p + 3 * VS);
                const double v0 = __ldg(A.val + p), v1 = __ldg(A.val + p + VS), v2 = __ldg(A.val + p + 2 * VS),
                             v3 = __ldg(A.val + p + 3 * VS);
                const double x0 = __ldg(x + c0), x1 = __ldg(x + c1), x2 = __ldg(x + c2), x3 = __ldg(x + c3);
                s = fma(v0, x0, s);
                s = fma(v1, x1, s);
                s = fma(v2, x2, s);
                s = fma(v3, x3, s);
            }
            for (; p < e; p += VS) s = fma(__ldg(A.val + p), __ldg(x + __ldg(A.col + p)), s);
        }
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
    bool long_row;
    double s = csr_row<VS>(A, row, x, lane, long_row);
    if (row < A.m && lane == 0 && !long_row) y[row] = s;
}

template <int VS>
__global__ void __launch_bounds__(256) k_csr_rk4(DevCSR A, const double* uin, double* y, double* __restrict__ acc,
                                                 double* __restrict__ uout, double dt, double hdt, double dt6,
                                                 int stage) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t row = t / VS;
    const int lane = int(t % VS);
    bool long_row;
    double k = csr_row<VS>(A, row, uin, lane, long_row);
    if (row < A.m && lane == 0 && !long_row) {
        double yy = y[row], aa = stage == 1 ? 0.0 : acc[row], un;
        rk_stage(stage, dt, hdt, dt6, k, yy, aa, un);
        if (stage == 4)
            y[row] = yy;
        else {
            acc[row] = aa;
            uout[row] = un;
        }
    }
}

// one warp per segment of a long row
__global__ void __launch_bounds__(256) k_csr_segments(DevCSR A, const double* __restrict__ x) {
    const int64_t seg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (seg >= A.nseg) return;
    double s = 0.0;
    for (int64_t p = A.seg_begin[seg] + lane; p < A.seg_end[seg]; p += 32)
        s = fma(__ldg(A.val + p), __ldg(x + __ldg(A.col + p)), s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) A.partial[seg] = s;
}

// one thread per long row: its segments in order; y = A x, or the RK4 stage
// update when acc is given
__global__ void k_csr_long_rows(DevCSR A, double* y, double* acc, const double* uin, double* uout, double dt,
                                double hdt, double dt6, int stage) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.nlong) return;
    double s = 0.0;
    for (int q = A.long_seg[i]; q < A.long_seg[i + 1]; q++) s += A.partial[q];
    const int64_t row = A.long_row[i];
    if (!acc) {
        y[row] = s;
        return;
    }
    double yy = y[row], aa = stage == 1 ? 0.0 : acc[row], un;
    rk_stage(stage, dt, hdt, dt6, s, yy, aa, un);
    if (stage == 4)
        y[row] = yy;
    else {
        acc[row] = aa;
        uout[row] = un;
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

// Vlasov right-hand side in the point basis (src/pdes.jl:185-191):
//   acc_out = (acc_in or 0) + w .* p; with `other` set, out = -other + acc_out.
__global__ void k_vlasov_combine(const double* __restrict__ w, const double* __restrict__ p, const double* acc_in,
                                 const double* __restrict__ other, double* out, int64_t n) {  // out may be acc_in
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double prod = w[i] * p[i];
        const double a = acc_in ? acc_in[i] + prod : prod;
        out[i] = other ? -other[i] + a : a;
    }
}

// ------------------------------------------------------------ launchers ----
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
    if (A.nlong > 0) {
        k_csr_segments<<<grid_for(A.nseg * 32), 256, 0, st>>>(A, x);
        k_csr_long_rows<<<grid_for(A.nlong), 256, 0, st>>>(A, y, nullptr, nullptr, nullptr, 0.0, 0.0, 0.0, 0);
    }
    return cudaGetLastError();
}

cudaError_t launch_csr_rk4(const DevCSR& A, const double* uin, double* y, double* acc, double* uout, double dt,
                           int stage, cudaStream_t st) {
    const int64_t th = A.m * A.vs;
    const double hdt = 0.5 * dt, dt6 = dt / 6.0;
    switch (A.vs) {
        case 1: k_csr_rk4<1><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, hdt, dt6, stage); break;
        case 2: k_csr_rk4<2><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, hdt, dt6, stage); break;
        case 4: k_csr_rk4<4><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, hdt, dt6, stage); break;
        case 8: k_csr_rk4<8><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, hdt, dt6, stage); break;
        case 16: k_csr_rk4<16><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, hdt, dt6, stage); break;
        default: k_csr_rk4<32><<<grid_for(th), 256, 0, st>>>(A, uin, y, acc, uout, dt, hdt, dt6, stage); break;
    }
    if (A.nlong > 0) {
        k_csr_segments<<<grid_for(A.nseg * 32), 256, 0, st>>>(A, uin);
        k_csr_long_rows<<<grid_for(A.nlong), 256, 0, st>>>(A, y, acc, uin, uout, dt, hdt, dt6, stage);
    }
    return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(const double* a, float* b, int64_t n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_f64_to_f32<<<grid_for(n) > 4096 ? 4096 : grid_for(n), 256, 0, st>>>(a, b, n);
    return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const float* a, double* b, int64_t n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_f32_to_f64<<<grid_for(n) > 4096 ? 4096 : grid_for(n), 256, 0, st>>>(a, b, n);
    return cudaGetLastError();
}

}  // namespace sgdg

namespace sgdg {
cudaError_t launch_vlasov_combine(const double* w, const double* p, const double* acc_in, const double* other,
                                  double* out, int64_t n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_vlasov_combine<<<grid_for(n) > 4096 ? 4096 : grid_for(n), 256, 0, st>>>(w, p, acc_in, other, out, n);
    return cudaGetLastError();
}
}  // namespace sgdg
