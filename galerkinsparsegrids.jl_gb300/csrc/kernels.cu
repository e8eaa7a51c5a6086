// kernels.cu -- the plain form and small helpers.
//
//  * k_csr: FP64 CSR mat-vec (the closure body *(RHS, x) of src/pdes.jl:63)
//    over NV vectors in one pass over A, or with NV = 1 fused with the
//    classical RK4 stage combination.  Rows are binned by length
//    (DevCSR.bin_*): a row of bin b gets 2^b lanes with at most eight entries
//    each (four in flight), so the short and the long rows of one matrix (the
//    nodal transforms hold both) keep the lanes equally busy and the lane
//    reduction (csr_reduce) stays small against the FMAs -- on GB300 both run
//    on the FP64 pipe, which bounds these kernels; every block of the grid
//    serves one bin.  Rows longer than A.split are summed by
//    k_csr_segments (one warp per segment) and k_csr_long_rows (segment
//    partials in order, then the same epilogue).
//    Element (j, i) of the vector set x is x[i * xi + j * xs]: xi = 1 and
//    xs = length for vectors one after another, xi = count and xs = 1 for
//    interleaved vectors, whose values at one column share a sector and come
//    in as one 32-byte (W = 4) or 16-byte (W = 2) load.
//  * k_vlasov_points: the point-basis combination of the Vlasov right-hand side.
//  * k_f64_to_f32 / k_f32_to_f64: precision conversions of whole vectors.
#include <cuda_runtime.h>

#include <cstdint>

#include "bounds.cuh"
#include "engine.h"
#include "rk.cuh"

namespace sgdg {

struct CsrRK {  // stage update of the RK4 epilogue: k = A uin, then rk_stage
    double* acc;
    double* uout;
    double dt, hdt, dt6;
    int stage;
};

// 256-bit read-only load (sm_100 and later); p 32-byte aligned
__device__ __forceinline__ void ld_nc_v4(const double* p, double& a, double& b, double& c, double& d) {
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];" : "=d"(a), "=d"(b), "=d"(c), "=d"(d) : "l"(p));
}

// the values of NV vectors at one column (element offset off = column * xi),
// W adjacent vectors per load (W = 2: 16-byte, W = 4: 32-byte aligned)
template <int NV, int W>
__device__ __forceinline__ void csr_gather(const double* __restrict__ x, int64_t off, int64_t xs, double (&v)[NV]) {
    if constexpr (W == 4) {
#pragma unroll
        for (int j = 0; j < NV; j += 4) ld_nc_v4(x + off + j, v[j], v[j + 1], v[j + 2], v[j + 3]);
    } else if constexpr (W == 2) {
#pragma unroll
        for (int j = 0; j < NV; j += 2) {
            const double2 t = __ldg(reinterpret_cast<const double2*>(x + off + j));
            v[j] = t.x;
            v[j + 1] = t.y;
        }
    } else {
#pragma unroll
        for (int j = 0; j < NV; j++) v[j] = __ldg(x + off + j * xs);
    }
}

// Sum of s[0..NV) over the VS lanes of a row group.  With NV = 2 or 4 the
// first steps exchange halves of the vector set instead of every value (a
// lane keeps the half selected by its lane bit and adds its partner's copy),
// so a row costs log2(VS) + NV - 2 FP64 additions per lane instead of
// NV log2(VS); each vector's sum has the pairing, and therefore the value, of
// the all-lane butterfly.  On return vector j's sum is in s[0] of the lanes
// whose group index has j in its top bits (csr_owner), or in s[j] of every
// lane when there was nothing to exchange (NV = 1 or 3, or VS too small).
template <int VS, int NV>
__device__ __forceinline__ void csr_reduce(double (&s)[NV], int lane) {
    if constexpr ((NV == 4 && VS >= 4) || (NV == 2 && VS >= 2)) {
        constexpr int o1 = VS / 2;
        const bool up1 = lane & o1;
        double h[NV / 2];
#pragma unroll
        for (int i = 0; i < NV / 2; i++) {
            const double keep = up1 ? s[NV / 2 + i] : s[i];
            const double give = up1 ? s[i] : s[NV / 2 + i];
            h[i] = keep + __shfl_xor_sync(0xffffffffu, give, o1);
        }
        double r;
        int o;
        if constexpr (NV == 4) {
            constexpr int o2 = VS / 4;
            const bool up2 = lane & o2;
            const double keep = up2 ? h[1] : h[0];
            const double give = up2 ? h[0] : h[1];
            r = keep + __shfl_xor_sync(0xffffffffu, give, o2);
            o = VS / 8;
        } else {
            r = h[0];
            o = VS / 4;
        }
        for (; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        s[0] = r;
    } else {
#pragma unroll
        for (int j = 0; j < NV; j++)
#pragma unroll
            for (int o = VS / 2; o > 0; o >>= 1) s[j] += __shfl_xor_sync(0xffffffffu, s[j], o);
    }
}

// Which vector's sum the lane holds after csr_reduce (-1: all of them, in
// s[j]); only lanes whose low bits are zero store it.
template <int VS, int NV>
__device__ __forceinline__ int csr_owner(int lane, bool& stores) {
    if constexpr ((NV == 4 && VS >= 4) || (NV == 2 && VS >= 2)) {
        constexpr int per = VS / NV;  // lanes holding one vector's sum
        stores = lane % per == 0;
        // vector index: bit VS/2 selects the upper half of the set, then bit VS/4 within it
        if constexpr (NV == 4)
            return ((lane & (VS / 2)) ? 2 : 0) + ((lane & (VS / 4)) ? 1 : 0);
        else
            return (lane & (VS / 2)) ? 1 : 0;
    } else {
        stores = lane == 0;
        return -1;
    }
}

// s[j] = row `row` of A times vector j, summed over VS lanes (row < 0: zeros,
// but the lanes still take part in the shuffles); see csr_reduce for where
// the sums end up
template <int VS, int NV, int W>
__device__ __forceinline__ void csr_row(const DevCSR& A, int64_t row, const double* __restrict__ x, int64_t xi,
                                        int64_t xs, int lane, double (&s)[NV]) {
#pragma unroll
    for (int j = 0; j < NV; j++) s[j] = 0.0;
    if (row >= 0) {
        const int64_t b = A.rowptr[row], e = A.rowptr[row + 1];
        int64_t p = b + lane;
        // four entries per lane in flight: the column loads, then the gathers of x
        for (; p + 3 * VS < e; p += 4 * VS) {
            int c0 = __ldg(A.col + p), c1 = __ldg(A.col + p + VS), c2 = __ldg(A.col + p + 2 * VS),
                c3 = __ldg(A.col + p + 3 * VS);
            if (!SGDG_IN(c0, A.m)) c0 = 0;  // debug build: counted, read column 0 instead
            if (!SGDG_IN(c1, A.m)) c1 = 0;
            if (!SGDG_IN(c2, A.m)) c2 = 0;
            if (!SGDG_IN(c3, A.m)) c3 = 0;
            const double v0 = __ldg(A.val + p), v1 = __ldg(A.val + p + VS), v2 = __ldg(A.val + p + 2 * VS),
                         v3 = __ldg(A.val + p + 3 * VS);
            double x0[NV], x1[NV], x2[NV], x3[NV];
            csr_gather<NV, W>(x, c0 * xi, xs, x0);
            csr_gather<NV, W>(x, c1 * xi, xs, x1);
            csr_gather<NV, W>(x, c2 * xi, xs, x2);
            csr_gather<NV, W>(x, c3 * xi, xs, x3);
#pragma unroll
            for (int j = 0; j < NV; j++) {
                s[j] = fma(v0, x0[j], s[j]);
                s[j] = fma(v1, x1[j], s[j]);
                s[j] = fma(v2, x2[j], s[j]);
                s[j] = fma(v3, x3[j], s[j]);
            }
        }
        for (; p < e; p += VS) {
            int c = __ldg(A.col + p);
            if (!SGDG_IN(c, A.m)) c = 0;
            const double v = __ldg(A.val + p);
            double xv[NV];
            csr_gather<NV, W>(x, c * xi, xs, xv);
#pragma unroll
            for (int j = 0; j < NV; j++) s[j] = fma(v, xv[j], s[j]);
        }
    }
    csr_reduce<VS, NV>(s, lane);
}

__device__ __forceinline__ void csr_rk_update(const CsrRK& rk, int64_t row, double k, double* y) {
    double yy = y[row], aa = rk.stage == 1 ? 0.0 : rk.acc[row], un;
    rk_stage(rk.stage, rk.dt, rk.hdt, rk.dt6, k, yy, aa, un);
    if (rk.stage == 4)
        y[row] = yy;
    else {
        rk.acc[row] = aa;
        rk.uout[row] = un;
    }
}

// the rows of bin `bin`, 2^bin = VS lanes each
template <int VS, int NV, int W, bool RK>
__device__ __forceinline__ void csr_bin(const DevCSR& A, int bin, int64_t rb, const double* __restrict__ x, int64_t xi,
                                        int64_t xs, double* y, int64_t yi, int64_t ys, const CsrRK& rk) {
    const int64_t t = (rb - A.bin_block[bin]) * blockDim.x + threadIdx.x;
    const int64_t idx = t / VS, first = A.bin_first[bin];
    const int lane = int(t % VS);
    int64_t row = idx < A.bin_first[bin + 1] - first ? (int64_t)A.bin_rows[first + idx] : -1;
    if (row >= 0 && !SGDG_IN(row, A.m)) row = -1;
    double s[NV];
    csr_row<VS, NV, W>(A, row, x, xi, xs, lane, s);
    bool stores;
    const int owner = csr_owner<VS, NV>(lane, stores);
    if (row >= 0 && stores) {
        if constexpr (RK)
            csr_rk_update(rk, row, s[0], y);
        else if (owner >= 0)
            y[row * yi + owner * ys] = s[0];
        else {
#pragma unroll
            for (int j = 0; j < NV; j++) y[row * yi + j * ys] = s[j];
        }
    }
}

// With nb > 1 solves sharing A (RK only; solve s's vectors at s * bs), block
// b is (row block, solve): the solves go in groups of sg, and within a group
// the solve index runs fastest, so the group's passes over a row block run
// side by side and read its matrix entries from L2 while the group's vectors
// stay there too (A is streamed once per group instead of once per solve).
template <int NV, int W, bool RK>
__global__ void __launch_bounds__(256) k_csr(DevCSR A, const double* __restrict__ x, int64_t xi, int64_t xs,
                                             double* y, int64_t yi, int64_t ys, CsrRK rk, int64_t bs, int64_t nb,
                                             int sg) {
    int64_t rb = blockIdx.x;
    if constexpr (RK) {
        if (nb > 1) {
            const int64_t nrb = A.bin_block[kCsrBins], b = blockIdx.x, full = nb / sg, fb = full * nrb * sg;
            int64_t sl;
            if (b < fb) {
                const int64_t g = b / (nrb * sg), r = b - g * nrb * sg;
                rb = r / sg;
                sl = g * sg + r % sg;
            } else {
                const int64_t tail = nb - full * sg, r = b - fb;
                rb = r / tail;
                sl = full * sg + r % tail;
            }
            const int64_t o = sl * bs;
            x += o;
            y += o;
            rk.acc += o;
            rk.uout += o;
        }
    }
    int bin = 0;
    while (bin + 1 < kCsrBins && rb >= A.bin_block[bin + 1]) bin++;
    switch (bin) {
        case 0: csr_bin<1, NV, W, RK>(A, 0, rb, x, xi, xs, y, yi, ys, rk); break;
        case 1: csr_bin<2, NV, W, RK>(A, 1, rb, x, xi, xs, y, yi, ys, rk); break;
        case 2: csr_bin<4, NV, W, RK>(A, 2, rb, x, xi, xs, y, yi, ys, rk); break;
        case 3: csr_bin<8, NV, W, RK>(A, 3, rb, x, xi, xs, y, yi, ys, rk); break;
        case 4: csr_bin<16, NV, W, RK>(A, 4, rb, x, xi, xs, y, yi, ys, rk); break;
        default: csr_bin<32, NV, W, RK>(A, 5, rb, x, xi, xs, y, yi, ys, rk); break;
    }
}

// one warp per segment of a long row; partial sums of vector j at
// A.partial[j * A.nseg + seg]
template <int NV, int W>
__global__ void __launch_bounds__(256) k_csr_segments(DevCSR A, const double* __restrict__ x, int64_t xi,
                                                      int64_t xs) {
    const int64_t seg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (seg >= A.nseg) return;
    double s[NV];
#pragma unroll
    for (int j = 0; j < NV; j++) s[j] = 0.0;
    const int64_t e = A.seg_end[seg];
    int64_t p = A.seg_begin[seg] + lane;
    for (; p + 96 < e; p += 128) {
        int c0 = __ldg(A.col + p), c1 = __ldg(A.col + p + 32), c2 = __ldg(A.col + p + 64), c3 = __ldg(A.col + p + 96);
        if (!SGDG_IN(c0, A.m)) c0 = 0;
        if (!SGDG_IN(c1, A.m)) c1 = 0;
        if (!SGDG_IN(c2, A.m)) c2 = 0;
        if (!SGDG_IN(c3, A.m)) c3 = 0;
        const double v0 = __ldg(A.val + p), v1 = __ldg(A.val + p + 32), v2 = __ldg(A.val + p + 64),
                     v3 = __ldg(A.val + p + 96);
        double x0[NV], x1[NV], x2[NV], x3[NV];
        csr_gather<NV, W>(x, c0 * xi, xs, x0);
        csr_gather<NV, W>(x, c1 * xi, xs, x1);
        csr_gather<NV, W>(x, c2 * xi, xs, x2);
        csr_gather<NV, W>(x, c3 * xi, xs, x3);
#pragma unroll
        for (int j = 0; j < NV; j++) {
            s[j] = fma(v0, x0[j], s[j]);
            s[j] = fma(v1, x1[j], s[j]);
            s[j] = fma(v2, x2[j], s[j]);
            s[j] = fma(v3, x3[j], s[j]);
        }
    }
    for (; p < e; p += 32) {
        int c = __ldg(A.col + p);
        if (!SGDG_IN(c, A.m)) c = 0;
        const double v = __ldg(A.val + p);
        double xv[NV];
        csr_gather<NV, W>(x, c * xi, xs, xv);
#pragma unroll
        for (int j = 0; j < NV; j++) s[j] = fma(v, xv[j], s[j]);
    }
    csr_reduce<32, NV>(s, lane);
    bool stores;
    const int owner = csr_owner<32, NV>(lane, stores);
    if (stores) {
        if (owner >= 0)
            A.partial[owner * A.nseg + seg] = s[0];
        else {
#pragma unroll
            for (int j = 0; j < NV; j++) A.partial[j * A.nseg + seg] = s[j];
        }
    }
}

// one thread per (long row, vector): the row's segment partials in order,
// then the store or (rk_on, one vector) the RK4 stage update
__global__ void k_csr_long_rows(DevCSR A, int nv, double* y, int64_t yi, int64_t ys, CsrRK rk, bool rk_on) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.nlong * nv) return;
    const int64_t i = t % A.nlong;
    const int j = int(t / A.nlong);
    double s = 0.0;
    for (int q = A.long_seg[i]; q < A.long_seg[i + 1]; q++) s += A.partial[j * A.nseg + q];
    const int64_t row = A.long_row[i];
    if (!SGDG_IN(row, A.m)) return;
    if (rk_on)
        csr_rk_update(rk, row, s, y);
    else
        y[row * yi + j * ys] = s;
}

__global__ void k_f64_to_f32(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void k_f32_to_f64(const float* __restrict__ a, double* __restrict__ b, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

// Vlasov right-hand side in the point basis (src/pdes.jl:185-191): with the
// 2D transformed derivatives interleaved, pt[i * 2D + d] (x dimensions d < D,
// then p),
//   out = -(sum_d v_d .* pt_d) + sum_d F_d .* pt_{D+d},
// each sum left to right with separate roundings of products and sums.
__global__ void k_vlasov_points(const double* __restrict__ v, const double* __restrict__ F,
                                const double* __restrict__ pt, int D, int64_t n, double* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double* q = pt + i * 2 * D;
        double c1 = __dmul_rn(v[i], q[0]), c2 = __dmul_rn(F[i], q[D]);
        for (int d = 1; d < D; d++) {
            c1 = __dadd_rn(c1, __dmul_rn(v[d * n + i], q[d]));
            c2 = __dadd_rn(c2, __dmul_rn(F[d * n + i], q[D + d]));
        }
        out[i] = __dadd_rn(-c1, c2);
    }
}

SGDG_BOUNDS_READER(csr_bounds_violations)

// ------------------------------------------------------------ launchers ----
static int grid_for(int64_t threads) {
    int64_t b = (threads + 255) / 256;
    return (int)(b > (1LL << 30) ? (1LL << 30) : (b < 1 ? 1 : b));
}

template <int NV, int W, bool RK>
static void csr_pass(const DevCSR& A, const double* x, int64_t xi, int64_t xs, double* y, int64_t yi, int64_t ys,
                     const CsrRK& rk, cudaStream_t st) {
    if (A.bin_block[kCsrBins] > 0)
        k_csr<NV, W, RK><<<A.bin_block[kCsrBins], 256, 0, st>>>(A, x, xi, xs, y, yi, ys, rk, 0, 1, 1);
    if (A.nlong > 0) {
        k_csr_segments<NV, W><<<grid_for(A.nseg * 32), 256, 0, st>>>(A, x, xi, xs);
        k_csr_long_rows<<<grid_for(A.nlong * NV), 256, 0, st>>>(A, NV, y, yi, ys, rk, RK);
    }
}

cudaError_t launch_csr_spmv(const DevCSR& A, const double* x, double* y, cudaStream_t st) {
    csr_pass<1, 1, false>(A, x, 1, 0, y, 1, 0, CsrRK{}, st);
    return cudaGetLastError();
}

// y_j = A x_j for j < nv, kCsrMaxVec vectors per pass over A; element (j, i)
// of x at x[i * xi + j * xs], of y at y[i * yi + j * ys]
cudaError_t launch_csr_spmv_multi(const DevCSR& A, int nv, const double* x, int64_t xi, int64_t xs, double* y,
                                  int64_t yi, int64_t ys, cudaStream_t st) {
    for (int j = 0; j < nv; j += kCsrMaxVec) {
        const double* xj = x + (int64_t)j * xs;
        double* yj = y + (int64_t)j * ys;
        const int w = nv - j < kCsrMaxVec ? nv - j : kCsrMaxVec;
        // one load per column for adjacent vectors whose group is aligned at every column
        const uintptr_t a = reinterpret_cast<uintptr_t>(xj);
        const int wide = xs != 1 ? 1 : (w == 4 && xi % 4 == 0 && a % 32 == 0) ? 4 : (w % 2 == 0 && xi % 2 == 0 && a % 16 == 0) ? 2 : 1;
        const CsrRK none{};
        if (w == 4 && wide == 4)
            csr_pass<4, 4, false>(A, xj, xi, xs, yj, yi, ys, none, st);
        else if (w == 4 && wide == 2)
            csr_pass<4, 2, false>(A, xj, xi, xs, yj, yi, ys, none, st);
        else if (w == 4)
            csr_pass<4, 1, false>(A, xj, xi, xs, yj, yi, ys, none, st);
        else if (w == 3)
            csr_pass<3, 1, false>(A, xj, xi, xs, yj, yi, ys, none, st);
        else if (w == 2 && wide == 2)
            csr_pass<2, 2, false>(A, xj, xi, xs, yj, yi, ys, none, st);
        else if (w == 2)
            csr_pass<2, 1, false>(A, xj, xi, xs, yj, yi, ys, none, st);
        else
            csr_pass<1, 1, false>(A, xj, xi, xs, yj, yi, ys, none, st);
    }
    return cudaGetLastError();
}

cudaError_t launch_csr_rk4(const DevCSR& A, const double* uin, double* y, double* acc, double* uout, double dt,
                           int stage, cudaStream_t st) {
    const CsrRK rk{acc, uout, dt, 0.5 * dt, dt / 6.0, stage};
    csr_pass<1, 1, true>(A, uin, 1, 0, y, 1, 0, rk, st);
    return cudaGetLastError();
}

// solves per group of the batched row kernel: 16 solves of the 3D k=3 n=7 wave
// (733 KB of state each) keep their vectors in L2 while they share A's rows;
// 1, 4, 8, 32 and 64 measured 33.0, 32.0, 31.9, 31.8 and 31.8 ms per step of
// 256 solves against 31.9 (the FP64 additions, not A's bytes, bound the pass)
constexpr int kPlainSolveGroup = 16;

// One RK4 stage of nb solves that share A, their vectors one after another
// (solve s at s * bs): one launch of the row kernel over (row block, solve)
// pairs, the solves in groups that stream A once each; a matrix with long
// rows (segment partials) takes one pass per solve.
cudaError_t launch_csr_rk4_batch(const DevCSR& A, int64_t nb, int64_t bs, const double* uin, double* y, double* acc,
                                 double* uout, double dt, int stage, cudaStream_t st) {
    const CsrRK rk{acc, uout, dt, 0.5 * dt, dt / 6.0, stage};
    const int64_t nrb = A.bin_block[kCsrBins];
    if (A.nlong == 0 && nb * nrb < (int64_t(1) << 31)) {
        if (nrb > 0 && nb > 0)
            k_csr<1, 1, true><<<(unsigned)(nrb * nb), 256, 0, st>>>(A, uin, 1, 0, y, 1, 0, rk, bs, nb,
                                                                   kPlainSolveGroup);
        return cudaGetLastError();
    }
    for (int64_t s = 0; s < nb; s++) {
        const CsrRK r{acc + s * bs, uout + s * bs, dt, 0.5 * dt, dt / 6.0, stage};
        csr_pass<1, 1, true>(A, uin + s * bs, 1, 0, y + s * bs, 1, 0, r, st);
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
cudaError_t launch_vlasov_points(const double* v, const double* F, const double* pt, int D, int64_t n, double* out,
                                 cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_vlasov_points<<<grid_for(n) > 4096 ? 4096 : grid_for(n), 256, 0, st>>>(v, F, pt, D, n, out);
    return cudaGetLastError();
}
}  // namespace sgdg
