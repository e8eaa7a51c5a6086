// evaluate.cu -- point evaluation of sparse-grid DG expansions on the GPU.
//
// reconstruct_DG (src/dg_methods.jl:150-165) sums, over every level block L,
// the k^D coefficients of the one cell of L that contains x, times the
// tensor-product basis V = prod_d v(k, L_d - 1, cell_d, m_d, x_d)
// (src/dg_methods.jl:27-35, 45-53) with cell_d = cell_index(x_d, L_d - 1)
// (src/dg_methods.jl:70-78):
//   level 0:  v = sqrt(2) P_{m-1}(2x - 1)
//   level l:  v = sqrt(2^l) h_m(2^l x - (2 cell - 1)),  h the multiwavelet
//             piece for y < 0 or y >= 0, zero for |y| > 1 (array2poly,
//             src/1d_dg_functions.jl:15-27).
// Points are batched: one warp per point.  The lanes first tabulate the k 1D
// values and the cell of every (dimension, level) in shared memory, then
// split the level blocks among themselves and contract each block's k^D
// coefficients one dimension at a time; a shuffle tree sums the lanes.  All
// arithmetic is FP64, like the reference.  A coordinate below 0 (or NaN)
// has no cell in the reference (an out-of-range index there) and is reported
// as SGDG_EINVAL; above 1 the last cell is used and |y| > 1 gives zero, as
// in the reference.
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>

#include "api_util.h"
#include "device_util.h"

namespace sgdg {
namespace {

constexpr int kEvalWarps = 4;  // warps (points in flight) per CTA

struct EvalShape {
    int D, k, n, nlev;
    int64_t kD;
    const int8_t* levels;      // nlev x D, 1-based
    const int32_t* lev_off;    // nlev
    const double* pieces;      // 3 k x k: level 0, level >= 1 left (y < 0), right (y >= 0); monomials in y
};

__device__ __forceinline__ double pow2(int j) { return __hiloint2double((1023 + j) << 20, 0); }

__global__ void __launch_bounds__(32 * kEvalWarps)
    k_evaluate(EvalShape S, const double* __restrict__ coeffs, int64_t npts, const double* __restrict__ xs,
               double* __restrict__ out, int* err) {
    extern __shared__ double esm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nl = S.n + 1;  // levels per dimension (0-based level 0..n)
    const int tsz = S.D * nl * S.k;
    double* tab = esm + (size_t)warp * (tsz + S.D * nl);  // [d][l][m] values, then [d][l] cells (0-based)
    double* cel = tab + tsz;
    const int k = S.k;
    for (int64_t p = (int64_t)blockIdx.x * kEvalWarps + warp; p < npts; p += (int64_t)gridDim.x * kEvalWarps) {
        for (int e = lane; e < tsz; e += 32) {
            const int d = e / (nl * k), r = e - d * nl * k, l = r / k, m = r - l * k;
            const double x = xs[p * S.D + d];
            if (!(x >= 0.0)) {  // below 0 or NaN
                atomicExch(err, 1);
                tab[e] = 0.0;
                if (m == 0) cel[d * nl + l] = 0.0;
                continue;
            }
            // cell_index(x, l): 1 for l <= 1; 2^(l-1) for x >= 1; else 1 + floor(2^(l-1) x)
            int cell = 1;
            if (l > 1) cell = x >= 1.0 ? (1 << (l - 1)) : 1 + (int)floor(pow2(l - 1) * x);
            double y, scale;
            const double* pc;
            if (l == 0) {
                y = 2.0 * x - 1.0;
                scale = 1.4142135623730951;  // sqrt(2)
                pc = S.pieces + m * k;
            } else {
                y = pow2(l) * x - (double)(2 * cell - 1);
                scale = (l & 1) ? 1.4142135623730951 * pow2(l >> 1) : pow2(l >> 1);  // sqrt(2^l)
                pc = S.pieces + (y < 0.0 ? 1 : 2) * k * k + m * k;
            }
            double s = 0.0;
            if (fabs(y) <= 1.0)
                for (int i = k - 1; i >= 0; i--) s = s * y + pc[i];
            tab[e] = scale * s;
            if (m == 0) cel[d * nl + l] = (double)(cell - 1);
        }
        __syncwarp();
        double acc = 0.0;
        for (int t = lane; t < S.nlev; t += 32) {
            const int8_t* L = S.levels + (size_t)t * S.D;
            int64_t cl = 0, stride = 1;
            for (int d = 0; d < S.D; d++) {
                cl += (int64_t)cel[d * nl + L[d] - 1] * stride;
                stride <<= (L[d] > 2 ? L[d] - 2 : 0);
            }
            const double* c = coeffs + S.lev_off[t] + S.kD * cl;
            const double* v0 = tab + (L[0] - 1) * k;
            int mo[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (S.D >= 3) {
                // outer modes (m_2 .. m_{D-1}, m_2 fastest) times the sum over
                // m_1 of v_1 times the inner sum over m_0: dimensions 0 and 1
                // contracted before the outer product (k^(D-2) (k^2 + k + D - 2)
                // FP64 operations per block instead of k^(D-1) (k + D - 1))
                const double* v1 = tab + (nl + L[1] - 1) * k;
                const int64_t nout = S.kD / (k * k);
                for (int64_t o = 0; o < nout; o++) {
                    double prod = 1.0;
                    for (int d = 2; d < S.D; d++) prod *= tab[(d * nl + L[d] - 1) * k + mo[d]];
                    const double* co = c + o * k * k;
                    double s1 = 0.0;
                    for (int m1 = 0; m1 < k; m1++) {
                        double s0 = 0.0;
                        for (int m0 = 0; m0 < k; m0++) s0 = fma(v0[m0], co[m1 * k + m0], s0);
                        s1 = fma(v1[m1], s0, s1);
                    }
                    acc = fma(prod, s1, acc);
                    for (int d = 2; d < S.D; d++) {  // next outer mode
                        if (++mo[d] < k) break;
                        mo[d] = 0;
                    }
                }
            } else {
                // outer modes (m_1 .. m_{D-1}, m_1 fastest) times the inner sum over m_0
                const int64_t nout = S.kD / k;
                for (int64_t o = 0; o < nout; o++) {
                    double prod = 1.0;
                    for (int d = 1; d < S.D; d++) prod *= tab[(d * nl + L[d] - 1) * k + mo[d]];
                    double s0 = 0.0;
                    for (int m0 = 0; m0 < k; m0++) s0 = fma(v0[m0], c[o * k + m0], s0);
                    acc = fma(prod, s0, acc);
                    for (int d = 1; d < S.D; d++) {  // next outer mode
                        if (++mo[d] < k) break;
                        mo[d] = 0;
                    }
                }
            }
        }
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (lane == 0) out[p] = acc;
        __syncwarp();
    }
}

// Sum over terms of separable products (tensor_construct,
// src/tensor_construct.jl:19-62, and sums of Fourier modes): coefficient i
// of the D-dim vector is  sum_t amp_t * part_t( e^{i phi_t} prod_d Z_td[i_d] )
// with i_d the 1D index of i along d (get_index_1D,
// src/additional_tools.jl:8-13: k * (block of (level, cell)) + mode) and
// part_t the real or imaginary part.  The complex products round each
// product and sum separately, as numpy does.  One thread per coefficient.
struct TermShape {
    int D, k, nlev, nterms;
    int64_t kD, N1, N;
    const int8_t* levels;
    const int32_t* lev_off;
    const double* Z;      // nterms x D x N1 (re, im)
    const double* coef;   // nterms x 4: amp, cos phi, sin phi, part (0 real, 1 imaginary)
};

__global__ void k_tensor_sum(TermShape S, double* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    int lo = 0, hi = S.nlev - 1;
    while (lo < hi) {  // level block holding i
        const int mid = (lo + hi + 1) >> 1;
        if (S.lev_off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    const int8_t* L = S.levels + (size_t)lo * S.D;
    const int64_t local = i - S.lev_off[lo];
    int64_t cl = local / S.kD, ml = local - cl * S.kD;
    int64_t i1[8];
    for (int d = 0; d < S.D; d++) {
        const int64_t nc = (int64_t)1 << (L[d] > 2 ? L[d] - 2 : 0);
        const int64_t c = cl % nc, m = ml % S.k;
        cl /= nc;
        ml /= S.k;
        i1[d] = S.k * ((L[d] >= 2 ? ((int64_t)1 << (L[d] - 2)) : 0) + c) + m;
    }
    double acc = 0.0;
    for (int t = 0; t < S.nterms; t++) {
        const double* cf = S.coef + 4 * t;
        double zr = cf[1], zi = cf[2];
        for (int d = 0; d < S.D; d++) {
            const double* z = S.Z + (((size_t)t * S.D + d) * S.N1 + i1[d]) * 2;
            const double ar = __dsub_rn(__dmul_rn(zr, z[0]), __dmul_rn(zi, z[1]));
            const double ai = __dadd_rn(__dmul_rn(zr, z[1]), __dmul_rn(zi, z[0]));
            zr = ar;
            zi = ai;
        }
        acc = __dadd_rn(acc, __dmul_rn(cf[0], cf[3] != 0.0 ? zi : zr));
    }
    out[i] = acc;
}

// device tables of one (D, k, n, scheme)
struct EvalTables {
    SparseIndex ix;
    DevBuf levels, lev_off, pieces;
    size_t smem = 0;
};

std::mutex g_eval_mu;
std::map<std::tuple<int, int, int, int>, std::unique_ptr<EvalTables>> g_eval;

const EvalTables& eval_tables(int D, int k, int n, int scheme) {
    std::lock_guard<std::mutex> g(g_eval_mu);
    auto key = std::make_tuple(D, k, n, scheme);
    auto f = g_eval.find(key);
    if (f != g_eval.end()) return *f->second;
    std::unique_ptr<EvalTables> T(new EvalTables);
    T->ix = make_index(D, k, n, scheme);
    const SparseIndex& ix = T->ix;
    std::vector<int8_t> lv(ix.levels.size());
    for (size_t i = 0; i < lv.size(); i++) lv[i] = (int8_t)ix.levels[i];
    std::vector<int32_t> lo(ix.lev_off.begin(), ix.lev_off.end());
    std::vector<double> pc((size_t)3 * k * k, 0.0);
    for (int m = 1; m <= k; m++) {
        const HierFn f0 = make_hier_fn(k, 0, 1, m), f1 = make_hier_fn(k, 1, 1, m);
        for (int i = 0; i < k; i++) {
            pc[(size_t)(m - 1) * k + i] = f0.left[i];
            pc[(size_t)k * k + (m - 1) * k + i] = f1.left[i];
            pc[(size_t)2 * k * k + (m - 1) * k + i] = f1.right[i];
        }
    }
    T->levels = upload(lv, nullptr);
    T->lev_off = upload(lo, nullptr);
    T->pieces = upload(pc, nullptr);
    CK(cudaStreamSynchronize(nullptr));
    T->smem = sizeof(double) * (size_t)kEvalWarps * ((size_t)D * (n + 1) * k + (size_t)D * (n + 1));
    const EvalTables& r = *T;
    g_eval.emplace(key, std::move(T));
    return r;
}

void evaluate_impl(int D, int k, int n, int scheme, const double* coeffs, int64_t npts, const double* xs,
                   double* out, cudaStream_t st) {
    if (npts < 0) throw Error(SGDG_EINVAL, "npts must be >= 0");
    const EvalTables& T = eval_tables(D, k, n, scheme);
    if (npts == 0) return;
    if (T.smem > 200 * 1024) throw Error(SGDG_EUNSUPPORTED, "point tables exceed shared memory");
    static bool configured = false;
    if (!configured) {
        CK(cudaFuncSetAttribute(k_evaluate, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        configured = true;
    }
    EvalShape S{D, k, n, T.ix.nlev, T.ix.kD, T.levels.as<int8_t>(), T.lev_off.as<int32_t>(), T.pieces.as<double>()};
    DevBuf err(sizeof(int));
    CK(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t need = (npts + kEvalWarps - 1) / kEvalWarps;
    const int grid = (int)std::min<int64_t>(need, (int64_t)sms * 16);
    k_evaluate<<<grid, 32 * kEvalWarps, T.smem, st>>>(S, coeffs, npts, xs, out, err.as<int>());
    CK(cudaGetLastError());
    int h_err = 0;
    CK(cudaMemcpyAsync(&h_err, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h_err) throw Error(SGDG_EINVAL, "a point coordinate is below 0 or NaN (no cell contains it)");
}

void tensor_sum_impl(int D, int k, int n, int scheme, int nterms, const double* Z, const double* coef, double* out,
                     cudaStream_t st) {
    const EvalTables& T = eval_tables(D, k, n, scheme);
    TermShape S{D, k, T.ix.nlev, nterms, T.ix.kD, (int64_t)k << n, T.ix.N, T.levels.as<int8_t>(),
                T.lev_off.as<int32_t>(), Z, coef};
    k_tensor_sum<<<(int)((T.ix.N + 255) / 256), 256, 0, st>>>(S, out);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
}

void check_shape(int D, int k, int n) {
    if (D < 1 || D > 8) throw Error(SGDG_EINVAL, "D must be in 1..8");
    if (k < 1 || k > kKMax) throw Error(SGDG_EINVAL, "k must be in 1..10");
    if (n < 0 || n > 24) throw Error(SGDG_EINVAL, "n must be in 0..24");
}

}  // namespace
}  // namespace sgdg

using namespace sgdg;

extern "C" {

int sgdg_evaluate(int D, int k, int n, int scheme, const double* coeffs, int64_t npts, const double* xs,
                  double* values) {
    API_BEGIN
    check_shape(D, k, n);
    NEED(coeffs);
    if (npts > 0) {
        NEED(xs);
        NEED(values);
    }
    require_gpu();
    const SparseIndex& ix = eval_tables(D, k, n, scheme).ix;
    if (npts == 0) return SGDG_OK;
    cudaStream_t st = nullptr;
    DevBuf dc(sizeof(double) * ix.N), dx(sizeof(double) * (size_t)npts * D), dv(sizeof(double) * (size_t)npts);
    CK(cudaMemcpyAsync(dc.p, coeffs, sizeof(double) * ix.N, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dx.p, xs, sizeof(double) * (size_t)npts * D, cudaMemcpyHostToDevice, st));
    evaluate_impl(D, k, n, scheme, dc.as<double>(), npts, dx.as<double>(), dv.as<double>(), st);
    CK(cudaMemcpyAsync(values, dv.p, sizeof(double) * (size_t)npts, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    API_END
}

int sgdg_tensor_sum(int D, int k, int n, int scheme, int nterms, const double* Z, const double* coef, double* out) {
    API_BEGIN
    check_shape(D, k, n);
    if (nterms < 1) throw Error(SGDG_EINVAL, "nterms must be >= 1");
    NEED(Z);
    NEED(coef);
    NEED(out);
    require_gpu();
    const SparseIndex& ix = eval_tables(D, k, n, scheme).ix;
    const size_t zlen = (size_t)nterms * D * ((size_t)k << n) * 2;
    cudaStream_t st = nullptr;
    DevBuf dz(sizeof(double) * zlen), dc(sizeof(double) * 4 * (size_t)nterms), dout(sizeof(double) * ix.N);
    CK(cudaMemcpyAsync(dz.p, Z, sizeof(double) * zlen, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dc.p, coef, sizeof(double) * 4 * nterms, cudaMemcpyHostToDevice, st));
    tensor_sum_impl(D, k, n, scheme, nterms, dz.as<double>(), dc.as<double>(), dout.as<double>(), st);
    CK(cudaMemcpyAsync(out, dout.p, sizeof(double) * ix.N, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    API_END
}

int sgdg_evaluate_device(int D, int k, int n, int scheme, const double* coeffs_dev, int64_t npts,
                         const double* xs_dev, double* values_dev, void* stream) {
    API_BEGIN
    check_shape(D, k, n);
    NEED(coeffs_dev);
    if (npts > 0) {
        NEED(xs_dev);
        NEED(values_dev);
    }
    require_gpu();
    evaluate_impl(D, k, n, scheme, coeffs_dev, npts, xs_dev, values_dev, (cudaStream_t)stream);
    API_END
}

}  // extern "C"
