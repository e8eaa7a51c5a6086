// project.cu -- vcoeffs_DG (src/dg_vmethods.jl:149-179, src/dg_methods.jl:
// 85-106): the coefficients of a function f on the sparse grid, <f, V> for
// every tensor-product basis function V = prod_d v(k, L_d - 1, c_d, m_d, x_d).
//
// The reference integrates each basis function with hcubature.  Here every
// level block is integrated at once by tensor quadrature on the polynomial
// pieces of its 1D functions: the caller samples f at the block's tensor
// grid of nodes (f is the caller's function, so that part runs on the host)
// and the GPU contracts the samples one dimension at a time (sum
// factorisation): pass q replaces dimension q's (cell, node) axis by its
// (cell, mode) axis, out[.., c k + m, ..] = sum_p W_L[c][m][p] in[.., c P + p, ..],
// with W_L the 1D basis values times the quadrature weights of level L.
// A last gather writes each block in the reference's coefficient order
// (cells, dimension 1 fastest, then modes, dimension 1 fastest).
#include <cuda_runtime.h>

#include <vector>

#include "api_util.h"
#include "device_util.h"

namespace sgdg {
namespace {

// one contraction pass over a block tensor: extents E[] (dimension 0
// fastest), dimension q goes from cells * P to cells * k
__global__ void k_project_pass(const double* __restrict__ in, double* __restrict__ out, const double* __restrict__ W,
                               int64_t inner, int cells, int P, int k, int64_t outer) {
    const int64_t total = inner * cells * k * outer;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = t % inner;
        const int64_t r = t / inner;
        const int v = (int)(r % ((int64_t)cells * k));
        const int64_t b = r / ((int64_t)cells * k);
        const int c = v / k, m = v - c * k;
        const double* w = W + ((int64_t)c * k + m) * P;
        const double* x = in + a + inner * ((int64_t)c * P + (int64_t)cells * P * b);
        double s = 0.0;
        for (int p = 0; p < P; p++) s = fma(w[p], x[inner * p], s);
        out[t] = s;
    }
}

// the contracted block (extents cells_q * k, dimension 0 fastest) into the
// reference order: index cl k^D + ml, cl = sum_q c_q prod_{r<q} cells_r,
// ml = sum_q m_q k^q
struct BlockShape {
    int D, k;
    int cells[kDMax];
};
__global__ void k_project_order(const double* __restrict__ in, double* __restrict__ out, BlockShape S, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = t, src = 0, stride = 1, cl = 0, cstride = 1, ml = 0, mstride = 1;
        for (int q = 0; q < S.D; q++) {
            const int ext = S.cells[q] * S.k;
            const int v = (int)(r % ext);
            r /= ext;
            const int c = v / S.k, m = v - c * S.k;
            src += v * stride;
            stride *= ext;
            cl += c * cstride;
            cstride *= S.cells[q];
            ml += m * mstride;
            mstride *= S.k;
        }
        out[cl * mstride + ml] = in[src];
    }
}

int grid_of(int64_t n) { return (int)std::min<int64_t>(4096, std::max<int64_t>(1, (n + 255) / 256)); }

}  // namespace
}  // namespace sgdg

using namespace sgdg;

int sgdg_vcoeffs_contract(int D, int k, int n, int scheme, const int32_t* npts, const double* wtab,
                          const double* samples, double* out) {
    API_BEGIN
    NEED(npts);
    NEED(wtab);
    NEED(samples);
    NEED(out);
    if (D < 1 || D > kDMax) throw Error(SGDG_EINVAL, "D must be in 1..8");
    const SparseIndex ix = make_index(D, k, n, scheme);
    require_gpu();
    // per level L = 1..n+1: its node count and the offset of W_L in wtab
    std::vector<int64_t> woff(n + 2, 0);
    for (int L = 1; L <= n + 1; L++) {
        if (npts[L - 1] < 1) throw Error(SGDG_EINVAL, "every level needs at least one quadrature node");
        woff[L] = woff[L - 1] + ncells(L) * k * (int64_t)npts[L - 1];
    }
    // sizes: all samples, the largest block before and during contraction
    int64_t nsamp = 0, big = 0;
    for (int b = 0; b < ix.nlev; b++) {
        int64_t ext = 1, mx = 1;
        for (int q = 0; q < D; q++) ext *= ncells(ix.levels[(size_t)b * D + q]) * npts[ix.levels[(size_t)b * D + q] - 1];
        for (int q = 0; q <= D; q++) {  // after q passes
            int64_t e = 1;
            for (int r = 0; r < D; r++) {
                const int L = ix.levels[(size_t)b * D + r];
                e *= ncells(L) * (r < q ? k : npts[L - 1]);
            }
            mx = std::max(mx, e);
        }
        nsamp += ext;
        big = std::max(big, mx);
    }
    cudaStream_t st = nullptr;
    DevBuf dw(sizeof(double) * (size_t)woff[n + 1]), ds(sizeof(double) * (size_t)nsamp);
    DevBuf t0(sizeof(double) * (size_t)big), t1(sizeof(double) * (size_t)big), dout(sizeof(double) * (size_t)ix.N);
    CK(cudaMemcpyAsync(dw.p, wtab, sizeof(double) * (size_t)woff[n + 1], cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ds.p, samples, sizeof(double) * (size_t)nsamp, cudaMemcpyHostToDevice, st));
    int64_t soff = 0;
    for (int b = 0; b < ix.nlev; b++) {
        const int* Lb = &ix.levels[(size_t)b * D];
        int64_t ext[kDMax];
        int64_t tot = 1;
        for (int q = 0; q < D; q++) {
            ext[q] = ncells(Lb[q]) * npts[Lb[q] - 1];
            tot *= ext[q];
        }
        const double* src = ds.as<double>() + soff;
        soff += tot;
        double* bufs[2] = {t0.as<double>(), t1.as<double>()};
        for (int q = 0; q < D; q++) {
            int64_t inner = 1, outer = 1;
            for (int r = 0; r < q; r++) inner *= ext[r];
            for (int r = q + 1; r < D; r++) outer *= ext[r];
            const int cells = (int)ncells(Lb[q]), P = npts[Lb[q] - 1];
            double* dst = bufs[q & 1];
            const int64_t total = inner * cells * k * outer;
            k_project_pass<<<grid_of(total), 256, 0, st>>>(src, dst, dw.as<double>() + woff[Lb[q] - 1], inner, cells, P, k,
                                                         outer);
            CK(cudaGetLastError());
            ext[q] = (int64_t)cells * k;
            src = dst;
        }
        BlockShape S{};
        S.D = D;
        S.k = k;
        for (int q = 0; q < D; q++) S.cells[q] = (int)ncells(Lb[q]);
        const int64_t nb = ix.lev_cells[b] * ix.kD;
        k_project_order<<<grid_of(nb), 256, 0, st>>>(src, dout.as<double>() + ix.lev_off[b], S, nb);
        CK(cudaGetLastError());
    }
    CK(cudaMemcpyAsync(out, dout.p, sizeof(double) * (size_t)ix.N, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    API_END
}
