// gpu_assemble.cu -- the plain-form operators assembled on the GPU.
//
// D_d (src/multidim_derivative.jl:19-58) couples only elements on one line
// along d (equal in every dimension but d), and row i's entries along its
// line are the leading block of the 1D operator for the line's length (the
// admissible levels of the pencil), mapped to global indices.  So is D_d D_d,
// with the leading block squared; the Laplacian (src/multidim_derivative.jl:
// 71-79) sums those over d, and lines of different dimensions meet only at
// the diagonal.  The host tabulates the 1D blocks per line length
// (line_tables, assemble.cpp) and the pencils' row offsets; the GPU
// enumerates every element of every pencil (one thread each), counts its
// row, and after a host prefix sum of the counts writes the row, columns in
// ascending order.  Sums over d merge the D sorted rows with the fold the
// host's spgemm_sum / add_scaled use (0.0 + term_0 + term_1 + ..., a missing
// term being 0.0, products rounded before the add), so the device operator
// holds the same stored entries and the same values as the host one.
#include <cuda_runtime.h>

#include <climits>

#include "../../include/sgdg.h"
#include "device_csr.h"

namespace sgdg {
namespace {

struct PencilDesc {
    int64_t ebase;    // first element of the pencil in the enumeration
    int32_t lmax, R;  // levels along d, columns
    int32_t lp, roff; // log2 cells of the dimensions below d; first row pair in rows
};

struct LineArgs {
    const PencilDesc* pen;
    int np;
    int64_t N;
    const int2* rows;        // (row offset, lc) per pencil row
    const int64_t* troff;    // table lm starts at trowptr[troff[lm - 1]]
    const int64_t* trowptr;
    const int32_t* tcol;
    const double* tval;
    int kD, kd1, kDm1, k;    // k^D, k^d, k^(D-1)
};

// element e of the enumeration: its global index, pencil, row in the pencil,
// and the column parts (a, b)
__device__ __forceinline__ void locate(const LineArgs& A, int64_t e, int& P, int& row, int& a, int& b) {
    int lo = 0, hi = A.np - 1;
    while (lo < hi) {  // last pencil with ebase <= e
        const int mid = (lo + hi + 1) >> 1;
        if (A.pen[mid].ebase <= e) lo = mid; else hi = mid - 1;
    }
    P = lo;
    const PencilDesc pd = A.pen[P];
    const int64_t local = e - pd.ebase;
    row = (int)(local / pd.R);
    const int r = (int)(local - (int64_t)row * pd.R);
    const int cr = r / A.kDm1, mr = r - cr * A.kDm1;
    const int mq = mr / A.kd1;
    a = A.kD * (cr & ((1 << pd.lp) - 1)) + (mr - mq * A.kd1) + mq * A.kd1 * A.k;
    b = A.kD * ((cr >> pd.lp) << pd.lp);
}

__global__ void k_line_count(LineArgs A, int32_t* rowlen) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.N) return;
    int P, row, a, b;
    locate(A, e, P, row, a, b);
    const PencilDesc pd = A.pen[P];
    const int2 ri = A.rows[pd.roff + row];
    const int64_t* rp = A.trowptr + A.troff[pd.lmax - 1];
    rowlen[ri.x + a + (b << ri.y)] = (int32_t)(rp[row + 1] - rp[row]);
}

__global__ void k_line_fill(LineArgs A, const int64_t* __restrict__ rowptr, int32_t* __restrict__ col,
                            double* __restrict__ val) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.N) return;
    int P, row, a, b;
    locate(A, e, P, row, a, b);
    const PencilDesc pd = A.pen[P];
    const int2 ri = A.rows[pd.roff + row];
    const int64_t* rp = A.trowptr + A.troff[pd.lmax - 1];
    int64_t w = rowptr[ri.x + a + (b << ri.y)];
    for (int64_t t = rp[row]; t < rp[row + 1]; t++, w++) {
        const int2 rq = A.rows[pd.roff + A.tcol[t]];
        col[w] = rq.x + a + (b << rq.y);
        val[w] = A.tval[t];
    }
}

constexpr int kSumMax = 8;
struct SumArgs {
    int nt;
    int64_t m;
    const int64_t* rp[kSumMax];
    const int32_t* cl[kSumMax];
    const double* vl[kSumMax];
    double s[kSumMax];
    int scaled;
};

// merge of the terms' sorted rows: count (rowlen) or write (col, val)
template <bool FILL>
__global__ void k_sum(SumArgs A, int32_t* rowlen, const int64_t* __restrict__ rowptr, int32_t* __restrict__ col,
                      double* __restrict__ val) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.m) return;
    int64_t pos[kSumMax], end[kSumMax];
    for (int t = 0; t < A.nt; t++) {
        pos[t] = A.rp[t][i];
        end[t] = A.rp[t][i + 1];
    }
    int64_t w = FILL ? rowptr[i] : 0;
    int32_t cnt = 0;
    for (;;) {
        int c = INT_MAX;
        for (int t = 0; t < A.nt; t++)
            if (pos[t] < end[t]) c = min(c, A.cl[t][pos[t]]);
        if (c == INT_MAX) break;
        double v = 0.0;
        for (int t = 0; t < A.nt; t++) {
            double x = 0.0;
            if (pos[t] < end[t] && A.cl[t][pos[t]] == c) {
                x = A.scaled ? __dmul_rn(A.s[t], A.vl[t][pos[t]]) : A.vl[t][pos[t]];
                pos[t]++;
            }
            v = __dadd_rn(v, x);
        }
        if (FILL) {
            col[w] = c;
            val[w] = v;
            w++;
        }
        cnt++;
    }
    if (!FILL) rowlen[i] = cnt;
}

// wave right-hand side [[0, I], [L, 0]] (src/pdes.jl:22-49): the identity half
__global__ void k_wave_identity(int64_t N, int32_t* col, double* val) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    col[i] = (int32_t)(N + i);
    val[i] = 1.0;
}

int grid_for(int64_t n) { return (int)std::max<int64_t>(1, (n + 255) / 256); }

// row pointers from device row lengths (host prefix sum)
std::vector<int64_t> scan_rows(const DevBuf& rowlen, int64_t m, cudaStream_t st) {
    std::vector<int32_t> h(m);
    if (m) CK(cudaMemcpyAsync(h.data(), rowlen.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::vector<int64_t> rp(m + 1, 0);
    for (int64_t r = 0; r < m; r++) rp[r + 1] = rp[r] + h[r];
    return rp;
}

// device tables of one dimension's pencils plus one kind of line table
struct LineSetup {
    DevBuf pen, rows, troff, trowptr, tcol, tval;
    LineArgs args{};
};

void setup_line(LineSetup& S, const SparseIndex& ix, const LineTables& T, int d, cudaStream_t st) {
    const std::vector<Pencil> ps = make_pencils(ix, d);
    std::vector<PencilDesc> pd;
    std::vector<int32_t> rows;
    int64_t e = 0;
    for (const Pencil& p : ps) {
        PencilDesc q{};
        q.ebase = e;
        q.lmax = p.lmax;
        q.R = (int32_t)p.R;
        q.lp = p.lp;
        q.roff = (int32_t)(rows.size() / 2);
        pencil_rows(p, ix.k, ix.kD, rows);
        e += (int64_t)ix.k * (int64_t(1) << (p.lmax - 1)) * p.R;
        pd.push_back(q);
    }
    if (e != ix.N) throw Error(SGDG_EINVAL, "pencils do not partition the index set");
    S.pen = upload(pd, st);
    S.rows = upload(rows, st);
    S.troff = upload(T.roff, st);
    S.trowptr = upload(T.rowptr, st);
    S.tcol = upload(T.col, st);
    S.tval = upload(T.val, st);
    int kd1 = 1, kDm1 = 1;
    for (int q = 0; q < d; q++) kd1 *= ix.k;
    for (int q = 0; q < ix.D - 1; q++) kDm1 *= ix.k;
    S.args = LineArgs{S.pen.as<PencilDesc>(), (int)pd.size(), ix.N, S.rows.as<int2>(), S.troff.as<int64_t>(),
                      S.trowptr.as<int64_t>(), S.tcol.as<int32_t>(), S.tval.as<double>(),
                      (int)ix.kD, kd1, kDm1, ix.k};
}

// one dimension's line operator as a device CSR; rp_host receives the row pointers
std::unique_ptr<DeviceCSR> line_operator(const SparseIndex& ix, const LineTables& T, int d, cudaStream_t st,
                                         std::vector<int64_t>& rp_host) {
    LineSetup S;
    setup_line(S, ix, T, d, st);
    DevBuf rowlen(sizeof(int32_t) * (size_t)ix.N);
    k_line_count<<<grid_for(ix.N), 256, 0, st>>>(S.args, rowlen.as<int32_t>());
    CK(cudaGetLastError());
    rp_host = scan_rows(rowlen, ix.N, st);
    auto A = std::make_unique<DeviceCSR>();
    A->rowptr = upload(rp_host, st);
    A->col.alloc(sizeof(int32_t) * (size_t)rp_host[ix.N]);
    A->val.alloc(sizeof(double) * (size_t)rp_host[ix.N]);
    k_line_fill<<<grid_for(ix.N), 256, 0, st>>>(S.args, A->rowptr.as<int64_t>(), A->col.as<int32_t>(),
                                                A->val.as<double>());
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));  // S's tables are freed on return
    return A;
}

// sum over terms (each a device CSR of m rows) with optional scales
std::unique_ptr<DeviceCSR> merge_terms(const std::vector<const DeviceCSR*>& terms, const double* s, int64_t m,
                                       cudaStream_t st, std::vector<int64_t>& rp_host) {
    if (terms.empty() || terms.size() > (size_t)kSumMax) throw Error(SGDG_EINVAL, "1..8 terms");
    SumArgs A{};
    A.nt = (int)terms.size();
    A.m = m;
    A.scaled = s != nullptr;
    for (int t = 0; t < A.nt; t++) {
        A.rp[t] = terms[t]->rowptr.as<int64_t>();
        A.cl[t] = terms[t]->col.as<int32_t>();
        A.vl[t] = terms[t]->val.as<double>();
        A.s[t] = s ? s[t] : 1.0;
    }
    DevBuf rowlen(sizeof(int32_t) * (size_t)m);
    k_sum<false><<<grid_for(m), 256, 0, st>>>(A, rowlen.as<int32_t>(), nullptr, nullptr, nullptr);
    CK(cudaGetLastError());
    rp_host = scan_rows(rowlen, m, st);
    auto R = std::make_unique<DeviceCSR>();
    R->rowptr = upload(rp_host, st);
    R->col.alloc(sizeof(int32_t) * (size_t)rp_host[m]);
    R->val.alloc(sizeof(double) * (size_t)rp_host[m]);
    k_sum<true><<<grid_for(m), 256, 0, st>>>(A, nullptr, R->rowptr.as<int64_t>(), R->col.as<int32_t>(),
                                             R->val.as<double>());
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    return R;
}

}  // namespace

std::unique_ptr<DeviceCSR> gpu_operator(const SparseIndex& ix, const DLF1D& dlf, int which, cudaStream_t st) {
    require_gpu();
    const int D = ix.D;
    std::vector<int64_t> rp;
    if (which >= 1 && which <= D) {
        const LineTables T = line_tables(dlf, dlf.n + 1, false);
        auto A = line_operator(ix, T, which - 1, st, rp);
        finish_device_csr(*A, rp, ix.N, st);
        return A;
    }
    if (which != SGDG_OP_LAPLACIAN && which != SGDG_OP_WAVE_RHS)
        throw Error(SGDG_EINVAL, "operator selector must be 1..D, 0 (laplacian) or -1 (wave RHS)");
    const LineTables T = line_tables(dlf, dlf.n + 1, true);
    std::vector<std::unique_ptr<DeviceCSR>> sq;
    std::vector<const DeviceCSR*> terms;
    for (int d = 0; d < D; d++) {
        std::vector<int64_t> tmp;
        sq.push_back(line_operator(ix, T, d, st, tmp));
        terms.push_back(sq.back().get());
    }
    auto L = merge_terms(terms, nullptr, ix.N, st, rp);
    sq.clear();
    if (which == SGDG_OP_LAPLACIAN) {
        finish_device_csr(*L, rp, ix.N, st);
        return L;
    }
    const int64_t N = ix.N, nnzL = rp[N];
    std::vector<int64_t> wp(2 * N + 1);
    for (int64_t i = 0; i <= N; i++) wp[i] = i;
    for (int64_t i = 1; i <= N; i++) wp[N + i] = N + rp[i];
    auto W = std::make_unique<DeviceCSR>();
    W->rowptr = upload(wp, st);
    W->col.alloc(sizeof(int32_t) * (size_t)(N + nnzL));
    W->val.alloc(sizeof(double) * (size_t)(N + nnzL));
    k_wave_identity<<<grid_for(N), 256, 0, st>>>(N, W->col.as<int32_t>(), W->val.as<double>());
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(W->col.as<int32_t>() + N, L->col.p, sizeof(int32_t) * (size_t)nnzL, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(W->val.as<double>() + N, L->val.p, sizeof(double) * (size_t)nnzL, cudaMemcpyDeviceToDevice, st));
    CK(cudaStreamSynchronize(st));
    finish_device_csr(*W, wp, 2 * N, st);
    return W;
}

std::unique_ptr<DeviceCSR> gpu_scaled_sum(const SparseIndex& ix, const DLF1D& dlf, const double* s, cudaStream_t st) {
    require_gpu();
    const LineTables T = line_tables(dlf, dlf.n + 1, false);
    std::vector<std::unique_ptr<DeviceCSR>> dd;
    std::vector<const DeviceCSR*> terms;
    for (int d = 0; d < ix.D; d++) {
        std::vector<int64_t> tmp;
        dd.push_back(line_operator(ix, T, d, st, tmp));
        terms.push_back(dd.back().get());
    }
    std::vector<int64_t> rp;
    auto A = merge_terms(terms, s, ix.N, st, rp);
    finish_device_csr(*A, rp, ix.N, st);
    return A;
}

CSR download_csr(const DeviceCSR& A, cudaStream_t st) {
    CSR h;
    h.m = h.n = A.d.m;
    h.rowptr.resize(A.d.m + 1);
    h.col.resize(A.d.nnz);
    h.val.resize(A.d.nnz);
    CK(cudaMemcpyAsync(h.rowptr.data(), A.rowptr.p, sizeof(int64_t) * (A.d.m + 1), cudaMemcpyDeviceToHost, st));
    if (A.d.nnz) {
        CK(cudaMemcpyAsync(h.col.data(), A.col.p, sizeof(int32_t) * A.d.nnz, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(h.val.data(), A.val.p, sizeof(double) * A.d.nnz, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    return h;
}

}  // namespace sgdg
