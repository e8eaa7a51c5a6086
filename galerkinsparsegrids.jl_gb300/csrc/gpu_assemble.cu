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
// term being 0.0, products rounded before the add) and drop sums that are
// exactly 0.0, so the device operator holds the same stored entries and the
// same values as the host one.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>

#include "../../include/sgdg.h"
#include "bounds.cuh"
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
    const int64_t i = ri.x + a + ((int64_t)b << ri.y);
    if (SGDG_IN(i, A.N)) rowlen[i] = (int32_t)(rp[row + 1] - rp[row]);
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
    const int64_t i = ri.x + a + ((int64_t)b << ri.y);
    if (!SGDG_IN(i, A.N)) return;
    int64_t w = rowptr[i];
    for (int64_t t = rp[row]; t < rp[row + 1]; t++, w++) {
        const int2 rq = A.rows[pd.roff + A.tcol[t]];
        const int64_t c = rq.x + a + ((int64_t)b << rq.y);
        if (!SGDG_IN(w - rowptr[i], rowptr[i + 1] - rowptr[i]) || !SGDG_IN(c, A.N)) continue;
        col[w] = (int32_t)c;
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

// merge of the terms' sorted rows: count (rowlen) or write (col, val) the
// entries whose sum is not exactly 0.0
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
        if (v == 0.0) continue;  // map(+) drops sums that are exactly 0.0
        if (FILL && SGDG_IN(w, rowptr[i + 1])) {
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
    for (int64_t r = 0; r < m; r++) {
        if (h[r] < 0) throw Error(SGDG_ECUDA, "negative row length from a device count");
        rp[r + 1] = rp[r] + h[r];
    }
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

// ---------------------------------------------------------- transforms ----
// The D-dim nodal transforms (src/multidim_nodal_basis.jl:40-109) restricted
// to the sparse grid: entry (i, j) is prod_d T1[i_d, j_d] (multiplied in
// dimension order, stopping at an exact 0) over 1D index pairs whose cells
// nest, for j's level tuple admissible, kept when |value| >= 1e-12 -- the
// set transform_dd (nodal.cpp) builds column by column.  Here one thread per
// row i enumerates its columns from the 1D rows of i_d (nesting pairs only,
// filtered on the host): level tuples, then cell tuples, then mode tuples,
// each with dimension 0 varying fastest, which is the order of the global
// index (level blocks in CartesianIndices order, then cells, then modes), so
// the row comes out sorted.
constexpr int kTLev = 16;         // levels per dimension (n + 1)
constexpr int kTRowsPerBlock = 8;  // k_transform: one warp per row
constexpr int64_t kTLongTuples = 1024;  // rows with this many level tuples or more: k_transform_long
constexpr int kTLongThreads = 256;      // k_transform_long: one block per row

struct TransArgs {
    int D, k, n, scheme, nlev;
    int64_t N, kD;
    const int8_t* levels;
    const int32_t* lev_off;
    const int32_t* code2lev;  // (n+1)^D level tuple code -> block, or -1
    const int64_t* rp1;       // filtered 1D rows
    const int32_t* col1;
    const double* val1;
};

__device__ __forceinline__ void dec1d(int k, int j1, int& L, int& c, int& m) {
    const int blk = j1 / k;
    m = j1 - blk * k;                         // 0-based mode
    L = blk == 0 ? 1 : (32 - __clz(blk)) + 1;  // 1-based level
    c = L >= 2 ? blk - (1 << (L - 2)) : 0;     // 0-based cell
}

// the cell-tuple group of dimension d that starts at entry cs: its end
__device__ __forceinline__ int cell_group_end(const TransArgs& A, int cs, int gend) {
    int L0, c0, m0;
    dec1d(A.k, A.col1[cs], L0, c0, m0);
    int ce = cs;
    while (ce < gend) {
        int L, c, m;
        dec1d(A.k, A.col1[ce], L, c, m);
        if (c != c0) break;
        ce++;
    }
    return ce;
}

// Entries of row i in level tuple g (group g[d] of every dimension's 1D row):
// nothing when the tuple is cut or not on the grid, else the cell tuples and
// within them the mode tuples (dimension 0 fastest), products |v| >= 1e-12.
// Returns the count; with FILL also writes them from position w on (never at
// or past lim).
template <bool FILL>
__device__ int32_t tuple_entries(const TransArgs& A, const int* g, const int (*gs)[kTLev], const int (*ge)[kTLev],
                                 const int (*gl)[kTLev], int64_t w, int64_t lim, int32_t* __restrict__ col,
                                 double* __restrict__ val) {
    const int D = A.D, k = A.k;
    int code = 0, lsum = 0, mult = 1;
    for (int d = 0; d < D; d++) {
        code += (gl[d][g[d]] - 1) * mult;
        mult *= A.n + 1;
        lsum += gl[d][g[d]];
    }
    const int blk = (A.scheme == 0 && lsum > A.n + D) ? -1 : A.code2lev[code];
    if (blk < 0) return 0;
    const int64_t base = A.lev_off[blk];
    int32_t cnt = 0;
    int cs[8], ce[8];
    for (int d = 0; d < D; d++) {
        cs[d] = gs[d][g[d]];
        ce[d] = cell_group_end(A, cs[d], ge[d][g[d]]);
    }
    for (;;) {  // cell tuples
        int64_t cell_lin = 0, cstride = 1;
        for (int d = 0; d < D; d++) {
            int L, c, m;
            dec1d(k, A.col1[cs[d]], L, c, m);
            cell_lin += (int64_t)c * cstride;
            cstride <<= (L > 2 ? L - 2 : 0);
        }
        int e[8];
        for (int d = 0; d < D; d++) e[d] = cs[d];
        for (;;) {  // mode tuples
            double v = 1.0;
            for (int d = 0; d < D; d++) {
                v = __dmul_rn(v, A.val1[e[d]]);
                if (v == 0.0) break;
            }
            if (!(fabs(v) < 1e-12)) {
                if (FILL && !(w + cnt < lim)) (void)SGDG_IN(w + cnt, lim);  // debug build: counted
                if (FILL && w + cnt < lim) {
                    int64_t mode_lin = 0, ms = 1;
                    for (int d = 0; d < D; d++) {
                        int L, c, m;
                        dec1d(k, A.col1[e[d]], L, c, m);
                        mode_lin += m * ms;
                        ms *= k;
                    }
                    col[w + cnt] = (int32_t)(base + A.kD * cell_lin + mode_lin);
                    val[w + cnt] = v;
                }
                cnt++;
            }
            int d = 0;
            for (; d < D; d++) {
                if (++e[d] < ce[d]) break;
                e[d] = cs[d];
            }
            if (d == D) break;
        }
        int d = 0;
        for (; d < D; d++) {  // next cell tuple
            if (ce[d] < ge[d][g[d]]) {
                cs[d] = ce[d];
                ce[d] = cell_group_end(A, cs[d], ge[d][g[d]]);
                break;
            }
            cs[d] = gs[d][g[d]];  // wrap to the first cell group of the level
            ce[d] = cell_group_end(A, cs[d], ge[d][g[d]]);
        }
        if (d == D) break;
    }
    return cnt;
}

// The level groups of row i's 1D row along dimension d (its nesting entries
// grouped by level: [gs, ge) entries of level gl), ng[d] of them.
__device__ void row_groups(const TransArgs& A, int64_t i, int d, int (*gs)[kTLev], int (*ge)[kTLev],
                           int (*gl)[kTLev], int* ng) {
    const int D = A.D, k = A.k;
    int lo = 0, hi = A.nlev - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.lev_off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    const int8_t* Li = A.levels + (size_t)lo * D;
    int64_t cl = (i - A.lev_off[lo]) / A.kD, ml = (i - A.lev_off[lo]) % A.kD;
    int64_t i1 = 0;
    for (int q = 0; q <= d; q++) {
        const int L = Li[q];
        const int64_t nc = (int64_t)1 << (L > 2 ? L - 2 : 0);
        const int64_t c = cl % nc, m = ml % k;
        cl /= nc;
        ml /= k;
        i1 = k * ((L >= 2 ? ((int64_t)1 << (L - 2)) : 0) + c) + m;
    }
    const int a = (int)A.rp1[i1], b = (int)A.rp1[i1 + 1];  // 1D transforms hold < 2^31 entries
    int n = 0, last = -1;
    for (int e = a; e < b; e++) {
        int L, c, m;
        dec1d(k, A.col1[e], L, c, m);
        if (L != last) {
            gs[d][n] = e;
            gl[d][n] = L;
            if (n > 0) ge[d][n - 1] = e;
            n++;
            last = L;
        }
    }
    if (n > 0) ge[d][n - 1] = b;
    ng[d] = n;
}

// One warp per row.  The row's level tuples (dimension 0 fastest, the order
// of the global index) are taken 32 at a time, one per lane; a warp scan of
// the lanes' entry counts places each lane's entries, so rounds and lanes
// write the row in order.  Row lengths differ by four orders of magnitude (a
// coarse modal row of n2m spans the whole grid): rows of kTLongTuples level
// tuples or more are left to k_transform_long.  The level groups of the
// row's 1D rows (one lane per dimension builds them) live in shared memory,
// one copy per warp.
template <bool FILL>
__global__ void __launch_bounds__(32 * kTRowsPerBlock)
    k_transform(TransArgs A, int32_t* rowlen, const int64_t* __restrict__ rowptr, int32_t* __restrict__ col,
                double* __restrict__ val) {
    __shared__ int s_grp[kTRowsPerBlock][3][8][kTLev];  // per warp: gs, ge, gl
    __shared__ int s_ng[kTRowsPerBlock][8];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t i = (int64_t)blockIdx.x * kTRowsPerBlock + wib;
    if (i >= A.N) return;  // the whole warp
    const int D = A.D;
    int(*gs)[kTLev] = s_grp[wib][0];
    int(*ge)[kTLev] = s_grp[wib][1];
    int(*gl)[kTLev] = s_grp[wib][2];
    int* ng = s_ng[wib];
    if (lane < D) row_groups(A, i, lane, gs, ge, gl, ng);
    __syncwarp();
    int64_t ntup = 1;
    for (int d = 0; d < D; d++) ntup *= ng[d];
    // an empty 1D row: no entries in row i; a long row: k_transform_long,
    // launched after this kernel for the rows the host listed, overwrites the
    // -1 (every row's count is written here, and a long row the host did not
    // list keeps -1, which the row-pointer scan rejects)
    if (ntup == 0 || ntup >= kTLongTuples) {
        if (!FILL && lane == 0) rowlen[i] = ntup == 0 ? 0 : -1;
        return;  // the whole warp
    }
    int64_t w = FILL ? rowptr[i] : 0;
    const int64_t lim = FILL ? rowptr[i + 1] : 0;
    for (int64_t t0 = 0; t0 < ntup; t0 += 32) {
        const int64_t t = t0 + lane;
        int g[8];
        int32_t c = 0;
        if (t < ntup) {
            int64_t r = t;
            for (int d = 0; d < D; d++) {
                g[d] = (int)(r % ng[d]);
                r /= ng[d];
            }
            c = tuple_entries<false>(A, g, gs, ge, gl, 0, 0, nullptr, nullptr);
        }
        int32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int32_t rsum = __shfl_sync(0xffffffffu, incl, 31);
        if (FILL && c > 0) tuple_entries<true>(A, g, gs, ge, gl, w + incl - c, lim, col, val);
        w += rsum;
    }
    if (!FILL && lane == 0) rowlen[i] = (int32_t)w;
}

// The rows with kTLongTuples level tuples or more, one block of
// kTLongThreads per row: the same walk as k_transform with the tuples taken
// kTLongThreads at a time and a block scan of the counts.
template <bool FILL>
__global__ void __launch_bounds__(kTLongThreads)
    k_transform_long(TransArgs A, const int32_t* __restrict__ rows, int32_t* rowlen,
                     const int64_t* __restrict__ rowptr, int32_t* __restrict__ col, double* __restrict__ val) {
    __shared__ int s_grp[3][8][kTLev];
    __shared__ int s_ng[8];
    __shared__ int32_t s_warp[kTLongThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t i = rows[blockIdx.x];
    const int D = A.D;
    int(*gs)[kTLev] = s_grp[0];
    int(*ge)[kTLev] = s_grp[1];
    int(*gl)[kTLev] = s_grp[2];
    if (tid < D) row_groups(A, i, tid, gs, ge, gl, s_ng);
    __syncthreads();
    int64_t ntup = 1;
    for (int d = 0; d < D; d++) ntup *= s_ng[d];
    int64_t w = FILL ? rowptr[i] : 0;
    const int64_t lim = FILL ? rowptr[i + 1] : 0;
    for (int64_t t0 = 0; t0 < ntup; t0 += kTLongThreads) {  // ntup is the same in every thread
        const int64_t t = t0 + tid;
        int g[8];
        int32_t c = 0;
        if (t < ntup) {
            int64_t r = t;
            for (int d = 0; d < D; d++) {
                g[d] = (int)(r % s_ng[d]);
                r /= s_ng[d];
            }
            c = tuple_entries<false>(A, g, gs, ge, gl, 0, 0, nullptr, nullptr);
        }
        int32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_warp[wid] = incl;
        __syncthreads();
        int32_t before = 0, total = 0;
        for (int q = 0; q < kTLongThreads / 32; q++) {
            const int32_t x = s_warp[q];
            if (q < wid) before += x;
            total += x;
        }
        if (FILL && c > 0) tuple_entries<true>(A, g, gs, ge, gl, w + before + incl - c, lim, col, val);
        w += total;
        __syncthreads();  // s_warp is rewritten next round
    }
    if (!FILL && tid == 0) rowlen[i] = (int32_t)w;
}

}  // namespace

std::unique_ptr<DeviceCSR> gpu_transform(const SparseIndex& ix, const CSR& T1, cudaStream_t st) {
    require_gpu();
    const int D = ix.D, k = ix.k, n = ix.n;
    if (n + 1 > kTLev) throw Error(SGDG_EUNSUPPORTED, "more than 16 levels per dimension");
    // 1D rows restricted to the index pairs whose cells nest (relevant_cell_1D)
    // support [c w, (c + 1) w) of the 1D index j1 (level L, 0-based cell c),
    // computed as transform_dd's nesting test computes it
    auto cellrange = [&](int j1, double& lo, double& hi) {
        const int blk = j1 / k;
        int L = 1;
        while (L < 32 && (blk >> (L - 1)) != 0) L++;
        const int c = L >= 2 ? blk - (1 << (L - 2)) : 0;
        const double w = 1.0 / (double)ncells(L);
        lo = c * w;
        hi = (c + 1) * w;
    };
    std::vector<int64_t> rp(T1.m + 1, 0);
    std::vector<int32_t> cl;
    std::vector<double> vl;
    std::vector<std::pair<int32_t, double>> row;
    for (int64_t r = 0; r < T1.m; r++) {
        double a1, b1;
        cellrange((int)r, a1, b1);
        row.clear();
        for (int64_t p = T1.rowptr[r]; p < T1.rowptr[r + 1]; p++) {
            double a2, b2;
            cellrange(T1.col[p], a2, b2);
            if ((a1 <= a2 && b1 >= b2) || (a1 >= a2 && b1 <= b2)) row.push_back({T1.col[p], T1.val[p]});
        }
        // the enumeration walks each row by level, cell and mode: columns ascending
        std::sort(row.begin(), row.end(), [](const std::pair<int32_t, double>& x, const std::pair<int32_t, double>& y) {
            return x.first < y.first;
        });
        for (auto& e : row) {
            cl.push_back(e.first);
            vl.push_back(e.second);
        }
        rp[r + 1] = (int64_t)cl.size();
    }
    std::vector<int8_t> lv(ix.levels.size());
    for (size_t q = 0; q < lv.size(); q++) lv[q] = (int8_t)ix.levels[q];
    std::vector<int32_t> lo(ix.lev_off.begin(), ix.lev_off.end());
    DevBuf d_lv = upload(lv, st), d_lo = upload(lo, st), d_code = upload(ix.code2lev, st), d_rp = upload(rp, st),
           d_cl = upload(cl, st), d_vl = upload(vl, st);
    TransArgs A{D, k, n, ix.scheme, ix.nlev, ix.N, ix.kD, d_lv.as<int8_t>(), d_lo.as<int32_t>(), d_code.as<int32_t>(),
                d_rp.as<int64_t>(), d_cl.as<int32_t>(), d_vl.as<double>()};
    // rows with kTLongTuples level tuples or more (the product over the
    // dimensions of the levels present in each 1D row, as the kernels count
    // them) go to k_transform_long
    std::vector<int> nlev1(T1.m, 0);
    for (int64_t r = 0; r < T1.m; r++) {
        int last = -1;
        for (int64_t p = rp[r]; p < rp[r + 1]; p++) {
            const int blk = cl[p] / k;
            int L = 1;
            while (L < 32 && (blk >> (L - 1)) != 0) L++;
            if (L != last) nlev1[r]++;
            last = L;
        }
    }
    std::vector<int32_t> long_rows;
    for (int b = 0; b < ix.nlev; b++) {
        const int* L = &ix.levels[(size_t)b * D];
        int64_t nc[8], cells = 1;
        for (int d = 0; d < D; d++) {
            nc[d] = ncells(L[d]);
            cells *= nc[d];
        }
        for (int64_t c = 0; c < cells; c++)
            for (int64_t m = 0; m < ix.kD; m++) {
                int64_t cr = c, mr = m, ntup = 1;
                for (int d = 0; d < D; d++) {
                    const int64_t i1 = k * ((L[d] >= 2 ? ((int64_t)1 << (L[d] - 2)) : 0) + cr % nc[d]) + mr % k;
                    cr /= nc[d];
                    mr /= k;
                    ntup *= nlev1[(size_t)i1];
                }
                if (ntup >= kTLongTuples) long_rows.push_back((int32_t)(ix.lev_off[b] + c * ix.kD + m));
            }
    }
    DevBuf d_long = upload(long_rows, st);
    const int nlong = (int)long_rows.size();
    DevBuf rowlen(sizeof(int32_t) * (size_t)ix.N);
    const int tgrid = (int)((ix.N + kTRowsPerBlock - 1) / kTRowsPerBlock);
    k_transform<false><<<tgrid, 32 * kTRowsPerBlock, 0, st>>>(A, rowlen.as<int32_t>(), nullptr, nullptr, nullptr);
    CK(cudaGetLastError());
    if (nlong > 0) {
        k_transform_long<false><<<nlong, kTLongThreads, 0, st>>>(A, d_long.as<int32_t>(), rowlen.as<int32_t>(), nullptr,
                                                                 nullptr, nullptr);
        CK(cudaGetLastError());
    }
    std::vector<int64_t> rph = scan_rows(rowlen, ix.N, st);
    auto R = std::make_unique<DeviceCSR>();
    R->rowptr = upload(rph, st);
    R->col.alloc(sizeof(int32_t) * (size_t)rph[ix.N]);
    R->val.alloc(sizeof(double) * (size_t)rph[ix.N]);
    k_transform<true><<<tgrid, 32 * kTRowsPerBlock, 0, st>>>(A, nullptr, R->rowptr.as<int64_t>(),
                                                              R->col.as<int32_t>(), R->val.as<double>());
    CK(cudaGetLastError());
    if (nlong > 0) {
        k_transform_long<true><<<nlong, kTLongThreads, 0, st>>>(A, d_long.as<int32_t>(), nullptr,
                                                                R->rowptr.as<int64_t>(), R->col.as<int32_t>(),
                                                                R->val.as<double>());
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(st));
    finish_device_csr(*R, rph, ix.N, st, kCsrLaneEntriesMulti);  // the transforms take four vectors a pass
    return R;
}

SGDG_BOUNDS_READER(asm_bounds_violations)

std::unique_ptr<DeviceCSR> gpu_operator(const SparseIndex& ix, const DLF1D& dlf, int which, cudaStream_t st,
                                        int per_lane) {
    require_gpu();
    const int D = ix.D;
    std::vector<int64_t> rp;
    if (which >= 1 && which <= D) {
        const LineTables T = line_tables(dlf, dlf.n + 1, false);
        auto A = line_operator(ix, T, which - 1, st, rp);
        finish_device_csr(*A, rp, ix.N, st, per_lane);
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
