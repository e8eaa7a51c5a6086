// dlf1d.cpp -- the 1D hierarchical periodic DG derivative with central flux.
//
// Built by the reference's own route, step by step in its arithmetic order,
// so that the stored pattern and the values are the ones the reference's
// sparse algebra produces:
//   Q  = hier2pos(k, n)                      src/1d_dg_functions.jl:242-263
//   A  = (-D_matrix(k, n) + periodic_LF_matrix(k, n))'
//                                            src/1d_derivative.jl:21-111
//   op = Q' * (A * Q)                        src/1d_derivative.jl:113-117
// The sums of the derivative matrix keep exactly the entries whose floating-
// point sums do not cancel to 0.0 (SparseArrays' map(+) drops exact zeros),
// and which sums cancel depends on every rounding before them; so the basis
// evaluation (Horner on the x^i / sgn(x) x^i coefficient pairs), the cell-edge
// evaluation at +-5e-16, the SpGEMM accumulation order (terms in increasing
// inner index, the first one assigned) and the exact-zero drops all follow
// the reference.  hquadrature (HCubature 1.4.0, atol 1e-12) integrates
// piecewise polynomials of degree <= 2k-2 here; it is restated as a 16-point
// Gauss-Legendre rule per finest cell, exact for these integrands.
//
// The result is block-dense: one full k x k block for every pair of (level,
// cell) blocks whose closed supports meet periodically (numerical zeros
// included); build_dlf checks that and stores it block by block.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>

#include "sgdg_core.h"

namespace sgdg {
namespace {

constexpr double kEdge = 5.0e-16;  // src/1d_derivative.jl:56
constexpr int kLegHalf = kKMax + 1;  // leg_coeffs vectors hold 2 (K_max + 1) numbers

// Gauss-Legendre nodes and weights on [-1, 1]: Newton's method on the
// three-term recurrence from the Chebyshev-like guess, stopping once a step
// moves the node by less than 1e-16.
void gauss_legendre(int q, std::vector<double>& x, std::vector<double>& w) {
    x.assign(q, 0.0);
    w.assign(q, 0.0);
    for (int i = 0; i < (q + 1) / 2; i++) {
        double z = std::cos(M_PI * (i + 0.75) / (q + 0.5)), slope = 0.0;
        for (int it = 0; it < 100; it++) {
            double pj = 1.0, pjm1 = 0.0;
            for (int j = 1; j <= q; j++) {
                const double pjm2 = pjm1;
                pjm1 = pj;
                pj = ((2.0 * j - 1.0) * z * pjm1 - (j - 1.0) * pjm2) / j;
            }
            slope = q * (z * pj - pjm1) / (z * z - 1.0);
            const double prev = z;
            z = prev - pj / slope;
            if (std::fabs(z - prev) < 1e-16) break;
        }
        x[i] = -z;
        x[q - 1 - i] = z;
        w[i] = w[q - 1 - i] = 2.0 / ((1.0 - z * z) * slope * slope);
    }
}

// array2poly (src/1d_dg_functions.jl:15-27): coefficients of x^i (first half)
// and sgn(x) x^i (second half) of a polynomial piece on [-1, 1], zero outside
double array2poly(const double* c, int half, double x) {
    if (std::fabs(x) > 1) return 0.0;
    double s = 0.0;
    for (int i = half - 1; i >= 0; i--) {
        s = s * x;
        s = s + (c[i] + (std::signbit(x) ? -c[i + half] : c[i + half]));
    }
    return s;
}

// product_matrix (src/dg_basis.jl:21-35): <x^i, x^j> on [-1, 1] with the
// reflected halves, exact rationals evaluated in floating point
int sign_pow(int e) { return e % 2 == 0 ? 1 : -1; }
double product_matrix(int i, int j, int n) {
    const int h = n / 2;
    if (i < h && j < h) return (double)(1 + sign_pow(i + j)) / (double)(1 + i + j);
    if (i >= h && j < h) return (double)(1 - sign_pow((i - h) + j)) / (double)(1 + (i - h) + j);
    if (i < h && j >= h) return product_matrix(j, i, n);
    return (double)(1 + sign_pow((i - h) + (j - h))) / (double)(1 + (i - h) + (j - h));
}

// inner_product (src/dg_basis.jl:37-50)
double inner_product(const double* a, const double* b, int n) {
    double value = 0.0;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            if (a[i] == 0 || b[j] == 0) continue;
            value += product_matrix(i, j, n) * a[i] * b[j];
        }
    return value;
}

// The reference's basis functions on [0, 1] from the coefficient arrays.
struct RefBasis {
    int k = 0;
    std::vector<double> leg;  // (K_max + 1) arrays of 2 (K_max + 1): normalised Legendre P_m
    const double* dg = nullptr;  // k arrays of 2k: the multiwavelets h_mode

    explicit RefBasis(int k_) : k(k_) {
        const Basis1D& B = basis(k_);
        dg = B.dg.data();
        leg.assign((size_t)(kKMax + 1) * 2 * kLegHalf, 0.0);
        for (int m = 0; m <= kKMax; m++)
            for (int t = 0; t <= kKMax; t++) leg[(size_t)m * 2 * kLegHalf + t] = B.leg[(size_t)m * (kKMax + 1) + t];
    }
    const double* legendre(int m) const { return &leg[(size_t)m * 2 * kLegHalf]; }
    // LegendreP (src/1d_dg_functions.jl:34-44)
    double P(int m, double x) const { return array2poly(legendre(m), kLegHalf, x); }
    // v (src/dg_methods.jl:27-36): hierarchical function of 0-based level
    double v(int level, int cell, int mode, double x) const {
        if (level == 0) return P(mode - 1, 2 * x - 1) * std::sqrt(2.0);
        return array2poly(dg + (size_t)(mode - 1) * 2 * k, k, (double)(int64_t(1) << level) * x - (double)(2 * cell - 1)) *
               std::sqrt(1.0 * (double)(int64_t(1) << level));
    }
    // leg and basis (src/1d_dg_functions.jl:83-97): position basis of a level
    double leg01(int mode, double x) const { return std::sqrt(2.0) * P(mode - 1, 2 * x - 1); }
    double pos(int level, int cell, int mode, double x) const {
        return leg01(mode, (double)(int64_t(1) << level) * x - (double)(cell - 1)) * std::pow(2.0, (double)level / 2.0);
    }
};

// Row-compressed sparse matrix for the reference's sparse algebra.  Rows
// are kept sorted; "sum" steps drop results that are exactly 0.0.
struct Sp {
    int64_t m = 0, n = 0;
    std::vector<int64_t> rp;
    std::vector<int32_t> ci;
    std::vector<double> v;
    explicit Sp(int64_t m_ = 0, int64_t n_ = 0) : m(m_), n(n_), rp(m_ + 1, 0) {}
    void push(int32_t c, double x) {
        ci.push_back(c);
        v.push_back(x);
    }
    void end_row(int64_t r) { rp[r + 1] = (int64_t)ci.size(); }
};

Sp transpose(const Sp& A) {
    Sp T(A.n, A.m);
    std::vector<int64_t> cnt(A.n + 1, 0);
    for (int32_t c : A.ci) cnt[c + 1]++;
    for (int64_t c = 0; c < A.n; c++) cnt[c + 1] += cnt[c];
    T.rp = cnt;
    T.ci.resize(A.ci.size());
    T.v.resize(A.v.size());
    for (int64_t r = 0; r < A.m; r++)
        for (int64_t p = A.rp[r]; p < A.rp[r + 1]; p++) {
            const int64_t q = cnt[A.ci[p]]++;
            T.ci[q] = (int32_t)r;
            T.v[q] = A.v[p];
        }
    return T;
}

// A * B, Gustavson by rows: C[r, c] accumulates A[r, j] * B[j, c] over the
// stored j of row r in increasing order, the first product assigned (the
// order of SparseArrays' column-by-column spmatmul); structural zeros kept.
Sp spgemm(const Sp& A, const Sp& B) {
    Sp C(A.m, B.n);
    std::vector<int64_t> mark(B.n, -1);
    std::vector<double> acc(B.n, 0.0);
    std::vector<int32_t> cols;
    for (int64_t r = 0; r < A.m; r++) {
        cols.clear();
        for (int64_t p = A.rp[r]; p < A.rp[r + 1]; p++) {
            const int32_t j = A.ci[p];
            const double a = A.v[p];
            for (int64_t q = B.rp[j]; q < B.rp[j + 1]; q++) {
                const int32_t c = B.ci[q];
                if (mark[c] != r) {
                    mark[c] = r;
                    acc[c] = a * B.v[q];
                    cols.push_back(c);
                } else {
                    acc[c] += a * B.v[q];
                }
            }
        }
        std::sort(cols.begin(), cols.end());
        for (int32_t c : cols) C.push(c, acc[c]);
        C.end_row(r);
    }
    return C;
}

// -A + B over the union of the patterns, results that are exactly zero dropped
// (SparseArrays' unary minus, then map(+); a missing operand is 0.0)
Sp neg_plus(const Sp& A, const Sp& B) {
    Sp C(A.m, A.n);
    for (int64_t r = 0; r < A.m; r++) {
        int64_t a = A.rp[r], b = B.rp[r];
        const int64_t ae = A.rp[r + 1], be = B.rp[r + 1];
        while (a < ae || b < be) {
            const int32_t ca = a < ae ? A.ci[a] : INT32_MAX, cb = b < be ? B.ci[b] : INT32_MAX;
            double x;
            int32_t c;
            if (ca == cb) {
                x = -1.0 * A.v[a++] + 1.0 * B.v[b++];
                c = ca;
            } else if (ca < cb) {
                x = -1.0 * A.v[a++] + 0.0;
                c = ca;
            } else {
                x = 0.0 + 1.0 * B.v[b++];
                c = cb;
            }
            if (x != 0) C.push(c, x);
        }
        C.end_row(r);
    }
    return C;
}

// hier2pos (src/1d_dg_functions.jl:242-263): Q[pos(cell, p), hier(level, cell', mode)]
// = <v_hier, basis_pos> over each finest cell, kept when |value| > 1e-12.
// Cells outside a hierarchical function's support contribute exact zeros
// (the function is 0.0 at every node there) and are not visited.
Sp hier2pos(const RefBasis& B, int n) {
    const int k = B.k;
    const int64_t len = (int64_t)k << n;
    std::vector<double> gx, gw;
    gauss_legendre(16, gx, gw);
    const double hcell = 1.0 / (double)(int64_t(1) << n);
    Sp Qt(len, len);  // built by hierarchical column, transposed at the end
    int64_t j = 0;
    for (int level = 0; level <= n; level++) {
        const int ncell = 1 << (level > 1 ? level - 1 : 0);
        for (int cell = 1; cell <= ncell; cell++)
            for (int mode = 1; mode <= k; mode++) {
                const int span = level == 0 ? 1 << n : 1 << (n - level + 1);
                const int i0 = level == 0 ? 1 : (cell - 1) * span + 1;
                for (int i = i0; i < i0 + span; i++) {
                    const double a = (double)(i - 1) * hcell, b = (double)i * hcell;
                    for (int p = 1; p <= k; p++) {
                        double s = 0.0;
                        for (int t = 0; t < 16; t++) {
                            const double x = 0.5 * (a + b) + 0.5 * (b - a) * gx[t];
                            s += gw[t] * B.v(level, cell, mode, x) * B.pos(n, i, p, x);
                        }
                        s *= 0.5 * (b - a);
                        if (std::fabs(s) > 1e-12) Qt.push((int32_t)((int64_t)(i - 1) * k + (p - 1)), s);
                    }
                }
                Qt.end_row(j);
                j++;
            }
    }
    return transpose(Qt);
}

// symbolic_diff (src/derivative_matrix_elements.jl:80-94) and
// legendreDlegendre (src/derivative_matrix_elements.jl:101-103)
double legendre_d_legendre(const RefBasis& B, int m1, int m2) {
    const int n = 2 * kLegHalf, h = kLegHalf;
    const double* v = B.legendre(m2 - 1);
    std::vector<double> d(n, 0.0);
    for (int i = 1; i <= n; i++) {
        if (i < h)
            d[i - 1] = (double)i * v[i];
        else if (i > h && i < 2 * h)
            d[i - 1] = (double)(i - h) * v[i];
    }
    return inner_product(B.legendre(m1 - 1), d.data(), n);
}

// D_matrix(k, level) (src/1d_derivative.jl:21-44, legvDv at
// src/derivative_matrix_elements.jl:106-112): cell-diagonal, |val| > 1e-15
Sp pos_derivative(const RefBasis& B, int level) {
    const int k = B.k, ncell = 1 << level;
    Sp D((int64_t)k << level, (int64_t)k << level);
    std::vector<double> lDl((size_t)k * k);
    for (int m1 = 1; m1 <= k; m1++)
        for (int m2 = 1; m2 <= k; m2++) lDl[(m1 - 1) * k + (m2 - 1)] = legendre_d_legendre(B, m1, m2);
    for (int cell = 1; cell <= ncell; cell++)
        for (int m1 = 1; m1 <= k; m1++) {
            for (int m2 = 1; m2 <= k; m2++) {
                const double val = (double)(int64_t(1) << (level + 1)) * lDl[(m1 - 1) * k + (m2 - 1)];
                if (std::fabs(val) > 1.0e-15) D.push((int32_t)((cell - 1) * k + (m2 - 1)), val);
            }
            D.end_row((int64_t)(cell - 1) * k + (m1 - 1));
        }
    return D;
}

// periodic_legvLFv (src/1d_derivative.jl:52-74, alpha = 0)
double periodic_lf_entry(const RefBasis& B, int level, int cell1, int mode1, int cell2, int mode2) {
    const double N = (double)(int64_t(1) << level);
    const double point1 = (double)(cell2 - 1) / N, point2 = (double)cell2 / N;
    double left1 = B.pos(level, cell1, mode1, point1 - kEdge);
    const double right1 = B.pos(level, cell1, mode1, point1 + kEdge);
    const double left2 = B.pos(level, cell1, mode1, point2 - kEdge);
    double right2 = B.pos(level, cell1, mode1, point2 + kEdge);
    if (cell2 == (1 << level)) right2 = B.pos(level, cell1, mode1, 0.0 + kEdge);
    if (cell2 == 1) left1 = B.pos(level, cell1, mode1, 1.0 - kEdge);
    const double LF1 = 0.5 * (left1 + right1) + 0.0 * (right1 - left1);
    const double LF2 = 0.5 * (left2 + right2) + 0.0 * (right2 - left2);
    const double val1 = B.pos(level, cell2, mode2, point1 + kEdge);
    const double val2 = B.pos(level, cell2, mode2, point2 - kEdge);
    return LF2 * val2 - LF1 * val1;
}

// periodic_LF_matrix (src/1d_derivative.jl:76-100), |val| > 1e-15.  The
// flux couples a cell only to itself and its periodic neighbours (basis()
// is 0.0 at every evaluation point of any other pair), so only those pairs
// are evaluated.
Sp periodic_lf(const RefBasis& B, int level) {
    const int k = B.k, ncell = 1 << level;
    Sp L((int64_t)k << level, (int64_t)k << level);
    for (int cell1 = 1; cell1 <= ncell; cell1++)
        for (int mode1 = 1; mode1 <= k; mode1++) {
            for (int cell2 = 1; cell2 <= ncell; cell2++) {
                const int dc = (cell2 - cell1 + ncell) % ncell;
                if (!(dc == 0 || dc == 1 || dc == ncell - 1)) continue;
                for (int mode2 = 1; mode2 <= k; mode2++) {
                    const double val = periodic_lf_entry(B, level, cell1, mode1, cell2, mode2);
                    if (std::fabs(val) > 1.0e-15) L.push((int32_t)((cell2 - 1) * k + (mode2 - 1)), val);
                }
            }
            L.end_row((int64_t)(cell1 - 1) * k + (mode1 - 1));
        }
    return L;
}

}  // namespace

static DLF1D build_dlf(int k, int n) {
    if (n < 2) throw Error(1, "n must be >= 2 (with <= 2 finest cells the reference's periodic fluxes cancel)");
    if (n > 20) throw Error(1, "n too large");
    const RefBasis B(k);
    const Sp Q = hier2pos(B, n);
    const Sp A = transpose(neg_plus(pos_derivative(B, n), periodic_lf(B, n)));  // periodic_pos_DLF_matrix
    const Sp R = spgemm(transpose(Q), spgemm(A, Q));                              // periodic_hier_DLF_matrix
    DLF1D op;
    op.k = k;
    op.n = n;
    op.nblocks = 1 << n;
    for (int L = 1; L <= n + 1; L++)
        for (int c = 1; c <= ncells(L); c++) {
            op.blk_level.push_back(L);
            op.blk_cell.push_back(c);
        }
    // block-CSR over (level, cell) blocks: every row of a row block must
    // list the same column blocks with all k modes
    op.rowptr.assign(op.nblocks + 1, 0);
    for (int rb = 0; rb < op.nblocks; rb++) {
        const int64_t r0 = (int64_t)rb * k;
        const int64_t len = R.rp[r0 + 1] - R.rp[r0];
        if (len % k != 0) throw Error(7, "1D operator: a row is not block-dense");
        const size_t first = op.val.size();
        op.val.resize(first + (size_t)(len / k) * k * k);
        for (int64_t b = 0; b < len / k; b++) op.colblk.push_back(R.ci[R.rp[r0] + b * k] / k);
        for (int i = 0; i < k; i++) {
            const int64_t p0 = R.rp[r0 + i];
            if (R.rp[r0 + i + 1] - p0 != len) throw Error(7, "1D operator: a row block is not block-dense");
            for (int64_t t = 0; t < len; t++) {
                const int64_t b = t / k;
                const int32_t c = R.ci[p0 + t];
                if (c != op.colblk[op.colblk.size() - len / k + b] * k + (int32_t)(t % k))
                    throw Error(7, "1D operator: a row block is not block-dense");
                op.val[first + (size_t)b * k * k + (size_t)i * k + (size_t)(t % k)] = R.v[p0 + t];
            }
        }
        op.rowptr[rb + 1] = (int32_t)op.colblk.size();
    }
    return op;
}

static CSR to_csr(const Sp& A) {
    CSR C;
    C.m = A.m;
    C.n = A.n;
    C.rowptr = A.rp;
    C.col = A.ci;
    C.val = A.v;
    return C;
}

// The position-basis route of wave_evolve_1D (src/pdes.jl:89-121 with
// basis = "pos"): D_op = periodic_pos_DLF_matrix (src/1d_derivative.jl:108-111)
// and laplac = D_op * D_op, a SpGEMM that keeps its structural zeros.
void pos_operators(int k, int n, CSR* dop, CSR* lap) {
    if (n < 2) throw Error(1, "n must be >= 2 (with <= 2 finest cells the reference's periodic fluxes cancel)");
    if (n > 20) throw Error(1, "n too large");
    basis(k);  // validates k
    const RefBasis B(k);
    const Sp A = transpose(neg_plus(pos_derivative(B, n), periodic_lf(B, n)));
    if (lap) *lap = to_csr(spgemm(A, A));
    if (dop) *dop = to_csr(A);
}

std::shared_ptr<const DLF1D> dlf1d(int k, int n) {
    static std::mutex mu;
    static std::map<std::pair<int, int>, std::shared_ptr<const DLF1D>> cache;
    basis(k);  // validates k
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find({k, n});
        if (it != cache.end()) return it->second;
    }
    auto op = std::make_shared<const DLF1D>(build_dlf(k, n));
    std::lock_guard<std::mutex> g(mu);
    cache[{k, n}] = op;
    return op;
}

}  // namespace sgdg

namespace sgdg {

// Block table of a 1D operator in block-CSR form (k x k blocks over the 2^n
// (level, cell) blocks): blocks whose entries are all below prune * (largest
// entry) are dropped, and blocks equal to 1e-12 of the largest entry share
// one table entry (they are the same block up to the roundoff of their
// separate evaluation).
static MFOperator mf_table(int k, int n, int nblocks, const std::vector<int32_t>& rowptr,
                           const std::vector<int32_t>& colblk, const std::vector<double>& val, double prune) {
    MFOperator M;
    M.k = k;
    M.n = n;
    M.rs = ((2 * k + 3) / 4) * 4;
    double vmax = 0.0;
    for (double v : val) vmax = std::max(vmax, std::fabs(v));
    const double drop = prune * vmax;
    std::map<std::vector<long long>, int> ids;
    M.rowptr.assign(nblocks + 1, 0);
    for (int rb = 0; rb < nblocks; rb++) {
        for (int p = rowptr[rb]; p < rowptr[rb + 1]; p++) {
            const double* b = &val[(size_t)p * k * k];
            double bmax = 0.0;
            for (int t = 0; t < k * k; t++) bmax = std::max(bmax, std::fabs(b[t]));
            if (bmax <= drop) continue;
            std::vector<long long> key(k * k);
            for (int t = 0; t < k * k; t++) key[t] = std::llround(b[t] / vmax * 1e12);
            auto it = ids.find(key);
            int id;
            if (it == ids.end()) {
                id = M.ndist++;
                ids.emplace(std::move(key), id);
                const size_t base = M.val.size();
                M.val.resize(base + (size_t)k * M.rs, 0.f);
                for (int i = 0; i < k; i++)
                    for (int j = 0; j < k; j++) {
                        const double x = b[i * k + j];
                        const float hi = (float)x;
                        M.val[base + (size_t)i * M.rs + 2 * j] = hi;
                        M.val[base + (size_t)i * M.rs + 2 * j + 1] = (float)(x - (double)hi);
                    }
            } else {
                id = it->second;
            }
            if (id >= 4096 || colblk[p] >= (1 << 19))
                throw Error(7, "1D operator too large for the matrix-free block table");
            M.ent.push_back((colblk[p] << 12) | id);
        }
        M.rowptr[rb + 1] = (int32_t)M.ent.size();
    }
    return M;
}

MFOperator mf_operator(int k, int n) {
    auto op = dlf1d(k, n);
    // the vanishing moments make fine x coarse blocks away from the coarse
    // function's breakpoints exact zeros, stored as roundoff (<= 1e-14 of the
    // largest entry; genuine entries are >= 7e-3 of it)
    return mf_table(k, n, op->nblocks, op->rowptr, op->colblk, op->val, 1e-10);
}

// The wave applies D_d D_d; on a pencil's line D_d is the leading block B of
// the 1D operator for the line length lm, so D_d D_d is B B there (not the
// leading block of the squared operator: the inner sum stops at the line's
// finest level).  B B has the block pattern of B once blocks at roundoff are
// dropped (a fine/coarse pair meets only at the coarse function's breaks,
// as for B), so one sweep of B B costs half of two sweeps of B.  The table
// holds B B of the pruned B for every lm = 1..n+1, in FP64 before the hi/lo
// split; blocks below 1e-10 of the largest entry of their lm are dropped.
MFSquareTables mf_square_tables(int k, int n) {
    auto op = dlf1d(k, n);
    double vmax = 0.0;
    for (double v : op->val) vmax = std::max(vmax, std::fabs(v));
    // the pruned blocks of the 1D operator, by row block
    const int nb = op->nblocks, kk = k * k;
    std::vector<std::vector<std::pair<int, const double*>>> rows(nb);
    for (int rb = 0; rb < nb; rb++)
        for (int p = op->rowptr[rb]; p < op->rowptr[rb + 1]; p++) {
            const double* b = &op->val[(size_t)p * kk];
            double bmax = 0.0;
            for (int t = 0; t < kk; t++) bmax = std::max(bmax, std::fabs(b[t]));
            if (bmax > 1e-10 * vmax) rows[rb].push_back({op->colblk[p], b});
        }
    MFSquareTables Q;
    Q.k = k;
    Q.n = n;
    Q.rs = ((2 * k + 3) / 4) * 4;
    std::map<std::vector<long long>, int> ids;
    for (int lm = 1; lm <= n + 1; lm++) {
        const int nrb = 1 << (lm - 1);
        std::vector<std::map<int, std::vector<double>>> sq(nrb);
        double smax = 0.0;
        for (int rb = 0; rb < nrb; rb++) {
            for (const auto& pb : rows[rb]) {
                if (pb.first >= nrb) continue;
                for (const auto& cb : rows[pb.first]) {
                    if (cb.first >= nrb) continue;
                    std::vector<double>& acc = sq[rb][cb.first];
                    if (acc.empty()) acc.assign(kk, 0.0);
                    for (int i = 0; i < k; i++)
                        for (int j = 0; j < k; j++) {
                            double t = 0.0;
                            for (int q = 0; q < k; q++) t += pb.second[i * k + q] * cb.second[q * k + j];
                            acc[i * k + j] += t;
                        }
                }
            }
            for (auto& e : sq[rb])
                for (double v : e.second) smax = std::max(smax, std::fabs(v));
        }
        Q.roff.push_back((int32_t)Q.rowptr.size());
        Q.rowptr.push_back((int32_t)Q.ent.size());
        for (int rb = 0; rb < nrb; rb++) {
            for (auto& e : sq[rb]) {
                const std::vector<double>& b = e.second;
                double bmax = 0.0;
                for (double v : b) bmax = std::max(bmax, std::fabs(v));
                if (bmax <= 1e-10 * smax) continue;
                std::vector<long long> key(kk);
                for (int t = 0; t < kk; t++) key[t] = std::llround(b[t] / smax * 1e12);
                key.push_back(lm);  // values are compared within one line length's scale
                auto it = ids.find(key);
                int id;
                if (it == ids.end()) {
                    id = Q.ndist++;
                    ids.emplace(std::move(key), id);
                    const size_t base = Q.val.size();
                    Q.val.resize(base + (size_t)k * Q.rs, 0.f);
                    for (int i = 0; i < k; i++)
                        for (int j = 0; j < k; j++) {
                            const double x = b[i * k + j];
                            const float hi = (float)x;
                            Q.val[base + (size_t)i * Q.rs + 2 * j] = hi;
                            Q.val[base + (size_t)i * Q.rs + 2 * j + 1] = (float)(x - (double)hi);
                        }
                } else {
                    id = it->second;
                }
                if (id >= 4096 || e.first >= (1 << 19))
                    throw Error(7, "squared line operators too large for the matrix-free block table");
                Q.ent.push_back((e.first << 12) | id);
            }
            Q.rowptr.push_back((int32_t)Q.ent.size());
        }
    }
    return Q;
}

MFOperator mf_transform_table(int k, int n, int which) {
    // element CSR of the 1D map -> dense k x k blocks per (level, cell) pair
    const CSR T = transform_1d(k, n, which);
    const int nb = 1 << n;
    std::vector<int32_t> rowptr(nb + 1, 0), colblk;
    std::vector<double> val;
    for (int rb = 0; rb < nb; rb++) {
        std::map<int, std::vector<double>> blocks;  // column block -> k x k
        for (int i = 0; i < k; i++) {
            const int64_t row = (int64_t)rb * k + i;
            for (int64_t p = T.rowptr[row]; p < T.rowptr[row + 1]; p++) {
                const int cb = T.col[p] / k, j = T.col[p] % k;
                auto& bl = blocks[cb];
                if (bl.empty()) bl.assign((size_t)k * k, 0.0);
                bl[(size_t)i * k + j] = T.val[p];
            }
        }
        for (auto& e : blocks) {
            colblk.push_back(e.first);
            val.insert(val.end(), e.second.begin(), e.second.end());
        }
        rowptr[rb + 1] = (int32_t)colblk.size();
    }
    return mf_table(k, n, nb, rowptr, colblk, val, 0.0);
}

}  // namespace sgdg
