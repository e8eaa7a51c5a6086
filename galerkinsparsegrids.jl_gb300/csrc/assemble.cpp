// assemble.cpp -- assembled (plain-form) operators in CSR.
//
// D_d follows src/multidim_derivative.jl:19-58: the entry (i, j) exists when
// i and j agree in every dimension but d and their dim-d triples are a stored
// pair of the 1D operator, and row i's level tuple is not cut; its value is
// the 1D entry.  Rows are produced directly (CSR) with columns sorted, which is
// the transpose-order of the reference's CSC build and yields the same set of
// stored entries (numerical zeros included).
//
// Products keep their structural pattern (SparseArrays' spmatmul stores every
// structural entry).  Sums follow SparseArrays' map(+): an entry present in
// only one operand is added to 0.0, and every result that is exactly 0.0 is
// dropped -- the reference's laplacian_matrix (src/multidim_derivative.jl:
// 71-79) and the advection sum of the D_d lose the entries whose products
// cancel exactly.  The 1D operator is built by the reference's route
// (dlf1d.cpp), so the same sums cancel here.
#include <algorithm>
#include <cstring>

#include "sgdg_core.h"

namespace sgdg {

CSR assemble_dd(const SparseIndex& ix, const DLF1D& op, int d) {
    const int D = ix.D, k = ix.k;
    if (d < 0 || d >= D) throw Error(1, "dimension out of range");
    CSR A;
    A.m = A.n = ix.N;
    A.rowptr.assign(ix.N + 1, 0);
    // pass 1: row lengths
    int L2[kDMax];
    auto blk1d = [&](int L, int c) { return (L >= 2 ? (1 << (L - 2)) : 0) + (c - 1); };
    // per level block: number of admissible column blocks per 1D row block
    std::vector<int64_t> rowlen(ix.N);
    for (int b = 0; b < ix.nlev; b++) {
        const int* L = &ix.levels[(size_t)b * D];
        int64_t nc[kDMax], P[kDMax];
        int64_t s = 1;
        for (int q = 0; q < D; q++) {
            nc[q] = ncells(L[q]);
            P[q] = s;
            s *= nc[q];
        }
        for (int q = 0; q < D; q++) L2[q] = L[q];
        for (int64_t cl = 0; cl < ix.lev_cells[b]; cl++) {
            int cd = int((cl / P[d]) % nc[d]) + 1;
            int rb = blk1d(L[d], cd);
            int64_t cnt = 0;
            for (int p = op.rowptr[rb]; p < op.rowptr[rb + 1]; p++) {
                L2[d] = op.blk_level[op.colblk[p]];
                if (!ix.cut(L2)) cnt += k;
            }
            int64_t base = ix.lev_off[b] + cl * ix.kD;
            for (int64_t ml = 0; ml < ix.kD; ml++) rowlen[base + ml] = cnt;
        }
    }
    for (int64_t i = 0; i < ix.N; i++) A.rowptr[i + 1] = A.rowptr[i] + rowlen[i];
    rowlen.clear();
    rowlen.shrink_to_fit();
    A.col.resize(A.nnz());
    A.val.resize(A.nnz());
    int64_t kd1 = 1;
    for (int q = 0; q < d; q++) kd1 *= k;
    for (int b = 0; b < ix.nlev; b++) {
        const int* L = &ix.levels[(size_t)b * D];
        int64_t nc[kDMax], P[kDMax];
        int64_t s = 1;
        for (int q = 0; q < D; q++) {
            nc[q] = ncells(L[q]);
            P[q] = s;
            s *= nc[q];
        }
        for (int q = 0; q < D; q++) L2[q] = L[q];
        for (int64_t cl = 0; cl < ix.lev_cells[b]; cl++) {
            int cd = int((cl / P[d]) % nc[d]) + 1;
            int rb = blk1d(L[d], cd);
            // split the cell index around dim d: cl = low + (cd-1)*P[d] + high*P[d]*nc[d]
            int64_t low = cl % P[d], high = cl / (P[d] * nc[d]);
            for (int64_t ml = 0; ml < ix.kD; ml++) {
                int64_t i = ix.lev_off[b] + cl * ix.kD + ml;
                int md = int((ml / kd1) % k);
                int64_t mlow = ml % kd1, mhigh = ml / (kd1 * k);
                int64_t w = A.rowptr[i];
                for (int p = op.rowptr[rb]; p < op.rowptr[rb + 1]; p++) {
                    int cb = op.colblk[p];
                    L2[d] = op.blk_level[cb];
                    if (ix.cut(L2)) continue;
                    int tb = ix.lookup_level(L2);
                    int64_t nc2 = ncells(L2[d]);
                    int64_t cl2 = low + int64_t(op.blk_cell[cb] - 1) * P[d] + high * P[d] * nc2;
                    int64_t jbase = ix.lev_off[tb] + cl2 * ix.kD + mlow + mhigh * kd1 * k;
                    const double* v = &op.val[(size_t)p * k * k + (size_t)md * k];
                    for (int mj = 0; mj < k; mj++) {
                        A.col[w] = int32_t(jbase + mj * kd1);
                        A.val[w] = v[mj];
                        w++;
                    }
                }
            }
        }
    }
    return A;
}

// sum_i A_i * A_i: each product with its structural pattern, summed with
// map(+)'s exact-zero drop
CSR spgemm_sum(const std::vector<const CSR*>& As) {
    const int64_t N = As[0]->m;
    CSR out;
    out.m = out.n = N;
    out.rowptr.assign(N + 1, 0);
    std::vector<int64_t> marker(N, -1);
    std::vector<double> acc(N, 0.0);
    std::vector<int32_t> cols;
    std::vector<std::pair<int32_t, double>> cur, prod, merged;
    for (int64_t i = 0; i < N; i++) {
        cur.clear();
        for (size_t t = 0; t < As.size(); t++) {
            const CSR& A = *As[t];
            cols.clear();
            for (int64_t p = A.rowptr[i]; p < A.rowptr[i + 1]; p++) {
                int32_t j = A.col[p];
                double a = A.val[p];
                for (int64_t q = A.rowptr[j]; q < A.rowptr[j + 1]; q++) {
                    int32_t c = A.col[q];
                    if (marker[c] != i * (int64_t)As.size() + (int64_t)t) {
                        marker[c] = i * (int64_t)As.size() + (int64_t)t;
                        acc[c] = a * A.val[q];
                        cols.push_back(c);
                    } else {
                        acc[c] += a * A.val[q];
                    }
                }
            }
            std::sort(cols.begin(), cols.end());
            prod.clear();
            for (int32_t c : cols) prod.push_back({c, acc[c]});
            // merged = cur + prod over the union of patterns
            merged.clear();
            size_t a = 0, b = 0;
            while (a < cur.size() || b < prod.size()) {
                int32_t ca = a < cur.size() ? cur[a].first : INT32_MAX;
                int32_t cb = b < prod.size() ? prod[b].first : INT32_MAX;
                double v;
                int32_t c;
                if (ca == cb) {
                    v = cur[a].second + prod[b].second;
                    c = ca;
                    a++;
                    b++;
                } else if (ca < cb) {
                    v = cur[a].second + 0.0;
                    c = ca;
                    a++;
                } else {
                    v = 0.0 + prod[b].second;
                    c = cb;
                    b++;
                }
                merged.push_back({c, v});
            }
            cur.swap(merged);
        }
        // a sum that cancels to exactly 0.0 is not stored (dropping it after
        // the last term leaves the same entries and values as dropping after
        // every term: 0.0 + x == x)
        int64_t kept = 0;
        for (auto& e : cur) {
            if (e.second == 0.0) continue;
            out.col.push_back(e.first);
            out.val.push_back(e.second);
            kept++;
        }
        out.rowptr[i + 1] = out.rowptr[i] + kept;
    }
    return out;
}

// sum_i s_i A_i over the union of patterns, exact zeros dropped
CSR add_scaled(const std::vector<const CSR*>& As, const std::vector<double>& s) {
    const int64_t N = As[0]->m;
    CSR out;
    out.m = out.n = N;
    out.rowptr.assign(N + 1, 0);
    std::vector<std::pair<int32_t, double>> cur, merged;
    for (int64_t i = 0; i < N; i++) {
        cur.clear();
        for (size_t t = 0; t < As.size(); t++) {
            const CSR& A = *As[t];
            merged.clear();
            size_t a = 0;
            int64_t b = A.rowptr[i], be = A.rowptr[i + 1];
            while (a < cur.size() || b < be) {
                int32_t ca = a < cur.size() ? cur[a].first : INT32_MAX;
                int32_t cb = b < be ? A.col[b] : INT32_MAX;
                double v;
                int32_t c;
                if (ca == cb) {
                    v = cur[a].second + s[t] * A.val[b];
                    c = ca;
                    a++;
                    b++;
                } else if (ca < cb) {
                    v = cur[a].second + 0.0;
                    c = ca;
                    a++;
                } else {
                    v = 0.0 + s[t] * A.val[b];
                    c = cb;
                    b++;
                }
                merged.push_back({c, v});
            }
            cur.swap(merged);
        }
        // a sum that cancels to exactly 0.0 is not stored (dropping it after
        // the last term leaves the same entries and values as dropping after
        // every term: 0.0 + x == x)
        int64_t kept = 0;
        for (auto& e : cur) {
            if (e.second == 0.0) continue;
            out.col.push_back(e.first);
            out.val.push_back(e.second);
            kept++;
        }
        out.rowptr[i + 1] = out.rowptr[i] + kept;
    }
    return out;
}

LineTables line_tables(const DLF1D& op, int levels, bool square) {
    const int k = op.k;
    LineTables T;
    T.k = k;
    T.levels = levels;
    std::vector<int64_t> marker;
    std::vector<double> acc;
    std::vector<int32_t> cols;
    for (int lm = 1; lm <= levels; lm++) {
        const int nrb = 1 << (lm - 1), m = nrb * k;
        // leading m x m block: the stored blocks of row block rb with column
        // block < nrb (the admissible levels), in stored order (assemble_dd)
        std::vector<int64_t> lp(m + 1, 0);
        std::vector<int32_t> lc;
        std::vector<double> lv;
        for (int rb = 0; rb < nrb; rb++)
            for (int md = 0; md < k; md++) {
                for (int p = op.rowptr[rb]; p < op.rowptr[rb + 1]; p++) {
                    const int cb = op.colblk[p];
                    if (cb >= nrb) continue;
                    for (int mj = 0; mj < k; mj++) {
                        lc.push_back(cb * k + mj);
                        lv.push_back(op.val[(size_t)p * k * k + (size_t)md * k + mj]);
                    }
                }
                lp[rb * k + md + 1] = (int64_t)lc.size();
            }
        T.roff.push_back((int64_t)T.rowptr.size());
        if (!square) {
            for (int64_t r = 0; r <= m; r++) T.rowptr.push_back((int64_t)T.col.size() + lp[r]);
            T.col.insert(T.col.end(), lc.begin(), lc.end());
            T.val.insert(T.val.end(), lv.begin(), lv.end());
            continue;
        }
        // its square, row by row in the order spgemm_sum accumulates (the
        // row's entries ascending, each times the entries of that row)
        marker.assign(m, -1);
        acc.assign(m, 0.0);
        const int64_t base = (int64_t)T.col.size();
        T.rowptr.push_back(base);
        for (int r = 0; r < m; r++) {
            cols.clear();
            for (int64_t p = lp[r]; p < lp[r + 1]; p++) {
                const int32_t j = lc[p];
                const double a = lv[p];
                for (int64_t q = lp[j]; q < lp[j + 1]; q++) {
                    const int32_t c = lc[q];
                    if (marker[c] != r) {
                        marker[c] = r;
                        acc[c] = a * lv[q];
                        cols.push_back(c);
                    } else {
                        acc[c] += a * lv[q];
                    }
                }
            }
            std::sort(cols.begin(), cols.end());
            for (int32_t c : cols) {
                T.col.push_back(c);
                T.val.push_back(acc[c]);
            }
            T.rowptr.push_back((int64_t)T.col.size());
        }
    }
    return T;
}

// src/pdes.jl:22-49: [[0, I], [lap, 0]]
CSR wave_rhs(const CSR& lap) {
    const int64_t N = lap.m;
    CSR R;
    R.m = R.n = 2 * N;
    R.rowptr.assign(2 * N + 1, 0);
    R.col.reserve(N + lap.nnz());
    R.val.reserve(N + lap.nnz());
    for (int64_t i = 0; i < N; i++) {
        R.col.push_back(int32_t(N + i));
        R.val.push_back(1.0);
        R.rowptr[i + 1] = R.rowptr[i] + 1;
    }
    for (int64_t i = 0; i < N; i++) {
        for (int64_t p = lap.rowptr[i]; p < lap.rowptr[i + 1]; p++) {
            R.col.push_back(lap.col[p]);
            R.val.push_back(lap.val[p]);
        }
        R.rowptr[N + i + 1] = R.rowptr[N + i] + (lap.rowptr[i + 1] - lap.rowptr[i]);
    }
    return R;
}

}  // namespace sgdg
