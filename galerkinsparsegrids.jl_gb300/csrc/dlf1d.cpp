// dlf1d.cpp -- the 1D hierarchical periodic DG derivative with central flux.
//
// The reference builds it in the finest position basis and conjugates
// (src/1d_derivative.jl:108-117: hier2pos' * (-D + LF)' * hier2pos).  Because
// hier2pos is an exact change of orthonormal basis, the same operator is,
// entry by entry in the hierarchical basis,
//     D[h', h] = - int v_h (d/dx v_h') dx  -  sum_e avg(v_h)(e) [[v_h']](e),
// where e runs over the points where the row function v_h' jumps (its support
// ends and midpoint, or the periodic point 0 = 1 at level 0), avg is the mean
// of the two one-sided limits (alpha = 0 flux, src/1d_derivative.jl:66-67) and
// [[g]](e) = g(e+) - g(e-).  This file evaluates that formula with exact
// one-sided limits and Gauss-Legendre quadrature (exact for these piecewise
// polynomials), so values agree with the reference to roundoff (the reference
// evaluates edges at +-5e-16, src/1d_derivative.jl:56-64, which moves its
// entries by ~1e-13 relative).
//
// Stored pattern: a dense k x k block for every pair of (level, cell) blocks
// whose closed supports meet periodically -- the structural pattern the
// reference's two SpGEMMs leave for n >= 2 (numerical zeros included).
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>

#include "sgdg_core.h"

namespace sgdg {
namespace {

void gauss_legendre(int q, std::vector<double>& x, std::vector<double>& w) {
    x.assign(q, 0.0);
    w.assign(q, 0.0);
    for (int i = 0; i < (q + 1) / 2; i++) {
        double z = std::cos(M_PI * (i + 0.75) / (q + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int j = 2; j <= q; j++) {
                double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
                p0 = p1;
                p1 = p2;
            }
            if (q == 1) {
                p1 = z;
                p0 = 1.0;
            }
            dp = q * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        x[i] = -z;
        x[q - 1 - i] = z;
        w[i] = w[q - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

bool touch(double a0, double a1, double b0, double b1) {
    if (a0 <= b1 && b0 <= a1) return true;
    return (a0 == 0.0 && b1 == 1.0) || (b0 == 0.0 && a1 == 1.0);
}

void block_support(int L, int c, double& x0, double& x1) {
    double w = 1.0 / double(ncells(L));
    x0 = (c - 1) * w;
    x1 = c * w;
}

}  // namespace

static DLF1D build_dlf(int k, int n) {
    if (n < 2) throw Error(1, "n must be >= 2 (with <= 2 finest cells the reference's periodic fluxes cancel)");
    if (n > 20) throw Error(1, "n too large");
    DLF1D op;
    op.k = k;
    op.n = n;
    op.nblocks = 1 << n;
    for (int L = 1; L <= n + 1; L++)
        for (int c = 1; c <= ncells(L); c++) {
            op.blk_level.push_back(L);
            op.blk_cell.push_back(c);
        }
    std::vector<double> gx, gw;
    gauss_legendre(k + 1, gx, gw);
    // hierarchical functions per block
    std::vector<std::vector<HierFn>> fns(op.nblocks);
    for (int b = 0; b < op.nblocks; b++)
        for (int m = 1; m <= k; m++) fns[b].push_back(make_hier_fn(k, op.blk_level[b] - 1, op.blk_cell[b], m));
    op.rowptr.assign(op.nblocks + 1, 0);
    for (int rb = 0; rb < op.nblocks; rb++) {
        double r0, r1;
        block_support(op.blk_level[rb], op.blk_cell[rb], r0, r1);
        const auto& row = fns[rb];
        // jump points of the row functions, taken mod 1 (0 and 1 are one point)
        std::vector<double> E;
        if (row[0].level == 0)
            E = {0.0};
        else
            for (double e : {row[0].x0, row[0].xm, row[0].x1}) {
                double em = e >= 1.0 ? e - 1.0 : e;
                if (std::find(E.begin(), E.end(), em) == E.end()) E.push_back(em);
            }
        for (int cb = 0; cb < op.nblocks; cb++) {
            double c0, c1;
            block_support(op.blk_level[cb], op.blk_cell[cb], c0, c1);
            if (!touch(r0, r1, c0, c1)) continue;
            const auto& col = fns[cb];
            // volume-term intervals: intersection split at both midpoints
            double lo = std::max(r0, c0), hi = std::min(r1, c1);
            std::vector<double> bp;
            if (lo < hi) {
                bp = {lo, hi};
                for (double p : {row[0].xm, col[0].xm})
                    if (p > lo && p < hi) bp.push_back(p);
                std::sort(bp.begin(), bp.end());
            }
            for (int i = 0; i < k; i++)
                for (int j = 0; j < k; j++) {
                    const HierFn& fr = row[i];
                    const HierFn& fc = col[j];
                    double vol = 0.0;
                    for (size_t s = 0; s + 1 < bp.size(); s++) {
                        double a = bp[s], b = bp[s + 1], hh = 0.5 * (b - a), mid = 0.5 * (a + b);
                        double acc = 0.0;
                        for (size_t t = 0; t < gx.size(); t++) {
                            double x = mid + hh * gx[t];
                            acc += gw[t] * hier_value(fc, x, +1) * hier_deriv(fr, x, +1);
                        }
                        vol += acc * hh;
                    }
                    double flux = 0.0;
                    for (double e : E) {
                        double avg = 0.5 * (hier_value(fc, e, -1) + hier_value(fc, e, +1));
                        double jump = hier_value(fr, e, +1) - hier_value(fr, e, -1);
                        flux += avg * jump;
                    }
                    op.val.push_back(-vol - flux);
                }
            op.colblk.push_back(cb);
        }
        op.rowptr[rb + 1] = (int32_t)op.colblk.size();
    }
    return op;
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
