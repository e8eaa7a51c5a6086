// nodal.cpp -- the nodal and point bases of the Vlasov evolver and the
// transforms between them and the modal (hierarchical) basis.
//
// The nodal basis (src/1d_nodal_basis.jl:46-108, k in {2, 3, 5}) is a
// hierarchical interpolating basis: at level 0 the Lagrange polynomials of the
// equispaced nodes of [0,1]; below, per cell, piecewise Lagrange functions of
// the k-1 new nodes of the cell (zero at the cell's ends and midpoint) and
// one function that is discontinuous at the midpoint (its left limit there
// is 1).  The point basis holds the values at the collocation points (the new
// nodes from the right, each cell's last point from the left), in the same
// (level, cell, mode) order.  Both definitions fix every transform value, so
// they are kept exactly.
//
// 1D transforms follow src/1d_nodal_basis.jl:183-414 with its thresholds:
//   modal -> nodal  = threshold(inv(nodal2pos) * hier2pos, 1e-12)
//   nodal -> points = threshold(nodal2points, 1e-12)
//   points -> nodal = threshold(inv(nodal2points), 1e-12)
//   nodal -> modal  = threshold(hier2pos' * nodal2pos, 1e-12)
// with the inner products integrated exactly (Gauss-Legendre on polynomial
// pieces) instead of by adaptive quadrature.  The D-dimensional transform
// (src/multidim_nodal_basis.jl:40-109) is the Kronecker product of the 1D map
// restricted to the sparse grid, over pairs of cells that nest in every
// dimension, dropping products below 1e-12.  All four 1D maps are triangular
// in the level (modal <-> nodal map level l only to levels <= l, nodal <->
// points only to levels >= l), which is what makes the restricted products
// mutual inverses on the sparse grid.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>

#include "sgdg_core.h"

namespace sgdg {
namespace {

constexpr double kAtol = 1e-12;

double lag_nodal(int k, int mode, double x) {
    if (x < 0 || x > 1) return 0.0;
    switch (k) {
        case 2: return mode == 1 ? x : 1 - x;  // node 1, then node 0
        case 3: {
            const double r[3] = {2 * (x - 0.5) * (x - 1), -4 * x * (x - 1), 2 * x * (x - 0.5)};
            return r[mode - 1];
        }
        default: {  // k = 5: nodes 0, 1/4, 1/2, 3/4, 1
            const double a = x, b = x - 0.25, c = x - 0.5, d = x - 0.75, e = x - 1;
            const double r[5] = {32.0 / 3 * b * c * d * e, -128.0 / 3 * a * c * d * e, 64 * a * b * d * e,
                                 -128.0 / 3 * a * b * c * e, 32.0 / 3 * a * b * c * d};
            return r[mode - 1];
        }
    }
}

// cell functions on y in [-1, 1] (the cell), midpoint y = 0
double h_nodal(int k, int mode, double y) {
    const bool left_open = y > -1 && y < 0;  // discontinuous mode lives on (-1, 0)
    if (k == 2) {
        if (mode == 1) return std::max(0.0, 1 - std::fabs(y));
        return left_open ? y + 1 : 0.0;
    }
    if (k == 3) {
        if (mode == 1) return std::max(0.0, -4 * y * (y + 1));
        if (mode == 2) return std::max(0.0, -4 * y * (y - 1));
        return left_open ? 2 * (y + 1) * (y + 0.5) : 0.0;
    }
    // k = 5: new nodes -3/4, -1/4, 1/4, 3/4, then the discontinuous mode
    if (mode <= 2) {
        if (y < -1 || y > 0) return 0.0;
        const double o = mode == 1 ? 0.25 : 0.75;
        return -128.0 / 3 * y * (y + 1) * (y + 0.5) * (y + o);
    }
    if (mode <= 4) {
        if (y > 1 || y < 0) return 0.0;
        const double o = mode == 3 ? 0.75 : 0.25;
        return -128.0 / 3 * y * (y - 1) * (y - 0.5) * (y - o);
    }
    return left_open ? 32.0 / 3 * (y + 1) * (y + 0.75) * (y + 0.5) * (y + 0.25) : 0.0;
}

double v_nodal(int k, int level, int cell, int mode, double x) {
    if (level == 0) return lag_nodal(k, mode, x);
    return h_nodal(k, mode, std::ldexp(x, level) - (2 * cell - 1));
}

// one-sided limit: the value at the adjacent double on that side
double v_nodal_side(int k, int level, int cell, int mode, double x, int side) {
    return v_nodal(k, level, cell, mode, std::nextafter(x, side > 0 ? 2.0 : -1.0));
}

struct Dense {
    int n = 0;
    std::vector<double> a;  // row-major
    explicit Dense(int n_) : n(n_), a((size_t)n_ * n_, 0.0) {}
    double& at(int i, int j) { return a[(size_t)i * n + j]; }
    double at(int i, int j) const { return a[(size_t)i * n + j]; }
};

void threshold(Dense& A, double atol) {
    for (auto& v : A.a)
        if (std::fabs(v) < atol) v = 0.0;
}

Dense invert(const Dense& A) {
    const int n = A.n;
    Dense M = A, R(n);
    for (int i = 0; i < n; i++) R.at(i, i) = 1.0;
    for (int c = 0; c < n; c++) {
        int piv = c;
        for (int r = c + 1; r < n; r++)
            if (std::fabs(M.at(r, c)) > std::fabs(M.at(piv, c))) piv = r;
        if (M.at(piv, c) == 0.0) throw Error(7, "singular transform matrix");
        if (piv != c)
            for (int t = 0; t < n; t++) {
                std::swap(M.at(c, t), M.at(piv, t));
                std::swap(R.at(c, t), R.at(piv, t));
            }
        const double d = M.at(c, c);
        for (int t = 0; t < n; t++) {
            M.at(c, t) /= d;
            R.at(c, t) /= d;
        }
        for (int r = 0; r < n; r++) {
            if (r == c) continue;
            const double f = M.at(r, c);
            if (f == 0.0) continue;
            for (int t = 0; t < n; t++) {
                M.at(r, t) -= f * M.at(c, t);
                R.at(r, t) -= f * R.at(c, t);
            }
        }
    }
    return R;
}

Dense matmul(const Dense& A, const Dense& B) {
    const int n = A.n;
    Dense C(n);
    for (int i = 0; i < n; i++)
        for (int t = 0; t < n; t++) {
            const double a = A.at(i, t);
            if (a == 0.0) continue;
            for (int j = 0; j < n; j++) C.at(i, j) += a * B.at(t, j);
        }
    return C;
}

Dense transpose(const Dense& A) {
    Dense T(A.n);
    for (int i = 0; i < A.n; i++)
        for (int j = 0; j < A.n; j++) T.at(j, i) = A.at(i, j);
    return T;
}

// visits the 1D blocks (level 0..n, cell, mode) in vector order
template <class F>
void for_blocks(int k, int n, F&& f) {
    int j = 0;
    for (int l = 0; l <= n; l++)
        for (int c = 1; c <= (1 << (l > 1 ? l - 1 : 0)); c++)
            for (int m = 1; m <= k; m++) f(j++, l, c, m);
}

Dense nodal_to_points(int k, int n) {
    Dense A(k << n);
    for_blocks(k, n, [&](int j, int level, int cell, int mode) {
        int i = 0;
        for (int l = 0; l <= n; l++) {
            const int nc = 1 << (l > 1 ? l - 1 : 0);
            for (int c = 1; c <= nc; c++) {
                for (int t = 0; t < k - 1; t++) {
                    const double node = l == 0 ? double(t) / (k - 1) : (2.0 * t + 1) / (2.0 * (k - 1));
                    A.at(i++, j) = v_nodal_side(k, level, cell, mode, (double(c - 1) + node) / nc, +1);
                }
                const double last = l == 0 ? 1.0 : (double(c) - 0.5) / nc;
                A.at(i++, j) = v_nodal_side(k, level, cell, mode, last, -1);
            }
        }
    });
    return A;
}

std::vector<double> gl_nodes(int q, std::vector<double>& w) {
    std::vector<double> x(q);
    w.assign(q, 0.0);
    for (int i = 0; i < (q + 1) / 2; i++) {
        double z = std::cos(M_PI * (i + 0.75) / (q + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int j = 2; j <= q; j++) {
                const double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
                p0 = p1;
                p1 = p2;
            }
            dp = q * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        x[i] = -z;
        x[q - 1 - i] = z;
        w[i] = w[q - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    return x;
}

// finest position basis: sqrt(2^n) sqrt(2) P_{m-1}(2 (2^n x - (c-1)) - 1)
double pos_basis(const std::vector<HierFn>& leg0, int n, int c, int m, double x) {
    return std::sqrt(std::ldexp(1.0, n)) * hier_value(leg0[m - 1], std::ldexp(x, n) - (c - 1), +1);
}

// <nodal function, finest position function> on both halves of every finest cell
Dense nodal_to_pos(int k, int n, double atol) {
    std::vector<double> gw;
    const std::vector<double> gx = gl_nodes(12, gw);
    std::vector<HierFn> leg0;
    for (int m = 1; m <= k; m++) leg0.push_back(make_hier_fn(k, 0, 1, m));
    Dense A(k << n);
    const double h = std::ldexp(1.0, -n);
    const double tiny = std::nextafter(atol, 1.0) - atol;  // eps(atol)
    for_blocks(k, n, [&](int j, int level, int cell, int mode) {
        const int ncl = 1 << (level > 1 ? level - 1 : 0);
        const double lo = double(cell - 1) / ncl, hi = double(cell) / ncl;
        for (int c = 1; c <= (1 << n); c++) {
            const double a0 = (c - 1) * h, am = (c - 0.5) * h, a1 = c * h;
            if (a0 > hi || a1 < lo) continue;
            for (int m = 1; m <= k; m++) {
                double val = 0.0;
                for (int s = 0; s < 2; s++) {
                    const double a = s ? am : a0, b = s ? a1 : am, mid = 0.5 * (a + b), hw = 0.5 * (b - a);
                    double acc = 0.0;
                    for (size_t t = 0; t < gx.size(); t++) {
                        const double x = mid + hw * gx[t];
                        acc += gw[t] * v_nodal(k, level, cell, mode, x) * pos_basis(leg0, n, c, m, x);
                    }
                    val += acc * hw;
                }
                if (std::fabs(val) > tiny) A.at((c - 1) * k + (m - 1), j) = val;
            }
        }
    });
    threshold(A, atol);
    return A;
}

// hier2pos (src/1d_dg_functions.jl:242-263): modal block j on the finest cells, |val| > 1e-12
Dense modal_to_pos(int k, int n) {
    std::vector<double> gw;
    const std::vector<double> gx = gl_nodes(16, gw);
    std::vector<HierFn> leg0;
    for (int m = 1; m <= k; m++) leg0.push_back(make_hier_fn(k, 0, 1, m));
    Dense A(k << n);
    const double h = std::ldexp(1.0, -n);
    for_blocks(k, n, [&](int j, int level, int cell, int mode) {
        const HierFn f = make_hier_fn(k, level, cell, mode);
        for (int c = 1; c <= (1 << n); c++) {
            const double a = (c - 1) * h, b = c * h;
            if (b <= f.x0 || a >= f.x1) continue;
            for (int m = 1; m <= k; m++) {
                double acc = 0.0;
                for (size_t t = 0; t < gx.size(); t++) {
                    const double x = 0.5 * (a + b) + 0.5 * h * gx[t];
                    acc += gw[t] * hier_value(f, x, +1) * pos_basis(leg0, n, c, m, x);
                }
                acc *= 0.5 * h;
                if (std::fabs(acc) > kAtol) A.at((c - 1) * k + (m - 1), j) = acc;
            }
        }
    });
    return A;
}

CSR to_csr(const Dense& A) {
    CSR R;
    R.m = R.n = A.n;
    R.rowptr.assign(A.n + 1, 0);
    for (int i = 0; i < A.n; i++) {
        for (int j = 0; j < A.n; j++)
            if (A.at(i, j) != 0.0) {
                R.col.push_back(j);
                R.val.push_back(A.at(i, j));
            }
        R.rowptr[i + 1] = (int64_t)R.col.size();
    }
    return R;
}

Dense build_1d(int k, int n, int which) {
    switch (which) {
        case TRANSFORM_MODAL_TO_NODAL: {
            Dense p2n = invert(nodal_to_pos(k, n, kAtol));
            threshold(p2n, kAtol);
            Dense R = matmul(p2n, modal_to_pos(k, n));
            threshold(R, kAtol);
            return R;
        }
        case TRANSFORM_NODAL_TO_POINTS: {
            Dense R = nodal_to_points(k, n);
            threshold(R, kAtol);
            return R;
        }
        case TRANSFORM_POINTS_TO_NODAL: {
            Dense P = nodal_to_points(k, n);
            threshold(P, 1e-15);
            Dense R = invert(P);
            threshold(R, kAtol);
            return R;
        }
        default: {
            Dense R = matmul(transpose(modal_to_pos(k, n)), nodal_to_pos(k, n, 1e-15));
            threshold(R, kAtol);
            return R;
        }
    }
}

}  // namespace

CSR transform_1d(int k, int n, int which) {
    if (k != 2 && k != 3 && k != 5) throw Error(1, "the nodal basis exists for k = 2, 3, 5");
    if (n < 0 || n > 9) throw Error(7, "nodal transforms support 0 <= n <= 9");
    if (which < 0 || which > 3) throw Error(1, "transform must be 0..3 (m2n, n2p, p2n, n2m)");
    static std::mutex mu;
    static std::map<std::tuple<int, int, int>, CSR> cache;
    std::lock_guard<std::mutex> g(mu);
    auto key = std::make_tuple(k, n, which);
    auto f = cache.find(key);
    if (f != cache.end()) return f->second;
    return cache.emplace(key, to_csr(build_1d(k, n, which))).first->second;
}

CSR transform_dd(const SparseIndex& ix, const CSR& T1) {
    const int D = ix.D, k = ix.k, n = ix.n;
    // 1D column lists: for each 1D column, its (row, value, row level, row cell)
    const int len = (int)T1.m;
    std::vector<std::vector<std::pair<int, double>>> cols(len);
    for (int i = 0; i < len; i++)
        for (int64_t p = T1.rowptr[i]; p < T1.rowptr[i + 1]; p++) cols[T1.col[p]].push_back({i, T1.val[p]});
    // 1D index -> (level 1-based, cell 1-based, mode 1-based)
    std::vector<int> lv(len), cl(len), md(len);
    {
        int i = 0;
        for (int L = 1; L <= n + 1; L++)
            for (int c = 1; c <= (int)ncells(L); c++)
                for (int m = 1; m <= k; m++) {
                    lv[i] = L;
                    cl[i] = c;
                    md[i] = m;
                    i++;
                }
    }
    auto nests = [&](int L1, int c1, int L2, int c2) {  // relevant_cell_1D on 1-based levels
        const double w1 = 1.0 / (double)ncells(L1), w2 = 1.0 / (double)ncells(L2);
        const double a1 = (c1 - 1) * w1, b1 = c1 * w1, a2 = (c2 - 1) * w2, b2 = c2 * w2;
        return (a1 <= a2 && b1 >= b2) || (a1 >= a2 && b1 <= b2);
    };
    // columns of one level tuple range -> COO (rows, columns, values)
    struct Part {
        std::vector<int32_t> I, J;
        std::vector<double> V;
    };
    auto columns = [&](int t0, int t1, Part& out) {
        std::vector<int32_t>& I = out.I;
        std::vector<int32_t>& J = out.J;
        std::vector<double>& V = out.V;
        std::vector<std::vector<std::pair<int, double>>> lists(D);
        int L[kDMax], C[kDMax], M[kDMax];
        int64_t j = t0 < ix.nlev ? ix.lev_off[t0] : ix.N;
        for (int t = t0; t < t1; t++) {
            for (int q = 0; q < D; q++) L[q] = ix.levels[(size_t)t * D + q];
            for (int64_t cc = 0; cc < ix.lev_cells[t]; cc++) {
                int64_t r = cc;
                for (int q = 0; q < D; q++) {
                    C[q] = int(r % ncells(L[q])) + 1;
                    r /= ncells(L[q]);
                }
                for (int64_t mm = 0; mm < ix.kD; mm++, j++) {
                    int64_t s = mm;
                    for (int q = 0; q < D; q++) {
                        M[q] = int(s % k) + 1;
                        s /= k;
                        const int j1 = k * (int)((L[q] >= 2 ? ncells(L[q]) : 0) + C[q] - 1) + M[q] - 1;
                        lists[q].clear();
                        for (auto& e : cols[j1])
                            if (nests(lv[e.first], cl[e.first], L[q], C[q])) lists[q].push_back(e);
                    }
                    // Cartesian product over dimensions, pruned by the level cutoff
                    int pos[kDMax] = {0};
                    int RL[kDMax];
                    int q = 0;
                    int lsum = 0;
                    while (q >= 0) {
                        if (q == D) {
                            // complete: value in dimension order, as the reference multiplies
                            double val = 1.0;
                            for (int p = 0; p < D; p++) {
                                val *= lists[p][pos[p] - 1].second;
                                if (val == 0) break;
                            }
                            if (!(std::fabs(val) < kAtol)) {
                                int RC[kDMax], RM[kDMax];
                                for (int p = 0; p < D; p++) {
                                    const int i1 = lists[p][pos[p] - 1].first;
                                    RC[p] = cl[i1];
                                    RM[p] = md[i1];
                                }
                                const int lid = ix.lookup_level(RL);
                                int64_t cl_lin = 0, cs = 1, ml_lin = 0, ms = 1;
                                for (int p = 0; p < D; p++) {
                                    cl_lin += (RC[p] - 1) * cs;
                                    cs *= ncells(RL[p]);
                                    ml_lin += (RM[p] - 1) * ms;
                                    ms *= k;
                                }
                                I.push_back((int32_t)(ix.lev_off[lid] + cl_lin * ix.kD + ml_lin));
                                J.push_back((int32_t)j);
                                V.push_back(val);
                            }
                            q--;
                            if (q >= 0) lsum -= RL[q];
                            continue;
                        }
                        if (pos[q] >= (int)lists[q].size()) {
                            pos[q] = 0;
                            q--;
                            if (q >= 0) lsum -= RL[q];
                            continue;
                        }
                        const int i1 = lists[q][pos[q]].first;
                        pos[q]++;
                        RL[q] = lv[i1];
                        // the remaining dimensions need at least level 1 each; the
                        // list is in increasing level, so the rest of it is cut too
                        if (ix.scheme == 0 && lsum + RL[q] + (D - 1 - q) > n + D) {
                            pos[q] = (int)lists[q].size();
                            continue;
                        }
                        lsum += RL[q];
                        q++;
                    }
                }
            }
        }
    };
    // level tuples split over threads in contiguous ranges (columns stay in order)
    const int nth = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<Part> parts(nth);
    std::vector<int> cut(nth + 1, ix.nlev);
    {
        // balance by coefficient count
        int64_t per = (ix.N + nth - 1) / nth, acc = 0;
        int p = 0;
        cut[0] = 0;
        for (int t = 0; t < ix.nlev && p < nth - 1; t++) {
            acc += ix.lev_cells[t] * ix.kD;
            if (acc >= per * (p + 1)) cut[++p] = t + 1;
        }
        for (int q = p + 1; q <= nth; q++) cut[q] = ix.nlev;
    }
    std::vector<std::thread> th;
    for (int p = 0; p < nth; p++) th.emplace_back(columns, cut[p], cut[p + 1], std::ref(parts[p]));
    for (auto& x : th) x.join();
    // CSR (columns come in increasing order within a row)
    CSR R;
    R.m = R.n = ix.N;
    R.rowptr.assign(ix.N + 1, 0);
    size_t total = 0;
    for (auto& pt : parts) {
        total += pt.I.size();
        for (int32_t i : pt.I) R.rowptr[(size_t)i + 1]++;
    }
    for (int64_t i = 0; i < ix.N; i++) R.rowptr[i + 1] += R.rowptr[i];
    R.col.resize(total);
    R.val.resize(total);
    std::vector<int64_t> fill(R.rowptr.begin(), R.rowptr.end() - 1);
    for (auto& pt : parts) {
        for (size_t e = 0; e < pt.I.size(); e++) {
            const int64_t p = fill[pt.I[e]]++;
            R.col[p] = pt.J[e];
            R.val[p] = pt.V[e];
        }
        std::vector<int32_t>().swap(pt.I);
        std::vector<int32_t>().swap(pt.J);
        std::vector<double>().swap(pt.V);
    }
    return R;
}

// Collocation point of the 1D point-basis index (level L, cell c, mode m,
// 1-based): the k-1 new nodes of the cell, then its last point
// (src/1d_nodal_basis.jl:183-213).
double nodal_point(int k, int L, int c, int m) {
    const int l = L - 1;
    const double nc = (double)(1 << (l > 1 ? l - 1 : 0));
    if (m < k) {
        const double node = l == 0 ? double(m - 1) / (k - 1) : (2.0 * (m - 1) + 1) / (2.0 * (k - 1));
        return (double(c - 1) + node) / nc;
    }
    return l == 0 ? 1.0 : (double(c) - 0.5) / nc;
}

// v_d = 2 p_d - 1 at every point of the phase-space grid (d = 0..Dx-1, p_d =
// phase dimension Dx + d): the velocity points of src/pdes.jl:166-172, which
// n2p m2n of the exact modal coefficients reproduce to roundoff.
std::vector<double> vlasov_velocity_points(const SparseIndex& ix, int Dx) {
    const int D = ix.D, k = ix.k;
    std::vector<double> out((size_t)Dx * ix.N);
    int64_t e = 0;
    for (int t = 0; t < ix.nlev; t++) {
        const int* L = &ix.levels[(size_t)t * D];
        for (int64_t cc = 0; cc < ix.lev_cells[t]; cc++)
            for (int64_t mm = 0; mm < ix.kD; mm++, e++) {
                int64_t r = cc, s = mm;
                for (int q = 0; q < D; q++) {
                    const int c = int(r % ncells(L[q])) + 1, m = int(s % k) + 1;
                    r /= ncells(L[q]);
                    s /= k;
                    if (q >= Dx) out[(size_t)(q - Dx) * ix.N + e] = 2.0 * nodal_point(k, L[q], c, m) - 1.0;
                }
            }
    }
    return out;
}

}  // namespace sgdg
