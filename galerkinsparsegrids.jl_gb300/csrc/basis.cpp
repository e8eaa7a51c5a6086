// basis.cpp -- the hierarchical DG basis of GalerkinSparseGrids.jl.
//
// The multiwavelets are defined by the construction steps of
// src/dg_basis.jl:104-190 (project out polynomials, raise vanishing moments,
// reverse Gram-Schmidt): a different orthonormal basis of the same wavelet
// space would change every coefficient vector, so the steps are kept and
// restated here.  Inner products are the exact integrals of
// src/dg_basis.jl:21-35 over [-1,1] for the representation
// "x^i for i<k, sgn(x) x^i for i>=k".
#include <cmath>
#include <mutex>

#include "sgdg_core.h"

namespace sgdg {
namespace {

// exact int_{-1}^{1} of (i-th element) * (j-th element), representation of length 2k
double exact_pair(int i, int j, int k) {
    int a = i % k, b = j % k;
    int sg = (i / k + j / k) % 2;  // number of sgn(x) factors mod 2
    int e = a + b;
    bool even_power = (e % 2) == 0;
    // sgn^2 = 1: integrand x^e, nonzero iff e even.  One sgn: |x| x^(e-1)... = sgn(x) x^e, nonzero iff e odd.
    if (sg == 0) return even_power ? 2.0 / (1 + e) : 0.0;
    return even_power ? 0.0 : 2.0 / (1 + e);
}

double inner(const std::vector<double>& p, const std::vector<double>& q, int k) {
    double s = 0.0;
    const int n = 2 * k;
    for (int i = 0; i < n; i++) {
        if (p[i] == 0) continue;
        for (int j = 0; j < n; j++) {
            if (q[j] == 0) continue;
            s += exact_pair(i, j, k) * p[i] * q[j];
        }
    }
    return s;
}

void axpy(std::vector<double>& y, double a, const std::vector<double>& x) {
    for (size_t t = 0; t < y.size(); t++) y[t] -= a * x[t];
}

// orthonormal Legendre polynomials of degree 0..kmax-1 as length-2k vectors
std::vector<std::vector<double>> legendre_vecs(int nvec, int k) {
    std::vector<std::vector<double>> out;
    for (int j = 0; j < nvec; j++) {
        std::vector<double> p(2 * k, 0.0);
        p[j] = 1.0;
        std::vector<double> orig = p;
        for (int i = 0; i < j; i++) axpy(p, inner(orig, out[i], k) / inner(out[i], out[i], k), out[i]);
        double nrm = std::sqrt(inner(p, p, k));
        for (auto& c : p) c /= nrm;
        out.push_back(p);
    }
    return out;
}

Basis1D build(int k) {
    Basis1D B;
    B.k = k;
    const int n = 2 * k;
    // start: f_j = sgn(x) x^(j-1), j = 1..k
    std::vector<std::vector<double>> f(k, std::vector<double>(n, 0.0));
    for (int j = 0; j < k; j++) f[j][k + j] = 1.0;
    // step 1: remove the polynomial part (project out Legendre 0..k-1)
    auto lp = legendre_vecs(k, k);
    auto g = f;
    for (int i = 0; i < k; i++)
        for (int j = 0; j < k; j++) axpy(g[i], inner(f[i], lp[j], k) / inner(lp[j], lp[j], k), lp[j]);
    // step 2: extra vanishing moments against sgn(x) x^(i-1)
    auto h = g;
    for (int i = 1; i <= k - 1; i++) {
        std::vector<double> probe(n, 0.0);
        probe[k + i - 1] = 1.0;
        const auto fi = g[i - 1];
        for (int j = i + 1; j <= k; j++) axpy(h[j - 1], inner(h[j - 1], probe, k) / inner(fi, probe, k), fi);
    }
    // step 3: reverse Gram-Schmidt, normalise
    std::vector<std::vector<double>> q(k);
    for (int i = k; i >= 1; i--) {
        std::vector<double> qi = h[i - 1];
        for (int j = i + 1; j <= k; j++) axpy(qi, inner(h[i - 1], q[j - 1], k) / inner(q[j - 1], q[j - 1], k), q[j - 1]);
        double nrm = std::sqrt(inner(qi, qi, k));
        for (auto& c : qi) c /= nrm;
        q[i - 1] = qi;
    }
    B.dg.assign((size_t)k * n, 0.0);
    for (int m = 0; m < k; m++)
        for (int t = 0; t < n; t++) B.dg[(size_t)m * n + t] = q[m][t];
    // Legendre 0..kKMax (monomial coefficients, length kKMax+1 each)
    auto L = legendre_vecs(kKMax + 1, kKMax + 1);
    B.leg.assign((size_t)(kKMax + 1) * (kKMax + 1), 0.0);
    for (int m = 0; m <= kKMax; m++)
        for (int t = 0; t <= kKMax; t++) B.leg[(size_t)m * (kKMax + 1) + t] = L[m][t];
    return B;
}

double horner(const double* c, int len, double y) {
    double s = 0.0;
    for (int i = len - 1; i >= 0; i--) s = s * y + c[i];
    return s;
}

double horner_d(const double* c, int len, double y) {
    double s = 0.0;
    for (int i = len - 1; i >= 1; i--) s = s * y + double(i) * c[i];
    return s;
}

}  // namespace

const Basis1D& basis(int k) {
    static std::mutex mu;
    static std::unique_ptr<Basis1D> cache[kKMax + 1];
    if (k < 1 || k > kKMax) throw Error(1, "k must be in 1..10 (K_max)");
    std::lock_guard<std::mutex> g(mu);
    if (!cache[k]) cache[k].reset(new Basis1D(build(k)));
    return *cache[k];
}

HierFn make_hier_fn(int k, int level, int cell, int mode) {
    const Basis1D& B = basis(k);
    HierFn f{};
    f.k = k;
    f.level = level;
    f.cell = cell;
    f.mode = mode;
    for (int i = 0; i < kKMax; i++) f.left[i] = f.right[i] = 0.0;
    if (level == 0) {
        // v = sqrt(2) P_{m-1}(2x-1)  (src/dg_methods.jl:28-30)
        f.x0 = 0.0;
        f.x1 = 1.0;
        f.xm = 0.5;
        f.scale = std::sqrt(2.0);
        f.dydx = 2.0;
        f.shift = 1.0;
        for (int i = 0; i < k; i++) f.left[i] = f.right[i] = B.leg[(size_t)(mode - 1) * (kKMax + 1) + i];
    } else {
        // v = sqrt(2^l) h_m(2^l x - (2c-1))  (src/dg_methods.jl:31-33)
        double w = 1.0 / double(int64_t(1) << (level - 1));
        f.x0 = (cell - 1) * w;
        f.x1 = cell * w;
        f.xm = (2 * cell - 1) * (0.5 * w);
        f.scale = std::sqrt(double(int64_t(1) << level));
        f.dydx = double(int64_t(1) << level);
        f.shift = double(2 * cell - 1);
        const double* c = &B.dg[(size_t)(mode - 1) * 2 * k];
        for (int i = 0; i < k; i++) {
            f.left[i] = c[i] - c[k + i];
            f.right[i] = c[i] + c[k + i];
        }
    }
    return f;
}

static bool locate(const HierFn& f, double& x, int side, const double*& piece) {
    if (side > 0 && x >= 1.0) x -= 1.0;
    if (side < 0 && x <= 0.0) x += 1.0;
    bool inside = side > 0 ? (f.x0 <= x && x < f.x1) : (f.x0 < x && x <= f.x1);
    if (!inside) return false;
    if (f.level == 0)
        piece = f.left;
    else
        piece = (side > 0 ? x < f.xm : x <= f.xm) ? f.left : f.right;
    return true;
}

double hier_value(const HierFn& f, double x, int side) {
    const double* p;
    if (!locate(f, x, side, p)) return 0.0;
    return f.scale * horner(p, f.k, f.dydx * x - f.shift);
}

double hier_deriv(const HierFn& f, double x, int side) {
    const double* p;
    if (!locate(f, x, side, p)) return 0.0;
    return f.scale * f.dydx * horner_d(p, f.k, f.dydx * x - f.shift);
}

}  // namespace sgdg
