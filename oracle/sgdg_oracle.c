/*
 * sgdg_oracle.c -- CPU FP64 restatement of GalerkinSparseGrids.jl's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline ("port" kind).  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU legs may load it; the product library never links it.
 *
 * It restates, operation by operation and in the same floating-point order
 * where the reference fixes one (compiled with -ffp-contract=off, no FMA):
 *   - src/dg_basis.jl:21-190          product_matrix, inner_product, Gram-Schmidt,
 *                                      legendre, orthogonalize_1/2, dg_basis
 *   - src/1d_dg_functions.jl:15-74  array2poly, LegendreP, dg_coeffs, h
 *   - src/1d_dg_functions.jl:83-117  leg, basis, pos_vcoeffs_DG
 *   - src/1d_dg_functions.jl:242-263  hier2pos (matrix form)
 *   - src/dg_methods.jl:27-36         v (hierarchical basis)
 *   - src/derivative_matrix_elements.jl:80-112  symbolic_diff, legendreDlegendre, legvDv
 *   - src/1d_derivative.jl:21-117     D_matrix(k,level), periodic_legvLFv, periodic_LF_matrix,
 *                                      periodic_pos_DLF_matrix, periodic_hier_DLF_matrix
 *   - src/schemes.jl:21-27, src/dg_vmethods.jl:35-142, src/additional_tools.jl:8-20
 *                                      cutoff, get_size, D2Vref/V2Dref ordering, get_index_1D
 *   - src/multidim_derivative.jl:19-79  D_matrix(Val(d),...), grad_matrix, laplacian_matrix
 *   - src/pdes.jl:22-49               wave_data
 * and the Julia SparseArrays semantics those files rely on:
 *   sparse(I,J,V,m,n,+) keeps numerical zeros; SpGEMM (Gustavson) keeps
 *   structural zeros; sparse +/- (map) drops results that are exactly zero.
 *
 * Third-party arithmetic absent from the reference tree is restated from its
 * published algorithm: hquadrature (HCubature 1.4.0) integrates polynomial
 * integrands here, which Gauss-Legendre with enough nodes integrates exactly
 * to roundoff; ODE.jl 2.4.0 is replaced by the classical RK4 tableau the
 * workloads ask for.  Bit-level values are therefore unpinned; the oracle is
 * pinned against the reference's own known-answer tests (tests/test_oracle_*).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "sgdg_oracle.h"

#define KMAX 10          /* K_max, src/1d_dg_functions.jl:7 */
#define LEGN (2 * (KMAX + 1))

static double g_leg[KMAX + 1][LEGN];         /* leg_coeffs = legendre(K_max)      */
static double g_dg[KMAX + 1][KMAX][2 * KMAX]; /* dg_coeffs[k][mode-1][coef]        */
static int g_ready = 0;

/* ------------------------------------------------------------------------- */
/* src/dg_basis.jl:21-35  product_matrix                                      */
/* ------------------------------------------------------------------------- */
static int m1pow(int e) { return (e % 2 == 0) ? 1 : -1; }

static double product_matrix(int i, int j, int n) {
    int k = n / 2;
    if (i < k && j < k) return (double)(1 + m1pow(i + j)) / (double)(1 + i + j);
    if (i >= k && j < k) return (double)(1 - m1pow((i - k) + j)) / (double)(1 + (i - k) + j);
    if (i < k && j >= k) return product_matrix(j, i, n);
    return (double)(1 + m1pow((i - k) + (j - k))) / (double)(1 + (i - k) + (j - k));
}

/* src/dg_basis.jl:37-50 */
static double inner_vv(const double *v1, const double *v2, int n) {
    double value = 0.0;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            if (v1[i] == 0 || v2[j] == 0) continue;
            value += (product_matrix(i, j, n) * v1[i]) * v2[j];
        }
    return value;
}

/* src/dg_basis.jl:52-60  (j is 1-based: the monomial x^(j-1) / its reflection) */
static double inner_vj(const double *v1, int j, int n) {
    double value = 0.0;
    for (int i = 0; i < n; i++) value += product_matrix(i, j - 1, n) * v1[i];
    return value;
}

/* src/dg_basis.jl:68-85  classical Gram-Schmidt on n/2 vectors of length n */
static void gram_schmidt(const double *Qi, double *Qf, int n) {
    int k = n / 2;
    memcpy(Qf, Qi, sizeof(double) * (size_t)k * n);
    for (int i = 0; i < k; i++) {
        for (int j = 0; j < i; j++) {
            double proj = inner_vv(Qi + i * n, Qf + j * n, n) / inner_vv(Qf + j * n, Qf + j * n, n);
            for (int t = 0; t < n; t++) Qf[i * n + t] = Qf[i * n + t] - proj * Qf[j * n + t];
        }
        double nrm = sqrt(inner_vv(Qf + i * n, Qf + i * n, n));
        for (int t = 0; t < n; t++) Qf[i * n + t] = Qf[i * n + t] / nrm;
    }
}

/* src/dg_basis.jl:88-94  legendre(K): K+1 vectors of length 2(K+1) */
static void legendre(int K, double *out) {
    int n = 2 * (K + 1);
    double *Q = calloc((size_t)(K + 1) * n, sizeof(double));
    for (int j = 0; j < K + 1; j++) Q[j * n + j] = 1.0;
    gram_schmidt(Q, out, n);
    free(Q);
}

/* src/dg_basis.jl:104-121 */
static void orthogonalize_1(const double *Qi, double *Qf, int k) {
    int n = 2 * k;
    double *lp = malloc(sizeof(double) * (size_t)k * n);
    legendre(k - 1, lp);
    memcpy(Qf, Qi, sizeof(double) * (size_t)k * n);
    for (int i = 0; i < k; i++)
        for (int j = 0; j < k; j++) {
            double proj = inner_vv(Qi + i * n, lp + j * n, n) / inner_vv(lp + j * n, lp + j * n, n);
            for (int t = 0; t < n; t++) Qf[i * n + t] = Qf[i * n + t] - proj * lp[j * n + t];
        }
    free(lp);
}

/* src/dg_basis.jl:130-146 */
static void orthogonalize_2(const double *Qi, double *Qf, int k) {
    int n = 2 * k;
    memcpy(Qf, Qi, sizeof(double) * (size_t)k * n);
    double *fi = malloc(sizeof(double) * n);
    for (int i = 1; i <= k - 1; i++) {
        memcpy(fi, Qi + (i - 1) * n, sizeof(double) * n);
        for (int j = i + 1; j <= k; j++) {
            double a = inner_vj(Qf + (j - 1) * n, k + i, n) / inner_vj(fi, k + i, n);
            for (int t = 0; t < n; t++) Qf[(j - 1) * n + t] = Qf[(j - 1) * n + t] - a * fi[t];
        }
    }
    free(fi);
}

/* src/dg_basis.jl:154-169 */
static void gram_schmidt_rev(const double *Qi, double *Qf, int k) {
    int n = 2 * k;
    memset(Qf, 0, sizeof(double) * (size_t)k * n);
    for (int i = k; i >= 1; i--) {
        const double *fi = Qi + (i - 1) * n;
        double *qi = Qf + (i - 1) * n;
        memcpy(qi, fi, sizeof(double) * n);
        for (int j = i + 1; j <= k; j++) {
            const double *qj = Qf + (j - 1) * n;
            double proj = inner_vv(fi, qj, n) / inner_vv(qj, qj, n);
            for (int t = 0; t < n; t++) qi[t] = qi[t] - proj * qj[t];
        }
        double nrm = sqrt(inner_vv(qi, qi, n));
        for (int t = 0; t < n; t++) qi[t] = qi[t] / nrm;
    }
}

/* src/dg_basis.jl:185-190 */
static void dg_basis(int k, double *out) {
    int n = 2 * k;
    double *Q = calloc((size_t)k * n, sizeof(double));
    double *T = malloc(sizeof(double) * (size_t)k * n);
    for (int j = 1; j <= k; j++) Q[(j - 1) * n + (k + j - 1)] = 1.0;
    orthogonalize_1(Q, T, k);
    orthogonalize_2(T, Q, k);
    gram_schmidt_rev(Q, out, k);
    free(Q);
    free(T);
}

int or_init(void) {
    if (g_ready) return 0;
    double tmp[(KMAX + 1) * LEGN];
    legendre(KMAX, tmp);
    for (int m = 0; m <= KMAX; m++) memcpy(g_leg[m], tmp + m * LEGN, sizeof(double) * LEGN);
    for (int k = 1; k <= KMAX; k++) {
        double *q = malloc(sizeof(double) * (size_t)k * 2 * k);
        dg_basis(k, q);
        for (int m = 0; m < k; m++) memcpy(g_dg[k][m], q + m * 2 * k, sizeof(double) * 2 * k);
        free(q);
    }
    g_ready = 1;
    return 0;
}

void or_dg_coeffs(int k, double *out) { /* out[mode*2k + coef] */
    or_init();
    for (int m = 0; m < k; m++) memcpy(out + m * 2 * k, g_dg[k][m], sizeof(double) * 2 * k);
}

void or_leg_coeffs(double *out) { /* out[m*22 + coef], m = 0..10 */
    or_init();
    for (int m = 0; m <= KMAX; m++) memcpy(out + m * LEGN, g_leg[m], sizeof(double) * LEGN);
}

/* ------------------------------------------------------------------------- */
/* Basis evaluation: src/1d_dg_functions.jl:15-32,38-46,66-74,83-97   */
/* ------------------------------------------------------------------------- */
static double array2poly(const double *v, int n, double x) {
    if (fabs(x) > 1) return 0.0;
    int k = n / 2;
    double s = 0.0;
    for (int i = k - 1; i >= 0; i--) {
        s = s * x;
        s = s + (v[i] + (signbit(x) ? -v[i + k] : v[i + k]));
    }
    return s;
}

static double LegendreP(int m, double x) { return array2poly(g_leg[m], LEGN, x); }
static double h_fn(int k, int mode, double x) { return array2poly(g_dg[k][mode - 1], 2 * k, x); }

/* src/dg_methods.jl:27-36 */
double or_v(int k, int level, int cell, int mode, double x) {
    if (level == 0) return LegendreP(mode - 1, 2 * x - 1) * sqrt(2.0);
    return h_fn(k, mode, (double)(1LL << level) * x - (double)(2 * cell - 1)) * sqrt(1.0 * (double)(1LL << level));
}

/* src/1d_dg_functions.jl:83-97 */
static double leg(int mode, double x) { return sqrt(2.0) * LegendreP(mode - 1, 2 * x - 1); }
double or_basis(int level, int cell, int mode, double x) {
    return leg(mode, (double)(1LL << level) * x - (double)(cell - 1)) * pow(2.0, (double)level / 2.0);
}

/* ------------------------------------------------------------------------- */
/* Gauss-Legendre nodes on [-1,1] (Newton on the three-term recurrence).      */
/* ------------------------------------------------------------------------- */
static void gauss_legendre(int q, double *x, double *w) {
    for (int i = 0; i < (q + 1) / 2; i++) {
        double z = cos(M_PI * (i + 0.75) / (q + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; it++) {
            double p1 = 1.0, p2 = 0.0;
            for (int j = 1; j <= q; j++) {
                double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = q * (z * p1 - p2) / (z * z - 1.0);
            double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-16) break;
        }
        x[i] = -z;
        x[q - 1 - i] = z;
        w[i] = w[q - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

/* ------------------------------------------------------------------------- */
/* Sparse matrices with Julia SparseArrays semantics                         */
/* ------------------------------------------------------------------------- */
typedef struct or_mat {
    int64_t m, n, nnz;
    int64_t *colptr; /* n+1 */
    int32_t *rowval; /* nnz, 0-based */
    double *nzval;
} or_mat;

static or_mat *mat_alloc(int64_t m, int64_t n, int64_t nnz) {
    or_mat *A = calloc(1, sizeof(or_mat));
    A->m = m;
    A->n = n;
    A->nnz = nnz;
    A->colptr = calloc((size_t)n + 1, sizeof(int64_t));
    A->rowval = malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
    A->nzval = malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    return A;
}

void or_mat_free(or_mat *A) {
    if (!A) return;
    free(A->colptr);
    free(A->rowval);
    free(A->nzval);
    free(A);
}

void or_mat_info(const or_mat *A, int64_t *m, int64_t *n, int64_t *nnz) {
    *m = A->m;
    *n = A->n;
    *nnz = A->nnz;
}

void or_mat_export_csc(const or_mat *A, int64_t *colptr, int32_t *rowval, double *nzval) {
    memcpy(colptr, A->colptr, sizeof(int64_t) * (size_t)(A->n + 1));
    memcpy(rowval, A->rowval, sizeof(int32_t) * (size_t)A->nnz);
    memcpy(nzval, A->nzval, sizeof(double) * (size_t)A->nnz);
}

/* COO growable buffer */
typedef struct {
    int64_t len, cap;
    int32_t *I, *J;
    double *V;
} coo_t;

static void coo_push(coo_t *c, int64_t i, int64_t j, double v) {
    if (c->len == c->cap) {
        c->cap = c->cap ? 2 * c->cap : 1024;
        c->I = realloc(c->I, sizeof(int32_t) * (size_t)c->cap);
        c->J = realloc(c->J, sizeof(int32_t) * (size_t)c->cap);
        c->V = realloc(c->V, sizeof(double) * (size_t)c->cap);
    }
    c->I[c->len] = (int32_t)i;
    c->J[c->len] = (int32_t)j;
    c->V[c->len] = v;
    c->len++;
}
static void coo_free(coo_t *c) {
    free(c->I);
    free(c->J);
    free(c->V);
}

/* sparse(I, J, V, m, n, +): numerical zeros are kept; duplicates are summed
 * in input order.  Rows come out sorted within each column. */
static or_mat *coo_to_csc(int64_t m, int64_t n, const coo_t *c) {
    int64_t nz = c->len;
    /* pass 1: bucket by row (stable) */
    int64_t *rp = calloc((size_t)m + 1, sizeof(int64_t));
    for (int64_t t = 0; t < nz; t++) rp[c->I[t] + 1]++;
    for (int64_t i = 0; i < m; i++) rp[i + 1] += rp[i];
    int64_t *ord = malloc(sizeof(int64_t) * (size_t)(nz > 0 ? nz : 1));
    int64_t *pos = malloc(sizeof(int64_t) * (size_t)(m + 1));
    memcpy(pos, rp, sizeof(int64_t) * (size_t)(m + 1));
    for (int64_t t = 0; t < nz; t++) ord[pos[c->I[t]]++] = t;
    /* pass 2: bucket by column, visiting rows in increasing order (stable) */
    int64_t *cp = calloc((size_t)n + 1, sizeof(int64_t));
    for (int64_t t = 0; t < nz; t++) cp[c->J[t] + 1]++;
    for (int64_t j = 0; j < n; j++) cp[j + 1] += cp[j];
    int64_t *cpos = malloc(sizeof(int64_t) * (size_t)(n + 1));
    memcpy(cpos, cp, sizeof(int64_t) * (size_t)(n + 1));
    int32_t *rows = malloc(sizeof(int32_t) * (size_t)(nz > 0 ? nz : 1));
    double *vals = malloc(sizeof(double) * (size_t)(nz > 0 ? nz : 1));
    for (int64_t q = 0; q < nz; q++) {
        int64_t t = ord[q];
        int64_t p = cpos[c->J[t]]++;
        rows[p] = c->I[t];
        vals[p] = c->V[t];
    }
    /* combine duplicates with + */
    or_mat *A = mat_alloc(m, n, nz);
    int64_t w = 0;
    for (int64_t j = 0; j < n; j++) {
        A->colptr[j] = w;
        for (int64_t p = cp[j]; p < cp[j + 1]; p++) {
            if (w > A->colptr[j] && A->rowval[w - 1] == rows[p])
                A->nzval[w - 1] = A->nzval[w - 1] + vals[p];
            else {
                A->rowval[w] = rows[p];
                A->nzval[w] = vals[p];
                w++;
            }
        }
    }
    A->colptr[n] = w;
    A->nnz = w;
    free(rp);
    free(ord);
    free(pos);
    free(cp);
    free(cpos);
    free(rows);
    free(vals);
    return A;
}

/* A' materialised (copy(adjoint(A))) */
static or_mat *mat_transpose(const or_mat *A) {
    or_mat *T = mat_alloc(A->n, A->m, A->nnz);
    for (int64_t p = 0; p < A->nnz; p++) T->colptr[A->rowval[p] + 1]++;
    for (int64_t i = 0; i < A->m; i++) T->colptr[i + 1] += T->colptr[i];
    int64_t *pos = malloc(sizeof(int64_t) * (size_t)(A->m + 1));
    memcpy(pos, T->colptr, sizeof(int64_t) * (size_t)(A->m + 1));
    for (int64_t j = 0; j < A->n; j++)
        for (int64_t p = A->colptr[j]; p < A->colptr[j + 1]; p++) {
            int64_t q = pos[A->rowval[p]]++;
            T->rowval[q] = (int32_t)j;
            T->nzval[q] = A->nzval[p];
        }
    free(pos);
    return T;
}

/* Gustavson SpGEMM, column by column; structural zeros are kept. */
static int cmp_i32(const void *a, const void *b) {
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

static or_mat *spmatmul(const or_mat *A, const or_mat *B) {
    int64_t m = A->m, n = B->n;
    int64_t cap = A->nnz + B->nnz + 16;
    int64_t *cp = calloc((size_t)n + 1, sizeof(int64_t));
    int32_t *rv = malloc(sizeof(int32_t) * (size_t)cap);
    double *nv = malloc(sizeof(double) * (size_t)cap);
    int64_t *xb = malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
    double *x = malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
    for (int64_t i = 0; i < m; i++) xb[i] = -1;
    int64_t ip = 0;
    for (int64_t i = 0; i < n; i++) {
        cp[i] = ip;
        for (int64_t jp = B->colptr[i]; jp < B->colptr[i + 1]; jp++) {
            double nzB = B->nzval[jp];
            int32_t j = B->rowval[jp];
            for (int64_t kp = A->colptr[j]; kp < A->colptr[j + 1]; kp++) {
                double nzC = A->nzval[kp] * nzB;
                int32_t kr = A->rowval[kp];
                if (xb[kr] != i) {
                    if (ip == cap) {
                        cap *= 2;
                        rv = realloc(rv, sizeof(int32_t) * (size_t)cap);
                        nv = realloc(nv, sizeof(double) * (size_t)cap);
                    }
                    rv[ip++] = kr;
                    xb[kr] = i;
                    x[kr] = nzC;
                } else {
                    x[kr] += nzC;
                }
            }
        }
        qsort(rv + cp[i], (size_t)(ip - cp[i]), sizeof(int32_t), cmp_i32);
        for (int64_t vp = cp[i]; vp < ip; vp++) nv[vp] = x[rv[vp]];
    }
    cp[n] = ip;
    or_mat *C = calloc(1, sizeof(or_mat));
    C->m = m;
    C->n = n;
    C->nnz = ip;
    C->colptr = cp;
    C->rowval = rv;
    C->nzval = nv;
    free(xb);
    free(x);
    return C;
}

/* map(f, A, B) for zero-preserving f: results that are exactly zero are dropped. */
static or_mat *map_add(const or_mat *A, const or_mat *B, double sa, double sb) {
    /* computes (sa*a) + (sb*b) entrywise over the union; sa/sb are +1/-1 so the
     * unary minus of -A is an exact sign flip, as SparseArrays' -(A). */
    int64_t cap = A->nnz + B->nnz + 1;
    or_mat *C = mat_alloc(A->m, A->n, cap);
    int64_t w = 0;
    for (int64_t j = 0; j < A->n; j++) {
        C->colptr[j] = w;
        int64_t pa = A->colptr[j], ea = A->colptr[j + 1];
        int64_t pb = B->colptr[j], eb = B->colptr[j + 1];
        while (pa < ea || pb < eb) {
            int32_t ia = pa < ea ? A->rowval[pa] : INT32_MAX;
            int32_t ib = pb < eb ? B->rowval[pb] : INT32_MAX;
            double cx;
            int32_t ci;
            if (ia == ib) {
                cx = sa * A->nzval[pa] + sb * B->nzval[pb];
                ci = ia;
                pa++;
                pb++;
            } else if (ia < ib) {
                cx = sa * A->nzval[pa] + 0.0;
                ci = ia;
                pa++;
            } else {
                cx = 0.0 + sb * B->nzval[pb];
                ci = ib;
                pb++;
            }
            if (cx != 0) {
                C->rowval[w] = ci;
                C->nzval[w] = cx;
                w++;
            }
        }
    }
    C->colptr[A->n] = w;
    C->nnz = w;
    return C;
}

/* ------------------------------------------------------------------------- */
/* 1D operators                                                               */
/* ------------------------------------------------------------------------- */

/* src/1d_dg_functions.jl:242-263: Q[pos(cell,p), hier(level,cell,mode)] by
 * quadrature over each finest cell; entries with |val| > atol=1e-12 kept. */
or_mat *or_hier2pos(int k, int n) {
    or_init();
    int64_t len = (int64_t)k << n;
    const int q = 16;
    double gx[16], gw[16];
    gauss_legendre(q, gx, gw);
    coo_t c = {0};
    double hcell = 1.0 / (double)(1LL << n);
    int64_t j = 0;
    for (int level = 0; level <= n; level++) {
        int ncell = 1 << (level > 1 ? level - 1 : 0);
        for (int cell = 1; cell <= ncell; cell++)
            for (int mode = 1; mode <= k; mode++) {
                for (int i = 1; i <= (1 << n); i++) {
                    double a = (double)(i - 1) * hcell, b = (double)i * hcell;
                    for (int p = 1; p <= k; p++) {
                        double s = 0.0;
                        for (int t = 0; t < q; t++) {
                            double x = 0.5 * (a + b) + 0.5 * (b - a) * gx[t];
                            s += gw[t] * or_v(k, level, cell, mode, x) * or_basis(n, i, p, x);
                        }
                        s *= 0.5 * (b - a);
                        if (fabs(s) > 1e-12) coo_push(&c, (int64_t)(i - 1) * k + (p - 1), j, s);
                    }
                }
                j++;
            }
    }
    or_mat *Q = coo_to_csc(len, len, &c);
    coo_free(&c);
    return Q;
}

/* src/derivative_matrix_elements.jl:80-94 */
static void symbolic_diff(const double *v, int n, double *ans) {
    int k = n / 2;
    for (int i = 1; i <= n; i++) {
        if (i < k)
            ans[i - 1] = (double)i * v[i];
        else if (i > k && i < 2 * k)
            ans[i - 1] = (double)(i - k) * v[i];
        else
            ans[i - 1] = 0.0;
    }
}

/* src/derivative_matrix_elements.jl:101-103 */
static double legendreDlegendre(int m1, int m2) {
    double d[LEGN];
    symbolic_diff(g_leg[m2 - 1], LEGN, d);
    return inner_vv(g_leg[m1 - 1], d, LEGN);
}

/* src/1d_derivative.jl:21-44 with legvDv (derivative_matrix_elements.jl:106-112) */
static or_mat *pos_D_matrix(int k, int level) {
    coo_t c = {0};
    int ncell = 1 << level;
    for (int cell1 = 1; cell1 <= ncell; cell1++)
        for (int mode1 = 1; mode1 <= k; mode1++) {
            int64_t i = (int64_t)(cell1 - 1) * k + (mode1 - 1);
            for (int cell2 = 1; cell2 <= ncell; cell2++) {
                if (cell2 != cell1) continue; /* legvDv is 0.0 off the diagonal cell */
                for (int mode2 = 1; mode2 <= k; mode2++) {
                    double val = (double)(1LL << (level + 1)) * legendreDlegendre(mode1, mode2);
                    if (fabs(val) > 1.0e-15) coo_push(&c, i, (int64_t)(cell2 - 1) * k + (mode2 - 1), val);
                }
            }
        }
    int64_t len = (int64_t)k << level;
    or_mat *A = coo_to_csc(len, len, &c);
    coo_free(&c);
    return A;
}

/* src/1d_derivative.jl:52-74 (alpha = 0) */
static double periodic_legvLFv(int level, int cell1, int mode1, int cell2, int mode2) {
    double N = (double)(1LL << level);
    double point1 = (double)(cell2 - 1) / N;
    double point2 = (double)cell2 / N;
    const double tiny = 5.0e-16;
    double left1 = or_basis(level, cell1, mode1, point1 - tiny);
    double right1 = or_basis(level, cell1, mode1, point1 + tiny);
    double left2 = or_basis(level, cell1, mode1, point2 - tiny);
    double right2 = or_basis(level, cell1, mode1, point2 + tiny);
    if (cell2 == (1 << level)) right2 = or_basis(level, cell1, mode1, 0.0 + tiny);
    if (cell2 == 1) left1 = or_basis(level, cell1, mode1, 1.0 - tiny);
    double LF1 = 0.5 * (left1 + right1) + 0.0 * (right1 - left1);
    double LF2 = 0.5 * (left2 + right2) + 0.0 * (right2 - left2);
    double val1 = or_basis(level, cell2, mode2, point1 + tiny);
    double val2 = or_basis(level, cell2, mode2, point2 - tiny);
    return LF2 * val2 - LF1 * val1;
}

/* src/1d_derivative.jl:76-100.  Entries vanish unless the cells are equal or
 * periodic neighbours (basis() is exactly zero outside its cell), so only
 * those pairs are evaluated; the loop order and kept entries are unchanged. */
static or_mat *periodic_LF_matrix(int k, int level) {
    coo_t c = {0};
    int ncell = 1 << level;
    for (int cell1 = 1; cell1 <= ncell; cell1++)
        for (int mode1 = 1; mode1 <= k; mode1++) {
            int64_t i = (int64_t)(cell1 - 1) * k + (mode1 - 1);
            for (int cell2 = 1; cell2 <= ncell; cell2++) {
                int dc = (cell2 - cell1 + ncell) % ncell;
                if (!(dc == 0 || dc == 1 || dc == ncell - 1)) continue;
                for (int mode2 = 1; mode2 <= k; mode2++) {
                    double val = periodic_legvLFv(level, cell1, mode1, cell2, mode2);
                    if (fabs(val) > 1.0e-15) coo_push(&c, i, (int64_t)(cell2 - 1) * k + (mode2 - 1), val);
                }
            }
        }
    int64_t len = (int64_t)k << level;
    or_mat *A = coo_to_csc(len, len, &c);
    coo_free(&c);
    return A;
}

/* src/1d_derivative.jl:108-111: A = (-D + LF)' */
or_mat *or_pos_dlf(int k, int n) {
    or_init();
    or_mat *D = pos_D_matrix(k, n);
    or_mat *LF = periodic_LF_matrix(k, n);
    or_mat *S = map_add(D, LF, -1.0, 1.0);
    or_mat *A = mat_transpose(S);
    or_mat_free(D);
    or_mat_free(LF);
    or_mat_free(S);
    return A;
}

/* src/pdes.jl:108-109 (wave_evolve_1D): laplac = *(D_op, D_op), SparseArrays'
 * spmatmul, structural zeros kept */
or_mat *or_matmul(const or_mat *A, const or_mat *B) {
    or_init();
    return spmatmul(A, B);
}

/* src/1d_derivative.jl:113-117: Q' * (A * Q) */
or_mat *or_dmat1d(int k, int n) {
    or_init();
    or_mat *Q = or_hier2pos(k, n);
    or_mat *A = or_pos_dlf(k, n);
    or_mat *AQ = spmatmul(A, Q);
    or_mat *Qt = mat_transpose(Q);
    or_mat *R = spmatmul(Qt, AQ);
    or_mat_free(Q);
    or_mat_free(A);
    or_mat_free(AQ);
    or_mat_free(Qt);
    return R;
}

/* ------------------------------------------------------------------------- */
/* Sparse-grid index map: src/schemes.jl:21-27, src/dg_vmethods.jl:35-142    */
/* ------------------------------------------------------------------------- */
typedef struct {
    int D, k, n, scheme;
    int64_t N, kD;
    int64_t ncodes;     /* (n+1)^D */
    int64_t *offset;    /* per level code: start index or -1 when cut */
    int nlev;           /* number of kept level tuples */
    int32_t *levels;    /* nlev x D, 1-based, in CartesianIndices order */
    int64_t *lev_off;   /* nlev */
} idx_t;

static int cutoff(const int *L, int D, int n, int scheme) {
    if (scheme == OR_SCHEME_FULL) return 0;
    int s = 0;
    for (int q = 0; q < D; q++) s += L[q];
    return s > n + D;
}

static int64_t ipow(int64_t b, int e) {
    int64_t r = 1;
    while (e-- > 0) r *= b;
    return r;
}

static int64_t ncells_of(int L) { return (int64_t)1 << (L > 2 ? L - 2 : 0); }

static void idx_build(idx_t *ix, int D, int k, int n, int scheme) {
    ix->D = D;
    ix->k = k;
    ix->n = n;
    ix->scheme = scheme;
    ix->kD = ipow(k, D);
    ix->ncodes = ipow(n + 1, D);
    ix->offset = malloc(sizeof(int64_t) * (size_t)ix->ncodes);
    ix->levels = malloc(sizeof(int32_t) * (size_t)(ix->ncodes * D));
    ix->lev_off = malloc(sizeof(int64_t) * (size_t)ix->ncodes);
    ix->nlev = 0;
    int64_t j = 0;
    int L[16];
    for (int64_t code = 0; code < ix->ncodes; code++) {
        int64_t c = code;
        for (int q = 0; q < D; q++) {
            L[q] = (int)(c % (n + 1)) + 1; /* dim 1 fastest */
            c /= (n + 1);
        }
        if (cutoff(L, D, n, scheme)) {
            ix->offset[code] = -1;
            continue;
        }
        ix->offset[code] = j;
        for (int q = 0; q < D; q++) ix->levels[ix->nlev * D + q] = L[q];
        ix->lev_off[ix->nlev] = j;
        ix->nlev++;
        int64_t cells = 1;
        for (int q = 0; q < D; q++) cells *= ncells_of(L[q]);
        j += cells * ix->kD;
    }
    ix->N = j;
}

static void idx_free(idx_t *ix) {
    free(ix->offset);
    free(ix->levels);
    free(ix->lev_off);
}

static int64_t level_code(const int *L, int D, int n) {
    int64_t code = 0;
    for (int q = D - 1; q >= 0; q--) code = code * (n + 1) + (L[q] - 1);
    return code;
}

/* D2Vref lookup: (L, C, M) 1-based -> 0-based vector index (or -1 if cut) */
static int64_t idx_lookup(const idx_t *ix, const int *L, const int *C, const int *M) {
    int D = ix->D;
    int64_t off = ix->offset[level_code(L, D, ix->n)];
    if (off < 0) return -1;
    int64_t cl = 0, stride = 1;
    for (int q = 0; q < D; q++) {
        cl += (int64_t)(C[q] - 1) * stride;
        stride *= ncells_of(L[q]);
    }
    int64_t ml = 0;
    stride = 1;
    for (int q = 0; q < D; q++) {
        ml += (int64_t)(M[q] - 1) * stride;
        stride *= ix->k;
    }
    return off + cl * ix->kD + ml;
}

int64_t or_get_size(int D, int k, int n, int scheme) {
    idx_t ix;
    idx_build(&ix, D, k, n, scheme);
    int64_t N = ix.N;
    idx_free(&ix);
    return N;
}

/* V2Dref: arrays of N*D 1-based (level, cell, mode), entry [i*D + q] */
void or_index_map(int D, int k, int n, int scheme, int32_t *Lout, int32_t *Cout, int32_t *Mout) {
    idx_t ix;
    idx_build(&ix, D, k, n, scheme);
    int64_t j = 0;
    for (int t = 0; t < ix.nlev; t++) {
        const int32_t *L = ix.levels + t * D;
        int64_t cells = 1;
        int64_t nc[16];
        for (int q = 0; q < D; q++) {
            nc[q] = ncells_of(L[q]);
            cells *= nc[q];
        }
        for (int64_t cl = 0; cl < cells; cl++)
            for (int64_t ml = 0; ml < ix.kD; ml++) {
                int64_t c = cl, m = ml;
                for (int q = 0; q < D; q++) {
                    Lout[j * D + q] = L[q];
                    Cout[j * D + q] = (int32_t)(c % nc[q]) + 1;
                    c /= nc[q];
                    Mout[j * D + q] = (int32_t)(m % k) + 1;
                    m /= k;
                }
                j++;
            }
    }
    idx_free(&ix);
}

/* ------------------------------------------------------------------------- */
/* D-dimensional derivative: src/multidim_derivative.jl:19-58               */
/* ------------------------------------------------------------------------- */
static or_mat *dmatrix_from_1d(const or_mat *Dm1, int D, int d, int k, int n, int scheme) {
    idx_t ix;
    idx_build(&ix, D, k, n, scheme);
    /* V2D_1D: 1D index -> (level, cell, mode), levels 1..n+1 */
    int64_t len1 = (int64_t)k << n;
    int32_t *l1 = malloc(sizeof(int32_t) * (size_t)len1), *c1 = malloc(sizeof(int32_t) * (size_t)len1),
            *m1 = malloc(sizeof(int32_t) * (size_t)len1);
    {
        int64_t t = 0;
        for (int L = 1; L <= n + 1; L++)
            for (int c = 1; c <= ncells_of(L); c++)
                for (int m = 1; m <= k; m++) {
                    l1[t] = L;
                    c1[t] = c;
                    m1[t] = m;
                    t++;
                }
    }
    coo_t coo = {0};
    int32_t *Lv = malloc(sizeof(int32_t) * (size_t)ix.N * D), *Cv = malloc(sizeof(int32_t) * (size_t)ix.N * D),
            *Mv = malloc(sizeof(int32_t) * (size_t)ix.N * D);
    or_index_map(D, k, n, scheme, Lv, Cv, Mv);
    int L2[16], C2[16], M2[16];
    for (int64_t j = 0; j < ix.N; j++) {
        const int32_t *L = Lv + j * D, *C = Cv + j * D, *M = Mv + j * D;
        int l = L[d - 1], c = C[d - 1], m = M[d - 1];
        /* get_index_1D (additional_tools.jl:18-20), 0-based */
        int64_t j1 = (int64_t)k * ((l >= 2 ? (1LL << (l - 2)) : 0) + (c - 1)) + (m - 1);
        for (int q = 0; q < D; q++) {
            L2[q] = L[q];
            C2[q] = C[q];
            M2[q] = M[q];
        }
        for (int64_t p = Dm1->colptr[j1]; p < Dm1->colptr[j1 + 1]; p++) {
            int32_t i1 = Dm1->rowval[p];
            L2[d - 1] = l1[i1];
            if (cutoff(L2, D, n, scheme)) continue;
            C2[d - 1] = c1[i1];
            M2[d - 1] = m1[i1];
            int64_t i = idx_lookup(&ix, L2, C2, M2);
            coo_push(&coo, i, j, Dm1->nzval[p]);
        }
    }
    or_mat *R = coo_to_csc(ix.N, ix.N, &coo);
    coo_free(&coo);
    free(l1);
    free(c1);
    free(m1);
    free(Lv);
    free(Cv);
    free(Mv);
    idx_free(&ix);
    return R;
}

or_mat *or_dmatrix(int D, int d, int k, int n, int scheme) {
    or_init();
    or_mat *Dm1 = or_dmat1d(k, n);
    or_mat *R = dmatrix_from_1d(Dm1, D, d, k, n, scheme);
    or_mat_free(Dm1);
    return R;
}

/* src/multidim_derivative.jl:71-79: lap = spzeros; lap += D_d * D_d */
or_mat *or_laplacian(int D, int k, int n, int scheme) {
    or_init();
    or_mat *Dm1 = or_dmat1d(k, n);
    int64_t N = or_get_size(D, k, n, scheme);
    or_mat *lap = mat_alloc(N, N, 0);
    for (int d = 1; d <= D; d++) {
        or_mat *Dd = dmatrix_from_1d(Dm1, D, d, k, n, scheme);
        or_mat *P = spmatmul(Dd, Dd);
        or_mat *S = map_add(lap, P, 1.0, 1.0);
        or_mat_free(lap);
        or_mat_free(P);
        or_mat_free(Dd);
        lap = S;
    }
    or_mat_free(Dm1);
    return lap;
}

/* src/pdes.jl:22-49: RHS = [[0, I], [lap, 0]] */
or_mat *or_wave_rhs(const or_mat *lap) {
    int64_t len = lap->n;
    coo_t c = {0};
    for (int64_t col = 0; col < len; col++)
        for (int64_t p = lap->colptr[col]; p < lap->colptr[col + 1]; p++)
            coo_push(&c, lap->rowval[p] + len, col, lap->nzval[p]);
    for (int64_t i = 0; i < len; i++) coo_push(&c, i, i + len, 1.0);
    or_mat *R = coo_to_csc(2 * len, 2 * len, &c);
    coo_free(&c);
    return R;
}

/* Advection operator -sum_d a_d D_d (composition of grad_matrix,
 * multidim_derivative.jl:67-69, assembled like laplacian_matrix's sum). */
or_mat *or_advection(int D, int k, int n, int scheme, const double *a) {
    or_init();
    or_mat *Dm1 = or_dmat1d(k, n);
    int64_t N = or_get_size(D, k, n, scheme);
    or_mat *acc = mat_alloc(N, N, 0);
    for (int d = 1; d <= D; d++) {
        or_mat *Dd = dmatrix_from_1d(Dm1, D, d, k, n, scheme);
        for (int64_t p = 0; p < Dd->nnz; p++) Dd->nzval[p] = -a[d - 1] * Dd->nzval[p];
        or_mat *S = map_add(acc, Dd, 1.0, 1.0);
        or_mat_free(acc);
        or_mat_free(Dd);
        acc = S;
    }
    or_mat_free(Dm1);
    return acc;
}

or_mat *or_from_csc(int64_t m, int64_t n, int64_t nnz, const int64_t *colptr, const int32_t *rowval,
                    const double *nzval) {
    or_mat *A = mat_alloc(m, n, nnz);
    memcpy(A->colptr, colptr, sizeof(int64_t) * (size_t)(n + 1));
    memcpy(A->rowval, rowval, sizeof(int32_t) * (size_t)nnz);
    memcpy(A->nzval, nzval, sizeof(double) * (size_t)nnz);
    return A;
}

/* ------------------------------------------------------------------------- */
/* Mat-vec and fixed-step classical RK4                                       */
/* ------------------------------------------------------------------------- */

/* Julia's CSC mat-vec: y = A*x, column-oriented, single thread. */
void or_spmv_csc(const or_mat *A, const double *x, double *y) {
    for (int64_t i = 0; i < A->m; i++) y[i] = 0.0;
    for (int64_t j = 0; j < A->n; j++) {
        double xj = x[j];
        for (int64_t p = A->colptr[j]; p < A->colptr[j + 1]; p++) y[A->rowval[p]] += A->nzval[p] * xj;
    }
}

/* Row-parallel CSR form of the same product (the multi-core CPU baseline).  */
typedef struct or_csr {
    int64_t m;
    int64_t *rowptr;
    int32_t *col;
    double *val;
} or_csr;

or_csr *or_csr_from_mat(const or_mat *A) {
    or_mat *T = mat_transpose(A);
    or_csr *R = calloc(1, sizeof(or_csr));
    R->m = A->m;
    R->rowptr = T->colptr;
    R->col = T->rowval;
    R->val = T->nzval;
    free(T);
    return R;
}

void or_csr_free(or_csr *R) {
    if (!R) return;
    free(R->rowptr);
    free(R->col);
    free(R->val);
    free(R);
}

void or_mat_export_csr(const or_mat *A, int64_t *rowptr, int32_t *col, double *val) {
    or_mat *T = mat_transpose(A);
    memcpy(rowptr, T->colptr, sizeof(int64_t) * (size_t)(A->m + 1));
    memcpy(col, T->rowval, sizeof(int32_t) * (size_t)A->nnz);
    memcpy(val, T->nzval, sizeof(double) * (size_t)A->nnz);
    or_mat_free(T);
}

static void csr_spmv(const or_csr *A, const double *x, double *y) {
#pragma omp for schedule(static)
    for (int64_t i = 0; i < A->m; i++) {
        double s = 0.0;
        for (int64_t p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) s += A->val[p] * x[A->col[p]];
        y[i] = s;
    }
}

void or_csr_spmv(const or_csr *A, const double *x, double *y, int nthreads) {
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    csr_spmv(A, x, y);
}

/* y <- RK4 step(s) of y' = A y with fixed dt:
 *   k1 = A y, k2 = A(y + dt/2 k1), k3 = A(y + dt/2 k2), k4 = A(y + dt k3),
 *   y += dt/6 (k1 + 2 k2 + 2 k3 + k4)                                     */
void or_rk4_csr(const or_csr *A, double *y, double dt, int64_t nsteps, int nthreads) {
    int64_t m = A->m;
    double *k = malloc(sizeof(double) * (size_t)m);
    double *u = malloc(sizeof(double) * (size_t)m);
    double *acc = malloc(sizeof(double) * (size_t)m);
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t s = 0; s < nsteps; s++) {
        csr_spmv(A, y, k);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < m; i++) {
            acc[i] = k[i];
            u[i] = y[i] + (0.5 * dt) * k[i];
        }
        csr_spmv(A, u, k);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < m; i++) {
            acc[i] += 2.0 * k[i];
            u[i] = y[i] + (0.5 * dt) * k[i];
        }
        csr_spmv(A, u, k);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < m; i++) {
            acc[i] += 2.0 * k[i];
            u[i] = y[i] + dt * k[i];
        }
        csr_spmv(A, u, k);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < m; i++) y[i] = y[i] + (dt / 6.0) * (acc[i] + k[i]);
    }
    free(k);
    free(u);
    free(acc);
}

int or_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* Projection and reconstruction helpers (src/dg_vmethods.jl:149-179,        */
/* src/tensor_construct.jl:19-63, src/dg_methods.jl:150-165)               */
/* ------------------------------------------------------------------------- */

/* 1D coefficients of exp(2*pi*i*a*x) on the hierarchical basis, in 1D vector
 * order (levels 1..n+1, cells, modes): re/im of int e^{2 pi i a x} v(x) dx.   */
static void fourier_1d(int k, int n, int a, double *re, double *im) {
    const int q = 24;
    double gx[24], gw[24];
    gauss_legendre(q, gx, gw);
    int64_t t = 0;
    for (int L = 1; L <= n + 1; L++) {
        int lvl = L - 1;
        int nc = (int)ncells_of(L);
        for (int c = 1; c <= nc; c++) {
            double w = 1.0 / (double)(1 << (lvl > 1 ? lvl - 1 : 0));
            double x0 = (c - 1) * w, x1 = c * w;
            for (int m = 1; m <= k; m++) {
                double sr = 0.0, si = 0.0;
                int halves = (lvl == 0) ? 1 : 2;
                for (int hf = 0; hf < halves; hf++) {
                    double a0 = x0 + hf * (x1 - x0) / halves, a1 = x0 + (hf + 1) * (x1 - x0) / halves;
                    for (int s = 0; s < q; s++) {
                        double x = 0.5 * (a0 + a1) + 0.5 * (a1 - a0) * gx[s];
                        double vv = or_v(k, lvl, c, m, x) * gw[s] * 0.5 * (a1 - a0);
                        sr += cos(2 * M_PI * a * x) * vv;
                        si += sin(2 * M_PI * a * x) * vv;
                    }
                }
                re[t] = sr;
                im[t] = si;
                t++;
            }
        }
    }
}

/* Coefficients of f(x) = sum_m amp[m] * trig_m(2 pi a_m . x + phase[m]) where
 * trig = cos (kind 1) or sin (kind 0): separable products of 1D coefficients. */
void or_fourier_coeffs(int D, int k, int n, int scheme, int nmodes, const int32_t *avec, const double *amp,
                       const int32_t *kind, const double *phase, double *out) {
    or_init();
    idx_t ix;
    idx_build(&ix, D, k, n, scheme);
    int64_t len1 = (int64_t)k << n;
    double *re = malloc(sizeof(double) * (size_t)(len1 * D)), *im = malloc(sizeof(double) * (size_t)(len1 * D));
    for (int64_t i = 0; i < ix.N; i++) out[i] = 0.0;
    int32_t *Lv = malloc(sizeof(int32_t) * (size_t)ix.N * D), *Cv = malloc(sizeof(int32_t) * (size_t)ix.N * D),
            *Mv = malloc(sizeof(int32_t) * (size_t)ix.N * D);
    or_index_map(D, k, n, scheme, Lv, Cv, Mv);
    for (int md = 0; md < nmodes; md++) {
        for (int q = 0; q < D; q++) fourier_1d(k, n, avec[md * D + q], re + q * len1, im + q * len1);
        double cph = cos(phase[md]), sph = sin(phase[md]);
        for (int64_t i = 0; i < ix.N; i++) {
            double pr = 1.0, pi = 0.0;
            for (int q = 0; q < D; q++) {
                int L = Lv[i * D + q], c = Cv[i * D + q], m = Mv[i * D + q];
                int64_t j1 = (int64_t)k * ((L >= 2 ? (1LL << (L - 2)) : 0) + (c - 1)) + (m - 1);
                double xr = re[q * len1 + j1], xi = im[q * len1 + j1];
                double nr = pr * xr - pi * xi, ni = pr * xi + pi * xr;
                pr = nr;
                pi = ni;
            }
            /* e^{i(theta+phase)} = (pr + i pi)(cph + i sph) */
            double zr = pr * cph - pi * sph, zi = pr * sph + pi * cph;
            out[i] += amp[md] * (kind[md] == 1 ? zr : zi);
        }
    }
    free(re);
    free(im);
    free(Lv);
    free(Cv);
    free(Mv);
    idx_free(&ix);
}

/* tensor_construct (src/tensor_construct.jl:19-63): coefficient of
 * prod_d f_d(x_d) from the 1D coefficient vectors coeffs1d[d*len1 + j1]. */
void or_tensor_construct(int D, int k, int n, int scheme, const double *coeffs1d, double *out) {
    idx_t ix;
    idx_build(&ix, D, k, n, scheme);
    int64_t len1 = (int64_t)k << n;
    int32_t *Lv = malloc(sizeof(int32_t) * (size_t)ix.N * D), *Cv = malloc(sizeof(int32_t) * (size_t)ix.N * D),
            *Mv = malloc(sizeof(int32_t) * (size_t)ix.N * D);
    or_index_map(D, k, n, scheme, Lv, Cv, Mv);
    for (int64_t i = 0; i < ix.N; i++) {
        double val = 1.0;
        for (int q = 0; q < D; q++) {
            int L = Lv[i * D + q], c = Cv[i * D + q], m = Mv[i * D + q];
            int64_t j1 = (int64_t)k * ((L >= 2 ? (1LL << (L - 2)) : 0) + (c - 1)) + (m - 1);
            val *= coeffs1d[q * len1 + j1];
        }
        out[i] = val;
    }
    free(Lv);
    free(Cv);
    free(Mv);
    idx_free(&ix);
}

/* reconstruct_DG at npts points (pts[p*D + q]) from a coefficient vector. */
void or_reconstruct(int D, int k, int n, int scheme, const double *coeffs, int64_t npts, const double *pts,
                    double *out) {
    or_init();
    idx_t ix;
    idx_build(&ix, D, k, n, scheme);
    int C[16], M[16];
    double vals[16][KMAX];
    for (int64_t p = 0; p < npts; p++) {
        const double *x = pts + p * D;
        double value = 0.0;
        for (int t = 0; t < ix.nlev; t++) {
            const int32_t *L = ix.levels + t * D;
            for (int q = 0; q < D; q++) {
                /* cell_index, src/dg_methods.jl:70-79 (l is the 0-based level) */
                int l = L[q] - 1;
                if (l <= 1)
                    C[q] = 1;
                else if (x[q] >= 1)
                    C[q] = 1 << (l - 1);
                else
                    C[q] = 1 + (int)floor((double)(1 << (l - 1)) * x[q]);
                for (int m = 0; m < k; m++) vals[q][m] = or_v(k, l, C[q], m + 1, x[q]);
            }
            for (int64_t ml = 0; ml < ix.kD; ml++) {
                int64_t mm = ml;
                double prod = 1.0;
                for (int q = 0; q < D; q++) {
                    M[q] = (int)(mm % k) + 1;
                    mm /= k;
                    prod *= vals[q][M[q] - 1];
                }
                value += coeffs[idx_lookup(&ix, (const int *)L, C, M)] * prod;
            }
        }
        out[p] = value;
    }
    idx_free(&ix);
}

/* cell_index (src/dg_methods.jl:70-79); l is the 0-based level */
int or_cell_index(double x, int l) {
    if (l <= 1) return 1;
    if (x >= 1) return 1 << (l - 1);
    return 1 + (int)floor((double)(1 << (l - 1)) * x);
}

/* ------------------------------------------------------------------------- */
/* Nodal basis and basis transforms: src/1d_nodal_basis.jl,                  */
/* src/multidim_nodal_basis.jl                                               */
/* ------------------------------------------------------------------------- */

/* lag_nodal, src/1d_nodal_basis.jl:46-66 (k in {2, 3, 5}) */
static double lag_nodal(int k, int mode, double x) {
    if (x < 0 || x > 1) return 0.0;
    if (k == 2) return mode == 1 ? x : 1 - x;
    if (k == 3) {
        if (mode == 1) return 2 * (x - 0.5) * (x - 1);
        if (mode == 2) return -4 * x * (x - 1);
        return 2 * x * (x - 0.5);
    }
    /* k == 5 */
    if (mode == 1) return 32.0 / 3 * (x - 0.25) * (x - 0.5) * (x - 0.75) * (x - 1);
    if (mode == 2) return -128.0 / 3 * x * (x - 0.5) * (x - 0.75) * (x - 1);
    if (mode == 3) return 64 * x * (x - 0.25) * (x - 0.75) * (x - 1);
    if (mode == 4) return -128.0 / 3 * x * (x - 0.25) * (x - 0.5) * (x - 1);
    return 32.0 / 3 * x * (x - 0.25) * (x - 0.5) * (x - 0.75);
}

/* h_nodal, src/1d_nodal_basis.jl:69-99 */
static double h_nodal(int k, int mode, double x) {
    if (k == 2) {
        if (mode == 1) return fmax(0.0, 1 - fabs(x));
        if (fabs(x) > 1 || x == 0) return 0.0;
        return x < 0 ? x + 1 : 0.0;
    }
    if (k == 3) {
        if (mode == 1) return fmax(0.0, -4 * x * (x + 1));
        if (mode == 2) return fmax(0.0, -4 * x * (x - 1));
        if (fabs(x) > 1 || x == 0) return 0.0;
        return x < 0 ? 2 * (x + 1) * (x + 0.5) : 0.0;
    }
    /* k == 5 */
    if (mode == 1) return (x < -1 || x > 0) ? 0.0 : -128.0 / 3 * x * (x + 1) * (x + 0.5) * (x + 0.25);
    if (mode == 2) return (x < -1 || x > 0) ? 0.0 : -128.0 / 3 * x * (x + 1) * (x + 0.5) * (x + 0.75);
    if (mode == 3) return (x > 1 || x < 0) ? 0.0 : -128.0 / 3 * x * (x - 1) * (x - 0.5) * (x - 0.75);
    if (mode == 4) return (x > 1 || x < 0) ? 0.0 : -128.0 / 3 * x * (x - 1) * (x - 0.5) * (x - 0.25);
    if (fabs(x) > 1 || x == 0) return 0.0;
    return x < 0 ? 32.0 / 3 * (x + 1) * (x + 0.75) * (x + 0.5) * (x + 0.25) : 0.0;
}

/* v_nodal, src/1d_nodal_basis.jl:102-108 */
static double v_nodal(int k, int level, int cell, int mode, double x) {
    if (level == 0) return lag_nodal(k, mode, x);
    return h_nodal(k, mode, (double)(1 << level) * x - (2 * cell - 1));
}

/* threshold(sparse, atol), src/additional_tools.jl:34-42: |v| < atol -> dropped */
static or_mat *mat_threshold(const or_mat *A, double atol) {
    or_mat *B = mat_alloc(A->m, A->n, A->nnz);
    int64_t w = 0;
    for (int64_t j = 0; j < A->n; j++) {
        B->colptr[j] = w;
        for (int64_t p = A->colptr[j]; p < A->colptr[j + 1]; p++)
            if (!(fabs(A->nzval[p]) < atol) && A->nzval[p] != 0) {
                B->rowval[w] = A->rowval[p];
                B->nzval[w] = A->nzval[p];
                w++;
            }
    }
    B->colptr[A->n] = w;
    B->nnz = w;
    return B;
}

/* threshold(inv(Matrix(A)), atol): Gauss-Jordan with partial pivoting on the
 * dense copy (LAPACK's getrf/getri in Julia; values agree to roundoff). */
static or_mat *mat_inverse_threshold(const or_mat *A, double atol) {
    int64_t n = A->n;
    double *M = calloc((size_t)(n * 2 * n), sizeof(double));
    for (int64_t j = 0; j < n; j++)
        for (int64_t p = A->colptr[j]; p < A->colptr[j + 1]; p++) M[A->rowval[p] * 2 * n + j] = A->nzval[p];
    for (int64_t i = 0; i < n; i++) M[i * 2 * n + n + i] = 1.0;
    for (int64_t c = 0; c < n; c++) {
        int64_t piv = c;
        for (int64_t r = c + 1; r < n; r++)
            if (fabs(M[r * 2 * n + c]) > fabs(M[piv * 2 * n + c])) piv = r;
        if (piv != c)
            for (int64_t t = 0; t < 2 * n; t++) {
                double s = M[c * 2 * n + t];
                M[c * 2 * n + t] = M[piv * 2 * n + t];
                M[piv * 2 * n + t] = s;
            }
        double d = M[c * 2 * n + c];
        for (int64_t t = 0; t < 2 * n; t++) M[c * 2 * n + t] /= d;
        for (int64_t r = 0; r < n; r++) {
            if (r == c) continue;
            double f = M[r * 2 * n + c];
            if (f == 0) continue;
            for (int64_t t = 0; t < 2 * n; t++) M[r * 2 * n + t] -= f * M[c * 2 * n + t];
        }
    }
    coo_t co = {0};
    for (int64_t j = 0; j < n; j++)
        for (int64_t i = 0; i < n; i++) {
            double v = M[i * 2 * n + n + j];
            if (!(fabs(v) < atol) && v != 0) coo_push(&co, i, j, v);
        }
    free(M);
    or_mat *R = coo_to_csc(n, n, &co);
    coo_free(&co);
    return R;
}

/* eval_points_1D / nodal2points_1D, src/1d_nodal_basis.jl:183-236: value of
 * every nodal function at the collocation points (level-major, k per cell:
 * k-1 nodes taken from the right, then the cell's last point from the left).
 * The reference evaluates at x +- 1e-16; here at the adjacent double on that
 * side, which selects the same one-sided limit at every collocation point. */
static double nodal_side(int k, int level, int cell, int mode, double x, int side) {
    /* one-sided limit: evaluate at the nearest double on that side */
    double xs = side > 0 ? nextafter(x, 2.0) : nextafter(x, -1.0);
    return v_nodal(k, level, cell, mode, xs);
}

static or_mat *nodal2points_1d(int k, int n, double atol) {
    int64_t len = (int64_t)k << n;
    coo_t co = {0};
    int64_t j = 0;
    for (int level = 0; level <= n; level++)
        for (int cell = 1; cell <= (1 << (level > 1 ? level - 1 : 0)); cell++)
            for (int mode = 1; mode <= k; mode++) {
                int64_t i = 0;
                for (int l = 0; l <= n; l++) {
                    int nc = 1 << (l > 1 ? l - 1 : 0);
                    for (int c = 1; c <= nc; c++) {
                        for (int t = 0; t < k - 1; t++) {
                            double node = l == 0 ? (double)t / (k - 1) : (2.0 * t + 1) / (2.0 * (k - 1));
                            double x = ((double)(c - 1) + node) / nc;
                            double val = nodal_side(k, level, cell, mode, x, +1);
                            if (val != 0) coo_push(&co, i, j, val);
                            i++;
                        }
                        double x = l == 0 ? 1.0 : ((double)c - 0.5) / nc;
                        double val = nodal_side(k, level, cell, mode, x, -1);
                        if (val != 0) coo_push(&co, i, j, val);
                        i++;
                    }
                }
                j++;
            }
    or_mat *A = coo_to_csc(len, len, &co);
    coo_free(&co);
    or_mat *B = mat_threshold(A, atol);
    or_mat_free(A);
    return B;
}

/* nodal2pos_1D, src/1d_nodal_basis.jl:287-338: inner products of each nodal
 * function with the finest position basis, integrated on the two halves of
 * every finest cell that meets the function's cell (Gauss-Legendre, exact for
 * these polynomial pieces, in place of hquadrature); entries with
 * |val| <= eps(atol) dropped, then threshold(atol). */
static or_mat *nodal2pos_1d(int k, int n, double atol) {
    int64_t len = (int64_t)k << n;
    const int q = 12;
    double gx[12], gw[12];
    gauss_legendre(q, gx, gw);
    coo_t co = {0};
    int64_t j = 0;
    double h = 1.0 / (double)(1LL << n);
    for (int level = 0; level <= n; level++) {
        int ncl = 1 << (level > 1 ? level - 1 : 0);
        for (int cell = 1; cell <= ncl; cell++)
            for (int mode = 1; mode <= k; mode++) {
                double nmin = (double)(cell - 1) / ncl, nmax = (double)cell / ncl;
                for (int c = 1; c <= (1 << n); c++) {
                    double pmin = (c - 1) * h, pmed = (c - 0.5) * h, pmax = c * h;
                    if (pmin > nmax || pmax < nmin) continue;
                    for (int m = 1; m <= k; m++) {
                        double val = 0.0;
                        double ab[2][2] = {{pmin, pmed}, {pmed, pmax}};
                        for (int s = 0; s < 2; s++) {
                            double a = ab[s][0], b = ab[s][1], acc = 0.0;
                            for (int t = 0; t < q; t++) {
                                double x = 0.5 * (a + b) + 0.5 * (b - a) * gx[t];
                                acc += gw[t] * v_nodal(k, level, cell, mode, x) * or_basis(n, c, m, x);
                            }
                            val += acc * 0.5 * (b - a);
                        }
                        if (fabs(val) > nextafter(atol, 1.0) - atol) /* eps(atol) */
                            coo_push(&co, (int64_t)(c - 1) * k + (m - 1), j, val);
                    }
                }
                j++;
            }
    }
    or_mat *A = coo_to_csc(len, len, &co);
    coo_free(&co);
    or_mat *B = mat_threshold(A, atol);
    or_mat_free(A);
    return B;
}

/* transform_1D, src/1d_nodal_basis.jl:350-414, for the four maps the Vlasov
 * evolver uses (atol = 1e-12 as called from transform):
 *   which 0: modal -> nodal  threshold(pos2nodal_1D(k,n) * hier2pos(k,n), atol)
 *   which 1: nodal -> points nodal2points_1D(k, n; atol)
 *   which 2: points -> nodal points2nodal_1D(k, n; atol)
 *   which 3: nodal -> modal  threshold(pos2hier(k,n) * nodal2pos_1D(k,n), atol) */
or_mat *or_transform_1d(int k, int n, int which) {
    or_init();
    const double atol = 1e-12;
    if (which == 0) {
        or_mat *n2pos = nodal2pos_1d(k, n, atol); /* pos2nodal_1D(k, n; atol=1e-12) */
        or_mat *pos2n = mat_inverse_threshold(n2pos, atol);
        or_mat *Q = or_hier2pos(k, n);
        or_mat *P = spmatmul(pos2n, Q);
        or_mat *R = mat_threshold(P, atol);
        or_mat_free(n2pos);
        or_mat_free(pos2n);
        or_mat_free(Q);
        or_mat_free(P);
        return R;
    }
    if (which == 1) return nodal2points_1d(k, n, atol);
    if (which == 2) {
        or_mat *n2p = nodal2points_1d(k, n, 1e-15);
        or_mat *R = mat_inverse_threshold(n2p, atol);
        or_mat_free(n2p);
        return R;
    }
    or_mat *n2pos = nodal2pos_1d(k, n, 1e-15);
    or_mat *Q = or_hier2pos(k, n);
    or_mat *Qt = mat_transpose(Q);
    or_mat *P = spmatmul(Qt, n2pos);
    or_mat *R = mat_threshold(P, atol);
    or_mat_free(n2pos);
    or_mat_free(Q);
    or_mat_free(Qt);
    or_mat_free(P);
    return R;
}

/* relevant_cell_1D, src/multidim_nodal_basis.jl:19-25 (0-based levels) */
static int relevant_cell_1d(int level1, int cell1, int level2, int cell2) {
    double l1 = (double)(cell1 - 1) / (1 << (level1 > 1 ? level1 - 1 : 0));
    double r1 = (double)cell1 / (1 << (level1 > 1 ? level1 - 1 : 0));
    double l2 = (double)(cell2 - 1) / (1 << (level2 > 1 ? level2 - 1 : 0));
    double r2 = (double)cell2 / (1 << (level2 > 1 ? level2 - 1 : 0));
    return (l1 <= l2 && r1 >= r2) || (l1 >= l2 && r1 <= r2);
}

/* transform(D, k, n, mat_1D), src/multidim_nodal_basis.jl:40-109: entry
 * (i, j) = prod_d mat_1D[i_1D(d), j_1D(d)] over pairs of sparse-grid indices
 * whose cells nest in every dimension; products with |val| < atol = 1e-12
 * are left out. */
or_mat *or_transform(int D, int k, int n, int scheme, const or_mat *T1) {
    idx_t ix;
    idx_build(&ix, D, k, n, scheme);
    /* dense 1D matrix (k 2^n square) for direct lookups, as Matrix(mat_1D) */
    int64_t len = T1->m;
    double *M1 = calloc((size_t)(len * len), sizeof(double));
    for (int64_t j = 0; j < T1->n; j++)
        for (int64_t p = T1->colptr[j]; p < T1->colptr[j + 1]; p++) M1[T1->rowval[p] * len + j] = T1->nzval[p];
    const double atol = 1e-12;
    /* Columns of one level tuple t1 are the contiguous run starting at
     * lev_off[t1]; each tuple's entries go to their own list (in the
     * sequential order), and the lists are joined in tuple order, so the
     * COO sequence -- and the assembled matrix -- is the sequential one. */
    coo_t *parts = calloc((size_t)ix.nlev, sizeof(coo_t));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int t1 = 0; t1 < ix.nlev; t1++) {
        coo_t *co = &parts[t1];
        int L1[16], C1[16], Mo1[16], L2[16], C2[16], Mo2[16];
        int64_t j = ix.lev_off[t1];
        for (int q = 0; q < D; q++) L1[q] = ix.levels[t1 * D + q];
        int64_t cells1 = 1;
        for (int q = 0; q < D; q++) cells1 *= ncells_of(L1[q]);
        for (int64_t cl1 = 0; cl1 < cells1; cl1++) {
            int64_t c = cl1;
            for (int q = 0; q < D; q++) {
                C1[q] = (int)(c % ncells_of(L1[q])) + 1;
                c /= ncells_of(L1[q]);
            }
            for (int64_t ml1 = 0; ml1 < ix.kD; ml1++) {
                int64_t mm = ml1;
                int js[16];
                for (int q = 0; q < D; q++) {
                    Mo1[q] = (int)(mm % k) + 1;
                    mm /= k;
                    js[q] = k * (int)((L1[q] >= 2 ? (1 << (L1[q] - 2)) : 0) + C1[q] - 1) + Mo1[q] - 1;
                }
                int64_t i = 0;
                for (int t2 = 0; t2 < ix.nlev; t2++) {
                    for (int q = 0; q < D; q++) L2[q] = ix.levels[t2 * D + q];
                    int64_t cells2 = 1;
                    for (int q = 0; q < D; q++) cells2 *= ncells_of(L2[q]);
                    for (int64_t cl2 = 0; cl2 < cells2; cl2++) {
                        int64_t cc = cl2;
                        int rel = 1;
                        for (int q = 0; q < D; q++) {
                            C2[q] = (int)(cc % ncells_of(L2[q])) + 1;
                            cc /= ncells_of(L2[q]);
                            rel &= relevant_cell_1d(L2[q] - 1, C2[q], L1[q] - 1, C1[q]);
                        }
                        if (!rel) {
                            i += ix.kD;
                            continue;
                        }
                        for (int64_t ml2 = 0; ml2 < ix.kD; ml2++) {
                            int64_t m2 = ml2;
                            double val = 1.0;
                            for (int q = 0; q < D; q++) {
                                Mo2[q] = (int)(m2 % k) + 1;
                                m2 /= k;
                                int i1 = k * (int)((L2[q] >= 2 ? (1 << (L2[q] - 2)) : 0) + C2[q] - 1) + Mo2[q] - 1;
                                val *= M1[(int64_t)i1 * len + js[q]];
                                if (val == 0) break;
                            }
                            if (!(fabs(val) < atol)) coo_push(co, i, j, val);
                            i++;
                        }
                    }
                }
                j++;
            }
        }
    }
    coo_t co = {0};
    for (int t1 = 0; t1 < ix.nlev; t1++) {
        for (int64_t e = 0; e < parts[t1].len; e++) coo_push(&co, parts[t1].I[e], parts[t1].J[e], parts[t1].V[e]);
        coo_free(&parts[t1]);
    }
    free(parts);
    free(M1);
    or_mat *R = coo_to_csc(ix.N, ix.N, &co);
    coo_free(&co);
    idx_free(&ix);
    return R;
}
