/*
 * sgdg_oracle.h -- CPU FP64 restatement of GalerkinSparseGrids.jl's hot path.
 * TEST INFRASTRUCTURE ONLY (parity oracle and timed CPU baseline).
 */
#ifndef SGDG_ORACLE_H
#define SGDG_ORACLE_H
#include <stdint.h>

#define OR_SCHEME_SPARSE 0
#define OR_SCHEME_FULL 1

typedef struct or_mat or_mat;
typedef struct or_csr or_csr;

int or_init(void);
void or_dg_coeffs(int k, double *out);
void or_leg_coeffs(double *out);
double or_v(int k, int level, int cell, int mode, double x);
double or_basis(int level, int cell, int mode, double x);

void or_mat_free(or_mat *A);
void or_mat_info(const or_mat *A, int64_t *m, int64_t *n, int64_t *nnz);
void or_mat_export_csc(const or_mat *A, int64_t *colptr, int32_t *rowval, double *nzval);
void or_mat_export_csr(const or_mat *A, int64_t *rowptr, int32_t *col, double *val);
or_mat *or_from_csc(int64_t m, int64_t n, int64_t nnz, const int64_t *colptr, const int32_t *rowval,
                    const double *nzval);

or_mat *or_hier2pos(int k, int n);
or_mat *or_pos_dlf(int k, int n);
or_mat *or_dmat1d(int k, int n);
or_mat *or_dmatrix(int D, int d, int k, int n, int scheme);
or_mat *or_laplacian(int D, int k, int n, int scheme);
or_mat *or_wave_rhs(const or_mat *lap);
or_mat *or_advection(int D, int k, int n, int scheme, const double *a);

int64_t or_get_size(int D, int k, int n, int scheme);
void or_index_map(int D, int k, int n, int scheme, int32_t *L, int32_t *C, int32_t *M);

void or_spmv_csc(const or_mat *A, const double *x, double *y);
or_csr *or_csr_from_mat(const or_mat *A);
void or_csr_free(or_csr *R);
void or_csr_spmv(const or_csr *A, const double *x, double *y, int nthreads);
void or_rk4_csr(const or_csr *A, double *y, double dt, int64_t nsteps, int nthreads);
int or_max_threads(void);

void or_fourier_coeffs(int D, int k, int n, int scheme, int nmodes, const int32_t *avec, const double *amp,
                       const int32_t *kind, const double *phase, double *out);
void or_tensor_construct(int D, int k, int n, int scheme, const double *coeffs1d, double *out);
int or_cell_index(double x, int l);
void or_reconstruct(int D, int k, int n, int scheme, const double *coeffs, int64_t npts, const double *pts,
                    double *out);

/* nodal basis transforms (src/1d_nodal_basis.jl, src/multidim_nodal_basis.jl):
 * which 0 modal->nodal, 1 nodal->points, 2 points->nodal, 3 nodal->modal */
or_mat *or_transform_1d(int k, int n, int which);
or_mat *or_transform(int D, int k, int n, int scheme, const or_mat *T1);
#endif
