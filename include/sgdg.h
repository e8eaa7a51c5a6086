/*
 * sgdg.h -- C ABI of libsgdg: the sparse-grid DG derivative operator of
 * GalerkinSparseGrids.jl applied inside explicit Runge-Kutta time stepping on
 * one NVIDIA GB300 (sm_103a).
 *
 * Conventions
 *  - Every entry point returns an int status (SGDG_OK = 0); the message of
 *    the last failure on the calling thread is read with sgdg_last_error.
 *    Nothing throws or aborts across this boundary.
 *  - Coefficient vectors use the reference's layout exactly (levels in
 *    column-major CartesianIndices order, then cells, then modes;
 *    src/dg_vmethods.jl:102-142), so a Julia Vector{Float64} from vcoeffs_DG
 *    passes through unchanged.  Arrays are caller-owned; pointers named *_dev
 *    are device pointers, all others are host memory.
 *  - Indices in exported CSR arrays are 0-based; level/cell/mode in
 *    sgdg_index_map are 1-based like the reference.
 *  - Handles are not safe for concurrent use from several threads; distinct
 *    handles are independent.  Compute calls need a CUDA GPU and fail with
 *    SGDG_ENOGPU otherwise (there is no CPU fallback).
 */
#ifndef SGDG_H
#define SGDG_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    SGDG_OK = 0,
    SGDG_EINVAL = 1,          /* bad argument (the reference throws ArgumentError/DomainError) */
    SGDG_ENOMEM_BUDGET = 2,   /* device allocation refused by the HBM budget or by the device */
    SGDG_ETIMEOUT = 3,        /* a bounded device wait gave up                                 */
    SGDG_ECUDA = 4,           /* CUDA runtime error                                            */
    SGDG_ECANCELLED = 5,      /* the request was cancelled                                     */
    SGDG_ENOGPU = 6,          /* no usable CUDA device                                         */
    SGDG_EUNSUPPORTED = 7,    /* valid input outside what this build implements                */
    SGDG_EIO = 8,             /* a file could not be opened or written                         */
    SGDG_ENONFINITE = 9       /* a served solve's state is no longer finite (NaN or infinity)   */
};

enum { SGDG_SCHEME_SPARSE = 0, SGDG_SCHEME_FULL = 1 };

/* Plain form: assembled FP64 CSR SpMV + FP64 RK4 update (the drop-in).
 * Matrix-free form: FP32 pencil apply of the 1D blocks, FP64 RK4 state.  */
enum { SGDG_METHOD_PLAIN = 0, SGDG_METHOD_MATFREE = 1 };

/* Operator selector "which": 1..D = D_matrix(D,d,k,n); 0 = laplacian_matrix;
 * -1 = the wave right-hand side [[0, I], [L, 0]] of wave_data.              */
enum { SGDG_OP_LAPLACIAN = 0, SGDG_OP_WAVE_RHS = -1 };

/* Problem kinds of batched / served solves. */
enum { SGDG_KIND_ADVECT = 0, SGDG_KIND_WAVE = 1 };

typedef struct sgdg_op sgdg_op;
typedef struct sgdg_batch sgdg_batch;

/* Library version string and the last error message of this thread. */
int sgdg_version(char *buf, size_t len);
int sgdg_last_error(char *buf, size_t len);

/* ---- index map ---------------------------------------------------------- */
/* get_size (src/dg_vmethods.jl:35-45). */
int sgdg_get_size(int D, int k, int n, int scheme, int64_t *N);
/* V2Dref (src/dg_vmethods.jl:123-142): N x D arrays (row-major, entry [i*D+q])
 * of 1-based level, cell and mode of every coefficient. */
int sgdg_index_map(int D, int k, int n, int scheme, int32_t *level, int32_t *cell, int32_t *mode);
/* dg_coeffs[k] (src/1d_dg_functions.jl:52-62): 2k x k, column-major
 * (out[mode*2k + i]; i < k: x^i, i >= k: sgn(x) x^(i-k)). */
int sgdg_dg_coeffs(int k, double *out);

/* ---- 1D operator -------------------------------------------------------- */
/* periodic_DLF_matrix(k, n) (src/1d_derivative.jl:113-117,136-148), CSR. */
int sgdg_dlf_1d_nnz(int k, int n, int64_t *nnz);
int sgdg_dlf_1d_export(int k, int n, int64_t *rowptr, int32_t *col, double *val);

/* ---- operators ---------------------------------------------------------- */
/* Operator handle for (D, k, n, scheme); replaces the setup of
 * D_matrix / grad_matrix / laplacian_matrix (src/multidim_derivative.jl:61-79).
 * Requires n >= 2 and 1 <= k <= 10. */
int sgdg_op_create(int D, int k, int n, int scheme, sgdg_op **out);
/* A 1D operator handle in the hierarchical basis (as sgdg_op_create(1, k, n,
 * SGDG_SCHEME_SPARSE, out)) or in the position basis of wave_evolve_1D
 * (src/pdes.jl:89-121, basis = "pos"): which = 1 is
 * periodic_DLF_matrix(k, n; basis = "pos") = periodic_pos_DLF_matrix
 * (src/1d_derivative.jl:108-111, 136-148), which = SGDG_OP_LAPLACIAN its
 * product D_op * D_op (structural zeros kept, as SparseArrays' `*` keeps them)
 * and SGDG_OP_WAVE_RHS wave_data around that (src/pdes.jl:22-49).  Vectors
 * hold the k 2^n position-basis coefficients, cell-major (index (cell - 1) k
 * + mode - 1).  The position basis runs the plain form only: the matrix-free
 * form and advection return SGDG_EUNSUPPORTED. */
enum { SGDG_BASIS_HIER = 0, SGDG_BASIS_POS = 1 };
int sgdg_op_create_1d(int k, int n, int basis, sgdg_op **out);
int sgdg_op_destroy(sgdg_op *op);
int sgdg_op_size(const sgdg_op *op, int64_t *N);
/* Stored entries of the assembled operator `which` (numerical zeros counted). */
int sgdg_op_nnz(sgdg_op *op, int which, int64_t *nnz);
/* The assembled operator as CSR (rowptr: rows+1 entries; columns sorted). */
int sgdg_op_export_csr(sgdg_op *op, int which, int64_t *rowptr, int32_t *col, double *val);
/* The same operator as the plain form holds it on the device, assembled on
 * the GPU (D_d from the pencils' leading 1D blocks, the Laplacian from their
 * squares merged over d, the wave right-hand side around it): stored entries
 * and values equal to sgdg_op_export_csr's.  nnz, then the host copy. */
int sgdg_op_device_nnz(sgdg_op *op, int which, int64_t *nnz);
int sgdg_op_export_device_csr(sgdg_op *op, int which, int64_t *rowptr, int32_t *col, double *val);

/* y = A x for operator `which` -- the RHS closure (t,x)->*(RHS,x) of
 * src/pdes.jl:63.  Host buffers (length N, or 2N for SGDG_OP_WAVE_RHS).
 * SGDG_METHOD_MATFREE supports which = 1..D and SGDG_OP_LAPLACIAN. */
int sgdg_apply(sgdg_op *op, int which, int method, const double *x, double *y);
/* Same with device pointers on a caller stream (cudaStream_t, may be NULL). */
int sgdg_apply_device(sgdg_op *op, int which, int method, const double *x_dev, double *y_dev, void *stream);

/* Matrix-free FP32 y = D_d x (which = 1..D) or y = laplacian x (which = 0) for
 * (D, k, n, scheme), device pointers, without allocating any device memory.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc -- code whose device memory is owned by another allocator (a
 * framework's caching or stream-ordered pool), runtimes that forbid device
 * allocation after start-up, and latency-critical loops that cannot take
 * cudaMalloc/cudaFree's implicit device synchronisation.  All scratch lives
 * in one 16 MiB device array that every GPU loading the library holds until
 * exit; problems needing more are rejected with SGDG_EINVAL.  Calls share
 * that array: calls overlapping on the GPU race and must be serialised.  The
 * first call on a device resolves the array's address; make it before any
 * stream capture.  Synchronous on `stream` (cudaStream_t, may be NULL). */
int sgdg_apply_noalloc(int D, int k, int n, int scheme, int which, const double *x_dev, double *y_dev,
                       void *stream);

/* Device index checks of a debug build (built with SGDG_DEBUG=1): every
 * gather and scatter index of the matrix-free, CSR and assembly kernels is
 * checked against its vector's length, and a failed check is counted and its
 * access skipped instead of trapping.  *checked = 1 in a debug build (0
 * otherwise, with *violations = 0); *violations = failed checks since the
 * last reset (reset != 0 clears them).  No counterpart in the reference:
 * it stands in for a memory checker on GPUs where none can run. */
int sgdg_debug_bounds(int *checked, int64_t *violations, int reset);

/* ---- evolvers ----------------------------------------------------------- */
/* wave_evolve (src/pdes.jl:54-70) with classical RK4 and nsteps fixed steps on
 * [t0, t1]: u_tt = laplacian(u), state [f; v].  Writes nout >= 2 equally
 * spaced states (times[nout], states[nout * 2N], the first is the initial
 * state), like ODE.jl's (times, states) at the requested output points. */
int sgdg_wave_evolve(sgdg_op *op, const double *f0, const double *v0, double t0, double t1, int64_t nsteps,
                     int nout, int method, double *times, double *states);
/* The plain form's stepping for many solves that share one operator: nsteps
 * classical RK4 steps of y' = A y, A the assembled FP64 operator `which`
 * (SGDG_OP_WAVE_RHS for wave_evolve's [[0, I], [L, 0]], SGDG_OP_LAPLACIAN or
 * 1..D), for nsolves states held on the device one after another (y_dev:
 * nsolves * size of A doubles, updated in place), dt fixed.  Each stage is
 * the FP64 CSR SpMV *(RHS, x) of src/pdes.jl:63 fused with the RK4 stage
 * update, launched over all solves at once; returns once the steps are done
 * on `stream` (cudaStream_t, may be NULL). */
int sgdg_op_plain_steps_device(sgdg_op *op, int which, int64_t nsolves, double *y_dev, double dt, int64_t nsteps,
                               void *stream);
/* Linear advection f_t = -sum_d a_d D_d f (velocity a[D]), composed from
 * grad_matrix the way wave_evolve composes laplacian_matrix. */
int sgdg_advect_evolve(sgdg_op *op, const double *a, const double *f0, double t0, double t1, int64_t nsteps,
                       int nout, int method, double *times, double *states);

/* ---- nodal bases and the Vlasov evolver ---------------------------------- */
/* Basis maps of the Vlasov evolver (k = 2, 3 or 5):
 * which 0 modal -> nodal, 1 nodal -> points, 2 points -> nodal, 3 nodal -> modal.
 * transform_1D(k, n, from, to) (src/1d_nodal_basis.jl:350-414), k 2^n square CSR. */
int sgdg_transform_1d_nnz(int k, int n, int which, int64_t *nnz);
int sgdg_transform_1d_export(int k, int n, int which, int64_t *rowptr, int32_t *col, double *val);
/* transform(D, k, n, from, to) (src/multidim_nodal_basis.jl:83-124): the 1D map
 * tensored over D dimensions on the sparse grid, CSR (N x N). */
int sgdg_transform_nnz(int D, int k, int n, int scheme, int which, int64_t *nnz);
int sgdg_transform_export(int D, int k, int n, int scheme, int which, int64_t *rowptr, int32_t *col, double *val);
/* The same transform assembled on the GPU (the handle of the Vlasov evolver
 * builds its device transforms this way): the same entries, order and values.
 * Writes *nnz; with rowptr, col and val all non-NULL also the CSR. */
int sgdg_transform_device_export(int D, int k, int n, int scheme, int which, int64_t *nnz, int64_t *rowptr,
                                 int32_t *col, double *val);

/* vlasov_evolve (src/pdes.jl:131-227) for D space dimensions: phase space of
 * 2D dimensions ordered x_1..x_D, p_1..p_D, velocity v_d = 2 p_d - 1.  The
 * handle builds what the reference takes as arguments or builds inside:
 * grad_matrix(2D, k, n), m2n, n2p, p2n, n2m and v_point. */
typedef struct sgdg_vlasov sgdg_vlasov;
int sgdg_vlasov_create(int D, int k, int n, int scheme, sgdg_vlasov **out);
int sgdg_vlasov_destroy(sgdg_vlasov *v);
int sgdg_vlasov_size(const sgdg_vlasov *v, int64_t *N);
/* v_point (D x N, point basis), src/pdes.jl:166-172 */
int sgdg_vlasov_v_point(const sgdg_vlasov *v, double *out);
/* the transforms held by the handle (which as above), CSR */
int sgdg_vlasov_transform_nnz(const sgdg_vlasov *v, int which, int64_t *nnz);
int sgdg_vlasov_transform_export(const sgdg_vlasov *v, int which, int64_t *rowptr, int32_t *col, double *val);
/* steprule (src/pdes.jl:174-192): out = df/dt for the modal state f and the
 * force F_point (D x N, point basis), FP64 on the GPU. */
int sgdg_vlasov_rhs(sgdg_vlasov *v, const double *F_point, const double *f, double *out);
/* Classical RK4 with nsteps fixed steps on [t0, t1]; nout >= 2 equally spaced
 * states (the first is f0).  SGDG_METHOD_PLAIN: the assembled FP64 sparse
 * operators; SGDG_METHOD_MATFREE: pencil sweeps of the derivative and of the
 * four transforms in FP32 (operators and weights as hi/lo FP32 pairs), FP64
 * RK state. */
int sgdg_vlasov_evolve(sgdg_vlasov *v, const double *F_point, const double *f0, double t0, double t1, int64_t nsteps,
                       int nout, int method, double *times, double *states);
/* The file vlasov_evolve writes, vlasov.h5 (src/pdes.jl:145-163 and
 * 217-223), at `path`: the Int64 scalars "dimensions", "order", "levels";
 * for m2n, n2p, p2n, n2m and Ds[1] .. Ds[2D] (grad_matrix(2D, k, n)) the
 * SparseMatrixCSC fields "<name>.m", ".n", ".colptr", ".rowval" (Int64,
 * 1-based) and ".nzval" (Float64); then "times" (nout) and "f_modal.%06d"
 * (i = 1..nout, N each, the rows of `states`).  nout = 0 writes the operators
 * only.  HDF5 with an old-style root group; SGDG_EIO when the file cannot be
 * written.  Host only. */
int sgdg_vlasov_write_h5(const sgdg_vlasov *v, const char *path, int64_t nout, const double *times,
                         const double *states);

/* ---- batches of independent solves (matrix-free form) ------------------- */
/* Many solves of uneven D, k, n advance together: each RK4 step is one
 * persistent launch over the pencil tiles of every solve and every stage
 * (groups of solves reach the stages at different times; a stage waits only
 * for its own group's previous stage), replayed from a CUDA graph.  State
 * stays on the device between calls. */
int sgdg_batch_create(sgdg_batch **out);
int sgdg_batch_destroy(sgdg_batch *b);
/* Adds a solve; y0 has N (advection) or 2N (wave: [f; v]) coefficients;
 * a[D] is the advection velocity (ignored for the wave).  Returns its id. */
int sgdg_batch_add(sgdg_batch *b, int kind, int D, int k, int n, int scheme, const double *a, double dt,
                   const double *y0, int *id);
/* Adds a Vlasov solve (matrix-free form): Dx space dimensions (phase space
 * 2 Dx, k in {2, 3, 5}), force F_point (Dx x N, point basis), modal f0 (N). */
int sgdg_batch_add_vlasov(sgdg_batch *b, int Dx, int k, int n, int scheme, double dt, const double *F_point,
                          const double *f0, int *id);
/* Removes a solve and frees its device state (ids of others are unchanged). */
int sgdg_batch_remove(sgdg_batch *b, int id);
/* Use a caller stream (cudaStream_t) for all work of this batch. */
int sgdg_batch_set_stream(sgdg_batch *b, void *stream);
/* Advances every solve in the batch by nsteps RK4 steps (asynchronous). */
int sgdg_batch_step(sgdg_batch *b, int64_t nsteps);
/* Copies solve `id`'s state to the host (synchronises the batch stream). */
int sgdg_batch_get_state(sgdg_batch *b, int id, double *y);
/* Number of stored state coefficients of solve `id` (N or 2N). */
int sgdg_batch_state_size(sgdg_batch *b, int id, int64_t *len);
/* Sum of state sizes over the live solves. */
int sgdg_batch_total_size(sgdg_batch *b, int64_t *len);
/* Replaces every live solve's state from one host array (solves concatenated
 * in increasing id order; page-locked memory makes the copies asynchronous,
 * the caller keeps it valid until the next synchronising call). */
int sgdg_batch_upload(sgdg_batch *b, const double *y_all);
/* Copies every live solve's state into one host array (same order) and
 * synchronises the batch stream. */
int sgdg_batch_download(sgdg_batch *b, double *y_all);
/* Host states in, RK4 steps, host states out (same layout as upload/download;
 * y_out may equal y_in), in one call that synchronises.  The batch's groups
 * of solves are split into nchunks (1..64) pipeline chunks on their own
 * streams, so one chunk's host<->device copies overlap the other chunks'
 * steps; a chunk's step launch takes one CTA per SM, so several chunks step
 * side by side.  16 chunks suit a batch of a few hundred solves.  Pinned host
 * memory is needed for the copies to overlap. */
int sgdg_batch_step_host(sgdg_batch *b, const double *y_in, double *y_out, int64_t nsteps, int nchunks);
/* Autotuner: for every (D, k) of the batch's solves that has no tuned tile
 * shape yet, times one RK stage's pencil tiles of the whole batch for each
 * candidate shape (tile width factor 2^wlog, wlog -2..3, x warp-cooperative
 * row levels 3..6; no state changes) and keeps the fastest in a process-wide
 * table that every batch, server and sgdg_apply_noalloc call then uses.
 * *ntuned = number of (D, k) tuned by this call. */
int sgdg_batch_autotune(sgdg_batch *b, int *ntuned);
/* The tile shape used for (D, k): columns per tile = c * max(1, 256 / row
 * blocks) * 2^wlog (at least c), row blocks of levels <= lmax - coop swept by
 * whole warps; *tuned = 1 if it came from the autotuner or
 * sgdg_set_tile_shape. */
int sgdg_tile_shape(int D, int k, int *wlog, int *coop, int *tuned);
/* Pins a tile shape for (D, k) (wlog -2..3, coop 1..30). */
int sgdg_set_tile_shape(int D, int k, int wlog, int coop);
/* Forgets every tuned or pinned shape (all (D, k) back to the default). */
int sgdg_clear_tile_shapes(void);
/* Launch statistics of one batch step: kernel launches and algorithmic bytes
 * (32 B per state coefficient per RK stage). */
int sgdg_batch_step_info(sgdg_batch *b, int64_t *launches_per_step, double *dof_updates_per_step);

/* ---- request loop (continuous batching of matrix-free solves) ------------ */
/* A server owns one batch engine and a queue.  sgdg_server_tick admits the
 * queued requests that have arrived, in submission order, while the HBM
 * budget (sgdg_set_hbm_budget) has room; advances every running request by
 * the same number of RK4 steps (the fewest any of them has left, at most
 * max_chunk_steps) in shared persistent launches; and retires the finished
 * ones, whose states wait on the host for sgdg_server_result.  A request that
 * cannot fit the budget even alone fails with SGDG_ENOMEM_BUDGET.  Results do
 * not depend on which other requests ran at the same time.  No counterpart in
 * the reference (each wave_evolve call there is one blocking solve). */
typedef struct sgdg_server sgdg_server;
enum { SGDG_REQ_QUEUED = 0, SGDG_REQ_RUNNING = 1, SGDG_REQ_DONE = 2, SGDG_REQ_FAILED = 3, SGDG_REQ_CANCELLED = 4 };
int sgdg_server_create(int max_chunk_steps, sgdg_server **out);
int sgdg_server_destroy(sgdg_server *s);
/* Use a caller stream (cudaStream_t; NULL = the server's own). */
int sgdg_server_set_stream(sgdg_server *s, void *stream);
/* Seconds since the server was created (steady clock); arrival, admission
 * and completion times are on this clock. */
int sgdg_server_clock(sgdg_server *s, double *seconds);
/* Queues one solve (same arguments as sgdg_batch_add) for nsteps RK4 steps.
 * t_arrival < 0 means now; a later time holds the request back until then
 * (submit in arrival order).  y0 is copied. */
int sgdg_server_submit(sgdg_server *s, int kind, int D, int k, int n, int scheme, const double *a, double dt,
                       const double *y0, int64_t nsteps, double t_arrival, int64_t *request_id);
/* One admit / advance / retire round; *completed = requests finished in it.
 * Synchronises the server's stream. */
int sgdg_server_tick(sgdg_server *s, int *completed);
/* State (SGDG_REQ_*), steps done and the three times of a request (-1 where
 * not reached yet). */
int sgdg_server_status(sgdg_server *s, int64_t request_id, int *state, int64_t *steps_done, double *t_arrival,
                       double *t_admit, double *t_done);
/* Copies a finished request's state (N or 2N values) and forgets the request;
 * a failed or cancelled request returns its error code instead. */
int sgdg_server_result(sgdg_server *s, int64_t request_id, double *y);
/* Checkpoint of a request without removing it: its state now (N or 2N
 * values; queued: the initial state, running: the state after the last
 * tick, finished: the result) and *steps_done (may be NULL).  Submitting that
 * state for the remaining steps resumes the solve with the same bits as an
 * uninterrupted run.  A failed or cancelled request returns its error code.
 * The reference has no resume (vlasov_evolve only dumps its trajectory). */
int sgdg_server_snapshot(sgdg_server *s, int64_t request_id, double *y, int64_t *steps_done);
/* Removes a queued or running request (its result becomes SGDG_ECANCELLED). */
int sgdg_server_cancel(sgdg_server *s, int64_t request_id);
/* Queue length, running requests, finished requests not yet collected, and
 * DOF-updates (state coefficients x RK stages) executed so far. */
int sgdg_server_counts(sgdg_server *s, int64_t *queued, int64_t *running, int64_t *finished, double *dof_updates);

/* ---------------------------------------------------------- evaluation --
 * Point values of a coefficient vector (the reference's vector layout) at
 * npts points xs[p * D + d] in [0, 1]^D: reconstruct_DG
 * (src/dg_methods.jl:150-165) batched, in FP64 on the GPU.  A coordinate
 * below 0 or NaN is SGDG_EINVAL (no cell contains it); above 1 the last cell
 * is used, as in cell_index (src/dg_methods.jl:70-78), and its basis
 * functions vanish there. */
int sgdg_evaluate(int D, int k, int n, int scheme, const double *coeffs, int64_t npts, const double *xs,
                  double *values);
/* vcoeffs_DG (src/dg_vmethods.jl:149-179) on the GPU for a function the
 * caller samples: every level block is integrated by tensor quadrature on
 * its 1D pieces.  npts[L-1] = quadrature nodes per cell of level L = 1..n+1;
 * wtab = for each L in turn, cells_L x k x npts[L-1] values (basis function
 * (cell, mode) at each node times its weight); samples = f at every block's
 * tensor grid of nodes, blocks in coefficient order, each block's grid with
 * dimension 1 fastest and, per dimension, node index cell * npts + node.
 * out = the N coefficients in the reference's order (host buffers). */
int sgdg_vcoeffs_contract(int D, int k, int n, int scheme, const int32_t *npts, const double *wtab,
                          const double *samples, double *out);

/* Sum of separable terms, computed on the GPU: coefficient i of the D-dim
 * vector is sum_t amp_t * part_t(e^{i phi_t} prod_d Z_td[i_d]) with i_d the
 * 1D index of i along d (get_index_1D, src/additional_tools.jl:8-13).  Z holds
 * nterms x D complex 1D coefficient vectors of k 2^n entries, (re, im)
 * interleaved; coef holds per term (amp, cos phi, sin phi, part), part 0 for
 * the real and 1 for the imaginary part.  One real term of real vectors is
 * tensor_construct (src/tensor_construct.jl:19-62); sums of modes
 * exp(2 pi i a.x) give Fourier initial conditions. */
int sgdg_tensor_sum(int D, int k, int n, int scheme, int nterms, const double *Z, const double *coef, double *out);
/* The same on device buffers, stream-ordered on `stream` (synchronises it). */
int sgdg_evaluate_device(int D, int k, int n, int scheme, const double *coeffs_dev, int64_t npts,
                         const double *xs_dev, double *values_dev, void *stream);

/* Self-test of the device-side bounded wait the persistent kernels use for
 * their dependencies: one thread waits for a counter that nothing increments.
 * Returns SGDG_ETIMEOUT (the expected outcome: the wait gave up, raised the
 * error flag and the kernel returned, leaving the context usable) and the
 * seconds the wait took; any other status is a failure. */
int sgdg_selftest_bounded_wait(double *seconds);

/* Dry run of the matrix-free work list (host only, no GPU needed): the item
 * list that a batch holding nclasses classes of solves would launch, for
 * checking the schedule and the tiles' index arithmetic.  spec holds 8 ints per
 * class: kind (0 advection, 1 wave, 2 Vlasov), D, k, n, scheme, solves, apply
 * (0: RK4 steps, so the list holds the whole step's four stages; 1: one
 * application) and the applied dimension (-1: the sum over all).  pass_only
 * builds one pass per dimension without the RK update; chunk of nchunks
 * selects the list of one pipeline chunk of sgdg_batch_step_host (each class's
 * groups cut into nchunks runs; 0 of 1 is the whole list).  *nitems and *nboff
 * receive the list's length and the total level-block offsets; when items
 * (capacity items_cap records of SGDG_WL_FIELDS int64) and blockoff (boff_cap)
 * are large enough they receive the records -- cls, d, tab, flags, src, dst,
 * wsel, stage, wait_ctr, wait_need, win_ctr, win_need, done_ctr, lmax, lp, boff,
 * R, g0, W, Wv, kd1, kDm1, rlong, rmagic, rshift, as the device items hold
 * them -- and every class's level-block offsets one after another; classes
 * (4 int64 per class, may be NULL) receives N, Ns, solves and the class's first
 * index in blockoff; *nctr (may be NULL) the number of counters.  The tile
 * shapes are the process-wide ones (sgdg_set_tile_shape). */
#define SGDG_WL_FIELDS 25
int sgdg_worklist_dryrun(int nclasses, const int *spec, int pass_only, int chunk, int nchunks, int64_t *items,
                         int64_t items_cap,
                         int64_t *nitems, int *nctr, int64_t *classes, int64_t *blockoff, int64_t boff_cap,
                         int64_t *nboff);

/* Self-test of the FP32 <-> FP64 conversions the stage kernel's RK update
 * does on the integer pipes (the FP64 pipe is the scarce one): for each of
 * the n host values x[i] the device rounds x[i] to FP32, and widens back to
 * FP64 both the float x[i] rounds to and the float whose bits are x[i]'s low
 * 32 bits, once by those routines and once by the hardware conversions.
 * *mismatches counts the x[i] with a result differing in any bit, *first is
 * the smallest such index (-1 if none). */
int sgdg_selftest_convert(const double *x, int64_t n, int64_t *mismatches, int64_t *first);

/* ---- resources ---------------------------------------------------------- */
/* Upper bound on device bytes the library may hold (0 = no limit). */
int sgdg_set_hbm_budget(int64_t bytes);
int sgdg_hbm_in_use(int64_t *bytes);
/* Blocks until all library work on the device has finished. */
int sgdg_sync(void);

#ifdef __cplusplus
}
#endif
#endif /* SGDG_H */
