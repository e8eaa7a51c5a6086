// capi.cu -- the C ABI of libsgdg (include/sgdg.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/sgdg.h"
#include "device_util.h"
#include "engine.h"
#include "api_util.h"
#include "device_csr.h"
#include "mf_engine.h"
#include "sgdg_core.h"

namespace sgdg {

cudaError_t launch_csr_spmv(const DevCSR& A, const double* x, double* y, cudaStream_t st);
cudaError_t mf_bounds_violations(unsigned int* out, bool reset);
cudaError_t csr_bounds_violations(unsigned int* out, bool reset);
cudaError_t asm_bounds_violations(unsigned int* out, bool reset);
cudaError_t launch_csr_rk4_batch(const DevCSR& A, int64_t nb, int64_t bs, const double* uin, double* y, double* acc,
                                 double* uout, double dt, int stage, cudaStream_t st);
cudaError_t launch_csr_rk4(const DevCSR& A, const double* uin, double* y, double* acc, double* uout, double dt,
                           int stage, cudaStream_t st);
cudaError_t launch_csr_spmv_multi(const DevCSR& A, int nv, const double* x, int64_t xi, int64_t xs, double* y,
                                  int64_t yi, int64_t ys, cudaStream_t st);
cudaError_t launch_vlasov_points(const double* v, const double* F, const double* pt, int D, int64_t n, double* out,
                                 cudaStream_t st);
cudaError_t launch_wait_selftest(const int* ctr, int need, int* err, cudaStream_t st);
cudaError_t launch_convert_selftest(const double* x, int64_t n, unsigned long long* bad, cudaStream_t st);

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }

// ------------------------------------------------------- plain form ----
}  // namespace sgdg

using namespace sgdg;

// ------------------------------------------------------------ handles ----
struct sgdg_op {
    SparseIndex ix;
    std::shared_ptr<const DLF1D> dlf;
    int basis = SGDG_BASIS_HIER;  // SGDG_BASIS_POS: the 1D position-basis operators
    std::vector<std::unique_ptr<CSR>> dd;  // D_d, built on demand
    std::unique_ptr<CSR> lap, wave;
    std::map<int, std::unique_ptr<DeviceCSR>> dev;  // plain-form device copies by `which`
    std::map<int, std::unique_ptr<MFEngine>> mf_apply;
    cudaStream_t stream = nullptr;

    const CSR& get(int which) {
        const int D = ix.D;
        if (basis == SGDG_BASIS_POS) {
            if (which != 1 && which != SGDG_OP_LAPLACIAN && which != SGDG_OP_WAVE_RHS)
                throw Error(SGDG_EINVAL, "operator selector must be 1, 0 (laplacian) or -1 (wave RHS)");
            if (!lap) {
                dd[0].reset(new CSR());
                lap.reset(new CSR());
                pos_operators(ix.k, ix.n, dd[0].get(), lap.get());
            }
            if (which == 1) return *dd[0];
            if (which == SGDG_OP_LAPLACIAN) return *lap;
            if (!wave) wave.reset(new CSR(wave_rhs(*lap)));
            return *wave;
        }
        if (which >= 1 && which <= D) {
            if (!dd[which - 1]) dd[which - 1].reset(new CSR(assemble_dd(ix, *dlf, which - 1)));
            return *dd[which - 1];
        }
        if (which == SGDG_OP_LAPLACIAN || which == SGDG_OP_WAVE_RHS) {
            if (!lap) {
                std::vector<const CSR*> v;
                for (int d = 1; d <= D; d++) v.push_back(&get(d));
                lap.reset(new CSR(spgemm_sum(v)));
            }
            if (which == SGDG_OP_LAPLACIAN) return *lap;
            if (!wave) wave.reset(new CSR(wave_rhs(*lap)));
            return *wave;
        }
        throw Error(SGDG_EINVAL, "operator selector must be 1..D, 0 (laplacian) or -1 (wave RHS)");
    }
    const DevCSR& device(int which) {
        auto it = dev.find(which);
        if (it == dev.end())
            it = dev.emplace(which, basis == SGDG_BASIS_POS ? to_device(get(which), stream)
                                                            : gpu_operator(ix, *dlf, which, stream))
                     .first;
        return it->second->d;
    }
    ~sgdg_op() {
        dev.clear();
        mf_apply.clear();
        if (stream) cudaStreamDestroy(stream);
    }
};

// ----------------------------------------------------------- Vlasov ----
// Operators of vlasov_evolve (src/pdes.jl:131-227) for D space dimensions:
// phase space of P = 2D dimensions (x_1..x_D, p_1..p_D), grad_matrix(P), the
// four nodal transforms and the velocity points v_d = n2p m2n (2 p_d - 1).
// The device operators are assembled on the GPU when the handle first goes
// there; the host copies of the transforms are built only when asked for
// (export), and the velocity points with the device transforms when a GPU
// is present, else with the host ones.
struct sgdg_vlasov {
    int D = 0, P = 0, k = 0, n = 0;
    SparseIndex ix;
    std::shared_ptr<const DLF1D> dlf;
    mutable std::unique_ptr<CSR> T[4];    // m2n, n2p, p2n, n2m on the host, built on request
    mutable std::vector<double> v_point;  // D x N, built on request
    mutable bool have_vpoint = false;
    std::vector<std::unique_ptr<DeviceCSR>> dDs;
    std::unique_ptr<DeviceCSR> dT[4];
    DevBuf vpt, F, t, s, p, c, z;  // t, s, p: P vectors each, interleaved (t[i * P + d])
    cudaStream_t stream = nullptr;
    ~sgdg_vlasov() {
        if (stream) cudaStreamDestroy(stream);
    }
    const CSR& host_transform(int w) const {
        if (!T[w]) T[w].reset(new CSR(transform_dd(ix, transform_1d(k, n, w))));
        return *T[w];
    }
    // modal coefficients of 2 p_d - 1: 1/sqrt(3) on mode 2 along dimension D + d
    // of the first block (the tensor product with 1), src/pdes.jl:166-172
    std::vector<double> v_modal(int d) const {
        std::vector<double> vm(ix.N, 0.0);
        vm[(size_t)std::pow((double)k, (double)(D + d))] = 1.0 / std::sqrt(3.0);
        return vm;
    }
    void vpoint_host() const {  // n2p m2n on the host
        const int64_t N = ix.N;
        v_point.assign((size_t)D * N, 0.0);
        std::vector<double> tmp(N), pt(N);
        auto spmv = [&](const CSR& A, const std::vector<double>& x, std::vector<double>& y) {
            for (int64_t i = 0; i < A.m; i++) {
                double acc = 0.0;
                for (int64_t q = A.rowptr[i]; q < A.rowptr[i + 1]; q++) acc += A.val[q] * x[A.col[q]];
                y[i] = acc;
            }
        };
        for (int d = 0; d < D; d++) {
            spmv(host_transform(0), v_modal(d), tmp);
            spmv(host_transform(1), tmp, pt);
            std::copy(pt.begin(), pt.end(), v_point.begin() + (size_t)d * N);
        }
        have_vpoint = true;
    }
    void to_gpu() {
        if (stream) return;
        require_gpu();
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        // the phase-space derivatives keep 8 entries per lane, like the transforms they feed
        // (at 32 the Vlasov plain step took 2.67 ms against 2.60)
        for (int d = 0; d < P; d++) dDs.push_back(gpu_operator(ix, *dlf, d + 1, stream, kCsrLaneEntriesMulti));
        for (int w = 0; w < 4; w++) dT[w] = gpu_transform(ix, transform_1d(k, n, w), stream);
        if (!have_vpoint) {  // n2p m2n with the device transforms
            const size_t b = sizeof(double) * (size_t)ix.N;
            DevBuf x(b), y(b), w(b);
            v_point.assign((size_t)D * ix.N, 0.0);
            for (int d = 0; d < D; d++) {
                const std::vector<double> vm = v_modal(d);
                CK(cudaMemcpyAsync(x.p, vm.data(), b, cudaMemcpyHostToDevice, stream));
                CK(launch_csr_spmv(dT[0]->d, x.as<double>(), y.as<double>(), stream));
                CK(launch_csr_spmv(dT[1]->d, y.as<double>(), w.as<double>(), stream));
                CK(cudaMemcpyAsync(v_point.data() + (size_t)d * ix.N, w.p, b, cudaMemcpyDeviceToHost, stream));
            }
            CK(cudaStreamSynchronize(stream));
            have_vpoint = true;
        }
        vpt = upload(v_point, stream);
        const size_t b = sizeof(double) * (size_t)ix.N;
        F.alloc(b * D);
        t.alloc(b * P);
        s.alloc(b * P);
        p.alloc(b * P);
        c.alloc(b);
        z.alloc(b);
    }
    // z = p2n (-sum_d v_d .* n2p m2n Dx_d u + sum_d F_d .* n2p m2n Dp_d u):
    // the P derivatives, interleaved (the P values of one coefficient share a
    // sector), then each transform on all P of them in one pass over its
    // matrix, the point products, and p2n
    cudaError_t rhs_points(const double* u) {
        const int64_t N = ix.N;
        double *tt = t.as<double>(), *ss = s.as<double>(), *pp = p.as<double>();
        cudaError_t e = cudaSuccess;
        for (int d = 0; d < P && e == cudaSuccess; d++)
            e = launch_csr_spmv_multi(dDs[d]->d, 1, u, 1, 0, tt + d, P, 0, stream);
        if (e == cudaSuccess) e = launch_csr_spmv_multi(dT[0]->d, P, tt, P, 1, ss, P, 1, stream);
        if (e == cudaSuccess) e = launch_csr_spmv_multi(dT[1]->d, P, ss, P, 1, pp, P, 1, stream);
        if (e == cudaSuccess) e = launch_vlasov_points(vpt.as<double>(), F.as<double>(), pp, D, N, c.as<double>(), stream);
        if (e == cudaSuccess) e = launch_csr_spmv(dT[2]->d, c.as<double>(), z.as<double>(), stream);
        return e;
    }
};

struct sgdg_batch {
    MFEngine eng;  // its destructor frees device memory only, never touches a stream
    cudaStream_t own = nullptr;
    ~sgdg_batch() {
        if (own) cudaStreamDestroy(own);
    }
};

static void copy_str(const std::string& s, char* buf, size_t len) {
    if (!buf || len == 0) return;
    size_t n = std::min(len - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
}

static cudaStream_t op_stream(sgdg_op* op) {
    require_gpu();
    if (!op->stream) CK(cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking));
    return op->stream;
}

// Point weights of the matrix-free Vlasov right-hand side: term d < Dx is
// -v_d .* (x-derivative), term Dx + d is F_d .* (p-derivative); each weight as
// an FP32 (hi, lo) pair (a rounded weight would perturb the operator
// systematically).  Layout: hi of all 2 Dx terms, then lo.
static std::vector<float> vlasov_weights(const SparseIndex& ix, int Dx, const double* F) {
    const int64_t N = ix.N;
    const int P = 2 * Dx;
    const std::vector<double> v = vlasov_velocity_points(ix, Dx);
    std::vector<float> w((size_t)2 * P * N);
    for (int t = 0; t < P; t++)
        for (int64_t e = 0; e < N; e++) {
            const double x = t < Dx ? -v[(size_t)t * N + e] : F[(size_t)(t - Dx) * N + e];
            const float hi = (float)x;
            w[(size_t)t * N + e] = hi;
            w[((size_t)P + t) * N + e] = (float)(x - (double)hi);
        }
    return w;
}

// nodal transforms: the D-dimensional restricted Kronecker product of a 1D map
static CSR build_transform(int D, int k, int n, int scheme, int which) {
    if (which < 0 || which > 3) throw Error(SGDG_EINVAL, "transform must be 0..3 (m2n, n2p, p2n, n2m)");
    return transform_dd(make_index(D, k, n, scheme), transform_1d(k, n, which));
}

static void export_csr(const CSR& A, int64_t* rowptr, int32_t* col, double* val) {
    std::memcpy(rowptr, A.rowptr.data(), sizeof(int64_t) * A.rowptr.size());
    if (A.nnz()) {
        std::memcpy(col, A.col.data(), sizeof(int32_t) * A.col.size());
        std::memcpy(val, A.val.data(), sizeof(double) * A.val.size());
    }
}

extern "C" {

// ---------------------------------------------------- nodal transforms ----

int sgdg_version(char* buf, size_t len) {
    copy_str("sgdg 0.1 (sm_103a)", buf, len);
    return SGDG_OK;
}

int sgdg_last_error(char* buf, size_t len) {
    copy_str(g_err, buf, len);
    return SGDG_OK;
}

int sgdg_get_size(int D, int k, int n, int scheme, int64_t* N) {
    API_BEGIN
    NEED(N);
    *N = make_index(D, k, n, scheme).N;
    API_END
}

int sgdg_index_map(int D, int k, int n, int scheme, int32_t* level, int32_t* cell, int32_t* mode) {
    API_BEGIN
    NEED(level);
    NEED(cell);
    NEED(mode);
    SparseIndex ix = make_index(D, k, n, scheme);
    int64_t j = 0;
    for (int b = 0; b < ix.nlev; b++) {
        const int* L = &ix.levels[(size_t)b * D];
        for (int64_t cl = 0; cl < ix.lev_cells[b]; cl++)
            for (int64_t ml = 0; ml < ix.kD; ml++) {
                int64_t c = cl, m = ml;
                for (int q = 0; q < D; q++) {
                    level[j * D + q] = L[q];
                    int64_t nc = ncells(L[q]);
                    cell[j * D + q] = int32_t(c % nc) + 1;
                    c /= nc;
                    mode[j * D + q] = int32_t(m % k) + 1;
                    m /= k;
                }
                j++;
            }
    }
    API_END
}

int sgdg_dg_coeffs(int k, double* out) {
    API_BEGIN
    NEED(out);
    const Basis1D& B = basis(k);
    std::memcpy(out, B.dg.data(), sizeof(double) * B.dg.size());
    API_END
}

static CSR dlf_csr(int k, int n) {
    auto op = dlf1d(k, n);
    CSR A;
    A.m = A.n = int64_t(k) << n;
    A.rowptr.assign(A.m + 1, 0);
    for (int rb = 0; rb < op->nblocks; rb++)
        for (int i = 0; i < k; i++) {
            int64_t row = (int64_t)rb * k + i;
            for (int p = op->rowptr[rb]; p < op->rowptr[rb + 1]; p++)
                for (int j = 0; j < k; j++) {
                    A.col.push_back(op->colblk[p] * k + j);
                    A.val.push_back(op->val[(size_t)p * k * k + i * k + j]);
                }
            A.rowptr[row + 1] = (int64_t)A.col.size();
        }
    return A;
}

int sgdg_dlf_1d_nnz(int k, int n, int64_t* nnz) {
    API_BEGIN
    NEED(nnz);
    basis(k);
    auto op = dlf1d(k, n);
    *nnz = (int64_t)op->colblk.size() * k * k;
    API_END
}

int sgdg_dlf_1d_export(int k, int n, int64_t* rowptr, int32_t* col, double* val) {
    API_BEGIN
    NEED(rowptr);
    NEED(col);
    NEED(val);
    CSR A = dlf_csr(k, n);
    std::memcpy(rowptr, A.rowptr.data(), sizeof(int64_t) * A.rowptr.size());
    std::memcpy(col, A.col.data(), sizeof(int32_t) * A.col.size());
    std::memcpy(val, A.val.data(), sizeof(double) * A.val.size());
    API_END
}

int sgdg_op_create(int D, int k, int n, int scheme, sgdg_op** out) {
    API_BEGIN
    NEED(out);
    *out = nullptr;
    if (n < 2) throw Error(SGDG_EINVAL, "n must be >= 2");
    auto op = std::make_unique<sgdg_op>();
    op->ix = make_index(D, k, n, scheme);
    op->dlf = dlf1d(k, n);
    op->dd.resize(D);
    *out = op.release();
    API_END
}

int sgdg_op_create_1d(int k, int n, int basis, sgdg_op** out) {
    API_BEGIN
    NEED(out);
    *out = nullptr;
    if (basis != SGDG_BASIS_HIER && basis != SGDG_BASIS_POS)
        throw Error(SGDG_EINVAL, "basis must be SGDG_BASIS_HIER (0) or SGDG_BASIS_POS (1)");
    if (n < 2) throw Error(SGDG_EINVAL, "n must be >= 2");
    auto op = std::make_unique<sgdg_op>();
    op->ix = make_index(1, k, n, SGDG_SCHEME_SPARSE);
    op->dlf = dlf1d(k, n);
    op->dd.resize(1);
    op->basis = basis;
    *out = op.release();
    API_END
}

int sgdg_op_destroy(sgdg_op* op) {
    API_BEGIN
    delete op;
    API_END
}

int sgdg_op_size(const sgdg_op* op, int64_t* N) {
    API_BEGIN
    NEED(op);
    NEED(N);
    *N = op->ix.N;
    API_END
}

int sgdg_op_nnz(sgdg_op* op, int which, int64_t* nnz) {
    API_BEGIN
    NEED(op);
    NEED(nnz);
    *nnz = op->get(which).nnz();
    API_END
}

int sgdg_op_device_nnz(sgdg_op* op, int which, int64_t* nnz) {
    API_BEGIN
    NEED(op);
    NEED(nnz);
    op_stream(op);
    *nnz = op->device(which).nnz;
    API_END
}

int sgdg_op_export_device_csr(sgdg_op* op, int which, int64_t* rowptr, int32_t* col, double* val) {
    API_BEGIN
    NEED(op);
    NEED(rowptr);
    NEED(col);
    NEED(val);
    cudaStream_t st = op_stream(op);
    op->device(which);
    const CSR A = download_csr(*op->dev.at(which), st);
    std::memcpy(rowptr, A.rowptr.data(), sizeof(int64_t) * A.rowptr.size());
    std::memcpy(col, A.col.data(), sizeof(int32_t) * A.col.size());
    std::memcpy(val, A.val.data(), sizeof(double) * A.val.size());
    API_END
}

int sgdg_op_export_csr(sgdg_op* op, int which, int64_t* rowptr, int32_t* col, double* val) {
    API_BEGIN
    NEED(op);
    NEED(rowptr);
    NEED(col);
    NEED(val);
    const CSR& A = op->get(which);
    std::memcpy(rowptr, A.rowptr.data(), sizeof(int64_t) * A.rowptr.size());
    std::memcpy(col, A.col.data(), sizeof(int32_t) * A.col.size());
    std::memcpy(val, A.val.data(), sizeof(double) * A.val.size());
    API_END
}

static void apply_device_impl(sgdg_op* op, int which, int method, const double* x, double* y, cudaStream_t st) {
    if (method == SGDG_METHOD_PLAIN) {
        const DevCSR& A = op->device(which);
        CK(launch_csr_spmv(A, x, y, st));
        return;
    }
    if (method != SGDG_METHOD_MATFREE) throw Error(SGDG_EINVAL, "method must be PLAIN (0) or MATFREE (1)");
    if (op->basis != SGDG_BASIS_HIER) throw Error(SGDG_EUNSUPPORTED, "the matrix-free form is hierarchical only");
    if (!(which == SGDG_OP_LAPLACIAN || (which >= 1 && which <= op->ix.D)))
        throw Error(SGDG_EUNSUPPORTED, "matrix-free apply supports which = 1..D or 0 (laplacian)");
    auto it = op->mf_apply.find(which);
    if (it == op->mf_apply.end()) {
        auto eng = std::make_unique<MFEngine>(st);
        SolveSpec sp{};
        sp.kind = which == SGDG_OP_LAPLACIAN ? MF_KIND_WAVE : MF_KIND_ADVECT;
        sp.D = op->ix.D;
        sp.k = op->ix.k;
        sp.n = op->ix.n;
        sp.scheme = op->ix.scheme;
        sp.dt = 0.0;
        sp.apply = true;
        sp.apply_dim = which >= 1 ? which - 1 : -1;
        eng->add(sp, nullptr);
        it = op->mf_apply.emplace(which, std::move(eng)).first;
    }
    it->second->set_stream(st);
    it->second->apply(x, y);
}

int sgdg_apply(sgdg_op* op, int which, int method, const double* x, double* y) {
    API_BEGIN
    NEED(op);
    NEED(x);
    NEED(y);
    cudaStream_t st = op_stream(op);
    const int64_t len = which == SGDG_OP_WAVE_RHS ? 2 * op->ix.N : op->ix.N;
    DevBuf dx(sizeof(double) * len), dy(sizeof(double) * len);
    CK(cudaMemcpyAsync(dx.p, x, sizeof(double) * len, cudaMemcpyHostToDevice, st));
    apply_device_impl(op, which, method, dx.as<double>(), dy.as<double>(), st);
    CK(cudaMemcpyAsync(y, dy.p, sizeof(double) * len, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    API_END
}

int sgdg_apply_device(sgdg_op* op, int which, int method, const double* x_dev, double* y_dev, void* stream) {
    API_BEGIN
    NEED(op);
    NEED(x_dev);
    NEED(y_dev);
    require_gpu();
    apply_device_impl(op, which, method, x_dev, y_dev, (cudaStream_t)stream);
    API_END
}

static std::vector<int64_t> out_steps(int64_t nsteps, int nout) {
    std::vector<int64_t> s(nout);
    for (int i = 0; i < nout; i++) s[i] = (int64_t)((__int128)nsteps * i / (nout - 1));
    return s;
}

static void plain_evolve(sgdg_op* op, int which_or_adv, const DeviceCSR* Aadv, const double* y0, int64_t len,
                         double t0, double t1, int64_t nsteps, int nout, double* times, double* states) {
    cudaStream_t st = op_stream(op);
    const DevCSR* A = Aadv ? &Aadv->d : &op->device(which_or_adv);
    DevBuf y(sizeof(double) * len), acc(sizeof(double) * len), u0(sizeof(double) * len), u1(sizeof(double) * len);
    CK(cudaMemcpyAsync(y.p, y0, sizeof(double) * len, cudaMemcpyHostToDevice, st));
    const double dt = (t1 - t0) / double(nsteps);
    // one RK4 step as a graph
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = launch_csr_rk4(*A, y.as<double>(), y.as<double>(), acc.as<double>(), u0.as<double>(), dt, 1, st);
    if (e == cudaSuccess)
        e = launch_csr_rk4(*A, u0.as<double>(), y.as<double>(), acc.as<double>(), u1.as<double>(), dt, 2, st);
    if (e == cudaSuccess)
        e = launch_csr_rk4(*A, u1.as<double>(), y.as<double>(), acc.as<double>(), u0.as<double>(), dt, 3, st);
    if (e == cudaSuccess)
        e = launch_csr_rk4(*A, u0.as<double>(), y.as<double>(), acc.as<double>(), u1.as<double>(), dt, 4, st);
    cudaError_t e2 = cudaStreamEndCapture(st, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        throw Error(SGDG_ECUDA, std::string("capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    cudaError_t e3 = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) throw Error(SGDG_ECUDA, std::string("instantiate: ") + cudaGetErrorString(e3));
    auto steps = out_steps(nsteps, nout);
    int64_t done = 0;
    cudaError_t err = cudaSuccess;
    for (int i = 0; i < nout && err == cudaSuccess; i++) {
        for (; done < steps[i] && err == cudaSuccess; done++) err = cudaGraphLaunch(ge, st);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(states + (size_t)i * len, y.p, sizeof(double) * len, cudaMemcpyDeviceToHost, st);
        if (times) times[i] = t0 + (t1 - t0) * double(steps[i]) / double(nsteps);
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    cudaGraphExecDestroy(ge);
    if (err != cudaSuccess) throw Error(SGDG_ECUDA, std::string("evolve: ") + cudaGetErrorString(err));
}

// nsteps plain FP64 RK4 steps of nsolves solves y' = A y sharing operator
// `which`, states device-resident one after another; one RK4 step (four
// batched stage launches) is captured as a graph and replayed.
static void plain_batch_steps(sgdg_op* op, int which, int64_t nsolves, double* y, double dt, int64_t nsteps,
                              cudaStream_t st) {
    const DevCSR& A = op->device(which);
    const int64_t len = A.m, total = nsolves * len;
    DevBuf acc(sizeof(double) * total), u0(sizeof(double) * total), u1(sizeof(double) * total);
    cudaStream_t cs = st;
    cudaStream_t own = nullptr;
    if (cs == nullptr) {  // graphs cannot be captured on the legacy stream
        CK(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
        cs = own;
        CK(cudaStreamSynchronize(nullptr));
    }
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    double* a = acc.as<double>();
    double* p0 = u0.as<double>();
    double* p1 = u1.as<double>();
    cudaError_t e = launch_csr_rk4_batch(A, nsolves, len, y, y, a, p0, dt, 1, cs);
    if (e == cudaSuccess) e = launch_csr_rk4_batch(A, nsolves, len, p0, y, a, p1, dt, 2, cs);
    if (e == cudaSuccess) e = launch_csr_rk4_batch(A, nsolves, len, p1, y, a, p0, dt, 3, cs);
    if (e == cudaSuccess) e = launch_csr_rk4_batch(A, nsolves, len, p0, y, a, p1, dt, 4, cs);
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (own) cudaStreamDestroy(own);
        throw Error(SGDG_ECUDA, std::string("capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    cudaError_t e3 = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) {
        if (own) cudaStreamDestroy(own);
        throw Error(SGDG_ECUDA, std::string("instantiate: ") + cudaGetErrorString(e3));
    }
    cudaError_t err = cudaSuccess;
    for (int64_t i = 0; i < nsteps && err == cudaSuccess; i++) err = cudaGraphLaunch(ge, cs);
    // the scratch vectors are freed on return: wait for the steps
    if (err == cudaSuccess) err = cudaStreamSynchronize(cs);
    cudaGraphExecDestroy(ge);
    if (own) cudaStreamDestroy(own);
    if (err != cudaSuccess) throw Error(SGDG_ECUDA, std::string("plain batch: ") + cudaGetErrorString(err));
}

static void mf_evolve(sgdg_op* op, int kind, const double* a, const double* y0, int64_t len, double t0, double t1,
                      int64_t nsteps, int nout, double* times, double* states) {
    if (op->basis != SGDG_BASIS_HIER) throw Error(SGDG_EUNSUPPORTED, "the matrix-free form is hierarchical only");
    cudaStream_t st = op_stream(op);
    MFEngine eng(st);
    SolveSpec sp{};
    sp.kind = kind;
    sp.D = op->ix.D;
    sp.k = op->ix.k;
    sp.n = op->ix.n;
    sp.scheme = op->ix.scheme;
    for (int d = 0; d < sp.D; d++) sp.a[d] = a ? a[d] : 0.0;
    sp.dt = (t1 - t0) / double(nsteps);
    sp.apply_dim = -1;
    int id = eng.add(sp, y0);
    auto steps = out_steps(nsteps, nout);
    int64_t done = 0;
    for (int i = 0; i < nout; i++) {
        eng.step(steps[i] - done);
        done = steps[i];
        eng.get_state(id, states + (size_t)i * len);
        if (times) times[i] = t0 + (t1 - t0) * double(steps[i]) / double(nsteps);
    }
}

static void check_evolve_args(int64_t nsteps, int nout, double t0, double t1) {
    if (nsteps < 1) throw Error(SGDG_EINVAL, "nsteps must be >= 1");
    if (nout < 2) throw Error(SGDG_EINVAL, "nout must be >= 2");
    if (!(std::isfinite(t0) && std::isfinite(t1)) || t1 == t0) throw Error(SGDG_EINVAL, "need finite t0 != t1");
}

int sgdg_op_plain_steps_device(sgdg_op* op, int which, int64_t nsolves, double* y_dev, double dt, int64_t nsteps,
                               void* stream) {
    API_BEGIN
    NEED(op);
    NEED(y_dev);
    if (nsolves < 1) throw Error(SGDG_EINVAL, "nsolves must be >= 1");
    if (nsteps < 0) throw Error(SGDG_EINVAL, "nsteps must be >= 0");
    if (!std::isfinite(dt)) throw Error(SGDG_EINVAL, "dt must be finite");
    require_gpu();
    if (nsteps > 0) plain_batch_steps(op, which, nsolves, y_dev, dt, nsteps, (cudaStream_t)stream);
    API_END
}

int sgdg_debug_bounds(int* checked, int64_t* violations, int reset) {
    API_BEGIN
    NEED(checked);
    NEED(violations);
    *violations = 0;
#ifdef SGDG_DEBUG
    *checked = 1;
#else
    *checked = 0;
    return SGDG_OK;  // nothing is checked (or counted) in this build
#endif
    require_gpu();
    unsigned int v = 0;
    for (auto f : {mf_bounds_violations, csr_bounds_violations, asm_bounds_violations}) {
        CK(f(&v, reset != 0));
        *violations += v;
    }
    API_END
}

int sgdg_wave_evolve(sgdg_op* op, const double* f0, const double* v0, double t0, double t1, int64_t nsteps, int nout,
                     int method, double* times, double* states) {
    API_BEGIN
    NEED(op);
    NEED(f0);
    NEED(v0);
    NEED(states);
    check_evolve_args(nsteps, nout, t0, t1);
    const int64_t N = op->ix.N;
    std::vector<double> y0(2 * N);
    std::memcpy(y0.data(), f0, sizeof(double) * N);
    std::memcpy(y0.data() + N, v0, sizeof(double) * N);
    if (method == SGDG_METHOD_PLAIN)
        plain_evolve(op, SGDG_OP_WAVE_RHS, nullptr, y0.data(), 2 * N, t0, t1, nsteps, nout, times, states);
    else if (method == SGDG_METHOD_MATFREE)
        mf_evolve(op, MF_KIND_WAVE, nullptr, y0.data(), 2 * N, t0, t1, nsteps, nout, times, states);
    else
        throw Error(SGDG_EINVAL, "method must be PLAIN (0) or MATFREE (1)");
    API_END
}

int sgdg_advect_evolve(sgdg_op* op, const double* a, const double* f0, double t0, double t1, int64_t nsteps, int nout,
                       int method, double* times, double* states) {
    API_BEGIN
    NEED(op);
    NEED(a);
    NEED(f0);
    NEED(states);
    check_evolve_args(nsteps, nout, t0, t1);
    if (op->basis != SGDG_BASIS_HIER) throw Error(SGDG_EUNSUPPORTED, "advection is hierarchical only");
    const int64_t N = op->ix.N;
    if (method == SGDG_METHOD_PLAIN) {
        // -sum_d a_d D_d, assembled on the GPU (the same entries as add_scaled)
        std::vector<double> s;
        for (int d = 1; d <= op->ix.D; d++) s.push_back(-a[d - 1]);
        auto A = gpu_scaled_sum(op->ix, *op->dlf, s.data(), op_stream(op));
        plain_evolve(op, 0, A.get(), f0, N, t0, t1, nsteps, nout, times, states);
    } else if (method == SGDG_METHOD_MATFREE) {
        mf_evolve(op, MF_KIND_ADVECT, a, f0, N, t0, t1, nsteps, nout, times, states);
    } else {
        throw Error(SGDG_EINVAL, "method must be PLAIN (0) or MATFREE (1)");
    }
    API_END
}

int sgdg_transform_1d_nnz(int k, int n, int which, int64_t* nnz) {
    API_BEGIN
    NEED(nnz);
    *nnz = transform_1d(k, n, which).nnz();
    API_END
}

int sgdg_transform_1d_export(int k, int n, int which, int64_t* rowptr, int32_t* col, double* val) {
    API_BEGIN
    NEED(rowptr);
    export_csr(transform_1d(k, n, which), rowptr, col, val);
    API_END
}

int sgdg_transform_nnz(int D, int k, int n, int scheme, int which, int64_t* nnz) {
    API_BEGIN
    NEED(nnz);
    *nnz = build_transform(D, k, n, scheme, which).nnz();
    API_END
}

int sgdg_transform_export(int D, int k, int n, int scheme, int which, int64_t* rowptr, int32_t* col, double* val) {
    API_BEGIN
    NEED(rowptr);
    export_csr(build_transform(D, k, n, scheme, which), rowptr, col, val);
    API_END
}

int sgdg_transform_device_export(int D, int k, int n, int scheme, int which, int64_t* nnz, int64_t* rowptr,
                                 int32_t* col, double* val) {
    API_BEGIN
    NEED(nnz);
    if (which < 0 || which > 3) throw Error(SGDG_EINVAL, "transform must be 0..3 (m2n, n2p, p2n, n2m)");
    if (k != 2 && k != 3 && k != 5) throw Error(SGDG_EINVAL, "the nodal basis exists for k = 2, 3, 5");
    require_gpu();
    const SparseIndex ix = make_index(D, k, n, scheme);
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    std::unique_ptr<DeviceCSR> A;
    try {
        A = gpu_transform(ix, transform_1d(k, n, which), st);
        const CSR h = download_csr(*A, st);
        *nnz = h.nnz();
        if (rowptr && col && val) export_csr(h, rowptr, col, val);
    } catch (...) {
        A.reset();
        cudaStreamDestroy(st);
        throw;
    }
    A.reset();
    cudaStreamDestroy(st);
    API_END
}

// ------------------------------------------------------------- Vlasov ----
int sgdg_vlasov_create(int D, int k, int n, int scheme, sgdg_vlasov** out) {
    API_BEGIN
    NEED(out);
    if (D < 1 || 2 * D > 8) throw Error(SGDG_EINVAL, "D (space dimensions) must be 1..4");
    if (k != 2 && k != 3 && k != 5) throw Error(SGDG_EINVAL, "the nodal basis exists for k = 2, 3, 5");
    auto v = std::make_unique<sgdg_vlasov>();
    v->D = D;
    v->P = 2 * D;
    v->k = k;
    v->n = n;
    v->ix = make_index(v->P, k, n, scheme);
    v->dlf = dlf1d(k, n);
    *out = v.release();
    API_END
}

int sgdg_vlasov_destroy(sgdg_vlasov* v) {
    API_BEGIN
    delete v;
    API_END
}

int sgdg_vlasov_size(const sgdg_vlasov* v, int64_t* N) {
    API_BEGIN
    NEED(v);
    NEED(N);
    *N = v->ix.N;
    API_END
}

int sgdg_vlasov_v_point(const sgdg_vlasov* v, double* out) {
    API_BEGIN
    NEED(v);
    NEED(out);
    if (!v->have_vpoint) {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0)
            const_cast<sgdg_vlasov*>(v)->to_gpu();
        else {
            cudaGetLastError();
            v->vpoint_host();
        }
    }
    std::copy(v->v_point.begin(), v->v_point.end(), out);
    API_END
}

int sgdg_vlasov_transform_nnz(const sgdg_vlasov* v, int which, int64_t* nnz) {
    API_BEGIN
    NEED(v);
    NEED(nnz);
    if (which < 0 || which > 3) throw Error(SGDG_EINVAL, "transform must be 0..3 (m2n, n2p, p2n, n2m)");
    *nnz = v->host_transform(which).nnz();
    API_END
}

int sgdg_vlasov_transform_export(const sgdg_vlasov* v, int which, int64_t* rowptr, int32_t* col, double* val) {
    API_BEGIN
    NEED(v);
    NEED(rowptr);
    if (which < 0 || which > 3) throw Error(SGDG_EINVAL, "transform must be 0..3 (m2n, n2p, p2n, n2m)");
    export_csr(v->host_transform(which), rowptr, col, val);
    API_END
}

int sgdg_vlasov_write_h5(const sgdg_vlasov* v, const char* path, int64_t nout, const double* times,
                         const double* states) {
    API_BEGIN
    NEED(v);
    NEED(path);
    if (nout < 0) throw Error(SGDG_EINVAL, "nout must be >= 0");
    if (nout > 0) {
        NEED(times);
        NEED(states);
    }
    H5Writer w(path);
    w.scalar_i64("dimensions", v->D);
    w.scalar_i64("order", v->k);
    w.scalar_i64("levels", v->n);
    static const char* names[4] = {"m2n", "n2p", "p2n", "n2m"};
    for (int t = 0; t < 4; t++) h5_write_csc(w, names[t], v->host_transform(t));
    for (int d = 0; d < v->P; d++)  // Ds[1] .. Ds[2D]: the 1-based names of the 0-based dimensions
        h5_write_csc(w, "Ds[" + std::to_string(d + 1) + "]", assemble_dd(v->ix, *v->dlf, d));
    if (nout > 0) {
        const int64_t N = v->ix.N;
        w.array_f64("times", times, nout);
        for (int64_t i = 0; i < nout; i++) {
            char name[32];
            std::snprintf(name, sizeof name, "f_modal.%06lld", (long long)(i + 1));
            w.array_f64(name, states + i * N, N);
        }
    }
    w.close();
    API_END
}

int sgdg_vlasov_rhs(sgdg_vlasov* v, const double* F_point, const double* f, double* out) {
    API_BEGIN
    NEED(v);
    NEED(F_point);
    NEED(f);
    NEED(out);
    v->to_gpu();
    const int64_t N = v->ix.N;
    const size_t b = sizeof(double) * (size_t)N;
    DevBuf u(b), r(b);
    CK(cudaMemcpyAsync(v->F.p, F_point, b * v->D, cudaMemcpyHostToDevice, v->stream));
    CK(cudaMemcpyAsync(u.p, f, b, cudaMemcpyHostToDevice, v->stream));
    CK(v->rhs_points(u.as<double>()));
    CK(launch_csr_spmv(v->dT[3]->d, v->z.as<double>(), r.as<double>(), v->stream));
    CK(cudaMemcpyAsync(out, r.p, b, cudaMemcpyDeviceToHost, v->stream));
    CK(cudaStreamSynchronize(v->stream));
    API_END
}

int sgdg_vlasov_evolve(sgdg_vlasov* v, const double* F_point, const double* f0, double t0, double t1, int64_t nsteps,
                       int nout, int method, double* times, double* states) {
    API_BEGIN
    NEED(v);
    NEED(F_point);
    NEED(f0);
    NEED(states);
    check_evolve_args(nsteps, nout, t0, t1);
    if (method == SGDG_METHOD_MATFREE) {
        if (!v->stream) {
            require_gpu();
            CK(cudaStreamCreateWithFlags(&v->stream, cudaStreamNonBlocking));
        }
        MFEngine eng(v->stream);
        SolveSpec sp{};
        sp.kind = MF_KIND_VLASOV;
        sp.D = v->P;
        sp.k = v->k;
        sp.n = v->n;
        sp.scheme = v->ix.scheme;
        sp.dt = (t1 - t0) / double(nsteps);
        sp.apply_dim = -1;
        const std::vector<float> w = vlasov_weights(v->ix, v->D, F_point);
        const int id = eng.add(sp, f0, w.data());
        auto steps = out_steps(nsteps, nout);
        int64_t done = 0;
        for (int i = 0; i < nout; i++) {
            eng.step(steps[i] - done);
            done = steps[i];
            eng.get_state(id, states + (size_t)i * v->ix.N);
            if (times) times[i] = t0 + (t1 - t0) * double(steps[i]) / double(nsteps);
        }
        return SGDG_OK;
    }
    if (method != SGDG_METHOD_PLAIN) throw Error(SGDG_EINVAL, "method must be PLAIN (0) or MATFREE (1)");
    v->to_gpu();
    cudaStream_t st = v->stream;
    const int64_t N = v->ix.N;
    const size_t b = sizeof(double) * (size_t)N;
    DevBuf y(b), acc(b), u0(b), u1(b);
    CK(cudaMemcpyAsync(v->F.p, F_point, b * v->D, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(y.p, f0, b, cudaMemcpyHostToDevice, st));
    const double dt = (t1 - t0) / double(nsteps);
    // one RK4 step as a graph: per stage the right-hand side in the point
    // basis, then n2m fused with the stage update
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const double* in[4] = {y.as<double>(), u0.as<double>(), u1.as<double>(), u0.as<double>()};
    double* outv[4] = {u0.as<double>(), u1.as<double>(), u0.as<double>(), u1.as<double>()};
    cudaError_t e = cudaSuccess;
    for (int stage = 1; stage <= 4 && e == cudaSuccess; stage++) {
        e = v->rhs_points(in[stage - 1]);
        if (e == cudaSuccess)
            e = launch_csr_rk4(v->dT[3]->d, v->z.as<double>(), y.as<double>(), acc.as<double>(), outv[stage - 1], dt,
                               stage, st);
    }
    cudaError_t e2 = cudaStreamEndCapture(st, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        throw Error(SGDG_ECUDA, std::string("capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    cudaError_t e3 = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) throw Error(SGDG_ECUDA, std::string("instantiate: ") + cudaGetErrorString(e3));
    auto steps = out_steps(nsteps, nout);
    int64_t done = 0;
    cudaError_t err = cudaSuccess;
    for (int i = 0; i < nout && err == cudaSuccess; i++) {
        for (; done < steps[i] && err == cudaSuccess; done++) err = cudaGraphLaunch(ge, st);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(states + (size_t)i * N, y.p, b, cudaMemcpyDeviceToHost, st);
        if (times) times[i] = t0 + (t1 - t0) * double(steps[i]) / double(nsteps);
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    cudaGraphExecDestroy(ge);
    if (err != cudaSuccess) throw Error(SGDG_ECUDA, std::string("vlasov evolve: ") + cudaGetErrorString(err));
    API_END
}

// ------------------------------------------------------------ batches ----
int sgdg_batch_create(sgdg_batch** out) {
    API_BEGIN
    NEED(out);
    require_gpu();
    auto b = std::make_unique<sgdg_batch>();
    CK(cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking));
    b->eng.set_stream(b->own);
    *out = b.release();
    API_END
}

int sgdg_batch_destroy(sgdg_batch* b) {
    API_BEGIN
    delete b;  // cudaFree of the arenas waits for the batch's outstanding work
    API_END
}

int sgdg_batch_add(sgdg_batch* b, int kind, int D, int k, int n, int scheme, const double* a, double dt,
                   const double* y0, int* id) {
    API_BEGIN
    NEED(b);
    NEED(y0);
    NEED(id);
    if (kind != SGDG_KIND_ADVECT && kind != SGDG_KIND_WAVE) throw Error(SGDG_EINVAL, "kind must be ADVECT or WAVE");
    if (kind == SGDG_KIND_ADVECT) NEED(a);
    if (n < 2) throw Error(SGDG_EINVAL, "n must be >= 2");
    if (!std::isfinite(dt)) throw Error(SGDG_EINVAL, "dt must be finite");
    SolveSpec sp{};
    sp.kind = kind == SGDG_KIND_WAVE ? MF_KIND_WAVE : MF_KIND_ADVECT;
    sp.D = D;
    sp.k = k;
    sp.n = n;
    sp.scheme = scheme;
    for (int d = 0; d < D && d < 8; d++) sp.a[d] = a ? a[d] : 0.0;
    sp.dt = dt;
    sp.apply_dim = -1;
    *id = b->eng.add(sp, y0);
    API_END
}

int sgdg_batch_autotune(sgdg_batch* b, int* ntuned) {
    API_BEGIN
    NEED(b);
    const auto done = b->eng.autotune();
    if (ntuned) *ntuned = (int)done.size();
    API_END
}

int sgdg_tile_shape(int D, int k, int* wlog, int* coop, int* tuned) {
    API_BEGIN
    const MFTile t = mf_tile(D, k);
    if (wlog) *wlog = t.wlog;
    if (coop) *coop = t.coop;
    if (tuned) *tuned = mf_tile_tuned(D, k) ? 1 : 0;
    API_END
}

int sgdg_set_tile_shape(int D, int k, int wlog, int coop) {
    API_BEGIN
    if (D < 1 || D > 8 || k < 1 || k > 5) throw Error(SGDG_EINVAL, "tile shapes exist for 1 <= D <= 8, 1 <= k <= 5");
    mf_set_tile(D, k, MFTile{wlog, coop});
    API_END
}

int sgdg_clear_tile_shapes(void) {
    API_BEGIN
    mf_clear_tiles();
    API_END
}

int sgdg_batch_add_vlasov(sgdg_batch* b, int Dx, int k, int n, int scheme, double dt, const double* F_point,
                          const double* f0, int* id) {
    API_BEGIN
    NEED(b);
    NEED(F_point);
    NEED(f0);
    NEED(id);
    if (Dx < 1 || 2 * Dx > 8) throw Error(SGDG_EINVAL, "Dx (space dimensions) must be 1..4");
    if (!std::isfinite(dt)) throw Error(SGDG_EINVAL, "dt must be finite");
    SolveSpec sp{};
    sp.kind = MF_KIND_VLASOV;
    sp.D = 2 * Dx;
    sp.k = k;
    sp.n = n;
    sp.scheme = scheme;
    sp.dt = dt;
    sp.apply_dim = -1;
    const SparseIndex ix = make_index(sp.D, k, n, scheme);
    const std::vector<float> w = vlasov_weights(ix, Dx, F_point);
    *id = b->eng.add(sp, f0, w.data());
    API_END
}

int sgdg_batch_remove(sgdg_batch* b, int id) {
    API_BEGIN
    NEED(b);
    b->eng.remove(id);
    API_END
}

int sgdg_batch_set_stream(sgdg_batch* b, void* stream) {
    API_BEGIN
    NEED(b);
    b->eng.set_stream(stream ? (cudaStream_t)stream : b->own);
    API_END
}

int sgdg_batch_step(sgdg_batch* b, int64_t nsteps) {
    API_BEGIN
    NEED(b);
    if (nsteps < 0) throw Error(SGDG_EINVAL, "nsteps must be >= 0");
    b->eng.step(nsteps);
    API_END
}

int sgdg_batch_get_state(sgdg_batch* b, int id, double* y) {
    API_BEGIN
    NEED(b);
    NEED(y);
    b->eng.get_state(id, y);
    API_END
}

int sgdg_batch_state_size(sgdg_batch* b, int id, int64_t* len) {
    API_BEGIN
    NEED(b);
    NEED(len);
    *len = b->eng.state_size(id);
    API_END
}

int sgdg_batch_total_size(sgdg_batch* b, int64_t* len) {
    API_BEGIN
    NEED(b);
    NEED(len);
    *len = b->eng.total_size();
    API_END
}

int sgdg_batch_upload(sgdg_batch* b, const double* y_all) {
    API_BEGIN
    NEED(b);
    NEED(y_all);
    b->eng.upload_all(y_all);
    API_END
}

int sgdg_batch_download(sgdg_batch* b, double* y_all) {
    API_BEGIN
    NEED(b);
    NEED(y_all);
    b->eng.download_all(y_all);
    API_END
}

int sgdg_batch_step_host(sgdg_batch* b, const double* y_in, double* y_out, int64_t nsteps, int nchunks) {
    API_BEGIN
    NEED(b);
    NEED(y_in);
    NEED(y_out);
    b->eng.step_host(y_in, y_out, nsteps, nchunks);
    API_END
}

int sgdg_batch_step_info(sgdg_batch* b, int64_t* launches, double* dofs) {
    API_BEGIN
    NEED(b);
    if (launches) *launches = b->eng.launches_per_step();
    if (dofs) *dofs = b->eng.dof_updates_per_step();
    API_END
}

int sgdg_selftest_bounded_wait(double* seconds) {
    API_BEGIN
    require_gpu();
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    DevBuf buf(2 * sizeof(int));
    int err = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMemsetAsync(buf.p, 0, 2 * sizeof(int), st);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    // counter 0 must reach 1, and nothing ever increments it
    if (e == cudaSuccess) e = launch_wait_selftest(buf.as<int>(), 1, buf.as<int>() + 1, st);
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, buf.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) throw Error(SGDG_ECUDA, std::string("bounded wait self-test: ") + cudaGetErrorString(e));
    if (seconds) *seconds = ms / 1e3;
    if (!err) throw Error(SGDG_ECUDA, "bounded wait self-test: the wait did not report giving up");
    throw Error(SGDG_ETIMEOUT, "bounded wait gave up as designed");
    API_END
}

int sgdg_worklist_dryrun(int nclasses, const int* spec, int pass_only, int chunk, int nchunks, int64_t* items,
                         int64_t items_cap,
                         int64_t* nitems, int* nctr, int64_t* classes, int64_t* blockoff, int64_t boff_cap,
                         int64_t* nboff) {
    API_BEGIN
    NEED(spec);
    NEED(nitems);
    NEED(nboff);
    if (nclasses < 1 || nclasses > 4096) throw Error(SGDG_EINVAL, "nclasses must be in 1..4096");
    if (nchunks < 1 || nchunks > 64 || chunk < 0 || chunk >= nchunks)
        throw Error(SGDG_EINVAL, "chunk must be in 0..nchunks-1, nchunks in 1..64");
    struct Host {
        std::vector<std::vector<Pencil>> pencils;
        std::vector<int32_t> boff_index;
        std::vector<int64_t> boff;
    };
    std::vector<Host> host(nclasses);
    std::vector<WLClass> cls;
    for (int c = 0; c < nclasses; c++) {
        const int* q = spec + 8 * c;
        const int kind = q[0], D = q[1], k = q[2], n = q[3], scheme = q[4], ns = q[5], apply = q[6], adim = q[7];
        if (kind != MF_KIND_ADVECT && kind != MF_KIND_WAVE && kind != MF_KIND_VLASOV)
            throw Error(SGDG_EINVAL, "kind must be 0 (advection), 1 (wave) or 2 (Vlasov)");
        if (D < 1 || D > 8 || k < 1 || k > 5) throw Error(SGDG_EUNSUPPORTED, "matrix-free form supports D <= 8, k <= 5");
        if (ns < 1) throw Error(SGDG_EINVAL, "a class needs at least one solve");
        if (apply && (adim < -1 || adim >= D)) throw Error(SGDG_EINVAL, "apply dimension out of range");
        if (kind == MF_KIND_VLASOV && (apply || D % 2 != 0))
            throw Error(SGDG_EINVAL, "a Vlasov solve has an even phase-space dimension and steps");
        dlf1d(k, n);  // validates n
        const SparseIndex ix = make_index(D, k, n, scheme);
        Host& h = host[c];
        for (int d = 0; d < D; d++) {
            h.pencils.push_back(make_pencils(ix, d));
            for (auto& pc : h.pencils.back()) {
                h.boff_index.push_back((int32_t)h.boff.size());
                for (auto o : pc.blockoff) h.boff.push_back(o);
            }
        }
        const int64_t Ns = kind == MF_KIND_WAVE && !apply ? 2 * ix.N : ix.N;
        if ((int64_t)ns * Ns >= (int64_t(1) << 31))
            throw Error(SGDG_EUNSUPPORTED, "a class of solves holds more than 2^31 coefficients");
        cls.push_back(WLClass{kind, D, k, n, apply != 0, apply ? adim : -1, ix.N, Ns, ns, h.pencils, h.boff_index});
    }
    std::vector<MFItem> list;
    int nc = 0;
    mf_work_list(cls, list, nc, pass_only != 0, nullptr, chunk, nchunks, nullptr);
    int64_t nb = 0;
    for (auto& h : host) nb += (int64_t)h.boff.size();
    *nitems = (int64_t)list.size();
    *nboff = nb;
    if (nctr) *nctr = nc;
    if (items && items_cap >= (int64_t)list.size()) {
        for (size_t i = 0; i < list.size(); i++) {
            const MFItem& it = list[i];
            const int64_t f[SGDG_WL_FIELDS] = {it.cls,      it.d,        it.tab,      it.flags,    it.src,
                                               it.dst,      it.wsel,     it.stage,    it.wait_ctr, it.wait_need,
                                               it.win_ctr,  it.win_need, it.done_ctr, it.lmax,     it.lp,
                                               it.boff,     it.R,        it.g0,       it.W,        it.Wv,
                                               it.kd1,      it.kDm1,     it.rlong,    it.rmagic,   it.rshift};
            std::copy(f, f + SGDG_WL_FIELDS, items + i * SGDG_WL_FIELDS);
        }
    }
    if (classes) {
        int64_t first = 0;
        for (int c = 0; c < nclasses; c++) {
            classes[4 * c] = cls[c].N;
            classes[4 * c + 1] = cls[c].Ns;
            classes[4 * c + 2] = cls[c].nslots;
            classes[4 * c + 3] = first;
            first += (int64_t)host[c].boff.size();
        }
    }
    if (blockoff && boff_cap >= nb) {
        int64_t o = 0;
        for (auto& h : host) {
            std::copy(h.boff.begin(), h.boff.end(), blockoff + o);
            o += (int64_t)h.boff.size();
        }
    }
    API_END
}

int sgdg_selftest_convert(const double* x, int64_t n, int64_t* mismatches, int64_t* first) {
    API_BEGIN
    require_gpu();
    if (n < 0) throw Error(SGDG_EINVAL, "n must be >= 0");
    if (n > 0) NEED(x);
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    DevBuf xs((size_t)(n > 0 ? n : 1) * sizeof(double));
    DevBuf bad(2 * sizeof(unsigned long long));
    unsigned long long out[2] = {0ull, ~0ull};
    cudaError_t e = cudaMemcpyAsync(bad.p, out, sizeof(out), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && n > 0) e = cudaMemcpyAsync(xs.p, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_convert_selftest(xs.as<double>(), n, bad.as<unsigned long long>(), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, bad.p, sizeof(out), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) throw Error(SGDG_ECUDA, std::string("conversion self-test: ") + cudaGetErrorString(e));
    if (mismatches) *mismatches = (int64_t)out[0];
    if (first) *first = out[0] ? (int64_t)out[1] : -1;
    API_END
}

int sgdg_set_hbm_budget(int64_t bytes) {
    API_BEGIN
    if (bytes < 0) throw Error(SGDG_EINVAL, "budget must be >= 0");
    g_budget = bytes;
    API_END
}

int sgdg_hbm_in_use(int64_t* bytes) {
    API_BEGIN
    NEED(bytes);
    *bytes = g_in_use.load();
    API_END
}

int sgdg_sync(void) {
    API_BEGIN
    require_gpu();
    CK(cudaDeviceSynchronize());
    API_END
}

}  // extern "C"
