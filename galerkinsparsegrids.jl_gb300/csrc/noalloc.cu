// noalloc.cu -- sgdg_apply_noalloc: the matrix-free operator application
// (D_d x or the Laplacian) with no device allocation at all.
//
// Some callers cannot call cudaMalloc: code running under an allocator they
// do not own (a framework's caching or stream-ordered pool that must see every
// device allocation), runtimes that forbid device allocation after start-up,
// and latency-critical loops that cannot afford cudaMalloc/cudaFree's implicit
// device-wide synchronisation.  This entry point keeps every buffer the
// matrix-free kernel needs besides the caller's input and output -- the work
// list, counters, the 1D operator tables, the FP32 staging of x and the FP32
// partial sums -- in one file-scope device array of fixed size.
//
// Properties a caller must know:
//  - The array is kNoAllocScratchBytes (16 MiB) per GPU and stays allocated
//    on every GPU that loads the library until the process exits.  Problems
//    whose scratch does not fit are rejected with SGDG_EINVAL.
//  - All calls share the one array and it keeps the last call's contents:
//    calls that overlap on the GPU (several host threads, several streams)
//    race and must be serialised by the caller.  Each call rewrites the parts
//    it reads, and clears the counters and the error flag that must start at
//    zero.
//  - The first call on a device looks up the array's device address (with
//    that device current) and caches it; make that first call before any
//    stream capture on the device.
//  - The call is synchronous on `stream`: it returns once y is written.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sgdg.h"
#include "engine.h"
#include "sgdg_core.h"

namespace sgdg {
cudaError_t launch_mf_stage(const MFItem* items, int nitems, const MFClass* classes, int* ctr, int nctr, int stage,
                            int in_sel, int* err, size_t smem, int table_bytes, int grid, cudaStream_t st);
cudaError_t mf_configure(size_t smem, int* blocks_per_sm);
int mf_columns_per_thread(int k);
cudaError_t launch_f64_to_f32(const double* a, float* b, int64_t n, cudaStream_t st);
cudaError_t launch_f32_to_f64(const float* a, double* b, int64_t n, cudaStream_t st);
}  // namespace sgdg

using namespace sgdg;

static constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {nullptr};

int noalloc_fail(int code, const std::string& msg) {
    set_error(msg);
    return code;
}

// device address of the scratch array for the current device (looked up once)
cudaError_t scratch_address(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

struct Region {
    size_t off = 0;
    size_t bytes = 0;
};

struct Layout {
    size_t top = 0;
    Region add(size_t bytes) {
        Region r;
        r.off = (top + 255) & ~size_t(255);
        r.bytes = bytes;
        top = r.off + bytes;
        return r;
    }
};

}  // namespace

extern "C" int sgdg_apply_noalloc(int D, int k, int n, int scheme, int which, const double* x_dev, double* y_dev,
                                  void* stream) {
    try {
        if (!x_dev || !y_dev) return noalloc_fail(SGDG_EINVAL, "x_dev and y_dev must not be NULL");
        if (n < 2) return noalloc_fail(SGDG_EINVAL, "n must be >= 2");
        if (k < 1 || k > 5) return noalloc_fail(SGDG_EUNSUPPORTED, "matrix-free form supports 1 <= k <= 5");
        const SparseIndex ix = make_index(D, k, n, scheme);
        if (!(which == SGDG_OP_LAPLACIAN || (which >= 1 && which <= D)))
            return noalloc_fail(SGDG_EINVAL, "which must be 1..D (D_d) or 0 (laplacian)");
        // the FP32 copy of x and the FP32 partial sums alone must fit: reject
        // before the pencils and the work list are built on the host
        if (ix.N > (int64_t)INT32_MAX || 2 * sizeof(float) * (size_t)ix.N > kNoAllocScratchBytes)
            return noalloc_fail(SGDG_EINVAL, "problem of " + std::to_string(ix.N) +
                                                 " coefficients needs more scratch than sgdg_apply_noalloc holds: "
                                                 "at most " + std::to_string(kNoAllocScratchBytes) +
                                                 " bytes (use sgdg_apply_device for larger problems)");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            return noalloc_fail(SGDG_ENOGPU, "no CUDA device");
        }
        cudaStream_t st = (cudaStream_t)stream;
        const bool wave = which == SGDG_OP_LAPLACIAN;
        const int N = (int)ix.N;

        // 1D operator blocks as the matrix-free kernel applies them
        const MFOperator M = mf_operator(k, n);
        const MFOperator* op = &M;
        const int rs = M.rs;
        const std::vector<float>& sval = M.val;

        // pencil tiles of the requested dimensions: one phase per dimension
        std::vector<int> dims;
        if (wave)
            for (int d = 0; d < D; d++) dims.push_back(d);
        else
            dims.push_back(which - 1);
        const int cpt = mf_columns_per_thread(k);
        const MFTile tile = mf_tile(D, k);
        int kDm1 = 1;
        for (int q = 0; q < D - 1; q++) kDm1 *= k;
        std::vector<int64_t> boff;
        std::vector<MFItem> items;
        size_t smem = 64;
        for (size_t ph = 0; ph < dims.size(); ph++) {
            const int d = dims[ph];
            int kd1 = 1;
            for (int q = 0; q < d; q++) kd1 *= k;
            for (const Pencil& p : make_pencils(ix, d)) {
                const int32_t pb = (int32_t)boff.size();
                for (auto o : p.blockoff) boff.push_back(o);
                const int nrb = 1 << (p.lmax - 1);
                const int Wp = mf_tile_cols(k, cpt, nrb, tile.wlog);
                smem = std::max(smem, mf_tile_smem(k, nrb, Wp));
                for (int64_t g0 = 0; g0 < p.R; g0 += Wp) {
                    MFItem it{};
                    it.tab = TABLE_DERIVATIVE;
                    it.src = -1;  // the stage input
                    it.cls = 0;
                    it.d = (int16_t)d;
                    it.flags = (int16_t)((ph == 0 ? TILE_FIRST : 0) | (ph + 1 == dims.size() ? TILE_LAST : 0));
                    it.done_ctr = 1 + (int)ph;
                    it.wait_ctr = ph > 0 ? (int)ph : -1;
                    it.lmax = p.lmax;
                    it.lp = p.lp;
                    it.boff = pb;
                    it.R = (int32_t)p.R;
                    mf_divisor(it.R, &it.rmagic, &it.rshift);
                    it.g0 = (int32_t)g0;
                    it.W = Wp;
                    it.Wv = (int32_t)std::min<int64_t>(Wp, p.R - g0);
                    it.kd1 = kd1;
                    it.kDm1 = kDm1;
                    it.rlong = mf_rlong(p.lmax, tile.coop);
                    items.push_back(it);
                }
            }
        }
        {
            // phase p waits until every item of phase p-1 is done
            std::vector<int> count(dims.size() + 1, 0);
            for (auto& it : items) count[it.done_ctr]++;
            for (auto& it : items) it.wait_need = it.wait_ctr >= 0 ? count[it.wait_ctr] : 0;
        }
        const int nctr = 1 + (int)dims.size();
        const int tb = mf_table_bytes((int)M.rowptr.size(), (int)M.ent.size(), (int)M.val.size());
        const int table_bytes = tb <= kMFTableSmemMax ? tb : 0;
        smem += (size_t)table_bytes;
        if (smem > 227 * 1024)
            return noalloc_fail(SGDG_EUNSUPPORTED, "operator table and pencil tile exceed shared memory");

        // scratch layout
        Layout L;
        const Region r_cls = L.add(sizeof(MFClass));
        const Region r_items = L.add(sizeof(MFItem) * items.size());
        const Region r_ctr = L.add(sizeof(int) * nctr);
        const Region r_err = L.add(sizeof(int));
        const Region r_rowptr = L.add(sizeof(int32_t) * op->rowptr.size());
        const Region r_ent = L.add(sizeof(int32_t) * op->ent.size());
        const Region r_sval = L.add(sizeof(float) * sval.size());
        const Region r_boff = L.add(sizeof(int64_t) * boff.size());
        const Region r_coef = L.add(sizeof(float) * 16);
        const Region r_status = L.add(sizeof(int32_t));
        const Region r_dt = L.add(sizeof(double) * 3);
        const Region r_u = L.add(sizeof(float) * (size_t)N);
        const Region r_rhs = L.add(sizeof(float) * (size_t)N);
        if (L.top > kNoAllocScratchBytes)
            return noalloc_fail(SGDG_EINVAL, "problem needs " + std::to_string(L.top) +
                                                 " bytes of scratch; sgdg_apply_noalloc holds at most " +
                                                 std::to_string(kNoAllocScratchBytes) +
                                                 " (use sgdg_apply_device for larger problems)");

        unsigned char* base = nullptr;
        cudaError_t e = scratch_address(&base);
        if (e != cudaSuccess) return noalloc_fail(SGDG_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));

        MFClass c{};
        c.s_rowptr = reinterpret_cast<const int32_t*>(base + r_rowptr.off);
        c.s_ent = reinterpret_cast<const int32_t*>(base + r_ent.off);
        c.s_val = reinterpret_cast<const float*>(base + r_sval.off);
        c.s_nrow = (int)M.rowptr.size();
        c.s_nent = (int)M.ent.size();
        c.s_nval = (int)M.val.size();
        c.s_shared = table_bytes > 0;
        c.blockoff = reinterpret_cast<const int64_t*>(base + r_boff.off);
        c.y = nullptr;
        c.acc = nullptr;
        c.u[0] = reinterpret_cast<float*>(base + r_u.off);
        c.u[1] = c.u[2] = c.u[3] = c.u[0];
        c.rhs = reinterpret_cast<float*>(base + r_rhs.off);
        c.dt = reinterpret_cast<const double*>(base + r_dt.off);
        c.coef = reinterpret_cast<const float*>(base + r_coef.off);
        c.status = reinterpret_cast<const int32_t*>(base + r_status.off);
        c.N = N;
        c.Ns = N;
        c.nslots = 1;
        c.D = D;
        c.k = k;
        c.kD = (int)ix.kD;
        c.kind = wave ? MF_KIND_WAVE : MF_KIND_ADVECT;
        c.rs = rs;
        const float coef[16] = {1.f, 1.f, 1.f, 1.f, 1.f, 1.f, 1.f, 1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const int32_t status = 0;
        const double dt[3] = {0.0, 0.0, 0.0};

        // every region this call reads is rewritten; counters and the error
        // flag start at zero (launch_mf_stage clears the counters)
        struct Copy {
            const Region& r;
            const void* src;
        };
        const Copy copies[] = {{r_cls, &c},
                               {r_items, items.data()},
                               {r_rowptr, op->rowptr.data()},
                               {r_ent, op->ent.data()},
                               {r_sval, sval.data()},
                               {r_boff, boff.data()},
                               {r_coef, coef},
                               {r_status, &status},
                               {r_dt, dt}};
        for (const Copy& cp : copies)
            if (cp.r.bytes) {
                e = cudaMemcpyAsync(base + cp.r.off, cp.src, cp.r.bytes, cudaMemcpyHostToDevice, st);
                if (e != cudaSuccess) return noalloc_fail(SGDG_ECUDA, std::string("copy: ") + cudaGetErrorString(e));
            }
        e = cudaMemsetAsync(base + r_err.off, 0, sizeof(int), st);
        int bps = 0, dev = 0, sms = 0;
        if (e == cudaSuccess) e = mf_configure(smem, &bps);
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = launch_f64_to_f32(x_dev, c.u[0], N, st);
        if (e == cudaSuccess)
            e = launch_mf_stage(reinterpret_cast<const MFItem*>(base + r_items.off), (int)items.size(),
                                reinterpret_cast<const MFClass*>(base + r_cls.off),
                                reinterpret_cast<int*>(base + r_ctr.off), nctr, 1, 0,
                                reinterpret_cast<int*>(base + r_err.off), smem, table_bytes, std::max(1, bps) * sms,
                                st);
        if (e == cudaSuccess) e = launch_f32_to_f64(c.rhs, y_dev, N, st);
        int err = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&err, base + r_err.off, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return noalloc_fail(SGDG_ECUDA, std::string("apply_noalloc: ") + cudaGetErrorString(e));
        if (err) return noalloc_fail(SGDG_ETIMEOUT, "a bounded device wait gave up; y is unreliable");
        return SGDG_OK;
    } catch (const Error& ex) {
        return noalloc_fail(ex.code, ex.what());
    } catch (const std::exception& ex) {
        return noalloc_fail(SGDG_EINVAL, ex.what());
    }
}
