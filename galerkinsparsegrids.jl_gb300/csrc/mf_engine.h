// mf_engine.h -- host driver of the matrix-free form (batches of solves).
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "device_util.h"
#include "engine.h"
#include "sgdg_core.h"

namespace sgdg {

struct SolveSpec {
    int kind = MF_KIND_ADVECT;  // MF_KIND_ADVECT / MF_KIND_WAVE / MF_KIND_VLASOV
    int D = 0, k = 0, n = 0, scheme = 0;  // Vlasov: D = phase-space dimensions
    double a[8] = {0};          // advection velocity
    double dt = 0.0;
    bool apply = false;         // operator application only (no RK): result in rhs
    int apply_dim = -1;         // apply mode: 0-based dimension, or -1 for the sum over all
};

// A class of solves as the work list sees it: host metadata only, so the
// list can be built (and checked) without a GPU.
struct WLClass {
    int kind, D, k, n;
    bool apply;
    int apply_dim;
    int64_t N, Ns;
    int nslots;
    const std::vector<std::vector<Pencil>>& pencils;  // per dimension
    const std::vector<int32_t>& boff_index;           // per (d, pencil): first entry in the class's blockoff
};

// Builds the matrix-free work list of the classes -- the whole RK4 step (four
// stages) for classes that step, one pass per dimension for classes that
// only apply or when pass_only -- with chunk / nchunks and ranges as for
// MFEngine::step_host; nctr receives the number of counters.  Returns the
// shared memory a tile needs (without the operator table).
size_t mf_work_list(const std::vector<WLClass>& cls, std::vector<MFItem>& items, int& nctr, bool pass_only,
                    const std::map<std::pair<int, int>, MFTile>* shapes, int chunk, int nchunks,
                    std::vector<std::array<int, 3>>* ranges);

class MFEngine {
   public:
    explicit MFEngine(cudaStream_t st = nullptr) : stream_(st) {}
    ~MFEngine();
    MFEngine(const MFEngine&) = delete;
    MFEngine& operator=(const MFEngine&) = delete;

    void set_stream(cudaStream_t st);
    cudaStream_t stream() const { return stream_; }

    // Adds a solve; y0 (host, Ns values) may be null (zero state).  A Vlasov
    // solve also takes its point weights: 2 x D x N floats (hi block, lo block)
    int add(const SolveSpec& sp, const double* y0, const float* weights = nullptr);
    void remove(int id);
    void cancel(int id);  // freezes the solve's state (its RK updates are skipped)
    bool live(int id) const;
    int64_t state_size(int id) const;
    int64_t total_size() const;

    void step(int64_t nsteps);                  // RK4 steps of every live solve (async)
    void flush() { plan(); }                    // applies pending joins and leaves now
    // tunes the tile shape of every (D, k) of the live solves that has none
    // yet (process-wide table); returns the (D, k) tuned now
    std::vector<std::pair<int, int>> autotune();
    void get_state(int id, double* host);       // synchronises
    void set_state(int id, const double* host); // async (pageable memory is staged)
    void upload_all(const double* host);
    void download_all(double* host);
    // Every live state from host_in (id order, like upload_all), nsteps RK4
    // steps, the results to host_out (may equal host_in); synchronises.  The
    // groups are split into nchunks chunks, each with its own work list,
    // counters, graph and stream, so one chunk's copies overlap the others'
    // steps.  Host memory should be pinned for the copies to overlap.
    void step_host(const double* host_in, double* host_out, int64_t nsteps, int nchunks);

    // apply mode (single solve): y_dev = op(x_dev)
    void apply(const double* x_dev, double* y_dev);

    double dof_updates_per_step() const;
    int64_t launches_per_step() const { return 1; }  // the whole RK4 step in one launch
    int check_error();  // returns SGDG_OK or SGDG_ETIMEOUT after a bounded wait gave up
    static int64_t solve_bytes(int64_t N, int64_t Ns, int kind = MF_KIND_ADVECT, int D = 0);  // device bytes of a solve
    int64_t pending_bytes() const { return pending_bytes_; }
    int64_t dead_bytes() const;  // arena shares of removed solves, freed by the next re-plan
    // device bytes a re-plan holds on top of the steady state: the largest
    // class's old FP64 state while its new arena is filled, and the old work list
    int64_t replan_reserve() const;

   private:
    struct Solve {
        SolveSpec spec;
        int64_t N = 0, Ns = 0;
        int cls = -1, slot = -1;
        bool live = true, cancelled = false;
        std::vector<double> pending;  // host state not yet on the device
        std::vector<float> weights;   // Vlasov point weights (kept on the host for re-plans)
    };
    struct STable {
        DevBuf rowptr, ent, val;
        int nrow = 0, nent = 0, nval = 0;
    };
    struct TTables {  // the four nodal transforms of one (k, n)
        STable t[4];
    };
    struct QTable {  // the squared line operators of one (k, n)
        DevBuf rowptr, ent, val;
        std::vector<int32_t> roff;
    };
    struct ClassArena {
        std::tuple<int, int, int, int, int, bool, int> key;
        SparseIndex ix;
        std::vector<std::vector<Pencil>> pencils;  // per dimension
        std::vector<int32_t> boff_index;           // per (d, pencil): first entry in blockoff
        int64_t N = 0, Ns = 0;
        std::vector<int> slots;                    // solve id per slot
        DevBuf y, acc, u0, u1, u2, u3, rhs, dt, coef, status, blockoff;
        DevBuf vb, vw;  // Vlasov: 2 scratch vectors per phase dimension and slot, point weights per slot
    };

    void plan();
    // chunk / nchunks: only the groups of that chunk (each class's groups cut
    // into nchunks contiguous runs); ranges receives (class, first slot, slots)
    void build_items(std::vector<MFItem>& items, int& nctr, bool pass_only = false,
                     const std::map<std::pair<int, int>, MFTile>* shapes = nullptr, int chunk = 0, int nchunks = 1,
                     std::vector<std::array<int, 3>>* ranges = nullptr);
    const STable& stab(int k, int n);
    const TTables& ttab(int k, int n);
    const QTable& qtab(int k, int n);
    void capture();
    void drop_graph();
    Solve& at(int id);
    const Solve& at(int id) const;

    cudaStream_t stream_ = nullptr;
    std::vector<Solve> solves_;
    std::vector<std::unique_ptr<ClassArena>> classes_;
    std::map<std::pair<int, int>, STable> stabs_;
    std::map<std::pair<int, int>, TTables> ttabs_;
    std::map<std::pair<int, int>, QTable> qtabs_;
    DevBuf classes_d_, items_d_, ctr_d_, err_d_;
    int nitems_ = 0, nctr_ = 0, grid_ = 0, sms_ = 0;  // grid_: resident CTAs per SM x SMs
    int64_t pending_bytes_ = 0;  // admitted but not yet allocated
    size_t smem_ = 0;
    int table_bytes_ = 0;  // shared-memory operator table reserved ahead of the tile
    bool dirty_ = true;
    cudaGraphExec_t graph_ = nullptr;
    struct Chunk {  // step_host's pipeline stage
        DevBuf items, ctr;
        int nitems = 0, nctr = 0;
        cudaStream_t st = nullptr;
        cudaGraphExec_t graph = nullptr;
        std::vector<std::array<int, 3>> ranges;  // (class, first slot, slots)
    };
    std::vector<Chunk> chunks_;
    void build_chunks(int nchunks);
};

}  // namespace sgdg
