// mf_engine.cu -- host driver of the matrix-free form.
//
// Solves with equal (kind, D, k, n, scheme) share a class: their vectors live
// in class arenas (slot-major) so pencil tiles can take columns from several
// solves.  plan() rebuilds the arenas of classes whose solves changed (states
// move into the new arena device-to-device), keeps the others as they are, and
// rebuilds the ordered work list.
// One RK4 step is one launch of k_mf_stage over a work list holding all four
// stages (each group's stages in order, different groups' stages interleaved),
// captured once in a CUDA graph; a membership change drops the graph and the
// next step re-captures it.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "mf_engine.h"

namespace sgdg {

cudaError_t launch_mf_stage(const MFItem* items, int nitems, const MFClass* classes, int* ctr, int nctr, int stage,
                            int in_sel, int* err, size_t smem, int table_bytes, int grid, cudaStream_t st);
cudaError_t mf_configure(size_t smem, int* blocks_per_sm);
int mf_columns_per_thread(int k);
cudaError_t launch_f64_to_f32(const double* a, float* b, int64_t n, cudaStream_t st);
cudaError_t launch_f32_to_f64(const float* a, double* b, int64_t n, cudaStream_t st);

static constexpr size_t kWaveLag = 3;       // steps between a group's consecutive phases in the work list
static constexpr int kStageKey = 1 << 22;   // counter keys of a whole-step list: key + (stage - 1) * kStageKey

// The wave's D_d D_d on a pencil of line length lmax: one sweep of the
// squared line operator for lmax <= kWaveSquareLevels, two sweeps of the
// line operator above.  One sweep halves the FP32 work, but its partial
// sums cancel more (entries grow like 4^l instead of 2^l), so the long
// lines keep two sweeps: 3D k=3 n=7 to t=1 stays at 7.3e-7 relative L2
// (7.4e-7 with two sweeps everywhere, 2.7e-6 with one sweep everywhere).
constexpr int kWaveSquareLevels = 5;
static int wave_square_levels() {  // SGDG_MF_WAVE_SQUARE overrides (0: two sweeps everywhere)
    static const int lv = [] {
        const char* e = std::getenv("SGDG_MF_WAVE_SQUARE");
        return e ? std::max(0, std::atoi(e)) : kWaveSquareLevels;
    }();
    return lv;
}
constexpr int64_t kGroupReuseBytes = 6LL << 20;  // reused u + rhs per group (~4 groups in flight)

// The arenas' cudaFree calls wait for outstanding work; the stream is not
// touched here because a caller's stream may already be gone.
MFEngine::~MFEngine() { drop_graph(); }

void MFEngine::set_stream(cudaStream_t st) {
    if (st != stream_) drop_graph();
    stream_ = st;
}

void MFEngine::drop_graph() {
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
    for (Chunk& c : chunks_) {
        if (c.graph) cudaGraphExecDestroy(c.graph);
        if (c.st) {
            cudaStreamSynchronize(c.st);
            cudaStreamDestroy(c.st);
        }
    }
    chunks_.clear();
}

MFEngine::Solve& MFEngine::at(int id) {
    if (id < 0 || id >= (int)solves_.size() || !solves_[id].live) throw Error(SGDG_EINVAL, "no such solve id");
    return solves_[id];
}
const MFEngine::Solve& MFEngine::at(int id) const {
    if (id < 0 || id >= (int)solves_.size() || !solves_[id].live) throw Error(SGDG_EINVAL, "no such solve id");
    return solves_[id];
}

bool MFEngine::live(int id) const { return id >= 0 && id < (int)solves_.size() && solves_[id].live; }

int MFEngine::add(const SolveSpec& sp, const double* y0, const float* weights) {
    require_gpu();
    if (sp.k < 1 || sp.k > 5) throw Error(SGDG_EUNSUPPORTED, "matrix-free form supports 1 <= k <= 5 (use the plain form)");
    if (sp.D > 8) throw Error(SGDG_EUNSUPPORTED, "matrix-free form supports D <= 8");
    if (sp.kind == MF_KIND_VLASOV) {
        if (sp.apply || sp.D % 2 != 0) throw Error(SGDG_EINVAL, "a Vlasov solve has an even phase-space dimension");
        if (sp.k != 2 && sp.k != 3 && sp.k != 5) throw Error(SGDG_EINVAL, "the nodal basis exists for k = 2, 3, 5");
        if (!weights) throw Error(SGDG_EINVAL, "a Vlasov solve needs its point weights");
    }
    Solve s;
    s.spec = sp;
    SparseIndex ix = make_index(sp.D, sp.k, sp.n, sp.scheme);
    dlf1d(sp.k, sp.n);  // validates n >= 2
    s.N = ix.N;
    s.Ns = sp.kind == MF_KIND_WAVE && !sp.apply ? 2 * ix.N : ix.N;
    // admission: the solve's arena share must fit the HBM budget now
    const int64_t need = solve_bytes(s.N, s.Ns, sp.kind, sp.D);
    const int64_t budget = g_budget.load();
    const int64_t held = g_in_use.load() - dead_bytes() + pending_bytes_;
    if (budget > 0 && held + need > budget)
        throw Error(SGDG_ENOMEM_BUDGET, "HBM budget: solve needs " + std::to_string(need) + " bytes, " +
                                            std::to_string(held) + " of " + std::to_string(budget) + " committed");
    if (y0) s.pending.assign(y0, y0 + s.Ns);
    else s.pending.assign(s.Ns, 0.0);
    if (sp.kind == MF_KIND_VLASOV) s.weights.assign(weights, weights + (size_t)2 * sp.D * s.N);
    solves_.push_back(std::move(s));
    pending_bytes_ += need;
    dirty_ = true;
    return (int)solves_.size() - 1;
}

int64_t MFEngine::solve_bytes(int64_t N, int64_t Ns, int kind, int D) {
    // y, acc (FP64), four stage inputs (FP32), partial sums (FP32); Vlasov:
    // two scratch vectors per phase dimension and 2 D point weights (FP32)
    return Ns * (8 + 8 + 4 * 4) + N * 4 + (kind == MF_KIND_VLASOV ? N * 4 * (4 * (int64_t)D) : 0);
}

int64_t MFEngine::dead_bytes() const {
    int64_t b = 0;
    for (auto& s : solves_)
        if (!s.live && s.cls >= 0) b += solve_bytes(s.N, s.Ns, s.spec.kind, s.spec.D);
    return b;
}

int64_t MFEngine::replan_reserve() const {
    int64_t r = (int64_t)items_d_.bytes + (int64_t)classes_d_.bytes;
    int64_t ymax = 0;
    for (auto& c : classes_) ymax = std::max<int64_t>(ymax, (int64_t)c->y.bytes);
    return r + ymax;
}

void MFEngine::remove(int id) {
    at(id).live = false;
    dirty_ = true;
}

void MFEngine::cancel(int id) {
    Solve& s = at(id);
    s.cancelled = true;
    if (!dirty_ && s.cls >= 0) {
        int one = 1;
        CK(cudaMemcpyAsync(classes_[s.cls]->status.as<int32_t>() + s.slot, &one, sizeof(int), cudaMemcpyHostToDevice,
                           stream_));
        CK(cudaStreamSynchronize(stream_));
    }
}

int64_t MFEngine::state_size(int id) const { return at(id).Ns; }

int64_t MFEngine::total_size() const {
    int64_t t = 0;
    for (auto& s : solves_)
        if (s.live) t += s.Ns;
    return t;
}

double MFEngine::dof_updates_per_step() const {
    double t = 0;
    for (auto& s : solves_)
        if (s.live && !s.cancelled) t += 4.0 * double(s.Ns);
    return t;
}

const MFEngine::STable& MFEngine::stab(int k, int n) {
    auto key = std::make_pair(k, n);
    auto it = stabs_.find(key);
    if (it != stabs_.end()) return it->second;
    const MFOperator M = mf_operator(k, n);
    STable S;
    S.rowptr = upload(M.rowptr, stream_);
    S.ent = upload(M.ent, stream_);
    S.val = upload(M.val, stream_);
    S.nrow = (int)M.rowptr.size();
    S.nent = (int)M.ent.size();
    S.nval = (int)M.val.size();
    CK(cudaStreamSynchronize(stream_));
    return stabs_.emplace(key, std::move(S)).first->second;
}

const MFEngine::TTables& MFEngine::ttab(int k, int n) {
    auto key = std::make_pair(k, n);
    auto it = ttabs_.find(key);
    if (it != ttabs_.end()) return it->second;
    TTables T;
    for (int w = 0; w < 4; w++) {
        const MFOperator M = mf_transform_table(k, n, w);
        T.t[w].rowptr = upload(M.rowptr, stream_);
        T.t[w].ent = upload(M.ent, stream_);
        T.t[w].val = upload(M.val, stream_);
        T.t[w].nrow = (int)M.rowptr.size();
        T.t[w].nent = (int)M.ent.size();
        T.t[w].nval = (int)M.val.size();
    }
    CK(cudaStreamSynchronize(stream_));
    return ttabs_.emplace(key, std::move(T)).first->second;
}

const MFEngine::QTable& MFEngine::qtab(int k, int n) {
    auto key = std::make_pair(k, n);
    auto it = qtabs_.find(key);
    if (it != qtabs_.end()) return it->second;
    const MFSquareTables Q = mf_square_tables(k, n);
    if ((int)Q.roff.size() > kMFMaxLevels) throw Error(SGDG_EUNSUPPORTED, "matrix-free form supports n <= 15");
    QTable T;
    T.rowptr = upload(Q.rowptr, stream_);
    T.ent = upload(Q.ent, stream_);
    T.val = upload(Q.val, stream_);
    T.roff = Q.roff;
    CK(cudaStreamSynchronize(stream_));
    return qtabs_.emplace(key, std::move(T)).first->second;
}

void MFEngine::plan() {
    if (!dirty_) return;
    drop_graph();
    if (!err_d_.p) {
        err_d_.alloc(sizeof(int));
        CK(cudaMemsetAsync(err_d_.p, 0, sizeof(int), stream_));
    }
    // 1. classes of live solves, in id order
    std::vector<std::unique_ptr<ClassArena>> next;
    std::map<std::tuple<int, int, int, int, int, bool, int>, int> cls_of;
    for (int id = 0; id < (int)solves_.size(); id++) {
        Solve& s = solves_[id];
        if (!s.live) continue;
        auto key = std::make_tuple(s.spec.kind, s.spec.D, s.spec.k, s.spec.n, s.spec.scheme, s.spec.apply,
                                   s.spec.apply_dim);
        auto f = cls_of.find(key);
        if (f == cls_of.end()) {
            auto c = std::make_unique<ClassArena>();
            c->key = key;
            c->ix = make_index(s.spec.D, s.spec.k, s.spec.n, s.spec.scheme);
            c->N = s.N;
            c->Ns = s.Ns;
            f = cls_of.emplace(key, (int)next.size()).first;
            next.push_back(std::move(c));
        }
        next[f->second]->slots.push_back(id);
    }
    // 2. arenas, state moves, per-slot tables.  A class's solves only ever
    // come from the old arena of the same key, which is freed as soon as they
    // have moved, so the transient overhead is one class arena.
    std::map<std::tuple<int, int, int, int, int, bool, int>, int> old_of;
    for (size_t oi = 0; oi < classes_.size(); oi++) old_of[classes_[oi]->key] = (int)oi;
    for (size_t ci = 0; ci < next.size(); ci++) {
        auto of = old_of.find(next[ci]->key);
        ClassArena* old_c = of == old_of.end() ? nullptr : classes_[of->second].get();
        if (old_c && old_c->slots == next[ci]->slots) {
            // same solves in the same slots: keep the arena as it is, unless a
            // host state is waiting to be uploaded
            bool pending = false;
            for (int id : old_c->slots) pending = pending || !solves_[id].pending.empty();
            if (!pending) {
                next[ci] = std::move(classes_[of->second]);
                continue;
            }
        }
        ClassArena& c = *next[ci];
        if (old_c) {  // free what the new arena does not need from the old one first
            old_c->acc.release();
            old_c->u0.release();
            old_c->u1.release();
            old_c->u2.release();
            old_c->u3.release();
            old_c->rhs.release();
        }
        const int ns = (int)c.slots.size();
        if ((int64_t)ns * c.Ns >= (int64_t(1) << 31))
            throw Error(SGDG_EUNSUPPORTED, "a class of solves holds more than 2^31 coefficients");
        const Solve& s0 = solves_[c.slots[0]];
        const int D = s0.spec.D;
        std::vector<int64_t> boff;
        for (int d = 0; d < D; d++) {
            c.pencils.push_back(make_pencils(c.ix, d));
            for (auto& p : c.pencils.back()) {
                c.boff_index.push_back((int32_t)boff.size());
                for (auto o : p.blockoff) boff.push_back(o);
            }
        }
        c.blockoff = upload(boff, stream_);
        c.y.alloc(sizeof(double) * ns * c.Ns);
        c.acc.alloc(sizeof(double) * ns * c.Ns);
        c.u0.alloc(sizeof(float) * ns * c.Ns);
        c.u1.alloc(sizeof(float) * ns * c.Ns);
        if (!s0.spec.apply) {  // the stage inputs of stages 3 and 4
            c.u2.alloc(sizeof(float) * ns * c.Ns);
            c.u3.alloc(sizeof(float) * ns * c.Ns);
        }
        c.rhs.alloc(sizeof(float) * ns * c.N);
        const bool vlasov = s0.spec.kind == MF_KIND_VLASOV;
        if (vlasov) {
            c.vb.alloc(sizeof(float) * 2 * (size_t)D * ns * c.N);  // two ping-pong vectors per phase dimension
            c.vw.alloc(sizeof(float) * 2 * (size_t)D * ns * c.N);
            for (int sl = 0; sl < ns; sl++) {
                const Solve& s = solves_[c.slots[sl]];
                CK(cudaMemcpyAsync(c.vw.as<float>() + (size_t)sl * 2 * D * c.N, s.weights.data(),
                                   sizeof(float) * s.weights.size(), cudaMemcpyHostToDevice, stream_));
            }
        }
        std::vector<double> dt(3 * (size_t)ns);
        std::vector<float> coef((size_t)ns * 16, 0.f);
        std::vector<int32_t> status(ns, 0);
        for (int sl = 0; sl < ns; sl++) {
            Solve& s = solves_[c.slots[sl]];
            dt[3 * sl] = s.spec.dt;
            dt[3 * sl + 1] = 0.5 * s.spec.dt;
            dt[3 * sl + 2] = s.spec.dt / 6.0;
            for (int d = 0; d < 8; d++) {
                // factor on D_d as an FP32 (hi, lo) pair: a rounded velocity
                // would perturb the operator systematically
                const double f =
                    s.spec.apply || s.spec.kind == MF_KIND_WAVE || s.spec.kind == MF_KIND_VLASOV ? 1.0 : -s.spec.a[d];
                coef[sl * 16 + d] = (float)f;
                coef[sl * 16 + 8 + d] = (float)(f - (double)(float)f);
            }
            status[sl] = s.cancelled ? 1 : 0;
            double* dst = c.y.as<double>() + (size_t)sl * c.Ns;
            if (!s.pending.empty()) {
                CK(cudaMemcpyAsync(dst, s.pending.data(), sizeof(double) * c.Ns, cudaMemcpyHostToDevice, stream_));
            } else if (s.cls >= 0) {
                const ClassArena& old = *classes_[s.cls];
                CK(cudaMemcpyAsync(dst, old.y.as<double>() + (size_t)s.slot * old.Ns, sizeof(double) * c.Ns,
                                   cudaMemcpyDeviceToDevice, stream_));
            } else {
                CK(cudaMemsetAsync(dst, 0, sizeof(double) * c.Ns, stream_));
            }
        }
        c.dt = upload(dt, stream_);
        c.coef = upload(coef, stream_);
        c.status = upload(status, stream_);
        CK(launch_f64_to_f32(c.y.as<double>(), c.u0.as<float>(), (int64_t)ns * c.Ns, stream_));
        if (old_c) old_c->y.release();  // cudaFree waits for the copies above
    }
    CK(cudaStreamSynchronize(stream_));
    pending_bytes_ = 0;
    // the old arenas are no longer referenced
    classes_.swap(next);
    next.clear();
    for (size_t ci = 0; ci < classes_.size(); ci++)
        for (size_t sl = 0; sl < classes_[ci]->slots.size(); sl++) {
            Solve& s = solves_[classes_[ci]->slots[sl]];
            s.cls = (int)ci;
            s.slot = (int)sl;
            s.pending.clear();
            s.pending.shrink_to_fit();
        }
    for (auto& s : solves_)
        if (!s.live) {
            s.cls = s.slot = -1;
        }
    // 3. class descriptors and the work list
    std::vector<MFClass> ch;
    for (auto& cp : classes_) {
        ClassArena& c = *cp;
        const Solve& s0 = solves_[c.slots[0]];
        const STable& S = stab(s0.spec.k, s0.spec.n);
        MFClass m{};
        m.s_rowptr = S.rowptr.as<int32_t>();
        m.s_ent = S.ent.as<int32_t>();
        m.s_val = S.val.as<float>();
        m.s_nrow = S.nrow;
        m.s_nent = S.nent;
        m.s_nval = S.nval;
        m.s_shared = mf_table_bytes(S.nrow, S.nent, S.nval) <= kMFTableSmemMax;
        m.blockoff = c.blockoff.as<int64_t>();
        m.y = c.y.as<double>();
        m.acc = c.acc.as<double>();
        m.u[0] = c.u0.as<float>();
        m.u[1] = c.u1.as<float>();
        m.u[2] = c.u2.p ? c.u2.as<float>() : m.u[0];
        m.u[3] = c.u3.p ? c.u3.as<float>() : m.u[1];
        m.rhs = c.rhs.as<float>();
        if (s0.spec.kind == MF_KIND_WAVE && !s0.spec.apply && wave_square_levels() > 0) {
            const QTable& Q = qtab(s0.spec.k, s0.spec.n);
            m.q_rowptr = Q.rowptr.as<int32_t>();
            m.q_ent = Q.ent.as<int32_t>();
            m.q_val = Q.val.as<float>();
            for (size_t l = 0; l < Q.roff.size(); l++) m.q_roff[l] = Q.roff[l];
        }
        m.dt = c.dt.as<double>();
        m.coef = c.coef.as<float>();
        m.status = c.status.as<int32_t>();
        m.N = (int32_t)c.N;
        m.Ns = (int32_t)c.Ns;
        m.nslots = (int32_t)c.slots.size();
        m.D = s0.spec.D;
        m.k = s0.spec.k;
        int kD = 1;
        for (int q = 0; q < m.D; q++) kD *= m.k;
        m.kD = kD;
        m.kind = s0.spec.kind;
        m.rs = ((2 * m.k + 3) / 4) * 4;
        if (m.kind == MF_KIND_VLASOV) {
            const TTables& T = ttab(m.k, s0.spec.n);
            for (int w = 0; w < 4; w++) {
                m.t_rowptr[w] = T.t[w].rowptr.as<int32_t>();
                m.t_nrow[w] = T.t[w].nrow;
                m.t_nent[w] = T.t[w].nent;
                m.t_nval[w] = T.t[w].nval;
                m.t_ent[w] = T.t[w].ent.as<int32_t>();
                m.t_val[w] = T.t[w].val.as<float>();
            }
            m.vbase = c.vb.as<float>();
            m.vstride = (int64_t)c.slots.size() * c.N;
            m.vw = c.vw.as<float>();
        }
        ch.push_back(m);
    }
    std::vector<MFItem> items;
    int nctr = 0;
    build_items(items, nctr);
    classes_d_ = upload(ch, stream_);
    items_d_ = upload(items, stream_);
    ctr_d_.alloc(sizeof(int) * (size_t)std::max(nctr, 1));
    nitems_ = (int)items.size();
    nctr_ = nctr;
    int bps = 0;
    CK(mf_configure(smem_, &bps));
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    grid_ = std::max(1, bps) * sms;
    sms_ = sms;
    CK(cudaStreamSynchronize(stream_));
    dirty_ = false;
}

// Work list.  Each class is cut into groups of slots; a group has one phase
// per dimension pass (the last one also applies the RK stage update, unless
// applying only), and phase p of a group depends on phase p-1 of the same
// group.  Groups are emitted in
// wavefront order -- step t holds phase t-g of group g, oldest group first --
// so when a phase is handed out, its predecessor was handed out a whole
// wavefront earlier and is normally complete: CTAs rarely wait, while the
// groups in flight (about one per phase) keep their reused vectors in L2.
size_t mf_work_list(const std::vector<WLClass>& cls, std::vector<MFItem>& items, int& nctr, bool pass_only,
                    const std::map<std::pair<int, int>, MFTile>* shapes, int chunk, int nchunks,
                    std::vector<std::array<int, 3>>* ranges) {
    struct Phase {
        std::vector<MFItem> items;
        int depth = 0;      // longest chain of phases before it in the group
        int done_key = 0;   // counter it increments (phases of a join share one)
        int wait_key = -1;  // counter it waits for (-1: none)
        int win_key = -1;   // whole-step list: the counter of the RK phase that wrote its stage input
        int stage = 0;      // RK stage of its items (0: the launch's stage)
    };
    struct Group {
        std::vector<Phase> phases;
    };
    std::vector<Group> groups;
    size_t smem = 64;
    for (size_t ci = 0; ci < cls.size(); ci++) {
        const WLClass& c = cls[ci];
        const WLClass& sp = c;
        const int D = sp.D, k = sp.k;
        const int cpt = mf_columns_per_thread(k);
        MFTile tile = mf_tile(D, k);
        if (shapes) {
            auto f = shapes->find({D, k});
            if (f != shapes->end()) tile = f->second;
        }
        std::vector<int> dims;
        if (sp.apply && sp.apply_dim >= 0)
            dims.push_back(sp.apply_dim);
        else
            for (int d = 0; d < D; d++) dims.push_back(d);
        const int ns = c.nslots;
        const int64_t per_solve = 8 * c.N;
        int gs = (int)std::max<int64_t>(1, std::min<int64_t>(ns, kGroupReuseBytes / std::max<int64_t>(1, per_solve)));
        {
            // groups start on 128-byte boundaries of the FP32 stage inputs (a
            // multiple of 32 / gcd(Ns, 32) slots), so no L1 line of a stage
            // input holds two groups' coefficients (groups reach a stage at
            // different times within a whole-step launch)
            int g32 = 32;
            for (int64_t a = c.Ns; g32 > 1 && a % 2 == 0; a /= 2) g32 /= 2;
            gs = std::min(ns, (gs + g32 - 1) / g32 * g32);
        }
        int kDm1 = 1;
        for (int q = 0; q < D - 1; q++) kDm1 *= k;
        const int ng = (ns + gs - 1) / gs;
        for (int s0 = 0; s0 < ns; s0 += gs) {
            const int s1 = std::min(ns, s0 + gs);
            if ((int64_t)(s0 / gs) * nchunks / ng != chunk) continue;  // another chunk's group
            if (ranges) ranges->push_back({(int)ci, s0, s1 - s0});
            Group grp;
            // one phase: tiles of every pencil along d over the group's slots
            auto phase = [&](int d, int tab, int src, int dst, int flags, int wsel, int depth, int done_key,
                             int wait_key) {
                int kd1 = 1;
                for (int q = 0; q < d; q++) kd1 *= k;
                std::vector<MFItem> list;
                int bi = 0;
                for (int dd = 0; dd < d; dd++) bi += (int)c.pencils[dd].size();
                for (size_t pi = 0; pi < c.pencils[d].size(); pi++) {
                    const Pencil& p = c.pencils[d][pi];
                    const int nrb = 1 << (p.lmax - 1);
                    const int Wp = mf_tile_cols(k, cpt, nrb, tile.wlog);
                    const int64_t cbeg = (int64_t)s0 * p.R, cend = (int64_t)s1 * p.R;
                    smem = std::max(smem, mf_tile_smem(k, nrb, Wp));
                    // the wave steps short lines with the squared table
                    const int ptab = tab == TABLE_DERIVATIVE && sp.kind == MF_KIND_WAVE && !sp.apply &&
                                             p.lmax <= wave_square_levels()
                                         ? TABLE_SQUARE
                                         : tab;
                    for (int64_t g0 = cbeg; g0 < cend; g0 += Wp) {
                        MFItem it{};
                        it.tab = (int16_t)ptab;
                        it.cls = (int16_t)ci;
                        it.d = (int16_t)d;
                        it.flags = (int16_t)flags;
                        it.src = (int16_t)src;
                        it.dst = (int16_t)dst;
                        it.wsel = (int16_t)wsel;
                        it.lmax = p.lmax;
                        it.lp = p.lp;
                        it.boff = c.boff_index[bi + pi];
                        it.R = (int32_t)p.R;
                        mf_divisor(it.R, &it.rmagic, &it.rshift);
                        it.g0 = (int32_t)g0;
                        it.W = Wp;
                        it.Wv = (int32_t)std::min<int64_t>(Wp, cend - g0);
                        it.kd1 = kd1;
                        it.kDm1 = kDm1;
                        it.rlong = mf_rlong(p.lmax, tile.coop);
                        list.push_back(it);
                    }
                }
                Phase ph;
                ph.items = std::move(list);
                ph.depth = depth;
                ph.done_key = done_key;
                ph.wait_key = wait_key;
                grp.phases.push_back(std::move(ph));
            };
            // the RK state is never updated while tuning (no state changes)
            const int rk = !sp.apply && !pass_only ? TILE_RK : 0;
            if (sp.kind != MF_KIND_VLASOV) {
                // one pass per dimension accumulating into rhs; the last applies the RK update
                for (size_t ph = 0; ph < dims.size(); ph++) {
                    const bool last = ph + 1 == dims.size();
                    phase(dims[ph], TABLE_DERIVATIVE, -1, 0, (ph == 0 ? TILE_FIRST : 0) | (last ? TILE_LAST | rk : 0),
                          0, (int)ph, (int)ph, (int)ph - 1);
                }
            } else {
                // Vlasov right-hand side (src/pdes.jl:174-192) as sweeps: for each
                // phase dimension d a chain -- D_d, then the modal->nodal and
                // nodal->points transforms (one sweep per dimension each; the
                // restricted Kronecker products factor exactly because the 1D
                // maps are level-triangular), the last sweep times the point
                // weight of d -- in its own two scratch vectors (2d, 2d + 1), so
                // the D chains run concurrently; then points->nodal, whose
                // first sweep gathers the sum of the D products (in order d =
                // 0, 1, ...) once every chain is done, and nodal->modal, whose
                // last sweep applies the RK update.  Within a chain every sweep
                // reads what the previous one wrote.
                const int P = D, kJoin = 1 << 20;
                int key = 0, maxdepth = 0, prod = -1;
                for (int d = 0; d < P; d++) {
                    int depth = 0, prev = -1, cur = 2 * d;
                    auto link = [&](int q, int tab, int src, int dst, int flags, int wsel, int done) {
                        phase(q, tab, src, dst, flags | (prev >= 0 ? TILE_WAIT_IN : 0), wsel, depth, done, prev);
                        prev = done;
                        depth++;
                    };
                    link(d, TABLE_DERIVATIVE, -1, cur, TILE_STORE, 0, key++);
                    for (int q = 0; q < P; q++, cur ^= 1)
                        link(q, TRANSFORM_MODAL_TO_NODAL, cur, cur ^ 1, TILE_STORE, 0, key++);
                    for (int q = 0; q < P - 1; q++, cur ^= 1)
                        link(q, TRANSFORM_NODAL_TO_POINTS, cur, cur ^ 1, TILE_STORE, 0, key++);
                    link(P - 1, TRANSFORM_NODAL_TO_POINTS, cur, cur ^ 1, TILE_WACC | TILE_FIRST, d, kJoin);
                    prod = (cur ^ 1) - 2 * d;  // parity of the product vectors (the same for every chain)
                    maxdepth = std::max(maxdepth, depth);
                }
                int depth = maxdepth, prev = kJoin, cur = prod ^ 1;  // a vector holding no product
                phase(0, TRANSFORM_POINTS_TO_NODAL, prod, cur, TILE_STORE | TILE_WAIT_IN | TILE_SUMIN, 0, depth++, key,
                      prev);
                prev = key++;
                for (int q = 1; q < P; q++, cur ^= 1) {
                    phase(q, TRANSFORM_POINTS_TO_NODAL, cur, cur ^ 1, TILE_STORE | TILE_WAIT_IN, 0, depth++, key, prev);
                    prev = key++;
                }
                for (int q = 0; q < P - 1; q++, cur ^= 1) {
                    phase(q, TRANSFORM_NODAL_TO_MODAL, cur, cur ^ 1, TILE_STORE | TILE_WAIT_IN, 0, depth++, key, prev);
                    prev = key++;
                }
                phase(P - 1, TRANSFORM_NODAL_TO_MODAL, cur, 0, TILE_FIRST | TILE_LAST | rk | TILE_WAIT_IN, 0, depth++, key,
                      prev);
            }
            if (rk) {
                // The whole RK4 step in one launch: the group's phase graph once
                // per stage, stage s + 1 after stage s.  Every phase that
                // gathers the stage input waits, before gathering, for the
                // group's RK phase of the previous stage (which wrote it); the
                // RK phase completes last within its stage, so everything of
                // stage s precedes stage s + 1.  A group's stages thus
                // interleave with other groups' stages instead of meeting at
                // launch boundaries.
                std::vector<Phase> base = std::move(grp.phases);
                grp.phases.clear();
                int rkkey = -1;
                for (const Phase& ph : base)
                    if (!ph.items.empty() && (ph.items[0].flags & TILE_RK)) rkkey = ph.done_key;
                for (int st = 0; st < 4; st++)
                    for (const Phase& ph : base) {
                        Phase q;
                        q.items = ph.items;
                        for (MFItem& it : q.items) it.stage = (int16_t)(st + 1);
                        q.stage = st + 1;
                        q.depth = ph.depth;  // within the stage (the order offsets the stages)
                        q.done_key = ph.done_key + st * kStageKey;
                        q.wait_key = ph.wait_key >= 0 ? ph.wait_key + st * kStageKey : -1;
                        const bool reads_input = !ph.items.empty() && ph.items[0].src < 0;
                        if (st > 0 && reads_input) q.win_key = rkkey + (st - 1) * kStageKey;
                        grp.phases.push_back(std::move(q));
                    }
            }
            groups.push_back(std::move(grp));
        }
    }
    // counters: 0 hands out items; one per (group, done key).  A phase waits
    // for every item of the phases that increment its wait key.
    nctr = 1;
    std::vector<std::map<int, int>> ctr_of(groups.size());
    std::vector<std::map<int, int>> items_of(groups.size());
    for (size_t g = 0; g < groups.size(); g++)
        for (const Phase& ph : groups[g].phases) {
            if (!ctr_of[g].count(ph.done_key)) ctr_of[g][ph.done_key] = nctr++;
            items_of[g][ph.done_key] += (int)ph.items.size();
        }
    // wavefront order: a phase of depth p of stage s (0-based) of group g in
    // step s SO + g + kWaveLag p, older stages and then deeper phases (older
    // groups) first within a step, so a phase's predecessors were handed out
    // at least kWaveLag steps earlier.  A stage's wavefront starts SO >=
    // kWaveLag dmax + 1 steps after the previous one's (so a group's RK phase
    // of stage s comes before its stage s + 1), and SO >= G, so the next
    // stage ramps up while the previous one drains: about as many groups are
    // in flight as in one stage's wavefront, and their vectors stay in L2.
    int dmax = 0, nst = 1;
    for (auto& g : groups)
        for (const Phase& ph : g.phases) {
            dmax = std::max(dmax, ph.depth);
            nst = std::max(nst, ph.stage);
        }
    const size_t G = groups.size(), pmax = (size_t)dmax + 1;
    const size_t SO = std::max(G, kWaveLag * (size_t)dmax + 1);
    for (size_t t = 0; t < (size_t)(nst - 1) * SO + G + kWaveLag * pmax; t++)
        for (int st = 0; st < nst; st++)
            for (size_t pp = pmax; pp-- > 0;) {
                const size_t t0 = (size_t)st * SO + kWaveLag * pp;
                if (t < t0 || t - t0 >= G) continue;
                const size_t g = t - t0;
                for (const Phase& ph : groups[g].phases) {
                    if (ph.depth != (int)pp || std::max(ph.stage, 1) != st + 1) continue;
                    for (MFItem it : ph.items) {
                        it.done_ctr = ctr_of[g].at(ph.done_key);
                        it.wait_ctr = ph.wait_key >= 0 ? ctr_of[g].at(ph.wait_key) : -1;
                        it.wait_need = ph.wait_key >= 0 ? items_of[g].at(ph.wait_key) : 0;
                        it.win_ctr = ph.win_key >= 0 ? ctr_of[g].at(ph.win_key) : -1;
                        it.win_need = ph.win_key >= 0 ? items_of[g].at(ph.win_key) : 0;
                        items.push_back(it);
                    }
                }
            }
    return smem;
}

void MFEngine::build_items(std::vector<MFItem>& items, int& nctr, bool pass_only,
                           const std::map<std::pair<int, int>, MFTile>* shapes, int chunk, int nchunks,
                           std::vector<std::array<int, 3>>* ranges) {
    std::vector<WLClass> cls;
    for (auto& cp : classes_) {
        const SolveSpec& sp = solves_[cp->slots[0]].spec;
        cls.push_back(WLClass{sp.kind, sp.D, sp.k, sp.n, sp.apply, sp.apply_dim, cp->N, cp->Ns,
                              (int)cp->slots.size(), cp->pencils, cp->boff_index});
    }
    size_t smem = mf_work_list(cls, items, nctr, pass_only, shapes, chunk, nchunks, ranges);
    int tb = 0;
    for (auto& cp : classes_) {
        const SolveSpec& sp = solves_[cp->slots[0]].spec;
        const STable& S = stab(sp.k, sp.n);
        const int b = mf_table_bytes(S.nrow, S.nent, S.nval);
        if (b <= kMFTableSmemMax) tb = std::max(tb, b);
        if (sp.kind == MF_KIND_VLASOV) {  // the transforms share the slot, one at a time
            const TTables& T = ttab(sp.k, sp.n);
            for (int w = 0; w < 4; w++) {
                const int bt = mf_table_bytes(T.t[w].nrow, T.t[w].nent, T.t[w].nval);
                if (bt <= kMFTableSmemMax) tb = std::max(tb, bt);
            }
        }
    }
    table_bytes_ = tb;
    smem += (size_t)tb;
    if (smem > 227 * 1024) throw Error(SGDG_EUNSUPPORTED, "operator table and pencil tile exceed shared memory");
    smem_ = smem;
}

// ------------------------------------------------------------- tiles ----
static std::mutex g_tile_mu;
static std::map<std::pair<int, int>, MFTile> g_tiles;

MFTile mf_tile(int D, int k) {
    std::lock_guard<std::mutex> g(g_tile_mu);
    auto f = g_tiles.find({D, k});
    return f == g_tiles.end() ? MFTile{} : f->second;
}

bool mf_tile_tuned(int D, int k) {
    std::lock_guard<std::mutex> g(g_tile_mu);
    return g_tiles.count({D, k}) != 0;
}

void mf_set_tile(int D, int k, const MFTile& t) {
    if (t.wlog < kMFWlogMin || t.wlog > kMFWlogMax || t.coop < 1 || t.coop > 30)
        throw Error(SGDG_EINVAL, "tile shape: wlog must be in -2..3 and coop in 1..30");
    std::lock_guard<std::mutex> g(g_tile_mu);
    g_tiles[{D, k}] = t;
}

void mf_clear_tiles() {
    std::lock_guard<std::mutex> g(g_tile_mu);
    g_tiles.clear();
}

// For each (D, k) of the live solves without a tuned shape, times the pass
// tiles of one RK stage of the whole batch (the RK items left out: pass tiles
// only read the stage input and overwrite the partial sums, so no state
// changes) for every candidate shape of that (D, k) -- the others at their
// current shapes -- and keeps the fastest.  A candidate must beat the current
// shape by 2 % to replace it.
std::vector<std::pair<int, int>> MFEngine::autotune() {
    plan();
    std::vector<std::pair<int, int>> todo, done;
    for (auto& cp : classes_) {
        const SolveSpec& sp = solves_[cp->slots[0]].spec;
        const std::pair<int, int> dk{sp.D, sp.k};
        if (!mf_tile_tuned(sp.D, sp.k) && std::find(todo.begin(), todo.end(), dk) == todo.end()) todo.push_back(dk);
    }
    if (todo.empty()) return done;
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    std::map<std::pair<int, int>, MFTile> shapes;
    auto time_shapes = [&]() -> float {
        std::vector<MFItem> items;
        int nctr = 0;
        build_items(items, nctr, true, &shapes);
        DevBuf ti = upload(items, stream_);
        DevBuf tc(sizeof(int) * (size_t)std::max(nctr, 1));
        int bps = 0;
        CK(mf_configure(smem_, &bps));
        const int grid = std::max(1, bps) * sms;
        float best = 1e30f;
        for (int rep = 0; rep < 4; rep++) {
            CK(cudaEventRecord(e0, stream_));
            CK(launch_mf_stage(ti.as<MFItem>(), (int)items.size(), classes_d_.as<MFClass>(), tc.as<int>(), nctr, 1, 0,
                               err_d_.as<int>(), smem_, table_bytes_, grid, stream_));
            CK(cudaEventRecord(e1, stream_));
            CK(cudaEventSynchronize(e1));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (rep > 0) best = std::min(best, ms);  // the first launch warms up
        }
        if (check_error() != SGDG_OK) throw Error(SGDG_ETIMEOUT, "a bounded device wait gave up while tuning");
        return best;
    };
    try {
        for (auto& dk : todo) {
            MFTile best = mf_tile(dk.first, dk.second);
            shapes[dk] = best;
            float tbest = time_shapes();
            for (int wlog = kMFWlogMin; wlog <= kMFWlogMax; wlog++)
                for (int coop : {3, 4, 5, 6}) {
                    const MFTile cand{wlog, coop};
                    if (cand.wlog == best.wlog && cand.coop == best.coop) continue;
                    shapes[dk] = cand;
                    const float t = time_shapes();
                    if (t < 0.98f * tbest) {
                        tbest = t;
                        best = cand;
                    }
                }
            shapes[dk] = best;
            mf_set_tile(dk.first, dk.second, best);
            done.push_back(dk);
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        dirty_ = true;
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dirty_ = true;  // rebuild the work list with the tuned shapes
    drop_graph();
    plan();
    return done;
}

void MFEngine::capture() {
    cudaStream_t cs = stream_;
    cudaStream_t own = nullptr;
    if (cs == nullptr) {  // graphs cannot be captured on the legacy stream
        CK(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
        cs = own;
    }
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    // the work list holds the whole RK4 step (every item carries its stage)
    cudaError_t err = launch_mf_stage(items_d_.as<MFItem>(), nitems_, classes_d_.as<MFClass>(), ctr_d_.as<int>(),
                                      nctr_, 1, 0, err_d_.as<int>(), smem_, table_bytes_, grid_, cs);
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (own) cudaStreamDestroy(own);
    if (err != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        throw Error(SGDG_ECUDA, std::string("graph capture: ") + cudaGetErrorString(err != cudaSuccess ? err : e2));
    }
    cudaError_t e3 = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) {
        graph_ = nullptr;
        throw Error(SGDG_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e3));
    }
}

void MFEngine::build_chunks(int nchunks) {
    if ((int)chunks_.size() == nchunks) return;  // chunks_ is dropped with the graph on a re-plan
    for (Chunk& c : chunks_) {
        if (c.graph) cudaGraphExecDestroy(c.graph);
        if (c.st) {
            cudaStreamSynchronize(c.st);
            cudaStreamDestroy(c.st);
        }
    }
    chunks_.clear();
    chunks_.resize(nchunks);
    const size_t smem = smem_;
    const int tb = table_bytes_;
    // a chunk holds a fraction of the groups, so its phases wait on one
    // another more; with one CTA per SM per launch, as many chunks' stage
    // launches as CTAs fit on an SM run side by side and cover each other's
    // waits
    const int cgrid = nchunks > 1 ? std::max(1, sms_) : grid_;
    for (int ci = 0; ci < nchunks; ci++) {
        Chunk& ch = chunks_[ci];
        std::vector<MFItem> items;
        int nctr = 0;
        build_items(items, nctr, false, nullptr, ci, nchunks, &ch.ranges);
        smem_ = smem;  // build_items sized the launch for this chunk only; keep the whole list's
        table_bytes_ = tb;
        CK(cudaStreamCreateWithFlags(&ch.st, cudaStreamNonBlocking));
        ch.nitems = (int)items.size();
        ch.nctr = nctr;
        if (ch.nitems == 0) continue;
        ch.items = upload(items, ch.st);
        ch.ctr.alloc(sizeof(int) * (size_t)std::max(nctr, 1));
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(ch.st, cudaStreamCaptureModeThreadLocal));
        cudaError_t err = launch_mf_stage(ch.items.as<MFItem>(), ch.nitems, classes_d_.as<MFClass>(), ch.ctr.as<int>(),
                                          ch.nctr, 1, 0, err_d_.as<int>(), smem_, table_bytes_, cgrid, ch.st);
        cudaError_t e2 = cudaStreamEndCapture(ch.st, &g);
        if (err != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            throw Error(SGDG_ECUDA, std::string("graph capture: ") + cudaGetErrorString(err != cudaSuccess ? err : e2));
        }
        cudaError_t e3 = cudaGraphInstantiate(&ch.graph, g, 0);
        cudaGraphDestroy(g);
        if (e3 != cudaSuccess) {
            ch.graph = nullptr;
            throw Error(SGDG_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e3));
        }
    }
    for (Chunk& ch : chunks_) CK(cudaStreamSynchronize(ch.st));
}

void MFEngine::step_host(const double* in, double* out, int64_t nsteps, int nchunks) {
    plan();
    if (nsteps < 0) throw Error(SGDG_EINVAL, "nsteps must be >= 0");
    nchunks = std::max(1, std::min(nchunks, 64));
    build_chunks(nchunks);
    std::vector<int64_t> off(solves_.size(), -1);  // host offset of every live id
    int64_t o = 0;
    for (size_t id = 0; id < solves_.size(); id++)
        if (solves_[id].live) {
            off[id] = o;
            o += solves_[id].Ns;
        }
    cudaEvent_t ready;
    CK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    CK(cudaEventRecord(ready, stream_));  // after the engine stream's earlier work
    // copies of a chunk's slots: runs that are consecutive both on the device
    // and on the host
    auto copies = [&](const Chunk& ch, bool h2d) {
        for (const auto& r : ch.ranges) {
            const ClassArena& c = *classes_[r[0]];
            for (int s = r[1]; s < r[1] + r[2];) {
                const int64_t h = off[c.slots[s]];
                int run = 1;
                while (s + run < r[1] + r[2] && off[c.slots[s + run]] == h + (int64_t)run * c.Ns) run++;
                double* dv = c.y.as<double>() + (size_t)s * c.Ns;
                const size_t bytes = sizeof(double) * (size_t)c.Ns * run;
                if (h2d)
                    CK(cudaMemcpyAsync(dv, in + h, bytes, cudaMemcpyHostToDevice, ch.st));
                else
                    CK(cudaMemcpyAsync(out + h, dv, bytes, cudaMemcpyDeviceToHost, ch.st));
                s += run;
            }
        }
    };
    for (Chunk& ch : chunks_) {
        if (ch.ranges.empty()) continue;
        CK(cudaStreamWaitEvent(ch.st, ready, 0));
        copies(ch, true);
        for (const auto& r : ch.ranges) {
            const ClassArena& c = *classes_[r[0]];
            CK(launch_f64_to_f32(c.y.as<double>() + (size_t)r[1] * c.Ns, c.u0.as<float>() + (size_t)r[1] * c.Ns,
                                 (int64_t)r[2] * c.Ns, ch.st));
        }
        if (ch.graph)
            for (int64_t i = 0; i < nsteps; i++) CK(cudaGraphLaunch(ch.graph, ch.st));
        copies(ch, false);
    }
    for (Chunk& ch : chunks_) CK(cudaStreamSynchronize(ch.st));
    CK(cudaEventDestroy(ready));
    if (check_error() != SGDG_OK) throw Error(SGDG_ETIMEOUT, "a bounded device wait gave up; state is unreliable");
}

void MFEngine::step(int64_t nsteps) {
    plan();
    if (nitems_ == 0 || nsteps <= 0) return;
    if (!graph_) capture();
    for (int64_t i = 0; i < nsteps; i++) CK(cudaGraphLaunch(graph_, stream_));
}

int MFEngine::check_error() {
    if (!err_d_.p) return SGDG_OK;
    int h = 0;
    CK(cudaMemcpyAsync(&h, err_d_.p, sizeof(int), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    if (h) {
        CK(cudaMemsetAsync(err_d_.p, 0, sizeof(int), stream_));
        return SGDG_ETIMEOUT;
    }
    return SGDG_OK;
}

void MFEngine::get_state(int id, double* host) {
    plan();
    const Solve& s = at(id);
    const ClassArena& c = *classes_[s.cls];
    CK(cudaMemcpyAsync(host, c.y.as<double>() + (size_t)s.slot * c.Ns, sizeof(double) * c.Ns, cudaMemcpyDeviceToHost,
                       stream_));
    CK(cudaStreamSynchronize(stream_));
    if (check_error() != SGDG_OK) throw Error(SGDG_ETIMEOUT, "a bounded device wait gave up; state is unreliable");
}

void MFEngine::set_state(int id, const double* host) {
    Solve& s = at(id);
    if (dirty_ || s.cls < 0) {
        s.pending.assign(host, host + s.Ns);
        dirty_ = true;
        return;
    }
    const ClassArena& c = *classes_[s.cls];
    double* dst = c.y.as<double>() + (size_t)s.slot * c.Ns;
    CK(cudaMemcpyAsync(dst, host, sizeof(double) * c.Ns, cudaMemcpyHostToDevice, stream_));
    CK(launch_f64_to_f32(dst, c.u0.as<float>() + (size_t)s.slot * c.Ns, c.Ns, stream_));
}

void MFEngine::upload_all(const double* host) {
    plan();
    int64_t off = 0;
    int id = 0;
    const int n = (int)solves_.size();
    while (id < n) {
        if (!solves_[id].live) {
            id++;
            continue;
        }
        // one copy for a run of ids that sit in consecutive slots of one class
        const Solve& s = solves_[id];
        const ClassArena& c = *classes_[s.cls];
        int run = 1;
        while (id + run < n && solves_[id + run].live && solves_[id + run].cls == s.cls &&
               solves_[id + run].slot == s.slot + run)
            run++;
        CK(cudaMemcpyAsync(c.y.as<double>() + (size_t)s.slot * c.Ns, host + off, sizeof(double) * c.Ns * run,
                           cudaMemcpyHostToDevice, stream_));
        off += (int64_t)run * c.Ns;
        id += run;
    }
    for (auto& cp : classes_)
        CK(launch_f64_to_f32(cp->y.as<double>(), cp->u0.as<float>(), (int64_t)cp->slots.size() * cp->Ns, stream_));
}

void MFEngine::download_all(double* host) {
    plan();
    int64_t off = 0;
    int id = 0;
    const int n = (int)solves_.size();
    while (id < n) {
        if (!solves_[id].live) {
            id++;
            continue;
        }
        // merge a run of ids that sit in consecutive slots of one class
        const Solve& s = solves_[id];
        const ClassArena& c = *classes_[s.cls];
        int run = 1;
        while (id + run < n && solves_[id + run].live && solves_[id + run].cls == s.cls &&
               solves_[id + run].slot == s.slot + run)
            run++;
        CK(cudaMemcpyAsync(host + off, c.y.as<double>() + (size_t)s.slot * c.Ns, sizeof(double) * c.Ns * run,
                           cudaMemcpyDeviceToHost, stream_));
        off += (int64_t)run * c.Ns;
        id += run;
    }
    CK(cudaStreamSynchronize(stream_));
    if (check_error() != SGDG_OK) throw Error(SGDG_ETIMEOUT, "a bounded device wait gave up; state is unreliable");
}

void MFEngine::apply(const double* x_dev, double* y_dev) {
    plan();
    if (classes_.size() != 1 || classes_[0]->slots.size() != 1) throw Error(SGDG_EINVAL, "apply needs one solve");
    const ClassArena& c = *classes_[0];
    CK(launch_f64_to_f32(x_dev, c.u0.as<float>(), c.N, stream_));
    CK(launch_mf_stage(items_d_.as<MFItem>(), nitems_, classes_d_.as<MFClass>(), ctr_d_.as<int>(), nctr_, 1, 0,
                       err_d_.as<int>(), smem_, table_bytes_, grid_, stream_));
    CK(launch_f32_to_f64(c.rhs.as<float>(), y_dev, c.N, stream_));
}

}  // namespace sgdg
