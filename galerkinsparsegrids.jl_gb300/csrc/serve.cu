// serve.cu -- request loop of the matrix-free form (continuous batching).
//
// Requests (one solve each: kind, D, k, n, velocity, dt, initial state and a
// step count) queue in arrival order.  Each tick
//   1. admits queued requests that have arrived, in order, while the HBM
//      budget has room for their state plus the engine's re-plan reserve
//      (a request that cannot fit even into an empty engine fails);
//   2. advances every running request by the same number of RK4 steps --
//      the fewest steps any running request has left, at most max_chunk --
//      in the engine's persistent launches, so requests that arrived while
//      others were on the GPU share those launches from their first step;
//   3. retires the requests that are done: their state goes to host memory
//      and their device memory is freed for the next admissions.
// Only classes whose membership changed are re-laid out, so a join or leave
// costs one class arena rebuild and a graph re-capture.
//
// Each request's columns are computed exactly as when it runs alone (tiles
// never mix columns' arithmetic), so its result does not depend on the mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/sgdg.h"
#include "api_util.h"
#include "device_util.h"
#include "mf_engine.h"

namespace sgdg {

class Server {
   public:
    struct Request {
        SolveSpec spec;
        int64_t N = 0, Ns = 0, nsteps = 0, steps_done = 0;
        int state = SGDG_REQ_QUEUED, eid = -1, code = SGDG_OK;
        std::string msg;
        std::vector<double> y0, result;
        double t_arrival = 0, t_admit = -1, t_done = -1;
    };

    Server(int max_chunk, cudaStream_t st) : max_chunk_(max_chunk), eng_(st), t0_(Clock::now()) {}

    double now() const { return std::chrono::duration<double>(Clock::now() - t0_).count(); }

    int64_t submit(const SolveSpec& sp, const double* y0, int64_t nsteps, double t_arrival) {
        if (sp.k < 1 || sp.k > 5) throw Error(SGDG_EUNSUPPORTED, "served solves support 1 <= k <= 5");
        if (sp.D < 1 || sp.D > 8) throw Error(SGDG_EUNSUPPORTED, "served solves support 1 <= D <= 8");
        if (sp.n < 2) throw Error(SGDG_EINVAL, "n must be >= 2");
        if (nsteps < 1) throw Error(SGDG_EINVAL, "nsteps must be >= 1");
        if (!std::isfinite(sp.dt)) throw Error(SGDG_EINVAL, "dt must be finite");
        const SparseIndex ix = make_index(sp.D, sp.k, sp.n, sp.scheme);
        Request r;
        r.spec = sp;
        r.N = ix.N;
        r.Ns = sp.kind == MF_KIND_WAVE ? 2 * ix.N : ix.N;
        r.nsteps = nsteps;
        r.y0.assign(y0, y0 + r.Ns);
        r.t_arrival = t_arrival >= 0 ? t_arrival : now();
        const int64_t id = next_id_++;
        reqs_.emplace(id, std::move(r));
        queue_.push_back(id);
        return id;
    }

    int tick() {
        require_gpu();
        admit();
        if (running_.empty()) return 0;
        int64_t chunk = max_chunk_;
        for (int64_t id : running_) chunk = std::min(chunk, reqs_[id].nsteps - reqs_[id].steps_done);
        const double dof = eng_.dof_updates_per_step();
        eng_.step(chunk);
        CK(cudaStreamSynchronize(eng_.stream()));
        if (eng_.check_error() != SGDG_OK) {
            for (int64_t id : running_) fail(reqs_[id], SGDG_ETIMEOUT, "a bounded device wait gave up");
            running_.clear();
            throw Error(SGDG_ETIMEOUT, "a bounded device wait gave up; running requests failed");
        }
        dof_updates_ += dof * double(chunk);
        std::vector<int64_t> still, done;
        for (int64_t id : running_) {
            Request& r = reqs_[id];
            r.steps_done += chunk;
            (r.steps_done < r.nsteps ? still : done).push_back(id);
        }
        // copy every finished state out before any removal re-plans the engine
        for (int64_t id : done) {
            Request& r = reqs_[id];
            r.result.resize(r.Ns);
            eng_.get_state(r.eid, r.result.data());
        }
        for (int64_t id : done) {
            Request& r = reqs_[id];
            eng_.remove(r.eid);
            r.eid = -1;
            // a solve whose state is no longer finite (a NaN or infinity in its
            // input, or a step beyond stability) fails alone: its columns
            // never mix with other requests' arithmetic
            int64_t bad = -1;
            for (int64_t i = 0; i < r.Ns && bad < 0; i++)
                if (!std::isfinite(r.result[i])) bad = i;
            if (bad >= 0) {
                fail(r, SGDG_ENONFINITE, "state not finite after " + std::to_string(r.steps_done) +
                                             " steps (first at coefficient " + std::to_string(bad) + ")");
                r.result.clear();
                continue;
            }
            r.state = SGDG_REQ_DONE;
            r.t_done = now();
        }
        running_.swap(still);
        return (int)done.size();
    }

    void cancel(int64_t id) {
        Request& r = get(id);
        if (r.state == SGDG_REQ_QUEUED) {
            queue_.erase(std::find(queue_.begin(), queue_.end(), id));
        } else if (r.state == SGDG_REQ_RUNNING) {
            eng_.remove(r.eid);
            r.eid = -1;
            running_.erase(std::find(running_.begin(), running_.end(), id));
        } else {
            return;
        }
        r.state = SGDG_REQ_CANCELLED;
        r.code = SGDG_ECANCELLED;
        r.msg = "cancelled";
        r.t_done = now();
        r.y0.clear();
    }

    const Request& info(int64_t id) { return get(id); }

    // Checkpoint of a request: its state now and the steps it has done (a
    // queued request: its initial state and 0; a running one: the device
    // state between ticks; a finished one: its result).  Submitting that
    // state for the remaining steps continues the solve exactly: a solve's
    // arithmetic does not depend on how its steps are chunked.
    int64_t snapshot(int64_t id, double* y) {
        Request& r = get(id);
        if (r.state == SGDG_REQ_QUEUED) {
            std::copy(r.y0.begin(), r.y0.end(), y);
        } else if (r.state == SGDG_REQ_RUNNING) {
            eng_.get_state(r.eid, y);
        } else if (r.state == SGDG_REQ_DONE) {
            std::copy(r.result.begin(), r.result.end(), y);
        } else {
            throw Error(r.code, r.msg);
        }
        return r.steps_done;
    }

    // copies the result out and forgets the request
    void result(int64_t id, double* y) {
        Request& r = get(id);
        if (r.state == SGDG_REQ_QUEUED || r.state == SGDG_REQ_RUNNING)
            throw Error(SGDG_EINVAL, "request " + std::to_string(id) + " is not finished");
        if (r.state != SGDG_REQ_DONE) {
            const Error e(r.code, r.msg);
            reqs_.erase(id);
            throw e;
        }
        std::copy(r.result.begin(), r.result.end(), y);
        reqs_.erase(id);
    }

    void counts(int64_t* queued, int64_t* running, int64_t* finished, double* dof) const {
        if (queued) *queued = (int64_t)queue_.size();
        if (running) *running = (int64_t)running_.size();
        if (finished) *finished = (int64_t)reqs_.size() - (int64_t)queue_.size() - (int64_t)running_.size();
        if (dof) *dof = dof_updates_;
    }

    void set_stream(cudaStream_t st) { eng_.set_stream(st); }

   private:
    using Clock = std::chrono::steady_clock;

    Request& get(int64_t id) {
        auto it = reqs_.find(id);
        if (it == reqs_.end()) throw Error(SGDG_EINVAL, "no such request " + std::to_string(id));
        return it->second;
    }

    void fail(Request& r, int code, const std::string& msg) {
        r.state = SGDG_REQ_FAILED;
        r.code = code;
        r.msg = msg;
        r.t_done = now();
        r.y0.clear();
    }

    void admit() {
        const double t = now();
        while (!queue_.empty()) {
            const int64_t id = queue_.front();
            Request& r = reqs_[id];
            if (r.t_arrival > t) break;  // not arrived yet (arrival order is submission order)
            const int64_t need = MFEngine::solve_bytes(r.N, r.Ns);
            const int64_t budget = g_budget.load();
            if (budget > 0) {
                // bytes held once removed solves are freed, plus what a re-plan holds on top
                const int64_t held = g_in_use.load() - eng_.dead_bytes() + eng_.pending_bytes();
                if (held + eng_.replan_reserve() + need > budget) {
                    // the head of the line waits for memory, unless nothing is left to free
                    if (!running_.empty() || eng_.pending_bytes() > 0) break;
                    if (eng_.dead_bytes() > 0) {  // free the finished solves' arenas and look again
                        eng_.flush();
                        continue;
                    }
                    fail(r, SGDG_ENOMEM_BUDGET,
                         "request needs " + std::to_string(need) + " device bytes (+ " +
                             std::to_string(eng_.replan_reserve()) + " re-plan reserve); the HBM budget is " +
                             std::to_string(budget) + " with " + std::to_string(held) + " held");
                    queue_.pop_front();
                    continue;
                }
            }
            r.eid = eng_.add(r.spec, r.y0.data());
            r.y0.clear();
            r.y0.shrink_to_fit();
            r.state = SGDG_REQ_RUNNING;
            r.t_admit = now();
            running_.push_back(id);
            queue_.pop_front();
        }
    }

    int64_t max_chunk_;
    MFEngine eng_;
    Clock::time_point t0_;
    std::map<int64_t, Request> reqs_;
    std::deque<int64_t> queue_;
    std::vector<int64_t> running_;
    int64_t next_id_ = 0;
    double dof_updates_ = 0.0;
};

}  // namespace sgdg

using namespace sgdg;

struct sgdg_server {
    std::unique_ptr<Server> srv;
    cudaStream_t own = nullptr;
    ~sgdg_server() {
        srv.reset();  // frees device memory (waits for outstanding work)
        if (own) cudaStreamDestroy(own);
    }
};

extern "C" {

int sgdg_server_create(int max_chunk_steps, sgdg_server** out) {
    API_BEGIN
    NEED(out);
    if (max_chunk_steps < 1) throw Error(SGDG_EINVAL, "max_chunk_steps must be >= 1");
    require_gpu();
    auto s = std::make_unique<sgdg_server>();
    CK(cudaStreamCreateWithFlags(&s->own, cudaStreamNonBlocking));
    s->srv = std::make_unique<Server>(max_chunk_steps, s->own);
    *out = s.release();
    API_END
}

int sgdg_server_destroy(sgdg_server* s) {
    API_BEGIN
    delete s;
    API_END
}

int sgdg_server_set_stream(sgdg_server* s, void* stream) {
    API_BEGIN
    NEED(s);
    s->srv->set_stream(stream ? (cudaStream_t)stream : s->own);
    API_END
}

int sgdg_server_clock(sgdg_server* s, double* seconds) {
    API_BEGIN
    NEED(s);
    NEED(seconds);
    *seconds = s->srv->now();
    API_END
}

int sgdg_server_submit(sgdg_server* s, int kind, int D, int k, int n, int scheme, const double* a, double dt,
                       const double* y0, int64_t nsteps, double t_arrival, int64_t* request_id) {
    API_BEGIN
    NEED(s);
    NEED(y0);
    NEED(request_id);
    if (kind != SGDG_KIND_ADVECT && kind != SGDG_KIND_WAVE) throw Error(SGDG_EINVAL, "kind must be ADVECT or WAVE");
    if (kind == SGDG_KIND_ADVECT) NEED(a);
    SolveSpec sp{};
    sp.kind = kind == SGDG_KIND_WAVE ? MF_KIND_WAVE : MF_KIND_ADVECT;
    sp.D = D;
    sp.k = k;
    sp.n = n;
    sp.scheme = scheme;
    for (int d = 0; d < D && d < 8; d++) sp.a[d] = a ? a[d] : 0.0;
    sp.dt = dt;
    sp.apply_dim = -1;
    *request_id = s->srv->submit(sp, y0, nsteps, t_arrival);
    API_END
}

int sgdg_server_tick(sgdg_server* s, int* completed) {
    API_BEGIN
    NEED(s);
    const int c = s->srv->tick();
    if (completed) *completed = c;
    API_END
}

int sgdg_server_status(sgdg_server* s, int64_t request_id, int* state, int64_t* steps_done, double* t_arrival,
                       double* t_admit, double* t_done) {
    API_BEGIN
    NEED(s);
    const auto& r = s->srv->info(request_id);
    if (state) *state = r.state;
    if (steps_done) *steps_done = r.steps_done;
    if (t_arrival) *t_arrival = r.t_arrival;
    if (t_admit) *t_admit = r.t_admit;
    if (t_done) *t_done = r.t_done;
    API_END
}

int sgdg_server_result(sgdg_server* s, int64_t request_id, double* y) {
    API_BEGIN
    NEED(s);
    NEED(y);
    s->srv->result(request_id, y);
    API_END
}

int sgdg_server_snapshot(sgdg_server* s, int64_t request_id, double* y, int64_t* steps_done) {
    API_BEGIN
    NEED(s);
    NEED(y);
    const int64_t done = s->srv->snapshot(request_id, y);
    if (steps_done) *steps_done = done;
    API_END
}

int sgdg_server_cancel(sgdg_server* s, int64_t request_id) {
    API_BEGIN
    NEED(s);
    s->srv->cancel(request_id);
    API_END
}

int sgdg_server_counts(sgdg_server* s, int64_t* queued, int64_t* running, int64_t* finished, double* dof_updates) {
    API_BEGIN
    NEED(s);
    s->srv->counts(queued, running, finished, dof_updates);
    API_END
}

}  // extern "C"
