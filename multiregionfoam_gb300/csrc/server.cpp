// server.cpp -- continuous batching of solve requests (see server.h).
//
// The server thread owns the context's streams while it runs.  Each pass of
// its loop: admit queued requests in arrival order while batch slots and the
// HBM budget allow (a mesh has at most one step in flight: its next time
// step waits for the previous one); launch each running batch's captured
// K-iteration graph once on the main stream; meanwhile, on a side stream,
// start the admitted requests (coefficients, b and x0 uploaded, views and
// factor, initial residual) in an admission batch -- they touch only their
// own meshes' memory, so this overlaps the running iterations; gather every
// running member's state; run the mixed-precision outer step for members
// whose inner loop ended; copy out and complete the members that
// converged; then the admitted requests join the running batch.  New
// requests therefore join while others are mid-solve, and all members share
// every kernel launch.
#include "server.h"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>

#include "../../include/mrgpu.h"

namespace mrg {

namespace {
double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// Route the context's work to another stream for a scope (the server thread
// is the context's only user while the server runs).
struct StreamSwap {
    Ctx* c;
    cudaStream_t old;
    StreamSwap(Ctx* ctx, cudaStream_t s) : c(ctx), old(ctx->st) { c->st = s; }
    ~StreamSwap() { c->st = old; }
};
}  // namespace

Server::Server(Ctx* ctx, const Controls& sym, const Controls* asym, size_t budget, int max_active)
    : ctx_(ctx), budget_(budget), max_active_(max_active > 0 ? max_active : 256)
{
    if (sym.solver != MRG_SOLVER_PCG && sym.solver != MRG_SOLVER_BICGSTAB)
        throw Error(MRG_E_INVALID, "symmetric controls must select PCG or BiCGStab");
    if (asym && asym->solver != MRG_SOLVER_PBICG && asym->solver != MRG_SOLVER_BICGSTAB)
        throw Error(MRG_E_INVALID, "asymmetric controls must select PBiCG or BiCGStab");
    fam_[0].cfg = sym;
    fam_[0].enabled = true;
    if (asym) {
        fam_[1].cfg = *asym;
        fam_[1].enabled = true;
    }
    for (Family& F : fam_) {
        F.main.init(ctx_);
        F.sub.init(ctx_);
        F.fb.init(ctx_);
        F.adm.init(ctx_);
    }
    MRG_CUDA(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
    MRG_CUDA(cudaEventCreateWithFlags(&side_done_, cudaEventDisableTiming));
    MRG_CUDA(cudaStreamSynchronize(ctx_->st));
    const char* e = std::getenv("MRG_SERVER_PROFILE");
    prof_.on = e && e[0] == '1';
    thread_ = std::thread([this] { loop(); });
}

Server::~Server()
{
    {
        std::lock_guard<std::mutex> lk(mu_);
        stopping_ = true;
    }
    cv_work_.notify_all();
    if (thread_.joinable()) thread_.join();
    cudaStreamSynchronize(ctx_->st);
    std::vector<Request*> left;
    {
        std::lock_guard<std::mutex> lk(mu_);
        for (auto& kv : reqs_)
            if (kv.second->state != 2) left.push_back(kv.second);
    }
    for (Request* r : left) complete(r, MRG_E_INVALID, "server destroyed before the request completed");
    for (auto& kv : reqs_) delete kv.second;
    for (auto& kv : slots_) ctx_->release(kv.second.d_bx);
    if (side_) {
        cudaStreamSynchronize(side_);
        cudaStreamDestroy(side_);
    }
    if (side_done_) cudaEventDestroy(side_done_);
    if (prof_.on)
        std::fprintf(stderr,
                     "mrg server: %d passes, %d rebuilds; host ms: idle %.1f, iterate %.1f, admissions %.1f, "
                     "harvest %.1f, rebuild %.1f\n",
                     prof_.passes, prof_.rebuilds, prof_.idle, prof_.iterate, prof_.start, prof_.harvest,
                     prof_.rebuild);
}

size_t Server::estimate(const Mesh& m) const
{
    // FP64 and FP32 work vectors, plan, coefficient views and their FP32
    // copies (about 224 B per cell and 128 B per face for a symmetric
    // matrix; asymmetric ones keep transposed views too).
    const size_t per_cell = 224, per_face = m.sym ? 128 : 192;
    return per_cell * (size_t)m.n + per_face * (size_t)m.nf + 16 * (size_t)m.n;
}

uint64_t Server::submit(Mesh* m, int asym, const double* diag, const double* upper, const double* lower,
                        const double* ibou, const double* iint, const double* b, const double* x0, double* x_out)
{
    if (!m || !diag || (m->nf > 0 && !upper) || !b || !x0 || !x_out) throw Error(MRG_E_INVALID, "NULL argument");
    if (m->ctx != ctx_) throw Error(MRG_E_INVALID, "the mesh belongs to another context");
    const int f = asym ? 1 : 0;
    if (!fam_[f].enabled) throw Error(MRG_E_INVALID, "this server takes no asymmetric (PBiCG) requests");
    if (asym && !lower) throw Error(MRG_E_INVALID, "an asymmetric request needs lower coefficients");
    auto* r = new Request();
    r->mesh = m;
    r->fam = f;
    r->diag = diag;
    r->upper = upper;
    r->lower = lower;
    r->ibou = ibou;
    r->iint = iint;
    r->b = b;
    r->x0 = x0;
    r->x_out = x_out;
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (stopping_) {
            delete r;
            throw Error(MRG_E_INVALID, "server is stopping");
        }
        if (queue_.size() >= 1u << 20) {
            delete r;
            throw Error(MRG_E_BUSY, "server queue full");
        }
        r->id = next_id_++;
        r->t_submit = now_ms();
        reqs_[r->id] = r;
        slots_[m];   // create the mesh's slot here, under the lock
        queue_.push_back(r);
        ++st_.submitted;
        st_.queued = (int)queue_.size();
    }
    cv_work_.notify_one();
    return r->id;
}

int Server::poll(uint64_t id, bool* done, Perf* perf, double* latency_ms, std::string* err)
{
    std::lock_guard<std::mutex> lk(mu_);
    auto it = reqs_.find(id);
    if (it == reqs_.end()) throw Error(MRG_E_INVALID, "unknown request id (or already collected)");
    Request* r = it->second;
    if (r->state != 2) {
        *done = false;
        return MRG_OK;
    }
    *done = true;
    if (perf) *perf = r->perf;
    if (latency_ms) *latency_ms = r->t_done - r->t_submit;
    if (err) *err = r->err;
    const int status = r->status;
    reqs_.erase(it);
    delete r;
    return status;
}

int Server::wait(uint64_t id, double timeout_ms, bool* done, Perf* perf, double* latency_ms, std::string* err)
{
    {
        std::unique_lock<std::mutex> lk(mu_);
        auto it = reqs_.find(id);
        if (it == reqs_.end()) throw Error(MRG_E_INVALID, "unknown request id (or already collected)");
        Request* r = it->second;
        auto ready = [r] { return r->state == 2; };
        if (timeout_ms < 0)
            cv_done_.wait(lk, ready);
        else
            cv_done_.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready);
    }
    return poll(id, done, perf, latency_ms, err);
}

ServerStats Server::stats()
{
    std::lock_guard<std::mutex> lk(mu_);
    return st_;
}

void Server::complete(Request* r, int status, const std::string& err)
{
    std::lock_guard<std::mutex> lk(mu_);
    r->state = 2;
    r->status = status;
    r->err = err;
    r->t_done = now_ms();
    st_.inflight_bytes -= std::min(st_.inflight_bytes, r->charged);
    r->charged = 0;
    auto it = slots_.find(r->mesh);
    if (it != slots_.end()) it->second.busy = false;
    ++st_.completed;
    cv_done_.notify_all();
}

void Server::loop()
{
    cudaSetDevice(ctx_->device);
    for (;;) {
        std::vector<Request*> admitted[2], rejected;
        {
            std::unique_lock<std::mutex> lk(mu_);
            const bool idle = fam_[0].running.empty() && fam_[1].running.empty() && fam_[0].fbrun.empty() &&
                              fam_[1].fbrun.empty();
            if (idle) cv_work_.wait(lk, [this] { return stopping_ || !queue_.empty(); });
            if (stopping_) break;
            for (auto it = queue_.begin(); it != queue_.end();) {
                Request* r = *it;
                Slot& sl = slots_[r->mesh];
                if (sl.busy) {   // the mesh's previous step is still in flight
                    ++it;
                    continue;
                }
                const int f = r->fam;
                if ((int)(fam_[f].running.size() + admitted[f].size()) >= max_active_) {
                    ++it;
                    continue;
                }
                const size_t need = sl.bytes ? sl.bytes : estimate(*r->mesh);
                if (budget_ && need > budget_) {
                    rejected.push_back(r);
                    it = queue_.erase(it);
                    continue;
                }
                if (budget_ && st_.inflight_bytes + need > budget_) break;   // first come, first served
                sl.busy = true;
                r->charged = need;
                r->state = 1;
                st_.inflight_bytes += need;
                st_.peak_inflight_bytes = std::max(st_.peak_inflight_bytes, st_.inflight_bytes);
                admitted[f].push_back(r);
                it = queue_.erase(it);
            }
            st_.queued = (int)queue_.size();
        }
        for (Request* r : rejected)
            complete(r, MRG_E_OOM, "the request's working set exceeds the server's HBM budget");
        double tp = prof_.on ? now_ms() : 0.0;
        if (prof_.on) {
            ++prof_.passes;
            if (prof_.t_sync > 0) prof_.idle += tp - prof_.t_sync;
            prof_.t_sync = 0;
        }
        for (int f = 0; f < 2; ++f) {
            try {
                if (!fam_[f].running.empty()) batch_iterate(fam_[f].main, fam_[f].cfg);
                if (!fam_[f].fbrun.empty()) batch_iterate(fam_[f].fb, fallback_controls(fam_[f].cfg), 0);
            } catch (const Error& e) {
                fail_family(f, e.code, e.what());
            }
        }
        if (prof_.on) {
            const double t = now_ms();
            prof_.iterate += t - tp;
            tp = t;
        }
        // admissions on the side stream, overlapping the iterations above
        bool any_admitted = false;
        {
            StreamSwap swap(ctx_, side_);
            for (int f = 0; f < 2; ++f)
                if (!admitted[f].empty()) {
                    start(f, admitted[f]);
                    any_admitted = true;
                }
            if (any_admitted) cudaEventRecord(side_done_, side_);
        }
        if (prof_.on) {
            const double t = now_ms();
            prof_.start += t - tp;
            tp = t;
        }
        for (int f = 0; f < 2; ++f) {
            try {
                bool changed = false;
                if (!fam_[f].running.empty() || !fam_[f].fbrun.empty()) changed = harvest(f);
                if (!fam_[f].joining.empty()) {
                    MRG_CUDA(cudaStreamWaitEvent(ctx_->st, side_done_, 0));
                    fam_[f].running.insert(fam_[f].running.end(), fam_[f].joining.begin(), fam_[f].joining.end());
                    fam_[f].joining.clear();
                    changed = true;
                }
                if (prof_.on) {
                    const double t = now_ms();
                    prof_.harvest += t - tp;
                    tp = t;
                }
                if (changed) {
                    rebuild(f);
                    if (prof_.on) {
                        const double t = now_ms();
                        prof_.rebuild += t - tp;
                        ++prof_.rebuilds;
                        tp = t;
                    }
                }
            } catch (const Error& e) {
                fail_family(f, e.code, e.what());
            }
        }
        std::lock_guard<std::mutex> lk(mu_);
        st_.running = (int)(fam_[0].running.size() + fam_[1].running.size() + fam_[0].fbrun.size() +
                            fam_[1].fbrun.size());
        st_.peak_running = std::max(st_.peak_running, st_.running);
    }
}

static std::vector<PlanState*> plans_of(const std::vector<Mesh*>& ms, int ordering)
{
    std::vector<PlanState*> ps;
    for (Mesh* m : ms) ps.push_back(&m->plan(ordering));
    return ps;
}

void Server::start(int f, std::vector<Request*>& rs)
{
    Family& F = fam_[f];
    cudaStream_t st = ctx_->st;
    for (Request* r : rs) {
        try {
            Mesh& m = *r->mesh;
            Slot* sl;
            {
                std::lock_guard<std::mutex> lk(mu_);
                sl = &slots_[&m];
            }
            const bool had_plan = m.plans[F.cfg.ordering] != nullptr;
            const size_t before = ctx_->used;
            upload_coeffs(m, r->diag, r->upper, r->lower, r->ibou, r->iint, cudaMemcpyHostToDevice, false);
            const size_t n = (size_t)m.n;
            if (!sl->d_bx) sl->d_bx = (double*)ctx_->alloc(16 * n);
            MRG_CUDA(cudaMemcpyAsync(sl->d_bx, r->b, 8 * n, cudaMemcpyHostToDevice, st));
            MRG_CUDA(cudaMemcpyAsync(sl->d_bx + n, r->x0, 8 * n, cudaMemcpyHostToDevice, st));
            PlanState& P = m.plan(F.cfg.ordering);
            P.sys.in_b = sl->d_bx;
            P.sys.in_x = sl->d_bx + n;
            P.sys.out_x = sl->d_bx + n;
            F.adm.set({&P});
            std::vector<Mesh*> ms{&m};
            prepare_batch(F.adm, ms, F.cfg);
            F.adm.sync_sys();
            batch_begin(F.adm, F.cfg);
            const size_t grew = ctx_->used - before;
            {
                std::lock_guard<std::mutex> lk(mu_);
                if (!sl->bytes) {
                    // measured when this admission built the working set
                    sl->bytes = had_plan ? std::max(grew, estimate(m)) : grew;
                    st_.inflight_bytes += sl->bytes;
                    st_.inflight_bytes -= std::min(st_.inflight_bytes, r->charged);
                    r->charged = sl->bytes;
                    st_.peak_inflight_bytes = std::max(st_.peak_inflight_bytes, st_.inflight_bytes);
                }
            }
            F.joining.push_back(r);
        } catch (const Error& e) {
            complete(r, e.code, e.what());
        }
    }
}

bool Server::harvest(int f)
{
    Family& F = fam_[f];
    const bool mixed = F.cfg.precision == MRG_PRECISION_MIXED;
    std::vector<Request*> outer, fallback, done;
    if (!F.running.empty()) {
        std::vector<Scal> sc;
        batch_status(F.main, sc);
        if (prof_.on && prof_.t_sync == 0) prof_.t_sync = now_ms();   // the main stream has drained
        for (size_t s = 0; s < F.running.size(); ++s) {
            if (sc[s].active) continue;
            if (mixed && sc[s].ostate)
                outer.push_back(F.running[s]);
            else if (mixed && sc[s].fallback == 1)
                fallback.push_back(F.running[s]);
            else
                done.push_back(F.running[s]);
        }
    }
    if (!F.fbrun.empty()) {
        std::vector<Scal> sc;
        batch_status(F.fb, sc);
        std::vector<Request*> ended;
        for (size_t s = 0; s < F.fbrun.size(); ++s)
            if (!sc[s].active) ended.push_back(F.fbrun[s]);
        if (!ended.empty()) {
            // the true FP64 residual of each finished FP64 continuation
            std::vector<Mesh*> ms;
            for (Request* r : ended) ms.push_back(r->mesh);
            F.sub.set(plans_of(ms, F.cfg.ordering));
            batch_fallback(F.sub, F.cfg);
            done.insert(done.end(), ended.begin(), ended.end());
        }
    }
    if (outer.empty() && fallback.empty() && done.empty()) return false;
    if (!outer.empty()) {
        // correction, FP64 residual and the next inner start of the members
        // whose FP32 loop ended; those whose refinement ended are complete
        // or, when it stalled, continue in FP64
        std::vector<Mesh*> ms;
        for (Request* r : outer) ms.push_back(r->mesh);
        F.sub.set(plans_of(ms, F.cfg.ordering));
        batch_outer(F.sub, F.cfg);
        std::vector<Scal> s2;
        batch_status(F.sub, s2);
        for (size_t i = 0; i < outer.size(); ++i) {
            if (s2[i].ostate) continue;
            if (s2[i].fallback == 1)
                fallback.push_back(outer[i]);
            else
                done.push_back(outer[i]);
        }
    }
    if (!fallback.empty()) {
        std::vector<Mesh*> ms;
        for (Request* r : fallback) ms.push_back(r->mesh);
        F.sub.set(plans_of(ms, F.cfg.ordering));
        batch_fallback(F.sub, F.cfg);
        std::vector<Scal> s4;
        batch_status(F.sub, s4);
        for (size_t i = 0; i < fallback.size(); ++i) {
            Request* r = fallback[i];
            F.running.erase(std::find(F.running.begin(), F.running.end(), r));
            if (s4[i].active)
                F.fbrun.push_back(r);
            else
                done.push_back(r);
        }
    }
    if (!done.empty()) finish(f, done);
    return true;
}

void Server::finish(int f, std::vector<Request*>& done)
{
    Family& F = fam_[f];
    std::vector<Mesh*> ms;
    for (Request* r : done) ms.push_back(r->mesh);
    F.sub.set(plans_of(ms, F.cfg.ordering));
    batch_finish(F.sub);
    std::vector<Scal> s3;
    batch_status(F.sub, s3);
    for (Request* r : done) {
        Slot* sl;
        {
            std::lock_guard<std::mutex> lk(mu_);
            sl = &slots_[r->mesh];
        }
        const size_t n = (size_t)r->mesh->n;
        MRG_CUDA(cudaMemcpyAsync(r->x_out, sl->d_bx + n, 8 * n, cudaMemcpyDeviceToHost, ctx_->st));
    }
    MRG_CUDA(cudaStreamSynchronize(ctx_->st));
    for (size_t i = 0; i < done.size(); ++i) {
        Request* r = done[i];
        Perf p = perf_of(s3[i], F.cfg.precision);
        r->perf = p;
        auto it = std::find(F.running.begin(), F.running.end(), r);
        if (it != F.running.end()) F.running.erase(it);
        it = std::find(F.fbrun.begin(), F.fbrun.end(), r);
        if (it != F.fbrun.end()) F.fbrun.erase(it);
        complete(r, p.status, p.status ? "non-finite residual (breakdown)" : "");
    }
}

void Server::rebuild(int f)
{
    Family& F = fam_[f];
    std::vector<Mesh*> ms;
    for (Request* r : F.running) ms.push_back(r->mesh);
    F.main.set(plans_of(ms, F.cfg.ordering));
    batch_recount(F.main);
    ms.clear();
    for (Request* r : F.fbrun) ms.push_back(r->mesh);
    F.fb.set(plans_of(ms, F.cfg.ordering));
    batch_recount(F.fb);
}

void Server::fail_family(int f, int code, const std::string& msg)
{
    Family& F = fam_[f];
    cudaStreamSynchronize(ctx_->st);
    cudaStreamSynchronize(side_);
    std::vector<Request*> rs;
    rs.swap(F.running);
    rs.insert(rs.end(), F.fbrun.begin(), F.fbrun.end());
    rs.insert(rs.end(), F.joining.begin(), F.joining.end());
    F.fbrun.clear();
    F.joining.clear();
    for (Request* r : rs) complete(r, code, msg);
    try {
        F.main.set({});
        F.fb.set({});
    } catch (const Error&) {
    }
}

}  // namespace mrg
