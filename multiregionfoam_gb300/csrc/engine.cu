// engine.cu -- host engine: device residency, plan upload, coefficient
// views, CUDA-graph iteration loops, FP32/FP64 iterative refinement.
#include "engine.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>

#include "../../include/mrgpu.h"
#include "kernels.h"

namespace mrg {

void cuda_check(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return;
    cudaGetLastError();
    int code = (e == cudaErrorMemoryAllocation) ? MRG_E_OOM : MRG_E_CUDA;
    throw Error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

// ------------------------------------------------------------------ Ctx
void* Ctx::alloc(size_t bytes)
{
    if (bytes == 0) bytes = 16;
    bytes = (bytes + 255) & ~(size_t)255;
    if (budget && used + bytes > budget)
        throw Error(MRG_E_OOM, "HBM budget exceeded: need " + std::to_string(bytes) + " B, used " +
                                   std::to_string(used) + " of " + std::to_string(budget));
    void* p = nullptr;
    MRG_CUDA(cudaMalloc(&p, bytes));
    MRG_CUDA(cudaMemsetAsync(p, 0, bytes, st));
    used += bytes;
    allocs[p] = bytes;
    return p;
}

void Ctx::release(void* p)
{
    if (!p) return;
    auto it = allocs.find(p);
    if (it == allocs.end()) return;
    used -= it->second;
    allocs.erase(it);
    cudaFree(p);
}

Ctx::~Ctx()
{
    if (st) cudaStreamSynchronize(st);
    for (auto& e : events)
        if (e) cudaEventDestroy(e);
    for (auto& kv : allocs) cudaFree(kv.first);
    allocs.clear();
    if (st) cudaStreamDestroy(st);
}

template <typename T>
static T* upload(Ctx* c, const std::vector<T>& v)
{
    T* p = (T*)c->alloc(sizeof(T) * std::max<size_t>(v.size(), 1));
    if (!v.empty()) MRG_CUDA(cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c->st));
    return p;
}

// ------------------------------------------------------------------ PlanState
PlanState::~PlanState()
{
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
    // device memory is owned by ctx allocations and freed with the mesh
}

void PlanState::sync_sys()
{
    MRG_CUDA(cudaMemcpyAsync(d_sys, &sys, sizeof(SysDev), cudaMemcpyHostToDevice, ctx->st));
}

static void release_plan(Ctx* c, PlanState* P)
{
    void* ptrs[] = {P->perm, P->a_sptr, P->a_col, P->a_src, P->chunk_start, P->lvl_chunk, P->f_sptr, P->f_col,
                    P->f_src, P->b_sptr, P->b_col, P->b_src, P->g_ptr, P->g_src, P->g_w, P->g_w32,
                    P->d_sys, P->d_tiles};
    for (void* p : ptrs) c->release(p);
    SysDev& S = P->sys;
    void* vals[] = {S.a_val, S.aT_val != S.a_val ? S.aT_val : nullptr, S.diag, S.sumA, S.f_c, S.f_cT, S.b_c,
                    S.b_cT, S.rD, S.D, S.a_val32, S.aT_val32 != S.a_val32 ? S.aT_val32 : nullptr, S.diag32,
                    S.f_c32, S.f_cT32, S.b_c32, S.b_cT32, S.rD32, S.partials, S.counter, S.sc};
    for (void* p : vals) c->release(p);
    for (auto* V : {&S.v64}) {
        void* vv[] = {V->x, V->b, V->r, V->w, V->y, V->p, V->q, V->rT, V->wT, V->yT, V->pT, V->qT};
        for (void* p : vv) c->release(p);
    }
    {
        auto* V = &S.v32;
        void* vv[] = {V->x, V->b, V->r, V->w, V->y, V->p, V->q, V->rT, V->wT, V->yT, V->pT, V->qT};
        for (void* p : vv) c->release(p);
    }
}

// ------------------------------------------------------------------ Mesh
Mesh::~Mesh()
{
    if (!ctx) return;
    cudaStreamSynchronize(ctx->st);
    for (auto& p : plans)
        if (p) release_plan(ctx, p.get());
    for (void* p : {(void*)raw_diag, (void*)raw_upper, (void*)raw_lower, (void*)raw_ibou, (void*)raw_iint})
        ctx->release(p);
}

PlanState& Mesh::plan(int ordering)
{
    if (ordering < 0 || ordering > 1) throw Error(MRG_E_INVALID, "ordering must be 0 (exact) or 1 (colour)");
    if (plans[ordering]) return *plans[ordering];
    auto P = std::make_unique<PlanState>();
    P->ctx = ctx;
    P->host = build_plan(n, nf, lower.data(), upper.data(), ifc, ordering);
    PlanHost& H = P->host;
    Ctx* c = ctx;
    P->perm = upload(c, H.perm);
    P->a_sptr = upload(c, H.a_sptr);
    P->a_col = upload(c, H.a_col);
    P->a_src = upload(c, H.a_src);
    P->chunk_start = upload(c, H.chunk_start);
    P->lvl_chunk = upload(c, H.lvl_chunk);
    P->f_sptr = upload(c, H.f_sptr);
    P->f_col = upload(c, H.f_col);
    P->f_src = upload(c, H.f_src);
    P->b_sptr = upload(c, H.b_sptr);
    P->b_col = upload(c, H.b_col);
    P->b_src = upload(c, H.b_src);
    P->g_ptr = upload(c, H.g_ptr);
    P->g_src = upload(c, H.g_src);
    P->g_w = upload(c, H.g_w);
    {
        std::vector<float> w32(H.g_w.begin(), H.g_w.end());
        P->g_w32 = upload(c, w32);
    }
    P->ntiles = H.npad / kTileRows;
    std::vector<int2> tiles(P->ntiles);
    for (int t = 0; t < P->ntiles; ++t) tiles[t] = make_int2(0, t);
    P->d_tiles = upload(c, tiles);

    SysDev& S = P->sys;
    std::memset(&S, 0, sizeof S);
    S.n = n;
    S.npad = H.npad;
    S.nsl = H.npad / kSlice;
    S.ntiles = P->ntiles;
    S.nchunks = H.nchunks;
    S.nlevels = H.nlevels;
    S.nf = nf;
    S.ni = ni;
    S.ngen = H.ngen;
    S.sym = 1;
    S.pc = PC_NONE;
    S.perm = P->perm;
    S.a_sptr = P->a_sptr;
    S.a_col = P->a_col;
    S.a_src = P->a_src;
    S.chunk_start = P->chunk_start;
    S.lvl_chunk = P->lvl_chunk;
    S.f_sptr = P->f_sptr;
    S.f_col = P->f_col;
    S.f_src = P->f_src;
    S.b_sptr = P->b_sptr;
    S.b_col = P->b_col;
    S.b_src = P->b_src;
    S.g_ptr = P->g_ptr;
    S.g_src = P->g_src;
    S.g_w = P->g_w;
    S.g_w32 = P->g_w32;
    const size_t nnz = H.a_col.size(), fnz = H.f_col.size(), bnz = H.b_col.size();
    const size_t np = (size_t)H.npad, nx = (size_t)H.npad + H.ngen;
    S.a_val = (double*)c->alloc(8 * nnz);
    S.aT_val = S.a_val;
    S.diag = (double*)c->alloc(8 * np);
    S.sumA = (double*)c->alloc(8 * np);
    S.f_c = (double*)c->alloc(8 * fnz);
    S.f_cT = (double*)c->alloc(8 * fnz);
    S.b_c = (double*)c->alloc(8 * bnz);
    S.b_cT = (double*)c->alloc(8 * bnz);
    S.rD = (double*)c->alloc(8 * np);
    S.D = (double*)c->alloc(8 * np);
    S.v64.x = (double*)c->alloc(8 * nx);
    S.v64.p = (double*)c->alloc(8 * nx);
    S.v64.b = (double*)c->alloc(8 * np);
    S.v64.r = (double*)c->alloc(8 * np);
    S.v64.w = (double*)c->alloc(8 * np);
    S.v64.y = (double*)c->alloc(8 * np);
    S.v64.q = (double*)c->alloc(8 * np);
    S.partials = (double*)c->alloc(8 * kMaxRed * (size_t)P->ntiles);
    S.counter = (unsigned*)c->alloc(64);
    S.sc = (Scal*)c->alloc(sizeof(Scal));
    P->d_sys = (SysDev*)c->alloc(sizeof(SysDev));
    P->sync_sys();
    // Keep only sizes on the host.
    H.perm.clear(); H.perm.shrink_to_fit();
    H.a_col.clear(); H.a_col.shrink_to_fit();
    H.a_src.clear(); H.a_src.shrink_to_fit();
    H.f_col.clear(); H.f_col.shrink_to_fit();
    H.f_src.clear(); H.f_src.shrink_to_fit();
    H.b_col.clear(); H.b_col.shrink_to_fit();
    H.b_src.clear(); H.b_src.shrink_to_fit();
    H.iperm.clear(); H.iperm.shrink_to_fit();
    H.level_of_row.clear(); H.level_of_row.shrink_to_fit();
    H.a_sptr.clear(); H.a_sptr.shrink_to_fit();
    H.f_sptr.clear(); H.f_sptr.shrink_to_fit();
    H.b_sptr.clear(); H.b_sptr.shrink_to_fit();
    // sizes retained for workspace allocation
    H.g_ptr.clear();
    H.g_src.clear();
    H.g_w.clear();
    H.chunk_start.clear();  // lvl_chunk (one int per level) stays for launch sizing
    plans[ordering] = std::move(P);
    // entry counts for the lazily allocated FP32 / transpose arrays
    nnz_cache[ordering][0] = nnz;
    nnz_cache[ordering][1] = fnz;
    nnz_cache[ordering][2] = bnz;
    MRG_CUDA(cudaStreamSynchronize(c->st));
    return *plans[ordering];
}

// ------------------------------------------------------------------ prepare
// One wave of 256-thread CTAs at the 4 per SM the kernels are compiled for.
static int grid_rows(const Ctx* c, int ntiles) { return std::max(1, std::min(ntiles, c->nsm * 4)); }
static int grid_sweep(const Ctx* c) { return c->nsm * 4; }

PlanState& prepare(Mesh& m, const Controls& cfg)
{
    if (!m.have_coeffs) throw Error(MRG_E_INVALID, "no coefficients uploaded for this mesh");
    PlanState& P = m.plan(cfg.ordering);
    Ctx* c = m.ctx;
    SysDev& S = P.sys;
    const size_t nnz = m.nnz_cache[cfg.ordering][0], fnz = m.nnz_cache[cfg.ordering][1],
                 bnz = m.nnz_cache[cfg.ordering][2];
    const size_t np = (size_t)S.npad, nx = (size_t)S.npad + S.ngen;
    bool rescatter = P.scattered != m.version;
    const bool asym = !m.sym || m.has_int;
    const bool need32 = cfg.precision == 1;
    const bool needT = cfg.solver == MRG_SOLVER_PBICG;
    S.sym = m.sym ? 1 : 0;
    S.raw_diag = m.raw_diag;
    S.raw_upper = m.raw_upper;
    S.raw_lower = m.raw_lower;
    S.raw_ibou = m.raw_ibou;
    S.raw_iint = m.raw_iint;
    if (asym && S.aT_val == S.a_val) {
        S.aT_val = (double*)c->alloc(8 * nnz);
        rescatter = true;
    }
    if (need32 && !P.have32) {
        S.a_val32 = (float*)c->alloc(4 * nnz);
        S.aT_val32 = asym ? (float*)c->alloc(4 * nnz) : S.a_val32;
        S.diag32 = (float*)c->alloc(4 * np);
        S.f_c32 = (float*)c->alloc(4 * fnz);
        S.f_cT32 = (float*)c->alloc(4 * fnz);
        S.b_c32 = (float*)c->alloc(4 * bnz);
        S.b_cT32 = (float*)c->alloc(4 * bnz);
        S.rD32 = (float*)c->alloc(4 * np);
        S.v32.x = (float*)c->alloc(4 * nx);
        S.v32.p = (float*)c->alloc(4 * nx);
        S.v32.r = (float*)c->alloc(4 * np);
        S.v32.w = (float*)c->alloc(4 * np);
        S.v32.y = (float*)c->alloc(4 * np);
        S.v32.q = (float*)c->alloc(4 * np);
        P.have32 = true;
        rescatter = true;
    }
    if (need32 && asym && S.aT_val32 == S.a_val32) {
        S.aT_val32 = (float*)c->alloc(4 * nnz);
        rescatter = true;
    }
    if (needT && !P.haveT) {
        S.v64.rT = (double*)c->alloc(8 * np);
        S.v64.wT = (double*)c->alloc(8 * np);
        S.v64.yT = (double*)c->alloc(8 * np);
        S.v64.pT = (double*)c->alloc(8 * nx);
        S.v64.qT = (double*)c->alloc(8 * np);
        P.haveT = true;
    }
    if (needT && need32 && !S.v32.rT) {
        S.v32.rT = (float*)c->alloc(4 * np);
        S.v32.wT = (float*)c->alloc(4 * np);
        S.v32.yT = (float*)c->alloc(4 * np);
        S.v32.pT = (float*)c->alloc(4 * nx);
        S.v32.qT = (float*)c->alloc(4 * np);
    }
    S.pc = cfg.pc;
    P.sync_sys();
    if (rescatter) {
        launch_rows(OP_SCATTER, 0, P.d_sys, P.d_tiles, P.ntiles, grid_rows(c, P.ntiles), 0, c->st);
        MRG_CUDA(cudaGetLastError());
        P.scattered = m.version;
        P.factored = 0;
    }
    const bool want32 = need32;
    if (cfg.pc >= PC_DIC) {
        if (P.factored != m.version || P.factored_pc != cfg.pc || (want32 && !P.factored32)) {
            launch_fill_sentinel(S.D, S.n, 0, c->st);
            launch_factor(P.d_sys, 1, S.nchunks, c->d_ctl, grid_sweep(c), want32 ? 1 : 0, c->st);
            MRG_CUDA(cudaGetLastError());
            P.factored = m.version;
            P.factored_pc = cfg.pc;
            P.factored32 = want32;
        }
    } else if (cfg.pc == PC_DIAG) {
        if (P.factored != m.version || P.factored_pc != cfg.pc || (want32 && !P.factored32)) {
            launch_rows(OP_DIAG_RD, 0, P.d_sys, P.d_tiles, P.ntiles, grid_rows(c, P.ntiles), 0, c->st);
            MRG_CUDA(cudaGetLastError());
            P.factored = m.version;
            P.factored_pc = cfg.pc;
            P.factored32 = want32;
        }
    }
    return P;
}

// ------------------------------------------------------------------ graphs
static void record_precondition(PlanState& P, const Controls& cfg, int prec, int trans, cudaStream_t st)
{
    Ctx* c = P.ctx;
    const SysDev& S = P.sys;
    if (cfg.pc >= PC_DIC) {
        if (cfg.ordering == MRG_ORDER_EXACT) {
            launch_sweep(prec, 1, trans, 1, 0, P.d_sys, 1, S.nchunks, c->d_ctl, grid_sweep(c), st);
            launch_sweep(prec, 0, trans, 1, 0, P.d_sys, 1, S.nchunks, c->d_ctl, grid_sweep(c), st);
        } else {
            // forward levels 1..nl-1, backward levels nl-2..0 (level 0 alone if
            // nl == 1); one chunk per warp of the widest level
            const int nl = S.nlevels;
            int widest = 1;
            for (int L = 0; L < nl; ++L)
                widest = std::max(widest, P.host.lvl_chunk[L + 1] - P.host.lvl_chunk[L]);
            const int g = std::max(1, std::min(65535, (widest + 7) / 8));
            for (int L = 1; L < nl; ++L) launch_sweep(prec, 1, trans, 0, L, P.d_sys, 1, 0, nullptr, g, st);
            for (int L = std::max(nl - 2, 0); L >= 0; --L)
                launch_sweep(prec, 0, trans, 0, L, P.d_sys, 1, 0, nullptr, g, st);
        }
    }
}

static void record_iteration(PlanState& P, const Controls& cfg, int prec, cudaStream_t st)
{
    Ctx* c = P.ctx;
    const int pb = cfg.solver == MRG_SOLVER_PBICG;
    const int g = grid_rows(c, P.ntiles);
    if (cfg.pc >= PC_DIC) {
        record_precondition(P, cfg, prec, 0, st);
        if (pb) record_precondition(P, cfg, prec, 1, st);
    } else if (cfg.pc == PC_DIAG) {
        launch_rows(OP_PRECOND_DIAG, prec, P.d_sys, P.d_tiles, P.ntiles, g, pb, st);
    } else {
        launch_rows(OP_PRECOND_NONE, prec, P.d_sys, P.d_tiles, P.ntiles, g, pb, st);
    }
    launch_rows(OP_RHO, prec, P.d_sys, P.d_tiles, P.ntiles, g, pb, st);
    launch_rows(OP_PUPDATE, prec, P.d_sys, P.d_tiles, P.ntiles, g, pb, st);
    if (P.sys.ngen) {
        launch_iface_gather(prec, 0, P.d_sys, 1, 64, st);
        if (pb) launch_iface_gather(prec, 2, P.d_sys, 1, 64, st);
    }
    launch_rows(OP_SPMV_QP, prec, P.d_sys, P.d_tiles, P.ntiles, g, pb, st);
    launch_rows(OP_UPDATE, prec, P.d_sys, P.d_tiles, P.ntiles, g, pb, st);
}

static PlanState::Graph iteration_graph(PlanState& P, const Controls& cfg, int prec, int k)
{
    std::string key = std::to_string(cfg.solver) + "/" + std::to_string(cfg.pc) + "/" +
                      std::to_string(cfg.ordering) + "/" + std::to_string(prec) + "/" + std::to_string(k);
    auto it = P.graphs.find(key);
    if (it != P.graphs.end()) return it->second;
    cudaStream_t st = P.ctx->st;
    cudaGraph_t g = nullptr;
    const unsigned long long before = launch_count();
    MRG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < k; ++i) record_iteration(P, cfg, prec, st);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    const long long nodes = (long long)(launch_count() - before);
    add_launches(-nodes);  // captured, not executed
    MRG_CUDA(e);
    cudaGraphExec_t ex = nullptr;
    MRG_CUDA(cudaGraphInstantiate(&ex, g, 0));
    cudaGraphDestroy(g);
    PlanState::Graph gr{ex, nodes};
    P.graphs[key] = gr;
    return gr;
}

struct Poll {
    Scal sc;
    Ctl ctl;
};

static Poll* pinned_poll()
{
    static thread_local Poll* p = nullptr;
    if (!p) MRG_CUDA(cudaMallocHost((void**)&p, sizeof(Poll)));
    return p;
}

static void poll(PlanState& P, Poll* h)
{
    Ctx* c = P.ctx;
    MRG_CUDA(cudaMemcpyAsync(&h->sc, P.sys.sc, sizeof(Scal), cudaMemcpyDeviceToHost, c->st));
    MRG_CUDA(cudaMemcpyAsync(&h->ctl, c->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, c->st));
    MRG_CUDA(cudaStreamSynchronize(c->st));
    if (h->ctl.err) {
        unsigned zero = 0;
        MRG_CUDA(cudaMemcpy(&c->d_ctl->err, &zero, sizeof zero, cudaMemcpyHostToDevice));
        throw Error(MRG_E_TIMEOUT, "device wait timed out in a preconditioner sweep");
    }
}

// Runs Krylov iterations until the device state says stop.
static void run_iterations(PlanState& P, const Controls& cfg, int prec, int max_iter, Poll* h)
{
    Ctx* c = P.ctx;
    const int k = std::max(1, cfg.k_launch);
    PlanState::Graph gr = iteration_graph(P, cfg, prec, k);
    poll(P, h);
    long launches = 0;
    const long cap = (long)max_iter / k + 2 + (long)cfg.min_iter / k;
    while (h->sc.active && launches <= cap) {
        MRG_CUDA(cudaGraphLaunch(gr.exec, c->st));
        add_launches(gr.nodes);
        ++launches;
        poll(P, h);
    }
}

static void write_controls(PlanState& P, double tol, double rel_tol, int min_iter, int max_iter)
{
    struct {
        double tol, rel_tol;
    } d{tol, rel_tol};
    struct {
        int min_iter, max_iter;
    } i{min_iter, max_iter};
    Ctx* c = P.ctx;
    char* base = (char*)P.sys.sc;
    MRG_CUDA(cudaMemcpyAsync(base + offsetof(Scal, tol), &d, sizeof d, cudaMemcpyHostToDevice, c->st));
    MRG_CUDA(cudaMemcpyAsync(base + offsetof(Scal, min_iter), &i, sizeof i, cudaMemcpyHostToDevice, c->st));
    MRG_CUDA(cudaStreamSynchronize(c->st));
}

static void init_sentinels(PlanState& P, const Controls& cfg, int prec)
{
    if (cfg.pc < PC_DIC || cfg.ordering != MRG_ORDER_EXACT) return;
    const SysDev& S = P.sys;
    Ctx* c = P.ctx;
    if (prec == 0) {
        launch_fill_sentinel(S.v64.y, S.n, 0, c->st);
        if (cfg.solver == MRG_SOLVER_PBICG) launch_fill_sentinel(S.v64.yT, S.n, 0, c->st);
    } else {
        launch_fill_sentinel(S.v32.y, S.n, 1, c->st);
        if (cfg.solver == MRG_SOLVER_PBICG) launch_fill_sentinel(S.v32.yT, S.n, 1, c->st);
    }
}

Perf solve_device(Mesh& m, const double* d_b, double* d_x, const Controls& cfg)
{
    Ctx* c = m.ctx;
    PlanState& P = prepare(m, cfg);
    const SysDev& S = P.sys;
    cudaStream_t st = c->st;
    const int pb = cfg.solver == MRG_SOLVER_PBICG;
    const int g = grid_rows(c, P.ntiles);
    Poll* h = pinned_poll();
    cudaEvent_t e0, e1;
    MRG_CUDA(cudaEventCreate(&e0));
    MRG_CUDA(cudaEventCreate(&e1));
    MRG_CUDA(cudaEventRecord(e0, st));
    Perf perf;
    try {
        launch_permute(1, P.d_sys, 0, d_b, S.v64.b, S.n, st);
        launch_permute(1, P.d_sys, 0, d_x, S.v64.x, S.n, st);
        write_controls(P, cfg.tol, cfg.rel_tol, cfg.min_iter, cfg.max_iter);
        if (S.ngen) launch_iface_gather(0, 1, P.d_sys, 1, 64, st);
        launch_rows(OP_SUMX, 0, P.d_sys, P.d_tiles, P.ntiles, g, 0, st);
        launch_rows(OP_INIT_RES, 0, P.d_sys, P.d_tiles, P.ntiles, g, pb, st);
        MRG_CUDA(cudaGetLastError());
        if (cfg.precision == MRG_PRECISION_FP64) {
            init_sentinels(P, cfg, 0);
            run_iterations(P, cfg, 0, cfg.max_iter, h);
            perf.res0 = h->sc.res0;
            perf.res = h->sc.res;
            perf.iters = h->sc.iter;
            perf.converged = h->sc.converged;
            perf.singular = h->sc.singular;
        } else {
            poll(P, h);
            const double nfac = h->sc.nfac, res0 = h->sc.res0;
            perf.res0 = res0;
            double res = res0;
            bool conv = h->sc.converged;
            int inner_total = 0, outer = 0;
            const int inner_max = cfg.inner_max_iter > 0 ? cfg.inner_max_iter : cfg.max_iter;
            double best = res;
            int stall = 0;
            while ((!conv || inner_total < cfg.min_iter) && outer < cfg.max_outer && inner_total < cfg.max_iter) {
                if (S.ngen) launch_iface_gather(0, 1, P.d_sys, 1, 64, st);
                launch_rows(OP_RESID64, 0, P.d_sys, P.d_tiles, P.ntiles, g, 0, st);
                // Each refinement step aims past the target (0.1 x the residual
                // still to remove) so the last step overshoots instead of
                // landing just under the tolerance; the FP32 inner solve is not
                // asked for more than inner_rel_tol per step.
                const double goal = std::max(cfg.tol, cfg.rel_tol > 1e-20 ? cfg.rel_tol * res0 : 0.0);
                const double inner_tol = std::min(0.5, std::max(cfg.inner_rel_tol, 0.1 * goal / res));
                write_controls(P, inner_tol, 0.0, 0, std::min(inner_max, cfg.max_iter - inner_total));
                launch_rows(OP_TO32, 0, P.d_sys, P.d_tiles, P.ntiles, g, 0, st);
                if (pb) {
                    // transpose residual of the correction system starts equal to r
                    MRG_CUDA(cudaMemcpyAsync(S.v32.rT, S.v32.r, 4 * (size_t)S.npad, cudaMemcpyDeviceToDevice, st));
                }
                init_sentinels(P, cfg, 1);
                run_iterations(P, cfg, 1, inner_max, h);
                inner_total += h->sc.iter;
                ++outer;
                launch_rows(OP_CORRECT, 0, P.d_sys, P.d_tiles, P.ntiles, g, 0, st);
                if (S.ngen) launch_iface_gather(0, 1, P.d_sys, 1, 64, st);
                launch_rows(OP_RESID64, 0, P.d_sys, P.d_tiles, P.ntiles, g, 0, st);
                poll(P, h);
                res = h->sc.osum / nfac;
                conv = res < cfg.tol || (cfg.rel_tol > 1e-20 && res < cfg.rel_tol * res0);
                if (!(res < best * 0.999)) {
                    if (++stall >= 3) break;
                } else {
                    stall = 0;
                    best = res;
                }
                if (h->sc.iter == 0) break;
            }
            perf.res = res;
            perf.iters = inner_total;
            perf.outer = outer;
            perf.converged = conv;
        }
        launch_permute(0, P.d_sys, 0, S.v64.x, d_x, S.n, st);
        MRG_CUDA(cudaEventRecord(e1, st));
        MRG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        perf.ms = ms;
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!std::isfinite(perf.res0) || !std::isfinite(perf.res)) perf.status = MRG_E_BREAKDOWN;
    return perf;
}

// ------------------------------------------------------------------ building blocks
void amul_device(Mesh& m, const double* d_x, double* d_y, int transpose)
{
    Controls cfg;
    cfg.pc = PC_NONE;
    cfg.solver = transpose ? MRG_SOLVER_PBICG : MRG_SOLVER_PCG;
    PlanState& P = prepare(m, cfg);
    const SysDev& S = P.sys;
    Ctx* c = m.ctx;
    launch_permute(1, P.d_sys, 0, d_x, S.v64.p, S.n, c->st);
    if (S.ngen) launch_iface_gather(0, 3, P.d_sys, 1, 64, c->st);
    launch_rows(transpose ? OP_TMUL : OP_AMUL, 0, P.d_sys, P.d_tiles, P.ntiles, grid_rows(c, P.ntiles), 0, c->st);
    launch_permute(0, P.d_sys, 0, S.v64.q, d_y, S.n, c->st);
    MRG_CUDA(cudaGetLastError());
    MRG_CUDA(cudaStreamSynchronize(c->st));
}

void residual_device(Mesh& m, const double* d_b, const double* d_x, double* res, double* nfac)
{
    Controls cfg;
    cfg.pc = PC_NONE;
    PlanState& P = prepare(m, cfg);
    const SysDev& S = P.sys;
    Ctx* c = m.ctx;
    launch_permute(1, P.d_sys, 0, d_b, S.v64.b, S.n, c->st);
    launch_permute(1, P.d_sys, 0, d_x, S.v64.x, S.n, c->st);
    write_controls(P, 0.0, 0.0, 0, 0);
    if (S.ngen) launch_iface_gather(0, 1, P.d_sys, 1, 64, c->st);
    const int g = grid_rows(c, P.ntiles);
    launch_rows(OP_SUMX, 0, P.d_sys, P.d_tiles, P.ntiles, g, 0, c->st);
    launch_rows(OP_INIT_RES, 0, P.d_sys, P.d_tiles, P.ntiles, g, 0, c->st);
    Poll* h = pinned_poll();
    poll(P, h);
    if (res) *res = h->sc.res0;
    if (nfac) *nfac = h->sc.nfac;
}

void precondition_device(Mesh& m, int pc, int ordering, const double* d_r, double* d_w, int transpose)
{
    Controls cfg;
    cfg.pc = pc;
    cfg.ordering = ordering;
    cfg.solver = transpose ? MRG_SOLVER_PBICG : MRG_SOLVER_PCG;
    PlanState& P = prepare(m, cfg);
    const SysDev& S = P.sys;
    Ctx* c = m.ctx;
    launch_permute(1, P.d_sys, 0, d_r, transpose ? S.v64.rT : S.v64.r, S.n, c->st);
    // mark the system active so the sweeps run
    {
        int one = 1;
        MRG_CUDA(cudaMemcpyAsync((char*)S.sc + offsetof(Scal, active), &one, sizeof one, cudaMemcpyHostToDevice,
                                 c->st));
    }
    if (pc >= PC_DIC) {
        if (ordering == MRG_ORDER_EXACT) launch_fill_sentinel(transpose ? S.v64.yT : S.v64.y, S.n, 0, c->st);
        record_precondition(P, cfg, 0, transpose, c->st);
    } else {
        launch_rows(pc == PC_DIAG ? OP_PRECOND_DIAG : OP_PRECOND_NONE, 0, P.d_sys, P.d_tiles, P.ntiles,
                    grid_rows(c, P.ntiles), transpose, c->st);
    }
    launch_permute(0, P.d_sys, 0, transpose ? S.v64.wT : S.v64.w, d_w, S.n, c->st);
    MRG_CUDA(cudaGetLastError());
    Poll* h = pinned_poll();
    poll(P, h);
}

void factor_diag_device(Mesh& m, int pc, int ordering, double* d_rD)
{
    Controls cfg;
    cfg.pc = pc;
    cfg.ordering = ordering;
    PlanState& P = prepare(m, cfg);
    Ctx* c = m.ctx;
    launch_permute(0, P.d_sys, 0, P.sys.rD, d_rD, P.sys.n, c->st);
    MRG_CUDA(cudaGetLastError());
    Poll* h = pinned_poll();
    poll(P, h);
}

float time_kernel(Mesh& m, const Controls& cfg, int kernel, int reps)
{
    if (reps < 1) throw Error(MRG_E_INVALID, "reps must be >= 1");
    if (kernel < 0 || kernel > 1) throw Error(MRG_E_INVALID, "unknown kernel id");
    PlanState& P = prepare(m, cfg);
    Ctx* c = m.ctx;
    const int prec = cfg.precision;
    const int pb = cfg.solver == MRG_SOLVER_PBICG;
    int one = 1;
    MRG_CUDA(cudaMemcpyAsync((char*)P.sys.sc + offsetof(Scal, active), &one, sizeof one, cudaMemcpyHostToDevice,
                             c->st));
    if (kernel == 1 && cfg.pc >= PC_DIC && cfg.ordering == MRG_ORDER_EXACT) init_sentinels(P, cfg, prec);
    auto once = [&] {
        if (kernel == 0)
            launch_rows(OP_SPMV_QP, prec, P.d_sys, P.d_tiles, P.ntiles, grid_rows(c, P.ntiles), pb, c->st);
        else
            record_precondition(P, cfg, prec, 0, c->st);
    };
    once();  // warm-up
    cudaEvent_t e0, e1;
    MRG_CUDA(cudaEventCreate(&e0));
    MRG_CUDA(cudaEventCreate(&e1));
    MRG_CUDA(cudaEventRecord(e0, c->st));
    for (int i = 0; i < reps; ++i) once();
    MRG_CUDA(cudaEventRecord(e1, c->st));
    MRG_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int zero = 0;
    MRG_CUDA(cudaMemcpyAsync((char*)P.sys.sc + offsetof(Scal, active), &zero, sizeof zero, cudaMemcpyHostToDevice,
                             c->st));
    MRG_CUDA(cudaStreamSynchronize(c->st));
    MRG_CUDA(cudaGetLastError());
    return ms / reps;
}

}  // namespace mrg
