// engine.cu -- host engine: device residency, plan upload, coefficient
// views, batches, CUDA-graph iteration loops, FP32/FP64 iterative refinement.
#include "engine.h"
#include "gamg.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
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

// The same with `extra` zero elements after the data (Ctx::alloc clears):
// the streamed SpMV copies a round's slice bounds as 12 ints from 8 r, up to
// 3 past the last bound.
template <typename T>
static T* upload_padded(Ctx* c, const std::vector<T>& v, size_t extra)
{
    T* p = (T*)c->alloc(sizeof(T) * (v.size() + extra));
    if (!v.empty()) MRG_CUDA(cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c->st));
    return p;
}

// One wave of 256-thread CTAs at the 4 per SM the kernels are compiled for.
static int grid_sweep(const Ctx* c) { return c->nsm * 4; }
// CTAs per SM of the sync-free exact sweeps (MRG_SF_CTAS, 1..4, default 3):
// every warp beyond the level front polls its dependencies in L2, and three
// CTAs an SM measured fastest (the 737k-cell PBiCG solve 200 -> 191 ms; the
// 3.1M-cell PCG solve within 1 %)
static int grid_sf(const Ctx* c)
{
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("MRG_SF_CTAS");
        v = e ? std::max(1, std::min(4, std::atoi(e))) : 3;
    }
    return c->nsm * v;
}

// ------------------------------------------------------------------ BatchHost
void BatchHost::init(Ctx* c)
{
    ctx = c;
    d = (Batch*)c->alloc(sizeof(Batch));
    d_ctl = (Ctl*)c->alloc(sizeof(Ctl));
}

BatchHost::~BatchHost()
{
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
    if (!ctx) return;
    for (void* p : {(void*)d, (void*)d_ctl, (void*)d_sys, (void*)d_tiles, (void*)d_segs, (void*)d_items,
                    (void*)d_item_off, (void*)d_scal, (void*)d_sf})
        ctx->release(p);
}

template <typename T>
static void ensure(Ctx* c, T*& p, size_t& cap, size_t n)
{
    if (cap >= n && p) return;
    c->release(p);
    cap = std::max<size_t>(n, 1);
    p = (T*)c->alloc(sizeof(T) * cap);
}

void BatchHost::set(const std::vector<PlanState*>& systems)
{
    members = systems;
    const int nsys = (int)systems.size();
    std::vector<SysDev> sv(nsys);
    std::vector<int2> tiles, segs;
    int maxchunks = 0, maxlevels = 0;
    for (int s = 0; s < nsys; ++s) {
        const PlanState* P = systems[s];
        sv[s] = P->sys;
        for (int t = 0; t < P->ntiles; ++t) tiles.push_back(make_int2(s, t));
        for (int j = 0; j < red_segments(P->ntiles); ++j) segs.push_back(make_int2(s, j));
        maxchunks = std::max(maxchunks, P->sys.nchunks);
        if (!P->sys.syncfree) maxlevels = std::max(maxlevels, P->sys.nlevels);
    }
    // level-sweep work list (colour-ordered members): (system, chunk) by level
    std::vector<int2> items;
    std::vector<int> off(maxlevels + 1, 0);
    widest_level = 1;
    for (int L = 0; L < maxlevels; ++L) {
        off[L] = (int)items.size();
        for (int s = 0; s < nsys; ++s) {
            const PlanState* P = systems[s];
            if (P->sys.syncfree || L >= P->sys.nlevels) continue;
            for (int c = P->host.lvl_chunk[L]; c < P->host.lvl_chunk[L + 1]; ++c) items.push_back(make_int2(s, c));
        }
        widest_level = std::max(widest_level, (int)items.size() - off[L]);
    }
    off[maxlevels] = (int)items.size();
    // sync-free sweep work of several systems: every chunk of the sync-free
    // members, level by level (a member's chunks in its own order), so a
    // sweep's tickets visit only chunks that exist and every dependency's
    // chunk comes earlier in the list (later for the backward sweep, which
    // reads it from the end); one system claims its chunks directly
    std::vector<int2> sf;
    if (nsys > 1) {
        int sl = 0;
        for (const PlanState* P : systems)
            if (P->sys.syncfree) sl = std::max(sl, P->sys.nlevels);
        for (int L = 0; L < sl; ++L)
            for (int s = 0; s < nsys; ++s) {
                const PlanState* P = systems[s];
                if (!P->sys.syncfree || L >= P->sys.nlevels) continue;
                for (int c = P->host.lvl_chunk[L]; c < P->host.lvl_chunk[L + 1]; ++c) sf.push_back(make_int2(s, c));
            }
    }
    ensure(ctx, d_sys, cap_sys, (size_t)nsys);
    ensure(ctx, d_tiles, cap_tiles, tiles.size());
    ensure(ctx, d_segs, cap_segs, segs.size());
    ensure(ctx, d_items, cap_items, items.size());
    ensure(ctx, d_item_off, cap_off, off.size());
    ensure(ctx, d_sf, cap_sf, sf.size());
    cudaStream_t st = ctx->st;
    if (nsys) MRG_CUDA(cudaMemcpyAsync(d_sys, sv.data(), sizeof(SysDev) * nsys, cudaMemcpyHostToDevice, st));
    if (!tiles.empty())
        MRG_CUDA(cudaMemcpyAsync(d_tiles, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice, st));
    if (!segs.empty())
        MRG_CUDA(cudaMemcpyAsync(d_segs, segs.data(), sizeof(int2) * segs.size(), cudaMemcpyHostToDevice, st));
    if (!items.empty())
        MRG_CUDA(cudaMemcpyAsync(d_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, st));
    MRG_CUDA(cudaMemcpyAsync(d_item_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, st));
    if (!sf.empty())
        MRG_CUDA(cudaMemcpyAsync(d_sf, sf.data(), sizeof(int2) * sf.size(), cudaMemcpyHostToDevice, st));
    h.sf_items = d_sf;
    h.n_sf = (int)sf.size();
    h.sys = d_sys;
    h.tiles = d_tiles;
    h.segs = d_segs;
    h.nsegs = (int)segs.size();
    h.items = d_items;
    h.item_off = d_item_off;
    h.ctl = d_ctl;
    h.nsys = nsys;
    h.ntiles = (int)tiles.size();
    h.maxchunks = maxchunks;
    h.maxlevels = maxlevels;
    MRG_CUDA(cudaMemcpyAsync(d, &h, sizeof(Batch), cudaMemcpyHostToDevice, st));
    // Graphs refer to the descriptor's address only; their key holds the
    // launch shapes (grids, level count), so one captured for an earlier
    // membership stays valid while the shapes match.
    if (graphs.size() > 32) {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
    }
    MRG_CUDA(cudaStreamSynchronize(st));
}

void BatchHost::sync_sys()
{
    const int nsys = (int)members.size();
    std::vector<SysDev> sv(nsys);
    for (int s = 0; s < nsys; ++s) sv[s] = members[s]->sys;
    if (nsys)
        MRG_CUDA(cudaMemcpyAsync(d_sys, sv.data(), sizeof(SysDev) * nsys, cudaMemcpyHostToDevice, ctx->st));
}

// ------------------------------------------------------------------ PlanState
PlanState::~PlanState() {}

void PlanState::sync_sys()
{
    MRG_CUDA(cudaMemcpyAsync(d_sys, &sys, sizeof(SysDev), cudaMemcpyHostToDevice, ctx->st));
}

static void release_plan(Ctx* c, PlanState* P)
{
    void* ptrs[] = {P->perm, P->a_sptr, P->a_col, P->a_src, P->a_col16, P->a_cbase, P->chunk_start, P->lvl_chunk,
                    P->f_sptr, P->f_col,
                    P->f_src, P->b_sptr, P->b_col, P->b_src, P->g_ptr, P->g_src, P->g_w, P->g_w32, P->d_sys,
                    P->pt_ptr, P->part_rows, P->part_step, P->f_row, P->b_row, P->f_loc, P->b_loc};
    for (void* p : ptrs) c->release(p);
    SysDev& S = P->sys;
    void* vals[] = {S.a_val, S.aT_val != S.a_val ? S.aT_val : nullptr, S.diag, S.sumA, S.f_c, S.f_cT, S.b_c,
                    S.b_cT, S.rD, S.D, S.a_val32, S.aT_val32 != S.a_val32 ? S.aT_val32 : nullptr, S.diag32,
                    S.f_c32, S.f_cT32, S.b_c32, S.b_cT32, S.rD32, S.partials, S.counter, S.sc, S.xb, S.rb};
    for (void* p : vals) c->release(p);
    for (void* p : {(void*)S.v64.x, (void*)S.v64.b, (void*)S.v64.r, (void*)S.v64.w, (void*)S.v64.y,
                    (void*)S.v64.p, (void*)S.v64.q, (void*)S.v64.rT, (void*)S.v64.wT, (void*)S.v64.yT,
                    (void*)S.v64.pT, (void*)S.v64.qT, (void*)S.v32.x, (void*)S.v32.b, (void*)S.v32.r,
                    (void*)S.v32.w, (void*)S.v32.y, (void*)S.v32.p, (void*)S.v32.q, (void*)S.v32.rT,
                    (void*)S.v32.wT, (void*)S.v32.yT, (void*)S.v32.pT, (void*)S.v32.qT})
        c->release(p);
}

// ------------------------------------------------------------------ Mesh

// Copy a mesh's coefficients into its raw device arrays (caller numbering)
// and bump its coefficient version; views and factors follow lazily.
void upload_coeffs(Mesh& m, const double* diag, const double* upper, const double* lower, const double* ibou,
                   const double* iint, cudaMemcpyKind kind, bool sync)
{
    if (!diag || (m.nf > 0 && !upper)) throw Error(MRG_E_INVALID, "diag/upper must not be NULL");
    if (m.ni > 0 && !ibou) throw Error(MRG_E_INVALID, "interface coefficients must not be NULL");
    Ctx* c = m.ctx;
    if (!m.raw_diag) m.raw_diag = (double*)c->alloc(8 * (size_t)m.n);
    if (!m.raw_upper) m.raw_upper = (double*)c->alloc(8 * (size_t)std::max(m.nf, 1));
    if (lower && !m.raw_lower) m.raw_lower = (double*)c->alloc(8 * (size_t)std::max(m.nf, 1));
    if (m.ni && !m.raw_ibou) m.raw_ibou = (double*)c->alloc(8 * (size_t)m.ni);
    if (iint && !m.raw_iint) m.raw_iint = (double*)c->alloc(8 * (size_t)m.ni);
    MRG_CUDA(cudaMemcpyAsync(m.raw_diag, diag, 8 * (size_t)m.n, kind, c->st));
    if (m.nf) MRG_CUDA(cudaMemcpyAsync(m.raw_upper, upper, 8 * (size_t)m.nf, kind, c->st));
    if (lower && m.nf) MRG_CUDA(cudaMemcpyAsync(m.raw_lower, lower, 8 * (size_t)m.nf, kind, c->st));
    if (m.ni) MRG_CUDA(cudaMemcpyAsync(m.raw_ibou, ibou, 8 * (size_t)m.ni, kind, c->st));
    if (iint && m.ni) MRG_CUDA(cudaMemcpyAsync(m.raw_iint, iint, 8 * (size_t)m.ni, kind, c->st));
    const bool new_sym = lower == nullptr, new_int = iint != nullptr;
    if (m.have_coeffs && (new_sym != m.sym || new_int != m.has_int)) {
        // symmetry changed: the transposed views must be rebuilt
        for (auto& p : m.plans)
            if (p) p->scattered = 0;
    }
    m.sym = new_sym;
    m.has_int = new_int;
    m.have_coeffs = true;
    ++m.version;
    if (sync) MRG_CUDA(cudaStreamSynchronize(c->st));
}


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
    // owner-computes exact sweeps: parts of about part_target cells (at most
    // one per SM), their values in shared memory; a mesh whose parts would
    // exceed kPartMaxCells keeps the ticketed kernel (measured on GB300: 3.1M
    // cells in 152 parts sweep 1.7x slower than ticketed, 262k cells in 64
    // parts 1.6x faster)
    if (ordering == 0 && c->nsm > 0) {
        const int parts = std::max(1, std::min(c->nsm, (n + part_target - 1) / part_target));
        if ((n + parts - 1) / parts <= kPartMaxCells) build_parts(H, parts);
    }
    if (H.nparts) {
        P->pt_ptr = upload(c, H.pt_ptr);
        P->part_rows = upload(c, H.part_rows);
        P->part_step = upload(c, H.part_step);
        P->f_row = upload(c, H.f_row);
        P->b_row = upload(c, H.b_row);
        P->f_loc = upload(c, H.f_loc);
        P->b_loc = upload(c, H.b_loc);
    }
    P->perm = upload(c, H.perm);
    P->a_sptr = upload_padded(c, H.a_sptr, 16);
    P->a_col = upload(c, H.a_col);
    P->a_src = upload(c, H.a_src);
    P->a_col16 = upload(c, H.a_col16);
    P->a_cbase = upload_padded(c, H.a_cbase, 8);
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
    P->nnz = H.a_col.size();
    P->fnz = H.f_col.size();
    P->bnz = H.b_col.size();

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
    S.syncfree = ordering == 0 ? 1 : 0;
    S.perm = P->perm;
    S.a_sptr = P->a_sptr;
    S.a_col = P->a_col;
    S.a_src = P->a_src;
    S.a_col16 = P->a_col16;
    S.a_cbase = P->a_cbase;
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
    S.nparts = H.nparts;
    S.part_cells = H.part_cells;
    S.pt_ptr = P->pt_ptr;
    S.part_rows = P->part_rows;
    S.part_step = P->part_step;
    S.f_row = reinterpret_cast<const int2*>(P->f_row);
    S.b_row = reinterpret_cast<const int2*>(P->b_row);
    S.f_loc = P->f_loc;
    S.b_loc = P->b_loc;
    const size_t np = (size_t)H.npad, nx = (size_t)H.npad + H.ngen;
    S.a_val = (double*)c->alloc(8 * P->nnz);
    S.aT_val = S.a_val;
    S.diag = (double*)c->alloc(8 * np);
    S.sumA = (double*)c->alloc(8 * np);
    S.f_c = (double*)c->alloc(8 * P->fnz);
    S.f_cT = (double*)c->alloc(8 * P->fnz);
    S.b_c = (double*)c->alloc(8 * P->bnz);
    S.b_cT = (double*)c->alloc(8 * P->bnz);
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
    // Keep only sizes (and the per-level chunk offsets) on the host.
    H.a_col16.clear();
    H.a_col16.shrink_to_fit();
    for (auto* v : {&H.perm, &H.a_col, &H.a_src, &H.f_col, &H.f_src, &H.b_col, &H.b_src, &H.iperm,
                    &H.level_of_row, &H.a_sptr, &H.f_sptr, &H.b_sptr, &H.g_ptr, &H.g_src, &H.chunk_start,
                    &H.a_cbase, &H.pt_ptr, &H.part_rows, &H.part_step, &H.f_row, &H.b_row, &H.f_loc, &H.b_loc}) {
        v->clear();
        v->shrink_to_fit();
    }
    H.g_w.clear();
    H.g_w.shrink_to_fit();
    P->single.init(c);
    P->single.set({P.get()});
    plans[ordering] = std::move(P);
    MRG_CUDA(cudaStreamSynchronize(c->st));
    return *plans[ordering];
}

// ------------------------------------------------------------------ prepare
// Allocations a system needs for these controls; returns true when its
// SysDev changed (the batch arrays must be re-uploaded).
static bool ensure_views(Mesh& m, PlanState& P, const Controls& cfg)
{
    Ctx* c = m.ctx;
    SysDev& S = P.sys;
    const size_t np = (size_t)S.npad, nx = (size_t)S.npad + S.ngen;
    const bool asym = !m.sym || m.has_int;
    const bool need32 = cfg.precision == MRG_PRECISION_MIXED;
    // PBiCG's transpose system, BiCGStab's extra vectors
    const bool needT = cfg.solver == MRG_SOLVER_PBICG || cfg.solver == MRG_SOLVER_BICGSTAB;
    bool changed = false;
    auto setp = [&](auto& field, auto value) {
        if (field != value) {
            field = value;
            changed = true;
        }
    };
    setp(S.sym, m.sym ? 1 : 0);
    setp(S.raw_diag, (const double*)m.raw_diag);
    setp(S.raw_upper, (const double*)m.raw_upper);
    setp(S.raw_lower, (const double*)m.raw_lower);
    setp(S.raw_ibou, (const double*)m.raw_ibou);
    setp(S.raw_iint, (const double*)m.raw_iint);
    setp(S.pc, cfg.pc);
    if (cfg.pc == PC_BLOCK) {
        setp(S.blk, (const BlockDev*)block_view(m, P).d);
        P.bs_blocks = m.blocks->bs;
    }
    if (asym && S.aT_val == S.a_val) {
        S.aT_val = (double*)c->alloc(8 * P.nnz);
        P.scattered = 0;
        changed = true;
    }
    if (need32 && !P.have32) {
        S.a_val32 = (float*)c->alloc(4 * P.nnz);
        S.aT_val32 = asym ? (float*)c->alloc(4 * P.nnz) : S.a_val32;
        S.diag32 = (float*)c->alloc(4 * np);
        S.f_c32 = (float*)c->alloc(4 * P.fnz);
        S.f_cT32 = (float*)c->alloc(4 * P.fnz);
        S.b_c32 = (float*)c->alloc(4 * P.bnz);
        S.b_cT32 = (float*)c->alloc(4 * P.bnz);
        S.rD32 = (float*)c->alloc(4 * np);
        S.v32.x = (float*)c->alloc(4 * nx);
        S.v32.p = (float*)c->alloc(4 * nx);
        S.v32.r = (float*)c->alloc(4 * np);
        S.v32.w = (float*)c->alloc(4 * np);
        S.v32.y = (float*)c->alloc(4 * np);
        S.v32.q = (float*)c->alloc(4 * np);
        S.xb = (double*)c->alloc(8 * np);
        S.rb = (double*)c->alloc(8 * np);
        S.chunk_rw = (float*)c->alloc(4 * (size_t)std::max(1, S.nchunks));
        P.have32 = true;
        P.scattered = 0;
        changed = true;
    }
    if (need32 && asym && S.aT_val32 == S.a_val32) {
        S.aT_val32 = (float*)c->alloc(4 * P.nnz);
        P.scattered = 0;
        changed = true;
    }
    if (needT && !P.haveT) {
        S.v64.rT = (double*)c->alloc(8 * np);
        S.v64.wT = (double*)c->alloc(8 * np);
        S.v64.yT = (double*)c->alloc(8 * np);
        S.v64.pT = (double*)c->alloc(8 * nx);
        S.v64.qT = (double*)c->alloc(8 * np);
        P.haveT = true;
        changed = true;
    }
    if (needT && need32 && !P.haveT32) {
        S.v32.rT = (float*)c->alloc(4 * np);
        S.v32.wT = (float*)c->alloc(4 * np);
        S.v32.yT = (float*)c->alloc(4 * np);
        S.v32.pT = (float*)c->alloc(4 * nx);
        S.v32.qT = (float*)c->alloc(4 * np);
        P.haveT32 = true;
        changed = true;
    }
    if (changed) P.sync_sys();
    return changed;
}

void prepare_batch(BatchHost& bh, const std::vector<Mesh*>& meshes, const Controls& cfg)
{
    Ctx* c = bh.ctx;
    bool changed = false, rescatter = false, refactor = false;
    const bool want32 = cfg.precision == MRG_PRECISION_MIXED;
    for (size_t s = 0; s < meshes.size(); ++s) {
        Mesh& m = *meshes[s];
        PlanState& P = *bh.members[s];
        if (!m.have_coeffs) throw Error(MRG_E_INVALID, "no coefficients uploaded for a mesh of the batch");
        changed |= ensure_views(m, P, cfg);
        if (P.scattered != m.version) rescatter = true;
        if (cfg.pc >= PC_DIAG &&
            (P.factored != m.version || P.factored_pc != cfg.pc || (want32 && !P.factored32)))
            refactor = true;
    }
    if (changed) {
        bh.sync_sys();
        // the single-system batches of the members see the same SysDev
        for (PlanState* P : bh.members)
            if (&P->single != &bh) P->single.sync_sys();
    }
    const int nt = bh.h.ntiles, ns = bh.h.nsegs;
    // the factor re-arms from the scatter (which writes D's sentinels)
    if (rescatter || (refactor && cfg.pc >= PC_DIC)) {
        launch_rows(OP_SCATTER, 0, bh.d, nt, ns, 0, c->st);
        MRG_CUDA(cudaGetLastError());
    }
    if (refactor) {
        if (cfg.pc == PC_BLOCK) {
            // every member's blocks from its scalar coefficients, sentinels
            // in its factor, then one factor launch over the batch
            int bs = 0;
            for (size_t s = 0; s < meshes.size(); ++s) {
                Mesh& m = *meshes[s];
                const BlockHost& B = *m.blocks;
                if (bs && B.bs != bs) throw Error(MRG_E_INVALID, "block preconditioner: members' block sizes differ");
                bs = B.bs;
                BlockView& v = block_view(m, *bh.members[s]);
                launch_block_gather(v.d, B.n, B.nf, B.bs, m.raw_diag, m.raw_upper, m.sym ? nullptr : m.raw_lower,
                                    c->st);
                launch_fill_sentinel(v.dD, (long long)B.n * B.bs * B.bs, 0, c->st);
            }
            launch_block_factor(bs, bh.d, grid_sweep(c), c->st);
        } else if (cfg.pc >= PC_DIC) {
            launch_factor(bh.d, grid_sweep(c), want32 ? 1 : 0, c->st);
        } else {
            launch_rows(OP_DIAG_RD, 0, bh.d, nt, ns, 0, c->st);
        }
        MRG_CUDA(cudaGetLastError());
    }
    for (size_t s = 0; s < meshes.size(); ++s) {
        PlanState& P = *bh.members[s];
        P.scattered = meshes[s]->version;
        if (refactor) {
            P.factored = meshes[s]->version;
            P.factored_pc = cfg.pc;
            P.factored32 = want32;
        }
    }
}

PlanState& prepare(Mesh& m, const Controls& cfg)
{
    if (!m.have_coeffs) throw Error(MRG_E_INVALID, "no coefficients uploaded for this mesh");
    PlanState& P = m.plan(cfg.ordering);
    std::vector<Mesh*> ms{&m};
    prepare_batch(P.single, ms, cfg);
    return P;
}

// ------------------------------------------------------------------ graphs
// trans: the sweeps' vector set (0 = r -> w, 1 = the transpose system,
// 2 / 3 = BiCGStab's M^-1 p / M^-1 s).
// The block size of a PC_BLOCK batch (its members share it).
static int block_bs(const BatchHost& bh)
{
    for (const PlanState* P : bh.members)
        if (P->bs_blocks > 0) return P->bs_blocks;
    return 1;
}

// Exact sweeps of a one-system batch by the owner-computes kernel
// (MRG_PART_SWEEPS=0: the ticketed sync-free kernel instead).
static bool part_sweeps()
{
    static int on = -1;
    if (on < 0) {
        const char* e = std::getenv("MRG_PART_SWEEPS");
        on = (e && e[0] == '0') ? 0 : 1;
    }
    return on == 1;
}

// The owner-computes launch shape of a batch's exact sweeps: one system
// with a partitioned plan (not while the watchdog test hook withholds a
// chunk), else parts = 0.
void part_choice(const BatchHost& bh, int& parts, int& cells, bool gs)
{
    const SysDev* S1 = bh.members.size() == 1 ? &bh.members[0]->sys : nullptr;
    parts = (S1 && S1->nparts > 0 && bh.ctx->unpublished1 == 0 && part_sweeps()) ? S1->nparts : 0;
    // DIC / DILU sweeps (no division a row) gain only from few parts with
    // enough rows per level each (measured on GB300: a 262k-cell CHT mesh in
    // 64 parts 1.6x faster than ticketed; 3.1M cells in 152 parts, and a
    // block expansion with 7 rows a part and level, 1.7x and 2.6x slower)
    if (parts && !gs && (parts > kPartMaxTri || (long long)S1->n < (long long)kPartRowsPerLevel * S1->nlevels * parts))
        parts = 0;
    cells = parts ? S1->part_cells : 0;
}

static void record_precondition(BatchHost& bh, const Controls& cfg, int prec, int trans, cudaStream_t st,
                                int rho_chunks = 0)
{
    Ctx* c = bh.ctx;
    if (cfg.pc < PC_DIC) return;
    if (cfg.pc == PC_BLOCK) {
        const int bs = block_bs(bh);
        launch_block_sweep(bs, 1, trans, bh.d, grid_sweep(c), st);
        launch_block_sweep(bs, 0, trans, bh.d, grid_sweep(c), st);
        return;
    }
    if (cfg.ordering == MRG_ORDER_EXACT) {
        // one system with a partitioned plan: the owner-computes kernel
        // (not while the watchdog test hook withholds a chunk)
        int parts = 0, cells = 0;
        part_choice(bh, parts, cells);
        launch_sweep(prec, 1, trans, 1, 0, bh.d, grid_sf(c), st, 0, parts, cells);
        launch_sweep(prec, 0, trans, 1, 0, bh.d, grid_sf(c), st, 0, parts, cells);
    } else {
        // forward levels 1..nl-1, backward levels nl-2..0 (level 0 alone if
        // nl == 1); one chunk per warp of the widest level
        const int nl = bh.h.maxlevels;
        const int div = std::max(1, bh.tune.sweep_div);
        const int g = std::max(1, std::min(persistent_grid(), (bh.widest_level + div - 1) / div));
        for (int L = 1; L < nl; ++L) launch_sweep(prec, 1, trans, 0, L, bh.d, g, st, rho_chunks);
        for (int L = std::max(nl - 2, 0); L >= 0; --L) launch_sweep(prec, 0, trans, 0, L, bh.d, g, st, rho_chunks);
    }
}

static bool any_general_iface(const BatchHost& bh)
{
    for (const PlanState* P : bh.members)
        if (P->sys.ngen) return true;
    return false;
}

// One BiCGStab iteration: p, M^-1 p, v = A M^-1 p (alpha), s and the
// half-step test, M^-1 s, t = A M^-1 s (omega), x and r.  A diagonal or no
// preconditioner is applied inside the p and s updates.
static void record_iteration_bs(BatchHost& bh, const Controls& cfg, int prec, cudaStream_t st)
{
    const int nt = bh.h.ntiles, ns = bh.h.nsegs;
    const bool gen = any_general_iface(bh);
    launch_rows(OP_BS_P, prec, bh.d, nt, ns, 0, st);
    if (cfg.pc >= PC_DIC) record_precondition(bh, cfg, prec, 2, st);
    if (gen) launch_iface_gather(prec, 0, bh.d, 64, st);
    launch_rows(OP_BS_V, prec, bh.d, nt, ns, 0, st);
    launch_rows(OP_BS_S, prec, bh.d, nt, ns, 0, st);
    if (cfg.pc >= PC_DIC) record_precondition(bh, cfg, prec, 3, st);
    if (gen) launch_iface_gather(prec, 2, bh.d, 64, st);
    launch_rows(OP_BS_T, prec, bh.d, nt, ns, 0, st);
    launch_rows(OP_BS_XR, prec, bh.d, nt, ns, 0, st);
}

// One smoothSolver iteration: nSweeps smoother sweeps, then the residual
// and the convergence test.  A Gauss-Seidel sweep: the interfaces'
// sweep-start values, the sweep into y, x = y.  A DIC / DILU sweep: r = b -
// A x, w = M^-1 r (the preconditioner's sweeps), x += w.
static void record_iteration_gs(BatchHost& bh, const Controls& cfg, cudaStream_t st)
{
    const int nt = bh.h.ntiles, ns = bh.h.nsegs;
    const bool gen = any_general_iface(bh);
    const bool fact = cfg.smoother != MRG_SMOOTHER_GAUSS_SEIDEL;
    const bool gs = cfg.smoother == MRG_SMOOTHER_GAUSS_SEIDEL || cfg.smoother == MRG_SMOOTHER_DIC_GAUSS_SEIDEL ||
                    cfg.smoother == MRG_SMOOTHER_DILU_GAUSS_SEIDEL;
    for (int k = 0; k < std::max(1, cfg.n_sweeps); ++k) {
        if (fact) {
            if (gen) launch_iface_gather(0, 1, bh.d, 64, st);
            launch_rows(OP_SM_RES, 0, bh.d, nt, ns, 0, st);
            record_precondition(bh, cfg, 0, 0, st);
            launch_rows(OP_SM_ADD, 0, bh.d, nt, ns, 0, st);
        }
        if (gs) {
            if (gen) launch_iface_gather(0, 1, bh.d, 64, st);
            int parts = 0, cells = 0;
            part_choice(bh, parts, cells, true);
            launch_gs_sweep(bh.d, grid_sweep(bh.ctx), st, parts, cells);
            launch_rows(OP_GS_COPY, 0, bh.d, nt, ns, 0, st);
        }
    }
    if (gen) launch_iface_gather(0, 1, bh.d, 64, st);
    launch_rows(OP_GS_RES, 0, bh.d, nt, ns, 0, st);
}

static void record_iteration(BatchHost& bh, const Controls& cfg, int prec, cudaStream_t st)
{
    if (cfg.solver == MRG_SOLVER_BICGSTAB) {
        record_iteration_bs(bh, cfg, prec, st);
        return;
    }
    if (cfg.solver == MRG_SOLVER_SMOOTH) {
        record_iteration_gs(bh, cfg, st);
        return;
    }
    const int pb = cfg.solver == MRG_SOLVER_PBICG;
    const int nt = bh.h.ntiles, ns = bh.h.nsegs;
    // FP32 PCG with a levelled DIC: the sweeps leave (r, w) per chunk and rho
    // sums those (the FP64 loop keeps the row-wise OP_RHO the oracle mirrors)
    const int rc = prec == 1 && !pb && cfg.pc >= PC_DIC && cfg.ordering != MRG_ORDER_EXACT;
    if (cfg.pc >= PC_DIC) {
        record_precondition(bh, cfg, prec, 0, st, rc);
        if (pb) record_precondition(bh, cfg, prec, 1, st);
    } else if (cfg.pc == PC_DIAG) {
        launch_rows(OP_PRECOND_DIAG, prec, bh.d, nt, ns, pb, st);
    } else {
        launch_rows(OP_PRECOND_NONE, prec, bh.d, nt, ns, pb, st);
    }
    launch_rows(rc ? OP_RHO_CH : OP_RHO, prec, bh.d, nt, ns, pb, st);
    launch_rows(OP_PUPDATE, prec, bh.d, nt, ns, pb, st);
    if (any_general_iface(bh)) {
        launch_iface_gather(prec, 0, bh.d, 64, st);
        if (pb) launch_iface_gather(prec, 2, bh.d, 64, st);
    }
    launch_rows(OP_SPMV_QP, prec, bh.d, nt, ns, pb, st, bh.tune.spmv);
    launch_rows(OP_UPDATE, prec, bh.d, nt, ns, pb, st);
}

// How K iterations are launched: K copies of the separate launches of
// record_iteration captured in one graph (the default: measured faster on
// GB300, a kernel boundary inside a graph costs about what a grid barrier
// does), or one persistent cooperative kernel whose phases are those
// launches (MRG_ITERATION=persistent; PCG and PBiCG).  Both give the same bits.
static bool persistent_iteration(const BatchHost& bh, const Controls& cfg)
{
    if (cfg.solver == MRG_SOLVER_BICGSTAB || cfg.solver == MRG_SOLVER_SMOOTH || cfg.pc == PC_BLOCK) return false;
    static int env = -1;
    if (env < 0) {
        const char* e = std::getenv("MRG_ITERATION");
        env = (e && std::string(e) == "persistent") ? 1 : 0;
    }
    return env == 1 || bh.tune.mode == 1;
}

static int iters_per_launch(const BatchHost& bh, const Controls& cfg)
{
    return std::max(1, bh.tune.k > 0 ? bh.tune.k : cfg.k_launch);
}

static void record_persistent(BatchHost& bh, const Controls& cfg, int prec, int k, cudaStream_t st)
{
    const int pb = cfg.solver == MRG_SOLVER_PBICG;
    const int sf = cfg.ordering == MRG_ORDER_EXACT && cfg.pc >= PC_DIC;
    MRG_CUDA(launch_iterate(prec, pb, sf, bh.d, k, cfg.pc, any_general_iface(bh) ? 1 : 0, st));
}

// The captured graph of K iterations.  A persistent launch that the driver
// refuses to capture is launched directly instead (exec stays null).
static BatchHost::Graph iteration_graph(BatchHost& bh, const Controls& cfg, int prec, int k)
{
    const bool pers = persistent_iteration(bh, cfg);
    const int cap = persistent_grid();
    const int g_rows = std::min(std::max(bh.h.ntiles, 1), cap), g_red = std::min(std::max(bh.h.nsegs, 1), cap);
    const int div = std::max(1, bh.tune.sweep_div);
    const int g_sweep = std::max(1, std::min(cap, (bh.widest_level + div - 1) / div));
    std::string key = std::to_string(cfg.solver) + "/" + std::to_string(cfg.pc) + "/" +
                      std::to_string(cfg.ordering) + "/" + std::to_string(prec) + "/" + std::to_string(k) + "/" +
                      std::to_string(g_rows) + "/" + std::to_string(g_red) + "/" + std::to_string(g_sweep) + "/" +
                      std::to_string(bh.h.maxlevels) + "/" + std::to_string(any_general_iface(bh) ? 1 : 0) + "/" +
                      std::to_string(cfg.smoother) + "/" + std::to_string(cfg.n_sweeps) + "/s" +
                      std::to_string(bh.tune.spmv) + (pers ? "/p" : "/l") + (bh.ctx->unpublished1 ? "/u" : "");
    {
        // the owner-computes launch shape is fixed at capture: it depends on
        // the member (a one-system batch), so it is part of the key
        int parts = 0, cells = 0, gparts = 0, gcells = 0;
        part_choice(bh, parts, cells);
        part_choice(bh, gparts, gcells, true);
        key += "/q" + std::to_string(parts) + "x" + std::to_string(cells) + "/g" + std::to_string(gparts);
    }
    auto it = bh.graphs.find(key);
    if (it != bh.graphs.end()) return it->second;
    cudaStream_t st = bh.ctx->st;
    cudaGraph_t g = nullptr;
    const unsigned long long before = launch_count();
    MRG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t rec = cudaSuccess;
    if (pers) {
        const int pb = cfg.solver == MRG_SOLVER_PBICG;
        const int sf = cfg.ordering == MRG_ORDER_EXACT && cfg.pc >= PC_DIC;
        rec = launch_iterate(prec, pb, sf, bh.d, k, cfg.pc, any_general_iface(bh) ? 1 : 0, st);
    } else {
        for (int i = 0; i < k; ++i) record_iteration(bh, cfg, prec, st);
    }
    cudaError_t e = cudaStreamEndCapture(st, &g);
    const long long nodes = (long long)(launch_count() - before);
    add_launches(-nodes);  // captured, not executed
    cudaGraphExec_t ex = nullptr;
    if (rec == cudaSuccess && e == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
    if (g) cudaGraphDestroy(g);
    if (pers && (rec != cudaSuccess || e != cudaSuccess)) {
        cudaGetLastError();   // capture refused: launch directly
        ex = nullptr;
    } else {
        MRG_CUDA(rec);
        MRG_CUDA(e);
    }
    BatchHost::Graph gr{ex, nodes};
    bh.graphs[key] = gr;
    return gr;
}

// One launch of K iterations (graph replay, or the persistent kernel).
static void launch_iterations(BatchHost& bh, const Controls& cfg, int prec, const BatchHost::Graph& gr)
{
    if (gr.exec) {
        MRG_CUDA(cudaGraphLaunch(gr.exec, bh.ctx->st));
        add_launches(gr.nodes);
    } else {
        record_persistent(bh, cfg, prec, iters_per_launch(bh, cfg), bh.ctx->st);
    }
}

static Ctl* pinned_ctl()
{
    static thread_local Ctl* p = nullptr;
    if (!p) MRG_CUDA(cudaMallocHost((void**)&p, sizeof(Ctl)));
    return p;
}

static void poll(BatchHost& bh, Ctl* h)
{
    Ctx* c = bh.ctx;
    MRG_CUDA(cudaMemcpyAsync(h, bh.d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, c->st));
    MRG_CUDA(cudaStreamSynchronize(c->st));
    if (h->err) {
        // clear the error bit and the persistent kernel's barrier counter (a
        // launch that gave up may have left CTAs counted at a barrier)
        unsigned zero[3] = {0, 0, 0};
        MRG_CUDA(cudaMemcpy(&bh.d_ctl->err, zero, sizeof(unsigned), cudaMemcpyHostToDevice));
        MRG_CUDA(cudaMemcpy(&bh.d_ctl->bar_count, zero, sizeof(unsigned), cudaMemcpyHostToDevice));
        throw Error(MRG_E_TIMEOUT, "a device-side wait timed out (sweep dependency or grid barrier)");
    }
}

static void launch_recount_host(BatchHost& bh);

// Replays the iteration graph until no member is in its Krylov loop.  A
// batch of 8 or more members whose active count has fallen to half hands the
// rest to its compacted sub-batch (recursively), so the loop's tail no
// longer walks the finished members' tiles; afterwards the batch's counters
// are recomputed from its members' states.
// MRG_BATCH_PROFILE=1: a batched solve prints, when it ends, its graph
// launches, compactions and the host time spent on compaction (member
// states, the sub-batch's tables) and on iteration graphs (capture or
// lookup) -- time the stream waits on the host.
namespace {
struct BatchProf {
    int on = -1;
    long launches = 0, compactions = 0;
    double compact_ms = 0, graph_ms = 0;
};
thread_local BatchProf g_bprof;   // per host thread: solves on several threads keep their own counts
bool bprof_on()
{
    if (g_bprof.on < 0) {
        const char* e = std::getenv("MRG_BATCH_PROFILE");
        g_bprof.on = e && e[0] == '1';
    }
    return g_bprof.on == 1;
}
double host_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}
}  // namespace

static void run_iterations(BatchHost& bh, const Controls& cfg, int prec, long cap_iters, Ctl* h)
{
    const int k = iters_per_launch(bh, cfg);
    const bool prof = bprof_on();
    double t0 = prof ? host_ms() : 0.0;
    BatchHost::Graph gr = iteration_graph(bh, cfg, prec, k);
    if (prof) g_bprof.graph_ms += host_ms() - t0;
    poll(bh, h);
    long launches = 0;
    const long cap = cap_iters / k + 2;
    const int nmem = (int)bh.members.size();
    while (h->n_active > 0 && launches <= cap) {
        if (nmem >= 8 && 2 * (long)h->n_active <= nmem) {
            if (prof) {
                t0 = host_ms();
                ++g_bprof.compactions;
            }
            std::vector<Scal> sc;
            batch_status(bh, sc);
            std::vector<PlanState*> act;
            for (int s = 0; s < nmem; ++s)
                if (sc[s].active) act.push_back(bh.members[s]);
            if (!bh.compact) {
                bh.compact.reset(new BatchHost());
                bh.compact->init(bh.ctx);
            }
            BatchHost& sub = *bh.compact;
            sub.tune = bh.tune;
            sub.set(act);
            launch_recount_host(sub);
            if (prof) g_bprof.compact_ms += host_ms() - t0;
            run_iterations(sub, cfg, prec, (cap - launches) * k, h);
            launch_recount_host(bh);
            poll(bh, h);
            return;
        }
        launch_iterations(bh, cfg, prec, gr);
        ++launches;
        if (prof) ++g_bprof.launches;
        poll(bh, h);
    }
}

static void write_ctl_controls(BatchHost& bh, const Controls& cfg)
{
    Ctl host{};
    host.tol = cfg.tol;
    host.rel_tol = cfg.rel_tol;
    host.inner_rel_tol = cfg.inner_rel_tol;
    host.min_iter = cfg.min_iter;
    host.max_iter = cfg.max_iter;
    // FP32 BiCG restarts from the FP64 residual every 150 iterations and
    // BiCGStab every 300 unless told otherwise: their short recurrences drift
    // in FP32 (BiCGStab's more slowly: on the 737k-cell GGI convection-
    // diffusion case 150 cost 17 refinement steps and the FP64 continuation,
    // 284 ms, 300 three steps, 123 ms)
    const int auto_inner = cfg.solver == MRG_SOLVER_PBICG      ? std::min(cfg.max_iter, 150)
                           : cfg.solver == MRG_SOLVER_BICGSTAB ? std::min(cfg.max_iter, 300)
                                                               : cfg.max_iter;
    host.inner_max = cfg.inner_max_iter > 0 ? cfg.inner_max_iter : auto_inner;
    host.max_outer = cfg.max_outer;
    host.mixed = cfg.precision == MRG_PRECISION_MIXED ? 1 : 0;
    host.n_sweeps = std::max(1, cfg.n_sweeps);
    host.wait_cycles = bh.ctx->wait_cycles;
    host.unpublished1 = bh.ctx->unpublished1;
    // tickets, error bits and active counts start at zero
    MRG_CUDA(cudaMemcpyAsync(bh.d_ctl, &host, sizeof(Ctl), cudaMemcpyHostToDevice, bh.ctx->st));
}

Perf perf_of(const Scal& q, int precision)
{
    Perf p;
    if (precision == MRG_PRECISION_FP64) {
        p.res0 = q.res0;
        p.res = q.res;
        p.iters = q.iter;
        p.converged = q.converged;
        p.singular = q.singular;
    } else if (q.fallback >= 2) {
        // refinement stalled and the solve finished with FP64 Krylov
        p.res0 = q.ores0;
        p.res = q.res;
        p.iters = q.inner_total + q.iter;
        p.outer = q.oiter;
        p.converged = q.converged;
        p.singular = q.singular;
        p.fallback = 1;
    } else {
        p.res0 = q.ores0;
        p.res = q.ores;
        p.iters = q.inner_total;
        p.outer = q.oiter;
        p.converged = q.oconv;
    }
    if (!std::isfinite(p.res0) || !std::isfinite(p.res)) p.status = MRG_E_BREAKDOWN;
    return p;
}

// Start of a Krylov loop (after the initial residual, the step into FP32 or
// the FP64 restart of a stalled refinement): BiCGStab's shadow residual and
// first rho, for the members that iterate.
static void krylov_start(BatchHost& bh, const Controls& cfg, int prec)
{
    if (cfg.solver == MRG_SOLVER_BICGSTAB)
        launch_rows(OP_BS_RHO0, prec, bh.d, bh.h.ntiles, bh.h.nsegs, 0, bh.ctx->st);
    if (cfg.solver == MRG_SOLVER_SMOOTH)   // the Gauss-Seidel sweep's output starts armed
        launch_rows(OP_GS_ARM, 0, bh.d, bh.h.ntiles, bh.h.nsegs, 0, bh.ctx->st);
}

std::vector<Perf> solve_batch(BatchHost& bh, const Controls& cfg)
{
    Ctx* c = bh.ctx;
    cudaStream_t st = c->st;
    const int pb = cfg.solver == MRG_SOLVER_PBICG;
    const int tsys = cfg.solver == MRG_SOLVER_PBICG || cfg.solver == MRG_SOLVER_BICGSTAB;   // T vectors
    const int nt = bh.h.ntiles, ns = bh.h.nsegs;
    const bool gen = any_general_iface(bh);
    Ctl* h = pinned_ctl();
    cudaEvent_t e0, e1;
    MRG_CUDA(cudaEventCreate(&e0));
    MRG_CUDA(cudaEventCreate(&e1));
    std::vector<Perf> out(bh.members.size());
    try {
        MRG_CUDA(cudaEventRecord(e0, st));
        write_ctl_controls(bh, cfg);
        launch_rows(OP_PERMUTE_IN, 0, bh.d, nt, ns, 0, st);
        launch_rows(OP_BEGIN, 0, bh.d, nt, ns, tsys, st);
        if (gen) launch_iface_gather(0, 1, bh.d, 64, st);
        launch_rows(OP_SUMX, 0, bh.d, nt, ns, 0, st);
        launch_rows(OP_INIT_RES, 0, bh.d, nt, ns, pb, st);
        MRG_CUDA(cudaGetLastError());
        if (cfg.precision == MRG_PRECISION_FP64) {
            krylov_start(bh, cfg, 0);
            run_iterations(bh, cfg, 0, cfg.max_iter + cfg.min_iter, h);
        } else {
            for (int outer = 0; outer <= cfg.max_outer + 1; ++outer) {
                if (gen) launch_iface_gather(0, 1, bh.d, 64, st);
                launch_rows(OP_RESID64, 0, bh.d, nt, ns, 0, st);
                launch_rows(OP_KEEPBEST, 0, bh.d, nt, ns, 0, st);
                poll(bh, h);
                if (h->n_oactive == 0) break;
                launch_rows(OP_TO32, 0, bh.d, nt, ns, tsys, st);
                krylov_start(bh, cfg, 1);
                run_iterations(bh, cfg, 1, cfg.max_iter, h);
                launch_rows(OP_CORRECT, 0, bh.d, nt, ns, 0, st);
            }
            // members whose refinement stalled finish with FP64 Krylov
            const Controls fb = fallback_controls(cfg);
            if (gen) launch_iface_gather(0, 1, bh.d, 64, st);
            launch_rows(OP_FALLBACK64, 0, bh.d, nt, ns, fb.solver == MRG_SOLVER_PBICG, st);
            krylov_start(bh, fb, 0);
            poll(bh, h);
            if (h->n_active > 0) {
                run_iterations(bh, fb, 0, fb.max_iter, h);
                if (gen) launch_iface_gather(0, 1, bh.d, 64, st);
                launch_rows(OP_FALLBACK64, 0, bh.d, nt, ns, 0, st);   // true residual of the result
            }
        }
        launch_rows(OP_PERMUTE_OUT, 0, bh.d, nt, ns, 0, st);
        MRG_CUDA(cudaEventRecord(e1, st));
        MRG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (bprof_on() && bh.members.size() > 1) {
            std::fprintf(stderr, "mrg batch: %zu systems, %.1f ms; %ld graph launches, %ld compactions; host ms: "
                                 "compaction %.1f, graphs %.1f\n",
                         bh.members.size(), ms, g_bprof.launches, g_bprof.compactions, g_bprof.compact_ms,
                         g_bprof.graph_ms);
            g_bprof = BatchProf{1};
        }
        std::vector<Scal> sc(bh.members.size());
        for (size_t s = 0; s < bh.members.size(); ++s)
            MRG_CUDA(cudaMemcpyAsync(&sc[s], bh.members[s]->sys.sc, sizeof(Scal), cudaMemcpyDeviceToHost, st));
        MRG_CUDA(cudaStreamSynchronize(st));
        for (size_t s = 0; s < bh.members.size(); ++s) {
            out[s] = perf_of(sc[s], cfg.precision);
            out[s].ms = ms;
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return out;
}

Perf solve_device(Mesh& m, const double* d_b, double* d_x, const Controls& cfg)
{
    if (cfg.solver == MRG_SOLVER_GAMG) return gamg_solve(m, d_b, d_x, cfg);
    PlanState& P = prepare(m, cfg);
    P.sys.in_b = d_b;
    P.sys.in_x = d_x;
    P.sys.out_x = d_x;
    P.sync_sys();
    P.single.sync_sys();
    return solve_batch(P.single, cfg)[0];
}

// ------------------------------------------------------------------ serving steps
// The steps of solve_batch, one at a time, for a server that changes a
// running batch's membership between iteration launches.  Each step works on
// whichever members the given batch holds; per-system state decides what a
// member does (Krylov-loop ops skip inactive members, refinement ops skip
// members outside the outer loop), so a member sees the same sequence of
// operations, and gets the same bits, as in solve_batch.
void batch_begin(BatchHost& bh, const Controls& cfg)
{
    cudaStream_t st = bh.ctx->st;
    const int pb = cfg.solver == MRG_SOLVER_PBICG;
    const int tsys = cfg.solver == MRG_SOLVER_PBICG || cfg.solver == MRG_SOLVER_BICGSTAB;
    const int nt = bh.h.ntiles, ns = bh.h.nsegs;
    const bool gen = any_general_iface(bh);
    write_ctl_controls(bh, cfg);
    launch_rows(OP_PERMUTE_IN, 0, bh.d, nt, ns, 0, st);
    launch_rows(OP_BEGIN, 0, bh.d, nt, ns, tsys, st);
    if (gen) launch_iface_gather(0, 1, bh.d, 64, st);
    launch_rows(OP_SUMX, 0, bh.d, nt, ns, 0, st);
    launch_rows(OP_INIT_RES, 0, bh.d, nt, ns, pb, st);
    if (cfg.precision == MRG_PRECISION_MIXED) {
        if (gen) launch_iface_gather(0, 1, bh.d, 64, st);
        launch_rows(OP_RESID64, 0, bh.d, nt, ns, 0, st);
        launch_rows(OP_KEEPBEST, 0, bh.d, nt, ns, 0, st);
        launch_rows(OP_TO32, 0, bh.d, nt, ns, tsys, st);
        krylov_start(bh, cfg, 1);
    } else {
        krylov_start(bh, cfg, 0);
    }
    MRG_CUDA(cudaGetLastError());
}

Controls fallback_controls(const Controls& cfg)
{
    Controls fb = cfg;
    if (fb.solver == MRG_SOLVER_BICGSTAB) fb.solver = MRG_SOLVER_PBICG;
    return fb;
}

void batch_fallback(BatchHost& bh, const Controls& cfg)
{
    const Controls fb = fallback_controls(cfg);
    if (any_general_iface(bh)) launch_iface_gather(0, 1, bh.d, 64, bh.ctx->st);
    launch_rows(OP_FALLBACK64, 0, bh.d, bh.h.ntiles, bh.h.nsegs, fb.solver == MRG_SOLVER_PBICG, bh.ctx->st);
    krylov_start(bh, fb, 0);
    MRG_CUDA(cudaGetLastError());
}

void batch_iterate(BatchHost& bh, const Controls& cfg, int prec)
{
    if (prec < 0) prec = cfg.precision == MRG_PRECISION_MIXED ? 1 : 0;
    BatchHost::Graph gr = iteration_graph(bh, cfg, prec, iters_per_launch(bh, cfg));
    launch_iterations(bh, cfg, prec, gr);
}

void batch_outer(BatchHost& bh, const Controls& cfg)
{
    cudaStream_t st = bh.ctx->st;
    const int tsys = cfg.solver == MRG_SOLVER_PBICG || cfg.solver == MRG_SOLVER_BICGSTAB;
    const int nt = bh.h.ntiles, ns = bh.h.nsegs;
    launch_rows(OP_CORRECT, 0, bh.d, nt, ns, 0, st);
    if (any_general_iface(bh)) launch_iface_gather(0, 1, bh.d, 64, st);
    launch_rows(OP_RESID64, 0, bh.d, nt, ns, 0, st);
    launch_rows(OP_KEEPBEST, 0, bh.d, nt, ns, 0, st);
    launch_rows(OP_TO32, 0, bh.d, nt, ns, tsys, st);
    krylov_start(bh, cfg, 1);
    MRG_CUDA(cudaGetLastError());
}

void batch_finish(BatchHost& bh)
{
    launch_rows(OP_PERMUTE_OUT, 0, bh.d, bh.h.ntiles, bh.h.nsegs, 0, bh.ctx->st);
    MRG_CUDA(cudaGetLastError());
}

void batch_recount(BatchHost& bh)
{
    launch_recount(bh.d, bh.ctx->st);
    MRG_CUDA(cudaGetLastError());
}

static void launch_recount_host(BatchHost& bh) { batch_recount(bh); }

const Ctl& batch_poll(BatchHost& bh)
{
    Ctl* h = pinned_ctl();
    poll(bh, h);
    return *h;
}

void batch_status(BatchHost& bh, std::vector<Scal>& out)
{
    const int nsys = (int)bh.members.size();
    out.resize(nsys);
    if (nsys == 0) return;
    ensure(bh.ctx, bh.d_scal, bh.cap_scal, (size_t)nsys);
    Ctl* h = pinned_ctl();
    launch_gather_scal(bh.d, bh.d_scal, bh.ctx->st);
    MRG_CUDA(cudaMemcpyAsync(out.data(), bh.d_scal, sizeof(Scal) * nsys, cudaMemcpyDeviceToHost, bh.ctx->st));
    poll(bh, h);
}

// ------------------------------------------------------------------ autotuner
Tuning tune_batch(BatchHost& bh, const Controls& cfg)
{
    Ctx* c = bh.ctx;
    cudaStream_t st = c->st;
    // the loop keeps iterating while being timed: no convergence, no limit
    Controls run = cfg;
    run.tol = 0.0;
    run.rel_tol = 0.0;
    run.min_iter = 0;
    run.max_iter = 1 << 30;
    run.inner_max_iter = 1 << 30;
    run.inner_rel_tol = 1e-30;
    const int prec = cfg.precision == MRG_PRECISION_MIXED ? 1 : 0;
    const bool levels = cfg.ordering == MRG_ORDER_COLOUR && cfg.pc >= PC_DIC;
    std::vector<Tuning> cands;
    for (int mode : {0, 1})
        for (int k : {4, 16})
            for (int div : {4, 8, 16}) {
                if (!levels && div != 8) continue;
                if (mode == 1 && (cfg.solver == MRG_SOLVER_BICGSTAB || cfg.solver == MRG_SOLVER_SMOOTH))
                    continue;   // no persistent form
                Tuning t;
                t.mode = mode;
                t.k = k;
                t.sweep_div = div;
                cands.push_back(t);
            }
    const Tuning saved = bh.tune;
    Ctl* h = pinned_ctl();
    cudaEvent_t e0, e1;
    MRG_CUDA(cudaEventCreate(&e0));
    MRG_CUDA(cudaEventCreate(&e1));
    Tuning best;
    best.us_per_iter = 1e300;
    try {
        for (Tuning t : cands) {
            bh.tune = t;
            bh.tune.tuned = 1;
            batch_begin(bh, run);
            BatchHost::Graph gr = iteration_graph(bh, run, prec, t.k);
            launch_iterations(bh, run, prec, gr);   // warm-up (and capture)
            poll(bh, h);
            if (h->n_active == 0) continue;
            const int reps = std::max(2, 64 / t.k);
            MRG_CUDA(cudaEventRecord(e0, st));
            for (int r = 0; r < reps; ++r) {
                launch_iterations(bh, run, prec, gr);
                poll(bh, h);   // the host loop polls after every launch
            }
            MRG_CUDA(cudaEventRecord(e1, st));
            MRG_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            MRG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            t.us_per_iter = 1e3 * ms / (reps * t.k);
            if (t.us_per_iter < best.us_per_iter) best = t;
        }
    } catch (...) {
        bh.tune = saved;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    if (best.us_per_iter >= 1e300) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        bh.tune = saved;
        return saved;
    }
    int ncand = (int)cands.size();
    // then the Amul kernel -- block shape (256 row threads, or a producer warp
    // beside them) and rows a warp takes per step -- for the PCG loop of the
    // graph mode, the others kept
    if (best.mode == 0 && cfg.solver == MRG_SOLVER_PCG) {
        try {
            for (int v : {1, 2, 3}) {
                if (prec == 0 && v == 3) continue;   // two rounds per step: FP32 only
                Tuning t = best;
                t.spmv = v;
                bh.tune = t;
                bh.tune.tuned = 1;
                batch_begin(bh, run);
                BatchHost::Graph gr = iteration_graph(bh, run, prec, t.k);
                launch_iterations(bh, run, prec, gr);
                poll(bh, h);
                if (h->n_active == 0) continue;
                const int reps = std::max(2, 64 / t.k);
                MRG_CUDA(cudaEventRecord(e0, st));
                for (int r = 0; r < reps; ++r) {
                    launch_iterations(bh, run, prec, gr);
                    poll(bh, h);
                }
                MRG_CUDA(cudaEventRecord(e1, st));
                MRG_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                MRG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                t.us_per_iter = 1e3 * ms / (reps * t.k);
                ++ncand;
                if (t.us_per_iter < best.us_per_iter) best = t;
            }
        } catch (...) {
            bh.tune = saved;
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    best.tuned = 1;
    best.candidates = ncand;
    bh.tune = best;
    return best;
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
    if (S.ngen) launch_iface_gather(0, 3, P.single.d, 64, c->st);
    launch_rows(transpose ? OP_TMUL : OP_AMUL, 0, P.single.d, P.ntiles, P.single.h.nsegs, 0, c->st);
    launch_permute(0, P.d_sys, 0, S.v64.q, d_y, S.n, c->st);
    MRG_CUDA(cudaGetLastError());
    MRG_CUDA(cudaStreamSynchronize(c->st));
}

void residual_device(Mesh& m, const double* d_b, const double* d_x, double* res, double* nfac)
{
    Controls cfg;
    cfg.pc = PC_NONE;
    cfg.tol = 0.0;
    cfg.max_iter = 0;
    PlanState& P = prepare(m, cfg);
    Ctx* c = m.ctx;
    P.sys.in_b = d_b;
    P.sys.in_x = d_x;
    P.sys.out_x = nullptr;
    P.sync_sys();
    P.single.sync_sys();
    BatchHost& bh = P.single;
    write_ctl_controls(bh, cfg);
    launch_rows(OP_PERMUTE_IN, 0, bh.d, P.ntiles, P.single.h.nsegs, 0, c->st);
    launch_rows(OP_BEGIN, 0, bh.d, P.ntiles, P.single.h.nsegs, 0, c->st);
    if (P.sys.ngen) launch_iface_gather(0, 1, bh.d, 64, c->st);
    launch_rows(OP_SUMX, 0, bh.d, P.ntiles, P.single.h.nsegs, 0, c->st);
    launch_rows(OP_INIT_RES, 0, bh.d, P.ntiles, P.single.h.nsegs, 0, c->st);
    Scal sc;
    MRG_CUDA(cudaMemcpyAsync(&sc, P.sys.sc, sizeof(Scal), cudaMemcpyDeviceToHost, c->st));
    MRG_CUDA(cudaStreamSynchronize(c->st));
    if (res) *res = sc.res0;
    if (nfac) *nfac = sc.nfac;
}

static void set_active_flag(PlanState& P, int on)
{
    MRG_CUDA(cudaMemcpyAsync((char*)P.sys.sc + offsetof(Scal, active), &on, sizeof on, cudaMemcpyHostToDevice,
                             P.ctx->st));
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
    set_active_flag(P, 1);
    if (pc >= PC_DIC) {
        if (ordering == MRG_ORDER_EXACT) launch_fill_sentinel(transpose ? S.v64.yT : S.v64.y, S.n, 0, c->st);
        record_precondition(P.single, cfg, 0, transpose, c->st);
    } else {
        launch_rows(pc == PC_DIAG ? OP_PRECOND_DIAG : OP_PRECOND_NONE, 0, P.single.d, P.ntiles, P.single.h.nsegs, transpose, c->st);
    }
    launch_permute(0, P.d_sys, 0, transpose ? S.v64.wT : S.v64.w, d_w, S.n, c->st);
    set_active_flag(P, 0);
    MRG_CUDA(cudaGetLastError());
    poll(P.single, pinned_ctl());
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
    poll(P.single, pinned_ctl());
}

float time_kernel(Mesh& m, const Controls& cfg, int kernel, int reps)
{
    if (reps < 1) throw Error(MRG_E_INVALID, "reps must be >= 1");
    if (kernel < 0 || kernel > 1) throw Error(MRG_E_INVALID, "unknown kernel id");
    PlanState& P = prepare(m, cfg);
    Ctx* c = m.ctx;
    const int prec = cfg.precision;
    const int pb = cfg.solver == MRG_SOLVER_PBICG;
    set_active_flag(P, 1);
    if (kernel == 1 && cfg.pc >= PC_DIC && cfg.ordering == MRG_ORDER_EXACT) {
        const SysDev& S = P.sys;
        if (prec == 0)
            launch_fill_sentinel(S.v64.y, S.n, 0, c->st);
        else
            launch_fill_sentinel(S.v32.y, S.n, 1, c->st);
    }
    auto once = [&] {
        if (kernel == 0)
            launch_rows(OP_SPMV_QP, prec, P.single.d, P.ntiles, P.single.h.nsegs, pb, c->st);
        else
            record_precondition(P.single, cfg, prec, 0, c->st);
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
    set_active_flag(P, 0);
    MRG_CUDA(cudaStreamSynchronize(c->st));
    MRG_CUDA(cudaGetLastError());
    return ms / reps;
}

}  // namespace mrg
