// gamg.cu -- GAMG solver (foam-order Gauss-Seidel smoothing) on the device.
//
// foam-extend's GAMG (the tutorials' fluid p / T solver: GAMG, smoother
// GaussSeidel, nCellsInCoarsestLevel 10, mergeLevels 1, cacheAgglomeration
// true) restated as the standard algebraic multigrid it names:
//   agglomeration  pairwise on face weights |upper| + |lower|, cells in
//                  order: an unpaired cell pairs with its unpaired neighbour
//                  of largest weight (first such face on ties), a cell
//                  without one joins its strongest neighbour's group (or
//                  stays alone); coarse cells numbered as created; levels
//                  are added while a level has more than nCellsInCoarsest
//                  Level cells and pairing still reduces it.  Built once on
//                  the host from the first matrix (cacheAgglomeration).
//   coarse matrix  diag = members' diagonals (ascending), then upper + lower
//                  of the faces inside the coarse cell (ascending); a coarse
//                  face sums its fine faces in face order, swapping upper and
//                  lower for a fine face whose owner lies in the coarse
//                  neighbour.  Restricted on the device at every solve.
//   V-cycle        zero coarse corrections: the finest residual restricted
//                  level by level (sums over members); the coarsest solved
//                  directly (dense LU without pivoting, factorised once per
//                  solve by one CTA, rows in parallel, each entry's updates
//                  in the serial order); going up, each level's correction
//                  is the prolonged coarser one smoothed by nPostSweeps foam
//                  Gauss-Seidel sweeps; the finest x gains the prolonged
//                  correction and nFinestSweeps sweeps; then the residual and
//                  foam's convergence test (iterations count V-cycles).
// The smoothed levels are meshes of their own with foam-order (level) plans,
// so their sweeps are k_gs_sweep's.  Results are those of a sequential
// evaluation in this order (the oracle restates it in numpy).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "../../include/mrgpu.h"
#include "gamg.h"
#include "kernels.h"

namespace mrg {
namespace {

constexpr int kMaxTop = 64;   // cells of the directly solved coarsest level

// ---------------------------------------------------------------- host setup
struct HostLevel {
    int n = 0;
    std::vector<int32_t> lower, upper;
    std::vector<double> diag, up, lo;     // lo empty: symmetric
};

// Pairwise agglomeration of one level: agg (fine -> coarse) and the count.
int agglomerate(const HostLevel& L, std::vector<int32_t>& agg)
{
    const int n = L.n, nf = (int)L.lower.size();
    std::vector<double> w(nf);
    for (int f = 0; f < nf; ++f) w[f] = std::fabs(L.up[f]) + std::fabs(L.lo.empty() ? L.up[f] : L.lo[f]);
    std::vector<int32_t> start(n + 1, 0), adj(2 * (size_t)nf);
    for (int f = 0; f < nf; ++f) {
        start[L.lower[f] + 1]++;
        start[L.upper[f] + 1]++;
    }
    for (int c = 0; c < n; ++c) start[c + 1] += start[c];
    std::vector<int32_t> fill(start.begin(), start.end() - 1);
    for (int f = 0; f < nf; ++f) {   // every cell's faces ascending
        adj[fill[L.lower[f]]++] = f;
        adj[fill[L.upper[f]]++] = f;
    }
    agg.assign(n, -1);
    int nc = 0;
    for (int c = 0; c < n; ++c) {
        if (agg[c] >= 0) continue;
        int best = -1;
        double bw = -std::numeric_limits<double>::infinity();
        for (int q = start[c]; q < start[c + 1]; ++q) {
            const int f = adj[q], o = L.lower[f] == c ? L.upper[f] : L.lower[f];
            if (agg[o] < 0 && w[f] > bw) {
                best = o;
                bw = w[f];
            }
        }
        if (best >= 0) {
            agg[c] = agg[best] = nc++;
            continue;
        }
        bw = -std::numeric_limits<double>::infinity();
        for (int q = start[c]; q < start[c + 1]; ++q) {
            const int f = adj[q], o = L.lower[f] == c ? L.upper[f] : L.lower[f];
            if (w[f] > bw) {
                best = o;
                bw = w[f];
            }
        }
        agg[c] = best >= 0 ? agg[best] : nc++;
    }
    return nc;
}

template <typename T>
T* upload(Ctx* c, const std::vector<T>& v)
{
    T* d = (T*)c->alloc(std::max<size_t>(sizeof(T) * v.size(), 16));
    if (!v.empty()) MRG_CUDA(cudaMemcpyAsync(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c->st));
    return d;
}

std::vector<int32_t> download_perm(Ctx* c, const PlanState& P, int n)
{
    std::vector<int32_t> perm(n);
    if (n) MRG_CUDA(cudaMemcpy(perm.data(), P.perm, 4 * (size_t)n, cudaMemcpyDeviceToHost));
    return perm;
}

// ---------------------------------------------------------------- kernels
__global__ void k_gamg_coeffs(int nc, int nfc, const int32_t* __restrict__ mem_ptr, const int32_t* __restrict__ mem_idx,
                              const int32_t* __restrict__ int_ptr, const int32_t* __restrict__ int_idx,
                              const int32_t* __restrict__ fc_ptr, const int32_t* __restrict__ fc_idx,
                              const int32_t* __restrict__ fc_flip, const double* __restrict__ fdiag,
                              const double* __restrict__ fup, const double* __restrict__ flo, double* __restrict__ diag,
                              double* __restrict__ up, double* __restrict__ lo)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nc + nfc; t += gridDim.x * blockDim.x) {
        if (t < nc) {
            double acc = 0.0;
            for (int k = mem_ptr[t]; k < mem_ptr[t + 1]; ++k) acc = __dadd_rn(acc, fdiag[mem_idx[k]]);
            for (int k = int_ptr[t]; k < int_ptr[t + 1]; ++k) {
                const int f = int_idx[k];
                acc = __dadd_rn(acc, fup[f]);
                acc = __dadd_rn(acc, flo[f]);
            }
            diag[t] = acc;
        } else {
            const int F = t - nc;
            double u = 0.0, l = 0.0;
            for (int k = fc_ptr[F]; k < fc_ptr[F + 1]; ++k) {
                const int f = fc_idx[k];
                const bool flip = fc_flip[k] != 0;
                u = __dadd_rn(u, flip ? flo[f] : fup[f]);
                l = __dadd_rn(l, flip ? fup[f] : flo[f]);
            }
            up[F] = u;
            if (lo) lo[F] = l;
        }
    }
}

// dst[R] = sum over src[idx] of the row's finer rows (ascending, from zero)
__global__ void k_gamg_restrict(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                const double* __restrict__ src, double* __restrict__ dst)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int k = ptr[r]; k < ptr[r + 1]; ++k) acc = __dadd_rn(acc, src[idx[k]]);
        dst[r] = acc;
    }
}

// x[i] = c[map[i]] (add = 0) or x[i] + c[map[i]] (add = 1)
__global__ void k_gamg_prolong(int n, const int32_t* __restrict__ map, const double* __restrict__ c, double* x,
                               int add)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = add ? __dadd_rn(x[i], c[map[i]]) : c[map[i]];
}

// Dense LU without pivoting of the coarsest level (m <= kMaxTop), one CTA:
// thread i owns row i; every entry receives its updates in k order.
__global__ void k_gamg_lu(int m, int nf, const int32_t* __restrict__ lower, const int32_t* __restrict__ upper,
                          const double* __restrict__ diag, const double* __restrict__ up,
                          const double* __restrict__ lo, double* __restrict__ LU)
{
    __shared__ double M[kMaxTop * kMaxTop];
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) M[e] = 0.0;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 0; i < m; ++i) M[i * m + i] = diag[i];
        for (int f = 0; f < nf; ++f) {
            M[lower[f] * m + upper[f]] = up[f];
            M[upper[f] * m + lower[f]] = lo ? lo[f] : up[f];
        }
    }
    __syncthreads();
    const int i = threadIdx.x;
    for (int k = 0; k < m; ++k) {
        if (i > k && i < m) {
            const double l = __ddiv_rn(M[i * m + k], M[k * m + k]);
            M[i * m + k] = l;
            for (int j = k + 1; j < m; ++j) M[i * m + j] = __dsub_rn(M[i * m + j], __dmul_rn(l, M[k * m + j]));
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) LU[e] = M[e];
}

// Forward and back substitution with the factors (one thread).
__global__ void k_gamg_dense_solve(int m, const double* __restrict__ LU, const double* __restrict__ b,
                                   double* __restrict__ x)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double y[kMaxTop];
    for (int i = 0; i < m; ++i) {
        double acc = b[i];
        for (int j = 0; j < i; ++j) acc = __dsub_rn(acc, __dmul_rn(LU[i * m + j], y[j]));
        y[i] = acc;
    }
    for (int i = m - 1; i >= 0; --i) {
        double acc = y[i];
        for (int j = i + 1; j < m; ++j) acc = __dsub_rn(acc, __dmul_rn(LU[i * m + j], x[j]));
        x[i] = __ddiv_rn(acc, LU[i * m + i]);
    }
}

__global__ void k_gamg_activate(const SysDev* __restrict__ S)
{
    S->sc->active = 1;
}

int grid_of(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4096)); }

// The controls a smoothed level's plan and views are prepared with.
Controls smooth_controls()
{
    Controls c;
    c.solver = MRG_SOLVER_SMOOTH;
    c.pc = PC_NONE;
    c.precision = MRG_PRECISION_FP64;
    c.ordering = MRG_ORDER_EXACT;
    return c;
}

void build(Mesh& m, const Controls& cfg)
{
    Ctx* c = m.ctx;
    auto g = std::make_unique<Gamg>();
    g->ctx = c;
    g->n_coarsest = cfg.gamg_coarsest;
    g->sym = m.sym;
    HostLevel cur;
    cur.n = m.n;
    cur.lower = m.lower;
    cur.upper = m.upper;
    cur.diag.resize(m.n);
    cur.up.resize(m.nf);
    MRG_CUDA(cudaMemcpy(cur.diag.data(), m.raw_diag, 8 * (size_t)m.n, cudaMemcpyDeviceToHost));
    if (m.nf) MRG_CUDA(cudaMemcpy(cur.up.data(), m.raw_upper, 8 * (size_t)m.nf, cudaMemcpyDeviceToHost));
    if (!m.sym) {
        cur.lo.resize(m.nf);
        if (m.nf) MRG_CUDA(cudaMemcpy(cur.lo.data(), m.raw_lower, 8 * (size_t)m.nf, cudaMemcpyDeviceToHost));
    }
    g->lv.resize(1);
    for (;;) {
        std::vector<int32_t> agg;
        int nc = 0;
        if (g->lv.size() == 1 && cur.n <= g->n_coarsest) {
            // already small: the one coarse level is the matrix itself
            agg.resize(cur.n);
            for (int i = 0; i < cur.n; ++i) agg[i] = i;
            nc = cur.n;
        } else {
            if (cur.n <= g->n_coarsest || g->lv.size() >= 50) break;
            nc = agglomerate(cur, agg);
            if (nc >= cur.n) break;
        }
        GamgLevel L;
        L.n = nc;
        L.agg = agg;
        L.members.assign(nc, {});
        for (int i = 0; i < cur.n; ++i) L.members[agg[i]].push_back(i);
        // coarse faces (sorted owner, neighbour) and the faces inside cells
        std::map<std::pair<int, int>, std::vector<std::pair<int, int>>> faces;
        std::vector<std::vector<int32_t>> inside(nc);
        for (int f = 0; f < (int)cur.lower.size(); ++f) {
            const int a = agg[cur.lower[f]], b = agg[cur.upper[f]];
            if (a == b)
                inside[a].push_back(f);
            else
                faces[{std::min(a, b), std::max(a, b)}].push_back({f, a > b ? 1 : 0});
        }
        HostLevel nxt;
        nxt.n = nc;
        std::vector<int32_t> mem_ptr{0}, mem_idx, int_ptr{0}, int_idx, fc_ptr{0}, fc_idx, fc_flip;
        for (int C = 0; C < nc; ++C) {
            double acc = 0.0;
            for (int i : L.members[C]) {
                acc = acc + cur.diag[i];
                mem_idx.push_back(i);
            }
            for (int f : inside[C]) {
                acc = acc + cur.up[f];
                acc = acc + (cur.lo.empty() ? cur.up[f] : cur.lo[f]);
                int_idx.push_back(f);
            }
            nxt.diag.push_back(acc);
            mem_ptr.push_back((int32_t)mem_idx.size());
            int_ptr.push_back((int32_t)int_idx.size());
        }
        for (auto& kv : faces) {
            nxt.lower.push_back(kv.first.first);
            nxt.upper.push_back(kv.first.second);
            double u = 0.0, l = 0.0;
            for (auto& ff : kv.second) {
                const int f = ff.first;
                const double fu = cur.up[f], fl = cur.lo.empty() ? cur.up[f] : cur.lo[f];
                u = u + (ff.second ? fl : fu);
                l = l + (ff.second ? fu : fl);
                fc_idx.push_back(f);
                fc_flip.push_back(ff.second);
            }
            nxt.up.push_back(u);
            if (!cur.lo.empty()) nxt.lo.push_back(l);
            fc_ptr.push_back((int32_t)fc_idx.size());
        }
        L.nf = (int)nxt.lower.size();
        L.mem_ptr = upload(c, mem_ptr);
        L.mem_idx = upload(c, mem_idx);
        L.int_ptr = upload(c, int_ptr);
        L.int_idx = upload(c, int_idx);
        L.fc_ptr = upload(c, fc_ptr);
        L.fc_idx = upload(c, fc_idx);
        L.fc_flip = upload(c, fc_flip);
        L.diag = (double*)c->alloc(8 * (size_t)std::max(nc, 1));
        L.upper = (double*)c->alloc(8 * (size_t)std::max(L.nf, 1));
        if (!m.sym) L.lower = (double*)c->alloc(8 * (size_t)std::max(L.nf, 1));
        L.lo_dev = upload(c, nxt.lower);
        L.up_dev = upload(c, nxt.upper);
        g->lv.push_back(std::move(L));
        const bool was_identity = nc == cur.n && g->lv.size() == 2 && cur.n <= g->n_coarsest;
        cur = std::move(nxt);
        if (was_identity) break;
    }
    if (g->lv.size() < 2) throw Error(MRG_E_INVALID, "GAMG: no coarse level");
    const int top = (int)g->lv.size() - 1;
    if (g->lv[top].n > kMaxTop)
        throw Error(MRG_E_INVALID, "GAMG: coarsening stalled above " + std::to_string(kMaxTop) + " cells");
    g->lv[top].top = true;
    // smoothed levels: meshes of their own
    for (int l = 1; l < top; ++l) {
        GamgLevel& L = g->lv[l];
        L.mesh = std::make_unique<Mesh>();
        L.mesh->ctx = c;
        L.mesh->n = L.n;
        L.mesh->nf = L.nf;
        L.mesh->lower.resize(L.nf);
        L.mesh->upper.resize(L.nf);
        MRG_CUDA(cudaMemcpy(L.mesh->lower.data(), L.lo_dev, 4 * (size_t)L.nf, cudaMemcpyDeviceToHost));
        MRG_CUDA(cudaMemcpy(L.mesh->upper.data(), L.up_dev, 4 * (size_t)L.nf, cudaMemcpyDeviceToHost));
    }
    const int mt = g->lv[top].n;
    g->lu = (double*)c->alloc(8 * (size_t)std::max(mt * mt, 1));
    g->src_top = (double*)c->alloc(8 * (size_t)std::max(mt, 1));
    g->c_top = (double*)c->alloc(8 * (size_t)std::max(mt, 1));
    MRG_CUDA(cudaStreamSynchronize(c->st));
    m.gamg = std::move(g);
}

// Restriction / prolongation maps in the plans' numbering (after the plans
// exist): level l's rows from level l-1's rows.
void build_maps(Mesh& m)
{
    Gamg& g = *m.gamg;
    Ctx* c = g.ctx;
    const int top = (int)g.lv.size() - 1;
    std::vector<int32_t> perm_f = download_perm(c, m.plan(MRG_ORDER_EXACT), m.n);   // level 0
    for (int l = 1; l <= top; ++l) {
        GamgLevel& L = g.lv[l];
        const int nfine = (int)L.agg.size();
        std::vector<int32_t> iperm_f(nfine);
        for (int i = 0; i < nfine; ++i) iperm_f[perm_f[i]] = i;
        std::vector<int32_t> perm_c(L.n), iperm_c(L.n);
        if (L.top) {
            for (int i = 0; i < L.n; ++i) perm_c[i] = iperm_c[i] = i;
        } else {
            perm_c = download_perm(c, L.mesh->plan(MRG_ORDER_EXACT), L.n);
            for (int i = 0; i < L.n; ++i) iperm_c[perm_c[i]] = i;
        }
        std::vector<int32_t> r_ptr{0}, r_idx, p_map(nfine);
        for (int R = 0; R < L.n; ++R) {
            for (int f : L.members[perm_c[R]]) r_idx.push_back(iperm_f[f]);
            r_ptr.push_back((int32_t)r_idx.size());
        }
        for (int i = 0; i < nfine; ++i) p_map[i] = iperm_c[L.agg[perm_f[i]]];
        L.r_ptr = upload(c, r_ptr);
        L.r_idx = upload(c, r_idx);
        L.p_map = upload(c, p_map);
        L.maps = true;
        perm_f = perm_c;
    }
    MRG_CUDA(cudaStreamSynchronize(c->st));
}

}  // namespace

Gamg::~Gamg()
{
    if (!ctx) return;
    for (GamgLevel& L : lv)
        for (void* p : {(void*)L.mem_ptr, (void*)L.mem_idx, (void*)L.int_ptr, (void*)L.int_idx, (void*)L.fc_ptr,
                        (void*)L.fc_idx, (void*)L.fc_flip, (void*)L.diag, (void*)L.upper, (void*)L.lower,
                        (void*)L.r_ptr, (void*)L.r_idx, (void*)L.p_map, (void*)L.lo_dev, (void*)L.up_dev})
            ctx->release(p);
    for (void* p : {(void*)lu, (void*)src_top, (void*)c_top}) ctx->release(p);
}

Perf gamg_solve(Mesh& m, const double* d_b, double* d_x, const Controls& cfg)
{
    if (m.ni > 0) throw Error(MRG_E_INVALID, "GAMG: meshes with interfaces are not supported (use the global form)");
    if (!m.have_coeffs) throw Error(MRG_E_INVALID, "no coefficients uploaded for this mesh");
    if (!m.gamg || m.gamg->n_coarsest != cfg.gamg_coarsest || m.gamg->sym != m.sym) {
        m.gamg.reset();
        build(m, cfg);
    }
    Gamg& g = *m.gamg;
    Ctx* c = m.ctx;
    cudaStream_t st = c->st;
    const int top = (int)g.lv.size() - 1;
    const Controls sc = smooth_controls();
    // coarse coefficients, level by level
    for (int l = 1; l <= top; ++l) {
        GamgLevel& L = g.lv[l];
        const double *fd, *fu, *fl;
        if (l == 1) {
            fd = m.raw_diag;
            fu = m.raw_upper;
            fl = m.sym ? m.raw_upper : m.raw_lower;
        } else {
            const GamgLevel& F = g.lv[l - 1];
            fd = F.diag;
            fu = F.upper;
            fl = m.sym ? F.upper : F.lower;
        }
        k_gamg_coeffs<<<grid_of((long long)L.n + L.nf), 256, 0, st>>>(L.n, L.nf, L.mem_ptr, L.mem_idx, L.int_ptr,
                                                                      L.int_idx, L.fc_ptr, L.fc_idx, L.fc_flip, fd,
                                                                      fu, fl, L.diag, L.upper, m.sym ? nullptr : L.lower);
        add_launches(1);
        if (L.mesh) upload_coeffs(*L.mesh, L.diag, L.upper, m.sym ? nullptr : L.lower, nullptr, nullptr,
                                  cudaMemcpyDeviceToDevice, false);
    }
    {
        const GamgLevel& T = g.lv[top];
        k_gamg_lu<<<1, kMaxTop, 0, st>>>(T.n, T.nf, T.lo_dev, T.up_dev, T.diag, T.upper, m.sym ? nullptr : T.lower,
                                         g.lu);
        add_launches(1);
    }
    // plans and views of every smoothed level, then the finest
    std::vector<PlanState*> P(top + 1, nullptr);
    for (int l = 1; l < top; ++l) P[l] = &prepare(*g.lv[l].mesh, sc);
    Controls fc = sc;
    fc.tol = cfg.tol;
    fc.rel_tol = cfg.rel_tol;
    fc.min_iter = cfg.min_iter;
    fc.max_iter = cfg.max_iter;
    fc.n_sweeps = 1;   // an iteration is one V-cycle
    PlanState& P0 = prepare(m, fc);
    P[0] = &P0;
    if (!g.lv[1].maps) build_maps(m);
    P0.sys.in_b = d_b;
    P0.sys.in_x = d_x;
    P0.sys.out_x = d_x;
    P0.sync_sys();
    P0.single.sync_sys();
    cudaEvent_t e0, e1;
    MRG_CUDA(cudaEventCreate(&e0));
    MRG_CUDA(cudaEventCreate(&e1));
    Perf out;
    try {
        MRG_CUDA(cudaEventRecord(e0, st));
        batch_begin(P0.single, fc);   // permute in, initial residual, arm the sweep output
        for (int l = 1; l < top; ++l) {
            k_gamg_activate<<<1, 1, 0, st>>>(P[l]->d_sys);
            launch_rows(OP_GS_ARM, 0, P[l]->single.d, P[l]->ntiles, P[l]->single.h.nsegs, 0, st);
            add_launches(1);
        }
        auto vec = [&](int l, int which) -> double* {   // 0: source b, 1: correction x
            if (l == top) return which == 0 ? g.src_top : g.c_top;
            return which == 0 ? P[l]->sys.v64.b : P[l]->sys.v64.x;
        };
        auto sweeps = [&](int l, int k) {
            BatchHost& bh = P[l]->single;
            for (int s = 0; s < k; ++s) {
                launch_gs_sweep(bh.d, c->nsm * 4, st);
                launch_rows(OP_GS_COPY, 0, bh.d, P[l]->ntiles, bh.h.nsegs, 0, st);
            }
        };
        long cycles = 0;
        const long cap = (long)cfg.max_iter + cfg.min_iter + 2;
        while (batch_poll(P0.single).n_active > 0 && cycles <= cap) {
            // down: restrict the finest residual, then each source
            for (int l = 1; l <= top; ++l) {
                const GamgLevel& L = g.lv[l];
                const double* src = l == 1 ? P0.sys.v64.r : vec(l - 1, 0);
                k_gamg_restrict<<<grid_of(L.n), 256, 0, st>>>(L.n, L.r_ptr, L.r_idx, src, vec(l, 0));
            }
            k_gamg_dense_solve<<<1, 32, 0, st>>>(g.lv[top].n, g.lu, g.src_top, g.c_top);
            add_launches(top + 1);
            // up: prolong and smooth the corrections
            for (int l = top - 1; l >= 1; --l) {
                k_gamg_prolong<<<grid_of(g.lv[l].n), 256, 0, st>>>(g.lv[l].n, g.lv[l + 1].p_map, vec(l + 1, 1),
                                                                   vec(l, 1), 0);
                add_launches(1);
                sweeps(l, cfg.gamg_post);
            }
            k_gamg_prolong<<<grid_of(m.n), 256, 0, st>>>(m.n, g.lv[1].p_map, vec(1, 1), P0.sys.v64.x, 1);
            add_launches(1);
            sweeps(0, cfg.gamg_finest);
            launch_rows(OP_GS_RES, 0, P0.single.d, P0.ntiles, P0.single.h.nsegs, 0, st);
            MRG_CUDA(cudaGetLastError());
            ++cycles;
        }
        // a wait that gave up on a coarse level shows in that level's block
        for (int l = 1; l < top; ++l) batch_poll(P[l]->single);
        batch_finish(P0.single);
        MRG_CUDA(cudaEventRecord(e1, st));
        MRG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        Scal s;
        MRG_CUDA(cudaMemcpy(&s, P0.sys.sc, sizeof(Scal), cudaMemcpyDeviceToHost));
        out = perf_of(s, MRG_PRECISION_FP64);
        out.ms = ms;
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return out;
}

}  // namespace mrg
