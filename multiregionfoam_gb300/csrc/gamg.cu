// gamg.cu -- GAMG solver (foam-order Gauss-Seidel smoothing) on the device.
//
// foam-extend's GAMG (the tutorials' fluid p / T solver: GAMG, smoother
// GaussSeidel, agglomerator faceAreaPair, nCellsInCoarsestLevel 10,
// mergeLevels 1, cacheAgglomeration true, scaleCorrection true,
// directSolveCoarsest false) restated from the published algorithm of foam's
// GAMG family:
//   face weights   faceAreaPair: |cmptMultiply(Sf / sqrt(|Sf|), (1, 1.01,
//                  1.02))| of the finest faces (mrg_mesh_set_face_areas);
//                  algebraicPair: |upper| of the finest matrix.  A coarser
//                  level's weights are its fine faces' weights summed.
//   pairing        (pairGAMGAgglomeration) cells in order; a cell's faces
//                  are those where it is the upper cell, then those where
//                  it is the lower one, each in face order; an ungrouped
//                  cell pairs with the ungrouped neighbour across its face
//                  of largest weight (strictly larger wins), otherwise joins
//                  the group across its face of largest weight; cells left
//                  alone become groups after the pass; the numbering is
//                  then reversed.  A level is kept while it has at least
//                  nCellsInCoarsestLevel cells.  Built once on the host
//                  (cacheAgglomeration).
//   coarse faces   (agglomerateLduAddressing) a face per (owner, neighbour)
//                  pair of groups, numbered by owner and then in order of
//                  first appearance in the fine face order.
//   coarse matrix  diag = the members' diagonals (fine cell order), then
//                  + (upper + lower) of each interior fine face (fine face
//                  order); a coarse face sums its fine faces in face order,
//                  upper and lower swapped for a fine face whose lower cell
//                  lies in the coarse upper cell.  Restricted on the device
//                  at every solve.
//   V-cycle        the finest residual restricted level by level (sums over
//                  members); the coarsest solved directly (dense LU without
//                  pivoting, factorised once per solve by one CTA, rows in
//                  parallel, each entry's updates in the serial order; foam's
//                  directSolveCoarsest false would iterate to the solver's
//                  tolerance instead); going up, each level's correction is
//                  the prolonged coarser one, scaled (scaleCorrection: on
//                  every level except the one below the coarsest) and
//                  smoothed by min(nPostSweeps + postSweepsLevelMultiplier
//                  * l, maxPostSweeps) foam Gauss-Seidel sweeps (l = 0 the
//                  first coarse level); the finest correction is prolonged,
//                  scaled and added to x, then nFinestSweeps sweeps; then the
//                  residual and foam's convergence test (iterations count
//                  V-cycles).
//   scale          (GAMGSolver::scale) Af = A f, sf = (s, f) / stabilise((Af,
//                  f), VSMALL), f = sf f + (s - sf Af) / diag.
// The smoothed levels are meshes of their own with foam-order (level) plans,
// so their sweeps are the smoothSolver's (k_gs_part / k_gs_sweep).  V-cycles run as captured CUDA graphs
// (two per launch); every kernel of a cycle checks that the finest level is
// still iterating, so a cycle after convergence changes nothing.  Results
// are those of a sequential evaluation in this order (the oracle restates it
// in numpy).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <string>
#include <vector>

#include "../../include/mrgpu.h"
#include "gamg.h"
#include "kernels.h"

namespace mrg {

std::vector<double> face_area_weights(const double* sf, int nf)
{
    std::vector<double> w(nf);
    for (int f = 0; f < nf; ++f) {
        const double x = sf[3 * (size_t)f], y = sf[3 * (size_t)f + 1], z = sf[3 * (size_t)f + 2];
        const double mag = std::sqrt(x * x + y * y + z * z);
        const double root = std::sqrt(mag);
        const double a = (x / root) * 1.0, b = (y / root) * 1.01, c = (z / root) * 1.02;
        w[f] = std::sqrt(a * a + b * b + c * c);
    }
    return w;
}

namespace {

constexpr int kMaxTop = 160;       // cells of the directly solved coarsest level
constexpr double kGreat = 1.0e15;  // foam's GREAT

// ---------------------------------------------------------------- host setup
struct HostLevel {
    int n = 0;
    std::vector<int32_t> lower, upper;
    std::vector<double> w;          // agglomeration weights of the faces
};

// foam's pairwise agglomeration of one level: agg (fine -> coarse), count.
int agglomerate(const HostLevel& L, std::vector<int32_t>& agg)
{
    const int n = L.n, nf = (int)L.lower.size();
    std::vector<int32_t> start(n + 1, 0), faces(2 * (size_t)nf);
    for (int f = 0; f < nf; ++f) {
        start[L.upper[f] + 1]++;
        start[L.lower[f] + 1]++;
    }
    for (int c = 0; c < n; ++c) start[c + 1] += start[c];
    std::vector<int32_t> fill(start.begin(), start.end() - 1);
    for (int f = 0; f < nf; ++f) faces[fill[L.upper[f]]++] = f;   // faces where the cell is upper first
    for (int f = 0; f < nf; ++f) faces[fill[L.lower[f]]++] = f;   // then those where it is lower
    agg.assign(n, -1);
    int nc = 0;
    for (int c = 0; c < n; ++c) {
        if (agg[c] >= 0) continue;
        int match = -1;
        double mw = -kGreat;
        for (int q = start[c]; q < start[c + 1]; ++q) {
            const int f = faces[q];
            if (agg[L.upper[f]] < 0 && agg[L.lower[f]] < 0 && L.w[f] > mw) {
                match = f;
                mw = L.w[f];
            }
        }
        if (match >= 0) {
            agg[L.upper[match]] = nc;
            agg[L.lower[match]] = nc;
            ++nc;
            continue;
        }
        mw = -kGreat;
        for (int q = start[c]; q < start[c + 1]; ++q) {
            const int f = faces[q];
            if (L.w[f] > mw) {
                match = f;
                mw = L.w[f];
            }
        }
        if (match >= 0) agg[c] = std::max(agg[L.upper[match]], agg[L.lower[match]]);
    }
    for (int c = 0; c < n; ++c)
        if (agg[c] < 0) agg[c] = nc++;
    for (int c = 0; c < n; ++c) agg[c] = nc - 1 - agg[c];
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
// Every kernel of a V-cycle returns at once when the finest level has
// stopped iterating (live->active == 0).
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
                acc = __dadd_rn(acc, __dadd_rn(fup[f], flo[f]));   // symmetric: upper + upper = 2 upper
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

// dst[R] (and dst2[R] when given) = sum over src of the row's finer rows
// (ascending, from zero)
__global__ void k_gamg_restrict(const Scal* __restrict__ live, int n, const int32_t* __restrict__ ptr,
                                const int32_t* __restrict__ idx, const double* __restrict__ src,
                                double* __restrict__ dst, double* __restrict__ dst2)
{
    if (!live->active) return;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int k = ptr[r]; k < ptr[r + 1]; ++k) acc = __dadd_rn(acc, src[idx[k]]);
        dst[r] = acc;
        if (dst2) dst2[r] = acc;
    }
}

// x[i] = c[map[i]] (add = 0) or x[i] + c[map[i]] (add = 1)
__global__ void k_gamg_prolong(const Scal* __restrict__ live, int n, const int32_t* __restrict__ map,
                               const double* __restrict__ c, double* x, int add)
{
    if (!live->active) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = add ? __dadd_rn(x[i], c[map[i]]) : c[map[i]];
}

// Dense LU without pivoting of the coarsest level (m <= kMaxTop), one CTA:
// thread i owns row i; every entry receives its updates in k order.
__global__ void k_gamg_lu(int m, int nf, const int32_t* __restrict__ lower, const int32_t* __restrict__ upper,
                          const double* __restrict__ diag, const double* __restrict__ up,
                          const double* __restrict__ lo, double* __restrict__ LU)
{
    extern __shared__ double M[];   // m * m
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
__global__ void k_gamg_dense_solve(const Scal* __restrict__ live, int m, const double* __restrict__ LU,
                                   const double* __restrict__ b, double* __restrict__ x)
{
    if (threadIdx.x != 0 || blockIdx.x != 0 || !live->active) return;
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

// The smoothed levels iterate exactly while the finest does.
__global__ void k_gamg_follow(const Scal* __restrict__ live, Scal* const* __restrict__ coarse, int nc)
{
    const int a = live->active;
    for (int l = threadIdx.x; l < nc; l += blockDim.x) coarse[l]->active = a;
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
    g->agglomerator = cfg.gamg_agglomerator;
    g->weights_version = m.agglom_version;
    g->sym = m.sym;
    HostLevel cur;
    cur.n = m.n;
    cur.lower = m.lower;
    cur.upper = m.upper;
    if (cfg.gamg_agglomerator == MRG_AGGLOMERATOR_FACE_AREA_PAIR) {
        if ((int)m.agglom_w.size() != m.nf)
            throw Error(MRG_E_INVALID, "GAMG agglomerator faceAreaPair needs the mesh's face area vectors "
                                       "(mrg_mesh_set_face_areas); algebraicPair needs none");
        cur.w = m.agglom_w;
    } else {
        cur.w.resize(m.nf);
        if (m.nf) MRG_CUDA(cudaMemcpy(cur.w.data(), m.raw_upper, 8 * (size_t)m.nf, cudaMemcpyDeviceToHost));
        for (double& v : cur.w) v = std::fabs(v);
    }
    g->lv.resize(1);
    std::vector<int32_t> fine_lower = cur.lower;
    for (;;) {
        if ((int)g->lv.size() >= 50) break;   // maxLevels
        std::vector<int32_t> agg;
        const int nc = agglomerate(cur, agg);
        if (nc < g->n_coarsest || nc >= cur.n) break;
        GamgLevel L;
        L.n = nc;
        L.agg = agg;
        L.members.assign(nc, {});
        for (int i = 0; i < cur.n; ++i) L.members[agg[i]].push_back(i);
        // coarse faces: per owner in order of first appearance
        const int nff = (int)cur.lower.size();
        std::vector<std::vector<int32_t>> own_faces(nc);
        std::vector<int32_t> nbr, restrict_(nff);
        std::vector<std::vector<int32_t>> inside(nc);
        for (int f = 0; f < nff; ++f) {
            const int ru = agg[cur.upper[f]], rl = agg[cur.lower[f]];
            if (ru == rl) {
                restrict_[f] = -(ru + 1);
                inside[ru].push_back(f);
                continue;
            }
            const int own = std::min(ru, rl), nei = std::max(ru, rl);
            int found = -1;
            for (int cf : own_faces[own])
                if (nbr[cf] == nei) {
                    found = cf;
                    break;
                }
            if (found < 0) {
                found = (int)nbr.size();
                nbr.push_back(nei);
                own_faces[own].push_back(found);
            }
            restrict_[f] = found;
        }
        const int nfc = (int)nbr.size();
        std::vector<int32_t> fmap(nfc);
        HostLevel nxt;
        nxt.n = nc;
        nxt.lower.resize(nfc);
        nxt.upper.resize(nfc);
        {
            int k = 0;
            for (int C = 0; C < nc; ++C)
                for (int cf : own_faces[C]) {
                    nxt.lower[k] = C;
                    nxt.upper[k] = nbr[cf];
                    fmap[cf] = k++;
                }
        }
        std::vector<std::vector<std::pair<int32_t, int32_t>>> fine_of(nfc);   // (fine face, flip)
        nxt.w.assign(nfc, 0.0);
        for (int f = 0; f < nff; ++f) {
            if (restrict_[f] < 0) continue;
            const int F = fmap[restrict_[f]];
            fine_of[F].push_back({f, nxt.lower[F] != agg[cur.lower[f]] ? 1 : 0});
            nxt.w[F] = nxt.w[F] + cur.w[f];
        }
        std::vector<int32_t> mem_ptr{0}, mem_idx, int_ptr{0}, int_idx, fc_ptr{0}, fc_idx, fc_flip;
        for (int C = 0; C < nc; ++C) {
            for (int i : L.members[C]) mem_idx.push_back(i);
            for (int f : inside[C]) int_idx.push_back(f);
            mem_ptr.push_back((int32_t)mem_idx.size());
            int_ptr.push_back((int32_t)int_idx.size());
        }
        for (int F = 0; F < nfc; ++F) {
            for (auto& ff : fine_of[F]) {
                fc_idx.push_back(ff.first);
                fc_flip.push_back(ff.second);
            }
            fc_ptr.push_back((int32_t)fc_idx.size());
        }
        L.nf = nfc;
        L.mem_ptr = upload(c, mem_ptr);
        L.mem_idx = upload(c, mem_idx);
        L.int_ptr = upload(c, int_ptr);
        L.int_idx = upload(c, int_idx);
        L.fc_ptr = upload(c, fc_ptr);
        L.fc_idx = upload(c, fc_idx);
        L.fc_flip = upload(c, fc_flip);
        L.diag = (double*)c->alloc(8 * (size_t)std::max(nc, 1));
        L.upper = (double*)c->alloc(8 * (size_t)std::max(nfc, 1));
        if (!m.sym) L.lower = (double*)c->alloc(8 * (size_t)std::max(nfc, 1));
        L.lo_dev = upload(c, nxt.lower);
        L.up_dev = upload(c, nxt.upper);
        g->lv.push_back(std::move(L));
        cur = std::move(nxt);
    }
    if (g->lv.size() < 2) {
        // no level kept (the first pairing already falls below
        // nCellsInCoarsestLevel): the matrix itself is the coarsest level
        g->identity = true;
        GamgLevel L;
        L.n = m.n;
        L.nf = m.nf;
        L.agg.resize(m.n);
        L.members.assign(m.n, {});
        std::vector<int32_t> mem_ptr{0}, mem_idx, int_ptr(m.n + 1, 0), fc_ptr{0}, fc_idx, fc_flip;
        for (int i = 0; i < m.n; ++i) {
            L.agg[i] = i;
            L.members[i].push_back(i);
            mem_idx.push_back(i);
            mem_ptr.push_back(i + 1);
        }
        for (int f = 0; f < m.nf; ++f) {
            fc_idx.push_back(f);
            fc_flip.push_back(0);
            fc_ptr.push_back(f + 1);
        }
        L.mem_ptr = upload(c, mem_ptr);
        L.mem_idx = upload(c, mem_idx);
        L.int_ptr = upload(c, int_ptr);
        L.int_idx = upload(c, std::vector<int32_t>{});
        L.fc_ptr = upload(c, fc_ptr);
        L.fc_idx = upload(c, fc_idx);
        L.fc_flip = upload(c, fc_flip);
        L.diag = (double*)c->alloc(8 * (size_t)std::max(m.n, 1));
        L.upper = (double*)c->alloc(8 * (size_t)std::max(m.nf, 1));
        if (!m.sym) L.lower = (double*)c->alloc(8 * (size_t)std::max(m.nf, 1));
        L.lo_dev = upload(c, m.lower);
        L.up_dev = upload(c, m.upper);
        g->lv.push_back(std::move(L));
    }
    const int top = (int)g->lv.size() - 1;
    if (g->lv[top].n > kMaxTop)
        throw Error(MRG_E_INVALID, "GAMG: the coarsest level has " + std::to_string(g->lv[top].n) +
                                       " cells, more than the direct solve's " + std::to_string(kMaxTop));
    g->lv[top].top = true;
    // smoothed levels: meshes of their own
    for (int l = 1; l < top; ++l) {
        GamgLevel& L = g->lv[l];
        L.mesh = std::make_unique<Mesh>();
        L.mesh->ctx = c;
        L.mesh->part_target = kPartTargetGs;
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
    g->d_coarse_sc = (Scal**)c->alloc(sizeof(Scal*) * (size_t)std::max(top, 1));
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

bool lu_attr_set(int device)
{
    static int done[64] = {};
    if (device < 0 || device >= 64) return false;
    if (!done[device]) {
        MRG_CUDA(cudaFuncSetAttribute(k_gamg_lu, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(sizeof(double) * kMaxTop * kMaxTop)));
        done[device] = 1;
    }
    return true;
}

}  // namespace

Gamg::~Gamg()
{
    for (auto& kv : graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (!ctx) return;
    for (GamgLevel& L : lv)
        for (void* p : {(void*)L.mem_ptr, (void*)L.mem_idx, (void*)L.int_ptr, (void*)L.int_idx, (void*)L.fc_ptr,
                        (void*)L.fc_idx, (void*)L.fc_flip, (void*)L.diag, (void*)L.upper, (void*)L.lower,
                        (void*)L.r_ptr, (void*)L.r_idx, (void*)L.p_map, (void*)L.lo_dev, (void*)L.up_dev})
            ctx->release(p);
    for (void* p : {(void*)lu, (void*)src_top, (void*)c_top, (void*)d_coarse_sc}) ctx->release(p);
}

Perf gamg_solve(Mesh& m, const double* d_b, double* d_x, const Controls& cfg)
{
    if (m.ni > 0) throw Error(MRG_E_INVALID, "GAMG: meshes with interfaces are not supported (use the global form)");
    if (!m.have_coeffs) throw Error(MRG_E_INVALID, "no coefficients uploaded for this mesh");
    if (!m.gamg || m.gamg->n_coarsest != cfg.gamg_coarsest || m.gamg->sym != m.sym ||
        m.gamg->agglomerator != cfg.gamg_agglomerator ||
        (cfg.gamg_agglomerator == MRG_AGGLOMERATOR_FACE_AREA_PAIR && m.gamg->weights_version != m.agglom_version)) {
        m.gamg.reset();
        build(m, cfg);
    }
    Gamg& g = *m.gamg;
    Ctx* c = m.ctx;
    cudaStream_t st = c->st;
    lu_attr_set(c->device);
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
        k_gamg_lu<<<1, std::max(32, ((T.n + 31) / 32) * 32), sizeof(double) * T.n * T.n, st>>>(
            T.n, T.nf, T.lo_dev, T.up_dev, T.diag, T.upper, m.sym ? nullptr : T.lower, g.lu);
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
    {
        std::vector<Scal*> csc;
        for (int l = 1; l < top; ++l) csc.push_back(P[l]->sys.sc);
        if (!csc.empty())
            MRG_CUDA(cudaMemcpyAsync(g.d_coarse_sc, csc.data(), sizeof(Scal*) * csc.size(), cudaMemcpyHostToDevice,
                                     st));
    }
    P0.sys.in_b = d_b;
    P0.sys.in_x = d_x;
    P0.sys.out_x = d_x;
    P0.sync_sys();
    P0.single.sync_sys();
    const Scal* live = P0.sys.sc;
    const bool scale = cfg.gamg_scale != 0;
    auto vec = [&](int l, int which) -> double* {   // 0: source b, 1: correction x, 2: r, 3: p
        if (l == top) return which == 0 ? g.src_top : g.c_top;
        const Vecs<double>& v = P[l]->sys.v64;
        return which == 0 ? v.b : which == 1 ? v.x : which == 2 ? v.r : v.p;
    };
    auto sweeps = [&](int l, int k) {
        BatchHost& bh = P[l]->single;
        int parts = 0, cells = 0;
        part_choice(bh, parts, cells, true);
        for (int s = 0; s < k; ++s) {
            launch_gs_sweep(bh.d, c->nsm * 4, st, parts, cells);
            launch_rows(OP_GS_COPY, 0, bh.d, P[l]->ntiles, bh.h.nsegs, 0, st);
        }
    };
    auto scaled = [&](int l, RowOp apply) {
        BatchHost& bh = P[l]->single;
        launch_rows(OP_GSCALE_DOT, 0, bh.d, P[l]->ntiles, bh.h.nsegs, 0, st);
        launch_rows(apply, 0, bh.d, P[l]->ntiles, bh.h.nsegs, 0, st);
    };
    // one V-cycle; the launches read only device state, so it is captured
    auto record_cycle = [&]() {
        if (top > 1) {
            k_gamg_follow<<<1, 64, 0, st>>>(live, g.d_coarse_sc, top - 1);
            add_launches(1);
        }
        // down: restrict the finest residual, then each source (a smoothed
        // level scaled against its source keeps a copy in r)
        for (int l = 1; l <= top; ++l) {
            const GamgLevel& L = g.lv[l];
            const double* src = l == 1 ? P0.sys.v64.r : vec(l - 1, 0);
            double* dst2 = (scale && l < top - 1) ? vec(l, 2) : nullptr;
            k_gamg_restrict<<<grid_of(L.n), 256, 0, st>>>(live, L.n, L.r_ptr, L.r_idx, src, vec(l, 0), dst2);
        }
        k_gamg_dense_solve<<<1, 32, 0, st>>>(live, g.lv[top].n, g.lu, g.src_top, g.c_top);
        add_launches(top + 1);
        // up: prolong, scale and smooth the corrections
        for (int l = top - 1; l >= 1; --l) {
            const bool sl = scale && l < top - 1;
            k_gamg_prolong<<<grid_of(g.lv[l].n), 256, 0, st>>>(live, g.lv[l].n, g.lv[l + 1].p_map, vec(l + 1, 1),
                                                               vec(l, sl ? 3 : 1), 0);
            add_launches(1);
            if (sl) scaled(l, OP_GSCALE_SET);
            sweeps(l, std::min(cfg.gamg_post + cfg.gamg_post_mult * (l - 1), cfg.gamg_max_post));
        }
        const bool sf = scale && !g.identity;
        k_gamg_prolong<<<grid_of(m.n), 256, 0, st>>>(live, m.n, g.lv[1].p_map, vec(1, 1),
                                                     sf ? P0.sys.v64.p : P0.sys.v64.x, sf ? 0 : 1);
        add_launches(1);
        if (sf) scaled(0, OP_GSCALE_ADD);
        sweeps(0, cfg.gamg_finest);
        launch_rows(OP_GS_RES, 0, P0.single.d, P0.ntiles, P0.single.h.nsegs, 0, st);
    };
    const int K = std::max(1, std::min(cfg.k_launch, 2));   // V-cycles per graph launch
    std::string key = std::to_string(K) + "/" + std::to_string(scale) + "/" + std::to_string(cfg.gamg_post) + "/" +
                      std::to_string(cfg.gamg_post_mult) + "/" + std::to_string(cfg.gamg_max_post) + "/" +
                      std::to_string(cfg.gamg_finest) + "/" + std::to_string(c->nsm) + "/" +
                      std::to_string(c->unpublished1);
    for (int l = 0; l < top; ++l) key += "/" + std::to_string((uintptr_t)P[l]);
    auto it = g.graphs.find(key);
    if (it == g.graphs.end()) {
        cudaGraph_t gr = nullptr;
        const unsigned long long before = launch_count();
        MRG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < K; ++k) record_cycle();
        const cudaError_t e = cudaStreamEndCapture(st, &gr);
        const long long nodes = (long long)(launch_count() - before);
        add_launches(-nodes);   // captured, not executed
        MRG_CUDA(e);
        cudaGraphExec_t ex = nullptr;
        const cudaError_t ei = cudaGraphInstantiate(&ex, gr, 0);
        cudaGraphDestroy(gr);
        MRG_CUDA(ei);
        it = g.graphs.emplace(key, Gamg::Graph{ex, nodes}).first;
    }
    const Gamg::Graph cyc = it->second;
    cudaEvent_t e0, e1;
    MRG_CUDA(cudaEventCreate(&e0));
    MRG_CUDA(cudaEventCreate(&e1));
    Perf out;
    try {
        MRG_CUDA(cudaEventRecord(e0, st));
        batch_begin(P0.single, fc);   // permute in, initial residual, arm the sweep output
        for (int l = 1; l < top; ++l) {
            launch_rows(OP_GS_ARM, 0, P[l]->single.d, P[l]->ntiles, P[l]->single.h.nsegs, 0, st);
        }
        long cycles = 0;
        const long cap = (long)cfg.max_iter + cfg.min_iter + 2;
        while (batch_poll(P0.single).n_active > 0 && cycles <= cap) {
            MRG_CUDA(cudaGraphLaunch(cyc.exec, st));
            add_launches(cyc.nodes);
            cycles += K;
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
