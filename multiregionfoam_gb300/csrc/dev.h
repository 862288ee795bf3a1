// dev.h -- plain-old-data views shared by host and device code.
//
// A "system" is one LDU matrix with its plan, coefficients, work vectors and
// scalar solver state, all resident in HBM.  A "batch" is a set of systems
// solved in lockstep: every kernel takes one device-resident Batch
// descriptor (the system array, a tile table over all systems, the per-level
// sweep work list and the control block), so a single solve is a batch of one
// and a captured CUDA graph stays valid when the batch's membership changes.
// Every per-system reduction is deterministic: one partial per contiguous
// tile segment of a fixed-size grid, summed in slot order by the last CTA.
#pragma once
#include <cstdint>

namespace mrg {

constexpr int kBlock = 256;   // threads per CTA for row kernels
constexpr int kMaxRed = 2;    // values reduced per tile
// A system of T tiles is reduced in G contiguous tile segments, segment j =
// tiles [j*T/G, (j+1)*T/G): G = ceil(T / 4) up to kSegSplit tiles, T above
// (one tile a segment, so a lone system of that size runs its row kernels on
// one CTA per tile instead of a quarter as many), at most kRedSegs.  The
// summation order of every per-system reduction depends only on the system
// itself -- not on the device, the launch grid or the other members of a
// batch.  Small systems keep four-tile segments: a batch of hundreds of them
// pays one segment flush per segment, and one-tile segments cost the 512-
// system batch a quarter of its speed.
constexpr int kRedSegs = 608;
constexpr int kSegTiles = 4;
constexpr int kSegSplit = 256;
__host__ __device__ inline int red_segments(int tiles)
{
    const int g = tiles > kSegSplit ? tiles : (tiles + kSegTiles - 1) / kSegTiles;
    return g < kRedSegs ? (g > 0 ? g : 1) : kRedSegs;
}

// Scalar state of one solve (lduSolverPerformance + Krylov scalars), plus
// the FP64 outer state of a mixed-precision solve.
struct Scal {
    double rho, rho_old, alpha, beta;
    double omega;          // BiCGStab: (t, s) / (t, t) of the current iteration
    double nfac, res0, res, xsum;
    double tol, rel_tol;
    double red[kMaxRed];   // last finalised reduction sums (diagnostics)
    double osum;           // mixed: sum|b - A x| of the FP64 outer residual
    double inv_scale;      // mixed: FP32 inner system is scaled by 1/inv_scale
    // mixed-precision outer (FP64) state and controls
    double onfac, ores0, ores, obest;
    double obest_sum;      // mixed: sum|b - A x| of the best refined iterate
    double otol, orel_tol, inner_rel_tol;
    int min_iter, max_iter;  // user controls (foam minIter / maxIter)
    int kmin, kmax;          // bounds of the current Krylov loop
    int iter, active, converged, singular;
    int status, mixed;
    int ostate, oconv, oiter, ostall;
    int inner_total, inner_max, max_outer;
    int okeep;             // mixed: 1 = the last refinement improved (keep x), 0 = roll back
    int fallback;          // mixed: 1 = refinement stalled, FP64 Krylov requested; 2 = running it;
                           // 3 = done (true residual checked)
    int n_sweeps;          // smoothSolver: Gauss-Seidel sweeps per iteration
};

// PCG / PBiCG use the slots by name (T = the transpose system).  BiCGStab
// keeps r (and s) in r, the shadow residual r~ in rT, the search direction
// in wT, M^-1 p in p and M^-1 s in pT (both SpMV inputs, so both carry the
// GGI tail), v = A M^-1 p in q and t = A M^-1 s in qT; y and yT are the
// triangular sweeps' intermediates.
template <typename V>
struct Vecs {
    V *x, *b, *r, *w, *y, *p, *q;   // A-system vectors (x,p carry the GGI tail)
    V *rT, *wT, *yT, *pT, *qT;      // transpose system (PBiCG; pT carries the GGI tail)
};

// Which preconditioner the sweeps apply.  PC_BLOCK: the block (bs x bs)
// incomplete factorisation of a block-expanded system (BlockDev), applied by
// its own kernels; the scalar factor and sweep kernels skip it.
enum { PC_NONE = 0, PC_DIAG = 1, PC_DIC = 2, PC_DILU = 3, PC_BLOCK = 4 };
__host__ __device__ inline bool scalar_tri(int pc) { return pc == PC_DIC || pc == PC_DILU; }

// A block-expanded system's block view (cell c's component a is the scalar
// caller row bs c + a): the cell mesh's exact plan (internal cell order,
// chunks of <= 32 cells of one level, forward / backward dependency ELLs
// with face codes as in the scalar plan), where each block entry's scalar
// coefficient sits, the blocks gathered from the scalar coefficients, the
// factor, and the scalar internal row of every (cell, component).
struct BlockDev {
    int bs, n, nf, nchunks;
    const int32_t *perm, *chunk_start;            // internal cell -> caller cell
    const int32_t *f_sptr, *f_col, *f_src, *b_sptr, *b_col, *b_src;
    const int32_t *dmap;                          // [n bs bs]: >= 0 diag row; < 0: -1 - scalar face (upper
                                                  // triangle of the block: upper, else lower)
    const int32_t *fmap;                          // [nf bs bs]: scalar face of U_f[a][b]
    double *D, *U, *L;                            // gathered blocks (caller cell / face order)
    double* dD;                                   // [n bs bs] inverse of the factored diagonal (internal)
    const int32_t* vmap;                          // [n bs]: scalar internal row of (internal cell, a)
    int sym;
};

struct SysDev {
    int n, npad, nsl, ntiles;
    int nchunks, nlevels, nf, ni, ngen, sym, pc;
    int syncfree;          // exact ordering: sentinel-based sweeps
    // plan
    const int32_t *perm, *a_sptr, *a_col, *a_src, *chunk_start, *lvl_chunk;
    const uint16_t* a_col16;   // a_col as offsets from a_cbase (rounds of 8 slices that fit)
    const int32_t* a_cbase;    // [nsl + 8] per-slice base, -1: the round keeps a_col
    const int32_t *f_sptr, *f_col, *f_src, *b_sptr, *b_col, *b_src;
    const int32_t *g_ptr, *g_src;
    const double* g_w;
    const float* g_w32;
    // owner-computes exact sweeps (k_sweep_part): nparts ranges of part_cells
    // caller cells, each part's rows in level order with their level
    // ordinals, each dependency's place in its row's part (-1: another part)
    // and each row's sweep entries; nparts = 0: not built
    const BlockDev* blk;   // PC_BLOCK: the block view (device)
    int nparts, part_cells;
    const int32_t *pt_ptr, *part_rows, *part_step, *f_loc, *b_loc;
    const int2 *f_row, *b_row;   // per row: (first sweep entry, entries)
    // raw coefficients in the caller's numbering
    const double *raw_diag, *raw_upper, *raw_lower, *raw_ibou, *raw_iint;
    // FP64 coefficient views (internal numbering)
    double *a_val, *aT_val, *diag, *sumA;
    double *f_c, *f_cT, *b_c, *b_cT, *rD, *D;
    // FP32 copies (mixed precision inner loop)
    float *a_val32, *aT_val32, *diag32;
    float *f_c32, *f_cT32, *b_c32, *b_cT32, *rD32;
    Vecs<double> v64;
    Vecs<float> v32;
    // mixed precision: best refined iterate and its FP64 residual
    double *xb, *rb;
    // FP32 PCG with a levelled DIC: sum of r w over each chunk, written by
    // the sweep that writes the chunk's w  [nchunks]
    float* chunk_rw;
    // caller-numbered input/output of the current solve
    const double *in_b, *in_x;
    double* out_x;
    // reductions / state
    double* partials;      // [ntiles * kMaxRed]
    unsigned* counter;     // [1]
    Scal* sc;
};

// Control block of one batch.
struct Ctl {
    unsigned ticket[8];    // sync-free sweep work counters
    unsigned err;          // error bits (1 = wait timeout)
    unsigned n_active;     // systems still in their Krylov loop
    unsigned n_oactive;    // systems still in their mixed-precision outer loop
    unsigned bar_count;    // persistent iteration kernel: CTAs at the grid barrier
    unsigned bar_gen;      // persistent iteration kernel: barrier generation
    int unpublished1;      // test hook: chunk unpublished1 - 1 of the exact forward
                           // sweep is never published, so every wait on it runs
                           // out (0: off, which a cleared block is)
    unsigned pad[2];
    long long wait_cycles; // budget of every device wait, SM cycles (0: the default)
    // controls written into every system's Scal by OP_BEGIN
    double tol, rel_tol, inner_rel_tol;
    int min_iter, max_iter, inner_max, max_outer, mixed, n_sweeps;
};

// A batch of systems, resident on the device.
struct Batch {
    SysDev* sys;           // [nsys]
    const int2* tiles;     // [ntiles] (system, tile within system), systems contiguous
    const int2* segs;      // [nsegs] (system, reduction segment), see kRedSegs
    const int2* items;     // level-sweep work: (system, chunk) grouped by level
    const int* item_off;   // [maxlevels + 1]
    const int2* sf_items;  // sync-free sweep work of a batch of several systems: (system, chunk) by level
    Ctl* ctl;
    int nsys, ntiles, nsegs, maxchunks, maxlevels, n_sf;
};

enum { ERR_TIMEOUT = 1u, ERR_BREAKDOWN = 2u };

}  // namespace mrg
