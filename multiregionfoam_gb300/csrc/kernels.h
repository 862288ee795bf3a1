// kernels.h -- launchers for the sm_103a kernels in kernels.cu.
//
// Every launcher takes a device-resident Batch descriptor (dev.h); the
// kernels read the batch's sizes from it at run time, so a captured graph of
// launches stays valid when the batch's contents change.  Host-side sizes
// passed here are upper bounds used only to size grids.
#pragma once
#include <cuda_runtime.h>

#include "dev.h"

namespace mrg {

// Row-kernel operations (tiles of 1024 rows).
enum RowOp {
    OP_SCATTER = 0,     // raw coefficients -> internal views (+ sumA), arms the factor
    OP_SUMX,            // xsum = sum(x)
    OP_INIT_RES,        // r = b - A x (rT = b - A^T x), normFactor, initial residual
    OP_RHO,             // rho = (w, r)  [PBiCG: (w, rT)], beta
    OP_PUPDATE,         // p = w + beta p  [+ pT]
    OP_SPMV_QP,         // q = A p [+ qT = A^T pT], (q, p) [PBiCG: (q, pT)], alpha
    OP_UPDATE,          // x += alpha p, r -= alpha q [+ rT], final residual, convergence
    OP_PRECOND_DIAG,    // w = rD r  [+ wT]
    OP_PRECOND_NONE,    // w = r     [+ wT]
    OP_RESID64,         // mixed: r64 = b - A x (FP64), outer convergence test
    OP_TO32,            // mixed: r32 = float(s * r64), inner state
    OP_CORRECT,         // mixed: x64 += d32 / s
    OP_AMUL,            // y = A x (test hook; x in v64.p, y in v64.q)
    OP_TMUL,            // y = A^T x (test hook)
    OP_DIAG_RD,         // rD = 1/diag (diagonal preconditioner)
    OP_BEGIN,           // start of a solve: controls into Scal, sweep sentinels
    OP_PERMUTE_IN,      // b, x from the caller's numbering (in_b, in_x)
    OP_PERMUTE_OUT,     // x to the caller's numbering (out_x)
    OP_KEEPBEST,        // mixed: after RESID64, keep (x, r) as the best or roll back to it
    OP_FALLBACK64,      // mixed, refinement stalled: FP64 Krylov restart from the best x
    OP_BS_RHO0,         // BiCGStab start: r~ = r, rho = (r~, r)
    OP_BS_P,            // BiCGStab: p = r + beta (p - omega v)  [+ M^-1 p when diagonal / none]
    OP_BS_V,            // BiCGStab: v = A M^-1 p, (r~, v), alpha
    OP_BS_S,            // BiCGStab: s = r - alpha v, x += alpha M^-1 p, sum|s|, half-step test
    OP_BS_T,            // BiCGStab: t = A M^-1 s, (t, s), (t, t), omega
    OP_BS_XR,           // BiCGStab: x += omega M^-1 s, r = s - omega t, sum|r|, (r~, r), convergence
    OP_GS_ARM,          // smoothSolver: arm the sweep's output y with sentinels
    OP_GS_COPY,         // smoothSolver: x = y (the sweep's result), re-arm y
    OP_GS_RES,          // smoothSolver: r = b - A x, sum|r|, iterations += nSweeps, convergence
    OP_SM_RES,          // smoothSolver DIC / DILU step: r = b - A x
    OP_SM_ADD,          // smoothSolver DIC / DILU step: x += w (w = M^-1 r)
    OP_RHO_CH,          // FP32 PCG, levelled DIC: rho = sum of the sweeps' per-chunk (r, w), beta
    OP_GSCALE_DOT,      // GAMG scaleCorrection: q = A p, (r, p) and (q, p), sf = (r, p) / (q, p)
    OP_GSCALE_SET,      // GAMG scaleCorrection, coarse level: x = sf p + (r - sf q) / diag
    OP_GSCALE_ADD,      // GAMG scaleCorrection, finest level: x += sf p + (r - sf q) / diag
    OP_COUNT
};

// precision: 0 = FP64 vectors/coefficients, 1 = FP32 (mixed inner loop).
// ntiles, nsegs: upper bounds on the batch's tile and segment counts.
// spmv (OP_SPMV_QP without the transpose): the Amul kernel -- 0 the
// default, 1 the per-warp staged kernel (256-thread CTAs), 2 the streamed
// kernel one round (32 rows a warp) per step, 3 two rounds per step (FP32;
// a producer warp beside 256 row threads).  Every choice gives the same bits.
void launch_rows(RowOp op, int precision, const Batch* dB, int ntiles, int nsegs, int pb, cudaStream_t st,
                 int spmv = 0);

// One Gauss-Seidel sweep of foam's smoother in foam's cell order (sync-free
// over the exact plan's chunks): y = sweep(x, b), lower neighbours from y
// (waited for), upper neighbours and interfaces from x.
// parts > 0 (a batch of one system whose plan has parts of part_cells
// cells): the owner-computes kernel, one CTA a part.
void launch_gs_sweep(const Batch* dB, int grid, cudaStream_t st, int parts = 0, int part_cells = 0);

// Owner-computes exact sweeps: the most cells a part holds (its FP64
// values sit in shared memory; larger parts: the ticketed sync-free kernel),
// and the part sizes aimed at -- DIC / DILU sweeps (a mesh's own plan) and
// the Gauss-Seidel sweeps of GAMG's coarse levels, whose FP64 division per
// row favours more, smaller parts (both measured best on GB300).
constexpr int kPartMaxCells = 8192;
constexpr int kPartTarget = 4096;
constexpr int kPartTargetGs = 2048;
// DIC / DILU sweeps take the owner-computes kernel only with at most
// kPartMaxTri parts and at least kPartRowsPerLevel rows a part and level.
constexpr int kPartMaxTri = 64;
constexpr int kPartRowsPerLevel = 16;

// Sentinel fill of a vector (sync-free readiness marker).
void launch_fill_sentinel(void* p, long long n, int precision, cudaStream_t st);

// Level-scheduled DIC/DILU factor, sync-free over chunks (forward order), for
// every system of the batch with a DIC/DILU preconditioner.
// with32: also write FP32 copies of rD and sweep coefficients.
void launch_factor(const Batch* dB, int grid, int with32, cudaStream_t st);

// One triangular sweep.  fwd: y = forward(r); else w = backward(y).
// trans selects the vectors and coefficients (vector set): 0 = r -> y -> w,
// 1 = rT -> yT -> wT with DILU's preconditionT coefficients, and for
// BiCGStab 2 = wT -> y -> p (M^-1 p) and 3 = r -> yT -> pT (M^-1 s).
// syncfree=1: all levels in one launch (exact ordering); else one level.
// rho_chunks=1 (FP32 levelled sweeps of vector set 0): every chunk whose w
// the launch writes also gets its sum of r w in chunk_rw, which OP_RHO_CH
// then reduces.  parts > 0 (syncfree, a batch of one system whose plan has
// parts of part_cells cells): the owner-computes kernel, one CTA a part.
void launch_sweep(int precision, int fwd, int trans, int syncfree, int level, const Batch* dB, int grid,
                  cudaStream_t st, int rho_chunks = 0, int parts = 0, int part_cells = 0);

// GGI gather of the general interface faces: x[npad + j] = sum w x[src]
// (which: 0 = p, 1 = x, 2 = pT; 0 and 2 skip inactive systems, 3 = p always).
void launch_iface_gather(int precision, int which, const Batch* dB, int grid, cudaStream_t st);

// Block preconditioner (PC_BLOCK, BlockDev): gather one system's blocks
// from its raw scalar coefficients (raw_lower NULL: symmetric); factor, and
// one sweep (fwd: y = forward(r), else w = backward(y); vs as launch_sweep's,
// 0, 2 or 3) of every PC_BLOCK member of the batch, sync-free over the cell
// plan's chunks.  bs: the members' block size (1..4).
void launch_block_gather(const BlockDev* d_blk, int n, int nf, int bs, const double* raw_diag,
                         const double* raw_upper, const double* raw_lower, cudaStream_t st);
void launch_block_factor(int bs, const Batch* dB, int grid, cudaStream_t st);
void launch_block_sweep(int bs, int fwd, int vs, const Batch* dB, int grid, cudaStream_t st);

// Internal <-> caller numbering (FP64) of one system (test hooks).
void launch_permute(int to_internal, const SysDev* d_sys, int sysidx, const double* src,
                    double* dst, int n, cudaStream_t st);

// Stand-alone GGI weighted gather (mrg_ggi_apply).
void launch_ggi(int n_dst, const int32_t* ptr, const int32_t* addr, const double* w,
                const double* src, double* dst, int ncomp, cudaStream_t st);

// Kernels launched so far in this process (captured launches included;
// the engine corrects for graph capture and replay).
// K Krylov iterations of the batch in one cooperative (persistent) launch
// whose phases are the launches of one iteration, separated by grid
// barriers; grid = every resident CTA.  syncfree: exact-order sweeps;
// otherwise levelled (colour) sweeps.  gen: members have general
// interfaces.  Returns the launch status.
cudaError_t launch_iterate(int precision, int pb, int syncfree, const Batch* dB, int K, int pc, int gen,
                           cudaStream_t st);

// Serving support: copy every member's Scal into out[nsys]; recompute the
// control block's n_active / n_oactive from the members' flags.
void launch_gather_scal(const Batch* dB, Scal* out, cudaStream_t st);
void launch_recount(const Batch* dB, cudaStream_t st);

unsigned long long launch_count();
// SM count of the device in use (sizes the persistent grids).
void set_device_sms(int nsm);
int persistent_grid();
void add_launches(long long d);

}  // namespace mrg
