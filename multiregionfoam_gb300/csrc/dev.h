// dev.h -- plain-old-data views shared by host and device code.
//
// A "system" is one LDU matrix with its plan, coefficients, work vectors and
// scalar solver state, all resident in HBM.  Kernels take an array of
// SysDev (one entry for a single solve, many for a batch) and a tile table;
// every per-system reduction is two-level and deterministic: one partial per
// 1024-row tile, summed in tile order by the last tile to finish.
#pragma once
#include <cstdint>

namespace mrg {

constexpr int kBlock = 256;   // threads per CTA for row kernels
constexpr int kMaxRed = 2;    // values reduced per tile

// Scalar state of one solve (lduSolverPerformance + Krylov scalars).
struct Scal {
    double rho, rho_old, alpha, beta;
    double nfac, res0, res, xsum;
    double tol, rel_tol;
    double red[kMaxRed];   // last finalised reduction sums (diagnostics)
    double osum;           // mixed: sum|b - A x| of the FP64 outer residual
    double inv_scale;      // mixed: FP32 inner system is scaled by 1/inv_scale
    int min_iter, max_iter;
    int iter, active, converged, singular;
    int status, pad;
};

template <typename V>
struct Vecs {
    V *x, *b, *r, *w, *y, *p, *q;   // A-system vectors (x,p carry the GGI tail)
    V *rT, *wT, *yT, *pT, *qT;      // transpose system (PBiCG)
};

// Which preconditioner the sweeps apply.
enum { PC_NONE = 0, PC_DIAG = 1, PC_DIC = 2, PC_DILU = 3 };

struct SysDev {
    int n, npad, nsl, ntiles;
    int nchunks, nlevels, nf, ni, ngen, sym, pc;
    int pad0;
    // plan
    const int32_t *perm, *a_sptr, *a_col, *a_src, *chunk_start, *lvl_chunk;
    const int32_t *f_sptr, *f_col, *f_src, *b_sptr, *b_col, *b_src;
    const int32_t *g_ptr, *g_src;
    const double* g_w;
    const float* g_w32;
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
    // reductions / state
    double* partials;      // [ntiles * kMaxRed]
    unsigned* counter;     // [1]
    Scal* sc;
};

// Per-launch control block shared by the systems of one batch.
struct Ctl {
    unsigned ticket[8];    // sync-free sweep work counters
    unsigned err;          // error bits (1 = wait timeout)
    unsigned n_active;
    unsigned pad[6];
};

enum { ERR_TIMEOUT = 1u, ERR_BREAKDOWN = 2u };

}  // namespace mrg
