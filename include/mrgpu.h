/*
 * mrgpu.h -- C ABI of the GB300 coupled-region LDU solver library (libmrgpu).
 *
 * This is the boundary a foam-extend 4.1 build of multiRegionFoam calls
 * through: the lduMatrix::solver adapters (gpuPCG, gpuPBiCG, gpuBiCGStab and
 * their gpuMixed* forms) and the GGI transfer adapter hand plain host or device
 * pointers and sizes to these functions.  No C++ or torch types cross it.
 *
 * Conventions
 *   - Every function returns an int status (MRG_OK or an MRG_E_* code); the
 *     text of the last error on the calling thread is mrg_last_error().
 *   - Arrays follow foam's lduAddressing/lduMatrix layout: lowerAddr (owner)
 *     and upperAddr (neighbour) per internal face, lower < upper, faces in
 *     upper-triangular order; diag[n], upper[F], lower[F] (NULL when the
 *     matrix is symmetric); int32 labels and double scalars (-DWM_LABEL_SIZE=32
 *     -DWM_DP in the reference's compile_commands.json).
 *   - Caller owns every host array; the library reads it during the call and
 *     keeps no reference.  The library owns its device copies.
 *   - x_inout is foam's psi: the initial guess on entry, the solution on exit.
 *   - One context per host thread, or external synchronisation.  Each context
 *     owns one CUDA stream; calls are synchronous with respect to the host
 *     unless stated otherwise.
 */
#ifndef MRGPU_H
#define MRGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------- */
enum {
    MRG_OK = 0,
    MRG_E_INVALID = 1,   /* bad argument, size or addressing               */
    MRG_E_OOM = 2,       /* device allocation failed or HBM budget exceeded */
    MRG_E_BREAKDOWN = 3, /* non-finite coefficients / factor breakdown      */
    MRG_E_TIMEOUT = 4,   /* a device-side wait gave up (watchdog)           */
    MRG_E_CUDA = 5,      /* CUDA runtime error                              */
    MRG_E_BUSY = 6       /* server queue full                               */
};

/* ---- solver selection (the fvSolution "solver" / "preconditioner" words) */
/* BiCGStab: the stabilised bi-conjugate gradient foam-extend's lduSolvers
 * register as "BiCGStab" for both matrix kinds, and the solver of the
 * reference tutorials' monolithic coupled matrices (system/solid/fvSolution
 * Tcoupled: BiCGStab, tolerance 1e-15, maxIter 200).  Preconditioned on the
 * right (van der Vorst 1992): one M^-1 p and one M^-1 s per iteration, the
 * residual of s tested after the first half step. */
/* SMOOTH: foam's smoothSolver with the GaussSeidel smoother (the tutorials'
 * fluid U solves): n_sweeps Gauss-Seidel sweeps in foam's cell order, then
 * the residual, until converged; FP64, exact ordering only. */
/* GAMG: foam's geometric-algebraic multigrid solver (the tutorials' fluid
 * p / T solves) with the GaussSeidel smoother: pairwise agglomeration
 * (faceAreaPair on the mesh's face areas, or algebraicPair on the first
 * matrix's coefficients; cached), a V-cycle per iteration (restricted
 * residual, a direct solve of the coarsest level, prolonged corrections
 * scaled (scaleCorrection) and smoothed by min(nPostSweeps +
 * postSweepsLevelMultiplier * level, maxPostSweeps) sweeps, nFinestSweeps
 * on the finest level); FP64, exact ordering, a mesh without interfaces,
 * one system at a time. */
enum { MRG_SOLVER_PCG = 0, MRG_SOLVER_PBICG = 1, MRG_SOLVER_BICGSTAB = 2, MRG_SOLVER_SMOOTH = 3,
       MRG_SOLVER_GAMG = 4 };
/* smoothSolver smoothers: GaussSeidel; DIC / DILU (each sweep adds
 * M^-1 (b - A psi) to psi with the incomplete factorisation M); and
 * DICGaussSeidel / DILUGaussSeidel (that step, then a Gauss-Seidel sweep). */
enum {
    MRG_SMOOTHER_GAUSS_SEIDEL = 0,
    MRG_SMOOTHER_DIC = 1,
    MRG_SMOOTHER_DILU = 2,
    MRG_SMOOTHER_DIC_GAUSS_SEIDEL = 3,
    MRG_SMOOTHER_DILU_GAUSS_SEIDEL = 4
};
enum {
    MRG_PRECOND_NONE = 0,     /* "none"     */
    MRG_PRECOND_DIAGONAL = 1, /* "diagonal" */
    MRG_PRECOND_DIC = 2,      /* "DIC"      */
    MRG_PRECOND_DILU = 3,     /* "DILU"     */
    MRG_PRECOND_BLOCK = 4     /* "Cholesky" of a block system (foam-extend's
                                 BlockCholeskyPrecon, the block solvers'
                                 preconditioner): incomplete factorisation on
                                 the bs x bs blocks of a mesh declared by
                                 mrg_mesh_set_blocks -- D_c = A_cc - sum of
                                 L_f inv(D_l) U_f over the faces into c;
                                 x_c = inv(D_c) r_c, then x_u -= inv(D_u) L_f x_l
                                 (faces ascending) and x_l -= inv(D_l) U_f x_u
                                 (descending).  PCG (symmetric) or BiCGStab,
                                 FP64, exact ordering                        */
};
enum {
    MRG_PRECISION_FP64 = 0,  /* plain method: FP64 throughout, foam order   */
    MRG_PRECISION_MIXED = 1  /* FP32 Krylov inner loop inside FP64 iterative
                                refinement (FP64 residual, solution, dots and
                                convergence test)                           */
};
enum {
    MRG_ORDER_EXACT = 0,   /* preconditioner sweeps in foam's face order
                              (level-scheduled; identical to the sequential
                              sweep)                                        */
    MRG_ORDER_COLOUR = 1   /* multi-colour renumbering for the
                              preconditioner (fewer sweep levels, different
                              incomplete factorisation)                      */
};
/* GAMG agglomerator ("agglomerator" word; foam's default is faceAreaPair) */
enum {
    MRG_AGGLOMERATOR_ALGEBRAIC_PAIR = 0,  /* |upper| of the finest matrix     */
    MRG_AGGLOMERATOR_FACE_AREA_PAIR = 1   /* face areas (mrg_mesh_set_face_areas) */
};

typedef struct mrg_ctx mrg_ctx;
typedef struct mrg_mesh mrg_mesh;
typedef struct mrg_ggi mrg_ggi;
typedef struct mrg_batch mrg_batch;
typedef struct mrg_server mrg_server;

/* The lduMatrix::solver controls dictionary (tolerance, relTol, minIter,
 * maxIter, preconditioner) plus the GPU-specific choices.  Zero-initialise
 * and call mrg_controls_default() to get foam's defaults. */
typedef struct {
    double tolerance;      /* foam default 1e-6                             */
    double rel_tol;        /* foam default 0                                */
    int min_iter;          /* foam default 0                                */
    int max_iter;          /* foam default 1000                             */
    int solver;            /* MRG_SOLVER_*                                  */
    int preconditioner;    /* MRG_PRECOND_*                                 */
    int precision;         /* MRG_PRECISION_*                               */
    int ordering;          /* MRG_ORDER_*                                   */
    double inner_rel_tol;  /* mixed: the most an FP32 inner solve is asked to
                              reduce its residual per refinement step
                              (default 1e-5); each step aims at 0.1 x the
                              residual still to remove, never below this    */
    int inner_max_iter;    /* mixed: inner iterations per outer step; 0 =
                              max_iter for PCG, 150 for PBiCG, 300 for
                              BiCGStab (an FP32 BiCG-type recurrence can
                              drift and diverge; restarting it from the FP64
                              residual keeps it stable)                      */
    int max_outer;         /* mixed: refinement steps (default 50)          */
    int iters_per_launch;  /* iterations per CUDA-graph launch (default 16) */
    int smoother;          /* MRG_SOLVER_SMOOTH: MRG_SMOOTHER_*             */
    int n_sweeps;          /* MRG_SOLVER_SMOOTH: sweeps per residual check
                              (foam's nSweeps, default 1)                   */
    int gamg_coarsest_cells; /* GAMG: nCellsInCoarsestLevel (default 10)     */
    int gamg_post_sweeps;  /* GAMG: nPostSweeps (default 2)                 */
    int gamg_finest_sweeps; /* GAMG: nFinestSweeps (default 2)              */
    int gamg_max_post_sweeps; /* GAMG: maxPostSweeps (default 4)            */
    int gamg_post_sweeps_level_multiplier; /* GAMG: postSweepsLevelMultiplier
                              (default 1)                                   */
    int gamg_scale_correction; /* GAMG: scaleCorrection (default 1)         */
    int gamg_agglomerator; /* GAMG: MRG_AGGLOMERATOR_* (default
                              algebraicPair: faceAreaPair needs the mesh's
                              face areas)                                   */
} mrg_controls;

/* lduSolverPerformance (initialResidual, finalResidual, nIterations,
 * converged) + GPU extras. */
typedef struct {
    double initial_residual;
    double final_residual;
    int n_iter;            /* Krylov iterations (mixed: total inner)        */
    int converged;
    int singular;
    int status;            /* MRG_OK or MRG_E_*                              */
    int n_outer;           /* mixed: refinement steps                       */
    int fallback;          /* mixed: 1 = the refinement stalled and the solve
                              finished with FP64 Krylov from its best iterate */
    double solve_ms;       /* device time of the solve (CUDA events)        */
} mrg_perf;

/* One coupled interface patch seen from one side: faceCells plus the GGI
 * weights that give each face's neighbour value from the shadow side's
 * cells (monolithicCouplingFvPatchField::initInterfaceMatrixUpdate,
 * monolithicCouplingFvPatchField.C:381-417).  src_ptr == NULL means one
 * source per face with weight 1 (conformal / directMap). */
typedef struct {
    int n_faces;
    const int32_t* face_cells;  /* [n_faces] cells receiving the update     */
    const int32_t* src_ptr;     /* [n_faces+1] CSR into src_cell/src_weight */
    const int32_t* src_cell;    /* shadow cells feeding each weight         */
    const double* src_weight;   /* GGI weights (NULL: all 1)                */
} mrg_iface_desc;

/* ---- library / context ---------------------------------------------- */

/* Text of the last error raised on the calling thread ("" if none). */
const char* mrg_last_error(void);

/* Library version string. */
const char* mrg_version(void);

/* Fill c with foam's defaults (tolerance 1e-6, relTol 0, minIter 0,
 * maxIter 1000, PCG, DIC, FP64, exact order). */
void mrg_controls_default(mrg_controls* c);

/* Create a context on CUDA device `device` with an HBM budget in bytes for
 * all meshes, coefficients and workspaces it allocates (0 = no limit).
 * Replaces the per-process set-up foam does in lduMatrix::solver::New. */
int mrg_ctx_create(int device, size_t hbm_budget_bytes, mrg_ctx** out);
int mrg_ctx_destroy(mrg_ctx* ctx);
/* Bytes currently allocated against the budget. */
int mrg_ctx_mem_used(mrg_ctx* ctx, size_t* bytes);

/* Device-wait watchdog of the context's solves (no counterpart in the
 * reference, whose CPU solver never waits on another thread).  Every wait of
 * a kernel on a value another CTA of the same launch publishes -- the
 * exact-order sweeps' and the factor's dependencies, the persistent
 * iteration kernel's grid barrier, the SpMV's bulk-copy stages -- gives up
 * after wait_cycles SM cycles (0 = the default, 4e9, about 2 s): the kernel
 * sets an error bit and returns, and the solve returns MRG_E_TIMEOUT with
 * the context usable for the next call.  unpublished_chunk >= 0 is a test
 * hook that makes such a wait run out on purpose: the exact-order forward
 * sweep then leaves that chunk of 32 rows (in the plan's level order) of
 * every member unpublished, so the rows that depend on it wait until the
 * budget is spent (-1 = off).  Both apply from the next solve on. */
int mrg_ctx_set_watchdog(mrg_ctx* ctx, long long wait_cycles, int unpublished_chunk);

/* Pinned host memory (for callers that want asynchronous copies). */
int mrg_host_alloc(size_t bytes, void** out);
int mrg_host_free(void* p);

/* ---- mesh addressing (resident) -------------------------------------
 * Replaces foam's lduAddressing (lowerAddr/upperAddr, ownerStartAddr,
 * losortAddr) consumed by lduMatrix::Amul and the DIC/DILU
 * preconditioners, plus the interface patches of
 * monolithicCouplingFvPatchField (monolithicCouplingFvPatchField.C:381-464).
 * The addressing stays on the device until mrg_mesh_destroy. */
int mrg_mesh_upload(mrg_ctx* ctx, int n_cells, int n_faces,
                    const int32_t* lower_addr, const int32_t* upper_addr,
                    int n_iface, const mrg_iface_desc* ifaces,
                    mrg_mesh** out);
int mrg_mesh_destroy(mrg_mesh* mesh);
/* Number of preconditioner sweep levels of the chosen ordering (critical
 * path length of the DIC/DILU triangular solves). */
int mrg_mesh_levels(mrg_mesh* mesh, int ordering, int* n_levels);
/* The faces' area vectors (fvMesh::Sf() of the internal faces, x y z per
 * face, n_faces * 3 values): what GAMG's faceAreaPair agglomerator weights
 * the pairing with (faceAreaPairGAMGAgglomeration: |cmptMultiply(Sf /
 * sqrt(|Sf|), (1, 1.01, 1.02))|).  Only the weights are kept (host side);
 * a cached GAMG hierarchy built from earlier areas is rebuilt at the next
 * GAMG solve. */
int mrg_mesh_set_face_areas(mrg_mesh* mesh, const double* sf);

/* ---- coefficients (per time step) -----------------------------------
 * lduMatrix::diag()/upper()/lower() plus the interfaces' coupleBouCoeffs
 * (Amul, sumA) and coupleIntCoeffs (Tmul; NULL = same as bou), each in
 * interface order (patches in mrg_mesh_upload order, faces within).
 * Host pointers; the _device variant takes device pointers. */
int mrg_coeffs_upload(mrg_mesh* mesh, const double* diag, const double* upper,
                      const double* lower_or_null, const double* iface_bou,
                      const double* iface_int_or_null);
int mrg_coeffs_upload_device(mrg_mesh* mesh, const double* diag,
                             const double* upper, const double* lower_or_null,
                             const double* iface_bou,
                             const double* iface_int_or_null);

/* ---- solve ------------------------------------------------------------
 * lduMatrix::solver::solve(psi, source, cmpt) of foam's PCG / PBiCG /
 * BiCGStab with the DIC / DILU / diagonal / none preconditioners
 * (called from multiRegionSystem.C:150-153 via coupledFvMatrix::solve and
 * :293 via fvMatrix::solve).  b and x_inout are host arrays of n_cells in
 * the caller's numbering; perf may be NULL. */
int mrg_solve(mrg_mesh* mesh, const double* b, double* x_inout,
              const mrg_controls* controls, mrg_perf* perf);
/* Same with device-resident b and x (no host copies). */
int mrg_solve_device(mrg_mesh* mesh, const double* d_b, double* d_x_inout,
                     const mrg_controls* controls, mrg_perf* perf);

/* ---- building blocks (each one of the hot-path kernels) ---------------
 * y = A x (lduMatrix::Amul with interface update) or y = A^T x (Tmul),
 * host arrays in the caller's numbering. */
int mrg_amul(mrg_mesh* mesh, const double* x, double* y, int transpose);
/* foam-normalised residual sum|b - A x| / normFactor of x for b
 * (lduMatrix::solver::normFactor + gSumMag). */
int mrg_residual(mrg_mesh* mesh, const double* b, const double* x,
                 double* residual, double* norm_factor);
/* w = M^-1 r (transpose != 0: M^-T r, DILU's preconditionT) for
 * preconditioner `precond` in ordering `ordering`. */
int mrg_precondition(mrg_mesh* mesh, int precond, int ordering,
                     const double* r, double* w, int transpose);
/* Reciprocal factor diagonal rD of DIC / DILU, caller's numbering. */
int mrg_factor_diag(mrg_mesh* mesh, int precond, int ordering, double* rD);

/* ---- GGI interpolation ----------------------------------------------
 * GGIInterpolation::masterToSlave / slaveToMaster as called from
 * ggiInterfaceToInterfaceMapping::transferFacesZoneToZone
 * (ggiInterfaceToInterfaceMappingTemplates.C:37-77) and
 * regionInterfaceType::interpolateFacesFrom{A,B}
 * (regionInterfaceTypeTemplates.C:35-133): dst[i] = sum_k w_ik src[addr_ik]
 * for n_dst faces, ncomp interleaved components (1 scalar, 3 vector,
 * 4 VectorN<scalar,4>).  Faces with no weights (uncovered) get 0. */
int mrg_ggi_create(mrg_ctx* ctx, int n_dst, int n_src, const int32_t* row_ptr,
                   const int32_t* src_addr, const double* weights,
                   mrg_ggi** out);
int mrg_ggi_destroy(mrg_ggi* ggi);
int mrg_ggi_apply(mrg_ggi* ggi, const double* src, double* dst, int ncomp);
int mrg_ggi_apply_device(mrg_ggi* ggi, const double* d_src, double* d_dst,
                         int ncomp);
/* Measurement hook (no counterpart in the reference): `reps` back-to-back
 * gathers of device arrays on the context's stream, timed with CUDA events;
 * the mean ms per gather in *ms_per_apply. */
int mrg_ggi_time(mrg_ggi* ggi, const double* d_src, double* d_dst, int ncomp,
                 int reps, float* ms_per_apply);
/* GGIInterpolation's weight construction (the interpolator
 * ggiInterfaceToInterfaceMapping.C:62-77 builds with rescale on and SMALL
 * non-overlap tolerances, rebuilt every interpolatorUpdateFrequency steps of
 * a moving interface, regionInterfaceType.C:489-510) on the device, for
 * planar patches: face f of A has vertices a_xy[2*a_ptr[f] .. 2*a_ptr[f+1])
 * (x, y pairs, counter-clockwise, 3 to 32 vertices, a_ptr[0] = 0); likewise
 * B.  weight = |A_i intersect B_j| / |receiving face|, rescaled so that each
 * covered face's weights sum to one; overlaps <= tol * min(|A_i|, |B_j|)
 * are dropped (foam's SMALL: 1e-15).  Returns the two directions as GGI
 * objects: a_from_b (A faces from B values, rows ascending B face) and
 * b_from_a.  MRG_E_INVALID for bad faces or an A face that meets more than
 * 256 B faces' bounding boxes. */
int mrg_ggi_build(mrg_ctx* ctx, int na, const int32_t* a_ptr, const double* a_xy,
                  int nb, const int32_t* b_ptr, const double* b_xy, double tol,
                  mrg_ggi** a_from_b, mrg_ggi** b_from_a);
/* directMapInterfaceToInterfaceMapping (the conformal mapping,
 * directMapInterfaceToInterfaceMapping.C:147-190 and :244-290) on the
 * device: each face of one patch is paired with the first face of the other
 * (in face order) whose centre is within tol -- the reference uses 0.001 x
 * the smallest edge length of the two patches -- and the pairings are
 * returned as one-weight GGI objects, so mrg_ggi_apply performs the
 * directMap transfer to[i] = from[map[i]] (.C:644-) exactly.  Centres are
 * n x (x, y, z).  MRG_E_INVALID when the patches differ in size or a face
 * has no partner ("interfaces are not conformal"). */
int mrg_direct_map_build(mrg_ctx* ctx, int na, const double* a_centres,
                         int nb, const double* b_centres, double tol,
                         mrg_ggi** a_from_b, mrg_ggi** b_from_a);
/* Sizes (any of the pointers may be NULL) and, when row_ptr / src_addr /
 * weights are non-NULL, the GGI's CSR copied to the host (n_dst + 1,
 * nnz, nnz entries). */
int mrg_ggi_get(mrg_ggi* ggi, int* n_dst, int* n_src, int* nnz, int32_t* row_ptr,
                int32_t* src_addr, double* weights);

/* ---- batched solves ----------------------------------------------------
 * Many independent systems (meshes with their current coefficients) solved
 * in lockstep: every iteration is one set of launches over all members, and
 * each member stops when its own convergence test passes.  Replaces a loop
 * of per-region fvMatrix::solve calls (multiRegionSystem.C:193-324,
 * assembleAndSolveEqns) or of independent cases; each member's result is
 * bit-identical to solving it alone.  `ordering` fixes which plan of each
 * mesh the batch uses; the controls' ordering must match. */
int mrg_batch_create(mrg_ctx* ctx, int n_meshes, mrg_mesh* const* meshes,
                     int ordering, mrg_batch** out);
int mrg_batch_destroy(mrg_batch* batch);
/* b[s], x_inout[s]: host vectors of member s (its mesh's numbering);
 * perfs: n_meshes records or NULL. */
int mrg_batch_solve(mrg_batch* batch, const double* const* b,
                    double* const* x_inout, const mrg_controls* controls,
                    mrg_perf* perfs);
int mrg_batch_solve_device(mrg_batch* batch, const double* const* d_b,
                           double* const* d_x_inout,
                           const mrg_controls* controls, mrg_perf* perfs);

/* ---- partitioned Dirichlet-Neumann coupling ----------------------------
 * One interface coupled by the partitioned (DN) method, the reference's
 * alternative to the monolithic solve: region A carries the jump
 * (Dirichlet) patch, region B the flux (Neumann) patch.  The patch states,
 * the relaxation history and the Aitken factors stay on the device.
 * Replaces, per coupling iteration, genericRegionCoupledJumpFvPatchField::
 * updateCoeffs (.C:164-217), genericRegionCoupledFluxFvPatchField::
 * updateCoeffs (.C:172-239), their rawResidual/normResidual (Jump .C:244-332,
 * Flux .C:241-409), fixedRelaxation / aitkenRelaxation::relax
 * (fixedRelaxation.C:76-101, aitkenRelaxation.C:74-100,
 * aitkenRelaxationTemplates.C:105-165) and dnaControl::criteriaSatisfied
 * (dnaControl.C:582-635) for a scalar field with
 * regionCoupledTemperatureJump (value jump (K-1) * nbr) and
 * regionCoupledHeatFlux (flux jump 0). */
typedef struct mrg_dn mrg_dn;
typedef struct {
    int n_cells;                 /* cells of the patch's region               */
    int n_faces;                 /* faces of the patch                        */
    const int32_t* face_cells;   /* [n_faces] faceCells                       */
    const double* delta_coeffs;  /* [n_faces] 1 / cell-to-face distance       */
    const double* k;             /* [n_faces] diffusivity at the face         */
    const double* area;          /* [n_faces] face area |Sf|                  */
    const int32_t* src_ptr;      /* [n_faces+1] this patch's faces from the   */
    const int32_t* src_face;     /*   other patch's faces: GGI CSR (or        */
    const double* src_weight;    /*   directMap: one weight 1 per face)       */
} mrg_dn_patch;
typedef struct {
    double K;          /* regionCoupledTemperatureJump: value = K * nbr      */
    double flux_jump;  /* regionCoupledHeatFlux: 0                           */
    double relax;      /* fixed factor, or Aitken's / IQN-ILS's initial one  */
    int relax_model;   /* 0 fixedRelaxation, 1 aitkenRelaxation, 2 IQNILS
                          (IQNILS.C, IQNILSTemplates.C:44-133; at most 32
                          modes per side, the oldest dropped first)          */
    int coupling_reuse; /* IQNILS couplingReuse: time steps whose modes are
                          kept (0: this time step's only)                    */
} mrg_dn_config;
int mrg_dn_create(mrg_ctx* ctx, const mrg_dn_patch* a, const mrg_dn_patch* b,
                  const mrg_dn_config* config, mrg_dn** out);
int mrg_dn_destroy(mrg_dn* dn);
/* The flux patch's own acceleration model (its accType / relax /
 * couplingReuse entries; genericRegionCoupledFluxFvPatchField.C:86-96): by
 * default B uses A's model and factor; a flux patch without accType in its
 * dictionary is fixedRelaxation with relax 1 (newAccelerationModel.C:51-65),
 * the tutorials' set-up.  Call before mrg_dn_set_state. */
int mrg_dn_set_flux_relaxation(mrg_dn* dn, int relax_model, double relax, int coupling_reuse);
/* Initial patch value on A and gradient on B (host arrays); resets the
 * relaxation history. */
int mrg_dn_set_state(mrg_dn* dn, const double* value_a, const double* grad_b);
/* A new time step restarts the relaxation's corrector count. */
int mrg_dn_new_time_step(mrg_dn* dn);
/* Jump update of A from region B's cell field (device), and flux update of
 * B from region A's cell field (device). */
int mrg_dn_update_jump(mrg_dn* dn, const double* d_t_b);
int mrg_dn_update_flux(mrg_dn* dn, const double* d_t_a);
/* d_b = d_b0 + the patch's source terms for region `side` (0: A, Dirichlet
 * k|Sf|deltaCoeffs value; 1: B, Neumann k|Sf| gradient).  The matching
 * Dirichlet diagonal term k|Sf|deltaCoeffs belongs to A's matrix. */
int mrg_dn_rhs(mrg_dn* dn, int side, const double* d_b0, double* d_b);
/* Normalised jump (A) and flux (B) residuals of the current state. */
int mrg_dn_residuals(mrg_dn* dn, const double* d_t_a, const double* d_t_b,
                     double* jump_res, double* flux_res);
/* Host copies of the patch states and the two Aitken factors (any may be
 * NULL). */
int mrg_dn_get_state(mrg_dn* dn, double* value_a, double* grad_b, double* aitken);
/* dnaControl::criteriaSatisfied: 0 on the first coupling iteration, else 1
 * when both residuals are within their limits. */
int mrg_dn_criteria(int corr, double jump_res, double flux_res, double max_jump_res,
                    double max_flux_res);

/* ---- monolithic interface coefficients ---------------------------------
 * The per-assembly interface terms of the monolithic conjugate-heat-transfer
 * boundary conditions, for both sides of a regionCouple interface:
 * monolithicThermalDiffusivityFvPatchScalarField::calcThermalDiffusivity /
 * calcTemperature (monolithicThermalDiffusivityFvPatchScalarField.C:
 * 167-394) and monolithicTemperatureFvPatchScalarField::source /
 * manipulateMatrix (monolithicTemperatureFvPatchScalarField.C:205-244).
 * A patch: faceCells into its region's cells, the coupled patch's linear
 * weights w (0 < w < 1), magLongDelta, deltaCoeffs and |Sf|, and the GGI
 * weights that interpolate the other side's face values onto its faces
 * (src_ptr[n_faces + 1], src_face, src_weight; rescaled, uncovered faces
 * empty, as the regionCouplePatch's interpolator gives them). */
typedef struct mrg_mono mrg_mono;
typedef struct {
    int n_cells, n_faces;
    const int32_t* face_cells;
    const double* weights;
    const double* mag_long_delta;
    const double* delta_coeffs;
    const double* mag_sf;
    const int32_t* src_ptr;
    const int32_t* src_face;
    const double* src_weight;
} mrg_mono_patch;
int mrg_mono_create(mrg_ctx* ctx, const mrg_mono_patch* side_a, const mrg_mono_patch* side_b,
                    mrg_mono** out);
int mrg_mono_destroy(mrg_mono* mono);
/* Interface diffusivity k and wall temperature Tw on the faces of `side`
 * (0 = A, 1 = B), device arrays: T_own / T_nbr are the two regions' cell
 * temperatures, f_own / f_nbr the diffusivities on the two patches
 * (monolithicBase::forig), Qr_own / Qr_nbr the radiative fluxes on the two
 * patches, or NULL for a side without radiation. */
int mrg_mono_update(mrg_mono* mono, int side, const double* d_T_own, const double* d_T_nbr,
                    const double* d_f_own, const double* d_f_nbr, const double* d_Qr_own,
                    const double* d_Qr_nbr, double* d_k, double* d_Tw);
/* The temperature patch's source s = kOwn (Tw - Tc) - k deltaCoeffs
 * (Tc_nei - Tc) added to the region's right-hand side, b[faceCells] +=
 * s |Sf| (device arrays; k and Tw as mrg_mono_update returned them). */
int mrg_mono_source(mrg_mono* mono, int side, const double* d_T_own, const double* d_T_nbr,
                    const double* d_Tw, const double* d_k, const double* d_f_own, double* d_b);

/* ---- autotuner ---------------------------------------------------------
 * No counterpart in the reference.  Times the Krylov loop of a mesh or batch
 * on its current coefficients under each candidate launch shape and keeps
 * the fastest for later solves with the same ordering: the iteration mode
 * (a captured graph of separate launches, or one persistent cooperative
 * kernel with grid barriers), the iterations per launch, the number of
 * level-sweep chunks per CTA and, for PCG's loop, the Amul kernel -- its
 * block shape and the rows a warp takes per step.  A launch shape never
 * changes a result bit.  b and x as for a solve (device pointers); x is not
 * modified. */
typedef struct {
    int mode;                  /* 0: graph of launches, 1: persistent kernel */
    int iters_per_launch;
    int sweep_chunks_per_cta;  /* colour ordering only                       */
    int spmv_kernel;           /* 1 per-warp staged, 2 / 3 streamed; 0: not
                                  tuned (the default kernel)               */
    int spmv_block_threads;    /* 256, or 288 with a producer warp (0: default) */
    int spmv_rows_per_warp_step; /* 32 or 64 (0: default)                    */
    int candidates;            /* shapes timed                               */
    int reserved;
    double us_per_iter;        /* of the chosen shape                        */
} mrg_tuning;
int mrg_mesh_tune(mrg_mesh* mesh, const double* d_b, const double* d_x,
                  const mrg_controls* controls, mrg_tuning* out);
int mrg_batch_tune(mrg_batch* batch, const double* const* d_b,
                   const double* const* d_x, const mrg_controls* controls,
                   mrg_tuning* out);

/* ---- serving: continuous batching of solve requests -------------------
 * No counterpart in the reference, which solves each region's equation in
 * turn inside its time loop (multiRegionSystem.C:193-324).  A server keeps
 * the meshes' addressing resident and takes requests "solve this mesh with
 * these new coefficients, b and x0" from any host thread; its own thread
 * admits them into a running batch (one for PCG requests, one for PBiCG)
 * between iteration-graph launches, while batch slots and the HBM budget
 * on in-flight working sets allow, and completes each when it converges.
 * A mesh has at most one request in flight; its next one waits.  Results
 * are bit-identical to mrg_solve with the same controls.  While a server
 * runs, only mrg_server_* calls may use its context; destroy it before its
 * meshes and context. */
typedef struct {
    uint64_t submitted, completed;
    int running, queued, peak_running, reserved;
    size_t inflight_bytes, peak_inflight_bytes;
} mrg_server_stats;
/* sym_controls: symmetric requests (PCG or BiCGStab, with preconditioner /
 * precision / ordering / tolerance); asym_controls: asymmetric requests
 * (PBiCG or BiCGStab), or NULL to refuse them.  hbm_budget: bytes
 * of in-flight working sets (0 = only the context's budget); max_active:
 * members per running batch (0 = 256). */
int mrg_server_create(mrg_ctx* ctx, const mrg_controls* sym_controls,
                      const mrg_controls* asym_controls, size_t hbm_budget,
                      int max_active, mrg_server** out);
int mrg_server_destroy(mrg_server* server);
/* Queue one solve of `mesh` (asym != 0: PBiCG family).  The host arrays
 * (mrg_coeffs_upload's, plus b, x0 and x_out) must stay valid and unchanged
 * until the request completes; pinned memory (mrg_host_alloc) copies
 * fastest.  MRG_E_BUSY when the queue is full. */
int mrg_server_submit(mrg_server* server, mrg_mesh* mesh, int asym,
                      const double* diag, const double* upper,
                      const double* lower_or_null, const double* iface_bou,
                      const double* iface_int_or_null, const double* b,
                      const double* x0, double* x_out, uint64_t* request_id);
/* *done = 1 once the request finished (x_out written, perf filled); the
 * record is then released and the return value is the request's status.
 * latency_ms: submit to completion. */
int mrg_server_poll(mrg_server* server, uint64_t request_id, int* done,
                    mrg_perf* perf, double* latency_ms);
/* As poll, blocking up to timeout_ms (< 0: no limit). */
int mrg_server_wait(mrg_server* server, uint64_t request_id, double timeout_ms,
                    int* done, mrg_perf* perf, double* latency_ms);
int mrg_server_get_stats(mrg_server* server, mrg_server_stats* out);

/* ---- device buffers, timing and diagnostics --------------------------
 * No counterpart in the reference (foam-extend times solves with
 * cpuTimeIncrement, multiRegionSystem.C:546-650).  They let a caller keep
 * inputs resident in HBM and time work on the context's own stream. */
int mrg_dev_alloc(mrg_ctx* ctx, size_t bytes, void** out);
int mrg_dev_free(mrg_ctx* ctx, void* p);
/* kind: 0 host->device, 1 device->host, 2 device->device (ctx stream, then
 * synchronised). */
int mrg_dev_copy(mrg_ctx* ctx, void* dst, const void* src, size_t bytes, int kind);
/* Record CUDA event `slot` (0..63) on the context's stream; elapsed time in
 * ms between two recorded slots (synchronises on the later one). */
int mrg_event_record(mrg_ctx* ctx, int slot);
int mrg_event_elapsed(mrg_ctx* ctx, int slot_a, int slot_b, float* ms);
/* Total kernels this library has launched in this process (graph nodes
 * counted per graph launch). */
int mrg_kernel_launches(uint64_t* count);
/* Time `reps` back-to-back launches of one hot-path kernel on the mesh's
 * current state (after a solve with the same controls): kernel 0 = Amul +
 * (q,p) reduction of the Krylov loop in `precision`, 1 = one preconditioner
 * application (forward + backward sweep).  Returns the mean ms per launch
 * measured with CUDA events on the context's stream. */
int mrg_time_kernel(mrg_mesh* mesh, const mrg_controls* controls, int kernel,
                    int reps, float* ms_per_launch);

/* ---- block-coupled systems (fvBlockMatrix<vectorN>) --------------------
 * Replaces the BlockLduSolver<Type>::New(...)->solve entry of foam-extend's
 * fvBlockMatrix::solve (filesToReplace/fvBlockMatrix.C:1360-1388; the
 * pressure-velocity coupled region's BlockLduMatrix<vector4>,
 * pUCoupledIcoFluid.C:592-617) by a scalar LDU system of bs * n_cells cells
 * that mrg_mesh_upload / mrg_coeffs_upload / mrg_solve take as they are:
 * cell c's component a is row bs c + a.  A block face f = (l, u) becomes
 * the bs^2 faces (bs l + a, bs u + b) with upper U_f[a][b] and lower
 * L_f[b][a]; a diagonal block D_c gives the diagonal D_c[a][a] and, for
 * a < b, the face (bs c + a, bs c + b) with upper D_c[a][b] and lower
 * D_c[b][a].  Faces come out in upper-triangular order (owner row, then
 * neighbour).  Any scalar preconditioner applies to the expansion, and
 * MRG_PRECOND_BLOCK (after mrg_mesh_set_blocks) works on its blocks.
 * mrg_block_addressing and mrg_block_coeffs are host-only (no GPU needed).
 *
 * mrg_mesh_set_blocks: declare a mesh uploaded from mrg_block_addressing's
 *   output the bs-expansion of the block mesh (n_cells, n_faces, lower /
 *   upper; checked), so MRG_PRECOND_BLOCK can factor its bs x bs blocks
 *   (gathered from the scalar coefficients whenever they change).  bs 1..4;
 *   the mesh has no interfaces.
 * mrg_block_addressing: *n_faces_out = bs^2 n_faces + bs (bs - 1) / 2
 *   n_cells; s_lower / s_upper [that many] (either NULL: the count only).
 * mrg_block_coeffs: diag [n_cells bs bs], upper and lower [n_faces bs bs]
 *   (row-major blocks; lower NULL: every lower block is its upper block
 *   transposed) -> s_diag [bs n_cells], s_upper, s_lower [n_faces_out], in
 *   mrg_block_addressing's face order.  bs is 1..8; the block addressing
 *   follows mrg_mesh_upload's rules (lower < upper, upper-triangular face
 *   order); MRG_E_INVALID otherwise or for bad sizes. */
int mrg_block_addressing(int n_cells, int n_faces, const int32_t* lower_addr,
                         const int32_t* upper_addr, int bs, int* n_faces_out,
                         int32_t* s_lower, int32_t* s_upper);
int mrg_mesh_set_blocks(mrg_mesh* mesh, int bs, int n_cells, int n_faces,
                        const int32_t* lower_addr, const int32_t* upper_addr);
int mrg_block_coeffs(int n_cells, int n_faces, const int32_t* lower_addr,
                     const int32_t* upper_addr, int bs, const double* diag,
                     const double* upper, const double* lower_or_null,
                     double* s_diag, double* s_upper, double* s_lower);

/* ---- residual without device allocation -------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory where they need a residual: code inside a host application whose
 * own allocator already holds the GPU's memory (a caching pool, or an MPS
 * client under a hard memory limit), or monitoring code beside asynchronous
 * solves, where cudaMalloc / cudaFree would synchronise the device.
 *
 * The same residual and norm factor as mrg_residual, for a matrix without
 * interfaces held in the caller's device arrays in foam's lduAddressing:
 * lowerAddr, upperAddr [n_faces]; ownerStartAddr, losortStartAddr
 * [n_cells + 1]; losortAddr [n_faces]; diag [n_cells], upper, lower
 * [n_faces] (d_lower NULL: symmetric); b, x [n_cells].  Runs on `stream` (a
 * cudaStream_t of the current device, NULL = the default stream) and
 * returns after it; residual and norm_factor are host pointers (either may
 * be NULL).  It allocates nothing: its reduction scratch is a fixed
 * 393,472-byte device array inside the library, held on every GPU that
 * loads it until the process exits, so n_cells is limited to 16,777,216
 * (larger: MRG_E_INVALID).  Every call looks up that array's address in the
 * current context (so a device reset or another current context between
 * calls is handled); the first call on a device also loads the library's
 * device code there: make it before any stream capture.  Every call shares
 * the array: calls that overlap on the GPU (other host threads, or streams
 * that do not wait for each other) race and give undefined results.  The
 * faces must be in foam's upper-triangular order (lowerAddr < upperAddr,
 * each cell's ownerStartAddr neighbours ascending, its losortAddr faces
 * ascending), which gives A x foam's Amul summation order; addressing that
 * breaks the order, or points outside its arrays (not read), returns
 * MRG_E_INVALID. */
int mrg_residual_noalloc(int n_cells, int n_faces,
                         const int32_t* d_lower_addr, const int32_t* d_upper_addr,
                         const int32_t* d_owner_start, const int32_t* d_losort,
                         const int32_t* d_losort_start, const double* d_diag,
                         const double* d_upper, const double* d_lower,
                         const double* d_b, const double* d_x, void* stream,
                         double* residual, double* norm_factor);

#ifdef __cplusplus
}
#endif

#endif /* MRGPU_H */
