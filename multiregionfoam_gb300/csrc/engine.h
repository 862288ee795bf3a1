// engine.h -- host-side objects behind the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "dev.h"
#include "plan.h"
#include "kernels.h"
#include "blockpc.h"

namespace mrg {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void cuda_check(cudaError_t e, const char* what);
#define MRG_CUDA(x) ::mrg::cuda_check((x), #x)

struct Ctx {
    int device = 0;
    int nsm = 0;
    cudaStream_t st = nullptr;
    size_t budget = 0, used = 0;
    std::map<void*, size_t> allocs;
    cudaEvent_t events[64] = {};
    double* stage[3] = {nullptr, nullptr, nullptr};  // host-pointer entry points
    size_t stage_cap = 0;
    // device-wait watchdog of the solves (mrg_ctx_set_watchdog): budget in SM
    // cycles (0: the kernels' default) and the test hook's chunk + 1 (0: off)
    long long wait_cycles = 0;
    int unpublished1 = 0;
    void* alloc(size_t bytes);
    void release(void* p);
    ~Ctx();
};

struct Controls {
    double tol = 1e-6, rel_tol = 0.0;
    int min_iter = 0, max_iter = 1000;
    int solver = 0, pc = 2, precision = 0, ordering = 0;
    double inner_rel_tol = 1e-5;
    int inner_max_iter = 0, max_outer = 50, k_launch = 16;
    int n_sweeps = 1;   // smoothSolver: sweeps per residual check
    int smoother = 0;   // smoothSolver: MRG_SMOOTHER_*
    int gamg_coarsest = 10, gamg_post = 2, gamg_finest = 2;   // GAMG: nCellsInCoarsestLevel, nPostSweeps,
                                                              // nFinestSweeps
    int gamg_max_post = 4, gamg_post_mult = 1;                // GAMG: maxPostSweeps, postSweepsLevelMultiplier
    int gamg_scale = 1, gamg_agglomerator = 0;                // GAMG: scaleCorrection, MRG_AGGLOMERATOR_*
};

struct Perf {
    double res0 = 0, res = 0;
    int iters = 0, converged = 0, singular = 0, status = 0, outer = 0;
    int fallback = 0;   // mixed: finished with FP64 Krylov after the refinement stalled
    double ms = 0;
};

struct PlanState;

// Launch shapes of a batch's Krylov loop, chosen by tune_batch (or the
// defaults).  None of them changes a result bit: they decide how the same
// kernels are launched, never what they compute.
struct Tuning {
    int tuned = 0;
    int mode = 0;        // 0: graph of separate launches, 1: persistent cooperative kernel
    int k = 0;           // iterations per launch (0: the controls' iters_per_launch)
    int sweep_div = 8;   // level-sweep grid: one CTA per sweep_div chunks of the widest level
    int spmv = 0;        // Amul kernel (launch_rows' spmv): 0 default, 1 per-warp staged, 2 / 3 streamed
                         // with 32 / 64 rows a warp step
    double us_per_iter = 0.0;
    int candidates = 0;
};

// A device-resident batch: the Batch descriptor, the system array, the tile
// table, the per-level sweep work list and the control block.  Captured
// iteration graphs refer only to the descriptor's address.
struct BatchHost {
    Ctx* ctx = nullptr;
    Batch h{};
    Batch* d = nullptr;
    Ctl* d_ctl = nullptr;
    SysDev* d_sys = nullptr;
    int2* d_tiles = nullptr;
    int2* d_segs = nullptr;
    int2* d_items = nullptr;
    int* d_item_off = nullptr;
    int2* d_sf = nullptr;      // sync-free sweep work list (several systems)
    Scal* d_scal = nullptr;    // gathered member states (serving)
    size_t cap_sys = 0, cap_tiles = 0, cap_segs = 0, cap_items = 0, cap_off = 0, cap_scal = 0, cap_sf = 0;
    int widest_level = 1;      // items of the widest sweep level (grid sizing)
    std::vector<PlanState*> members;
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        long long nodes = 0;   // kernels per replay (for the launch counter)
    };
    std::map<std::string, Graph> graphs;
    Tuning tune;
    // Compacted sub-batch: once most members of a long batched loop have
    // converged, the rest iterate in a batch of their own (their states and
    // results are per system, so nothing changes but the work skipped).
    std::unique_ptr<BatchHost> compact;
    void init(Ctx* c);
    // (Re)build the arrays for these systems; the order fixes the tile table.
    void set(const std::vector<PlanState*>& systems);
    // Re-upload the system array (after a member's SysDev changed).
    void sync_sys();
    ~BatchHost();
};

// Device copy of one plan + coefficient views + workspaces for one ordering.
struct PlanState {
    Ctx* ctx = nullptr;
    PlanHost host;  // large host arrays are released after upload
    int32_t *perm = nullptr, *a_sptr = nullptr, *a_col = nullptr, *a_src = nullptr;
    uint16_t* a_col16 = nullptr;
    int32_t* a_cbase = nullptr;
    int32_t *chunk_start = nullptr, *lvl_chunk = nullptr;
    int32_t *f_sptr = nullptr, *f_col = nullptr, *f_src = nullptr;
    int32_t *b_sptr = nullptr, *b_col = nullptr, *b_src = nullptr;
    int32_t *g_ptr = nullptr, *g_src = nullptr;
    double* g_w = nullptr;
    float* g_w32 = nullptr;
    int32_t *pt_ptr = nullptr, *part_rows = nullptr, *part_step = nullptr, *f_row = nullptr;
    int32_t *f_loc = nullptr, *b_loc = nullptr, *b_row = nullptr;
    SysDev sys{};           // host mirror
    SysDev* d_sys = nullptr;
    int ntiles = 0;
    int bs_blocks = 0;        // PC_BLOCK: the mesh's block size
    size_t nnz = 0, fnz = 0, bnz = 0;
    bool have32 = false, haveT = false, haveT32 = false;
    uint64_t scattered = 0;   // coefficient version scattered into the views
    uint64_t factored = 0;    // coefficient version factored
    int factored_pc = -1;
    bool factored32 = false;
    BatchHost single;         // this system alone
    ~PlanState();
    void sync_sys();          // copy host mirror to device
};

struct Gamg;

struct Mesh {
    Ctx* ctx = nullptr;
    int n = 0, nf = 0, ni = 0;
    std::vector<int32_t> lower, upper;
    IfaceHost ifc;
    double *raw_diag = nullptr, *raw_upper = nullptr, *raw_lower = nullptr;
    double *raw_ibou = nullptr, *raw_iint = nullptr;
    bool sym = true, has_int = false, have_coeffs = false;
    uint64_t version = 0;
    std::unique_ptr<PlanState> plans[2];
    std::unique_ptr<Gamg> gamg;   // GAMG hierarchy (built at the first GAMG solve)
    int part_target = kPartTarget;  // cells a part of the exact plan aims at (owner-computes sweeps)
    std::unique_ptr<BlockHost> blocks;      // block structure (mrg_mesh_set_blocks), for PC_BLOCK
    std::unique_ptr<BlockView> bviews[2];   // its views per ordering
    std::vector<double> agglom_w;   // faceAreaPair weights of the faces (mrg_mesh_set_face_areas)
    uint64_t agglom_version = 0;    // bumped by every mrg_mesh_set_face_areas
    PlanState& plan(int ordering);
    ~Mesh();
};

struct Ggi {
    Ctx* ctx = nullptr;
    int n_dst = 0, n_src = 0;
    int32_t *ptr = nullptr, *addr = nullptr;
    double* w = nullptr;
    double *d_src = nullptr, *d_dst = nullptr;
    int cap_comp = 0;
    ~Ggi();
};

// Make views, FP32 copies, transpose vectors and factors of every member
// current for these controls (one scatter and one factor launch per batch).
void prepare_batch(BatchHost& bh, const std::vector<Mesh*>& meshes, const Controls& c);
// Solve every member of the batch; each member's SysDev in_b/in_x/out_x point
// at its caller-numbered device vectors.  Returns one Perf per member.
std::vector<Perf> solve_batch(BatchHost& bh, const Controls& c);

// Solve record of one member from its scalar state.
Perf perf_of(const Scal& q, int precision);

// Serving steps (the stages of solve_batch, for a batch whose membership
// changes between them): begin = permute in + initial residual (+ first
// refinement step when mixed); iterate = one launch of the captured K-iteration
// graph; outer = correction + FP64 residual + next inner start (mixed);
// finish = permute the solution out; recount = recompute the control block's
// active counts after a membership change; status = gather every member's
// scalar state to the host (checks the device error bits).
void batch_begin(BatchHost& bh, const Controls& c);
void batch_iterate(BatchHost& bh, const Controls& c, int prec = -1);
// Mixed members whose refinement stalled (fallback requested): FP64 residual
// of the best iterate and the start of an FP64 Krylov loop.
// The FP64 continuation of mixed solves whose refinement stalled: the same
// controls with PBiCG in place of BiCGStab (FP64 BiCGStab can break down on
// convection-dominated systems where PBiCG -- foam's plain method for
// asymmetric matrices -- converges).
Controls fallback_controls(const Controls& cfg);
void batch_fallback(BatchHost& bh, const Controls& c);
void batch_outer(BatchHost& bh, const Controls& c);
void batch_finish(BatchHost& bh);
void batch_recount(BatchHost& bh);
// The batch's control block, read after the stream drains (throws on a
// device-side wait timeout).
const Ctl& batch_poll(BatchHost& bh);
void batch_status(BatchHost& bh, std::vector<Scal>& out);

// Autotuner: time the Krylov loop of the prepared batch (members' in_b/in_x
// set) under each candidate launch shape -- iteration mode, iterations per
// launch, level-sweep grid -- and keep the fastest in bh.tune.  The members'
// outputs are not written.
Tuning tune_batch(BatchHost& bh, const Controls& c);

// Copy coefficients into a mesh's raw device arrays (caller numbering) and
// bump its version; `sync` waits for the copies.
void upload_coeffs(Mesh& m, const double* diag, const double* upper, const double* lower, const double* ibou,
                   const double* iint, cudaMemcpyKind kind, bool sync);

// Single-system conveniences (batch of one).
PlanState& prepare(Mesh& m, const Controls& c);
// Owner-computes exact sweeps of a batch: parts (0: the ticketed kernel) and
// cells a part.
// gs: for Gauss-Seidel sweeps (else DIC / DILU sweeps).
void part_choice(const BatchHost& bh, int& parts, int& cells, bool gs = false);
Perf solve_device(Mesh& m, const double* d_b, double* d_x, const Controls& c);

void amul_device(Mesh& m, const double* d_x, double* d_y, int transpose);
void residual_device(Mesh& m, const double* d_b, const double* d_x, double* res, double* nfac);
void precondition_device(Mesh& m, int pc, int ordering, const double* d_r, double* d_w, int transpose);
void factor_diag_device(Mesh& m, int pc, int ordering, double* d_rD);
// Mean ms per launch of one hot-path kernel (0: Amul + (q,p); 1: one
// preconditioner application) on the current state.
float time_kernel(Mesh& m, const Controls& c, int kernel, int reps);

}  // namespace mrg
