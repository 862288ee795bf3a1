// gpuLduSolvers.C -- foam-extend lduMatrix::solver adapters for libmrgpu.
//
// Registers six solver names in foam's run-time selection tables so that an
// fvSolution entry swaps the GPU solve in with no other change:
//
//   gpuPCG            symMatrix   FP64 PCG, preconditioner DIC|FDIC|diagonal|none
//   gpuPBiCG          asymMatrix  FP64 PBiCG, preconditioner DILU|diagonal|none
//   gpuBiCGStab       both        FP64 BiCGStab, preconditioner DIC|DILU|diagonal|none
//   gpuMixedPCG       symMatrix   FP32 PCG inside FP64 iterative refinement
//   gpuMixedPBiCG     asymMatrix  FP32 PBiCG inside FP64 iterative refinement
//   gpuMixedBiCGStab  both        FP32 BiCGStab inside FP64 iterative refinement
//   gpuGAMG           both        FP64 GAMG, GaussSeidel smoothing; nCellsInCoarsestLevel,
//                                 nPostSweeps, nFinestSweeps
//   gpuBICCG          both        FP64 PBiCG + DILU (foam's BICCG)
//   gpuSmoothSolver   both        FP64 smoothSolver; smoother GaussSeidel | DIC | DILU |
//                                 DICGaussSeidel | DILUGaussSeidel; nSweeps
//
// Each adapter replaces lduMatrix::solver::solve(psi, source, cmpt) (the call
// fvMatrix::solve makes at multiRegionSystem.C:293, and coupledFvMatrix's at
// multiRegionSystem.C:150-153): the matrix addressing (lduAddressing) is
// uploaded once and kept resident, the coefficients (diag/upper/lower and the
// interfaces' coupleBouCoeffs/coupleIntCoeffs, as assembled by
// monolithicCouplingFvPatchField) are uploaded per solve, and the returned
// performance record has foam's meaning (initial/final residual normalised
// by foam's normFactor, iteration count, converged flag).  Errors from the
// library become FatalError, as foam's own solvers do.
//
// Extra (optional) controls: "gpuOrdering" exact|colour, "innerRelTol",
// "hbmBudget" (bytes, per process), "gpuDevice".
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>

#include "lduMatrix.H"
#include "mrgpu.h"

namespace Foam {

namespace {

struct GpuState {
    mrg_ctx* ctx = nullptr;
    // resident addressing, keyed by the lduAddressing object
    std::map<const void*, mrg_mesh*> meshes;
    std::mutex lock;
    ~GpuState()
    {
        for (auto& kv : meshes) mrg_mesh_destroy(kv.second);
        if (ctx) mrg_ctx_destroy(ctx);
    }
};

GpuState& state()
{
    static GpuState s;
    return s;
}

void check(int rc, const char* what)
{
    if (rc != MRG_OK)
        throw FatalError(std::string("gpu solver: ") + what + " failed: " + mrg_last_error());
}

// foam-extend's "Cholesky" (the tutorials' coupled-solve preconditioner) is
// the incomplete Cholesky factorisation without fill-in: DIC on a symmetric
// matrix, its LU analogue DILU on an asymmetric one.
int precondCode(const word& p, bool sym)
{
    if (p == "DIC" || p == "FDIC") return MRG_PRECOND_DIC;
    if (p == "DILU") return MRG_PRECOND_DILU;
    if (p == "Cholesky") return sym ? MRG_PRECOND_DIC : MRG_PRECOND_DILU;
    if (p == "diagonal") return MRG_PRECOND_DIAGONAL;
    if (p == "none") return MRG_PRECOND_NONE;
    throw FatalError("gpu solver: unsupported preconditioner " + p + (sym ? " (symmetric)" : " (asymmetric)"));
}

}  // namespace

class gpuLduSolver : public lduMatrix::solver {
public:
    gpuLduSolver(const word& fieldName, const lduMatrix& matrix, const FieldField& bou, const FieldField& intc,
                 const lduInterfaceFieldPtrsList& ifs, const dictionary& controls, int solverKind, int precision)
        : lduMatrix::solver(fieldName, matrix, bou, intc, ifs, controls), solverKind_(solverKind),
          precision_(precision)
    {
    }

    lduMatrix::solverPerformance solve(scalarField& psi, const scalarField& source,
                                       const direction) const override
    {
        GpuState& S = state();
        std::lock_guard<std::mutex> g(S.lock);
        if (!S.ctx) {
            const int dev = (int)controls_.lookupOrDefault("gpuDevice", 0);
            const size_t budget = (size_t)controls_.lookupOrDefault("hbmBudget", 0);
            check(mrg_ctx_create(dev, budget, &S.ctx), "mrg_ctx_create");
        }
        const lduAddressing& a = matrix_.lduAddr();
        const label n = a.size(), nf = (label)a.lowerAddr().size();
        if ((label)psi.size() != n || (label)source.size() != n)
            throw FatalError("gpu solver: psi/source size does not match the matrix");
        mrg_mesh*& mesh = S.meshes[&a];
        // flatten the interfaces (patch order, face order)
        std::vector<mrg_iface_desc> desc;
        scalarField bouFlat, intFlat;
        bool intDiffers = false;
        for (size_t p = 0; p < interfaces_.size(); ++p) {
            const lduInterfaceField* f = interfaces_[p];
            if (!f) continue;
            mrg_iface_desc d;
            d.n_faces = (int)f->faceCells.size();
            d.face_cells = f->faceCells.data();
            d.src_ptr = f->srcPtr.empty() ? nullptr : f->srcPtr.data();
            d.src_cell = f->srcCells.data();
            d.src_weight = f->srcWeights.empty() ? nullptr : f->srcWeights.data();
            desc.push_back(d);
            const scalarField& b = coupleBouCoeffs_[p];
            const scalarField& i = coupleIntCoeffs_.size() > p ? coupleIntCoeffs_[p] : b;
            bouFlat.insert(bouFlat.end(), b.begin(), b.end());
            intFlat.insert(intFlat.end(), i.begin(), i.end());
            if (i != b) intDiffers = true;
        }
        if (!mesh) {
            check(mrg_mesh_upload(S.ctx, n, nf, a.lowerAddr().data(), a.upperAddr().data(), (int)desc.size(),
                                  desc.empty() ? nullptr : desc.data(), &mesh),
                  "mrg_mesh_upload");
        }
        check(mrg_coeffs_upload(mesh, matrix_.diag().data(), matrix_.upper().data(),
                                matrix_.hasLower() ? matrix_.lower().data() : nullptr,
                                bouFlat.empty() ? nullptr : bouFlat.data(),
                                intDiffers ? intFlat.data() : nullptr),
              "mrg_coeffs_upload");
        mrg_controls c;
        mrg_controls_default(&c);
        c.tolerance = tolerance_;
        c.rel_tol = relTol_;
        c.min_iter = minIter_;
        c.max_iter = maxIter_;
        c.solver = solverKind_;
        if (solverKind_ == MRG_SOLVER_GAMG) {
            // GAMG's own words; the agglomeration is pairwise on the
            // coefficients whatever agglomerator names, and it is cached
            if (controls_.lookupWord("smoother", "GaussSeidel") != "GaussSeidel")
                throw FatalError("gpuGAMG: unsupported smoother " + controls_.lookupWord("smoother"));
            c.smoother = MRG_SMOOTHER_GAUSS_SEIDEL;
            c.gamg_coarsest_cells = (int)controls_.lookupOrDefault("nCellsInCoarsestLevel", 10.0);
            c.gamg_post_sweeps = (int)controls_.lookupOrDefault("nPostSweeps", 2.0);
            c.gamg_finest_sweeps = (int)controls_.lookupOrDefault("nFinestSweeps", 2.0);
        } else if (solverKind_ == MRG_SOLVER_SMOOTH) {
            // smoothSolver's own words: smoother and nSweeps
            const word sm = controls_.lookupWord("smoother", "GaussSeidel");
            if (sm == "GaussSeidel") c.smoother = MRG_SMOOTHER_GAUSS_SEIDEL;
            else if (sm == "DIC") c.smoother = MRG_SMOOTHER_DIC;
            else if (sm == "DILU") c.smoother = MRG_SMOOTHER_DILU;
            else if (sm == "DICGaussSeidel") c.smoother = MRG_SMOOTHER_DIC_GAUSS_SEIDEL;
            else if (sm == "DILUGaussSeidel") c.smoother = MRG_SMOOTHER_DILU_GAUSS_SEIDEL;
            else throw FatalError("gpuSmoothSolver: unsupported smoother " + sm);
            c.n_sweeps = (int)controls_.lookupOrDefault("nSweeps", 1.0);
        } else {
            c.preconditioner = precondCode(controls_.lookupWord("preconditioner", "none"), matrix_.symmetric());
        }
        c.precision = precision_;
        c.ordering = controls_.lookupWord("gpuOrdering", precision_ == MRG_PRECISION_MIXED ? "colour" : "exact") ==
                             "colour"
                         ? MRG_ORDER_COLOUR
                         : MRG_ORDER_EXACT;
        c.inner_rel_tol = controls_.lookupOrDefault("innerRelTol", 1e-5);
        mrg_perf perf;
        check(mrg_solve(mesh, source.data(), psi.data(), &c, &perf), "mrg_solve");
        lduMatrix::solverPerformance out;
        static const char* const names[2][5] = {{"gpuPCG", "gpuPBiCG", "gpuBiCGStab", "gpuSmoothSolver", "gpuGAMG"},
                                                 {"gpuMixedPCG", "gpuMixedPBiCG", "gpuMixedBiCGStab", "-", "-"}};
        out.solverName = names[precision_ ? 1 : 0][solverKind_];
        out.fieldName = fieldName_;
        out.initialResidual = perf.initial_residual;
        out.finalResidual = perf.final_residual;
        out.nIterations = perf.n_iter;
        out.converged = perf.converged != 0;
        out.singular = perf.singular != 0;
        return out;
    }

private:
    int solverKind_, precision_;
};

#define MRG_DEFINE_SOLVER(Name, Kind, Prec)                                                              \
    class Name : public gpuLduSolver {                                                                   \
    public:                                                                                              \
        Name(const word& f, const lduMatrix& m, const FieldField& b, const FieldField& i,                \
             const lduInterfaceFieldPtrsList& ifs, const dictionary& c)                                  \
            : gpuLduSolver(f, m, b, i, ifs, c, Kind, Prec)                                               \
        {                                                                                                \
        }                                                                                                \
    };

MRG_DEFINE_SOLVER(gpuPCG, MRG_SOLVER_PCG, MRG_PRECISION_FP64)
MRG_DEFINE_SOLVER(gpuPBiCG, MRG_SOLVER_PBICG, MRG_PRECISION_FP64)
MRG_DEFINE_SOLVER(gpuMixedPCG, MRG_SOLVER_PCG, MRG_PRECISION_MIXED)
MRG_DEFINE_SOLVER(gpuMixedPBiCG, MRG_SOLVER_PBICG, MRG_PRECISION_MIXED)
MRG_DEFINE_SOLVER(gpuBiCGStab, MRG_SOLVER_BICGSTAB, MRG_PRECISION_FP64)
MRG_DEFINE_SOLVER(gpuMixedBiCGStab, MRG_SOLVER_BICGSTAB, MRG_PRECISION_MIXED)
MRG_DEFINE_SOLVER(gpuSmoothSolver, MRG_SOLVER_SMOOTH, MRG_PRECISION_FP64)
MRG_DEFINE_SOLVER(gpuGAMG, MRG_SOLVER_GAMG, MRG_PRECISION_FP64)

// foam's BICCG: PBiCG with the DILU preconditioner built in (the tutorials'
// fluid p solves); the preconditioner word is not read.
class gpuBICCG : public gpuLduSolver {
public:
    gpuBICCG(const word& f, const lduMatrix& m, const FieldField& b, const FieldField& i,
             const lduInterfaceFieldPtrsList& ifs, const dictionary& c)
        : gpuLduSolver(f, m, b, i, ifs, with_dilu(c), MRG_SOLVER_PBICG, MRG_PRECISION_FP64)
    {
    }

private:
    static dictionary with_dilu(dictionary c)
    {
        c.set("preconditioner", std::string("DILU"));
        return c;
    }
};

// addToRunTimeSelectionTable(lduMatrix::solver, gpuPCG, symMatrix) etc.
static addSymMatrixSolver<gpuPCG> addGpuPCG("gpuPCG");
static addSymMatrixSolver<gpuMixedPCG> addGpuMixedPCG("gpuMixedPCG");
static addAsymMatrixSolver<gpuPBiCG> addGpuPBiCG("gpuPBiCG");
static addAsymMatrixSolver<gpuMixedPBiCG> addGpuMixedPBiCG("gpuMixedPBiCG");
// PBiCG also accepts symmetric matrices in foam (it is registered in both
// tables); so do the GPU variants.
static addSymMatrixSolver<gpuPBiCG> addGpuPBiCGSym("gpuPBiCG");
static addSymMatrixSolver<gpuMixedPBiCG> addGpuMixedPBiCGSym("gpuMixedPBiCG");
// BiCGStab is registered in both tables, as foam-extend's BiCGStab is.
static addSymMatrixSolver<gpuBiCGStab> addGpuBiCGStabSym("gpuBiCGStab");
static addAsymMatrixSolver<gpuBiCGStab> addGpuBiCGStab("gpuBiCGStab");
static addSymMatrixSolver<gpuMixedBiCGStab> addGpuMixedBiCGStabSym("gpuMixedBiCGStab");
static addAsymMatrixSolver<gpuMixedBiCGStab> addGpuMixedBiCGStab("gpuMixedBiCGStab");
static addSymMatrixSolver<gpuGAMG> addGpuGAMGSym("gpuGAMG");
static addAsymMatrixSolver<gpuGAMG> addGpuGAMG("gpuGAMG");
static addSymMatrixSolver<gpuBICCG> addGpuBICCGSym("gpuBICCG");
static addAsymMatrixSolver<gpuBICCG> addGpuBICCG("gpuBICCG");
// smoothSolver, like foam's, takes either kind of matrix.
static addSymMatrixSolver<gpuSmoothSolver> addGpuSmoothSolverSym("gpuSmoothSolver");
static addAsymMatrixSolver<gpuSmoothSolver> addGpuSmoothSolver("gpuSmoothSolver");

}  // namespace Foam
