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
//   gpuGAMG           both        FP64 GAMG, GaussSeidel smoothing; agglomerator faceAreaPair
//                                 (the fvMesh's Sf) | algebraicPair, nCellsInCoarsestLevel,
//                                 nPostSweeps, maxPostSweeps, postSweepsLevelMultiplier,
//                                 nFinestSweeps, scaleCorrection
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
// The same names (all but gpuGAMG) are registered in foam-extend's
// coupledLduSolver tables too: the monolithic solve of coupledFvMatrix
// (multiRegionSystem.C:150-153, dictionary "<fld>coupled", e.g. the
// tutorials' "Tcoupled { solver BiCGStab; preconditioner { preconditioner
// Cholesky; } ... }") concatenates the region matrices into one LDU system
// (cells and faces region by region, so upper-triangular order holds) with
// the regionCouple interfaces as its interface rows, solves it, and hands
// each region its part of the solution.
//
// Interfaces: each monolithicCouplingFvPatchField interface is described to
// the library from its regionCouple patch -- the patch's faceCells receive
// the update, and each face's neighbour value is the GGI interpolation of
// the shadow patch's faceCells values (slaveToMaster weights on the master
// side, masterToSlave on the slave side), exactly the buffer
// initInterfaceMatrixUpdate builds (monolithicCouplingFvPatchField.C:381-
// 417) and updateInterfaceMatrix subtracts (:441-454).
//
// "preconditioner" is read as a word or, as the coupled solvers' entries
// write it, as a sub-dictionary holding the word ("preconditioner {
// preconditioner Cholesky; }").
//
// Extra (optional) controls: "gpuOrdering" exact|colour, "innerRelTol",
// "hbmBudget" (bytes, per process), "gpuDevice".
#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <set>
#include <string>

#include "lduMatrix.H"
#include "mrgpu.h"

namespace Foam {

namespace {

// Resident addressing, keyed by the lduAddressing objects of the matrix
// (one, or one per region of a coupled matrix) and a hash of the interface
// descriptions (a moved interface, with new GGI weights, uploads anew).
typedef std::pair<std::vector<const void*>, uint64_t> MeshKey;

struct GpuState {
    mrg_ctx* ctx = nullptr;
    std::map<MeshKey, mrg_mesh*> meshes;
    std::set<mrg_mesh*> faceAreas;   // meshes given their face areas (faceAreaPair)
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

// The preconditioner word: "preconditioner DIC;" or, as the coupled
// solvers write it, "preconditioner { preconditioner Cholesky; }".
word precondWord(const dictionary& d)
{
    if (d.isDict("preconditioner")) return d.subDict("preconditioner").lookupWord("preconditioner", "none");
    return d.lookupWord("preconditioner", "none");
}

void ensureContext(GpuState& S, const dictionary& d)
{
    if (S.ctx) return;
    const int dev = (int)d.lookupOrDefault("gpuDevice", 0);
    const size_t budget = (size_t)d.lookupOrDefault("hbmBudget", 0);
    check(mrg_ctx_create(dev, budget, &S.ctx), "mrg_ctx_create");
}

// The interfaces of one or more region matrices, flattened for the library
// in the concatenated cell numbering (region r's cells from offset[r]).
struct FlatInterfaces {
    std::vector<mrg_iface_desc> desc;
    std::vector<std::vector<int32_t>> cells, ptr, src;
    std::vector<std::vector<double>> w;
    scalarField bou, intc;
    bool intDiffers = false;
    uint64_t hash = 1469598103934665603ull;   // FNV-1a over the descriptions

    void mix(const void* p, size_t n)
    {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) hash = (hash ^ b[i]) * 1099511628211ull;
    }
};

// rows[r] = region r's interfaces, bou / intc their coefficients.
FlatInterfaces flattenInterfaces(const std::vector<const lduInterfaceFieldPtrsList*>& rows,
                                 const std::vector<const FieldField*>& bou, const std::vector<const FieldField*>& intc,
                                 const std::vector<label>& offset)
{
    // where every regionCouple patch lives: (row, its faceCells)
    std::map<const regionCouplePolyPatch*, label> rowOf;
    for (size_t r = 0; r < rows.size(); ++r)
        for (const lduInterfaceField* f : *rows[r])
            if (f) rowOf[&f->regionCouplePatch()] = (label)r;
    FlatInterfaces F;
    for (size_t r = 0; r < rows.size(); ++r) {
        const lduInterfaceFieldPtrsList& ifs = *rows[r];
        for (size_t p = 0; p < ifs.size(); ++p) {
            if (!ifs[p]) continue;
            const regionCouplePolyPatch& P = ifs[p]->regionCouplePatch();
            const regionCouplePolyPatch& Q = P.shadow();
            auto q = rowOf.find(&Q);
            if (q == rowOf.end())
                throw FatalError("gpu solver: the shadow of interface " + P.name() + " (" + Q.name() +
                                 ") is in no region of this matrix");
            const GGIInterpolation& g = P.patchToPatch();
            const labelListList& addr = P.master() ? g.masterAddr() : g.slaveAddr();
            const scalarListList& wt = P.master() ? g.masterWeights() : g.slaveWeights();
            const label nFaces = P.size();
            if ((label)addr.size() != nFaces || (label)wt.size() != nFaces)
                throw FatalError("gpu solver: interpolator of " + P.name() + " does not match its faces");
            std::vector<int32_t> cells(nFaces), ptr(nFaces + 1, 0), src;
            std::vector<double> w;
            const labelList& qCells = Q.faceCells();
            for (label i = 0; i < nFaces; ++i) {
                cells[i] = P.faceCells()[i] + offset[r];
                for (size_t k = 0; k < addr[i].size(); ++k) {
                    const label j = addr[i][k];
                    if (j < 0 || j >= (label)qCells.size())
                        throw FatalError("gpu solver: interpolator of " + P.name() + " addresses a face beyond " +
                                         Q.name());
                    src.push_back(qCells[j] + offset[q->second]);
                    w.push_back(wt[i][k]);
                }
                ptr[i + 1] = (int32_t)src.size();
            }
            F.mix(cells.data(), cells.size() * sizeof(int32_t));
            F.mix(ptr.data(), ptr.size() * sizeof(int32_t));
            F.mix(src.data(), src.size() * sizeof(int32_t));
            F.mix(w.data(), w.size() * sizeof(double));
            F.cells.push_back(std::move(cells));
            F.ptr.push_back(std::move(ptr));
            F.src.push_back(std::move(src));
            F.w.push_back(std::move(w));
            const scalarField& b = (*bou[r])[p];
            const scalarField& i = intc[r]->size() > p ? (*intc[r])[p] : b;
            if ((label)b.size() != nFaces || (label)i.size() != nFaces)
                throw FatalError("gpu solver: coupling coefficients of " + P.name() + " do not match its faces");
            F.bou.insert(F.bou.end(), b.begin(), b.end());
            F.intc.insert(F.intc.end(), i.begin(), i.end());
            if (i != b) F.intDiffers = true;
        }
    }
    for (size_t k = 0; k < F.cells.size(); ++k) {
        mrg_iface_desc d;
        d.n_faces = (int)F.cells[k].size();
        d.face_cells = F.cells[k].data();
        d.src_ptr = F.ptr[k].data();
        d.src_cell = F.src[k].empty() ? nullptr : F.src[k].data();
        d.src_weight = F.w[k].empty() ? nullptr : F.w[k].data();
        F.desc.push_back(d);
    }
    return F;
}

// foam's Switch words
bool isTrue(const word& w)
{
    if (w == "true" || w == "on" || w == "yes" || w == "y" || w == "1") return true;
    if (w == "false" || w == "off" || w == "no" || w == "n" || w == "0" || w == "none") return false;
    throw FatalError("not a switch: " + w);
}

// The library's controls from a solver dictionary.
mrg_controls makeControls(const dictionary& d, int solverKind, int precision, bool symmetric, scalar tolerance,
                          scalar relTol, label minIter, label maxIter)
{
    mrg_controls c;
    mrg_controls_default(&c);
    c.tolerance = tolerance;
    c.rel_tol = relTol;
    c.min_iter = minIter;
    c.max_iter = maxIter;
    c.solver = solverKind;
    if (solverKind == MRG_SOLVER_GAMG) {
        // GAMG's own words (foam's defaults); the agglomeration is always
        // cached and the coarsest level always solved directly
        // (directSolveCoarsest is read as true)
        if (d.lookupWord("smoother", "GaussSeidel") != "GaussSeidel")
            throw FatalError("gpuGAMG: unsupported smoother " + d.lookupWord("smoother"));
        c.smoother = MRG_SMOOTHER_GAUSS_SEIDEL;
        c.gamg_coarsest_cells = (int)d.lookupOrDefault("nCellsInCoarsestLevel", 10.0);
        c.gamg_post_sweeps = (int)d.lookupOrDefault("nPostSweeps", 2.0);
        c.gamg_finest_sweeps = (int)d.lookupOrDefault("nFinestSweeps", 2.0);
        c.gamg_max_post_sweeps = (int)d.lookupOrDefault("maxPostSweeps", 4.0);
        c.gamg_post_sweeps_level_multiplier = (int)d.lookupOrDefault("postSweepsLevelMultiplier", 1.0);
        c.gamg_scale_correction = isTrue(d.lookupWord("scaleCorrection", "true")) ? 1 : 0;
        const word ag = d.lookupWord("agglomerator", "faceAreaPair");
        if (ag == "faceAreaPair") c.gamg_agglomerator = MRG_AGGLOMERATOR_FACE_AREA_PAIR;
        else if (ag == "algebraicPair") c.gamg_agglomerator = MRG_AGGLOMERATOR_ALGEBRAIC_PAIR;
        else throw FatalError("gpuGAMG: unsupported agglomerator " + ag);
        if ((int)d.lookupOrDefault("nPreSweeps", 0.0) != 0)
            throw FatalError("gpuGAMG: nPreSweeps must be 0 (pre-smoothing is not built)");
        if ((int)d.lookupOrDefault("mergeLevels", 1.0) != 1)
            throw FatalError("gpuGAMG: mergeLevels must be 1");
    } else if (solverKind == MRG_SOLVER_SMOOTH) {
        // smoothSolver's own words: smoother and nSweeps
        const word sm = d.lookupWord("smoother", "GaussSeidel");
        if (sm == "GaussSeidel") c.smoother = MRG_SMOOTHER_GAUSS_SEIDEL;
        else if (sm == "DIC") c.smoother = MRG_SMOOTHER_DIC;
        else if (sm == "DILU") c.smoother = MRG_SMOOTHER_DILU;
        else if (sm == "DICGaussSeidel") c.smoother = MRG_SMOOTHER_DIC_GAUSS_SEIDEL;
        else if (sm == "DILUGaussSeidel") c.smoother = MRG_SMOOTHER_DILU_GAUSS_SEIDEL;
        else throw FatalError("gpuSmoothSolver: unsupported smoother " + sm);
        c.n_sweeps = (int)d.lookupOrDefault("nSweeps", 1.0);
    } else {
        c.preconditioner = precondCode(precondWord(d), symmetric);
    }
    c.precision = precision;
    c.ordering = d.lookupWord("gpuOrdering", precision == MRG_PRECISION_MIXED ? "colour" : "exact") == "colour"
                     ? MRG_ORDER_COLOUR
                     : MRG_ORDER_EXACT;
    c.inner_rel_tol = d.lookupOrDefault("innerRelTol", 1e-5);
    return c;
}

const char* solverName(int kind, int precision)
{
    static const char* const names[2][5] = {{"gpuPCG", "gpuPBiCG", "gpuBiCGStab", "gpuSmoothSolver", "gpuGAMG"},
                                             {"gpuMixedPCG", "gpuMixedPBiCG", "gpuMixedBiCGStab", "-", "-"}};
    return names[precision ? 1 : 0][kind];
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
        ensureContext(S, controls_);
        const lduAddressing& a = matrix_.lduAddr();
        const label n = a.size(), nf = (label)a.lowerAddr().size();
        if ((label)psi.size() != n || (label)source.size() != n)
            throw FatalError("gpu solver: psi/source size does not match the matrix");
        FlatInterfaces F = flattenInterfaces({&interfaces_}, {&coupleBouCoeffs_}, {&coupleIntCoeffs_}, {0});
        mrg_mesh*& mesh = S.meshes[MeshKey({&a}, F.hash)];
        if (!mesh) {
            check(mrg_mesh_upload(S.ctx, n, nf, a.lowerAddr().data(), a.upperAddr().data(), (int)F.desc.size(),
                                  F.desc.empty() ? nullptr : F.desc.data(), &mesh),
                  "mrg_mesh_upload");
        }
        check(mrg_coeffs_upload(mesh, matrix_.diag().data(), matrix_.upper().data(),
                                matrix_.hasLower() ? matrix_.lower().data() : nullptr,
                                F.bou.empty() ? nullptr : F.bou.data(), F.intDiffers ? F.intc.data() : nullptr),
              "mrg_coeffs_upload");
        const mrg_controls c = makeControls(controls_, solverKind_, precision_, matrix_.symmetric(), tolerance_,
                                            relTol_, minIter_, maxIter_);
        if (c.solver == MRG_SOLVER_GAMG && c.gamg_agglomerator == MRG_AGGLOMERATOR_FACE_AREA_PAIR &&
            !S.faceAreas.count(mesh)) {
            // faceAreaPair weighs the pairing with the mesh's face area vectors
            const fvMesh* fm = matrix_.hasMesh() ? dynamic_cast<const fvMesh*>(&matrix_.mesh()) : nullptr;
            if (!fm) throw FatalError("gpuGAMG: agglomerator faceAreaPair needs the matrix's fvMesh");
            const vectorField& Sf = fm->Sf().internalField();
            if ((label)Sf.size() != nf) throw FatalError("gpuGAMG: Sf does not match the faces");
            std::vector<double> sf(3 * (size_t)nf);
            for (label f = 0; f < nf; ++f) {
                sf[3 * (size_t)f] = Sf[f].x();
                sf[3 * (size_t)f + 1] = Sf[f].y();
                sf[3 * (size_t)f + 2] = Sf[f].z();
            }
            check(mrg_mesh_set_face_areas(mesh, sf.data()), "mrg_mesh_set_face_areas");
            S.faceAreas.insert(mesh);
        }
        mrg_perf perf;
        check(mrg_solve(mesh, source.data(), psi.data(), &c, &perf), "mrg_solve");
        lduMatrix::solverPerformance out;
        out.solverName = solverName(solverKind_, precision_);
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

// ---- coupledLduSolver adapters ------------------------------------------
// coupledFvMatrix::solve -> coupledLduSolver::New(...)->solve(x, b): the
// region matrices concatenated into one LDU system (region r's cells from
// the sum of the earlier regions' sizes, its faces after theirs), the
// regionCouple interfaces as its interface rows, one solve, each region's
// part of the solution copied back.  The performance record is the
// concatenated system's: foam's normalised residual over all regions.
class gpuCoupledLduSolver : public coupledLduSolver {
public:
    gpuCoupledLduSolver(const word& fieldName, const coupledLduMatrix& matrix, const FieldFieldList& bou,
                        const FieldFieldList& intc, const lduInterfaceFieldPtrsListList& ifs, const dictionary& dict,
                        int solverKind, int precision)
        : coupledLduSolver(fieldName, matrix, bou, intc, ifs, dict), solverKind_(solverKind), precision_(precision)
    {
    }

    coupledSolverPerformance solve(FieldField& x, const FieldField& b, const direction) const override
    {
        GpuState& S = state();
        std::lock_guard<std::mutex> g(S.lock);
        ensureContext(S, dict_);
        const label R = matrix_.size();
        if ((label)x.size() != R || (label)b.size() != R || (label)interfaces_.size() != R ||
            (label)bouCoeffs_.size() != R)
            throw FatalError("gpu coupled solver: x, b, interfaces and coefficients need one entry per region");
        std::vector<label> offset(R + 1, 0);
        std::vector<const void*> key;
        label nf = 0;
        const bool sym = matrix_.symmetric();
        for (label r = 0; r < R; ++r) {
            const lduMatrix& m = matrix_[r];
            const label n = m.lduAddr().size();
            if ((label)x[r].size() != n || (label)b[r].size() != n)
                throw FatalError("gpu coupled solver: x/b size does not match region matrix " + std::to_string(r));
            offset[r + 1] = offset[r] + n;
            nf += (label)m.lduAddr().lowerAddr().size();
            key.push_back(&m.lduAddr());
        }
        std::vector<const lduInterfaceFieldPtrsList*> rows;
        std::vector<const FieldField*> bous, ints;
        for (label r = 0; r < R; ++r) {
            rows.push_back(&interfaces_[r]);
            bous.push_back(&bouCoeffs_[r]);
            ints.push_back(intCoeffs_.size() > (size_t)r ? &intCoeffs_[r] : &bouCoeffs_[r]);
        }
        FlatInterfaces F = flattenInterfaces(rows, bous, ints, offset);
        const label n = offset[R];
        std::vector<int32_t> lower, upper;
        scalarField diag, up, lo, bb, xx;
        lower.reserve(nf);
        upper.reserve(nf);
        for (label r = 0; r < R; ++r) {
            const lduMatrix& m = matrix_[r];
            for (label v : m.lduAddr().lowerAddr()) lower.push_back(v + offset[r]);
            for (label v : m.lduAddr().upperAddr()) upper.push_back(v + offset[r]);
            diag.insert(diag.end(), m.diag().begin(), m.diag().end());
            up.insert(up.end(), m.upper().begin(), m.upper().end());
            // a symmetric region among asymmetric ones: lower = upper
            const scalarField& l = m.hasLower() ? m.lower() : m.upper();
            if (!sym) lo.insert(lo.end(), l.begin(), l.end());
            bb.insert(bb.end(), b[r].begin(), b[r].end());
            xx.insert(xx.end(), x[r].begin(), x[r].end());
        }
        mrg_mesh*& mesh = S.meshes[MeshKey(key, F.hash)];
        if (!mesh) {
            check(mrg_mesh_upload(S.ctx, n, nf, lower.data(), upper.data(), (int)F.desc.size(),
                                  F.desc.empty() ? nullptr : F.desc.data(), &mesh),
                  "mrg_mesh_upload");
        }
        check(mrg_coeffs_upload(mesh, diag.data(), up.data(), sym ? nullptr : lo.data(),
                                F.bou.empty() ? nullptr : F.bou.data(), F.intDiffers ? F.intc.data() : nullptr),
              "mrg_coeffs_upload");
        const mrg_controls c =
            makeControls(dict_, solverKind_, precision_, sym, tolerance_, relTol_, minIter_, maxIter_);
        mrg_perf perf;
        check(mrg_solve(mesh, bb.data(), xx.data(), &c, &perf), "mrg_solve");
        for (label r = 0; r < R; ++r)
            std::copy(xx.begin() + offset[r], xx.begin() + offset[r + 1], x[r].begin());
        coupledSolverPerformance out;
        out.solverName = solverName(solverKind_, precision_);
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

#define MRG_DEFINE_COUPLED(Name, Kind, Prec)                                                              \
    class Name : public gpuCoupledLduSolver {                                                             \
    public:                                                                                               \
        Name(const word& f, const coupledLduMatrix& m, const FieldFieldList& b, const FieldFieldList& i, \
             const lduInterfaceFieldPtrsListList& ifs, const dictionary& c)                               \
            : gpuCoupledLduSolver(f, m, b, i, ifs, c, Kind, Prec)                                         \
        {                                                                                                 \
        }                                                                                                 \
    };

MRG_DEFINE_COUPLED(gpuCoupledPCG, MRG_SOLVER_PCG, MRG_PRECISION_FP64)
MRG_DEFINE_COUPLED(gpuCoupledPBiCG, MRG_SOLVER_PBICG, MRG_PRECISION_FP64)
MRG_DEFINE_COUPLED(gpuCoupledBiCGStab, MRG_SOLVER_BICGSTAB, MRG_PRECISION_FP64)
MRG_DEFINE_COUPLED(gpuCoupledMixedPCG, MRG_SOLVER_PCG, MRG_PRECISION_MIXED)
MRG_DEFINE_COUPLED(gpuCoupledMixedPBiCG, MRG_SOLVER_PBICG, MRG_PRECISION_MIXED)
MRG_DEFINE_COUPLED(gpuCoupledMixedBiCGStab, MRG_SOLVER_BICGSTAB, MRG_PRECISION_MIXED)
MRG_DEFINE_COUPLED(gpuCoupledSmoothSolver, MRG_SOLVER_SMOOTH, MRG_PRECISION_FP64)

// addToRunTimeSelectionTable(coupledLduSolver, ..., symMatrix / asymMatrix):
// the coupled table, under the same names as the lduMatrix::solver table.
static addSymCoupledSolver<gpuCoupledPCG> addGpuCoupledPCG("gpuPCG");
static addSymCoupledSolver<gpuCoupledMixedPCG> addGpuCoupledMixedPCG("gpuMixedPCG");
static addSymCoupledSolver<gpuCoupledPBiCG> addGpuCoupledPBiCGSym("gpuPBiCG");
static addAsymCoupledSolver<gpuCoupledPBiCG> addGpuCoupledPBiCG("gpuPBiCG");
static addSymCoupledSolver<gpuCoupledMixedPBiCG> addGpuCoupledMixedPBiCGSym("gpuMixedPBiCG");
static addAsymCoupledSolver<gpuCoupledMixedPBiCG> addGpuCoupledMixedPBiCG("gpuMixedPBiCG");
static addSymCoupledSolver<gpuCoupledBiCGStab> addGpuCoupledBiCGStabSym("gpuBiCGStab");
static addAsymCoupledSolver<gpuCoupledBiCGStab> addGpuCoupledBiCGStab("gpuBiCGStab");
static addSymCoupledSolver<gpuCoupledMixedBiCGStab> addGpuCoupledMixedBiCGStabSym("gpuMixedBiCGStab");
static addAsymCoupledSolver<gpuCoupledMixedBiCGStab> addGpuCoupledMixedBiCGStab("gpuMixedBiCGStab");
static addSymCoupledSolver<gpuCoupledSmoothSolver> addGpuCoupledSmoothSym("gpuSmoothSolver");
static addAsymCoupledSolver<gpuCoupledSmoothSolver> addGpuCoupledSmooth("gpuSmoothSolver");

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
