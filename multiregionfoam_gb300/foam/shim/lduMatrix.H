// lduMatrix.H -- project-written stand-in for the parts of foam-extend 4.1's
// lduMatrix / lduAddressing / lduMatrix::solver API that the GPU solver
// adapter uses.  It reproduces the API *shape* (names, argument meaning,
// run-time selection by solver name) so the adapter compiles and can be
// exercised without foam-extend; against a real foam-extend build the adapter
// includes foam's own headers instead (the shim's
// lduMatrix::solverPerformance is foam's lduSolverPerformance, and
// addSymMatrixSolver / addAsymMatrixSolver become
// addToRunTimeSelectionTable(lduMatrix::solver, T, symMatrix / asymMatrix)).
// No foam-extend
// source is reproduced here.
#pragma once

#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace Foam {

typedef double scalar;
typedef int32_t label;
typedef unsigned char direction;
typedef std::string word;
typedef std::vector<scalar> scalarField;
typedef std::vector<label> labelList;

// FatalError: foam aborts; the shim throws.
struct FatalError : std::runtime_error {
    explicit FatalError(const std::string& m) : std::runtime_error(m) {}
};

// A flat controls dictionary (solver, preconditioner, tolerance, relTol, ...).
class dictionary {
public:
    void set(const word& k, const std::string& v) { s_[k] = v; }
    void set(const word& k, scalar v) { d_[k] = v; }
    bool found(const word& k) const { return s_.count(k) || d_.count(k); }
    word lookupWord(const word& k, const word& def = "") const
    {
        auto it = s_.find(k);
        return it == s_.end() ? def : it->second;
    }
    scalar lookupOrDefault(const word& k, scalar def) const
    {
        auto it = d_.find(k);
        return it == d_.end() ? def : it->second;
    }

private:
    std::map<word, std::string> s_;
    std::map<word, scalar> d_;
};

// lduAddressing: lowerAddr (owner) < upperAddr (neighbour), faces in
// upper-triangular order.
class lduAddressing {
public:
    lduAddressing(label n, labelList lower, labelList upper)
        : n_(n), lower_(std::move(lower)), upper_(std::move(upper)) {}
    label size() const { return n_; }
    const labelList& lowerAddr() const { return lower_; }
    const labelList& upperAddr() const { return upper_; }

private:
    label n_;
    labelList lower_, upper_;
};

// A monolithic regionCouple interface seen from one side: the cells it
// updates (faceCells) and, per face, the shadow-side cells and GGI weights
// that interpolate the neighbour value
// (monolithicCouplingFvPatchField::initInterfaceMatrixUpdate).
struct lduInterfaceField {
    labelList faceCells;
    labelList srcPtr;       // CSR into srcCells/srcWeights (size faceCells+1)
    labelList srcCells;
    scalarField srcWeights;
};
typedef std::vector<const lduInterfaceField*> lduInterfaceFieldPtrsList;
typedef std::vector<scalarField> FieldField;  // per-interface coefficients

class lduMatrix {
public:
    explicit lduMatrix(const lduAddressing& a) : addr_(a) {}
    const lduAddressing& lduAddr() const { return addr_; }
    scalarField& diag() { return diag_; }
    scalarField& upper() { return upper_; }
    scalarField& lower() { return lower_; }
    const scalarField& diag() const { return diag_; }
    const scalarField& upper() const { return upper_; }
    const scalarField& lower() const { return lower_; }
    bool hasLower() const { return !lower_.empty(); }
    bool symmetric() const { return !hasLower(); }
    bool asymmetric() const { return hasLower(); }

    // lduSolverPerformance
    struct solverPerformance {
        word solverName, fieldName;
        scalar initialResidual = 0, finalResidual = 0;
        label nIterations = 0;
        bool converged = false, singular = false;
    };

    // lduMatrix::solver: run-time selected by the "solver" word.
    class solver {
    public:
        typedef std::function<std::unique_ptr<solver>(const word&, const lduMatrix&, const FieldField&,
                                                      const FieldField&, const lduInterfaceFieldPtrsList&,
                                                      const dictionary&)>
            ctor;
        solver(const word& fieldName, const lduMatrix& matrix, const FieldField& coupleBouCoeffs,
               const FieldField& coupleIntCoeffs, const lduInterfaceFieldPtrsList& interfaces,
               const dictionary& controls)
            : fieldName_(fieldName), matrix_(matrix), coupleBouCoeffs_(coupleBouCoeffs),
              coupleIntCoeffs_(coupleIntCoeffs), interfaces_(interfaces), controls_(controls)
        {
            tolerance_ = controls.lookupOrDefault("tolerance", 1e-6);
            relTol_ = controls.lookupOrDefault("relTol", 0.0);
            minIter_ = (label)controls.lookupOrDefault("minIter", 0);
            maxIter_ = (label)controls.lookupOrDefault("maxIter", 1000);
        }
        virtual ~solver() = default;
        virtual solverPerformance solve(scalarField& psi, const scalarField& source,
                                        const direction cmpt = 0) const = 0;

        static std::map<word, ctor>& symMatrixConstructorTable()
        {
            static std::map<word, ctor> t;
            return t;
        }
        static std::map<word, ctor>& asymMatrixConstructorTable()
        {
            static std::map<word, ctor> t;
            return t;
        }
        // lduMatrix::solver::New: symmetric matrices look in the symMatrix
        // table, asymmetric ones in the asymMatrix table.
        static std::unique_ptr<solver> New(const word& fieldName, const lduMatrix& matrix,
                                           const FieldField& bou, const FieldField& intc,
                                           const lduInterfaceFieldPtrsList& ifs, const dictionary& controls)
        {
            const word name = controls.lookupWord("solver");
            auto& table = matrix.symmetric() ? symMatrixConstructorTable() : asymMatrixConstructorTable();
            auto it = table.find(name);
            if (it == table.end())
                throw FatalError("Unknown " + std::string(matrix.symmetric() ? "symmetric" : "asymmetric") +
                                 " matrix solver " + name);
            return it->second(fieldName, matrix, bou, intc, ifs, controls);
        }

    protected:
        word fieldName_;
        const lduMatrix& matrix_;
        const FieldField& coupleBouCoeffs_;
        const FieldField& coupleIntCoeffs_;
        const lduInterfaceFieldPtrsList& interfaces_;
        dictionary controls_;
        scalar tolerance_, relTol_;
        label minIter_, maxIter_;
    };

private:
    const lduAddressing& addr_;
    scalarField diag_, upper_, lower_;
};

// Registration helper (foam: addToRunTimeSelectionTable).
template <class Type>
struct addSymMatrixSolver {
    explicit addSymMatrixSolver(const word& name)
    {
        lduMatrix::solver::symMatrixConstructorTable()[name] =
            [](const word& f, const lduMatrix& m, const FieldField& b, const FieldField& i,
               const lduInterfaceFieldPtrsList& ifs, const dictionary& c) {
                return std::unique_ptr<lduMatrix::solver>(new Type(f, m, b, i, ifs, c));
            };
    }
};
template <class Type>
struct addAsymMatrixSolver {
    explicit addAsymMatrixSolver(const word& name)
    {
        lduMatrix::solver::asymMatrixConstructorTable()[name] =
            [](const word& f, const lduMatrix& m, const FieldField& b, const FieldField& i,
               const lduInterfaceFieldPtrsList& ifs, const dictionary& c) {
                return std::unique_ptr<lduMatrix::solver>(new Type(f, m, b, i, ifs, c));
            };
    }
};

}  // namespace Foam
