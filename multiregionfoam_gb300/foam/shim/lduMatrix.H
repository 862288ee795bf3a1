// lduMatrix.H -- project-written stand-in for the parts of foam-extend 4.1's
// lduMatrix / lduAddressing / lduMatrix::solver API that the GPU solver
// adapter uses.  It reproduces the API *shape* (names, argument meaning,
// run-time selection by solver name) so the adapter compiles and can be
// exercised without foam-extend; against a real foam-extend build the adapter
// includes foam's own headers instead (the shim's
// lduMatrix::solverPerformance is foam's lduSolverPerformance, and
// addSymMatrixSolver / addAsymMatrixSolver become
// addToRunTimeSelectionTable(lduMatrix::solver, T, symMatrix / asymMatrix),
// addSymCoupledSolver / addAsymCoupledSolver the same for coupledLduSolver).
// Names and argument meaning follow foam-extend 4.1's API as this project
// restates it; the regionCouple and GGI classes expose only what the
// adapter reads.  No foam-extend source is reproduced here.
#pragma once

#include <cctype>
#include <cstdint>
#include <cstdlib>
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

// A controls dictionary: word and number entries and nested sub-
// dictionaries (foam's "preconditioner { preconditioner Cholesky; }"), with
// a reader for the fvSolution entry syntax (`key value;`, `key { ... }`,
// `//` and `/* */` comments).
class dictionary {
public:
    dictionary() = default;
    // Parse the entries of one dictionary body (the text between an
    // fvSolution entry's braces, or a whole file of entries).
    static dictionary parse(const std::string& text)
    {
        size_t pos = 0;
        return parseBody(text, pos, false);
    }
    // set() replaces any entry of the same keyword, whatever its kind
    void set(const word& k, const std::string& v)
    {
        erase(k);
        s_[k] = v;
    }
    void set(const word& k, scalar v)
    {
        erase(k);
        d_[k] = v;
    }
    void set(const word& k, const dictionary& sub)
    {
        erase(k);
        sub_[k] = std::make_shared<dictionary>(sub);
    }
    void erase(const word& k)
    {
        s_.erase(k);
        d_.erase(k);
        sub_.erase(k);
    }
    bool found(const word& k) const { return s_.count(k) || d_.count(k) || sub_.count(k); }
    bool isDict(const word& k) const { return sub_.count(k) != 0; }
    const dictionary& subDict(const word& k) const
    {
        auto it = sub_.find(k);
        if (it == sub_.end()) throw FatalError("keyword " + k + " is undefined or not a sub-dictionary");
        return *it->second;
    }
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
    std::map<word, std::shared_ptr<dictionary>> sub_;

    static void skipSpace(const std::string& t, size_t& p)
    {
        for (;;) {
            while (p < t.size() && std::isspace((unsigned char)t[p])) ++p;
            if (t.compare(p, 2, "//") == 0) {
                while (p < t.size() && t[p] != '\n') ++p;
            } else if (t.compare(p, 2, "/*") == 0) {
                const size_t e = t.find("*/", p + 2);
                p = e == std::string::npos ? t.size() : e + 2;
            } else {
                return;
            }
        }
    }
    static std::string token(const std::string& t, size_t& p)
    {
        skipSpace(t, p);
        const size_t b = p;
        while (p < t.size() && !std::isspace((unsigned char)t[p]) && t[p] != ';' && t[p] != '{' && t[p] != '}') ++p;
        return t.substr(b, p - b);
    }
    static dictionary parseBody(const std::string& t, size_t& p, bool braced)
    {
        dictionary d;
        for (;;) {
            skipSpace(t, p);
            if (p >= t.size()) {
                if (braced) throw FatalError("dictionary: missing '}'");
                return d;
            }
            if (t[p] == '}') {
                if (!braced) throw FatalError("dictionary: unexpected '}'");
                ++p;
                return d;
            }
            const std::string key = token(t, p);
            if (key.empty()) throw FatalError("dictionary: expected a keyword");
            skipSpace(t, p);
            if (p < t.size() && t[p] == '{') {
                ++p;
                d.set(key, parseBody(t, p, true));
                continue;
            }
            const std::string val = token(t, p);
            skipSpace(t, p);
            if (p >= t.size() || t[p] != ';') throw FatalError("dictionary: expected ';' after " + key);
            ++p;
            char* end = nullptr;
            const double v = std::strtod(val.c_str(), &end);
            if (!val.empty() && end && *end == '\0')
                d.set(key, v);
            else
                d.set(key, val);
        }
    }
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

typedef std::vector<labelList> labelListList;
typedef std::vector<scalarField> scalarListList;

// A 3-vector (foam's vector): x(), y(), z().
class vector {
public:
    vector(scalar x = 0, scalar y = 0, scalar z = 0) : v_{x, y, z} {}
    scalar x() const { return v_[0]; }
    scalar y() const { return v_[1]; }
    scalar z() const { return v_[2]; }

private:
    scalar v_[3];
};
typedef std::vector<vector> vectorField;

// lduMesh: what an lduMatrix is built on (its addressing).  An fvMesh is
// one, and carries the geometry; of it the adapter reads only the internal
// faces' area vectors (Sf().internalField()), which GAMG's faceAreaPair
// agglomeration weights the pairing with.
class lduMesh {
public:
    virtual ~lduMesh() = default;
    virtual const lduAddressing& lduAddr() const = 0;
};

class surfaceVectorField {
public:
    explicit surfaceVectorField(vectorField internal) : internal_(std::move(internal)) {}
    const vectorField& internalField() const { return internal_; }

private:
    vectorField internal_;
};

class fvMesh : public lduMesh {
public:
    fvMesh(const lduAddressing& addr, vectorField Sf) : addr_(addr), Sf_(std::move(Sf)) {}
    const lduAddressing& lduAddr() const override { return addr_; }
    const surfaceVectorField& Sf() const { return Sf_; }

private:
    const lduAddressing& addr_;
    surfaceVectorField Sf_;
};

// GGIInterpolation: the interpolator a regionCouplePolyPatch pair holds
// (ggiInterfaceToInterfaceMapping.C:62-77 builds the same kind, with
// rescaled weights).  For master face m, masterAddr()[m] lists the slave
// faces it overlaps and masterWeights()[m] their weights (slaveToMaster
// gives master face m the sum w * slave value); slaveAddr / slaveWeights
// the reverse (masterToSlave).  An uncovered face has empty lists.
class GGIInterpolation {
public:
    GGIInterpolation(labelListList masterAddr, scalarListList masterWeights, labelListList slaveAddr,
                     scalarListList slaveWeights)
        : mAddr_(std::move(masterAddr)), mW_(std::move(masterWeights)), sAddr_(std::move(slaveAddr)),
          sW_(std::move(slaveWeights))
    {
    }
    const labelListList& masterAddr() const { return mAddr_; }
    const scalarListList& masterWeights() const { return mW_; }
    const labelListList& slaveAddr() const { return sAddr_; }
    const scalarListList& slaveWeights() const { return sW_; }

private:
    labelListList mAddr_;
    scalarListList mW_;
    labelListList sAddr_;
    scalarListList sW_;
};

// regionCouplePolyPatch / regionCoupleFvPatch: one side of a region-to-
// region interface -- the cells next to its faces (faceCells), whether it
// is the master side, its shadow patch in the other region, and the pair's
// GGI interpolator (held by the master).  interpolate(shadowFaceValues)
// gives this side's faces the shadow side's values (slaveToMaster on the
// master, masterToSlave on the slave), which is how
// monolithicCouplingFvPatchField builds the neighbour values of its matrix
// update (monolithicCouplingFvPatchField.C:381-417).
class regionCouplePolyPatch {
public:
    regionCouplePolyPatch(const word& name, labelList faceCells, bool master)
        : name_(name), faceCells_(std::move(faceCells)), master_(master)
    {
    }
    // join a master and a slave patch through their interpolator
    static void couple(regionCouplePolyPatch& master, regionCouplePolyPatch& slave, const GGIInterpolation& ggi)
    {
        if (!master.master_ || slave.master_) throw FatalError("couple(master, slave): roles swapped");
        master.shadow_ = &slave;
        slave.shadow_ = &master;
        master.ggi_ = slave.ggi_ = &ggi;
    }
    const word& name() const { return name_; }
    const labelList& faceCells() const { return faceCells_; }
    label size() const { return (label)faceCells_.size(); }
    bool master() const { return master_; }
    bool coupled() const { return shadow_ != nullptr; }
    const regionCouplePolyPatch& shadow() const
    {
        if (!shadow_) throw FatalError("regionCouple patch " + name_ + " is not coupled");
        return *shadow_;
    }
    const GGIInterpolation& patchToPatch() const
    {
        if (!ggi_) throw FatalError("regionCouple patch " + name_ + " has no interpolator");
        return *ggi_;
    }
    // this side's face values from the shadow side's face values
    scalarField interpolate(const scalarField& shadowFaceValues) const
    {
        const GGIInterpolation& g = patchToPatch();
        const labelListList& addr = master_ ? g.masterAddr() : g.slaveAddr();
        const scalarListList& w = master_ ? g.masterWeights() : g.slaveWeights();
        scalarField out(faceCells_.size(), 0.0);
        for (size_t i = 0; i < out.size(); ++i)
            for (size_t k = 0; k < addr[i].size(); ++k) out[i] += w[i][k] * shadowFaceValues[addr[i][k]];
        return out;
    }

private:
    word name_;
    labelList faceCells_;
    bool master_;
    const regionCouplePolyPatch* shadow_ = nullptr;
    const GGIInterpolation* ggi_ = nullptr;
};

// The matrix interface of a monolithically coupled patch field
// (monolithicCouplingFvPatchField as an lduInterfaceField): its regionCouple
// patch; the coefficients come separately, as coupleBouCoeffs /
// coupleIntCoeffs.
class lduInterfaceField {
public:
    explicit lduInterfaceField(const regionCouplePolyPatch& patch) : patch_(&patch) {}
    const regionCouplePolyPatch& regionCouplePatch() const { return *patch_; }

private:
    const regionCouplePolyPatch* patch_;
};
typedef std::vector<const lduInterfaceField*> lduInterfaceFieldPtrsList;
typedef std::vector<scalarField> FieldField;  // per-interface coefficients

class lduMatrix {
public:
    explicit lduMatrix(const lduAddressing& a) : addr_(a) {}
    explicit lduMatrix(const lduMesh& m) : addr_(m.lduAddr()), mesh_(&m) {}
    const lduAddressing& lduAddr() const { return addr_; }
    const lduMesh& mesh() const
    {
        if (!mesh_) throw FatalError("lduMatrix: built on bare addressing, no mesh");
        return *mesh_;
    }
    bool hasMesh() const { return mesh_ != nullptr; }
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
    const lduMesh* mesh_ = nullptr;
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

// ---- the coupled (multi-region) matrix form --------------------------
// coupledLduMatrix: the region matrices of a coupledFvMatrix, row r being
// region r's lduMatrix; they couple only through their interfaces, whose
// shadow patches lie in other rows (multiRegionSystem.C:85-153 assembles
// one per coupled field and solves it with solver(fld + "coupled")).
class coupledLduMatrix {
public:
    void append(const lduMatrix& m) { rows_.push_back(&m); }
    label size() const { return (label)rows_.size(); }
    const lduMatrix& operator[](label r) const { return *rows_[r]; }
    bool symmetric() const
    {
        for (const lduMatrix* m : rows_)
            if (!m->symmetric()) return false;
        return true;
    }

private:
    std::vector<const lduMatrix*> rows_;
};
typedef std::vector<FieldField> FieldFieldList;                          // PtrList<FieldField<Field, scalar>>
typedef std::vector<lduInterfaceFieldPtrsList> lduInterfaceFieldPtrsListList;

// coupledLduSolver: run-time selected by the "solver" word of the
// "<fld>coupled" dictionary, from the symMatrix or asymMatrix table.
class coupledLduSolver {
public:
    struct coupledSolverPerformance {
        word solverName, fieldName;
        scalar initialResidual = 0, finalResidual = 0;
        label nIterations = 0;
        bool converged = false, singular = false;
    };
    typedef std::function<std::unique_ptr<coupledLduSolver>(const word&, const coupledLduMatrix&,
                                                            const FieldFieldList&, const FieldFieldList&,
                                                            const lduInterfaceFieldPtrsListList&,
                                                            const dictionary&)>
        ctor;
    coupledLduSolver(const word& fieldName, const coupledLduMatrix& matrix, const FieldFieldList& bouCoeffs,
                     const FieldFieldList& intCoeffs, const lduInterfaceFieldPtrsListList& interfaces,
                     const dictionary& dict)
        : fieldName_(fieldName), matrix_(matrix), bouCoeffs_(bouCoeffs), intCoeffs_(intCoeffs),
          interfaces_(interfaces), dict_(dict)
    {
        tolerance_ = dict.lookupOrDefault("tolerance", 1e-6);
        relTol_ = dict.lookupOrDefault("relTol", 0.0);
        minIter_ = (label)dict.lookupOrDefault("minIter", 0);
        maxIter_ = (label)dict.lookupOrDefault("maxIter", 1000);
    }
    virtual ~coupledLduSolver() = default;
    // x[r], b[r]: region r's field and source
    virtual coupledSolverPerformance solve(FieldField& x, const FieldField& b, const direction cmpt = 0) const = 0;

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
    static std::unique_ptr<coupledLduSolver> New(const word& fieldName, const coupledLduMatrix& matrix,
                                                 const FieldFieldList& bou, const FieldFieldList& intc,
                                                 const lduInterfaceFieldPtrsListList& ifs, const dictionary& dict)
    {
        const word name = dict.lookupWord("solver");
        auto& table = matrix.symmetric() ? symMatrixConstructorTable() : asymMatrixConstructorTable();
        auto it = table.find(name);
        if (it == table.end())
            throw FatalError("Unknown " + std::string(matrix.symmetric() ? "symmetric" : "asymmetric") +
                             " coupled matrix solver " + name);
        return it->second(fieldName, matrix, bou, intc, ifs, dict);
    }

protected:
    word fieldName_;
    const coupledLduMatrix& matrix_;
    const FieldFieldList& bouCoeffs_;
    const FieldFieldList& intCoeffs_;
    const lduInterfaceFieldPtrsListList& interfaces_;
    dictionary dict_;
    scalar tolerance_, relTol_;
    label minIter_, maxIter_;
};

template <class Type>
struct addSymCoupledSolver {
    explicit addSymCoupledSolver(const word& name)
    {
        coupledLduSolver::symMatrixConstructorTable()[name] =
            [](const word& f, const coupledLduMatrix& m, const FieldFieldList& b, const FieldFieldList& i,
               const lduInterfaceFieldPtrsListList& ifs, const dictionary& c) {
                return std::unique_ptr<coupledLduSolver>(new Type(f, m, b, i, ifs, c));
            };
    }
};
template <class Type>
struct addAsymCoupledSolver {
    explicit addAsymCoupledSolver(const word& name)
    {
        coupledLduSolver::asymMatrixConstructorTable()[name] =
            [](const word& f, const coupledLduMatrix& m, const FieldFieldList& b, const FieldFieldList& i,
               const lduInterfaceFieldPtrsListList& ifs, const dictionary& c) {
                return std::unique_ptr<coupledLduSolver>(new Type(f, m, b, i, ifs, c));
            };
    }
};

}  // namespace Foam
