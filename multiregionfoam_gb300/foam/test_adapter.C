// test_adapter.C -- drives the solver adapters the way foam-extend does:
// build the matrices and the regionCouple interface pair, select the solver
// by the dictionary's "solver" word through the run-time table, solve.
//
//   one matrix (R = 1): lduMatrix::solver::New(...)->solve(psi, source), as
//     fvMatrix::solve calls it (multiRegionSystem.C:293);
//   two region matrices (R = 2): coupledLduSolver::New(...)->solve(x, b),
//     as coupledFvMatrix::solve calls it for solver(fld + "coupled")
//     (multiRegionSystem.C:150-153).
//
// usage: test_adapter <system.bin> <solver> <preconditioner> <tolerance> <out.bin> [key=value ...]
//        test_adapter --dict <file> <entry> <system.bin> <out.bin>
//          (the controls are the sub-dictionary <entry> of <file>, foam syntax)
//        test_adapter --print-dict <file> <entry>
//          (prints the controls read from that entry; no GPU)
// system.bin: int32 R; per region: int32 n, nf, has_lower; int32 lower[nf],
//             upper[nf]; f64 diag[n], upper_c[nf], (lower_c[nf]), b[n], x0[n];
//             int32 nsf (0, or nf: the matrix is built on an fvMesh with
//             these face area vectors), f64 sf[3 * nsf];
//             int32 npatch (0 or 2); with 2 (a master patch A and its slave
//             shadow B): int32 regionA, regionB, nA, nB; int32 cellsA[nA],
//             cellsB[nB]; A's interpolator from B (masterAddr / masterWeights
//             as CSR): int32 ptr[nA+1], addr[ptr[nA]], f64 w[ptr[nA]]; B's
//             from A (slaveAddr / slaveWeights): int32 ptr[nB+1], addr, f64 w;
//             f64 bouA[nA], bouB[nB] (coupleBouCoeffs = coupleIntCoeffs)
// out.bin:    f64 x (regions concatenated) after the second solve.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <vector>

#include "lduMatrix.H"

using namespace Foam;

template <class T>
static std::vector<T> readv(FILE* f, size_t n)
{
    std::vector<T> v(n);
    if (n && fread(v.data(), sizeof(T), n, f) != n) {
        fprintf(stderr, "short read\n");
        exit(2);
    }
    return v;
}

struct Region {
    std::unique_ptr<lduAddressing> addr;
    std::unique_ptr<fvMesh> mesh;
    std::unique_ptr<lduMatrix> A;
    scalarField b, x0;
};

// CSR -> list of lists
template <class T>
static std::vector<std::vector<T>> lists(const std::vector<int32_t>& ptr, const std::vector<T>& v)
{
    std::vector<std::vector<T>> out(ptr.size() - 1);
    for (size_t i = 0; i + 1 < ptr.size(); ++i) out[i].assign(v.begin() + ptr[i], v.begin() + ptr[i + 1]);
    return out;
}

int main(int argc, char** argv)
{
    std::string sysPath, outPath;
    dictionary controls;
    if (argc == 4 && std::strcmp(argv[1], "--print-dict") == 0) {
        // the controls the adapters would read from entry argv[3] of file
        // argv[2] (no GPU is touched)
        std::ifstream in(argv[2]);
        std::stringstream ss;
        ss << in.rdbuf();
        try {
            const dictionary d = dictionary::parse(ss.str()).subDict(argv[3]);
            const word pc = d.isDict("preconditioner")
                                ? d.subDict("preconditioner").lookupWord("preconditioner", "none")
                                : d.lookupWord("preconditioner", "none");
            printf("{\"solver\": \"%s\", \"preconditioner\": \"%s\", \"nested\": %d, \"tolerance\": %.17g, "
                   "\"relTol\": %.17g, \"minIter\": %g, \"maxIter\": %g}\n",
                   d.lookupWord("solver").c_str(), pc.c_str(), (int)d.isDict("preconditioner"),
                   d.lookupOrDefault("tolerance", -1.0), d.lookupOrDefault("relTol", -1.0),
                   d.lookupOrDefault("minIter", -1.0), d.lookupOrDefault("maxIter", -1.0));
        } catch (const FatalError& e) {
            printf("{\"error\": \"%s\"}\n", e.what());
            return 1;
        }
        return 0;
    }
    if (argc >= 6 && std::strcmp(argv[1], "--dict") == 0) {
        std::ifstream in(argv[2]);
        std::stringstream ss;
        ss << in.rdbuf();
        try {
            controls = dictionary::parse(ss.str()).subDict(argv[3]);
        } catch (const FatalError& e) {
            printf("{\"error\": \"%s\"}\n", e.what());
            return 1;
        }
        sysPath = argv[4];
        outPath = argv[5];
    } else if (argc >= 6) {
        sysPath = argv[1];
        outPath = argv[5];
        controls.set("solver", std::string(argv[2]));
        controls.set("preconditioner", std::string(argv[3]));
        controls.set("tolerance", atof(argv[4]));
        controls.set("relTol", 0.0);
        controls.set("maxIter", 5000.0);
        for (int a = 6; a < argc; ++a) {   // further fvSolution entries: key=value (a number or a word)
            const std::string kv(argv[a]);
            const size_t eq = kv.find('=');
            if (eq == std::string::npos) return 2;
            const std::string k = kv.substr(0, eq), v = kv.substr(eq + 1);
            char* end = nullptr;
            const double d = strtod(v.c_str(), &end);
            if (end && *end == '\0' && !v.empty())
                controls.set(k, d);
            else
                controls.set(k, v);
        }
    } else {
        fprintf(stderr,
                "usage: %s system.bin solver preconditioner tolerance out.bin [key=value ...]\n"
                "       %s --dict file entry system.bin out.bin\n",
                argv[0], argv[0]);
        return 2;
    }

    FILE* f = fopen(sysPath.c_str(), "rb");
    if (!f) return 2;
    const int R = readv<int32_t>(f, 1)[0];
    if (R < 1 || R > 2) return 2;
    std::vector<Region> regions(R);
    for (Region& g : regions) {
        std::vector<int32_t> hdr = readv<int32_t>(f, 3);
        const int n = hdr[0], nf = hdr[1], hasLower = hdr[2];
        labelList lower = readv<int32_t>(f, nf), upper = readv<int32_t>(f, nf);
        g.addr.reset(new lduAddressing(n, lower, upper));
        scalarField diag = readv<double>(f, n), up = readv<double>(f, nf), lo;
        if (hasLower) lo = readv<double>(f, nf);
        g.b = readv<double>(f, n);
        g.x0 = readv<double>(f, n);
        const int nsf = readv<int32_t>(f, 1)[0];
        if (nsf != 0 && nsf != nf) return 2;
        if (nsf) {
            std::vector<double> sf = readv<double>(f, 3 * (size_t)nsf);
            vectorField Sf;
            for (int k = 0; k < nsf; ++k) Sf.emplace_back(sf[3 * k], sf[3 * k + 1], sf[3 * k + 2]);
            g.mesh.reset(new fvMesh(*g.addr, std::move(Sf)));
            g.A.reset(new lduMatrix(*g.mesh));
        } else {
            g.A.reset(new lduMatrix(*g.addr));
        }
        g.A->diag() = diag;
        g.A->upper() = up;
        if (hasLower) g.A->lower() = lo;
    }
    const int npatch = readv<int32_t>(f, 1)[0];
    std::unique_ptr<regionCouplePolyPatch> pa, pb;
    std::unique_ptr<GGIInterpolation> ggi;
    std::unique_ptr<lduInterfaceField> ia, ib;
    FieldFieldList bou(R), intc(R);
    lduInterfaceFieldPtrsListList ifs(R);
    if (npatch == 2) {
        std::vector<int32_t> h = readv<int32_t>(f, 4);
        const int ra = h[0], rb = h[1], na = h[2], nb = h[3];
        if (ra < 0 || ra >= R || rb < 0 || rb >= R) return 2;
        labelList ca = readv<int32_t>(f, na), cb = readv<int32_t>(f, nb);
        std::vector<int32_t> mptr = readv<int32_t>(f, na + 1);
        std::vector<int32_t> maddr = readv<int32_t>(f, mptr.back());
        std::vector<double> mw = readv<double>(f, mptr.back());
        std::vector<int32_t> sptr = readv<int32_t>(f, nb + 1);
        std::vector<int32_t> saddr = readv<int32_t>(f, sptr.back());
        std::vector<double> sw = readv<double>(f, sptr.back());
        ggi.reset(new GGIInterpolation(lists(mptr, maddr), lists(mptr, mw), lists(sptr, saddr), lists(sptr, sw)));
        pa.reset(new regionCouplePolyPatch("interfaceA", ca, true));
        pb.reset(new regionCouplePolyPatch("interfaceB", cb, false));
        regionCouplePolyPatch::couple(*pa, *pb, *ggi);
        ia.reset(new lduInterfaceField(*pa));
        ib.reset(new lduInterfaceField(*pb));
        ifs[ra].push_back(ia.get());
        bou[ra].push_back(readv<double>(f, na));
        ifs[rb].push_back(ib.get());
        bou[rb].push_back(readv<double>(f, nb));
        intc = bou;
    } else if (npatch != 0) {
        return 2;
    }
    fclose(f);

    std::vector<double> x;
    std::string name;
    double r0 = 0, r1 = 0;
    int nIter = 0, converged = 0;
    try {
        for (int rep = 0; rep < 2; ++rep) {  // the second solve reuses the resident addressing
            if (R == 1) {
                scalarField psi = regions[0].x0;
                auto s = lduMatrix::solver::New("T", *regions[0].A, bou[0], intc[0], ifs[0], controls);
                const lduMatrix::solverPerformance p = s->solve(psi, regions[0].b);
                x = psi;
                name = p.solverName;
                r0 = p.initialResidual;
                r1 = p.finalResidual;
                nIter = p.nIterations;
                converged = p.converged;
            } else {
                coupledLduMatrix M;
                FieldField X, B;
                for (Region& g : regions) {
                    M.append(*g.A);
                    X.push_back(g.x0);
                    B.push_back(g.b);
                }
                auto s = coupledLduSolver::New("T", M, bou, intc, ifs, controls);
                const coupledLduSolver::coupledSolverPerformance p = s->solve(X, B);
                x.clear();
                for (const scalarField& xr : X) x.insert(x.end(), xr.begin(), xr.end());
                name = p.solverName;
                r0 = p.initialResidual;
                r1 = p.finalResidual;
                nIter = p.nIterations;
                converged = p.converged;
            }
        }
    } catch (const FatalError& e) {
        printf("{\"error\": \"%s\"}\n", e.what());
        return 1;
    }
    FILE* o = fopen(outPath.c_str(), "wb");
    fwrite(x.data(), sizeof(double), x.size(), o);
    fclose(o);
    printf("{\"solver\": \"%s\", \"initial_residual\": %.17g, \"final_residual\": %.17g, \"n_iter\": %d, "
           "\"converged\": %d}\n",
           name.c_str(), r0, r1, nIter, converged);
    return 0;
}
