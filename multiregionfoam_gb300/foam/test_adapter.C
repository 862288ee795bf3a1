// test_adapter.C -- drives the lduMatrix::solver adapters the way
// fvMatrix::solve does: build the matrix, select the solver by the
// fvSolution "solver" word through the run-time table, call solve(psi,
// source).  Used by the GPU tests; reads one system from a binary file.
//
// usage: test_adapter <system.bin> <solver> <preconditioner> <tolerance> <out.bin>
// system.bin: int32 n, nf, ni, has_lower, nsrc; int32 lower[nf], upper[nf];
//             f64 diag[n], upper_c[nf], (lower_c[nf]); f64 b[n], x0[n];
//             int32 cells[ni], ptr[ni+1], src[nsrc]; f64 w[nsrc], bou[ni]
// out.bin:    f64 x[n] after the second solve.
#include <cstdio>
#include <cstdlib>
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

int main(int argc, char** argv)
{
    if (argc < 6) {
        fprintf(stderr, "usage: %s system.bin solver preconditioner tolerance out.bin [key=value ...]\n", argv[0]);
        return 2;
    }
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    std::vector<int32_t> hdr = readv<int32_t>(f, 5);
    const int n = hdr[0], nf = hdr[1], ni = hdr[2], hasLower = hdr[3], nsrc = hdr[4];
    labelList lower = readv<int32_t>(f, nf), upper = readv<int32_t>(f, nf);
    lduAddressing addr(n, lower, upper);
    lduMatrix A(addr);
    A.diag() = readv<double>(f, n);
    A.upper() = readv<double>(f, nf);
    if (hasLower) A.lower() = readv<double>(f, nf);
    scalarField b = readv<double>(f, n), x0 = readv<double>(f, n);
    lduInterfaceField iface;
    FieldField bou, intc;
    lduInterfaceFieldPtrsList ifs;
    if (ni > 0) {
        iface.faceCells = readv<int32_t>(f, ni);
        iface.srcPtr = readv<int32_t>(f, ni + 1);
        iface.srcCells = readv<int32_t>(f, nsrc);
        iface.srcWeights = readv<double>(f, nsrc);
        bou.push_back(readv<double>(f, ni));
        intc = bou;
        ifs.push_back(&iface);
    }
    fclose(f);

    dictionary controls;
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

    lduMatrix::solverPerformance perf;
    scalarField x;
    try {
        for (int rep = 0; rep < 2; ++rep) {  // second solve reuses the resident addressing
            x = x0;
            auto s = lduMatrix::solver::New("T", A, bou, intc, ifs, controls);
            perf = s->solve(x, b);
        }
    } catch (const FatalError& e) {
        printf("{\"error\": \"%s\"}\n", e.what());
        return 1;
    }
    FILE* o = fopen(argv[5], "wb");
    fwrite(x.data(), sizeof(double), x.size(), o);
    fclose(o);
    printf("{\"solver\": \"%s\", \"initial_residual\": %.17g, \"final_residual\": %.17g, \"n_iter\": %d, "
           "\"converged\": %d}\n",
           perf.solverName.c_str(), perf.initialResidual, perf.finalResidual, perf.nIterations, (int)perf.converged);
    return 0;
}
