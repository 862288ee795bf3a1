// block.cpp -- block-coupled (bs x bs) LDU systems as scalar LDU systems.
//
// foam-extend's fvBlockMatrix<Type>::solve hands its BlockLduMatrix to
// BlockLduSolver<Type>::New(...)->solve (filesToReplace/fvBlockMatrix.C:
// 1360-1388; the pressure-velocity coupled region assembles a
// BlockLduMatrix<vector4>, pUCoupledIcoFluid.C:592-617).  Here cell c's
// component a becomes row bs c + a of a scalar LDU system with the same
// Amul: a block face f = (l, u) gives the bs^2 scalar faces (bs l + a,
// bs u + b) with upper U_f[a][b] (row l a, column u b) and lower L_f[b][a]
// (row u b, column l a); a diagonal block D_c gives the diagonal D_c[a][a]
// and, for a < b, the face (bs c + a, bs c + b) with upper D_c[a][b] and
// lower D_c[b][a].  The scalar faces are in upper-triangular order (owner
// row ascending, then neighbour), so every solver of the library applies.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/mrgpu.h"
#include "plan.h"

namespace mrg {
void set_last_error(const std::string& msg);
}

namespace {

// Scalar faces of the expansion in order, each with its source entry.
struct Expansion {
    int bs = 0;
    std::vector<int32_t> s_lower, s_upper;
    std::vector<int64_t> src;   // >= 0: face * bs^2 + a bs + b; < 0: -1 - (cell * bs^2 + a bs + b)
};

int check(int n, int nf, const int32_t* lower, const int32_t* upper, int bs)
{
    if (bs < 1 || bs > 8) {
        mrg::set_last_error("block size must be 1..8");
        return MRG_E_INVALID;
    }
    if (n < 0 || nf < 0 || (int64_t)n * bs > INT32_MAX ||
        (int64_t)nf * bs * bs + (int64_t)n * bs * (bs - 1) / 2 > INT32_MAX) {
        mrg::set_last_error("block system too large for int32 scalar addressing");
        return MRG_E_INVALID;
    }
    if (nf > 0 && (!lower || !upper)) {
        mrg::set_last_error("block addressing arrays are NULL");
        return MRG_E_INVALID;
    }
    mrg::IfaceHost none;
    none.ptr = {0};
    const std::string msg = mrg::validate_addressing(n, nf, lower, upper, none);
    if (!msg.empty()) {
        mrg::set_last_error("block addressing: " + msg);
        return MRG_E_INVALID;
    }
    return MRG_OK;
}

// want_addr: the scalar addressing; want_src: each scalar face's source
// entry (the coefficients need only the latter).
Expansion expand(int n, int nf, const int32_t* lower, const int32_t* upper, int bs, bool want_addr, bool want_src)
{
    // block faces of each owner, by neighbour
    std::vector<int32_t> start(n + 1, 0), own(nf);
    for (int f = 0; f < nf; ++f) ++start[lower[f] + 1];
    for (int c = 0; c < n; ++c) start[c + 1] += start[c];
    {
        std::vector<int32_t> fill(start.begin(), start.end() - 1);
        for (int f = 0; f < nf; ++f) own[fill[lower[f]]++] = f;
    }
    for (int c = 0; c < n; ++c)
        std::stable_sort(own.begin() + start[c], own.begin() + start[c + 1],
                         [&](int32_t x, int32_t y) { return upper[x] < upper[y]; });
    Expansion E;
    E.bs = bs;
    const size_t ns = (size_t)nf * bs * bs + (size_t)n * bs * (bs - 1) / 2;
    if (want_addr) {
        E.s_lower.reserve(ns);
        E.s_upper.reserve(ns);
    }
    if (want_src) E.src.reserve(ns);
    const int64_t bb = (int64_t)bs * bs;
    for (int c = 0; c < n; ++c)
        for (int a = 0; a < bs; ++a) {
            const int32_t row = c * bs + a;
            for (int b = a + 1; b < bs; ++b) {
                if (want_addr) {
                    E.s_lower.push_back(row);
                    E.s_upper.push_back(c * bs + b);
                }
                if (want_src) E.src.push_back(-1 - (c * bb + a * bs + b));
            }
            for (int k = start[c]; k < start[c + 1]; ++k) {
                const int f = own[k];
                for (int b = 0; b < bs; ++b) {
                    if (want_addr) {
                        E.s_lower.push_back(row);
                        E.s_upper.push_back(upper[f] * bs + b);
                    }
                    if (want_src) E.src.push_back(f * bb + a * bs + b);
                }
            }
        }
    return E;
}

}  // namespace

namespace mrg {
// The expansion's scalar addressing and each scalar face's source entry
// (for the block preconditioner's maps); "" on success, else a message.
std::string block_expansion(int n, int nf, const int32_t* lower, const int32_t* upper, int bs,
                            std::vector<int32_t>& s_lower, std::vector<int32_t>& s_upper, std::vector<int64_t>& src)
{
    if (check(n, nf, lower, upper, bs) != MRG_OK) return "invalid block addressing";
    Expansion E = expand(n, nf, lower, upper, bs, true, true);
    s_lower = std::move(E.s_lower);
    s_upper = std::move(E.s_upper);
    src = std::move(E.src);
    return "";
}
}  // namespace mrg

// ABI entries: clear the last error, turn a failed host allocation into
// MRG_E_OOM.
template <typename F>
int block_guard(F&& f)
{
    try {
        mrg::set_last_error("");
        return f();
    } catch (const std::bad_alloc&) {
        mrg::set_last_error("host allocation failed");
        return MRG_E_OOM;
    }
}

extern "C" {

int mrg_block_addressing(int n_cells, int n_faces, const int32_t* lower_addr, const int32_t* upper_addr, int bs,
                         int* n_faces_out, int32_t* s_lower, int32_t* s_upper)
{
    return block_guard([&]() -> int {
        const int st = check(n_cells, n_faces, lower_addr, upper_addr, bs);
        if (st != MRG_OK) return st;
        const int64_t ns = (int64_t)n_faces * bs * bs + (int64_t)n_cells * bs * (bs - 1) / 2;
        if (n_faces_out) *n_faces_out = (int)ns;
        if (!s_lower || !s_upper) return MRG_OK;
        const Expansion E = expand(n_cells, n_faces, lower_addr, upper_addr, bs, true, false);
        std::memcpy(s_lower, E.s_lower.data(), sizeof(int32_t) * E.s_lower.size());
        std::memcpy(s_upper, E.s_upper.data(), sizeof(int32_t) * E.s_upper.size());
        return MRG_OK;
    });
}

int mrg_block_coeffs(int n_cells, int n_faces, const int32_t* lower_addr, const int32_t* upper_addr, int bs,
                     const double* diag, const double* upper, const double* lower_or_null, double* s_diag,
                     double* s_upper, double* s_lower)
{
    return block_guard([&]() -> int {
        const int st = check(n_cells, n_faces, lower_addr, upper_addr, bs);
        if (st != MRG_OK) return st;
        if ((n_cells > 0 && (!diag || !s_diag)) || (n_faces > 0 && !upper) || !s_upper || !s_lower) {
            mrg::set_last_error("block coefficient arrays are NULL");
            return MRG_E_INVALID;
        }
        const int64_t bb = (int64_t)bs * bs;
        for (int c = 0; c < n_cells; ++c)
            for (int a = 0; a < bs; ++a) s_diag[c * bs + a] = diag[c * bb + a * bs + a];
        const Expansion E = expand(n_cells, n_faces, lower_addr, upper_addr, bs, false, true);
        for (size_t k = 0; k < E.src.size(); ++k) {
            const int64_t s = E.src[k];
            if (s < 0) {   // diagonal block's pair (a, b), a < b: upper D[a][b], lower D[b][a]
                const int64_t q = -1 - s, c = q / bb, a = (q % bb) / bs, b = q % bs;
                s_upper[k] = diag[c * bb + a * bs + b];
                s_lower[k] = diag[c * bb + b * bs + a];
            } else {       // block face f, (a, b): upper U_f[a][b], lower L_f[b][a] (NULL: U_f transposed)
                const int64_t f = s / bb, a = (s % bb) / bs, b = s % bs;
                s_upper[k] = upper[f * bb + a * bs + b];
                s_lower[k] = lower_or_null ? lower_or_null[f * bb + b * bs + a] : upper[f * bb + a * bs + b];
            }
        }
        return MRG_OK;
    });
}

}  // extern "C"
