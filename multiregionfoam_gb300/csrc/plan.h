// plan.h -- host-side layout planning for one LDU mesh (addressing only).
//
// A plan fixes, for one cell ordering, everything the kernels need that does
// not depend on the coefficient values:
//   * the internal row order (perm: internal row -> caller's cell),
//   * the Amul/Tmul rows as a sliced ELL (32-row slices, column-major inside
//     a slice) with the entries of every row in ascending foam face order,
//     followed by the row's interface entries in interface order -- the
//     accumulation order of lduMatrix::Amul + updateMatrixInterfaces,
//   * the preconditioner sweep structure: chunks of <= 32 rows that share a
//     sweep level, and per chunk a sliced ELL of forward dependencies
//     (ascending face order) and backward dependencies (descending face
//     order) -- the per-cell order of foam's face-ordered DIC/DILU sweeps,
//   * the general (non-conformal) interface faces as a GGI gather CSR.
//
// Coefficient "source" codes used by the scatter kernels:
//   s in [0,F)        -> upper[s]            (A[lowerAddr][upperAddr])
//   s in [F,2F)       -> lower[s-F]          (A[upperAddr][lowerAddr])
//   s in [2F,2F+NI)   -> -iface_coeff[s-2F]  (bou for Amul, int for Tmul)
//   s = -1            -> padding
// The transpose of a face source swaps the two halves.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace mrg {

constexpr int kSlice = 32;     // rows per ELL slice (one warp)
constexpr int kTileRows = 1024; // rows per reduction tile

struct IfaceHost {
    // Flattened over patches.
    std::vector<int32_t> cells;  // faceCells
    std::vector<int32_t> ptr;    // CSR into src/w
    std::vector<int32_t> src;    // shadow cells
    std::vector<double> w;       // GGI weights
    int size() const { return (int)cells.size(); }
};

struct PlanHost {
    int n = 0, npad = 0, nf = 0, ni = 0;
    int ordering = 0;
    int nlevels = 0, nchunks = 0;
    int ngen = 0;  // general interface faces (gathered into x[npad + j])
    std::vector<int32_t> perm, iperm, level_of_row;
    // Amul sliced ELL: npad/32 slices
    std::vector<int32_t> a_sptr, a_col, a_src;
    // the same column indices as 16-bit offsets from a per-slice base, for
    // every round of 8 slices (256 rows) whose slices all span at most
    // 65,535 columns (0xFFFF marks padding); a_cbase[slice] is the base, or
    // -1 for the 8 slices of a round that keeps 32-bit columns
    std::vector<uint16_t> a_col16;
    std::vector<int32_t> a_cbase;
    // sweep chunks
    std::vector<int32_t> chunk_start;  // [nchunks+1]
    std::vector<int32_t> lvl_chunk;    // [nlevels+1]
    std::vector<int32_t> f_sptr, f_col, f_src;  // forward deps, per chunk
    std::vector<int32_t> b_sptr, b_col, b_src;  // backward deps, per chunk
    // general interface gather
    std::vector<int32_t> g_ptr, g_src;
    std::vector<double> g_w;
    int max_row_len = 0;
    // exact plans, owner-computes sweeps (build_parts): the caller's cells
    // cut into nparts ranges of part_cells cells; part p's rows are
    // part_rows[pt_ptr[p] .. pt_ptr[p + 1]) in level order, part_step the
    // ordinal of each one's level among the part's levels; f_loc / b_loc: per
    // sweep dependency entry, the dependency's cell offset in the row's own
    // part, or -1; f_row / b_row: per row (first entry of the row, entries)
    int nparts = 0, part_cells = 0;
    std::vector<int32_t> pt_ptr, part_rows, part_step, f_loc, b_loc, f_row, b_row;
};

// Owner-computes partition of an exact plan (see PlanHost): nparts ranges of
// ceil(n / nparts) caller cells.
void build_parts(PlanHost& P, int nparts);

// Validates the addressing; returns "" on success, else a message.
std::string validate_addressing(int n, int nf, const int32_t* lower,
                                const int32_t* upper, const IfaceHost& ifc);

// ordering: 0 = exact (level order of foam's face-ordered sweeps),
//           1 = greedy multi-colour.
PlanHost build_plan(int n, int nf, const int32_t* lower, const int32_t* upper,
                    const IfaceHost& ifc, int ordering);

}  // namespace mrg
