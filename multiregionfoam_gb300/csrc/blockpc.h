// blockpc.h -- the block (bs x bs) incomplete factorisation preconditioner
// of a block-expanded system (foam-extend's block Cholesky preconditioner of
// BlockLduSolver, the preconditioner fvBlockMatrix<vectorN>::solve selects).
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "dev.h"

namespace mrg {

struct Ctx;
struct Mesh;
struct PlanState;

// The block structure of a mesh (mrg_mesh_set_blocks): the cell mesh's exact
// plan and the block entries' places among the scalar coefficients, on the
// device.
struct BlockHost {
    Ctx* ctx = nullptr;
    int bs = 0, n = 0, nf = 0, nchunks = 0;
    std::vector<int32_t> perm;   // internal cell -> caller cell (host copy, for the vector maps)
    int32_t *d_perm = nullptr, *chunk_start = nullptr;
    int32_t *f_sptr = nullptr, *f_col = nullptr, *f_src = nullptr;
    int32_t *b_sptr = nullptr, *b_col = nullptr, *b_src = nullptr;
    int32_t *dmap = nullptr, *fmap = nullptr;
    double *D = nullptr, *U = nullptr, *L = nullptr;
    ~BlockHost();
};

// The block view of one plan (its vector numbering): the maps above plus the
// (cell, component) -> scalar internal row map and the factor.
struct BlockView {
    Ctx* ctx = nullptr;
    BlockDev h{};
    BlockDev* d = nullptr;
    int32_t* vmap = nullptr;
    double* dD = nullptr;
    ~BlockView();
};

// Declare mesh m the bs-expansion (mrg_block_addressing) of the cell mesh
// (n cells, nf faces, lower / upper); throws Error when it is not.
void set_blocks(Mesh& m, int bs, int n, int nf, const int32_t* lower, const int32_t* upper);

// The block view of plan P of mesh m (built at the first call).
BlockView& block_view(Mesh& m, PlanState& P);

}  // namespace mrg
