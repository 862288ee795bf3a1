// noalloc.h -- the residual entry point that allocates no device memory
// (noalloc.cu); throws mrg::Error like the engine's functions.
#pragma once
#include <cstdint>

namespace mrg {

void residual_noalloc(int n_cells, int n_faces, const int32_t* lower_addr, const int32_t* upper_addr,
                      const int32_t* owner_start, const int32_t* losort, const int32_t* losort_start, const double* diag,
                      const double* upper, const double* lower, const double* b, const double* x, void* stream,
                      double* residual, double* norm_factor);

}  // namespace mrg
