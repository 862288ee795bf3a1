// noalloc.h -- the residual entry point that allocates no device memory
// (noalloc.cu); throws mrg::Error like the engine's functions.
#pragma once

namespace mrg {

void residual_noalloc(int n_cells, int n_faces, const int* lower_addr, const int* upper_addr,
                      const int* owner_start, const int* losort, const int* losort_start, const double* diag,
                      const double* upper, const double* lower, const double* b, const double* x, void* stream,
                      double* residual, double* norm_factor);

}  // namespace mrg
