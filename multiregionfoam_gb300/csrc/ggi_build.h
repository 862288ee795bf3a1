// ggi_build.h -- GGI interface weights built on the device.
#pragma once
#include <cstdint>

#include "engine.h"

namespace mrg {

// Overlap weights between two planar patches of convex faces (2-D vertex
// lists, counter-clockwise, 3 to 32 vertices a face; ptr[0] = 0).  Fills
// a_from_b (rows = A faces, ascending B face) and b_from_a (rows = B faces,
// ascending A face): intersection area / receiving face area, rescaled so
// every covered face's weights sum to one; pairs whose overlap is at most
// tol * min(face areas) are dropped.  Throws Error on bad input or when an
// A face has more than 256 candidate B faces.
void ggi_build(Ctx* c, int na, const int32_t* a_ptr, const double* a_xy, int nb, const int32_t* b_ptr,
               const double* b_xy, double tol, Ggi& a_from_b, Ggi& b_from_a);

// directMapInterfaceToInterfaceMapping's conformal face maps
// (directMapInterfaceToInterfaceMapping.C:147-190 and :244-290): for every
// face of one patch the first face of the other (in face order) whose centre
// lies within tol (|c_B - c_A| < tol; the reference takes tol = 0.001 x the
// smallest edge length of the two patches), as one-weight GGIs: a_from_b
// (each A face's B partner) and b_from_a.  Centres are (x, y, z) triples.
// Throws Error (MRG_E_INVALID) when the patch sizes differ or a face has no
// partner ("interfaces are not conformal").
void direct_map_build(Ctx* c, int na, const double* a_centres, int nb, const double* b_centres, double tol,
                      Ggi& a_from_b, Ggi& b_from_a);

}  // namespace mrg
