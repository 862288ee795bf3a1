// mono.h -- monolithic interface coefficients on the device.
#pragma once
#include <cstdint>
#include <vector>

#include "engine.h"

namespace mrg {

// One side of a monolithic interface (a regionCouple patch and what the
// monolithic boundary conditions read from it).
struct MonoSide {
    int n_cells = 0, n_faces = 0;
    int32_t* face_cells = nullptr;                  // [n_faces]
    double *w = nullptr, *mld = nullptr, *dc = nullptr, *sf = nullptr;   // weights, magLongDelta, deltaCoeffs, magSf
    int32_t *src_ptr = nullptr, *src_face = nullptr;  // GGI from the other side's faces
    double* src_w = nullptr;
    int32_t *cell_ptr = nullptr, *cell_face = nullptr, *cells = nullptr;  // faces grouped by cell, face order
    int n_groups = 0;
    double* s = nullptr;                              // [n_faces] source scratch
};

struct Mono {
    Ctx* ctx = nullptr;
    MonoSide side[2];
    ~Mono();
};

struct MonoPatchHost {
    int n_cells, n_faces;
    const int32_t* face_cells;
    const double *weights, *mag_long_delta, *delta_coeffs, *mag_sf;
    const int32_t *src_ptr, *src_face;
    const double* src_weight;
};

void mono_create(Mono& m, Ctx* c, const MonoPatchHost& a, const MonoPatchHost& b);
// calcThermalDiffusivity and calcTemperature of one side: k and Tw per face.
void mono_update(Mono& m, int side, const double* T_own, const double* T_nbr, const double* f_own,
                 const double* f_nbr, const double* Qr_own, const double* Qr_nbr, double* k, double* Tw);
// monolithicTemperature::source + manipulateMatrix: b[faceCells] += s magSf.
void mono_source(Mono& m, int side, const double* T_own, const double* T_nbr, const double* Tw, const double* kw,
                 const double* f_own, double* b);

}  // namespace mrg
