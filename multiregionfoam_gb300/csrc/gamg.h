// gamg.h -- GAMG solver (foam-order Gauss-Seidel smoothing) on the device.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "engine.h"

namespace mrg {

// One coarse level: how its coefficients and vectors come from the finer one.
struct GamgLevel {
    int n = 0, nf = 0;
    bool top = false;                                  // the coarsest: solved directly, caller numbering
    std::unique_ptr<Mesh> mesh;                        // smoothed levels: addressing + foam-order plan
    std::vector<int32_t> agg;                          // finer caller cell -> this level's cell
    std::vector<std::vector<int32_t>> members;         // this level's cell -> finer cells (ascending)
    // coefficient restriction (caller numbering of both levels)
    int32_t *mem_ptr = nullptr, *mem_idx = nullptr;    // cell -> finer cells
    int32_t *int_ptr = nullptr, *int_idx = nullptr;    // cell -> finer faces inside it
    int32_t *fc_ptr = nullptr, *fc_idx = nullptr, *fc_flip = nullptr;   // face -> finer faces (+ flip)
    double *diag = nullptr, *upper = nullptr, *lower = nullptr;         // this level's raw coefficients
    // vector transfer (plan numbering; the coarsest's own is its caller numbering)
    int32_t *r_ptr = nullptr, *r_idx = nullptr;        // restriction: row -> finer rows
    int32_t* p_map = nullptr;                          // prolongation: finer row -> row
    int32_t *lo_dev = nullptr, *up_dev = nullptr;      // the coarsest's addressing (dense solve)
    bool maps = false;
};

struct Gamg {
    Ctx* ctx = nullptr;
    int n_coarsest = 10;
    int agglomerator = 0;                              // MRG_AGGLOMERATOR_* the hierarchy was built with
    uint64_t weights_version = 0;                      // the mesh's face-area version it was built from
    bool sym = true;
    bool identity = false;                             // no level kept: the matrix is the coarsest
    std::vector<GamgLevel> lv;                         // lv[0]: the finest (the caller's mesh), unused
    double *lu = nullptr, *src_top = nullptr, *c_top = nullptr;
    Scal** d_coarse_sc = nullptr;                      // the smoothed levels' scalar states
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        long long nodes = 0;
    };
    std::map<std::string, Graph> graphs;               // captured V-cycles
    ~Gamg();
};

// GAMG solve of a mesh (FP64, foam-order smoothing); b and x device arrays
// in the caller's numbering.  The hierarchy is built at the first call (or
// when nCellsInCoarsestLevel, the agglomerator or the face areas change)
// from the current coefficients or the mesh's face areas.
Perf gamg_solve(Mesh& m, const double* d_b, double* d_x, const Controls& cfg);

// faceAreaPair weights of faces with area vectors sf[3 f .. 3 f + 2].
std::vector<double> face_area_weights(const double* sf, int nf);

}  // namespace mrg
