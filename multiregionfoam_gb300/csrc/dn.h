// dn.h -- device-resident partitioned Dirichlet-Neumann interface coupling
// (dn.cu).  Region A carries the jump (Dirichlet) patch, region B the flux
// (Neumann) patch; every array below is device memory owned by the object.
#pragma once
#include <cstdint>

#include "engine.h"

namespace mrg {

// IQN-ILS modes kept per side; once full, the oldest column is dropped.
constexpr int kIqnModes = 32;

struct Dn {
    Ctx* ctx = nullptr;
    int na = 0, nb = 0, ncells_a = 0, ncells_b = 0, nca = 0, ncb = 0, model = 1;
    double K = 1.0, flux_jump = 0.0, relax = 1.0;
    int32_t *fc_a = nullptr, *fc_b = nullptr;
    double *delta_a = nullptr, *k_a = nullptr, *area_a = nullptr;
    double *delta_b = nullptr, *k_b = nullptr, *area_b = nullptr;
    int32_t *pa = nullptr, *xa = nullptr, *pb = nullptr, *xb = nullptr;
    double *wa = nullptr, *wb = nullptr;
    int *ca_ptr = nullptr, *ca_face = nullptr, *ca_cell = nullptr;
    int *cb_ptr = nullptr, *cb_face = nullptr, *cb_cell = nullptr;
    double *value_a = nullptr, *grad_b = nullptr;
    double *prev_a = nullptr, *res_a = nullptr, *pres_a = nullptr;
    double *prev_b = nullptr, *res_b = nullptr, *pres_b = nullptr;
    double *tmp_a = nullptr, *tmp_b = nullptr;
    double* scal = nullptr;
    int* corr = nullptr;     // [0] A, [1] B corrector counts, [2] time index
    // IQN-ILS (model 2), per side: kIqnModes columns of V (residual
    // differences) and W (field differences) in a ring, the Gram-Schmidt
    // workspace Q, the reference field and residual, the unrelaxed field,
    // the columns' time indices and (head, count) of the ring
    int reuse = 0;
    // flux side's own model, factor and couplingReuse (default: A's)
    int model_b = 1, reuse_b = 0;
    double relax_b = 1.0;
    double *iqn_v = nullptr, *iqn_w = nullptr, *iqn_q = nullptr;   // [2][modes][n_side]
    double *iqn_fref = nullptr, *iqn_rref = nullptr, *iqn_cur = nullptr;   // [2][n_side]
    int *iqn_t = nullptr, *iqn_ring = nullptr;   // [2][modes], [2][2]
    ~Dn();
};

Dn* dn_create(Ctx* c, int n_cells_a, int na, const int32_t* fc_a, const double* delta_a, const double* k_a,
              const double* area_a, int n_cells_b, int nb, const int32_t* fc_b, const double* delta_b,
              const double* k_b, const double* area_b, const int32_t* a_ptr, const int32_t* a_addr,
              const double* a_w, const int32_t* b_ptr, const int32_t* b_addr, const double* b_w, double K,
              double flux_jump, int model, double relax, int reuse = 0);
void dn_set_flux_relaxation(Dn& d, int model, double relax, int reuse);
void dn_set_state(Dn& d, const double* value_a, const double* grad_b);
void dn_new_time_step(Dn& d);
void dn_update_a(Dn& d, const double* d_t_b);
void dn_update_b(Dn& d, const double* d_t_a);
void dn_rhs(Dn& d, int side, const double* d_b0, double* d_b);
void dn_residuals(Dn& d, const double* d_t_a, const double* d_t_b, double* jump, double* flux);
void dn_get_state(Dn& d, double* value_a, double* grad_b, double* aitken);

}  // namespace mrg
