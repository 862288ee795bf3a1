// dn.cu -- partitioned Dirichlet-Neumann interface coupling on the device.
//
// One DN-coupled interface between region A (jump / Dirichlet patch) and
// region B (flux / Neumann patch), following multiRegionFoam's
//   genericRegionCoupledJumpFvPatchField::updateCoeffs (.C:164-217) with
//     regionCoupledTemperatureJump::valueJump (.C:83-104): value_A = K * nbr
//   genericRegionCoupledFluxFvPatchField::updateCoeffs (.C:172-239) with
//     regionCoupledHeatFlux::fluxJump = 0 (.C:83-86):
//     grad_B = (-interp(k_A snGrad_A) + jump) / k_B
//   rawResidual / normResidual (Jump .C:244-332, Flux .C:241-409)
//   fixedRelaxation::relax (fixedRelaxation.C:76-101),
//   aitkenRelaxation::relax / updateAitkenFactor (aitkenRelaxation.C:74-100,
//     aitkenRelaxationTemplates.C:105-165) and
//   IQNILS::relax / updateVW / updateIQNILS (IQNILS.C:96-201,
//     IQNILSTemplates.C:44-133): quasi-Newton interface least squares with
//     the residual differences QR-factored by modified Gram-Schmidt
// The patch states, the relaxation history and the Aitken factors live on
// the device, so a DN coupling iteration (update A, solve A, update B,
// solve B, residuals) needs no host round trip except the two residual
// scalars read for the convergence test.  Patches are small (interface
// faces), so each update is one CTA that sums in a fixed order: results do
// not depend on the device.  Element-wise arithmetic uses explicit IEEE
// operations (no contraction) so that it matches a plain restatement.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/mrgpu.h"
#include "dn.h"
#include "kernels.h"

namespace mrg {
namespace {

constexpr int kDnBlock = 1024;
constexpr double kSmall = 1e-15;   // foam's SMALL

struct DnView {
    int na, nb, model, model_b;
    double K, flux_jump, init_relax, init_relax_b;
    const int *fc_a, *fc_b;
    const double *delta_a, *k_a, *area_a, *delta_b, *k_b, *area_b;
    const int *pa, *xa, *pb, *xb;       // GGI CSR: A faces from B faces, B faces from A faces
    const double *wa, *wb;
    const int *ca_ptr, *ca_face, *ca_cell, *cb_ptr, *cb_face, *cb_cell;   // faces per unique cell
    int nca, ncb;
    double *value_a, *grad_b;
    double *prev_a, *res_a, *pres_a, *prev_b, *res_b, *pres_b;
    double *tmp_a, *tmp_b;
    double* scal;   // [0] aitken_a, [1] aitken_b, [2] jump residual, [3] flux residual
    int* corr;      // [0] A, [1] B, [2] time index
    int reuse, reuse_b;
    double *iqn_v, *iqn_w, *iqn_q, *iqn_fref, *iqn_rref, *iqn_cur;
    int *iqn_t, *iqn_ring;
};

__device__ double dn_block_sum(double v, double* sh)
{
    // fixed-order tree over the CTA: result valid in every thread
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int s = kDnBlock / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] = __dadd_rn(sh[t], sh[t + s]);
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

__device__ double csr_row(const int* ptr, const int* addr, const double* w, const double* src, int i)
{
    double acc = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) acc = __dadd_rn(acc, __dmul_rn(w[k], src[addr[k]]));
    return acc;
}

// Relax n values cur[i] (already in res as cur - prev after the call) and
// write the relaxed field to out and prev.  side 0: A, 1: B.
__device__ void dn_relax(const DnView& D, int side, int n, double* prev, double* res, double* pres, double* out,
                         double* sh)
{
    __shared__ double s_w;
    const int model = side ? D.model_b : D.model;
    const double init_relax = side ? D.init_relax_b : D.init_relax;
    double s1 = 0.0, s2 = 0.0;
    for (int i = threadIdx.x; i < n; i += kDnBlock) {
        const double d = __dsub_rn(res[i], pres[i]);
        s1 = __dadd_rn(s1, __dmul_rn(pres[i], d));
        s2 = __dadd_rn(s2, __dmul_rn(d, d));
    }
    s1 = dn_block_sum(s1, sh);
    s2 = dn_block_sum(s2, sh);
    if (threadIdx.x == 0) {
        double w = init_relax;
        if (model == 1) {
            double a = D.scal[side];
            if (D.corr[side] < 3) {
                a = a < init_relax ? init_relax : a;
            } else {
                a = fabs(__dmul_rn(-a, __ddiv_rn(s1, __dadd_rn(s2, kSmall))));
                if (a > 1.0)
                    a = 1.0;
                else if (a < kSmall)
                    a = init_relax;
            }
            D.scal[side] = a;
            w = a;
        }
        s_w = w;
        D.corr[side] += 1;
    }
    __syncthreads();
    const double w = s_w;
    for (int i = threadIdx.x; i < n; i += kDnBlock) {
        const double v = __dadd_rn(prev[i], __dmul_rn(w, res[i]));
        prev[i] = v;
        out[i] = v;
    }
}

// IQNILS::relax for one side: cur (the unrelaxed field) in iqn_cur, res =
// cur - prev already stored.  updateVW: on a time step's first corrector
// drop the columns older than `reuse` time steps; on its second keep cur and
// res as the references; from the third on append V = res - resRef and
// W = cur - fldRef.  With more than one column the field becomes cur + W c,
// c the least-squares solution of V c = -res by modified Gram-Schmidt QR
// with columns of |R_ii| <= 1e-10 max_j sum_i |R_ij| dropped
// (updateIQNILS); otherwise prev + relax * res.  Every sum is a fixed-order
// CTA reduction; element-wise steps are single IEEE operations.
__device__ void dn_iqnils(const DnView& D, int side, int n, double* prev, double* res, double* out, double* sh)
{
    __shared__ int s_head, s_count, s_corr;
    __shared__ double R[kIqnModes][kIqnModes], Cv[kIqnModes];
    const int off = side ? D.na : 0;   // side offset in the [A | B] arrays
    const size_t coff = side ? (size_t)kIqnModes * D.na : 0;
    double* V = D.iqn_v + coff;
    double* W = D.iqn_w + coff;
    double* Q = D.iqn_q + coff;
    double* fref = D.iqn_fref + off;
    double* rref = D.iqn_rref + off;
    const double* cur = D.iqn_cur + off;
    int* T = D.iqn_t + side * kIqnModes;
    int* ring = D.iqn_ring + 2 * side;
    const int t = threadIdx.x;
    if (t == 0) {
        int head = ring[0], count = ring[1];
        const int corr = D.corr[side], now = D.corr[2];
        if (corr == 1) {
            while (count > 0 && now - (side ? D.reuse_b : D.reuse) > T[head]) {
                head = (head + 1) % kIqnModes;
                --count;
            }
        } else if (corr >= 3 && count == kIqnModes) {
            head = (head + 1) % kIqnModes;   // full: the oldest column goes
            --count;
        }
        s_head = head;
        s_count = count;
        s_corr = corr;
    }
    __syncthreads();
    const int corr = s_corr;
    if (corr == 2) {
        for (int i = t; i < n; i += kDnBlock) {
            fref[i] = cur[i];
            rref[i] = res[i];
        }
    } else if (corr >= 3) {
        const int slot = (s_head + s_count) % kIqnModes;
        for (int i = t; i < n; i += kDnBlock) {
            V[(size_t)slot * n + i] = __dsub_rn(res[i], rref[i]);
            W[(size_t)slot * n + i] = __dsub_rn(cur[i], fref[i]);
        }
        if (t == 0) {
            T[slot] = D.corr[2];
            s_count = s_count + 1;
        }
    }
    __syncthreads();
    const int head = s_head, cols = s_count;
    if (cols > 1) {
        // Q[i] = V[cols - 1 - i]: newest column first
        for (int i = 0; i < cols; ++i) {
            const double* v = V + (size_t)((head + cols - 1 - i) % kIqnModes) * n;
            for (int e = t; e < n; e += kDnBlock) Q[(size_t)i * n + e] = v[e];
        }
        __syncthreads();
        for (int i = 0; i < cols; ++i) {
            double* qi = Q + (size_t)i * n;
            double s2 = 0.0;
            for (int e = t; e < n; e += kDnBlock) s2 = __dadd_rn(s2, __dmul_rn(qi[e], qi[e]));
            const double rii = __dsqrt_rn(dn_block_sum(s2, sh));
            if (t == 0) R[i][i] = rii;
            for (int e = t; e < n; e += kDnBlock) qi[e] = __ddiv_rn(qi[e], rii);
            __syncthreads();
            for (int j = i + 1; j < cols; ++j) {
                double* qj = Q + (size_t)j * n;
                double sij = 0.0;
                for (int e = t; e < n; e += kDnBlock) sij = __dadd_rn(sij, __dmul_rn(qi[e], qj[e]));
                const double rij = dn_block_sum(sij, sh);
                if (t == 0) R[i][j] = rij;
                for (int e = t; e < n; e += kDnBlock) qj[e] = __dsub_rn(qj[e], __dmul_rn(rij, qi[e]));
                __syncthreads();
            }
            double ci = 0.0;
            for (int e = t; e < n; e += kDnBlock) ci = __dadd_rn(ci, __dmul_rn(qi[e], -res[e]));
            ci = dn_block_sum(ci, sh);
            if (t == 0) Cv[i] = ci;
        }
        if (t == 0) {
            // back-substitution of R c = C, columns below the tolerance dropped
            double eps = 0.0;
            for (int j = 0; j < cols; ++j) {
                double cs = 0.0;
                for (int i = 0; i <= j; ++i) cs = __dadd_rn(cs, fabs(R[i][j]));
                eps = j == 0 ? cs : fmax(eps, cs);
            }
            eps = __dmul_rn(1.0e-10, eps);
            for (int i = 0; i < cols; ++i) {
                if (fabs(R[i][i]) > eps) {
                    for (int j = i + 1; j < cols; ++j) R[i][j] = __ddiv_rn(R[i][j], R[i][i]);
                    Cv[i] = __ddiv_rn(Cv[i], R[i][i]);
                    R[i][i] = 1.0;
                }
            }
            for (int j = cols - 1; j >= 0; --j) {
                if (fabs(R[j][j]) > eps) {
                    for (int i = 0; i < j; ++i) Cv[i] = __dsub_rn(Cv[i], __dmul_rn(Cv[j], R[i][j]));
                } else {
                    Cv[j] = 0.0;
                }
            }
        }
        __syncthreads();
        for (int e = t; e < n; e += kDnBlock) {
            double v = cur[e];
            for (int k = 0; k < cols; ++k)
                v = __dadd_rn(v, __dmul_rn(W[(size_t)((head + k) % kIqnModes) * n + e], Cv[cols - 1 - k]));
            prev[e] = v;
            out[e] = v;
        }
    } else {
        for (int e = t; e < n; e += kDnBlock) {
            const double v = __dadd_rn(prev[e], __dmul_rn(side ? D.init_relax_b : D.init_relax, res[e]));
            prev[e] = v;
            out[e] = v;
        }
    }
    __syncthreads();
    if (t == 0) {
        ring[0] = head;
        ring[1] = cols;
        D.corr[side] = corr + 1;
    }
}

__global__ void __launch_bounds__(kDnBlock) k_dn_update_a(DnView D, const double* __restrict__ t_b)
{
    __shared__ double sh[kDnBlock];
    for (int j = threadIdx.x; j < D.nb; j += kDnBlock)
        D.tmp_b[j] = __dadd_rn(t_b[D.fc_b[j]], __ddiv_rn(D.grad_b[j], D.delta_b[j]));
    __syncthreads();
    for (int i = threadIdx.x; i < D.na; i += kDnBlock) {
        const double nbr = csr_row(D.pa, D.xa, D.wa, D.tmp_b, i);
        const double cur = __dadd_rn(nbr, __dmul_rn(D.K - 1.0, nbr));
        D.pres_a[i] = D.res_a[i];
        D.res_a[i] = __dsub_rn(cur, D.prev_a[i]);
        if (D.model == 2) D.iqn_cur[i] = cur;
    }
    __syncthreads();
    if (D.model == 2)
        dn_iqnils(D, 0, D.na, D.prev_a, D.res_a, D.value_a, sh);
    else
        dn_relax(D, 0, D.na, D.prev_a, D.res_a, D.pres_a, D.value_a, sh);
}

__global__ void __launch_bounds__(kDnBlock) k_dn_update_b(DnView D, const double* __restrict__ t_a)
{
    __shared__ double sh[kDnBlock];
    for (int i = threadIdx.x; i < D.na; i += kDnBlock)
        D.tmp_a[i] = __dmul_rn(__dmul_rn(D.k_a[i], D.delta_a[i]), __dsub_rn(D.value_a[i], t_a[D.fc_a[i]]));
    __syncthreads();
    for (int j = threadIdx.x; j < D.nb; j += kDnBlock) {
        const double f = __dadd_rn(-csr_row(D.pb, D.xb, D.wb, D.tmp_a, j), D.flux_jump);
        const double cur = __ddiv_rn(f, D.k_b[j]);
        D.pres_b[j] = D.res_b[j];
        D.res_b[j] = __dsub_rn(cur, D.prev_b[j]);
        if (D.model_b == 2) D.iqn_cur[D.na + j] = cur;
    }
    __syncthreads();
    if (D.model_b == 2)
        dn_iqnils(D, 1, D.nb, D.prev_b, D.res_b, D.grad_b, sh);
    else
        dn_relax(D, 1, D.nb, D.prev_b, D.res_b, D.pres_b, D.grad_b, sh);
}

__global__ void k_dn_copy(const double* __restrict__ b0, double* __restrict__ b, int n)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) b[c] = b0[c];
}

// Add the interface terms of one side to b, cell by cell, faces in
// ascending order: A (Dirichlet): k area delta value; B (Neumann): k area
// gradient.
__global__ void k_dn_rhs_add(DnView D, int side, double* __restrict__ b)
{
    const int nc = side ? D.ncb : D.nca;
    const int* ptr = side ? D.cb_ptr : D.ca_ptr;
    const int* face = side ? D.cb_face : D.ca_face;
    const int* cell = side ? D.cb_cell : D.ca_cell;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        double acc = b[cell[c]];
        for (int k = ptr[c]; k < ptr[c + 1]; ++k) {
            const int f = face[k];
            const double t = side ? __dmul_rn(__dmul_rn(D.k_b[f], D.area_b[f]), D.grad_b[f])
                                  : __dmul_rn(__dmul_rn(__dmul_rn(D.k_a[f], D.area_a[f]), D.delta_a[f]), D.value_a[f]);
            acc = __dadd_rn(acc, t);
        }
        b[cell[c]] = acc;
    }
}

__global__ void __launch_bounds__(kDnBlock) k_dn_residuals(DnView D, const double* __restrict__ t_a,
                                                            const double* __restrict__ t_b)
{
    __shared__ double sh[kDnBlock];
    for (int j = threadIdx.x; j < D.nb; j += kDnBlock)
        D.tmp_b[j] = __dadd_rn(t_b[D.fc_b[j]], __ddiv_rn(D.grad_b[j], D.delta_b[j]));
    for (int i = threadIdx.x; i < D.na; i += kDnBlock)
        D.tmp_a[i] = __dmul_rn(__dmul_rn(D.k_a[i], D.delta_a[i]), __dsub_rn(D.value_a[i], t_a[D.fc_a[i]]));
    __syncthreads();
    // jump residual on A
    double r2 = 0.0, o2 = 0.0, n2 = 0.0;
    for (int i = threadIdx.x; i < D.na; i += kDnBlock) {
        const double nbr = csr_row(D.pa, D.xa, D.wa, D.tmp_b, i);
        const double jump = __dmul_rn(D.K - 1.0, nbr);
        const double raw = fabs(__dsub_rn(__dsub_rn(D.value_a[i], nbr), jump));
        r2 = __dadd_rn(r2, __dmul_rn(raw, raw));
        o2 = __dadd_rn(o2, __dmul_rn(D.value_a[i], D.value_a[i]));
        const double nj = __dadd_rn(nbr, jump);
        n2 = __dadd_rn(n2, __dmul_rn(nj, nj));
    }
    r2 = dn_block_sum(r2, sh);
    o2 = dn_block_sum(o2, sh);
    n2 = dn_block_sum(n2, sh);
    // flux residual on B
    double f2 = 0.0, fo2 = 0.0, fn2 = 0.0;
    for (int j = threadIdx.x; j < D.nb; j += kDnBlock) {
        const double fnbr = csr_row(D.pb, D.xb, D.wb, D.tmp_a, j);
        const double fown = __dmul_rn(D.grad_b[j], D.k_b[j]);
        const double raw = fabs(__dsub_rn(__dadd_rn(fown, fnbr), D.flux_jump));
        f2 = __dadd_rn(f2, __dmul_rn(raw, raw));
        fo2 = __dadd_rn(fo2, __dmul_rn(fown, fown));
        const double nf = __dadd_rn(-fnbr, D.flux_jump);
        fn2 = __dadd_rn(fn2, __dmul_rn(nf, nf));
    }
    f2 = dn_block_sum(f2, sh);
    fo2 = dn_block_sum(fo2, sh);
    fn2 = dn_block_sum(fn2, sh);
    if (threadIdx.x == 0) {
        const double nj = fmax(fmin(sqrt(o2), sqrt(n2)), kSmall);
        const double nf = fmax(fmin(sqrt(fo2), sqrt(fn2)), kSmall);
        D.scal[2] = __ddiv_rn(sqrt(r2), nj);
        D.scal[3] = __ddiv_rn(sqrt(f2), nf);
    }
}

DnView view_of(const Dn& d)
{
    DnView v;
    v.na = d.na;
    v.nb = d.nb;
    v.model = d.model;
    v.model_b = d.model_b;
    v.K = d.K;
    v.flux_jump = d.flux_jump;
    v.init_relax = d.relax;
    v.init_relax_b = d.relax_b;
    v.fc_a = d.fc_a;
    v.fc_b = d.fc_b;
    v.delta_a = d.delta_a;
    v.k_a = d.k_a;
    v.area_a = d.area_a;
    v.delta_b = d.delta_b;
    v.k_b = d.k_b;
    v.area_b = d.area_b;
    v.pa = d.pa;
    v.xa = d.xa;
    v.wa = d.wa;
    v.pb = d.pb;
    v.xb = d.xb;
    v.wb = d.wb;
    v.ca_ptr = d.ca_ptr;
    v.ca_face = d.ca_face;
    v.ca_cell = d.ca_cell;
    v.cb_ptr = d.cb_ptr;
    v.cb_face = d.cb_face;
    v.cb_cell = d.cb_cell;
    v.nca = d.nca;
    v.ncb = d.ncb;
    v.value_a = d.value_a;
    v.grad_b = d.grad_b;
    v.prev_a = d.prev_a;
    v.res_a = d.res_a;
    v.pres_a = d.pres_a;
    v.prev_b = d.prev_b;
    v.res_b = d.res_b;
    v.pres_b = d.pres_b;
    v.tmp_a = d.tmp_a;
    v.tmp_b = d.tmp_b;
    v.scal = d.scal;
    v.corr = d.corr;
    v.reuse = d.reuse;
    v.reuse_b = d.reuse_b;
    v.iqn_v = d.iqn_v;
    v.iqn_w = d.iqn_w;
    v.iqn_q = d.iqn_q;
    v.iqn_fref = d.iqn_fref;
    v.iqn_rref = d.iqn_rref;
    v.iqn_cur = d.iqn_cur;
    v.iqn_t = d.iqn_t;
    v.iqn_ring = d.iqn_ring;
    return v;
}

template <typename T>
T* upload(Ctx* c, const T* h, size_t n)
{
    T* p = (T*)c->alloc(sizeof(T) * std::max<size_t>(n, 1));
    if (n) MRG_CUDA(cudaMemcpyAsync(p, h, sizeof(T) * n, cudaMemcpyHostToDevice, c->st));
    return p;
}

// Faces grouped by their cell (faces in ascending order within a cell).
void group_faces(int n, const int32_t* fc, std::vector<int>& ptr, std::vector<int>& face, std::vector<int>& cell)
{
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return fc[a] < fc[b]; });
    ptr.assign(1, 0);
    face.clear();
    cell.clear();
    for (int k = 0; k < n; ++k) {
        const int f = order[k];
        if (cell.empty() || cell.back() != fc[f]) {
            if (!cell.empty()) ptr.push_back((int)face.size());
            cell.push_back(fc[f]);
        }
        face.push_back(f);
    }
    ptr.push_back((int)face.size());
    if (cell.empty()) ptr.assign(1, 0);
}

// IQN-ILS storage for both sides (either side may select the model).
void alloc_iqnils(Dn& d)
{
    if (d.iqn_v) return;
    Ctx* c = d.ctx;
    const size_t both = (size_t)d.na + d.nb;
    for (double** q : {&d.iqn_v, &d.iqn_w, &d.iqn_q}) *q = (double*)c->alloc(8 * (size_t)kIqnModes * both);
    for (double** q : {&d.iqn_fref, &d.iqn_rref, &d.iqn_cur}) *q = (double*)c->alloc(8 * both);
    d.iqn_t = (int*)c->alloc(4 * 2 * kIqnModes);
    d.iqn_ring = (int*)c->alloc(4 * 4);
}

void check_csr(int n_rows, int n_src, const int32_t* ptr, const int32_t* addr, const char* what)
{
    if (!ptr || (n_rows > 0 && !addr)) throw Error(MRG_E_INVALID, std::string(what) + ": NULL CSR");
    if (ptr[0] != 0) throw Error(MRG_E_INVALID, std::string(what) + ": CSR must start at 0");
    for (int i = 0; i < n_rows; ++i) {
        if (ptr[i + 1] < ptr[i]) throw Error(MRG_E_INVALID, std::string(what) + ": CSR pointer decreases");
        for (int k = ptr[i]; k < ptr[i + 1]; ++k)
            if (addr[k] < 0 || addr[k] >= n_src)
                throw Error(MRG_E_INVALID, std::string(what) + ": source face out of range");
    }
}

}  // namespace

Dn* dn_create(Ctx* c, int n_cells_a, int na, const int32_t* fc_a, const double* delta_a, const double* k_a,
              const double* area_a, int n_cells_b, int nb, const int32_t* fc_b, const double* delta_b,
              const double* k_b, const double* area_b, const int32_t* a_ptr, const int32_t* a_addr,
              const double* a_w, const int32_t* b_ptr, const int32_t* b_addr, const double* b_w, double K,
              double flux_jump, int model, double relax, int reuse)
{
    if (na <= 0 || nb <= 0 || n_cells_a <= 0 || n_cells_b <= 0) throw Error(MRG_E_INVALID, "empty patch or region");
    if (!fc_a || !delta_a || !k_a || !area_a || !fc_b || !delta_b || !k_b || !area_b || !a_w || !b_w)
        throw Error(MRG_E_INVALID, "NULL patch array");
    if (model < 0 || model > 2)
        throw Error(MRG_E_INVALID, "relaxation model must be 0 (fixed), 1 (Aitken) or 2 (IQN-ILS)");
    if (reuse < 0) throw Error(MRG_E_INVALID, "couplingReuse must be >= 0");
    for (int i = 0; i < na; ++i)
        if (fc_a[i] < 0 || fc_a[i] >= n_cells_a) throw Error(MRG_E_INVALID, "patch A faceCells out of range");
    for (int j = 0; j < nb; ++j)
        if (fc_b[j] < 0 || fc_b[j] >= n_cells_b) throw Error(MRG_E_INVALID, "patch B faceCells out of range");
    check_csr(na, nb, a_ptr, a_addr, "A-from-B weights");
    check_csr(nb, na, b_ptr, b_addr, "B-from-A weights");
    auto* d = new Dn();
    try {
        d->ctx = c;
        d->na = na;
        d->nb = nb;
        d->ncells_a = n_cells_a;
        d->ncells_b = n_cells_b;
        d->model = model;
        d->K = K;
        d->flux_jump = flux_jump;
        d->relax = relax;
        d->fc_a = upload(c, fc_a, na);
        d->fc_b = upload(c, fc_b, nb);
        d->delta_a = upload(c, delta_a, na);
        d->k_a = upload(c, k_a, na);
        d->area_a = upload(c, area_a, na);
        d->delta_b = upload(c, delta_b, nb);
        d->k_b = upload(c, k_b, nb);
        d->area_b = upload(c, area_b, nb);
        d->pa = upload(c, a_ptr, na + 1);
        d->xa = upload(c, a_addr, (size_t)a_ptr[na]);
        d->wa = upload(c, a_w, (size_t)a_ptr[na]);
        d->pb = upload(c, b_ptr, nb + 1);
        d->xb = upload(c, b_addr, (size_t)b_ptr[nb]);
        d->wb = upload(c, b_w, (size_t)b_ptr[nb]);
        std::vector<int> p, f, cl;
        group_faces(na, fc_a, p, f, cl);
        d->nca = (int)cl.size();
        d->ca_ptr = upload(c, p.data(), p.size());
        d->ca_face = upload(c, f.data(), f.size());
        d->ca_cell = upload(c, cl.data(), cl.size());
        group_faces(nb, fc_b, p, f, cl);
        d->ncb = (int)cl.size();
        d->cb_ptr = upload(c, p.data(), p.size());
        d->cb_face = upload(c, f.data(), f.size());
        d->cb_cell = upload(c, cl.data(), cl.size());
        for (double** q : {&d->value_a, &d->prev_a, &d->res_a, &d->pres_a, &d->tmp_a})
            *q = (double*)c->alloc(8 * (size_t)na);
        for (double** q : {&d->grad_b, &d->prev_b, &d->res_b, &d->pres_b, &d->tmp_b})
            *q = (double*)c->alloc(8 * (size_t)nb);
        d->scal = (double*)c->alloc(8 * 8);
        d->corr = (int*)c->alloc(4 * 4);
        d->reuse = reuse;
        d->model_b = model;
        d->relax_b = relax;
        d->reuse_b = reuse;
        if (model == 2) alloc_iqnils(*d);
        MRG_CUDA(cudaStreamSynchronize(c->st));
    } catch (...) {
        delete d;
        throw;
    }
    return d;
}

Dn::~Dn()
{
    if (!ctx) return;
    cudaStreamSynchronize(ctx->st);
    for (const void* p : {(const void*)fc_a, (const void*)fc_b, (const void*)delta_a, (const void*)k_a,
                          (const void*)area_a, (const void*)delta_b, (const void*)k_b, (const void*)area_b,
                          (const void*)pa, (const void*)xa, (const void*)wa, (const void*)pb, (const void*)xb,
                          (const void*)wb, (const void*)ca_ptr, (const void*)ca_face, (const void*)ca_cell,
                          (const void*)cb_ptr, (const void*)cb_face, (const void*)cb_cell, (const void*)value_a,
                          (const void*)prev_a, (const void*)res_a, (const void*)pres_a, (const void*)tmp_a,
                          (const void*)grad_b, (const void*)prev_b, (const void*)res_b, (const void*)pres_b,
                          (const void*)tmp_b, (const void*)scal, (const void*)corr, (const void*)iqn_v,
                          (const void*)iqn_w, (const void*)iqn_q, (const void*)iqn_fref, (const void*)iqn_rref,
                          (const void*)iqn_cur, (const void*)iqn_t, (const void*)iqn_ring})
        if (p) ctx->release(const_cast<void*>(p));
}

void dn_set_flux_relaxation(Dn& d, int model, double relax, int reuse)
{
    if (model < 0 || model > 2)
        throw Error(MRG_E_INVALID, "relaxation model must be 0 (fixed), 1 (Aitken) or 2 (IQN-ILS)");
    if (reuse < 0) throw Error(MRG_E_INVALID, "couplingReuse must be >= 0");
    if (model == 2) alloc_iqnils(d);
    d.model_b = model;
    d.relax_b = relax;
    d.reuse_b = reuse;
}

void dn_set_state(Dn& d, const double* value_a, const double* grad_b)
{
    Ctx* c = d.ctx;
    cudaStream_t st = c->st;
    MRG_CUDA(cudaMemcpyAsync(d.value_a, value_a, 8 * (size_t)d.na, cudaMemcpyHostToDevice, st));
    MRG_CUDA(cudaMemcpyAsync(d.prev_a, value_a, 8 * (size_t)d.na, cudaMemcpyHostToDevice, st));
    MRG_CUDA(cudaMemcpyAsync(d.grad_b, grad_b, 8 * (size_t)d.nb, cudaMemcpyHostToDevice, st));
    MRG_CUDA(cudaMemcpyAsync(d.prev_b, grad_b, 8 * (size_t)d.nb, cudaMemcpyHostToDevice, st));
    for (double* q : {d.res_a, d.pres_a}) MRG_CUDA(cudaMemsetAsync(q, 0, 8 * (size_t)d.na, st));
    for (double* q : {d.res_b, d.pres_b}) MRG_CUDA(cudaMemsetAsync(q, 0, 8 * (size_t)d.nb, st));
    const double sc[8] = {d.relax, d.relax_b, 0, 0, 0, 0, 0, 0};
    const int corr[4] = {1, 1, 0, 0};
    MRG_CUDA(cudaMemcpyAsync(d.scal, sc, sizeof sc, cudaMemcpyHostToDevice, st));
    MRG_CUDA(cudaMemcpyAsync(d.corr, corr, sizeof corr, cudaMemcpyHostToDevice, st));
    if (d.iqn_ring) MRG_CUDA(cudaMemsetAsync(d.iqn_ring, 0, 4 * 4, st));   // no IQN-ILS columns
    MRG_CUDA(cudaStreamSynchronize(st));
}

void dn_new_time_step(Dn& d)
{
    // corrector counts back to 1, the time index one further
    int corr[3];
    MRG_CUDA(cudaMemcpyAsync(corr, d.corr, sizeof corr, cudaMemcpyDeviceToHost, d.ctx->st));
    MRG_CUDA(cudaStreamSynchronize(d.ctx->st));
    corr[0] = corr[1] = 1;
    corr[2] += 1;
    MRG_CUDA(cudaMemcpyAsync(d.corr, corr, sizeof corr, cudaMemcpyHostToDevice, d.ctx->st));
    MRG_CUDA(cudaStreamSynchronize(d.ctx->st));
}

void dn_update_a(Dn& d, const double* d_t_b)
{
    k_dn_update_a<<<1, kDnBlock, 0, d.ctx->st>>>(view_of(d), d_t_b);
    MRG_CUDA(cudaGetLastError());
    add_launches(1);
}

void dn_update_b(Dn& d, const double* d_t_a)
{
    k_dn_update_b<<<1, kDnBlock, 0, d.ctx->st>>>(view_of(d), d_t_a);
    MRG_CUDA(cudaGetLastError());
    add_launches(1);
}

void dn_rhs(Dn& d, int side, const double* d_b0, double* d_b)
{
    const int n = side ? d.ncells_b : d.ncells_a;
    int grid = (n + 255) / 256;
    grid = std::min(std::max(grid, 1), 1024);
    const DnView v = view_of(d);
    if (d_b0 != d_b) k_dn_copy<<<grid, 256, 0, d.ctx->st>>>(d_b0, d_b, n);
    const int nc = side ? d.ncb : d.nca;
    k_dn_rhs_add<<<std::max(1, std::min((nc + 255) / 256, 1024)), 256, 0, d.ctx->st>>>(v, side, d_b);
    MRG_CUDA(cudaGetLastError());
    add_launches(d_b0 != d_b ? 2 : 1);
}

void dn_residuals(Dn& d, const double* d_t_a, const double* d_t_b, double* jump, double* flux)
{
    k_dn_residuals<<<1, kDnBlock, 0, d.ctx->st>>>(view_of(d), d_t_a, d_t_b);
    MRG_CUDA(cudaGetLastError());
    add_launches(1);
    double sc[4];
    MRG_CUDA(cudaMemcpyAsync(sc, d.scal, sizeof sc, cudaMemcpyDeviceToHost, d.ctx->st));
    MRG_CUDA(cudaStreamSynchronize(d.ctx->st));
    if (jump) *jump = sc[2];
    if (flux) *flux = sc[3];
}

void dn_get_state(Dn& d, double* value_a, double* grad_b, double* aitken)
{
    cudaStream_t st = d.ctx->st;
    if (value_a) MRG_CUDA(cudaMemcpyAsync(value_a, d.value_a, 8 * (size_t)d.na, cudaMemcpyDeviceToHost, st));
    if (grad_b) MRG_CUDA(cudaMemcpyAsync(grad_b, d.grad_b, 8 * (size_t)d.nb, cudaMemcpyDeviceToHost, st));
    double sc[2];
    MRG_CUDA(cudaMemcpyAsync(sc, d.scal, sizeof sc, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
    if (aitken) {
        aitken[0] = sc[0];
        aitken[1] = sc[1];
    }
}

}  // namespace mrg
