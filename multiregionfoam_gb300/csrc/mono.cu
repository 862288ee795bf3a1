// mono.cu -- monolithic interface coefficients on the device.
//
// The per-face interface terms the reference's monolithic conjugate-heat-
// transfer boundary conditions compute at every assembly, for both sides of
// a regionCouple interface:
//   monolithicThermalDiffusivityFvPatchScalarField::calcThermalDiffusivity
//   (monolithicThermalDiffusivityFvPatchScalarField.C:167-276) and
//   calcTemperature (.C:280-394): the neighbour's cell temperature Tc,
//   diffusivity f (monolithicBase::forig, monolithicBase.C:97-122) and
//   radiative flux Qr are GGI-interpolated onto this side's faces in one
//   gather (the reference packs them into a VectorN<scalar, 4>, .C:205-244);
//   with the linear patch weights w and |delta| (magLongDelta)
//     kOwn = f_own / (1 - w) / |delta|,  kNei = f_nei / w / |delta|
//     k    = kOwn (kNei + Qr / stabilise(Tc_nei - Tc_own, SMALL))
//            / (deltaCoeffs (kOwn + kNei)), clipped to [0.01, 100] kHarm
//     Tw   = (Qr + kOwn Tc_own + kNei Tc_nei) / (kOwn + kNei)
//   with kHarm the harmonic interpolate of f_own and f_nei (.C:258-260);
//   monolithicTemperatureFvPatchScalarField::source (.C:205-224) and
//   manipulateMatrix (.C:227-244):
//     s = kOwn (Tw - Tc_own) - kw deltaCoeffs (Tc_nei - Tc_own),
//     b[faceCells] += s |Sf|
//   (kw = the diffusivity patch value k, monolithicBase::kw, .C:135-160).
// Every operation is an explicit IEEE one in the order of the reference's
// expressions (no contraction), so the results are those of a sequential
// evaluation.  The matrix source is accumulated per cell in face order by
// one thread per cell (faces grouped by cell when the interface is created).
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/mrgpu.h"
#include "kernels.h"
#include "mono.h"

namespace mrg {
namespace {

constexpr double kSmall = 1.0e-15;   // foam's SMALL (double precision)

struct SideView {
    int n_faces;
    const int32_t *face_cells, *src_ptr, *src_face;
    const double *w, *mld, *dc, *sf, *src_w;
};

SideView view(const MonoSide& s)
{
    return SideView{s.n_faces, s.face_cells, s.src_ptr, s.src_face, s.w, s.mld, s.dc, s.sf, s.src_w};
}

// GGI interpolate of the neighbour's Tc (and f, Qr when given) onto face i:
// weight order, from zero, one rounding per product and per sum.
__device__ __forceinline__ void gather(const SideView& S, int i, const int32_t* __restrict__ nbr_fc,
                                       const double* __restrict__ T_nbr, const double* __restrict__ f_nbr,
                                       const double* __restrict__ Qr_nbr, double& tc, double& fn, double& qr)
{
    tc = 0.0;
    fn = 0.0;
    qr = 0.0;
    for (int j = S.src_ptr[i]; j < S.src_ptr[i + 1]; ++j) {
        const int q = S.src_face[j];
        const double w = S.src_w[j];
        tc = __dadd_rn(tc, __dmul_rn(w, T_nbr[nbr_fc[q]]));
        if (f_nbr) fn = __dadd_rn(fn, __dmul_rn(w, f_nbr[q]));
        if (Qr_nbr) qr = __dadd_rn(qr, __dmul_rn(w, Qr_nbr[q]));
    }
}

__device__ __forceinline__ double k_own(const SideView& S, int i, double f)
{
    return __ddiv_rn(__ddiv_rn(f, __dsub_rn(1.0, S.w[i])), S.mld[i]);
}

__global__ void k_mono_update(SideView S, const int32_t* __restrict__ nbr_fc, const double* __restrict__ T_own,
                              const double* __restrict__ T_nbr, const double* __restrict__ f_own,
                              const double* __restrict__ f_nbr, const double* __restrict__ Qr_own,
                              const double* __restrict__ Qr_nbr, double* __restrict__ k, double* __restrict__ Tw)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n_faces; i += gridDim.x * blockDim.x) {
        double tc, fn, qn;
        gather(S, i, nbr_fc, T_nbr, f_nbr, Qr_nbr, tc, fn, qn);
        const double tco = T_own[S.face_cells[i]], fo = f_own[i], w = S.w[i];
        double Qr = 0.0;
        if (Qr_own) Qr = __dadd_rn(Qr, Qr_own[i]);
        if (Qr_nbr) Qr = __dadd_rn(Qr, qn);
        // harmonic interpolate with the linear weights: weights such that
        // wh f_own + (1 - wh) f_nei = 1 / (w / f_own + (1 - w) / f_nei)
        const double a = __dmul_rn(w, fn), b = __dmul_rn(__dsub_rn(1.0, w), fo);
        const double wh = __ddiv_rn(a, __dadd_rn(a, b));
        const double kH = __dadd_rn(__dmul_rn(wh, fo), __dmul_rn(__dsub_rn(1.0, wh), fn));
        const double kO = k_own(S, i, fo);
        const double kN = __ddiv_rn(__ddiv_rn(fn, w), S.mld[i]);
        const double dT = __dsub_rn(tc, tco);
        const double st = dT >= 0.0 ? __dadd_rn(dT, kSmall) : __dsub_rn(dT, kSmall);
        double kk = __dmul_rn(kO, __dadd_rn(kN, __ddiv_rn(Qr, st)));
        kk = __ddiv_rn(kk, __dmul_rn(S.dc[i], __dadd_rn(kO, kN)));
        const double hi = __dmul_rn(100.0, kH), lo = __dmul_rn(0.01, kH);
        kk = kk < hi ? kk : hi;
        kk = kk > lo ? kk : lo;
        k[i] = kk;
        Tw[i] = __ddiv_rn(__dadd_rn(__dadd_rn(Qr, __dmul_rn(kO, tco)), __dmul_rn(kN, tc)), __dadd_rn(kO, kN));
    }
}

__global__ void k_mono_s(SideView S, const int32_t* __restrict__ nbr_fc, const double* __restrict__ T_own,
                         const double* __restrict__ T_nbr, const double* __restrict__ Tw,
                         const double* __restrict__ kw, const double* __restrict__ f_own, double* __restrict__ s)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n_faces; i += gridDim.x * blockDim.x) {
        double tc, fn, qn;
        gather(S, i, nbr_fc, T_nbr, nullptr, nullptr, tc, fn, qn);
        const double tco = T_own[S.face_cells[i]];
        const double kd = __dmul_rn(kw[i], S.dc[i]);
        const double kO = k_own(S, i, f_own[i]);
        s[i] = __dsub_rn(__dmul_rn(kO, __dsub_rn(Tw[i], tco)), __dmul_rn(kd, __dsub_rn(tc, tco)));
    }
}

// b[cell] += s_f |Sf|_f over the cell's faces in face order.
__global__ void k_mono_add(int n_groups, const int32_t* __restrict__ cell_ptr, const int32_t* __restrict__ cell_face,
                           const int32_t* __restrict__ cells, const double* __restrict__ s,
                           const double* __restrict__ sf, double* __restrict__ b)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n_groups; g += gridDim.x * blockDim.x) {
        double v = b[cells[g]];
        for (int j = cell_ptr[g]; j < cell_ptr[g + 1]; ++j) {
            const int f = cell_face[j];
            v = __dadd_rn(v, __dmul_rn(s[f], sf[f]));
        }
        b[cells[g]] = v;
    }
}

int grid_of(int n) { return std::max(1, std::min((n + 255) / 256, 2048)); }

void check_side(const MonoPatchHost& p, const MonoPatchHost& other, const char* name)
{
    const std::string who(name);
    if (p.n_faces < 0 || p.n_cells < 0) throw Error(MRG_E_INVALID, who + ": negative size");
    if (p.n_faces > 0 && (!p.face_cells || !p.weights || !p.mag_long_delta || !p.delta_coeffs || !p.mag_sf ||
                          !p.src_ptr))
        throw Error(MRG_E_INVALID, who + ": NULL array");
    for (int i = 0; i < p.n_faces; ++i) {
        if (p.face_cells[i] < 0 || p.face_cells[i] >= p.n_cells)
            throw Error(MRG_E_INVALID, who + ": face cell out of range");
        if (!(p.weights[i] > 0.0 && p.weights[i] < 1.0))
            throw Error(MRG_E_INVALID, who + ": patch weights must lie in (0, 1)");
    }
    if (p.n_faces > 0) {
        if (p.src_ptr[0] != 0) throw Error(MRG_E_INVALID, who + ": GGI pointer must start at 0");
        for (int i = 0; i < p.n_faces; ++i)
            if (p.src_ptr[i + 1] < p.src_ptr[i]) throw Error(MRG_E_INVALID, who + ": GGI pointer decreases");
        const int nnz = p.src_ptr[p.n_faces];
        if (nnz > 0 && (!p.src_face || !p.src_weight)) throw Error(MRG_E_INVALID, who + ": NULL GGI weights");
        for (int j = 0; j < nnz; ++j)
            if (p.src_face[j] < 0 || p.src_face[j] >= other.n_faces)
                throw Error(MRG_E_INVALID, who + ": GGI source face out of range");
    }
}

}  // namespace

Mono::~Mono()
{
    if (!ctx) return;
    for (MonoSide& s : side)
        for (void* p : {(void*)s.face_cells, (void*)s.w, (void*)s.mld, (void*)s.dc, (void*)s.sf, (void*)s.src_ptr,
                        (void*)s.src_face, (void*)s.src_w, (void*)s.cell_ptr, (void*)s.cell_face, (void*)s.cells,
                        (void*)s.s})
            ctx->release(p);
}

void mono_create(Mono& m, Ctx* c, const MonoPatchHost& a, const MonoPatchHost& b)
{
    check_side(a, b, "side A");
    check_side(b, a, "side B");
    m.ctx = c;
    const MonoPatchHost* hp[2] = {&a, &b};
    for (int k = 0; k < 2; ++k) {
        const MonoPatchHost& p = *hp[k];
        MonoSide& s = m.side[k];
        s.n_cells = p.n_cells;
        s.n_faces = p.n_faces;
        const size_t nf = (size_t)std::max(p.n_faces, 1);
        const int nnz = p.n_faces > 0 ? p.src_ptr[p.n_faces] : 0;
        auto up = [&](const void* h, size_t bytes) {
            void* d = c->alloc(std::max<size_t>(bytes, 16));
            if (bytes) MRG_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c->st));
            return d;
        };
        s.face_cells = (int32_t*)up(p.face_cells, 4 * (size_t)p.n_faces);
        s.w = (double*)up(p.weights, 8 * (size_t)p.n_faces);
        s.mld = (double*)up(p.mag_long_delta, 8 * (size_t)p.n_faces);
        s.dc = (double*)up(p.delta_coeffs, 8 * (size_t)p.n_faces);
        s.sf = (double*)up(p.mag_sf, 8 * (size_t)p.n_faces);
        std::vector<int32_t> zero(1, 0);
        s.src_ptr = (int32_t*)up(p.n_faces > 0 ? p.src_ptr : zero.data(), 4 * (size_t)(p.n_faces + 1));
        s.src_face = (int32_t*)up(p.src_face, 4 * (size_t)nnz);
        s.src_w = (double*)up(p.src_weight, 8 * (size_t)nnz);
        s.s = (double*)c->alloc(8 * nf);
        // faces grouped by cell, each group in face order
        std::vector<int32_t> order(p.n_faces);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(),
                         [&](int x, int y) { return p.face_cells[x] < p.face_cells[y]; });
        std::vector<int32_t> ptr{0}, cells;
        for (int j = 0; j < p.n_faces; ++j) {
            if (j == 0 || p.face_cells[order[j]] != p.face_cells[order[j - 1]]) {
                if (j > 0) ptr.push_back(j);
                cells.push_back(p.face_cells[order[j]]);
            }
        }
        if (p.n_faces > 0) ptr.push_back(p.n_faces);
        s.n_groups = (int)cells.size();
        s.cell_ptr = (int32_t*)up(ptr.data(), 4 * ptr.size());
        s.cell_face = (int32_t*)up(order.data(), 4 * order.size());
        s.cells = (int32_t*)up(cells.data(), 4 * cells.size());
        MRG_CUDA(cudaStreamSynchronize(c->st));
    }
}

void mono_update(Mono& m, int side, const double* T_own, const double* T_nbr, const double* f_own,
                 const double* f_nbr, const double* Qr_own, const double* Qr_nbr, double* k, double* Tw)
{
    const MonoSide& S = m.side[side];
    const MonoSide& N = m.side[1 - side];
    if (S.n_faces == 0) return;
    k_mono_update<<<grid_of(S.n_faces), 256, 0, m.ctx->st>>>(view(S), N.face_cells, T_own, T_nbr, f_own, f_nbr,
                                                              Qr_own, Qr_nbr, k, Tw);
    add_launches(1);
    MRG_CUDA(cudaGetLastError());
}

void mono_source(Mono& m, int side, const double* T_own, const double* T_nbr, const double* Tw, const double* kw,
                 const double* f_own, double* b)
{
    MonoSide& S = m.side[side];
    const MonoSide& N = m.side[1 - side];
    if (S.n_faces == 0) return;
    k_mono_s<<<grid_of(S.n_faces), 256, 0, m.ctx->st>>>(view(S), N.face_cells, T_own, T_nbr, Tw, kw, f_own, S.s);
    k_mono_add<<<grid_of(S.n_groups), 256, 0, m.ctx->st>>>(S.n_groups, S.cell_ptr, S.cell_face, S.cells, S.s, S.sf,
                                                            b);
    add_launches(2);
    MRG_CUDA(cudaGetLastError());
}

}  // namespace mrg
