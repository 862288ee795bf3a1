// kernels.cu -- sm_103a kernels of the coupled-region LDU solve path.
//
// Arithmetic contract.  Every FP64 operation is an explicit IEEE intrinsic
// (__dmul_rn, __fma_rn, __dadd_rn, __ddiv_rn), so the per-cell results of
// Amul, sumA, the DIC/DILU factor, the sweeps and the GGI gather are
// bit-identical to the oracle's "fused" mode (same operations, same order).
// The order is foam's: each cell accumulates its face terms in ascending face
// index, interface terms after all face terms (lduMatrix::Amul then
// updateMatrixInterfaces), forward sweep terms in ascending and backward
// terms in descending face order.
//
// GB300 notes.  FP64 issue rate is ~1/64 of FP32 on this part, so FP64 kernels
// are written to minimise FP64 instructions: one FMA per matrix entry, sweep
// coefficients rD[row]*a pre-multiplied once per factorisation, no FP64 work
// on padding.  Everything else is HBM- or latency-bound: no tensor cores.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "kernels.h"
#include "plan.h"

namespace mrg {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr long long kSentBits64 = 0x7FF4DEADBEEF0001LL;  // signalling-NaN payload
constexpr unsigned kSentBits32 = 0x7FA5A5A5u;
// A device wait gives up after this many SM cycles (~2 s) unless the
// batch's control block sets its own budget, and flags ERR_TIMEOUT, so no
// kernel can spin forever.
constexpr long long kWaitCycles = 4000000000LL;
__device__ __forceinline__ long long wait_budget(const Ctl* ctl)
{
    const long long w = ctl->wait_cycles;
    return w > 0 ? w : kWaitCycles;
}

// Programmatic dependent launch.  The Krylov-loop kernels are launched with
// programmatic stream serialisation, so a kernel's CTAs can be scheduled
// while the previous kernel of the stream drains (its launch latency hidden
// behind the other's tail).  Each such kernel waits here for the previous
// kernel to complete and its writes to be visible before it reads anything a
// kernel writes, and then lets the next kernel be scheduled.  Before the
// wait it may read only what the host alone writes (the batch descriptor,
// its tables and the system descriptors), which the stream order already
// made visible.  Launched without the attribute, both instructions do
// nothing.
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename V> __device__ __forceinline__ V sent();
template <> __device__ __forceinline__ double sent<double>() { return __longlong_as_double(kSentBits64); }
template <> __device__ __forceinline__ float sent<float>() { return __uint_as_float(kSentBits32); }
__device__ __forceinline__ bool is_sent(double v) { return __double_as_longlong(v) == kSentBits64; }
__device__ __forceinline__ bool is_sent(float v) { return __float_as_uint(v) == kSentBits32; }

// float -> double on the integer pipe.  GB300 issues FP64 (conversions
// included) at a small fraction of the FP32 rate, so the FP64 reductions of
// the FP32 inner loop widen their operands with bit arithmetic only (a
// hardware-conversion fallback for rare cases would be if-converted by the
// compiler and then run for every element):
//   normal     same sign and mantissa, exponent rebiased by 1023 - 127
//   subnormal  m * 2^-149 = 1.f * 2^(p - 149), p = index of m's top bit
//   zero       signed zero
//   inf / NaN  exponent 0x7ff, mantissa shifted, NaN made quiet
// The result equals (double)f for every float (checked over all 2^32 bit
// patterns; NaN maps to NaN).
__device__ __forceinline__ double widen(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned m = u & 0x007fffffu;
    unsigned long long bits = (unsigned long long)(u & 0x80000000u) << 32;
    if (e - 1u < 0xfeu) {
        bits |= ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    } else if (e == 0xffu) {
        bits |= (0x7ffull << 52) | ((unsigned long long)m << 29) | (m ? (1ull << 51) : 0ull);
    } else if (m) {
        const int p = 31 - __clz((int)m);
        bits |= ((unsigned long long)(p + 874) << 52) | (((unsigned long long)m << (52 - p)) & 0xfffffffffffffull);
    }
    return __longlong_as_double((long long)bits);
}
__device__ __forceinline__ double widen(double d) { return d; }

__device__ __forceinline__ double vmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float vmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double vfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Sum over a warp's lanes in butterfly order (every lane gets the same
// value: each step adds two lanes' values, and their sum commutes).
__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Reduction terms of N consecutive rows (N = 2 or 4) into an FP64
// accumulator.  FP64: every row's term in FP64, row by row (the order the
// FP64 path is mirrored in).  FP32: the N terms are summed pairwise in
// FP32 and the partial widened and added once -- one FP64 operation per N
// rows instead of one per row on a part whose FP64 rate is a small
// fraction of its FP32 rate; the partial's rounding (a few FP32 ulps) is
// that of the FP32 vectors themselves.
template <int N>
__device__ __forceinline__ void acc_dot(double& acc, const double (&a)[N], const double (&b)[N])
{
#pragma unroll
    for (int k = 0; k < N; ++k) acc = __fma_rn(a[k], b[k], acc);
}
template <int N>
__device__ __forceinline__ void acc_dot(double& acc, const float (&a)[N], const float (&b)[N])
{
    static_assert(N == 2 || N == 4, "pairwise FP32 partial of 2 or 4 rows");
    float s = __fmaf_rn(a[1], b[1], __fmul_rn(a[0], b[0]));
    if constexpr (N == 4) s = __fadd_rn(s, __fmaf_rn(a[3], b[3], __fmul_rn(a[2], b[2])));
    acc += widen(s);
}
template <int N>
__device__ __forceinline__ void acc_abs(double& acc, const double (&a)[N])
{
#pragma unroll
    for (int k = 0; k < N; ++k) acc += fabs(a[k]);
}
template <int N>
__device__ __forceinline__ void acc_abs(double& acc, const float (&a)[N])
{
    static_assert(N == 2 || N == 4, "pairwise FP32 partial of 2 or 4 rows");
    float s = __fadd_rn(fabsf(a[0]), fabsf(a[1]));
    if constexpr (N == 4) s = __fadd_rn(s, __fadd_rn(fabsf(a[2]), fabsf(a[3])));
    acc += widen(s);
}
__device__ __forceinline__ double ld_relaxed(const double* p)
{
    double v;
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ float ld_relaxed(const float* p)
{
    float v;
    asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(double* p, double v)
{
    asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(float* p, float v)
{
    asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}

// Wait until a value produced in the same launch is published (not the
// sentinel).  Bounded: on timeout, or when another wait already timed out,
// it returns whatever it read and the error bit stays set for the host.
template <typename V>
__device__ __forceinline__ V wait_ready(const V* p, Ctl* ctl)
{
    V v = ld_relaxed(p);
    if (!is_sent(v)) return v;
    long long t0 = clock64();
    for (int it = 1;; ++it) {
        if (it > 32) __nanosleep(64);
        v = ld_relaxed(p);
        if (!is_sent(v)) return v;
        if ((it & 255) == 0) {
            if (*(volatile unsigned*)&ctl->err) return v;
            if (clock64() - t0 > wait_budget(ctl)) {
                atomicOr(&ctl->err, ERR_TIMEOUT);
                return v;
            }
        }
    }
}

// The value at p once published, given an earlier look v at it: the looks
// at all of a row's dependencies are relaxed loads issued together, so their
// round trips overlap; only a look that still saw the sentinel waits.
template <typename V>
__device__ __forceinline__ V ready(V v, const V* p, Ctl* ctl)
{
    return is_sent(v) ? wait_ready(p, ctl) : v;
}

// Coefficient value for a plan source code (see plan.h).
__device__ __forceinline__ double src_val(const SysDev& S, int s, bool trans)
{
    const int F = S.nf;
    if (s < 2 * F) {
        if (trans) s = (s < F) ? s + F : s - F;
        if (s < F) return S.raw_upper[s];
        return S.sym ? S.raw_upper[s - F] : S.raw_lower[s - F];
    }
    const int j = s - 2 * F;
    const double c = (trans && S.raw_iint) ? S.raw_iint[j] : S.raw_ibou[j];
    return -c;
}
__device__ __forceinline__ int swap_src(int s, int F) { return s < F ? s + F : (s < 2 * F ? s - F : s); }

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

// Deterministic block sum of NR values (fixed order).  Result valid in tid 0.
// Lane l of warp 0 adds the eight warps' values at lane l in warp order, then
// one shuffle tree finishes: 12 FP64 adds on 32 lanes instead of a shuffle
// tree on all 256 threads (FP64 adds are scarce on GB300).
// NB: the CTA also runs a producer warp beyond the kBlock threads, so the
// kBlock row threads meet at named barrier 1 instead of __syncthreads.
template <bool NB>
__device__ __forceinline__ void row_barrier()
{
    if constexpr (NB)
        asm volatile("bar.sync 1, %0;" ::"n"(kBlock) : "memory");
    else
        __syncthreads();
}

template <int NR, bool NB = false>
__device__ __forceinline__ void block_sum(double (&a)[NR], double* sh)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
#pragma unroll
    for (int k = 0; k < NR; ++k) sh[k * kBlock + tid] = a[k];
    row_barrier<NB>();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            double s = sh[k * kBlock + lane];
#pragma unroll
            for (int w = 1; w < kBlock / 32; ++w) s += sh[k * kBlock + w * 32 + lane];
            a[k] = warp_sum(s);
        }
    }
    row_barrier<NB>();
}

// ---------------------------------------------------------------- vector picks
template <typename V> struct VP;
template <> struct VP<double> {
    static __device__ __forceinline__ const Vecs<double>& v(const SysDev& S) { return S.v64; }
    static __device__ __forceinline__ const double* aval(const SysDev& S, bool t) { return t ? S.aT_val : S.a_val; }
    static __device__ __forceinline__ const double* diag(const SysDev& S) { return S.diag; }
    static __device__ __forceinline__ const double* rD(const SysDev& S) { return S.rD; }
    static __device__ __forceinline__ const double* fc(const SysDev& S, bool t) { return t ? S.f_cT : S.f_c; }
    static __device__ __forceinline__ const double* bc(const SysDev& S, bool t) { return t ? S.b_cT : S.b_c; }
    static __device__ __forceinline__ const double* gw(const SysDev& S) { return S.g_w; }
};
template <> struct VP<float> {
    static __device__ __forceinline__ const Vecs<float>& v(const SysDev& S) { return S.v32; }
    static __device__ __forceinline__ const float* aval(const SysDev& S, bool t) { return t ? S.aT_val32 : S.a_val32; }
    static __device__ __forceinline__ const float* diag(const SysDev& S) { return S.diag32; }
    static __device__ __forceinline__ const float* rD(const SysDev& S) { return S.rD32; }
    static __device__ __forceinline__ const float* fc(const SysDev& S, bool t) { return t ? S.f_cT32 : S.f_c32; }
    static __device__ __forceinline__ const float* bc(const SysDev& S, bool t) { return t ? S.b_cT32 : S.b_c32; }
    static __device__ __forceinline__ const float* gw(const SysDev& S) { return S.g_w32; }
};

// Sliced-ELL row product y_i = diag_i x_i + sum_k a_k x[col_k] (foam order).
// All column indices of the row are loaded first, then every coefficient and
// gathered x, then the FMA chain runs: the loads of one row are in flight
// together instead of one dependent round trip per entry.  Padding (col -1)
// is skipped, so no FP64 work is spent on it.
// kMaxW entries of a row are loaded and multiplied per round, unrolled: six
// covers the interior rows of hexahedral meshes in one round; wider rows
// (interface faces, polyhedra) take further rounds of the same shape.
#ifndef MRG_KMAXW
#define MRG_KMAXW 6
#endif
constexpr int kMaxW = MRG_KMAXW;
// Row and sweep kernels are compiled for at least 4 resident 256-thread CTAs
// per SM.  Reducing row kernels walk the batch's segment table (kRedSegs in
// dev.h), non-reducing row kernels take one tile per CTA.
constexpr int kMinCtas = 4;

// Entries k0 .. k0 + kMaxW - 1 (of W) of an ELL row stored at stride 32 from
// col / val: the round's loads are all in flight together, then the FMAs run
// in slot order (padding, col -1, skipped).  LDG: col and val are read-only
// global data (otherwise plain loads, e.g. from shared memory).
template <typename V, bool LDG>
__device__ __forceinline__ V ell_round(const int* col, const V* val, const V* __restrict__ x, int k0, int W, V y)
{
    int c[kMaxW];
    V a[kMaxW], xv[kMaxW];
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) {
        const int e = (k0 + k) * 32;
        c[k] = k0 + k < W ? (LDG ? __ldg(col + e) : col[e]) : -1;
    }
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) {
        const int e = (k0 + k) * 32;
        a[k] = c[k] >= 0 ? (LDG ? __ldg(val + e) : val[e]) : V(0);
        xv[k] = c[k] >= 0 ? __ldca(x + c[k]) : V(0);
    }
#pragma unroll
    for (int k = 0; k < kMaxW; ++k)
        if (c[k] >= 0) y = vfma(a[k], xv[k], y);
    return y;
}

template <typename V>
__device__ __forceinline__ V ell_row(const int* __restrict__ sptr, const int* __restrict__ acol,
                                     const V* __restrict__ val, const V* __restrict__ dg, const V* __restrict__ x,
                                     int i)
{
    const int sl = i >> 5, lane = i & 31;
    const int e0 = __ldg(sptr + sl), W = (__ldg(sptr + sl + 1) - e0) >> 5;
    V y = vmul(__ldg(dg + i), __ldca(x + i));
    if (W <= kMaxW) return ell_round<V, true>(acol + e0 + lane, val + e0 + lane, x, 0, W, y);
    for (int k0 = 0; k0 < W; k0 += kMaxW) y = ell_round<V, true>(acol + e0 + lane, val + e0 + lane, x, k0, W, y);
    return y;
}

// Sliced-ELL product of one 1024-row tile, warp w taking the tile's slices
// w, w+8, w+16, w+24.  The arithmetic of each row is ell_row's (diagonal
// first, then entries in slot order, padding skipped), but the latency chain
// is shorter: the 33 slice bounds of the tile are one coalesced load per warp
// (handed out by shuffles), and the next slice's column indexes are fetched
// while the current slice's coefficients and gathered x are in flight, so a
// slice costs about one dependent round trip instead of three.
// emit(i, y, x_i) consumes row i's product and its own x value.
template <typename V, typename Emit>
__device__ __forceinline__ void ell_tile(const int* __restrict__ sptr, const int* __restrict__ acol,
                                         const V* __restrict__ val, const V* __restrict__ dg,
                                         const V* __restrict__ x, int sl0, Emit&& emit)
{
    constexpr int kWarps = kBlock / 32, kPer = 32 / kWarps;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int sp = __ldg(sptr + sl0 + lane);
    const int spend = __ldg(sptr + sl0 + 32);
    int e0 = __shfl_sync(kFull, sp, wid);
    int W = (__shfl_sync(kFull, sp, wid + 1) - e0) >> 5;
    int c[kMaxW];
    if (W <= kMaxW) {
#pragma unroll
        for (int k = 0; k < kMaxW; ++k) c[k] = k < W ? __ldg(acol + e0 + lane + k * 32) : -1;
    }
#pragma unroll 1
    for (int j = 0; j < kPer; ++j) {
        const int s = wid + kWarps * j;
        const int i = (sl0 + s) * 32 + lane;
        int ne0 = 0, nW = kMaxW + 1;
        if (j + 1 < kPer) {
            ne0 = __shfl_sync(kFull, sp, s + kWarps);
            const int ne1 = (s + kWarps + 1 < 32) ? __shfl_sync(kFull, sp, s + kWarps + 1) : spend;
            nW = (ne1 - ne0) >> 5;
        }
        const V xi = __ldca(x + i);
        V y = vmul(__ldg(dg + i), xi);
        const V* __restrict__ v = val + e0 + lane;
        if (W <= kMaxW) {
            V a[kMaxW], xv[kMaxW];
            unsigned live = 0;
#pragma unroll
            for (int k = 0; k < kMaxW; ++k) {
                live |= (c[k] >= 0 ? 1u : 0u) << k;
                a[k] = c[k] >= 0 ? __ldg(v + k * 32) : V(0);
                xv[k] = c[k] >= 0 ? __ldca(x + c[k]) : V(0);
            }
            if (nW <= kMaxW) {
#pragma unroll
                for (int k = 0; k < kMaxW; ++k) c[k] = k < nW ? __ldg(acol + ne0 + lane + k * 32) : -1;
            }
#pragma unroll
            for (int k = 0; k < kMaxW; ++k)
                if (live & (1u << k)) y = vfma(a[k], xv[k], y);
        } else {
            for (int k0 = 0; k0 < W; k0 += kMaxW) y = ell_round<V, true>(acol + e0 + lane, v, x, k0, W, y);
            if (nW <= kMaxW) {
#pragma unroll
                for (int k = 0; k < kMaxW; ++k) c[k] = k < nW ? __ldg(acol + ne0 + lane + k * 32) : -1;
            }
        }
        emit(i, y, xi);
        e0 = ne0;
        W = nW;
    }
}

// Per-system finalisation, executed by thread 0 of the CTA that completes the
// system's reduction.  Systems entering or leaving a Krylov loop (or the
// mixed-precision outer loop) are counted in the batch's control block, which
// is all the host polls.
__device__ __forceinline__ void set_active(Ctl* ctl, Scal* sc, int on)
{
    if (sc->active == on) return;
    sc->active = on;
    atomicAdd(&ctl->n_active, on ? 1u : 0xffffffffu);
}

__device__ __forceinline__ void set_outer(Ctl* ctl, Scal* sc, int on)
{
    if (sc->ostate == on) return;
    sc->ostate = on;
    atomicAdd(&ctl->n_oactive, on ? 1u : 0xffffffffu);
}

__device__ void finalize(const Batch& B, const SysDev& S, RowOp op, const double* sums)
{
    Scal* sc = S.sc;
    Ctl* ctl = B.ctl;
    sc->red[0] = sums[0];
    sc->red[1] = sums[1];
    switch (op) {
    case OP_SUMX:
        sc->xsum = sums[0];
        break;
    case OP_INIT_RES: {
        sc->nfac = sums[0] + 1.0e-20;
        sc->res0 = sums[1] / sc->nfac;
        sc->res = sc->res0;
        sc->iter = 0;
        sc->singular = 0;
        sc->rho = 1.0e20;
        const bool conv = sc->res < sc->tol || (sc->rel_tol > 1.0e-20 && sc->res < sc->rel_tol * sc->res0);
        sc->converged = conv;
        sc->kmin = sc->min_iter;
        sc->kmax = sc->max_iter;
        const int go = (sc->min_iter > 0 || !conv) ? 1 : 0;
        if (sc->mixed) {
            // FP64 outer state of iterative refinement; the FP32 Krylov loop
            // starts at OP_TO32.
            sc->onfac = sc->nfac;
            sc->ores0 = sc->res0;
            sc->ores = sc->res0;
            sc->obest = sc->res0;
            sc->obest_sum = sums[1];
            sc->okeep = 1;
            sc->oconv = conv;
            sc->oiter = 0;
            sc->ostall = 0;
            sc->inner_total = 0;
            set_outer(ctl, sc, go);
        } else {
            set_active(ctl, sc, go);
        }
        break;
    }
    case OP_RHO:
    case OP_RHO_CH:
        sc->rho_old = sc->rho;
        sc->rho = sums[0];
        sc->beta = sc->iter > 0 ? sc->rho / sc->rho_old : 0.0;
        break;
    case OP_SPMV_QP:
        if (fabs(sums[0]) / sc->nfac < 1.0e-300) {
            sc->singular = 1;
            sc->alpha = 0.0;
            set_active(ctl, sc, 0);
        } else {
            sc->alpha = sc->rho / sums[0];
        }
        break;
    case OP_UPDATE: {
        sc->res = sums[0] / sc->nfac;
        sc->iter += 1;
        const bool conv = sc->res < sc->tol || (sc->rel_tol > 1.0e-20 && sc->res < sc->rel_tol * sc->res0);
        sc->converged = conv;
        const bool more = (sc->iter < sc->kmax && !conv) || sc->iter < sc->kmin;
        if (!more) set_active(ctl, sc, 0);
        break;
    }
    case OP_RESID64: {
        // true FP64 residual of the refined solution: foam's convergence test.
        // A refinement step that made the residual worse (an FP32 BiCG
        // recurrence that drifted) is rolled back by OP_KEEPBEST and the
        // next inner solve restarts sooner; the solve never returns an
        // iterate worse than the best it has seen.
        const double o = sums[0] / sc->onfac;
        const bool improved = sc->oiter == 0 || o < sc->obest;
        if (improved) {
            if (o < 0.999 * sc->obest || sc->oiter == 0)
                sc->ostall = 0;
            else
                sc->ostall += 1;
            sc->obest = o;
            sc->obest_sum = sums[0];
            sc->okeep = 1;
        } else {
            sc->ostall += 1;
            sc->okeep = 0;
            sc->inner_max = sc->inner_max / 2 > 25 ? sc->inner_max / 2 : 25;
        }
        sc->osum = sc->obest_sum;
        sc->ores = sc->obest;
        const bool conv = sc->ores < sc->otol || (sc->orel_tol > 1.0e-20 && sc->ores < sc->orel_tol * sc->ores0);
        sc->oconv = conv;
        const bool more = ((!conv || sc->inner_total < sc->min_iter) && sc->oiter < sc->max_outer &&
                           sc->inner_total < sc->max_iter && sc->ostall < 3);
        if (!more) {
            set_outer(ctl, sc, 0);
            if (!conv) sc->fallback = 1;   // refinement stalled: finish in FP64
        }
        break;
    }
    case OP_FALLBACK64: {
        if (sc->fallback == 2) {
            // after the FP64 loop: the true FP64 residual of x is what the
            // mixed form reports and tests
            sc->fallback = 3;
            sc->res = sums[0] / sc->onfac;
            sc->converged = sc->res < sc->tol || (sc->rel_tol > 1.0e-20 && sc->res < sc->rel_tol * sc->res0);
            break;
        }
        // FP64 Krylov from the best refined iterate, with the solve's own
        // normFactor and initial residual, so the convergence test and the
        // reported residuals mean what they mean for the plain method
        sc->fallback = 2;
        sc->tol = sc->otol;
        sc->rel_tol = sc->orel_tol;
        sc->nfac = sc->onfac;
        sc->res0 = sc->ores0;
        sc->res = sums[0] / sc->onfac;
        sc->iter = 0;
        sc->singular = 0;
        sc->rho = 1.0e20;
        sc->kmin = 0;
        sc->kmax = sc->max_iter;
        const bool conv = sc->res < sc->tol || (sc->rel_tol > 1.0e-20 && sc->res < sc->rel_tol * sc->res0);
        sc->converged = conv;
        set_active(ctl, sc, conv ? 0 : 1);
        break;
    }
    case OP_TO32: {
        // inner FP32 solve of A d = r: residual measured relative to its start;
        // it aims at 0.1x the FP64 residual still to remove (overshooting the
        // tolerance on the last step), never asked for less than inner_rel_tol
        const double goal = fmax(sc->otol, sc->orel_tol > 1.0e-20 ? sc->orel_tol * sc->ores0 : 0.0);
        double itol = 0.1 * goal / fmax(sc->ores, 1.0e-300);
        itol = fmin(0.5, fmax(sc->inner_rel_tol, itol));
        sc->inv_scale = sc->osum > 0.0 ? sc->osum / (double)S.n : 1.0;
        sc->nfac = sums[0] > 0.0 ? sums[0] : 1.0;
        sc->res0 = sums[0] / sc->nfac;
        sc->res = sc->res0;
        sc->tol = itol;
        sc->rel_tol = 0.0;
        sc->kmin = 0;
        const int left = sc->max_iter - sc->inner_total;
        sc->kmax = sc->inner_max < left ? sc->inner_max : left;
        sc->iter = 0;
        sc->singular = 0;
        sc->rho = 1.0e20;
        sc->converged = 0;
        set_active(ctl, sc, sums[0] > 0.0 ? 1 : 0);
        break;
    }
    case OP_GS_RES: {
        // smoothSolver: residual after nSweeps sweeps (foam counts sweeps)
        sc->res = sums[0] / sc->nfac;
        sc->iter += sc->n_sweeps;
        const bool conv = sc->res < sc->tol || (sc->rel_tol > 1.0e-20 && sc->res < sc->rel_tol * sc->res0);
        sc->converged = conv;
        const bool more = (sc->iter < sc->kmax && !conv) || sc->iter < sc->kmin;
        if (!more) set_active(ctl, sc, 0);
        break;
    }
    case OP_BS_RHO0:
        // BiCGStab start: rho = (r~, r) with r~ = r; a zero rho cannot start
        sc->rho = sums[0];
        sc->rho_old = sums[0];
        if (fabs(sums[0]) < 1.0e-300) {
            sc->singular = 1;
            set_active(ctl, sc, 0);
        }
        break;
    case OP_BS_V:
        if (fabs(sums[0]) / sc->nfac < 1.0e-300) {
            sc->singular = 1;
            sc->alpha = 0.0;
            set_active(ctl, sc, 0);
        } else {
            sc->alpha = sc->rho / sums[0];
        }
        break;
    case OP_BS_S: {
        // half step: when s already meets the tolerance, x + alpha M^-1 p
        // is the solution and the iteration ends here
        const double res = sums[0] / sc->nfac;
        const bool conv = res < sc->tol || (sc->rel_tol > 1.0e-20 && res < sc->rel_tol * sc->res0);
        if (conv && sc->iter + 1 >= sc->kmin) {
            sc->res = res;
            sc->iter += 1;
            sc->converged = 1;
            set_active(ctl, sc, 0);
        }
        break;
    }
    case OP_BS_T:
        sc->omega = sums[1] > 0.0 ? sums[0] / sums[1] : 0.0;
        break;
    case OP_GSCALE_DOT:
        // foam's GAMGSolver::scale: sf = (s, f) / stabilise((A f, f), VSMALL)
        sc->alpha = sums[0] / (sums[1] >= 0.0 ? sums[1] + 1.0e-300 : sums[1] - 1.0e-300);
        break;
    case OP_BS_XR: {
        sc->res = sums[0] / sc->nfac;
        sc->iter += 1;
        const bool conv = sc->res < sc->tol || (sc->rel_tol > 1.0e-20 && sc->res < sc->rel_tol * sc->res0);
        sc->converged = conv;
        bool more = (sc->iter < sc->kmax && !conv) || sc->iter < sc->kmin;
        sc->rho_old = sc->rho;
        sc->rho = sums[1];
        if (more && (fabs(sc->omega) < 1.0e-300 || fabs(sc->rho) < 1.0e-300)) {
            sc->singular = 1;   // the recurrence cannot continue
            more = false;
        }
        if (more) sc->beta = (sc->rho / sc->rho_old) * (sc->alpha / sc->omega);
        if (!more) set_active(ctl, sc, 0);
        break;
    }
    default:
        break;
    }
}

// 4-row vector access: thread t of a tile owns the rows row0 + 4t .. 4t+3
// (one 16-byte load per FP32 array, two per FP64 array).
__device__ __forceinline__ void ld4(const float* __restrict__ p, float (&o)[4])
{
    const float4 t = __ldca(reinterpret_cast<const float4*>(p));
    o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
}
__device__ __forceinline__ void ld4(const double* __restrict__ p, double (&o)[4])
{
    const double2 a = __ldca(reinterpret_cast<const double2*>(p));
    const double2 b = __ldca(reinterpret_cast<const double2*>(p) + 1);
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}
// Plain (coherent) loads for arrays the same kernel also writes.
__device__ __forceinline__ void ld4w(const float* p, float (&o)[4])
{
    const float4 t = *reinterpret_cast<const float4*>(p);
    o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
}
__device__ __forceinline__ void ld4w(const double* p, double (&o)[4])
{
    const double2 a = reinterpret_cast<const double2*>(p)[0];
    const double2 b = reinterpret_cast<const double2*>(p)[1];
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, const float (&v)[4])
{
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&v)[4])
{
    reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}

// One 1024-row tile of a row operation.  Elementwise ops give thread t the
// four consecutive rows row0 + 4t .. 4t+3 (vector loads); ELL ops give warp w
// the slices row0/32 + w + 8k, k = 0..3.  Reductions accumulate into acc
// (FP64) in that row order.  S is the CTA's shared-memory copy of the system
// descriptor; pointers are taken into __restrict__ locals.
template <typename V, RowOp OP, bool PB>
__device__ __forceinline__ void tile_body(const Batch& B, const SysDev& S, int row0, double (&acc)[kMaxRed])
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int sl0 = row0 >> 5, sl1 = sl0 + kTileRows / 32;
    const int r4 = row0 + 4 * tid;  // first of this thread's four elementwise rows
    const int* __restrict__ sptr = S.a_sptr;
    const int* __restrict__ acol = S.a_col;
    if constexpr (OP == OP_BEGIN) {
        // Start of a solve: arm the sync-free sweep sentinels and copy the
        // batch's controls into the system's scalar state.
        const int n = S.n;
        if (S.syncfree && S.pc >= PC_DIC) {
            double* __restrict__ y = S.v64.y;
            double* __restrict__ yT = S.v64.yT;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (r4 + k < n) {
                    y[r4 + k] = sent<double>();
                    if (PB) yT[r4 + k] = sent<double>();
                }
        }
        if (row0 == 0 && tid == 0) {
            const Ctl* c = B.ctl;
            Scal* sc = S.sc;
            sc->tol = c->tol;
            sc->rel_tol = c->rel_tol;
            sc->otol = c->tol;
            sc->orel_tol = c->rel_tol;
            sc->inner_rel_tol = c->inner_rel_tol;
            sc->min_iter = c->min_iter;
            sc->max_iter = c->max_iter;
            sc->kmin = c->min_iter;
            sc->kmax = c->max_iter;
            sc->inner_max = c->inner_max;
            sc->max_outer = c->max_outer;
            sc->mixed = c->mixed;
            sc->active = 0;
            sc->ostate = 0;
            sc->iter = 0;
            sc->oiter = 0;
            sc->inner_total = 0;
            sc->converged = 0;
            sc->oconv = 0;
            sc->fallback = 0;
            sc->singular = 0;
            sc->n_sweeps = c->n_sweeps > 0 ? c->n_sweeps : 1;
        }
    } else if constexpr (OP == OP_PERMUTE_IN) {
        const int* __restrict__ perm = S.perm;
        const double* __restrict__ ib = S.in_b;
        const double* __restrict__ ix = S.in_x;
        double* __restrict__ b = S.v64.b;
        double* __restrict__ x = S.v64.x;
        const int n = S.n;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = r4 + k;
            if (i < n) {
                const int c = __ldg(perm + i);
                b[i] = __ldg(ib + c);
                x[i] = __ldg(ix + c);
            } else {
                // padding rows start every solve at zero: a solve that ended
                // early (a watchdog timeout) may have left non-finite values
                // there, which the padded row kernels would read
                b[i] = 0.0;
                x[i] = 0.0;
            }
        }
    } else if constexpr (OP == OP_PERMUTE_OUT) {
        const int* __restrict__ perm = S.perm;
        const double* __restrict__ x = S.v64.x;
        double* __restrict__ ox = S.out_x;
        const int n = S.n;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = r4 + k;
            if (i < n) ox[__ldg(perm + i)] = x[i];
        }
    } else if constexpr (OP == OP_SCATTER) {
        // FP64 views (+ FP32 copies when allocated); one warp per slice.
        const bool asym = S.aT_val != S.a_val;
        const int* __restrict__ asrc = S.a_src;
        const int* __restrict__ perm = S.perm;
        const double* __restrict__ rdiag = S.raw_diag;
        double* __restrict__ dg = S.diag;
        double* __restrict__ sA = S.sumA;
        double* __restrict__ av = S.a_val;
        double* __restrict__ atv = S.aT_val;
        float* __restrict__ dg32 = S.diag32;
        float* __restrict__ av32 = S.a_val32;
        float* __restrict__ atv32 = S.aT_val32;
        const int n = S.n;
        double* __restrict__ Dfac = S.D;
        for (int sl = sl0 + wid; sl < sl1; sl += kBlock / 32) {
            const int e0 = sptr[sl], e1 = sptr[sl + 1];
            const int i = sl * 32 + lane;
            const double d = i < n ? rdiag[perm[i]] : 0.0;
            dg[i] = d;
            if (i < n) Dfac[i] = sent<double>();  // arms the sync-free factorisation
            if (dg32) dg32[i] = (float)d;
            double s = d;
            for (int e = e0 + lane; e < e1; e += 32) {
                const int sc = asrc[e];
                const double a = sc < 0 ? 0.0 : src_val(S, sc, false);
                av[e] = a;
                if (av32) av32[e] = (float)a;
                if (asym) {
                    const double at = sc < 0 ? 0.0 : src_val(S, sc, true);
                    atv[e] = at;
                    if (atv32) atv32[e] = (float)at;
                }
                if (sc >= 0) s = __dadd_rn(s, a);
            }
            sA[i] = s;
        }
    } else if constexpr (OP == OP_SUMX) {
        V x[4];
        ld4(VP<V>::v(S).x + r4, x);
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[0] += widen(x[k]);
    } else if constexpr (OP == OP_INIT_RES) {
        const double xbar = S.sc->xsum / (double)S.n;
        const double* __restrict__ av = S.a_val;
        const double* __restrict__ atv = S.aT_val;
        const double* __restrict__ dg = S.diag;
        const double* __restrict__ sA = S.sumA;
        const double* __restrict__ x = S.v64.x;
        const double* __restrict__ b = S.v64.b;
        double* __restrict__ r = S.v64.r;
        double* __restrict__ rT = S.v64.rT;
        for (int sl = sl0 + wid; sl < sl1; sl += kBlock / 32) {
            const int i = sl * 32 + lane;
            const double ax = ell_row<double>(sptr, acol, av, dg, x, i);
            const double bi = b[i];
            const double tr = __dmul_rn(sA[i], xbar);
            acc[0] += fabs(ax - tr) + fabs(bi - tr);
            const double ri = bi - ax;
            r[i] = ri;
            acc[1] += fabs(ri);
            if (PB) rT[i] = bi - ell_row<double>(sptr, acol, atv, dg, x, i);
        }
    } else if constexpr (OP == OP_RHO) {
        const Vecs<V>& v = VP<V>::v(S);
        V w[4], rr[4];
        ld4(v.w + r4, w);
        ld4((PB ? v.rT : v.r) + r4, rr);
        acc_dot<4>(acc[0], w, rr);
    } else if constexpr (OP == OP_PUPDATE) {
        const Vecs<V>& v = VP<V>::v(S);
        const int it = S.sc->iter;
        const V beta = (V)S.sc->beta;
        V w[4], p[4];
        ld4(v.w + r4, w);
        if (it == 0) {
            st4(v.p + r4, w);
        } else {
            ld4w(v.p + r4, p);
#pragma unroll
            for (int k = 0; k < 4; ++k) p[k] = vfma(beta, p[k], w[k]);
            st4(v.p + r4, p);
        }
        if (PB) {
            V wT[4], pT[4];
            ld4(v.wT + r4, wT);
            if (it == 0) {
                st4(v.pT + r4, wT);
            } else {
                ld4w(v.pT + r4, pT);
#pragma unroll
                for (int k = 0; k < 4; ++k) pT[k] = vfma(beta, pT[k], wT[k]);
                st4(v.pT + r4, pT);
            }
        }
    } else if constexpr (OP == OP_SPMV_QP) {
        const Vecs<V>& v = VP<V>::v(S);
        const V* __restrict__ av = VP<V>::aval(S, false);
        const V* __restrict__ atv = VP<V>::aval(S, true);
        const V* __restrict__ dg = VP<V>::diag(S);
        const V* __restrict__ p = v.p;
        const V* __restrict__ pT = v.pT;
        V* __restrict__ q = v.q;
        V* __restrict__ qT = v.qT;
        if constexpr (!PB) {
            ell_tile<V>(sptr, acol, av, dg, p, sl0, [&](int i, V qi, V pi) {
                q[i] = qi;
                acc[0] = __fma_rn(widen(qi), widen(pi), acc[0]);
            });
        } else {
            for (int sl = sl0 + wid; sl < sl1; sl += kBlock / 32) {
                const int i = sl * 32 + lane;
                const V qi = ell_row<V>(sptr, acol, av, dg, p, i);
                q[i] = qi;
                qT[i] = ell_row<V>(sptr, acol, atv, dg, pT, i);
                acc[0] = __fma_rn(widen(qi), widen(pT[i]), acc[0]);
            }
        }
    } else if constexpr (OP == OP_UPDATE) {
        const Vecs<V>& v = VP<V>::v(S);
        const V alpha = (V)S.sc->alpha;
        V x[4], r[4], p[4], q[4];
        ld4w(v.x + r4, x);
        ld4w(v.r + r4, r);
        ld4(v.p + r4, p);
        ld4(v.q + r4, q);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            x[k] = vfma(alpha, p[k], x[k]);
            r[k] = vfma(-alpha, q[k], r[k]);
        }
        st4(v.x + r4, x);
        st4(v.r + r4, r);
        if (PB) {
            V rT[4], qT[4];
            ld4w(v.rT + r4, rT);
            ld4(v.qT + r4, qT);
#pragma unroll
            for (int k = 0; k < 4; ++k) rT[k] = vfma(-alpha, qT[k], rT[k]);
            st4(v.rT + r4, rT);
        }
        acc_abs<4>(acc[0], r);
    } else if constexpr (OP == OP_PRECOND_DIAG) {
        const Vecs<V>& v = VP<V>::v(S);
        V d[4], r[4], w[4];
        ld4(VP<V>::rD(S) + r4, d);
        ld4(v.r + r4, r);
#pragma unroll
        for (int k = 0; k < 4; ++k) w[k] = vmul(d[k], r[k]);
        st4(v.w + r4, w);
        if (PB) {
            ld4(v.rT + r4, r);
#pragma unroll
            for (int k = 0; k < 4; ++k) w[k] = vmul(d[k], r[k]);
            st4(v.wT + r4, w);
        }
    } else if constexpr (OP == OP_PRECOND_NONE) {
        const Vecs<V>& v = VP<V>::v(S);
        V r[4];
        ld4(v.r + r4, r);
        st4(v.w + r4, r);
        if (PB) {
            ld4(v.rT + r4, r);
            st4(v.wT + r4, r);
        }
    } else if constexpr (OP == OP_DIAG_RD) {
        const int n = S.n;
        double d[4], rd[4];
        ld4(S.diag + r4, d);
#pragma unroll
        for (int k = 0; k < 4; ++k) rd[k] = r4 + k < n ? __ddiv_rn(1.0, d[k]) : 0.0;
        st4(S.rD + r4, rd);
        if (S.rD32) {
            float f[4] = {(float)rd[0], (float)rd[1], (float)rd[2], (float)rd[3]};
            st4(S.rD32 + r4, f);
        }
    } else if constexpr (OP == OP_KEEPBEST) {
        if (!S.xb) return;
        const int keep = S.sc->okeep;
        double* __restrict__ x = S.v64.x;
        double* __restrict__ r = S.v64.r;
        double* __restrict__ xb = S.xb;
        double* __restrict__ rb = S.rb;
        double a[4], b[4];
        if (keep) {
            ld4w(x + r4, a);
            ld4w(r + r4, b);
            st4(xb + r4, a);
            st4(rb + r4, b);
        } else {
            ld4w(xb + r4, a);
            ld4w(rb + r4, b);
            st4(x + r4, a);
            st4(r + r4, b);
        }
    } else if constexpr (OP == OP_RESID64 || OP == OP_FALLBACK64) {
        const double* __restrict__ av = S.a_val;
        const double* __restrict__ atv = S.aT_val;
        const double* __restrict__ dg = S.diag;
        const double* __restrict__ x = S.v64.x;
        const double* __restrict__ b = S.v64.b;
        double* __restrict__ r = S.v64.r;
        double* __restrict__ rT = S.v64.rT;
        for (int sl = sl0 + wid; sl < sl1; sl += kBlock / 32) {
            const int i = sl * 32 + lane;
            const double bi = __ldca(b + i);
            const double ri = bi - ell_row<double>(sptr, acol, av, dg, x, i);
            r[i] = ri;
            acc[0] += fabs(ri);
            if (OP == OP_FALLBACK64 && PB) rT[i] = bi - ell_row<double>(sptr, acol, atv, dg, x, i);
        }
    } else if constexpr (OP == OP_TO32) {
        // s scales the FP64 residual to O(1) per cell before rounding to FP32.
        const double s = S.sc->osum > 0.0 ? (double)S.n / S.sc->osum : 1.0;
        const bool arm = S.syncfree && S.pc >= PC_DIC;
        const int n = S.n;
        double r64[4];
        ld4(S.v64.r + r4, r64);
        float r32[4];
        const float zero[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int k = 0; k < 4; ++k) r32[k] = (float)(r64[k] * s);
        st4(S.v32.r + r4, r32);
        if (PB) st4(S.v32.rT + r4, r32);  // the correction system starts from d = 0
        st4(S.v32.x + r4, zero);
        if (arm) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (r4 + k < n) {
                    S.v32.y[r4 + k] = sent<float>();
                    if (PB) S.v32.yT[r4 + k] = sent<float>();
                }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[0] += fabs(widen(r32[k]));
    } else if constexpr (OP == OP_CORRECT) {
        const double s = S.sc->inv_scale;
        float d32[4];
        double x[4];
        ld4(S.v32.x + r4, d32);
        ld4w(S.v64.x + r4, x);
#pragma unroll
        for (int k = 0; k < 4; ++k) x[k] = __fma_rn(widen(d32[k]), s, x[k]);
        st4(S.v64.x + r4, x);
        if (row0 == 0 && tid == 0) {
            Scal* sc = S.sc;
            sc->inner_total += sc->iter;
            sc->oiter += 1;
            if (sc->iter == 0) set_outer(B.ctl, sc, 0);  // the inner solve made no progress
        }
    } else if constexpr (OP == OP_BS_RHO0) {
        // BiCGStab start: shadow residual r~ = r, rho = (r~, r)
        const Vecs<V>& v = VP<V>::v(S);
        V r[4];
        ld4(v.r + r4, r);
        st4(v.rT + r4, r);
        acc_dot<4>(acc[0], r, r);
    } else if constexpr (OP == OP_BS_P) {
        // p = r + beta (p - omega v), p = r on the first iteration (into
        // wT); with a diagonal or no preconditioner M^-1 p goes straight to p
        const Vecs<V>& v = VP<V>::v(S);
        V r[4], p[4];
        ld4(v.r + r4, r);
        if (S.sc->iter == 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k) p[k] = r[k];
        } else {
            const V beta = (V)S.sc->beta, omega = (V)S.sc->omega;
            V q[4];
            ld4w(v.wT + r4, p);
            ld4(v.q + r4, q);
#pragma unroll
            for (int k = 0; k < 4; ++k) p[k] = vfma(beta, vfma(-omega, q[k], p[k]), r[k]);
        }
        st4(v.wT + r4, p);
        if (S.pc == PC_DIAG) {
            V d[4];
            ld4(VP<V>::rD(S) + r4, d);
#pragma unroll
            for (int k = 0; k < 4; ++k) p[k] = vmul(d[k], p[k]);
            st4(v.p + r4, p);
        } else if (S.pc == PC_NONE) {
            st4(v.p + r4, p);
        }
    } else if constexpr (OP == OP_BS_V) {
        // v = A M^-1 p, (r~, v)
        const Vecs<V>& v = VP<V>::v(S);
        const V* __restrict__ rt = v.rT;
        V* __restrict__ q = v.q;
        ell_tile<V>(sptr, acol, VP<V>::aval(S, false), VP<V>::diag(S), v.p, sl0, [&](int i, V vi, V) {
            q[i] = vi;
            acc[0] = __fma_rn(widen(vi), widen(__ldca(rt + i)), acc[0]);
        });
    } else if constexpr (OP == OP_BS_S) {
        // s = r - alpha v (in r), x += alpha M^-1 p, sum|s|; with a diagonal
        // or no preconditioner M^-1 s goes straight to pT
        const Vecs<V>& v = VP<V>::v(S);
        const V alpha = (V)S.sc->alpha;
        V x[4], r[4], ph[4], q[4];
        ld4w(v.x + r4, x);
        ld4w(v.r + r4, r);
        ld4(v.p + r4, ph);
        ld4(v.q + r4, q);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            x[k] = vfma(alpha, ph[k], x[k]);
            r[k] = vfma(-alpha, q[k], r[k]);
        }
        st4(v.x + r4, x);
        st4(v.r + r4, r);
        acc_abs<4>(acc[0], r);
        if (S.pc == PC_DIAG) {
            V d[4];
            ld4(VP<V>::rD(S) + r4, d);
#pragma unroll
            for (int k = 0; k < 4; ++k) r[k] = vmul(d[k], r[k]);
            st4(v.pT + r4, r);
        } else if (S.pc == PC_NONE) {
            st4(v.pT + r4, r);
        }
    } else if constexpr (OP == OP_BS_T) {
        // t = A M^-1 s, (t, s), (t, t)
        const Vecs<V>& v = VP<V>::v(S);
        const V* __restrict__ sv = v.r;
        V* __restrict__ t = v.qT;
        ell_tile<V>(sptr, acol, VP<V>::aval(S, false), VP<V>::diag(S), v.pT, sl0, [&](int i, V ti, V) {
            t[i] = ti;
            const double tw = widen(ti);
            acc[0] = __fma_rn(tw, widen(__ldca(sv + i)), acc[0]);
            acc[1] = __fma_rn(tw, tw, acc[1]);
        });
    } else if constexpr (OP == OP_BS_XR) {
        // x += omega M^-1 s, r = s - omega t, sum|r|, (r~, r)
        const Vecs<V>& v = VP<V>::v(S);
        const V omega = (V)S.sc->omega;
        V x[4], r[4], sh[4], t[4], rt[4];
        ld4w(v.x + r4, x);
        ld4w(v.r + r4, r);
        ld4(v.pT + r4, sh);
        ld4(v.qT + r4, t);
        ld4(v.rT + r4, rt);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            x[k] = vfma(omega, sh[k], x[k]);
            r[k] = vfma(-omega, t[k], r[k]);
        }
        st4(v.x + r4, x);
        st4(v.r + r4, r);
        acc_abs<4>(acc[0], r);
        acc_dot<4>(acc[1], rt, r);
    } else if constexpr (OP == OP_GS_ARM || OP == OP_GS_COPY) {
        const int n = S.n;
        double* __restrict__ x = S.v64.x;
        double* __restrict__ y = S.v64.y;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (r4 + k < n) {
                if (OP == OP_GS_COPY) x[r4 + k] = y[r4 + k];
                y[r4 + k] = sent<double>();
            }
    } else if constexpr (OP == OP_SM_RES) {
        const double* __restrict__ x = S.v64.x;
        const double* __restrict__ b = S.v64.b;
        double* __restrict__ r = S.v64.r;
        for (int sl = sl0 + wid; sl < sl1; sl += kBlock / 32) {
            const int i = sl * 32 + lane;
            r[i] = __ldca(b + i) - ell_row<double>(sptr, acol, S.a_val, S.diag, x, i);
        }
    } else if constexpr (OP == OP_SM_ADD) {
        double x[4], w[4];
        ld4w(S.v64.x + r4, x);
        ld4(S.v64.w + r4, w);
#pragma unroll
        for (int k = 0; k < 4; ++k) x[k] = __dadd_rn(x[k], w[k]);
        st4(S.v64.x + r4, x);
    } else if constexpr (OP == OP_GS_RES) {
        const double* __restrict__ x = S.v64.x;
        const double* __restrict__ b = S.v64.b;
        double* __restrict__ r = S.v64.r;
        for (int sl = sl0 + wid; sl < sl1; sl += kBlock / 32) {
            const int i = sl * 32 + lane;
            const double ri = __ldca(b + i) - ell_row<double>(sptr, acol, S.a_val, S.diag, x, i);
            r[i] = ri;
            acc[0] += fabs(ri);
        }
    } else if constexpr (OP == OP_GSCALE_DOT) {
        // GAMG scaleCorrection of a correction f (in p) against its source s
        // (in r): q = A f, (s, f), (A f, f); padding rows add fma(0, 0, .)
        const double* __restrict__ f = S.v64.p;
        const double* __restrict__ sv = S.v64.r;
        double* __restrict__ q = S.v64.q;
        const int n = S.n;
        for (int sl = sl0 + wid; sl < sl1; sl += kBlock / 32) {
            const int i = sl * 32 + lane;
            const double qi = ell_row<double>(sptr, acol, S.a_val, S.diag, f, i);
            q[i] = qi;
            const bool in = i < n;
            const double fi = in ? __ldca(f + i) : 0.0;
            acc[0] = __fma_rn(in ? __ldca(sv + i) : 0.0, fi, acc[0]);
            acc[1] = __fma_rn(in ? qi : 0.0, fi, acc[1]);
        }
    } else if constexpr (OP == OP_GSCALE_SET || OP == OP_GSCALE_ADD) {
        // f = sf f + (s - sf A f) / diag, one rounding per operation; the
        // finest level adds it to x, a coarse level's correction is it
        const double sf = S.sc->alpha;
        const double* __restrict__ f = S.v64.p;
        const double* __restrict__ sv = S.v64.r;
        const double* __restrict__ q = S.v64.q;
        const double* __restrict__ dg = S.diag;
        double* __restrict__ x = S.v64.x;
        const int n = S.n;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = r4 + k;
            if (i < n) {
                const double t = __ddiv_rn(__dsub_rn(__ldca(sv + i), __dmul_rn(sf, __ldca(q + i))), __ldca(dg + i));
                const double v = __dadd_rn(__dmul_rn(sf, __ldca(f + i)), t);
                x[i] = OP == OP_GSCALE_ADD ? __dadd_rn(x[i], v) : v;
            }
        }
    } else if constexpr (OP == OP_AMUL || OP == OP_TMUL) {
        const double* __restrict__ av = OP == OP_TMUL ? S.aT_val : S.a_val;
        const double* __restrict__ dg = S.diag;
        const double* __restrict__ p = S.v64.p;
        double* __restrict__ q = S.v64.q;
        for (int sl = sl0 + wid; sl < sl1; sl += kBlock / 32) {
            const int i = sl * 32 + lane;
            q[i] = ell_row<double>(sptr, acol, av, dg, p, i);
        }
    }
}

// Two tiles (rows a and b) of an op with a two-tile body, not PBiCG:
// both tiles' loads are issued before either's arithmetic and stores (two
// calls of tile_body keep the second tile's loads behind the first one's
// stores, which may alias for the compiler).  Each row's arithmetic and
// the order of the reduction terms (tile a's rows, then tile b's) are
// tile_body's, so the bits are too.
// Ops with a two-tile body: the x/r and p updates, and in FP32 BiCGStab's s
// and x/r updates (their FP64 pairs would spill).
template <typename V, RowOp OP>
constexpr bool kPairOp =
    OP == OP_UPDATE || OP == OP_PUPDATE || (sizeof(V) == 4 && (OP == OP_BS_S || OP == OP_BS_XR));

template <typename V, RowOp OP>
__device__ __forceinline__ void tile_pair(const SysDev& S, int row_a, int row_b, double (&acc)[kMaxRed])
{
    static_assert(kPairOp<V, OP>, "ops with a two-tile body");
    const Vecs<V>& v = VP<V>::v(S);
    const int r4[2] = {row_a + 4 * (int)threadIdx.x, row_b + 4 * (int)threadIdx.x};
    if constexpr (OP == OP_UPDATE) {
        const V alpha = (V)S.sc->alpha;
        V x[2][4], r[2][4], p[2][4], q[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            ld4w(v.x + r4[h], x[h]);
            ld4w(v.r + r4[h], r[h]);
            ld4(v.p + r4[h], p[h]);
            ld4(v.q + r4[h], q[h]);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                x[h][k] = vfma(alpha, p[h][k], x[h][k]);
                r[h][k] = vfma(-alpha, q[h][k], r[h][k]);
            }
            st4(v.x + r4[h], x[h]);
            st4(v.r + r4[h], r[h]);
            acc_abs<4>(acc[0], r[h]);
        }
    } else if constexpr (OP == OP_BS_S) {
        // s = r - alpha v (in r), x += alpha M^-1 p, sum|s|; M^-1 s into pT
        // for a diagonal or no preconditioner
        const V alpha = (V)S.sc->alpha;
        const int pc = S.pc;
        V x[2][4], r[2][4], ph[2][4], q[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            ld4w(v.x + r4[h], x[h]);
            ld4w(v.r + r4[h], r[h]);
            ld4(v.p + r4[h], ph[h]);
            ld4(v.q + r4[h], q[h]);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                x[h][k] = vfma(alpha, ph[h][k], x[h][k]);
                r[h][k] = vfma(-alpha, q[h][k], r[h][k]);
            }
            st4(v.x + r4[h], x[h]);
            st4(v.r + r4[h], r[h]);
            acc_abs<4>(acc[0], r[h]);
            if (pc == PC_DIAG) {
                V d[4];
                ld4(VP<V>::rD(S) + r4[h], d);
#pragma unroll
                for (int k = 0; k < 4; ++k) d[k] = vmul(d[k], r[h][k]);
                st4(v.pT + r4[h], d);
            } else if (pc == PC_NONE) {
                st4(v.pT + r4[h], r[h]);
            }
        }
    } else if constexpr (OP == OP_BS_XR) {
        // x += omega M^-1 s, r = s - omega t, sum|r|, (r~, r)
        const V omega = (V)S.sc->omega;
        V x[2][4], r[2][4], sh[2][4], t[2][4], rt[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            ld4w(v.x + r4[h], x[h]);
            ld4w(v.r + r4[h], r[h]);
            ld4(v.pT + r4[h], sh[h]);
            ld4(v.qT + r4[h], t[h]);
            ld4(v.rT + r4[h], rt[h]);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                x[h][k] = vfma(omega, sh[h][k], x[h][k]);
                r[h][k] = vfma(-omega, t[h][k], r[h][k]);
            }
            st4(v.x + r4[h], x[h]);
            st4(v.r + r4[h], r[h]);
            acc_abs<4>(acc[0], r[h]);
            acc_dot<4>(acc[1], rt[h], r[h]);
        }
    } else {
        const int it = S.sc->iter;
        const V beta = (V)S.sc->beta;
        V w[2][4], p[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            ld4(v.w + r4[h], w[h]);
            if (it != 0) ld4w(v.p + r4[h], p[h]);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (it == 0) {
                st4(v.p + r4[h], w[h]);
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) p[h][k] = vfma(beta, p[h][k], w[h][k]);
                st4(v.p + r4[h], p[h]);
            }
        }
    }
}

template <RowOp OP>
struct OpTraits {
    static constexpr bool kRed = (OP == OP_SUMX || OP == OP_INIT_RES || OP == OP_RHO || OP == OP_SPMV_QP ||
                                  OP == OP_UPDATE || OP == OP_RESID64 || OP == OP_TO32 || OP == OP_FALLBACK64 ||
                                  OP == OP_BS_RHO0 || OP == OP_BS_V || OP == OP_BS_S || OP == OP_BS_T ||
                                  OP == OP_BS_XR || OP == OP_GS_RES || OP == OP_RHO_CH || OP == OP_GSCALE_DOT);
    // Krylov-loop ops run only for systems whose loop is active; the
    // refinement ops only for systems whose outer loop is active.
    static constexpr bool kNeedActive = (OP == OP_RHO || OP == OP_PUPDATE || OP == OP_SPMV_QP ||
                                         OP == OP_UPDATE || OP == OP_PRECOND_DIAG || OP == OP_PRECOND_NONE ||
                                         OP == OP_BS_RHO0 || OP == OP_BS_P || OP == OP_BS_V || OP == OP_BS_S ||
                                         OP == OP_BS_T || OP == OP_BS_XR || OP == OP_GS_COPY || OP == OP_GS_RES ||
                                         OP == OP_SM_RES || OP == OP_SM_ADD || OP == OP_RHO_CH ||
                                         OP == OP_GSCALE_DOT || OP == OP_GSCALE_SET || OP == OP_GSCALE_ADD);
    static constexpr bool kNeedOuter = (OP == OP_RESID64 || OP == OP_TO32 || OP == OP_CORRECT);
    // Values reduced: the initial residual needs two (normFactor and
    // sum|r|), BiCGStab's t step ((t, s), (t, t)) and its update (sum|r|,
    // (r~, r)) too.  Every tree level costs one FP64 add per thread per value.
    static constexpr int kNR = (OP == OP_INIT_RES || OP == OP_BS_T || OP == OP_BS_XR || OP == OP_GSCALE_DOT) ? 2 : 1;
    // four consecutive rows per thread, no gathers: worth interleaving tiles
    static constexpr bool kElem = (OP == OP_SUMX || OP == OP_RHO || OP == OP_PUPDATE || OP == OP_UPDATE ||
                                   OP == OP_PRECOND_DIAG || OP == OP_PRECOND_NONE || OP == OP_TO32 ||
                                   OP == OP_CORRECT || OP == OP_KEEPBEST || OP == OP_BS_RHO0 || OP == OP_BS_P ||
                                   OP == OP_BS_S || OP == OP_BS_XR || OP == OP_GS_ARM || OP == OP_GS_COPY ||
                                   OP == OP_SM_ADD || OP == OP_GSCALE_SET || OP == OP_GSCALE_ADD);
};

template <RowOp OP>
__device__ __forceinline__ bool system_live(const SysDev& S)
{
    if (OpTraits<OP>::kNeedActive) return S.sc->active != 0;
    if (OpTraits<OP>::kNeedOuter) return S.sc->ostate != 0;
    if (OP == OP_FALLBACK64) return S.sc->fallback == 1 || S.sc->fallback == 2;
    return true;
}

// Close reduction segment `seg` of one system (consecutive units -- tiles,
// or for the FP32 SpMV rounds -- `count` of them, handled by this CTA, of
// `total` units the system has; total < 0: its tile count): block tree, partial into slot `seg`, and
// the CTA that completes the system's tile count sums the G slots -- thread
// t the slots t, t + 256, ... in order -- and finalises.  Every slot is
// rewritten by every reduction, so none needs clearing.  Deterministic: the
// order depends only on the system.
template <RowOp OP, bool NB = false>
__device__ __forceinline__ void flush_segment(const Batch& B, const SysDev& S, int seg, int count,
                                              double (&acc)[kMaxRed], double* sh, int* s_last, int total = -1)
{
    constexpr int NR = OpTraits<OP>::kNR;
    const int tid = threadIdx.x;
    double a[NR];
#pragma unroll
    for (int k = 0; k < NR; ++k) a[k] = acc[k];
    block_sum<NR, NB>(a, sh);
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < NR; ++k) S.partials[seg * kMaxRed + k] = a[k];
        __threadfence();
        const unsigned prev = atomicAdd(S.counter, (unsigned)count);
        *s_last = (prev + (unsigned)count == (unsigned)(total < 0 ? S.ntiles : total));
    }
    row_barrier<NB>();
    if (*s_last) {
        const int G = red_segments(S.ntiles);
        // every slot this thread sums, loaded before the first add
        constexpr int kMaxPer = (kRedSegs + kBlock - 1) / kBlock;
        double v[kMaxPer][NR];
#pragma unroll
        for (int c = 0; c < kMaxPer; ++c) {
            const int j = tid + c * kBlock;
#pragma unroll
            for (int k = 0; k < NR; ++k) v[c][k] = j < G ? __ldcg(S.partials + j * kMaxRed + k) : 0.0;
        }
        double tot[NR];
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            tot[k] = 0.0;
#pragma unroll
            for (int c = 0; c < kMaxPer; ++c)
                if (tid + c * kBlock < G) tot[k] += v[c][k];
        }
        block_sum<NR, NB>(tot, sh);
        if (tid == 0) {
            double sums[kMaxRed] = {0.0, 0.0};
#pragma unroll
            for (int k = 0; k < NR; ++k) sums[k] = tot[k];
            finalize(B, S, OP, sums);
            *S.counter = 0u;
            __threadfence();
        }
    }
    row_barrier<NB>();
}

// Amul + (q, p) over rounds [rb, re) of one system (round r: the rows of
// slice 8 r + w for warp w, kBlock / 32 = 8 warps), row by row in round order.
template <typename V>
__device__ __forceinline__ void spmv_rounds(const SysDev& S, int rb, int re, double (&acc)[kMaxRed])
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const V* __restrict__ av = VP<V>::aval(S, false);
    const V* __restrict__ dg = VP<V>::diag(S);
    const V* __restrict__ p = VP<V>::v(S).p;
    V* __restrict__ q = VP<V>::v(S).q;
    for (int r = rb; r < re; ++r) {
        const int i = ((kBlock / 32) * r + wid) * 32 + lane;
        const V xi = __ldca(p + i);
        const V y = ell_row<V>(S.a_sptr, S.a_col, av, dg, p, i);
        q[i] = y;
        acc[0] = __fma_rn(widen(y), widen(xi), acc[0]);
    }
}

// Row kernel over a batch.  Non-reducing ops: grid-stride over the tile
// table.  Reducing ops: grid-stride over the segment table; a segment
// (system s, j) covers the contiguous tiles [j*T/G, (j+1)*T/G) of s (T its
// tile count, G = min(T, kRedSegs)), accumulates across them and pays the
// fence/atomic/tree cost once.  The system's descriptor is copied into
// shared memory once per CTA and system, so threads read its pointers from
// shared memory instead of each issuing ~40 global loads.
static_assert(sizeof(SysDev) % 8 == 0, "SysDev is copied as 8-byte words");

__device__ __forceinline__ void load_sys(SysDev* dst, const SysDev* src)
{
    __syncthreads();  // the previous system's copy is no longer in use
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(dst);
    for (int k = threadIdx.x; k < (int)(sizeof(SysDev) / 8); k += blockDim.x) d[k] = s[k];
    __syncthreads();
}

// The system of this CTA's first work item (segment table for reducing
// ops, tile table otherwise), -1 if it has none.
template <bool RED>
__device__ __forceinline__ int first_system(const Batch& B)
{
    const int g = blockIdx.x;
    if (g >= (RED ? B.nsegs : B.ntiles)) return -1;
    if (B.nsys == 1) return 0;
    return RED ? B.segs[g].x : B.tiles[g].x;
}

// Tiles [t0, t1) of one reduction segment of a system, accumulated in acc
// (element-wise ops: two tiles' loads in flight, the same order).
template <typename V, RowOp OP, bool PB>
__device__ __forceinline__ void segment_tiles(const Batch& B, const SysDev& sS, int t0, int t1,
                                              double (&acc)[kMaxRed])
{
    if constexpr (OpTraits<OP>::kElem) {
        int t = t0;
        for (; t + 1 < t1; t += 2) {
            if constexpr (!PB && kPairOp<V, OP>) {
                tile_pair<V, OP>(sS, t * kTileRows, (t + 1) * kTileRows, acc);
            } else {
                tile_body<V, OP, PB>(B, sS, t * kTileRows, acc);
                tile_body<V, OP, PB>(B, sS, (t + 1) * kTileRows, acc);
            }
        }
        if (t < t1) tile_body<V, OP, PB>(B, sS, t * kTileRows, acc);
    } else {
        for (int t = t0; t < t1; ++t) tile_body<V, OP, PB>(B, sS, t * kTileRows, acc);
    }
}

// One row operation over the whole batch by this CTA: grid-stride over the
// tile table (non-reducing ops) or the segment table (reducing ops).  `cur`
// names the system whose descriptor sS holds, so a persistent kernel that
// runs several operations in turn copies it only when the system changes;
// whether the system takes part is re-read on every call.
template <typename V, RowOp OP, bool PB>
__device__ __forceinline__ void rows_phase(const Batch& B, SysDev& sS, double* sh, int* s_last, int& cur)
{
    int lcur = -1;
    bool live = false;
    if constexpr (!OpTraits<OP>::kRed) {
        // element-wise ops: two tiles per step when both belong to the same
        // system, so one tile's loads are in flight while the other computes
        for (int t = blockIdx.x; t < B.ntiles; t += gridDim.x) {
            const int2 tl = B.nsys == 1 ? make_int2(0, t) : B.tiles[t];
            if (tl.x != lcur) {
                lcur = tl.x;
                if (tl.x != cur) {
                    cur = tl.x;
                    load_sys(&sS, B.sys + cur);
                }
                live = system_live<OP>(sS);
            }
            if (!live) continue;
            double acc[kMaxRed] = {0.0, 0.0};
            if constexpr (OpTraits<OP>::kElem) {
                const int t2 = t + gridDim.x;
                if (B.nsys == 1 && t2 < B.ntiles) {
                    if constexpr (!PB && kPairOp<V, OP>) {
                        tile_pair<V, OP>(sS, tl.y * kTileRows, t2 * kTileRows, acc);
                    } else {
                        tile_body<V, OP, PB>(B, sS, tl.y * kTileRows, acc);
                        tile_body<V, OP, PB>(B, sS, t2 * kTileRows, acc);
                    }
                    t = t2;
                    continue;
                }
            }
            tile_body<V, OP, PB>(B, sS, tl.y * kTileRows, acc);
        }
    } else {
        for (int g = blockIdx.x; g < B.nsegs; g += gridDim.x) {
            const int2 sg = B.nsys == 1 ? make_int2(0, g) : B.segs[g];
            if (sg.x != lcur) {
                lcur = sg.x;
                if (sg.x != cur) {
                    cur = sg.x;
                    load_sys(&sS, B.sys + cur);
                }
                live = system_live<OP>(sS);  // uniform over all of the system's segments
            }
            if (!live) continue;
            const unsigned T = (unsigned)sS.ntiles, G = (unsigned)red_segments(sS.ntiles);
            if constexpr (OP == OP_RHO_CH) {
                // rho from the sweeps' chunk sums: segment sg.y takes the
                // chunks [c0, c1), thread t its chunks c0 + t, c0 + t + kBlock,
                // ...; the tile count keeps the segment bookkeeping
                const long long nch = sS.nchunks;
                const int c0 = (int)(sg.y * nch / G), c1 = (int)((sg.y + 1) * nch / G);
                const int t0 = (int)(((unsigned)sg.y * T) / G), t1 = (int)(((unsigned)(sg.y + 1) * T) / G);
                double acc[kMaxRed] = {0.0, 0.0};
                for (int c = c0 + (int)threadIdx.x; c < c1; c += kBlock) acc[0] += widen(__ldcg(sS.chunk_rw + c));
                flush_segment<OP>(B, sS, sg.y, t1 - t0, acc, sh, s_last);
                continue;
            }
            if constexpr (OP == OP_SPMV_QP && !PB && sizeof(V) == 4) {
                // FP32 Amul + (q, p): segments of rounds, each thread's rows
                // and their order k_spmv_warp's, so both give the same bits
                const unsigned long long U = 4ull * T;
                const int u0 = (int)(((unsigned long long)sg.y * U) / G);
                const int u1 = (int)(((unsigned long long)(sg.y + 1) * U) / G);
                double acc[kMaxRed] = {0.0, 0.0};
                spmv_rounds<V>(sS, u0, u1, acc);
                flush_segment<OP>(B, sS, sg.y, u1 - u0, acc, sh, s_last, (int)U);
                continue;
            }
            const int t0 = (int)(((unsigned)sg.y * T) / G), t1 = (int)(((unsigned)(sg.y + 1) * T) / G);
            double acc[kMaxRed] = {0.0, 0.0};
            segment_tiles<V, OP, PB>(B, sS, t0, t1, acc);
            flush_segment<OP>(B, sS, sg.y, t1 - t0, acc, sh, s_last);
        }
    }
}

template <typename V, RowOp OP, bool PB>
__global__ void __launch_bounds__(kBlock, kMinCtas) k_rows(const Batch* __restrict__ pB)
{
    __shared__ double sh[kBlock * kMaxRed];
    __shared__ int s_last;
    __shared__ __align__(16) SysDev sS;
    // descriptors (host-written) while the previous kernel drains
    const Batch B = *pB;
    int cur = first_system<OpTraits<OP>::kRed>(B);
    if (cur >= 0) load_sys(&sS, B.sys + cur);
    pdl_enter();
    rows_phase<V, OP, PB>(B, sS, sh, &s_last, cur);
}

// ---------------------------------------------------------------- staged SpMV
// Amul + (q, p) of the Krylov loop with the sliced-ELL column indices (and,
// in FP64, the coefficients) staged in shared memory by the bulk-copy
// engine.  Rows are walked in rounds of 8 slices, one slice per warp (round
// r: slices 8 r .. 8 r + 7, so a 1024-row tile is four rounds and warp w
// takes its slices w, w+8, w+16, w+24 -- ell_tile's rows in ell_tile's
// order).  Every warp keeps its own ring of stages, each holding one of its
// slices, and its own mbarriers; its lane 0 keeps the copies of the warp's
// next slices in flight (one cp.async.bulk per array per slice), and a stage
// is released by __syncwarp, so within a segment no warp waits for another.
// In FP32 a warp takes two rounds per step and issues both rounds'
// coefficient, own-x, diagonal and gathered-x loads before any arithmetic:
// the gathers are the latency that bounds this kernel.  A slice wider than
// a stage (W > kMaxW) is read from global memory instead.  Waits are
// bounded: on timeout the error bit is set and the CTA leaves after its
// copies land.
template <typename V> struct SpmvStages;
// Stages per warp -- FP32: four (column indices; 24 KB per CTA), two rounds
// per step with their coefficients, own x and gathered x loaded together;
// FP64: two (indices and coefficients), one round per step.
template <> struct SpmvStages<float> { static constexpr int n = 4, rounds = 2, vals = 0; };
template <> struct SpmvStages<double> { static constexpr int n = 2, rounds = 1, vals = 1; };
static_assert(4 % SpmvStages<double>::rounds == 0, "FP64 segments are whole tiles of four rounds");
static_assert(kTileRows == 4 * kBlock, "a tile is four rounds of one slice per warp");
constexpr int kSliceEntries = kMaxW * 32;                    // entries one stage holds

__device__ __forceinline__ unsigned smem_u32(const void* p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, unsigned bytes)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     smem_u32(b)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, unsigned bytes, unsigned long long* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// L2 policy for data read once per launch (coefficients, column indices,
// the diagonal): evicted first, so the gathered vector -- written by the
// previous kernel and read up to seven times here -- keeps its L2 lines.
__device__ __forceinline__ unsigned long long l2_evict_first()
{
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ void bulk_to_smem_stream(void* dst, const void* src, unsigned bytes,
                                                    unsigned long long* bar, unsigned long long pol)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
        "%4;" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}
__device__ __forceinline__ float ldg_stream(const float* p, unsigned long long pol)
{
    float v;
    asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ double ldg_stream(const double* p, unsigned long long pol)
{
    double v;
    asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, "
        "p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for a stage's phase; false (error bit set) on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity, Ctl* ctl)
{
    if (mbar_try_wait(b, parity)) return true;
    const long long t0 = clock64();
    for (int it = 1;; ++it) {
        if (mbar_try_wait(b, parity)) return true;
        if ((it & 63) == 0 && clock64() - t0 > wait_budget(ctl)) {
            atomicOr(&ctl->err, ERR_TIMEOUT);
            return false;
        }
    }
}

template <typename V>
constexpr size_t spmv_smem()
{
    return (size_t)(kBlock / 32) * SpmvStages<V>::n * kSliceEntries *
           (sizeof(int) + (SpmvStages<V>::vals ? sizeof(V) : 0));
}

// Segments: FP64 whole tiles (the reduction order the oracle mirrors);
// FP32 rounds, so that segments differ by one round at most instead of one
// tile (at five tiles a segment, a fifth of the work).  rows_phase's FP32
// Amul + (q, p) (the persistent kernel's) walks the same rounds.
template <typename V>
__global__ void __launch_bounds__(kBlock, kMinCtas) k_spmv_warp(const Batch* __restrict__ pB)
{
    constexpr int S = SpmvStages<V>::n;
    constexpr int RP = SpmvStages<V>::rounds;
    constexpr bool kVals = SpmvStages<V>::vals;
    constexpr int NW = kBlock / 32;
    __shared__ double sh[kBlock * kMaxRed];
    __shared__ int s_last, s_abort;
    __shared__ __align__(16) SysDev sS;
    __shared__ __align__(8) unsigned long long full[NW][S];
    extern __shared__ __align__(128) unsigned char dyn[];
    const Batch B = *pB;   // descriptors (host-written) while the previous kernel drains
    Ctl* ctl = B.ctl;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    // this warp's stage k: indices at col_st(k), coefficients at val_st(k),
    // mbarrier full[wid][k]
    int* const st_col = reinterpret_cast<int*>(dyn);
    V* const st_val = reinterpret_cast<V*>(dyn + sizeof(int) * NW * S * kSliceEntries);
#define col_st(k) (st_col + (wid * S + (k)) * kSliceEntries)
#define val_st(k) (st_val + (wid * S + (k)) * kSliceEntries)
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < S; ++k) mbar_init(&full[wid][k], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid == 0) s_abort = 0;
    int cur = first_system<true>(B);
    if (cur >= 0) load_sys(&sS, B.sys + cur);   // its __syncthreads also covers the mbarrier init
    pdl_enter();
    unsigned parity = 0;   // bit k: parity of this warp's stage k's next completion
    int lcur = -1;
    bool live = false;
    for (int g = blockIdx.x; g < B.nsegs; g += gridDim.x) {
        const int2 sg = B.nsys == 1 ? make_int2(0, g) : B.segs[g];
        if (sg.x != lcur) {
            lcur = sg.x;
            if (sg.x != cur) {
                cur = sg.x;
                load_sys(&sS, B.sys + cur);
            }
            live = system_live<OP_SPMV_QP>(sS);
        }
        if (!live) continue;
        constexpr bool kRoundSeg = sizeof(V) == 4;
        const unsigned T = (unsigned)sS.ntiles, G = (unsigned)red_segments(sS.ntiles);
        const unsigned long long U = kRoundSeg ? 4ull * T : (unsigned long long)T;
        const int u0 = (int)(((unsigned long long)sg.y * U) / G), u1 = (int)(((unsigned long long)(sg.y + 1) * U) / G);
        // rounds [rb, re) of the system; round r: this warp's slice NW r + wid,
        // into stage r % S (each stage's parity is tracked on its own, so the
        // ring may start at any stage)
        const int rb = kRoundSeg ? u0 : 4 * u0;
        const int re = kRoundSeg ? u1 : 4 * u1;
        const int* __restrict__ sptr = sS.a_sptr;
        const int* __restrict__ acol = sS.a_col;
        const V* __restrict__ aval = VP<V>::aval(sS, false);
        const V* __restrict__ dg = VP<V>::diag(sS);
        const V* __restrict__ p = VP<V>::v(sS).p;
        V* __restrict__ q = VP<V>::v(sS).q;
        const unsigned long long pol = l2_evict_first();
        auto issue = [&](int r) {
            const int sl = NW * r + wid;
            const int e0 = __ldg(sptr + sl), cnt = __ldg(sptr + sl + 1) - e0;
            const int stg = r % S;
            if (cnt > 0 && cnt <= kSliceEntries) {
                mbar_expect_tx(&full[wid][stg], (unsigned)cnt * (unsigned)(sizeof(int) + (kVals ? sizeof(V) : 0)));
                bulk_to_smem_stream(col_st(stg), acol + e0, (unsigned)cnt * sizeof(int), &full[wid][stg], pol);
                if (kVals)
                    bulk_to_smem_stream(val_st(stg), aval + e0, (unsigned)cnt * sizeof(V), &full[wid][stg], pol);
            } else {
                mbar_expect_tx(&full[wid][stg], 0u);
            }
        };
        if (lane == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            for (int r = rb; r < rb + S - RP && r < re; ++r) issue(r);
        }
        double acc[kMaxRed] = {0.0, 0.0};
        bool ok = true;
        int r = rb;
        for (; r < re; r += RP) {
            if (lane == 0)
                for (int j = 0; j < RP; ++j)
                    if (r + S - RP + j < re) issue(r + S - RP + j);
            for (int j = 0; j < RP && r + j < re; ++j) {
                const int stg = (r + j) % S;
                if (!mbar_wait(&full[wid][stg], (parity >> stg) & 1u, ctl)) ok = false;
                parity ^= 1u << stg;
            }
            if (!__all_sync(kFull, ok)) {
                ok = false;
                break;
            }
            // a slice is staged exactly when it fits a stage (W <= kMaxW):
            // the fast path reads its indices by shared-memory offset
            int i_[RP], W_[RP], e_[RP], cs[RP];
            bool fast = true;
#pragma unroll
            for (int j = 0; j < RP; ++j) {
                const int rj = r + j;   // FP32 segments may end on an odd round
                const bool on = rj < re;
                const int sl = NW * rj + wid;
                e_[j] = on ? __ldg(sptr + sl) : 0;
                W_[j] = on ? (__ldg(sptr + sl + 1) - e_[j]) >> 5 : 0;
                i_[j] = sl * 32 + lane;
                cs[j] = (wid * S + rj % S) * kSliceEntries + lane;
                fast = fast && on && W_[j] <= kMaxW;
            }
            if (fast) {
                V xi[RP], dv[RP], xv[RP][kMaxW], av[RP][kMaxW];
                unsigned lv[RP];
#pragma unroll
                for (int j = 0; j < RP; ++j) {
                    xi[j] = __ldca(p + i_[j]);
                    dv[j] = ldg_stream(dg + i_[j], pol);
                    lv[j] = 0;
#pragma unroll
                    for (int k = 0; k < kMaxW; ++k) {
                        const int ck = k < W_[j] ? st_col[cs[j] + k * 32] : -1;
                        lv[j] |= (ck >= 0 ? 1u : 0u) << k;
                        xv[j][k] = ck >= 0 ? __ldca(p + ck) : V(0);
                        if constexpr (!kVals) av[j][k] = ck >= 0 ? ldg_stream(aval + e_[j] + lane + k * 32, pol) : V(0);
                    }
                }
#pragma unroll
                for (int j = 0; j < RP; ++j) {
                    V y = vmul(dv[j], xi[j]);
#pragma unroll
                    for (int k = 0; k < kMaxW; ++k)
                        if (lv[j] & (1u << k)) y = vfma(kVals ? st_val[cs[j] + k * 32] : av[j][k], xv[j][k], y);
                    q[i_[j]] = y;
                    acc[0] = __fma_rn(widen(y), widen(xi[j]), acc[0]);
                }
            } else {
                for (int j = 0; j < RP && r + j < re; ++j) {
                    const bool staged = W_[j] <= kMaxW;
                    const int* cp = staged ? st_col + cs[j] : acol + e_[j] + lane;
                    const V* ap = (staged && kVals) ? st_val + cs[j] : aval + e_[j] + lane;
                    const V xi = __ldca(p + i_[j]);
                    V y = vmul(__ldg(dg + i_[j]), xi);
                    for (int k0 = 0; k0 < W_[j]; k0 += kMaxW) y = ell_round<V, false>(cp, ap, p, k0, W_[j], y);
                    q[i_[j]] = y;
                    acc[0] = __fma_rn(widen(y), widen(xi), acc[0]);
                }
            }
            __syncwarp();   // this step's stages are free for the rounds S ahead
            if (lane == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        if (!ok) {
            // the copies this warp issued (rounds r .. r + S - 1) land before
            // the CTA leaves (the step's own rounds had their parity bit
            // flipped already); the flush below still runs so every warp
            // meets its barriers
            if (lane == 0) {
                for (int k = r; k < re && k < r + S; ++k)
                    mbar_wait(&full[wid][k % S], ((parity >> (k % S)) & 1u) ^ (k < r + RP ? 1u : 0u), ctl);
                s_abort = 1;
            }
            __syncwarp();
        }
        flush_segment<OP_SPMV_QP>(B, sS, sg.y, u1 - u0, acc, sh, &s_last, (int)U);
        if (s_abort) return;   // read after the flush's closing barrier
    }
}
#undef col_st
#undef val_st

// ------------------------------------------------------------ streamed SpMV
// Amul + (q, p) with the streamed operands brought in by the bulk-copy
// (TMA) engine: a producer warp walks the CTA's segments round by round
// (256 rows: the 8 slices of 32 rows the 8 row warps take, as in
// k_spmv_warp) and copies, per round, into a ring of S shared-memory
// stages: the round's slice bounds, column indices and coefficients (one
// contiguous range each, since a round's slices are consecutive in the
// sliced ELL), and with one round per step also the rows' own x and
// diagonal.  The copies of coefficients, indices and diagonal carry an L2
// evict-first policy, so the gathered vector keeps its L2 lines.  The row
// warps load only the gathered x (and, with two rounds per step, own x and
// diagonal) from global memory: the DRAM latency of the streams is off
// their chain and the copies of the next rounds are in flight while a round
// computes.  With RP = 2 a warp takes two rounds per step and has both
// rounds' gathers in flight at once.  Each row's arithmetic and each
// thread's rows and their order are k_spmv_warp's, so all kernels give the
// same bits (FP64: the order the oracle mirrors).  A round whose entries
// exceed a stage (kStageCap) has only its bounds (and own x, diagonal)
// staged; its rows read indices and coefficients from global memory.  Waits
// are bounded: on a timeout the error bit is set, the row warps leave their
// loop, and the producer waits (bounded) for the copies it issued before the
// CTA exits.
// S stages; XD: own x and diagonal staged (else the row warps load them);
// N16: rounds whose slices have 16-bit column offsets copy those instead of
// the 32-bit indices; CB: bytes a column index takes in a stage -- 2: only
// rounds with 16-bit columns are staged (a round with 32-bit columns reads
// its indices and coefficients from global memory), 4: both kinds; ER: a
// warp releases its stage as soon as the stage's values are in registers
// (before its gathers), else after its rows are done.
template <typename V, int RP> struct StreamCfg;
// one round per step: three stages of 14.5 KB (FP32) / two of 22.6 KB (FP64),
// 32-bit columns (measured fastest for one round per step on GB300)
template <> struct StreamCfg<float, 1> {
    static constexpr int S = 3, CB = 4;
    static constexpr bool XD = true, N16 = false, ER = false;
};
template <> struct StreamCfg<double, 1> {
    static constexpr int S = 2, CB = 4;
    static constexpr bool XD = true, N16 = false, ER = false;
};
// two rounds per step: five stages of 9.1 KB (FP32; own x and diagonal
// loaded by the row warps, 16-bit columns), so three rounds are in flight
// while two compute
template <> struct StreamCfg<float, 2> {
    static constexpr int S = 5, CB = 2;
    static constexpr bool XD = false, N16 = true, ER = true;
};
constexpr int kStageCap = kBlock * kMaxW;                              // entries per stage
// stage head: the round's 9 slice bounds (48 B copied) at 0, its 8 slices'
// 16-bit column bases (32 B; -1: 32-bit columns) at 64
constexpr int kStageHead = 128;
template <typename V, int RP>
__host__ __device__ constexpr unsigned stream_xd_bytes()
{
    return StreamCfg<V, RP>::XD ? (unsigned)(2 * kBlock * sizeof(V)) : 0u;
}
template <typename V, int RP>
__host__ __device__ constexpr unsigned stream_stage_bytes()
{
    return (unsigned)(kStageHead + stream_xd_bytes<V, RP>() + kStageCap * (StreamCfg<V, RP>::CB + sizeof(V)));
}
static_assert(stream_stage_bytes<float, 1>() % 16 == 0 && stream_stage_bytes<double, 1>() % 16 == 0 &&
                  stream_stage_bytes<float, 2>() % 16 == 0 && (kStageHead + 2 * kBlock * 4) % 16 == 0 &&
                  (kStageCap * 2) % 16 == 0,
              "every bulk-copy destination in a stage is 16-byte aligned");
template <typename V, int RP>
constexpr size_t stream_smem()
{
    return (size_t)StreamCfg<V, RP>::S * stream_stage_bytes<V, RP>();
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* b)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(b))
                 : "memory");
}
// Bounded wait that also gives up once another warp of the CTA aborted.
__device__ __forceinline__ bool mbar_wait_or_abort(unsigned long long* b, unsigned parity, Ctl* ctl,
                                                   volatile int* abort)
{
    if (mbar_try_wait(b, parity)) return true;
    const long long t0 = clock64();
    for (int it = 1;; ++it) {
        if (mbar_try_wait(b, parity)) return true;
        if ((it & 63) == 0) {
            if (*abort) return false;
            if (clock64() - t0 > wait_budget(ctl)) {
                atomicOr(&ctl->err, ERR_TIMEOUT);
                return false;
            }
        }
    }
}

// The rounds [rb, re) of reduction segment sg.y of a system (FP32: segments
// of rounds; FP64: of whole tiles, the oracle's order).
template <typename V>
__device__ __forceinline__ void stream_rounds(const SysDev& S, int segy, int& rb, int& re, int& u0, int& u1,
                                              unsigned long long& U)
{
    constexpr bool kRoundSeg = sizeof(V) == 4;
    const unsigned T = (unsigned)S.ntiles, G = (unsigned)red_segments(S.ntiles);
    U = kRoundSeg ? 4ull * T : (unsigned long long)T;
    u0 = (int)(((unsigned long long)segy * U) / G);
    u1 = (int)(((unsigned long long)(segy + 1) * U) / G);
    rb = kRoundSeg ? u0 : 4 * u0;
    re = kRoundSeg ? u1 : 4 * u1;
}

template <typename V, int RP>
__global__ void __launch_bounds__(kBlock + 32, kMinCtas) k_spmv_stream(const Batch* __restrict__ pB)
{
    constexpr int S = StreamCfg<V, RP>::S;
    constexpr bool XD = StreamCfg<V, RP>::XD;
    constexpr int CB = StreamCfg<V, RP>::CB;
    constexpr bool N16 = StreamCfg<V, RP>::N16, ER = StreamCfg<V, RP>::ER;
    static_assert(N16 || CB == 4, "32-bit columns need 4 bytes an entry");
    constexpr unsigned VO = (unsigned)(kStageHead + kStageCap * CB);   // coefficients, after the columns
    static_assert(S > RP, "the producer needs a stage beyond the ones a step computes");
    constexpr int NW = kBlock / 32;
    constexpr unsigned SB = stream_stage_bytes<V, RP>();
    constexpr unsigned XB = stream_xd_bytes<V, RP>();
    __shared__ double sh[kBlock * kMaxRed];
    __shared__ int s_last;
    __shared__ volatile int s_abort;
    __shared__ __align__(16) SysDev sS;   // the row warps' system
    __shared__ __align__(16) SysDev sP;   // the producer's system
    __shared__ __align__(8) unsigned long long full[S], empty[S];
    extern __shared__ __align__(128) unsigned char dyn[];
    const Batch B = *pB;   // descriptors (host-written) while the previous kernel drains
    Ctl* ctl = B.ctl;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < S; ++k) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], NW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    __syncthreads();
    pdl_enter();

    if (wid == NW) {
        // ---------------------------------------------------------- producer
        unsigned seq = 0;        // rounds issued by this CTA so far
        int cur = -1, lcur = -1;
        bool live = false;
        for (int g = blockIdx.x; g < B.nsegs && !s_abort; g += gridDim.x) {
            const int2 sg = B.nsys == 1 ? make_int2(0, g) : B.segs[g];
            if (sg.x != lcur) {
                lcur = sg.x;
                if (sg.x != cur) {
                    cur = sg.x;
                    __syncwarp();
                    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(B.sys + cur);
                    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sP);
                    for (int k = lane; k < (int)(sizeof(SysDev) / 8); k += 32) dst[k] = src[k];
                    __syncwarp();
                }
                live = system_live<OP_SPMV_QP>(sP);
            }
            if (!live) continue;
            int rb, re, u0, u1;
            unsigned long long U;
            stream_rounds<V>(sP, sg.y, rb, re, u0, u1, U);
            const int* __restrict__ sptr = sP.a_sptr;
            const int* __restrict__ acol = sP.a_col;
            const V* __restrict__ aval = VP<V>::aval(sP, false);
            const V* __restrict__ dg = VP<V>::diag(sP);
            const V* __restrict__ p = VP<V>::v(sP).p;
            // round starts in the sliced ELL, a window of 32 rounds per
            // load (lane j: round w0 + j), the next window loaded a window
            // ahead
            const int* __restrict__ cbase = sP.a_cbase;
            const uint16_t* __restrict__ acol16 = sP.a_col16;
            auto win = [&](int w0, int& e, int& eend, int& cb) {
                const int a = min(w0 + lane, re), z = min(w0 + 32, re);
                e = __ldg(sptr + 8 * a);
                eend = __ldg(sptr + 8 * z);
                cb = N16 ? __ldg(cbase + 8 * a) : -1;
            };
            int ec, ecend, cbc, en = 0, enend = 0, cbn = 0;
            win(rb, ec, ecend, cbc);
            if (rb + 32 < re) win(rb + 32, en, enend, cbn);
            for (int r = rb; r < re; ++r, ++seq) {
                const int j = (r - rb) & 31;
                if (j == 0 && r > rb) {
                    ec = en;
                    ecend = enend;
                    cbc = cbn;
                    if (r + 32 < re) win(r + 32, en, enend, cbn);
                }
                const int e0 = __shfl_sync(kFull, ec, j);
                const int e1 = j < 31 ? __shfl_sync(kFull, ec, j + 1) : ecend;
                const bool narrow = __shfl_sync(kFull, cbc, j) >= 0;   // 16-bit columns
                const int stg = (int)(seq % S);
                const unsigned ph = (seq / S) & 1u;
                bool ok = true;
                if (seq >= (unsigned)S && lane == 0) ok = mbar_wait_or_abort(&empty[stg], ph ^ 1u, ctl, &s_abort);
                if (!__shfl_sync(kFull, (int)ok, 0)) {
                    if (lane == 0) s_abort = 1;
                    break;
                }
                if (lane == 0) {
                    const unsigned long long pol = l2_evict_first();
                    unsigned char* st = dyn + (size_t)stg * SB;
                    const int cnt = e1 - e0;
                    const bool staged = cnt <= kStageCap && (narrow || CB == 4);
                    const unsigned colb = narrow ? 2u : 4u;
                    const unsigned bytes =
                        (N16 ? 80u : 48u) + XB + (staged ? (unsigned)cnt * (colb + (unsigned)sizeof(V)) : 0u);
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    mbar_expect_tx(&full[stg], bytes);
                    bulk_to_smem(st, sptr + 8 * r, 48u, &full[stg]);
                    if constexpr (N16) bulk_to_smem(st + 64, cbase + 8 * r, 32u, &full[stg]);
                    if constexpr (XD) {
                        bulk_to_smem(st + kStageHead, p + (size_t)kBlock * r, kBlock * (unsigned)sizeof(V),
                                     &full[stg]);
                        bulk_to_smem_stream(st + kStageHead + kBlock * sizeof(V), dg + (size_t)kBlock * r,
                                            kBlock * (unsigned)sizeof(V), &full[stg], pol);
                    }
                    if (staged && cnt > 0) {
                        if (narrow)
                            bulk_to_smem_stream(st + kStageHead + XB, acol16 + e0, (unsigned)cnt * 2u, &full[stg],
                                                pol);
                        else
                            bulk_to_smem_stream(st + kStageHead + XB, acol + e0, (unsigned)cnt * 4u, &full[stg],
                                                pol);
                        bulk_to_smem_stream(st + XB + VO, aval + e0, (unsigned)cnt * (unsigned)sizeof(V), &full[stg],
                                            pol);
                    }
                }
                __syncwarp();
            }
            if (s_abort) break;
        }
        // every copy issued lands before the CTA may exit: wait (bounded)
        // for the last phase issued into each stage
        if (lane == 0) {
            for (int k = 0; k < S && (unsigned)k < seq; ++k) {
                const unsigned last = seq - 1 - (unsigned)((seq - 1 - k) % S);   // last seq issued into stage
                const int stg = (int)(last % S);
                mbar_wait(&full[stg], (last / S) & 1u, ctl);
            }
        }
        return;
    }

    // -------------------------------------------------------------- row warps
    unsigned seq = 0;
    int cur = -1, lcur = -1;
    bool live = false;
    const unsigned long long pol = l2_evict_first();
    for (int g = blockIdx.x; g < B.nsegs; g += gridDim.x) {
        const int2 sg = B.nsys == 1 ? make_int2(0, g) : B.segs[g];
        if (sg.x != lcur) {
            lcur = sg.x;
            if (sg.x != cur) {
                cur = sg.x;
                // the row warps' copy of the system, behind their own barrier
                row_barrier<true>();
                const unsigned long long* src = reinterpret_cast<const unsigned long long*>(B.sys + cur);
                unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sS);
                for (int k = tid; k < (int)(sizeof(SysDev) / 8); k += kBlock) dst[k] = src[k];
                row_barrier<true>();
            }
            live = system_live<OP_SPMV_QP>(sS);
        }
        if (!live) continue;
        int rb, re, u0, u1;
        unsigned long long U;
        stream_rounds<V>(sS, sg.y, rb, re, u0, u1, U);
        const int* __restrict__ acol = sS.a_col;
        const V* __restrict__ aval = VP<V>::aval(sS, false);
        const V* __restrict__ dg = VP<V>::diag(sS);
        const V* __restrict__ p = VP<V>::v(sS).p;
        V* __restrict__ q = VP<V>::v(sS).q;
        double acc[kMaxRed] = {0.0, 0.0};
        // a step takes RP rounds, the segment's last step what is left (an
        // FP32 segment may end on an odd round): the stage sequence advances
        // by the rounds taken, as the producer's does
        for (int r = rb, nr = 0; r < re; r += nr, seq += (unsigned)nr) {
            nr = min(RP, re - r);
            bool ok = true;
            if (lane == 0)
                for (int j = 0; j < nr && ok; ++j)
                    ok = mbar_wait_or_abort(&full[(seq + j) % S], ((seq + j) / S) & 1u, ctl, &s_abort);
            ok = __shfl_sync(kFull, (int)ok, 0) != 0;
            if (!ok) {
                if (lane == 0) s_abort = 1;
                break;
            }
            // every lane observes the completed phases itself (acquire)
            for (int j = 0; j < nr; ++j) mbar_try_wait(&full[(seq + j) % S], ((seq + j) / S) & 1u);
            const unsigned char* stj[RP];
            int ew[RP], W[RP], o[RP], i_[RP], cb[RP];
            bool fast = true;
#pragma unroll
            for (int j = 0; j < RP; ++j) {
                stj[j] = dyn + (size_t)((seq + j) % S) * SB;
                const int* spv = reinterpret_cast<const int*>(stj[j]);
                const bool on = j < nr;
                const int base = on ? spv[0] : 0;
                ew[j] = on ? spv[wid] : 0;
                W[j] = on ? (spv[wid + 1] - ew[j]) >> 5 : 0;
                o[j] = ew[j] - base + lane;
                i_[j] = (NW * (r + j) + wid) * 32 + lane;
                cb[j] = (N16 && on) ? reinterpret_cast<const int*>(stj[j] + 64)[wid] : -1;
                fast = fast && on && spv[NW] - base <= kStageCap && (cb[j] >= 0 || CB == 4) && W[j] <= kMaxW;
            }
            bool released = false;
            // column k of this lane's row in stage j: a 16-bit offset from the
            // slice's base (0xFFFF: padding) or a 32-bit index
            auto col_of = [&](int j, int k) -> int {
                const unsigned char* sc = stj[j] + kStageHead + XB;
                if (N16 && cb[j] >= 0) {
                    const unsigned v = reinterpret_cast<const uint16_t*>(sc)[o[j] + k * 32];
                    return v == 0xFFFFu ? -1 : cb[j] + (int)v;
                }
                return reinterpret_cast<const int*>(sc)[o[j] + k * 32];
            };
            if (fast) {
                // everything the rows need from the stages into registers,
                // the stages released, then the gathers and the arithmetic:
                // the producer refills a stage while its rows' gathers fly
                V xi[RP], dv[RP], xv[RP][kMaxW], av[RP][kMaxW];
                int c[RP][kMaxW];
#pragma unroll
                for (int j = 0; j < RP; ++j) {
                    if constexpr (XD) {
                        xi[j] = reinterpret_cast<const V*>(stj[j] + kStageHead)[wid * 32 + lane];
                        dv[j] = reinterpret_cast<const V*>(stj[j] + kStageHead + kBlock * sizeof(V))[wid * 32 + lane];
                    } else {
                        xi[j] = __ldca(p + i_[j]);
                        dv[j] = ldg_stream(dg + i_[j], pol);
                    }
                    const V* sval = reinterpret_cast<const V*>(stj[j] + XB + VO);
#pragma unroll
                    for (int k = 0; k < kMaxW; ++k) {
                        c[j][k] = k < W[j] ? col_of(j, k) : -1;
                        av[j][k] = k < W[j] ? sval[o[j] + k * 32] : V(0);
                    }
                }
                if constexpr (ER) {
                    __syncwarp();
                    if (lane == 0)
                        for (int j = 0; j < nr; ++j) mbar_arrive(&empty[(seq + j) % S]);
                    released = true;
                }
#pragma unroll
                for (int j = 0; j < RP; ++j)
#pragma unroll
                    for (int k = 0; k < kMaxW; ++k) xv[j][k] = c[j][k] >= 0 ? __ldca(p + c[j][k]) : V(0);
#pragma unroll
                for (int j = 0; j < RP; ++j) {
                    V y = vmul(dv[j], xi[j]);
#pragma unroll
                    for (int k = 0; k < kMaxW; ++k)
                        if (c[j][k] >= 0) y = vfma(av[j][k], xv[j][k], y);
                    q[i_[j]] = y;
                    acc[0] = __fma_rn(widen(y), widen(xi[j]), acc[0]);
                }
            } else {
                for (int j = 0; j < nr; ++j) {
                    const int* spv = reinterpret_cast<const int*>(stj[j]);
                    const bool staged = spv[NW] - spv[0] <= kStageCap && (cb[j] >= 0 || CB == 4);
                    const V* sval = reinterpret_cast<const V*>(stj[j] + XB + VO);
                    V xi, dv;
                    if constexpr (XD) {
                        xi = reinterpret_cast<const V*>(stj[j] + kStageHead)[wid * 32 + lane];
                        dv = reinterpret_cast<const V*>(stj[j] + kStageHead + kBlock * sizeof(V))[wid * 32 + lane];
                    } else {
                        xi = __ldca(p + i_[j]);
                        dv = __ldg(dg + i_[j]);
                    }
                    V y = vmul(dv, xi);
                    if (staged) {
                        // kMaxW entries a round, as ell_round: indices, then
                        // coefficients and gathers, then the FMAs in order
                        for (int k0 = 0; k0 < W[j]; k0 += kMaxW) {
                            int c[kMaxW];
                            V a[kMaxW], xv[kMaxW];
#pragma unroll
                            for (int k = 0; k < kMaxW; ++k) c[k] = k0 + k < W[j] ? col_of(j, k0 + k) : -1;
#pragma unroll
                            for (int k = 0; k < kMaxW; ++k) {
                                a[k] = c[k] >= 0 ? sval[o[j] + (k0 + k) * 32] : V(0);
                                xv[k] = c[k] >= 0 ? __ldca(p + c[k]) : V(0);
                            }
#pragma unroll
                            for (int k = 0; k < kMaxW; ++k)
                                if (c[k] >= 0) y = vfma(a[k], xv[k], y);
                        }
                    } else {
                        for (int k0 = 0; k0 < W[j]; k0 += kMaxW)
                            y = ell_round<V, true>(acol + ew[j] + lane, aval + ew[j] + lane, p, k0, W[j], y);
                    }
                    q[i_[j]] = y;
                    acc[0] = __fma_rn(widen(y), widen(xi), acc[0]);
                }
            }
            if (!released) {
                __syncwarp();   // every lane's reads of the stages are done
                if (lane == 0)
                    for (int j = 0; j < nr; ++j) mbar_arrive(&empty[(seq + j) % S]);
            }
        }
        flush_segment<OP_SPMV_QP, true>(B, sS, sg.y, u1 - u0, acc, sh, &s_last, (int)U);
        if (s_abort) return;   // read after the flush's closing barrier
    }
}

// Amul + (q, p) kernel: default (2) the streamed kernel with one round per
// step in FP32 and the per-warp staged kernel in FP64 (each the faster in
// the solve); MRG_SPMV=warp (0) the per-warp staged kernel; =stream1 (1)
// the streamed kernel with one round per step in FP32 and FP64; =stream2
// (3) the streamed kernel with two rounds per step in FP32.  All give the
// same bits.
static int spmv_mode()
{
    static int mode = -1;
    if (mode < 0) {
        const char* e = std::getenv("MRG_SPMV");
        mode = !e ? 2 : std::strcmp(e, "warp") == 0 ? 0 : std::strcmp(e, "stream1") == 0 ? 1
                                                      : std::strcmp(e, "stream2") == 0 ? 3 : 2;
    }
    return mode;
}

// FP32 levelled sweeps two chunks per warp step (k_sweep_lvl with PAIRS);
// MRG_SWEEP_PAIRS=0 takes one chunk per step.
static bool sweep_pairs()
{
    static int on = -1;
    if (on < 0) {
        const char* e = std::getenv("MRG_SWEEP_PAIRS");
        on = (e && e[0] == '0') ? 0 : 1;
    }
    return on == 1;
}

// Launch with programmatic stream serialisation (pdl_enter in the kernel);
// MRG_PDL=0 launches plainly.
static bool pdl_enabled()
{
    static int on = -1;
    if (on < 0) {
        const char* e = std::getenv("MRG_PDL");
        on = (e && e[0] == '0') ? 0 : 1;
    }
    return on == 1;
}

template <typename... P, typename... A>
static void launch_pdl(void (*k)(P...), int grid, int block, size_t smem, cudaStream_t st, A... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    cudaLaunchKernelEx(&cfg, k, args...);   // errors surface through cudaGetLastError
}

// CTAs of a persistent launch: one wave of kMinCtas CTAs per SM.
static int g_grid_cap = 152 * kMinCtas;

template <typename V, RowOp OP>
void launch_one(const Batch* dB, int ntiles, int nsegs, int pb, cudaStream_t st, int spmv = 0)
{
    // ntiles / nsegs: the host's upper bounds on the batch's table sizes
    // Persistent grid: one wave that walks the tiles / segments, so each CTA
    // pays its prologue (descriptor and system copy) once.
    int grid = OpTraits<OP>::kRed ? nsegs : ntiles;
    grid = grid < g_grid_cap ? grid : g_grid_cap;
    if (grid < 1) grid = 1;
    if constexpr (OP == OP_SPMV_QP) {
        if (!pb) {
            // the batch's tuned choice, else the process default
            const int mode = spmv == 1 ? 0 : spmv == 2 ? 1 : spmv == 3 ? 3 : spmv_mode();
            constexpr bool fp64 = sizeof(V) == 8;
            if (mode == 0 || (fp64 && mode != 1))
                launch_pdl(k_spmv_warp<V>, grid, kBlock, spmv_smem<V>(), st, dB);
            else if (fp64 || mode != 3)
                launch_pdl(k_spmv_stream<V, 1>, grid, kBlock + 32, stream_smem<V, 1>(), st, dB);
            else
                launch_pdl(k_spmv_stream<float, 2>, grid, kBlock + 32, stream_smem<float, 2>(), st, dB);
            return;
        }
    }
    if (pb)
        launch_pdl(k_rows<V, OP, true>, grid, kBlock, 0, st, dB);
    else
        launch_pdl(k_rows<V, OP, false>, grid, kBlock, 0, st, dB);
}

// ---------------------------------------------------------------- factor
// D_row = diag_row - sum_deps (A[row][dep]*A[dep][row]) / D_dep  (DIC: upper^2,
// DILU: upper*lower), then rD = 1/D and the sweep coefficients
// rD_row*A[row][dep] (forward, backward) and rD_row*A[dep][row] (transpose).
__device__ __forceinline__ void factor_row(const SysDev& S, int c, int lane, Ctl* ctl, int with32)
{
    const int r0 = S.chunk_start[c], r1 = S.chunk_start[c + 1];
    const int i = r0 + lane;
    if (i >= r1) return;
    const int F = S.nf;
    double D = S.diag[i];
    const int fe0 = S.f_sptr[c], fW = (S.f_sptr[c + 1] - fe0) >> 5;
    for (int k0 = 0; k0 < fW; k0 += kMaxW) {
        // a round of dependencies: indices, coefficients and looks at their
        // D first, then the updates in order
        int col[kMaxW];
        double a[kMaxW], at[kMaxW], Dd[kMaxW];
#pragma unroll
        for (int k = 0; k < kMaxW; ++k) {
            col[k] = k0 + k < fW ? S.f_col[fe0 + (k0 + k) * 32 + lane] : -1;
            if (col[k] >= 0) {
                const int sc = S.f_src[fe0 + (k0 + k) * 32 + lane];
                a[k] = src_val(S, sc, false);
                at[k] = src_val(S, swap_src(sc, F), false);
                Dd[k] = ld_relaxed(S.D + col[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < kMaxW; ++k)
            if (col[k] >= 0) D = __dsub_rn(D, __ddiv_rn(__dmul_rn(a[k], at[k]), ready(Dd[k], S.D + col[k], ctl)));
    }
    st_relaxed(S.D + i, D);
    const double rd = __ddiv_rn(1.0, D);
    S.rD[i] = rd;
    if (with32) S.rD32[i] = (float)rd;
    // Levelled (colour) plans never store level 0's forward values rD r: the
    // forward sweep reads r there, so the dependency's rD is folded into the
    // coefficient here, once per factorisation, instead of being gathered
    // beside r on every sweep.  Sync-free (foam-order) plans keep foam's
    // coefficients.
    const int lvl0_end = (!S.syncfree && S.nlevels > 1) ? S.chunk_start[S.lvl_chunk[1]] : 0;
    for (int k = 0; k < fW; ++k) {
        const int e = fe0 + k * 32 + lane;
        const int sc = S.f_src[e];
        if (sc < 0) break;
        const double a = src_val(S, sc, false), at = src_val(S, swap_src(sc, F), false);
        double cf = __dmul_rn(rd, a), cfT = __dmul_rn(rd, at);
        const int col = S.f_col[e];
        if (col < lvl0_end) {
            const double rdc = __ddiv_rn(1.0, wait_ready(S.D + col, ctl));
            cf = __dmul_rn(cf, rdc);
            cfT = __dmul_rn(cfT, rdc);
        }
        S.f_c[e] = cf;
        S.f_cT[e] = cfT;
        if (with32) {
            S.f_c32[e] = (float)cf;
            S.f_cT32[e] = (float)cfT;
        }
    }
    const int be0 = S.b_sptr[c], bW = (S.b_sptr[c + 1] - be0) >> 5;
    for (int k = 0; k < bW; ++k) {
        const int e = be0 + k * 32 + lane;
        const int sc = S.b_src[e];
        if (sc < 0) break;
        const double a = src_val(S, sc, false), at = src_val(S, swap_src(sc, F), false);
        const double cb = __dmul_rn(rd, a), cbT = __dmul_rn(rd, at);
        S.b_c[e] = cb;
        S.b_cT[e] = cbT;
        if (with32) {
            S.b_c32[e] = (float)cb;
            S.b_cT32[e] = (float)cbT;
        }
    }
}

__global__ void __launch_bounds__(kBlock, kMinCtas) k_factor(const Batch* __restrict__ pB, int with32)
{
    pdl_enter();
    const Batch B = *pB;
    const SysDev* __restrict__ Ss = B.sys;
    const int nsys = B.nsys;
    Ctl* ctl = B.ctl;
    const int lane = threadIdx.x & 31;
    const unsigned total = (unsigned)nsys * (unsigned)B.maxchunks;
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&ctl->ticket[0], 1u);
        t = __shfl_sync(kFull, t, 0);
        if (t >= total) break;
        const int s = (int)(t % (unsigned)nsys), c = (int)(t / (unsigned)nsys);
        const SysDev& S = Ss[s];
        if (c >= S.nchunks || !scalar_tri(S.pc)) continue;  // warp-uniform
        factor_row(S, c, lane, ctl, with32);
    }
    // Last warp out resets the work counter for the next launch.
    if (lane == 0) {
        const unsigned nw = gridDim.x * (blockDim.x / 32);
        __threadfence();
        if (atomicAdd(&ctl->ticket[1], 1u) == nw - 1u) {
            ctl->ticket[0] = 0u;
            ctl->ticket[1] = 0u;
            __threadfence();
        }
    }
}

// ---------------------------------------------------------------- sweeps
// Forward:  y_i = rD_i r_i - sum_{deps ascending} (rD_i A[i][d]) y_d
// Backward: w_i = y_i     - sum_{deps descending} (rD_i A[i][d]) w_d
// The dependency indices and coefficients of a row are loaded before any
// dependency value is read, so only the dependency values sit on the
// critical path.
//
// Sync-free variant (exact ordering): one launch covers every level; a warp
// claims chunks in topological order from a counter and waits (bounded) for
// each dependency to leave the sentinel state.  The forward sweep re-arms w
// with sentinels for the backward sweep and vice versa.
//
// Level variant (colour ordering): one launch per level, plain loads.  Level
// 0 is never stored (the forward coefficients of its dependants carry its rD,
// so they read r; its own backward pass starts from rD r) and the last level
// writes w directly (it has no backward dependencies), so a two-colour sweep
// is two launches: forward level 1, backward level 0.
// Pointers one sweep needs, copied into registers once per system so the
// stores of the sweep cannot force them to be re-read from the SysDev.
template <typename V>
struct SweepPtrs {
    const int* cstart;
    const int* sptr;
    const int* col;
    const V* coef;
    const V* rD;
    const V* r;
    V* y;
    V* w;
};

// vs (vector set): 0 = r -> y -> w; 1 = rT -> yT -> wT with the transpose
// coefficients (PBiCG's preconditionT); BiCGStab: 2 = wT -> y -> p (M^-1 p),
// 3 = r -> yT -> pT (M^-1 s).
template <typename V, bool FWD>
__device__ __forceinline__ SweepPtrs<V> sweep_ptrs(const SysDev& S, int vs)
{
    const Vecs<V>& v = VP<V>::v(S);
    SweepPtrs<V> P;
    P.cstart = S.chunk_start;
    P.sptr = FWD ? S.f_sptr : S.b_sptr;
    P.col = FWD ? S.f_col : S.b_col;
    P.coef = FWD ? VP<V>::fc(S, vs == 1) : VP<V>::bc(S, vs == 1);
    P.rD = VP<V>::rD(S);
    switch (vs) {
    case 1: P.r = v.rT; P.y = v.yT; P.w = v.wT; break;
    case 2: P.r = v.wT; P.y = v.y; P.w = v.p; break;
    case 3: P.r = v.r; P.y = v.yT; P.w = v.pT; break;
    default: P.r = v.r; P.y = v.y; P.w = v.w; break;
    }
    return P;
}

// Entries k0 .. k0 + kMaxW - 1 (of W) of one sweep row: acc -= coef * dep in
// slot order.  Sync-free sweeps wait (bounded) for each dependency value;
// levelled forward sweeps read r for level-0 dependencies (their rD is in
// the coefficient).
template <typename V, bool FWD>
__device__ __forceinline__ void sweep_round(const SweepPtrs<V>& P, int e0, int k0, int W, int lane, bool syncfree,
                                            Ctl* ctl, int lvl0_end, const V* dep, V& acc)
{
    const V* __restrict__ r = P.r;
    int col[kMaxW];
    V cf[kMaxW];
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) col[k] = k0 + k < W ? __ldg(P.col + e0 + (k0 + k) * 32 + lane) : -1;
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) cf[k] = col[k] >= 0 ? __ldg(P.coef + e0 + (k0 + k) * 32 + lane) : V(0);
    if (syncfree) {
        V d[kMaxW];
#pragma unroll
        for (int k = 0; k < kMaxW; ++k) d[k] = col[k] >= 0 ? ld_relaxed(dep + col[k]) : V(0);
#pragma unroll
        for (int k = 0; k < kMaxW; ++k)
            if (col[k] >= 0) acc = vfma(-cf[k], ready(d[k], dep + col[k], ctl), acc);
    } else {
        V d[kMaxW];
#pragma unroll
        for (int k = 0; k < kMaxW; ++k) {
            const int ck = col[k];
            if (FWD)
                d[k] = ck < 0 ? V(0) : __ldca((ck < lvl0_end ? r : dep) + ck);   // level 0: rD folded into cf
            else
                d[k] = ck < 0 ? V(0) : __ldca(dep + ck);
        }
#pragma unroll
        for (int k = 0; k < kMaxW; ++k)
            if (col[k] >= 0) acc = vfma(-cf[k], d[k], acc);
    }
}

// Row i of a sweep (sweep_rows without the chunk sum); with want_rw, rwi =
// r_i w_i of the w the row writes.
template <typename V, bool FWD>
__device__ __forceinline__ void sweep_row_body(const SweepPtrs<V>& P, int i, int e0, int W, bool syncfree, Ctl* ctl,
                                               int lvl0_end, bool last_level, bool first_level, bool want_rw,
                                               float& rwi)
{
    const int lane = threadIdx.x & 31;
    V* __restrict__ y = P.y;
    V* __restrict__ w = P.w;
    const V* __restrict__ r = P.r;
    const V* __restrict__ rD = P.rD;
    V* dep = FWD ? y : w;
    const bool from_r = FWD || (!syncfree && first_level);
    const V ri = from_r || want_rw ? __ldca(r + i) : V(0);
    V acc;
    if (from_r)
        acc = vmul(__ldg(rD + i), ri);
    else
        acc = __ldca(y + i);
    // rounds of kMaxW entries (one round for most rows, unrolled without a
    // loop): a round's indices and coefficients are loaded before any of its
    // dependency values is read
    const int rounds = W <= kMaxW ? 1 : (W + kMaxW - 1) / kMaxW;
    if (rounds == 1)
        sweep_round<V, FWD>(P, e0, 0, W, lane, syncfree, ctl, lvl0_end, dep, acc);
    else
        for (int k0 = 0; k0 < W; k0 += kMaxW) sweep_round<V, FWD>(P, e0, k0, W, lane, syncfree, ctl, lvl0_end, dep, acc);
    if (syncfree) {
        if (FWD) {
            st_relaxed(y + i, acc);
            w[i] = sent<V>();
        } else {
            st_relaxed(w + i, acc);
            y[i] = sent<V>();
        }
    } else {
        if (FWD && !last_level)
            y[i] = acc;
        else
            w[i] = acc;
    }
    if (want_rw) rwi = (float)vmul(ri, acc);
}

// Rows i = r0 + lane < r1 of one chunk whose sweep entries start at e0 and
// are W wide.  rw (levelled sweeps writing the chunk's w): rw[c] = the
// chunk's sum of r w (FP32 products, warp_sum).
template <typename V, bool FWD>
__device__ __forceinline__ void sweep_rows(const SweepPtrs<V>& P, int r0, int r1, int e0, int W, bool syncfree,
                                           Ctl* ctl, int lvl0_end, bool last_level, bool first_level,
                                           float* rw = nullptr, int c = 0)
{
    const int lane = threadIdx.x & 31;
    const int i = r0 + lane;
    const bool on = i < r1;
    if (!on && rw == nullptr) return;   // with rw the whole warp forms the chunk's sum
    float rwi = 0.f;
    if (on) {
        sweep_row_body<V, FWD>(P, i, e0, W, syncfree, ctl, lvl0_end, last_level, first_level, rw != nullptr, rwi);
    }
    if (rw != nullptr) {
        const float t = warp_sum(rwi);
        if (lane == 0) rw[c] = t;
    }
}

// Levelled FP32 sweeps can take two chunks per warp step (k_sweep_lvl
// with PAIRS); the pair's loads need more registers than kMinCtas CTAs per
// SM leave, so that kernel runs kSweepPairCtas per SM.
constexpr int kSweepPairCtas = 3;

// Two chunks of one level of a levelled sweep, both at most one round wide
// (W <= kMaxW), by one warp: both chunks' own values, indices,
// coefficients and dependency values are loaded before any arithmetic, so
// the two chains of dependent loads (indices, then gathered values) are in
// flight together.  Each row accumulates in the order sweep_rows uses.
template <typename V, bool FWD>
__device__ __forceinline__ void sweep_rows_pair(const SweepPtrs<V>& P, const int (&r0)[2], const int (&r1)[2],
                                                const int (&e0)[2], const int (&W)[2], int lvl0_end,
                                                bool last_level, bool first_level, float* rw, const int (&c)[2])
{
    const int lane = threadIdx.x & 31;
    V* __restrict__ y = P.y;
    V* __restrict__ w = P.w;
    const V* __restrict__ r = P.r;
    const V* __restrict__ rD = P.rD;
    const V* dep = FWD ? y : w;
    const bool from_r = FWD || first_level;
    int i[2];
    bool live[2];
    V a0[2], a1[2];
    int col[2][kMaxW];
    V cf[2][kMaxW], d[2][kMaxW];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        i[h] = r0[h] + lane;
        live[h] = i[h] < r1[h];
        a0[h] = live[h] ? (from_r ? __ldg(rD + i[h]) : __ldca(y + i[h])) : V(0);
        a1[h] = live[h] && (from_r || rw != nullptr) ? __ldca(r + i[h]) : V(0);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int k = 0; k < kMaxW; ++k)
            col[h][k] = live[h] && k < W[h] ? __ldg(P.col + e0[h] + k * 32 + lane) : -1;
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int k = 0; k < kMaxW; ++k) {
            const int ck = col[h][k];
            cf[h][k] = ck >= 0 ? __ldg(P.coef + e0[h] + k * 32 + lane) : V(0);
            if (FWD)
                d[h][k] = ck < 0 ? V(0) : __ldca((ck < lvl0_end ? r : dep) + ck);   // level 0: rD folded into cf
            else
                d[h][k] = ck < 0 ? V(0) : __ldca(dep + ck);
        }
    // an absent entry has cf = d = 0, and fma(-0, 0, acc) is acc bit for bit
    // (signed zeros included), so the indices die once the gathers are issued
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        V acc = from_r ? vmul(a0[h], a1[h]) : a0[h];
#pragma unroll
        for (int k = 0; k < kMaxW; ++k) acc = vfma(-cf[h][k], d[h][k], acc);
        if (live[h]) {
            if (FWD && !last_level)
                y[i[h]] = acc;
            else
                w[i[h]] = acc;
        }
        if (rw != nullptr) {   // as sweep_rows: r_i w_i, warp_sum
            const float t = warp_sum(live[h] ? (float)vmul(a1[h], acc) : 0.f);
            if ((threadIdx.x & 31) == 0) rw[c[h]] = t;
        }
    }
}

template <typename V, bool FWD>
__device__ __forceinline__ void sweep_chunk(const SweepPtrs<V>& P, int c, bool syncfree, Ctl* ctl, int lvl0_end,
                                            bool last_level, bool first_level)
{
    const int r0 = __ldg(P.cstart + c), r1 = __ldg(P.cstart + c + 1);
    const int e0 = __ldg(P.sptr + c), W = (__ldg(P.sptr + c + 1) - e0) >> 5;
    sweep_rows<V, FWD>(P, r0, r1, e0, W, syncfree, ctl, lvl0_end, last_level, first_level);
}

template <typename V, bool FWD>
__device__ __forceinline__ void sweep_sf_phase(const Batch& B, int trans)
{
    const SysDev* __restrict__ Ss = B.sys;
    const int nsys = B.nsys;
    Ctl* ctl = B.ctl;
    const int lane = threadIdx.x & 31;
    // several systems: the batch's list of their chunks by level (the
    // backward sweep reads it from the end); one system: its chunks in order
    const bool list = B.n_sf > 0;
    const unsigned total = list ? (unsigned)B.n_sf : (unsigned)nsys * (unsigned)B.maxchunks;
    const int slot = FWD ? 2 : 4;
    const int unpublished = FWD ? ctl->unpublished1 - 1 : -1;   // watchdog test hook
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&ctl->ticket[slot], 1u);
        t = __shfl_sync(kFull, t, 0);
        if (t >= total) break;
        int s, c;
        if (list) {
            const int2 it = B.sf_items[FWD ? t : total - 1u - t];
            s = it.x;
            c = it.y;
        } else {
            s = (int)(t % (unsigned)nsys);
            c = (int)(t / (unsigned)nsys);
        }
        const SysDev& S = Ss[s];
        const int nch = S.nchunks;
        if (c >= nch || !S.sc->active || !S.syncfree || !scalar_tri(S.pc)) continue;
        const int chunk = list || FWD ? c : nch - 1 - c;
        if (chunk == unpublished) continue;
        const SweepPtrs<V> P = sweep_ptrs<V, FWD>(S, trans);
        sweep_chunk<V, FWD>(P, chunk, true, ctl, 0, false, false);
    }
    if (lane == 0) {
        const unsigned nw = gridDim.x * (blockDim.x / 32);
        __threadfence();
        if (atomicAdd(&ctl->ticket[slot + 1], 1u) == nw - 1u) {
            ctl->ticket[slot] = 0u;
            ctl->ticket[slot + 1] = 0u;
            __threadfence();
        }
    }
}

template <typename V, bool FWD>
__global__ void __launch_bounds__(kBlock, kMinCtas) k_sweep_sf(const Batch* __restrict__ pB, int trans)
{
    pdl_enter();
    const Batch B = *pB;
    sweep_sf_phase<V, FWD>(B, trans);
}

// ------------------------------------------------- owner-computes exact sweeps
// The exact (foam-order) triangular sweep of a batch of one system whose
// plan is cut into parts (ranges of part_cells caller cells, PlanHost):
// each CTA computes one part, level by level, with one barrier between the
// part's levels.  A dependency inside the part is read from the CTA's
// shared-memory copy of the part's values; one in another part is waited
// for (bounded), as in k_sweep_sf, and every value is also published in
// global memory for the other parts and the next kernels.  Parts are
// claimed in sweep order (forward ascending, backward descending) through a
// ticket, and a row depends only on cells before it in sweep order, so a
// CTA waits only on parts that running CTAs hold: no co-residency is
// needed.  Each row's arithmetic, entries and their order are k_sweep_sf's,
// so both give the same bits.  A cross-part wait costs a round trip
// through L2; a level inside a part costs one barrier.
constexpr int kPartBlock = 256;

// One row of an owner-computes sweep, loaded ahead of its level: the start
// value, the first kMaxW entries' columns, coefficients and places in the
// part, and a look at each entry from another part (the sentinel when it is
// not published yet).  None of it depends on the level's predecessors.
template <typename V>
struct PartRow {
    V a0;
    int e, W, slot;   // slot: the row's cell offset in its part
    int col[kMaxW], loc[kMaxW];
    V cf[kMaxW], pre[kMaxW];
};

template <typename V, bool FWD>
__device__ __forceinline__ void part_load(const SweepPtrs<V>& P, const int2* __restrict__ rows,
                                          const int* __restrict__ loc, const int* __restrict__ perm, int base,
                                          const V* dep, int i, PartRow<V>& R)
{
    const int2 ew = __ldg(rows + i);
    R.e = ew.x;
    R.W = ew.y;
    R.slot = __ldg(perm + i) - base;
    R.a0 = FWD ? vmul(__ldg(P.rD + i), __ldca(P.r + i)) : __ldca(P.y + i);
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) R.col[k] = k < ew.y ? __ldg(P.col + ew.x + k * 32) : -1;
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) {
        const bool on = R.col[k] >= 0;
        R.cf[k] = on ? __ldg(P.coef + ew.x + k * 32) : V(0);
        R.loc[k] = on ? __ldg(loc + ew.x + k * 32) : 0;
    }
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) R.pre[k] = (R.col[k] >= 0 && R.loc[k] < 0) ? ld_relaxed(dep + R.col[k]) : V(0);
}

// The row's value: entries in slot order, a dependency in the part from
// shared memory, one outside from its look-ahead when that was published,
// else waited for; entries beyond kMaxW loaded here.
template <typename V>
__device__ __forceinline__ V part_value(const SweepPtrs<V>& P, const int* __restrict__ loc, const V* dep,
                                        const V* own, const PartRow<V>& R, Ctl* ctl)
{
    V acc = R.a0;
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) {
        if (R.col[k] < 0) continue;
        const V v = R.loc[k] >= 0 ? own[R.loc[k]] : (!is_sent(R.pre[k]) ? R.pre[k] : wait_ready(dep + R.col[k], ctl));
        acc = vfma(-R.cf[k], v, acc);
    }
    for (int k = kMaxW; k < R.W; ++k) {
        const int e = R.e + k * 32;
        const int col = __ldg(P.col + e);
        if (col < 0) continue;
        const int l = __ldg(loc + e);
        acc = vfma(-__ldg(P.coef + e), l >= 0 ? own[l] : wait_ready(dep + col, ctl), acc);
    }
    return acc;
}

// The part's rows in sweep order are taken kPartBlock at a time (a window,
// usually several levels): every thread loads its row of the window, and of
// the next window, ahead; the window's levels then run in turn, one barrier
// each, each thread computing its row at its level.
template <typename V, bool FWD>
__global__ void __launch_bounds__(kPartBlock, 1) k_sweep_part(const Batch* __restrict__ pB, int trans)
{
    extern __shared__ __align__(16) unsigned char dyn_part[];
    V* own = reinterpret_cast<V*>(dyn_part);
    __shared__ int s_part;
    pdl_enter();
    const Batch B = *pB;
    Ctl* ctl = B.ctl;
    const SysDev& S = B.sys[0];
    if (threadIdx.x == 0) s_part = (int)atomicAdd(&ctl->ticket[6], 1u);
    __syncthreads();
    const int np = S.nparts;
    if (s_part < np && S.sc->active && S.syncfree && scalar_tri(S.pc)) {
        const int part = FWD ? s_part : np - 1 - s_part;
        const SweepPtrs<V> P = sweep_ptrs<V, FWD>(S, trans);
        const int* __restrict__ loc = FWD ? S.f_loc : S.b_loc;
        const int2* __restrict__ rows = FWD ? S.f_row : S.b_row;
        const int* __restrict__ prow = S.part_rows;
        const int* __restrict__ pstep = S.part_step;
        const int* __restrict__ perm = S.perm;
        const int base = part * S.part_cells;
        const int r0 = __ldg(S.pt_ptr + part), r1 = __ldg(S.pt_ptr + part + 1), nr = r1 - r0;
        V* __restrict__ y = P.y;
        V* __restrict__ w = P.w;
        const V* dep = FWD ? y : w;
        const int tid = (int)threadIdx.x;
        auto at = [&](int j) { return FWD ? r0 + j : r1 - 1 - j; };   // j-th row in sweep order
        // two row buffers by name (a window's rows and the next one's), so
        // they stay in registers
        auto fetch = [&](int j, PartRow<V>& R, int& ri, int& rs) {
            ri = -1;
            if (j < nr) {
                const int q = at(j);
                ri = __ldg(prow + q);
                rs = __ldg(pstep + q);
                part_load<V, FWD>(P, rows, loc, perm, base, dep, ri, R);
            }
        };
        auto window = [&](int w0, const PartRow<V>& R, int ri, int rs) {
            const int sa = __ldg(pstep + at(w0)), sb = __ldg(pstep + at(min(w0 + kPartBlock, nr) - 1));
            for (int st = sa;; st += FWD ? 1 : -1) {
                if (ri >= 0 && rs == st) {
                    const V acc = part_value<V>(P, loc, dep, own, R, ctl);
                    own[R.slot] = acc;
                    if (FWD) {
                        st_relaxed(y + ri, acc);
                        w[ri] = sent<V>();
                    } else {
                        st_relaxed(w + ri, acc);
                        y[ri] = sent<V>();
                    }
                }
                __syncthreads();
                if (st == sb) break;
            }
        };
        PartRow<V> RA, RB;
        int ia, sa, ib, sb;
        fetch(tid, RA, ia, sa);
        for (int w0 = 0; w0 < nr; w0 += 2 * kPartBlock) {
            fetch(w0 + kPartBlock + tid, RB, ib, sb);
            window(w0, RA, ia, sa);
            if (w0 + kPartBlock >= nr) break;
            fetch(w0 + 2 * kPartBlock + tid, RA, ia, sa);
            window(w0 + kPartBlock, RB, ib, sb);
        }
    }
    // the last CTA out resets the ticket for the next launch
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&ctl->ticket[7], 1u) == gridDim.x - 1u) {
            ctl->ticket[6] = 0u;
            ctl->ticket[7] = 0u;
            __threadfence();
        }
    }
}

// One level L of a levelled sweep for every system that has it: forward
// levels 1..nlevels-1, backward levels nlevels-2..0 (level 0 alone when
// nlevels == 1).  Work comes from the batch's per-level list of (system,
// chunk) items, one chunk per warp, warp g taking items g, g + nw, ...
// Lane k of a warp fetches the item and the row / entry bounds of the
// warp's k-th next chunk, so 32 chunks' metadata costs one chain of
// dependent loads instead of one chain per chunk.
template <typename V, bool FWD, bool PAIRS = false>
__device__ __forceinline__ void sweep_lvl_phase(const Batch& B, int L, int trans, int rho_chunks = 0)
{
    if (L >= B.maxlevels) return;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int i0 = B.item_off[L], i1 = B.item_off[L + 1];
    int cur = -1;
    bool ok = false, last = false, first = false;
    int lvl0_end = 0;
    float* rw = nullptr;   // chunk sums of r w: where this launch writes w
    SweepPtrs<V> P;
    for (int base = i0 + gw; base < i1; base += 32 * nw) {
        const int my = base + lane * nw;
        int ms = -1, mc = 0, mr0 = 0, mr1 = 0, me0 = 0, mW = 0;
        if (my < i1) {
            const int2 item = B.items[my];
            ms = item.x;
            mc = item.y;
            const SysDev& S = B.sys[ms];
            const int* __restrict__ cs = S.chunk_start;
            const int* __restrict__ sp = FWD ? S.f_sptr : S.b_sptr;
            mr0 = __ldg(cs + mc);
            mr1 = __ldg(cs + mc + 1);
            me0 = __ldg(sp + mc);
            mW = (__ldg(sp + mc + 1) - me0) >> 5;
        }
        const int cnt = min(32, (i1 - base + nw - 1) / nw);
        for (int j = 0; j < cnt; ++j) {
            const int s = __shfl_sync(kFull, ms, j);
            const int r0 = __shfl_sync(kFull, mr0, j), r1 = __shfl_sync(kFull, mr1, j);
            const int e0 = __shfl_sync(kFull, me0, j), W = __shfl_sync(kFull, mW, j);
            if (s != cur) {
                cur = s;
                const SysDev& S = B.sys[cur];
                const int nl = S.nlevels;
                ok = S.sc->active && scalar_tri(S.pc) && !S.syncfree &&
                     (FWD ? (L >= 1 && L <= nl - 1) : (L <= nl - 2 || (nl == 1 && L == 0)));
                if (ok) {
                    lvl0_end = S.chunk_start[S.lvl_chunk[1 < nl ? 1 : nl]];
                    last = L == nl - 1;
                    first = L == 0;
                    P = sweep_ptrs<V, FWD>(S, trans);
                    rw = rho_chunks && (!FWD || last) ? S.chunk_rw : nullptr;
                }
            }
            if (!ok) continue;
            const int c = __shfl_sync(kFull, mc, j);
            if constexpr (PAIRS) {
                // pair with the warp's next item when it is the same system's
                // and both fit one round
                if (j + 1 < cnt && W <= kMaxW) {
                    const int s2 = __shfl_sync(kFull, ms, j + 1), W2 = __shfl_sync(kFull, mW, j + 1);
                    const int r0b = __shfl_sync(kFull, mr0, j + 1), r1b = __shfl_sync(kFull, mr1, j + 1);
                    const int e0b = __shfl_sync(kFull, me0, j + 1), cb = __shfl_sync(kFull, mc, j + 1);
                    if (s2 == cur && W2 <= kMaxW) {
                        const int pr0[2] = {r0, r0b}, pr1[2] = {r1, r1b}, pe0[2] = {e0, e0b}, pW[2] = {W, W2};
                        const int pc[2] = {c, cb};
                        sweep_rows_pair<V, FWD>(P, pr0, pr1, pe0, pW, lvl0_end, last, first, rw, pc);
                        ++j;
                        continue;
                    }
                }
            }
            sweep_rows<V, FWD>(P, r0, r1, e0, W, false, nullptr, lvl0_end, last, first, rw, c);
        }
    }
}

template <typename V, bool FWD, bool PAIRS>
__global__ void __launch_bounds__(kBlock, PAIRS ? kSweepPairCtas : kMinCtas)
    k_sweep_lvl(const Batch* __restrict__ pB, int L, int trans, int rho_chunks)
{
    const Batch B = *pB;   // host-written: read while the previous kernel drains
    pdl_enter();
    sweep_lvl_phase<V, FWD, PAIRS>(B, L, trans, rho_chunks);
}

// ---------------------------------------------------------------- Gauss-Seidel
// foam's GaussSeidel smoother, one sweep, row i (exact plan, foam order):
//   acc = b_i; acc -= a * x~ for the interface entries (interface order:
//   foam moves them to the source first, with psi at the sweep's start);
//   then the face entries in the row's order -- lower neighbours first (their
//   new values, waited for), upper neighbours after (old values); y_i =
//   acc / diag_i.  The ELL row holds foam's per-cell order, and its source
//   codes tell the three kinds of entry apart (>= 2F interface, >= F this
//   cell is the face's upper cell so the neighbour is its lower one).
// Entries are taken kMaxW at a time: a round's codes, columns and
// coefficients are loaded together, then its values (x loads issued before
// the first wait), then the FMAs in slot order.  Own = nullptr: every lower
// neighbour is waited for in y; else a lower neighbour whose cell lies in
// [base, base + pc) is read from own[cell - base] (owner-computes kernel).
__device__ __forceinline__ double gs_row_acc(const SysDev& S, int i, Ctl* ctl, const double* own, int base, int pc)
{
    const int F = S.nf;
    const int sl = i >> 5, lane = i & 31;
    const int e0 = __ldg(S.a_sptr + sl), W = (__ldg(S.a_sptr + sl + 1) - e0) >> 5;
    const double* __restrict__ x = S.v64.x;
    const double* y = S.v64.y;
    double acc = __ldca(S.v64.b + i);
    if (S.ni > 0) {
        // interface entries first (foam moves them to the source)
        for (int k = 0; k < W; ++k) {
            const int e = e0 + k * 32 + lane;
            const int sc = __ldg(S.a_src + e);
            if (sc >= 2 * F) acc = __fma_rn(-__ldg(S.a_val + e), __ldca(x + __ldg(S.a_col + e)), acc);
        }
    }
    for (int k0 = 0; k0 < W; k0 += kMaxW) {
        int sc[kMaxW], col[kMaxW];
        double a[kMaxW], v[kMaxW];
#pragma unroll
        for (int k = 0; k < kMaxW; ++k) {
            const int e = e0 + (k0 + k) * 32 + lane;
            sc[k] = k0 + k < W ? __ldg(S.a_src + e) : -1;
            if (sc[k] >= 2 * F) sc[k] = -1;   // interface entry: done above
            col[k] = sc[k] >= 0 ? __ldg(S.a_col + e) : 0;
            a[k] = sc[k] >= 0 ? __ldg(S.a_val + e) : 0.0;
        }
        int loc[kMaxW];
#pragma unroll
        for (int k = 0; k < kMaxW; ++k) {
            loc[k] = -1;
            if (own && sc[k] >= F) loc[k] = __ldg(S.perm + col[k]) - base;
            if (sc[k] >= 0 && sc[k] < F)
                v[k] = __ldca(x + col[k]);   // upper neighbours: old values
            else if (sc[k] >= F && (unsigned)loc[k] >= (unsigned)pc)
                v[k] = ld_relaxed(y + col[k]);   // lower neighbours outside the part: a look
            else
                v[k] = 0.0;
        }
#pragma unroll
        for (int k = 0; k < kMaxW; ++k) {
            if (sc[k] < 0) continue;
            if (sc[k] >= F)
                v[k] = (unsigned)loc[k] < (unsigned)pc ? own[loc[k]] : ready(v[k], y + col[k], ctl);
            acc = __fma_rn(-a[k], v[k], acc);
        }
    }
    return __ddiv_rn(acc, __ldg(S.diag + i));
}

__device__ __forceinline__ void gs_row(const SysDev& S, int i, Ctl* ctl)
{
    st_relaxed(S.v64.y + i, gs_row_acc(S, i, ctl, nullptr, 0, 0));
}

__global__ void __launch_bounds__(kBlock, kMinCtas) k_gs_sweep(const Batch* __restrict__ pB)
{
    pdl_enter();
    const Batch B = *pB;
    const SysDev* __restrict__ Ss = B.sys;
    const int nsys = B.nsys;
    Ctl* ctl = B.ctl;
    const int lane = threadIdx.x & 31;
    const unsigned total = (unsigned)nsys * (unsigned)B.maxchunks;
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&ctl->ticket[2], 1u);
        t = __shfl_sync(kFull, t, 0);
        if (t >= total) break;
        const int s = (int)(t % (unsigned)nsys), c = (int)(t / (unsigned)nsys);
        const SysDev& S = Ss[s];
        if (c >= S.nchunks || !S.sc->active || !S.syncfree) continue;   // warp-uniform
        const int r0 = S.chunk_start[c], r1 = S.chunk_start[c + 1];
        if (r0 + lane < r1) gs_row(S, r0 + lane, ctl);
    }
    // last warp out resets the work counter for the next launch
    if (lane == 0) {
        const unsigned nw = gridDim.x * (blockDim.x / 32);
        __threadfence();
        if (atomicAdd(&ctl->ticket[3], 1u) == nw - 1u) {
            ctl->ticket[2] = 0u;
            ctl->ticket[3] = 0u;
            __threadfence();
        }
    }
}

// One Gauss-Seidel sweep of a batch of one system by owner-computes parts
// (k_sweep_part's scheme): each CTA computes its part's rows level by level,
// a lower neighbour inside the part read from shared memory, one in
// another part waited for; upper neighbours and interfaces read x.  Rows as
// gs_row, so both kernels give the same bits.
// A Gauss-Seidel row loaded ahead of its level (rows without interface
// entries and at most kMaxW entries; others are computed by gs_row_acc at
// their level): codes, columns, coefficients, the old x of upper neighbours,
// each lower neighbour's place in the part or a look at its published value.
struct GsRow {
    int slow, slot;   // slot: the row's cell offset in its part
    int sc[kMaxW], col[kMaxW], loc[kMaxW];
    double a[kMaxW], v[kMaxW], b, d;
};

__device__ __forceinline__ void gs_load(const SysDev& S, int i, int base, int pc, GsRow& R)
{
    const int F = S.nf;
    const int sl = i >> 5, lane = i & 31;
    const int e0 = __ldg(S.a_sptr + sl), W = (__ldg(S.a_sptr + sl + 1) - e0) >> 5;
    R.slow = S.ni > 0 || W > kMaxW;
    R.slot = __ldg(S.perm + i) - base;
    if (R.slow) return;
    R.b = __ldca(S.v64.b + i);
    R.d = __ldg(S.diag + i);
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) {
        const int e = e0 + k * 32 + lane;
        R.sc[k] = k < W ? __ldg(S.a_src + e) : -1;
        R.col[k] = R.sc[k] >= 0 ? __ldg(S.a_col + e) : 0;
        R.a[k] = R.sc[k] >= 0 ? __ldg(S.a_val + e) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) {
        R.loc[k] = R.sc[k] >= F ? __ldg(S.perm + R.col[k]) - base : -1;
        if (R.sc[k] >= 0 && R.sc[k] < F)
            R.v[k] = __ldca(S.v64.x + R.col[k]);   // upper neighbour: old value
        else if (R.sc[k] >= F && (unsigned)R.loc[k] >= (unsigned)pc)
            R.v[k] = ld_relaxed(S.v64.y + R.col[k]);   // another part's: a look
        else
            R.v[k] = 0.0;
    }
}

__device__ __forceinline__ double gs_value(const SysDev& S, int i, const GsRow& R, Ctl* ctl, const double* own,
                                           int base, int pc)
{
    if (R.slow) return gs_row_acc(S, i, ctl, own, base, pc);
    const int F = S.nf;
    double acc = R.b;
#pragma unroll
    for (int k = 0; k < kMaxW; ++k) {
        if (R.sc[k] < 0) continue;
        double v = R.v[k];
        if (R.sc[k] >= F)
            v = (unsigned)R.loc[k] < (unsigned)pc ? own[R.loc[k]]
                                                   : (!is_sent(v) ? v : wait_ready(S.v64.y + R.col[k], ctl));
        acc = __fma_rn(-R.a[k], v, acc);
    }
    return __ddiv_rn(acc, R.d);
}

__global__ void __launch_bounds__(kPartBlock, 1) k_gs_part(const Batch* __restrict__ pB)
{
    extern __shared__ __align__(16) unsigned char dyn_part[];
    double* own = reinterpret_cast<double*>(dyn_part);
    __shared__ int s_part;
    pdl_enter();
    const Batch B = *pB;
    Ctl* ctl = B.ctl;
    const SysDev& S = B.sys[0];
    if (threadIdx.x == 0) s_part = (int)atomicAdd(&ctl->ticket[6], 1u);
    __syncthreads();
    if (s_part < S.nparts && S.sc->active && S.syncfree) {
        const int part = s_part, pc = S.part_cells, base = part * pc;
        double* y = S.v64.y;
        const int* __restrict__ prow = S.part_rows;
        const int* __restrict__ pstep = S.part_step;
        const int r0 = __ldg(S.pt_ptr + part), nr = __ldg(S.pt_ptr + part + 1) - r0;
        const int tid = (int)threadIdx.x;
        auto fetch = [&](int j, GsRow& R, int& ri, int& rs) {
            ri = -1;
            if (j < nr) {
                ri = __ldg(prow + r0 + j);
                rs = __ldg(pstep + r0 + j);
                gs_load(S, ri, base, pc, R);
            }
        };
        auto window = [&](int w0, const GsRow& R, int ri, int rs) {
            const int sa = __ldg(pstep + r0 + w0), sb = __ldg(pstep + r0 + min(w0 + kPartBlock, nr) - 1);
            for (int st = sa; st <= sb; ++st) {
                if (ri >= 0 && rs == st) {
                    const double yi = gs_value(S, ri, R, ctl, own, base, pc);
                    own[R.slot] = yi;
                    st_relaxed(y + ri, yi);
                }
                __syncthreads();
            }
        };
        GsRow RA, RB;
        int ia, sa, ib, sb;
        fetch(tid, RA, ia, sa);
        for (int w0 = 0; w0 < nr; w0 += 2 * kPartBlock) {
            fetch(w0 + kPartBlock + tid, RB, ib, sb);
            window(w0, RA, ia, sa);
            if (w0 + kPartBlock >= nr) break;
            fetch(w0 + 2 * kPartBlock + tid, RA, ia, sa);
            window(w0 + kPartBlock, RB, ib, sb);
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&ctl->ticket[7], 1u) == gridDim.x - 1u) {
            ctl->ticket[6] = 0u;
            ctl->ticket[7] = 0u;
            __threadfence();
        }
    }
}

// ------------------------------------------------------ block preconditioner
// The block incomplete factorisation of foam-extend's block Cholesky
// preconditioner (BlockCholeskyPrecon) on bs x bs blocks, restated:
//   factor   cells in order: D_c = A_cc - sum over faces f with upper cell c
//            (ascending) of L_f inv(D_l) U_f, then dD_c = inv(D_c);
//   apply    x_c = dD_c r_c; forward, faces ascending: x_u -= dD_u (L_f x_l);
//            backward, faces descending: x_l -= dD_l (U_f x_u).
// U_f is the block A[l][u], L_f the block A[u][l].  Every product sums its
// terms in index order from the first, one rounding per multiply and add;
// the inverse is Gauss-Jordan elimination without pivoting.  Cells run
// sync-free over the cell plan's chunks (one thread a cell, one warp a
// chunk), each dependency's values waited for (bounded) as in k_sweep_sf.

// Gather: D[c][a][b], U[f][a][b], L[f][b][a] (row-major blocks).
__global__ void k_block_gather(const BlockDev* __restrict__ pb, int n, int nf, int bs,
                               const double* __restrict__ rd, const double* __restrict__ ru,
                               const double* __restrict__ rl)
{
    const BlockDev& K = *pb;
    const long long bb = (long long)bs * bs, nd = (long long)n * bb, tot = nd + (long long)nf * bb;
    const double* lo = rl ? rl : ru;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
         t += (long long)gridDim.x * blockDim.x) {
        if (t < nd) {
            const int code = K.dmap[t];
            const int a = (int)((t % bb) / bs), b = (int)(t % bs);
            K.D[t] = code >= 0 ? rd[code] : (a < b ? ru[-1 - code] : lo[-1 - code]);
        } else {
            const long long e = t - nd, f = e / bb;
            const int a = (int)((e % bb) / bs), b = (int)(e % bs);
            const int k = K.fmap[e];   // scalar face (bs l + a, bs u + b)
            K.U[e] = ru[k];
            K.L[f * bb + b * bs + a] = lo[k];
        }
    }
}

template <int BS>
__device__ __forceinline__ void bmat_mul(const double (&A)[BS][BS], const double (&B)[BS][BS], double (&C)[BS][BS])
{
#pragma unroll
    for (int a = 0; a < BS; ++a)
#pragma unroll
        for (int b = 0; b < BS; ++b) {
            double acc = __dmul_rn(A[a][0], B[0][b]);
#pragma unroll
            for (int k = 1; k < BS; ++k) acc = __dadd_rn(acc, __dmul_rn(A[a][k], B[k][b]));
            C[a][b] = acc;
        }
}

template <int BS>
__device__ __forceinline__ void bmat_vec(const double (&A)[BS][BS], const double (&v)[BS], double (&o)[BS])
{
#pragma unroll
    for (int a = 0; a < BS; ++a) {
        double acc = __dmul_rn(A[a][0], v[0]);
#pragma unroll
        for (int k = 1; k < BS; ++k) acc = __dadd_rn(acc, __dmul_rn(A[a][k], v[k]));
        o[a] = acc;
    }
}

// Gauss-Jordan without pivoting: for each k, row k scaled by 1 / M[k][k],
// then every other row i minus M[i][k] times row k (both halves).
template <int BS>
__device__ __forceinline__ void bmat_inv(double (&M)[BS][BS], double (&I)[BS][BS])
{
#pragma unroll
    for (int a = 0; a < BS; ++a)
#pragma unroll
        for (int b = 0; b < BS; ++b) I[a][b] = a == b ? 1.0 : 0.0;
#pragma unroll
    for (int k = 0; k < BS; ++k) {
        const double p = __ddiv_rn(1.0, M[k][k]);
#pragma unroll
        for (int j = 0; j < BS; ++j) {
            M[k][j] = __dmul_rn(M[k][j], p);
            I[k][j] = __dmul_rn(I[k][j], p);
        }
#pragma unroll
        for (int i = 0; i < BS; ++i) {
            if (i == k) continue;
            const double f = M[i][k];
#pragma unroll
            for (int j = 0; j < BS; ++j) {
                M[i][j] = __dsub_rn(M[i][j], __dmul_rn(f, M[k][j]));
                I[i][j] = __dsub_rn(I[i][j], __dmul_rn(f, I[k][j]));
            }
        }
    }
}

template <int BS>
__device__ __forceinline__ void block_factor_cell(const BlockDev& K, int c, int lane, Ctl* ctl)
{
    const int r0 = __ldg(K.chunk_start + c), r1 = __ldg(K.chunk_start + c + 1);
    const int i = r0 + lane;
    if (i >= r1) return;
    constexpr int BB = BS * BS;
    const int cell = __ldg(K.perm + i);
    double M[BS][BS];
#pragma unroll
    for (int a = 0; a < BS; ++a)
#pragma unroll
        for (int b = 0; b < BS; ++b) M[a][b] = __ldg(K.D + (size_t)cell * BB + a * BS + b);
    const int e0 = __ldg(K.f_sptr + c), W = (__ldg(K.f_sptr + c + 1) - e0) >> 5;
    for (int k = 0; k < W; ++k) {
        const int e = e0 + k * 32 + lane;
        const int l = __ldg(K.f_col + e);
        if (l < 0) continue;
        const int f = __ldg(K.f_src + e) - K.nf;   // A[c][l]: this cell is the face's upper cell
        double Dl[BS][BS], Uf[BS][BS], Lf[BS][BS], T[BS][BS], P[BS][BS];
#pragma unroll
        for (int a = 0; a < BS; ++a)
#pragma unroll
            for (int b = 0; b < BS; ++b) {
                Uf[a][b] = __ldg(K.U + (size_t)f * BB + a * BS + b);
                Lf[a][b] = __ldg(K.L + (size_t)f * BB + a * BS + b);
            }
#pragma unroll
        for (int a = 0; a < BS; ++a)
#pragma unroll
            for (int b = 0; b < BS; ++b) Dl[a][b] = ld_relaxed(K.dD + (size_t)l * BB + a * BS + b);
#pragma unroll
        for (int a = 0; a < BS; ++a)
#pragma unroll
            for (int b = 0; b < BS; ++b) Dl[a][b] = ready(Dl[a][b], K.dD + (size_t)l * BB + a * BS + b, ctl);
        bmat_mul<BS>(Dl, Uf, T);
        bmat_mul<BS>(Lf, T, P);
#pragma unroll
        for (int a = 0; a < BS; ++a)
#pragma unroll
            for (int b = 0; b < BS; ++b) M[a][b] = __dsub_rn(M[a][b], P[a][b]);
    }
    double I[BS][BS];
    bmat_inv<BS>(M, I);
#pragma unroll
    for (int a = 0; a < BS; ++a)
#pragma unroll
        for (int b = 0; b < BS; ++b) st_relaxed(K.dD + (size_t)i * BB + a * BS + b, I[a][b]);
}

template <int BS>
__global__ void __launch_bounds__(kBlock, 1) k_block_factor(const Batch* __restrict__ pB)
{
    pdl_enter();
    const Batch B = *pB;
    Ctl* ctl = B.ctl;
    const int lane = threadIdx.x & 31, nsys = B.nsys;
    const unsigned total = (unsigned)nsys * (unsigned)B.maxchunks;
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&ctl->ticket[0], 1u);
        t = __shfl_sync(kFull, t, 0);
        if (t >= total) break;
        const int s = (int)(t % (unsigned)nsys), c = (int)(t / (unsigned)nsys);
        const SysDev& S = B.sys[s];
        if (S.pc != PC_BLOCK) continue;
        const BlockDev& K = *S.blk;
        if (c >= K.nchunks) continue;   // warp-uniform
        block_factor_cell<BS>(K, c, lane, ctl);
    }
    if (lane == 0) {
        const unsigned nw = gridDim.x * (blockDim.x / 32);
        __threadfence();
        if (atomicAdd(&ctl->ticket[1], 1u) == nw - 1u) {
            ctl->ticket[0] = 0u;
            ctl->ticket[1] = 0u;
            __threadfence();
        }
    }
}

template <int BS, bool FWD>
__device__ __forceinline__ void block_sweep_cell(const BlockDev& K, int c, int lane, const double* r, double* y,
                                                 double* w, Ctl* ctl)
{
    const int r0 = __ldg(K.chunk_start + c), r1 = __ldg(K.chunk_start + c + 1);
    const int i = r0 + lane;
    if (i >= r1) return;
    constexpr int BB = BS * BS;
    double dD[BS][BS], x[BS];
#pragma unroll
    for (int a = 0; a < BS; ++a)
#pragma unroll
        for (int b = 0; b < BS; ++b) dD[a][b] = __ldcg(K.dD + (size_t)i * BB + a * BS + b);
    int vi[BS];
#pragma unroll
    for (int a = 0; a < BS; ++a) vi[a] = __ldg(K.vmap + (size_t)i * BS + a);
    if (FWD) {
        double rc[BS];
#pragma unroll
        for (int a = 0; a < BS; ++a) rc[a] = __ldca(r + vi[a]);
        bmat_vec<BS>(dD, rc, x);
    } else {
#pragma unroll
        for (int a = 0; a < BS; ++a) x[a] = __ldca(y + vi[a]);
    }
    const int* sptr = FWD ? K.f_sptr : K.b_sptr;
    const int* col = FWD ? K.f_col : K.b_col;
    const int* src = FWD ? K.f_src : K.b_src;
    const double* blk = FWD ? K.L : K.U;
    const double* dep = FWD ? y : w;
    const int e0 = __ldg(sptr + c), W = (__ldg(sptr + c + 1) - e0) >> 5;
    for (int k = 0; k < W; ++k) {
        const int e = e0 + k * 32 + lane;
        const int l = __ldg(col + e);
        if (l < 0) continue;
        const int code = __ldg(src + e);
        const int f = FWD ? code - K.nf : code;   // forward: A[c][l] (lower); backward: A[c][u] (upper)
        double Bf[BS][BS], v[BS], t[BS], u[BS];
#pragma unroll
        for (int a = 0; a < BS; ++a)
#pragma unroll
            for (int b = 0; b < BS; ++b) Bf[a][b] = __ldg(blk + (size_t)f * BB + a * BS + b);
        int vl[BS];
#pragma unroll
        for (int a = 0; a < BS; ++a) vl[a] = __ldg(K.vmap + (size_t)l * BS + a);
#pragma unroll
        for (int a = 0; a < BS; ++a) v[a] = ld_relaxed(dep + vl[a]);
#pragma unroll
        for (int a = 0; a < BS; ++a) v[a] = ready(v[a], dep + vl[a], ctl);
        bmat_vec<BS>(Bf, v, t);
        bmat_vec<BS>(dD, t, u);
#pragma unroll
        for (int a = 0; a < BS; ++a) x[a] = __dsub_rn(x[a], u[a]);
    }
#pragma unroll
    for (int a = 0; a < BS; ++a) {
        if (FWD) {
            st_relaxed(y + vi[a], x[a]);
            w[vi[a]] = sent<double>();
        } else {
            st_relaxed(w + vi[a], x[a]);
            y[vi[a]] = sent<double>();
        }
    }
}

template <int BS, bool FWD>
__global__ void __launch_bounds__(kBlock, 1) k_block_sweep(const Batch* __restrict__ pB, int vs)
{
    pdl_enter();
    const Batch B = *pB;
    Ctl* ctl = B.ctl;
    const int lane = threadIdx.x & 31, nsys = B.nsys;
    const unsigned total = (unsigned)nsys * (unsigned)B.maxchunks;
    const int slot = FWD ? 2 : 4;
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&ctl->ticket[slot], 1u);
        t = __shfl_sync(kFull, t, 0);
        if (t >= total) break;
        const int s = (int)(t % (unsigned)nsys), c = (int)(t / (unsigned)nsys);
        const SysDev& S = B.sys[s];
        if (S.pc != PC_BLOCK || !S.sc->active) continue;
        const BlockDev& K = *S.blk;
        if (c >= K.nchunks) continue;   // warp-uniform
        const Vecs<double>& v = S.v64;
        const double* r = vs == 2 ? v.wT : v.r;
        double* y = vs == 3 ? v.yT : v.y;
        double* w = vs == 2 ? v.p : (vs == 3 ? v.pT : v.w);
        block_sweep_cell<BS, FWD>(K, FWD ? c : K.nchunks - 1 - c, lane, r, y, w, ctl);
    }
    if (lane == 0) {
        const unsigned nw = gridDim.x * (blockDim.x / 32);
        __threadfence();
        if (atomicAdd(&ctl->ticket[slot + 1], 1u) == nw - 1u) {
            ctl->ticket[slot] = 0u;
            ctl->ticket[slot + 1] = 0u;
            __threadfence();
        }
    }
}

// ---------------------------------------------------------------- misc
template <typename V>
__global__ void k_fill_sent(V* p, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = sent<V>();
}

template <typename V>
__device__ __forceinline__ void iface_phase(const Batch& B, int which)
{
    const SysDev* __restrict__ Ss = B.sys;
    const int nsys = B.nsys;
    for (int s = 0; s < nsys; ++s) {
        const SysDev& S = Ss[s];
        if (S.ngen == 0) continue;
        if ((which == 0 || which == 2) && !S.sc->active) continue;
        const Vecs<V>& v = VP<V>::v(S);
        V* x = (which == 0 || which == 3) ? v.p : (which == 1 ? v.x : v.pT);
        const V* w = VP<V>::gw(S);
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < S.ngen; j += gridDim.x * blockDim.x) {
            V acc = V(0);
            for (int k = S.g_ptr[j]; k < S.g_ptr[j + 1]; ++k) acc = vfma(w[k], __ldca(x + S.g_src[k]), acc);
            x[S.npad + j] = acc;
        }
    }
}

template <typename V>
__global__ void k_iface_gather(const Batch* __restrict__ pB, int which)
{
    pdl_enter();
    const Batch B = *pB;
    iface_phase<V>(B, which);
}

__global__ void k_permute(const SysDev* __restrict__ Ss, int s, int to_internal, const double* __restrict__ src,
                          double* __restrict__ dst, int n)
{
    const SysDev& S = Ss[s];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = S.perm[i];
        if (to_internal)
            dst[i] = src[c];
        else
            dst[c] = src[i];
    }
}

// GGI weighted gather, one thread per (face, component):
// dst[i*nc + c] = sum_k w_k src[addr_k*nc + c], accumulated from 0 in weight order.
__global__ void k_ggi(int n_dst, const int32_t* __restrict__ ptr, const int32_t* __restrict__ addr,
                      const double* __restrict__ w, const double* __restrict__ src, double* __restrict__ dst,
                      int nc)
{
    const long long tot = (long long)n_dst * nc;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t / nc), c = (int)(t % nc);
        double acc = 0.0;
        for (int k = __ldg(ptr + i); k < __ldg(ptr + i + 1); ++k)
            acc = __fma_rn(__ldg(w + k), __ldg(src + (size_t)__ldg(addr + k) * nc + c), acc);
        dst[t] = acc;
    }
}


// Serving support.
__global__ void k_gather_scal(const Batch* __restrict__ pB, Scal* __restrict__ out)
{
    const int nsys = pB->nsys;
    const SysDev* __restrict__ Ss = pB->sys;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsys; s += gridDim.x * blockDim.x) out[s] = *Ss[s].sc;
}

// n_active / n_oactive of the batch's control block from its members' flags
// (one CTA; counts are small integers, so the order of the sums is free).
__global__ void k_recount(const Batch* __restrict__ pB)
{
    __shared__ unsigned na, no;
    if (threadIdx.x == 0) na = no = 0u;
    __syncthreads();
    const int nsys = pB->nsys;
    unsigned a = 0, o = 0;
    for (int s = threadIdx.x; s < nsys; s += blockDim.x) {
        const Scal* sc = pB->sys[s].sc;
        a += sc->active ? 1u : 0u;
        o += sc->ostate ? 1u : 0u;
    }
    atomicAdd(&na, a);
    atomicAdd(&no, o);
    __syncthreads();
    if (threadIdx.x == 0) {
        pB->ctl->n_active = na;
        pB->ctl->n_oactive = no;
    }
}

// ---------------------------------------------------------------- persistent iteration
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier of a cooperative launch (every CTA is resident).
// Thread 0 of each CTA reads the generation, then arrives on the batch's
// counter; the last to arrive resets the counter and publishes the next
// generation (release), the others wait for it (acquire), so every write
// made before the barrier is visible to every load after it.  The wait is
// bounded: on timeout, or when another wait has already failed, it sets the
// error bit and returns false, and the kernel leaves.
__device__ bool grid_barrier(Ctl* ctl)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = ld_acquire_u32(&ctl->bar_gen);
        __threadfence();
        int ok = 1;
        if (atomicAdd(&ctl->bar_count, 1u) == gridDim.x - 1u) {
            atomicExch(&ctl->bar_count, 0u);
            __threadfence();
            st_release_u32(&ctl->bar_gen, gen + 1u);
        } else {
            const long long t0 = clock64();
            for (int it = 1; ld_acquire_u32(&ctl->bar_gen) == gen; ++it) {
                if (it > 16) __nanosleep(32);
                if ((it & 127) == 0) {
                    if (*(volatile unsigned*)&ctl->err) {
                        ok = 0;
                        break;
                    }
                    if (clock64() - t0 > wait_budget(ctl)) {
                        atomicOr(&ctl->err, ERR_TIMEOUT);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        __threadfence();   // acquire side for the last arriver as well
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// K Krylov iterations of every active member of the batch in one
// cooperative launch: the kernels of record_iteration (precondition, rho,
// p update, interface gather, q = A p, x/r update) run as phases separated
// by grid barriers, with the same per-row arithmetic and the same
// per-system reduction order, so the results are bit-identical to the
// separate launches.  Stops early once no member is active.
template <typename V, bool PB, bool SF, bool RC>
__global__ void __launch_bounds__(kBlock, kMinCtas) k_iterate(const Batch* __restrict__ pB, int K, int pc, int gen)
{
    __shared__ double sh[kBlock * kMaxRed];
    __shared__ int s_last;
    __shared__ __align__(16) SysDev sS;
    const Batch B = *pB;
    Ctl* ctl = B.ctl;
    const int nl = B.maxlevels;
    // RC (FP32 PCG with a levelled DIC): rho from the sweeps' chunk sums, as
    // the separate launches
    static_assert(!RC || (sizeof(V) == 4 && !PB && !SF), "chunk sums belong to FP32 levelled PCG");
    constexpr int rc = RC ? 1 : 0;
    int cur = -1;
    for (int it = 0; it < K; ++it) {
        if (pc >= PC_DIC) {
            for (int tr = 0; tr < (PB ? 2 : 1); ++tr) {
                if constexpr (SF) {
                    sweep_sf_phase<V, true>(B, tr);
                    if (!grid_barrier(ctl)) return;
                    sweep_sf_phase<V, false>(B, tr);
                    if (!grid_barrier(ctl)) return;
                } else {
                    for (int L = 1; L < nl; ++L) {
                        sweep_lvl_phase<V, true>(B, L, tr, rc);
                        if (!grid_barrier(ctl)) return;
                    }
                    for (int L = nl - 2 > 0 ? nl - 2 : 0; L >= 0; --L) {
                        sweep_lvl_phase<V, false>(B, L, tr, rc);
                        if (!grid_barrier(ctl)) return;
                    }
                }
            }
        } else if (pc == PC_DIAG) {
            rows_phase<V, OP_PRECOND_DIAG, PB>(B, sS, sh, &s_last, cur);
            if (!grid_barrier(ctl)) return;
        } else {
            rows_phase<V, OP_PRECOND_NONE, PB>(B, sS, sh, &s_last, cur);
            if (!grid_barrier(ctl)) return;
        }
        if constexpr (RC)
            rows_phase<V, OP_RHO_CH, PB>(B, sS, sh, &s_last, cur);
        else
            rows_phase<V, OP_RHO, PB>(B, sS, sh, &s_last, cur);
        if (!grid_barrier(ctl)) return;
        rows_phase<V, OP_PUPDATE, PB>(B, sS, sh, &s_last, cur);
        if (!grid_barrier(ctl)) return;
        if (gen) {
            iface_phase<V>(B, 0);
            if (PB) iface_phase<V>(B, 2);
            if (!grid_barrier(ctl)) return;
        }
        rows_phase<V, OP_SPMV_QP, PB>(B, sS, sh, &s_last, cur);
        if (!grid_barrier(ctl)) return;
        rows_phase<V, OP_UPDATE, PB>(B, sS, sh, &s_last, cur);
        if (!grid_barrier(ctl)) return;
        if (*(volatile unsigned*)&ctl->n_active == 0u) break;
    }
}
}  // namespace

// ---------------------------------------------------------------- launchers
static std::atomic<unsigned long long> g_launches{0};
unsigned long long launch_count() { return g_launches.load(); }
void set_device_sms(int nsm)
{
    g_grid_cap = (nsm > 0 ? nsm : 152) * kMinCtas;
    // the staged SpMV's stages exceed the default dynamic shared memory
    // limit; set once per device, outside any stream capture
    cudaFuncSetAttribute(k_spmv_warp<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spmv_smem<float>());
    cudaFuncSetAttribute(k_spmv_warp<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spmv_smem<double>());
    cudaFuncSetAttribute(k_spmv_stream<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)stream_smem<float, 1>());
    cudaFuncSetAttribute(k_spmv_stream<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)stream_smem<double, 1>());
    cudaFuncSetAttribute(k_spmv_stream<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)stream_smem<float, 2>());
    const int part_smem = (int)(kPartMaxCells * sizeof(double));
    cudaFuncSetAttribute(k_sweep_part<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, part_smem);
    cudaFuncSetAttribute(k_sweep_part<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, part_smem);
    cudaFuncSetAttribute(k_sweep_part<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, part_smem);
    cudaFuncSetAttribute(k_sweep_part<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, part_smem);
    cudaFuncSetAttribute(k_gs_part, cudaFuncAttributeMaxDynamicSharedMemorySize, part_smem);
}
int persistent_grid() { return g_grid_cap; }
void add_launches(long long d) { g_launches.fetch_add((unsigned long long)d); }

void launch_rows(RowOp op, int precision, const Batch* dB, int ntiles, int nsegs, int pb, cudaStream_t st,
                 int spmv)
{
    if (ntiles <= 0) return;
    ++g_launches;
#define MRG_CASE64(OPX) \
    case OPX: launch_one<double, OPX>(dB, ntiles, nsegs, pb, st); break;
#define MRG_CASE32(OPX) \
    case OPX: launch_one<float, OPX>(dB, ntiles, nsegs, pb, st); break;
    if (precision == 0) {
        switch (op) {
            MRG_CASE64(OP_SCATTER)
            MRG_CASE64(OP_SUMX)
            MRG_CASE64(OP_INIT_RES)
            MRG_CASE64(OP_RHO)
            MRG_CASE64(OP_PUPDATE)
        case OP_SPMV_QP: launch_one<double, OP_SPMV_QP>(dB, ntiles, nsegs, pb, st, spmv); break;
            MRG_CASE64(OP_UPDATE)
            MRG_CASE64(OP_PRECOND_DIAG)
            MRG_CASE64(OP_PRECOND_NONE)
            MRG_CASE64(OP_RESID64)
            MRG_CASE64(OP_TO32)
            MRG_CASE64(OP_CORRECT)
            MRG_CASE64(OP_AMUL)
            MRG_CASE64(OP_TMUL)
            MRG_CASE64(OP_DIAG_RD)
            MRG_CASE64(OP_BEGIN)
            MRG_CASE64(OP_PERMUTE_IN)
            MRG_CASE64(OP_PERMUTE_OUT)
            MRG_CASE64(OP_KEEPBEST)
            MRG_CASE64(OP_FALLBACK64)
            MRG_CASE64(OP_BS_RHO0)
            MRG_CASE64(OP_BS_P)
            MRG_CASE64(OP_BS_V)
            MRG_CASE64(OP_BS_S)
            MRG_CASE64(OP_BS_T)
            MRG_CASE64(OP_BS_XR)
            MRG_CASE64(OP_GS_ARM)
            MRG_CASE64(OP_GS_COPY)
            MRG_CASE64(OP_GS_RES)
            MRG_CASE64(OP_SM_RES)
            MRG_CASE64(OP_SM_ADD)
            MRG_CASE64(OP_GSCALE_DOT)
            MRG_CASE64(OP_GSCALE_SET)
            MRG_CASE64(OP_GSCALE_ADD)
        default: break;
        }
    } else {
        switch (op) {
            MRG_CASE32(OP_RHO)
            MRG_CASE32(OP_PUPDATE)
        case OP_SPMV_QP: launch_one<float, OP_SPMV_QP>(dB, ntiles, nsegs, pb, st, spmv); break;
            MRG_CASE32(OP_UPDATE)
            MRG_CASE32(OP_PRECOND_DIAG)
            MRG_CASE32(OP_PRECOND_NONE)
            MRG_CASE32(OP_BS_RHO0)
            MRG_CASE32(OP_BS_P)
            MRG_CASE32(OP_BS_V)
            MRG_CASE32(OP_BS_S)
            MRG_CASE32(OP_BS_T)
            MRG_CASE32(OP_BS_XR)
            MRG_CASE32(OP_RHO_CH)
        default: break;
        }
    }
#undef MRG_CASE64
#undef MRG_CASE32
}

void launch_fill_sentinel(void* p, long long n, int precision, cudaStream_t st)
{
    if (n <= 0) return;
    ++g_launches;
    int grid = (int)((n + 255) / 256);
    if (grid > 4096) grid = 4096;
    if (precision == 0)
        k_fill_sent<double><<<grid, 256, 0, st>>>((double*)p, n);
    else
        k_fill_sent<float><<<grid, 256, 0, st>>>((float*)p, n);
}

void launch_factor(const Batch* dB, int grid, int with32, cudaStream_t st)
{
    ++g_launches;
    launch_pdl(k_factor, grid, kBlock, 0, st, dB, with32);
}

void launch_sweep(int precision, int fwd, int trans, int syncfree, int level, const Batch* dB, int grid,
                  cudaStream_t st, int rho_chunks, int parts, int part_cells)
{
    ++g_launches;
    if (grid < 1) grid = 1;
    if (syncfree && parts > 0) {
        const size_t smem = (size_t)part_cells * (precision == 0 ? sizeof(double) : sizeof(float));
        if (precision == 0) {
            if (fwd)
                launch_pdl(k_sweep_part<double, true>, parts, kPartBlock, smem, st, dB, trans);
            else
                launch_pdl(k_sweep_part<double, false>, parts, kPartBlock, smem, st, dB, trans);
        } else {
            if (fwd)
                launch_pdl(k_sweep_part<float, true>, parts, kPartBlock, smem, st, dB, trans);
            else
                launch_pdl(k_sweep_part<float, false>, parts, kPartBlock, smem, st, dB, trans);
        }
    } else if (syncfree) {
        if (precision == 0) {
            if (fwd)
                launch_pdl(k_sweep_sf<double, true>, grid, kBlock, 0, st, dB, trans);
            else
                launch_pdl(k_sweep_sf<double, false>, grid, kBlock, 0, st, dB, trans);
        } else {
            if (fwd)
                launch_pdl(k_sweep_sf<float, true>, grid, kBlock, 0, st, dB, trans);
            else
                launch_pdl(k_sweep_sf<float, false>, grid, kBlock, 0, st, dB, trans);
        }
    } else {
        if (precision == 0) {
            if (fwd)
                launch_pdl(k_sweep_lvl<double, true, false>, grid, kBlock, 0, st, dB, level, trans, 0);
            else
                launch_pdl(k_sweep_lvl<double, false, false>, grid, kBlock, 0, st, dB, level, trans, 0);
        } else if (sweep_pairs()) {
            // the grid the caller sized for kMinCtas CTAs per SM, at the
            // paired kernel's occupancy
            const int g = std::max(1, grid / kMinCtas * kSweepPairCtas);
            if (fwd)
                launch_pdl(k_sweep_lvl<float, true, true>, g, kBlock, 0, st, dB, level, trans, rho_chunks);
            else
                launch_pdl(k_sweep_lvl<float, false, true>, g, kBlock, 0, st, dB, level, trans, rho_chunks);
        } else {
            if (fwd)
                launch_pdl(k_sweep_lvl<float, true, false>, grid, kBlock, 0, st, dB, level, trans, rho_chunks);
            else
                launch_pdl(k_sweep_lvl<float, false, false>, grid, kBlock, 0, st, dB, level, trans, rho_chunks);
        }
    }
}

void launch_iface_gather(int precision, int which, const Batch* dB, int grid, cudaStream_t st)
{
    ++g_launches;
    if (precision == 0)
        launch_pdl(k_iface_gather<double>, grid, 256, 0, st, dB, which);
    else
        launch_pdl(k_iface_gather<float>, grid, 256, 0, st, dB, which);
}

void launch_block_gather(const BlockDev* d_blk, int n, int nf, int bs, const double* raw_diag,
                         const double* raw_upper, const double* raw_lower, cudaStream_t st)
{
    ++g_launches;
    const long long tot = ((long long)n + nf) * bs * bs;
    const int grid = (int)std::max<long long>(1, std::min<long long>((tot + 255) / 256, 4096));
    k_block_gather<<<grid, 256, 0, st>>>(d_blk, n, nf, bs, raw_diag, raw_upper, raw_lower);
}

void launch_block_factor(int bs, const Batch* dB, int grid, cudaStream_t st)
{
    ++g_launches;
    switch (bs) {
    case 1: launch_pdl(k_block_factor<1>, grid, kBlock, 0, st, dB); break;
    case 2: launch_pdl(k_block_factor<2>, grid, kBlock, 0, st, dB); break;
    case 3: launch_pdl(k_block_factor<3>, grid, kBlock, 0, st, dB); break;
    default: launch_pdl(k_block_factor<4>, grid, kBlock, 0, st, dB); break;
    }
}

void launch_block_sweep(int bs, int fwd, int vs, const Batch* dB, int grid, cudaStream_t st)
{
    ++g_launches;
#define MRG_BSWEEP(N)                                                       \
    if (fwd)                                                                \
        launch_pdl(k_block_sweep<N, true>, grid, kBlock, 0, st, dB, vs);    \
    else                                                                    \
        launch_pdl(k_block_sweep<N, false>, grid, kBlock, 0, st, dB, vs);
    switch (bs) {
    case 1: MRG_BSWEEP(1) break;
    case 2: MRG_BSWEEP(2) break;
    case 3: MRG_BSWEEP(3) break;
    default: MRG_BSWEEP(4) break;
    }
#undef MRG_BSWEEP
}

void launch_gs_sweep(const Batch* dB, int grid, cudaStream_t st, int parts, int part_cells)
{
    ++g_launches;
    if (parts > 0)
        launch_pdl(k_gs_part, parts, kPartBlock, (size_t)part_cells * sizeof(double), st, dB);
    else
        launch_pdl(k_gs_sweep, grid, kBlock, 0, st, dB);
}

void launch_permute(int to_internal, const SysDev* d, int s, const double* src, double* dst, int n, cudaStream_t st)
{
    ++g_launches;
    int grid = (n + 255) / 256;
    if (grid > 2048) grid = 2048;
    if (grid < 1) grid = 1;
    k_permute<<<grid, 256, 0, st>>>(d, s, to_internal, src, dst, n);
}

template <typename V, bool PB, bool SF, bool RC = false>
static cudaError_t launch_iterate_t(const Batch* dB, int K, int pc, int gen, cudaStream_t st)
{
    static int per_sm = 0;
    auto kern = k_iterate<V, PB, SF, RC>;
    if (!per_sm) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, 0);
        if (e != cudaSuccess || per_sm < 1) per_sm = 1;
        if (per_sm > kMinCtas) per_sm = kMinCtas;
    }
    const int grid = per_sm * (g_grid_cap / kMinCtas);
    void* args[] = {(void*)&dB, (void*)&K, (void*)&pc, (void*)&gen};
    return cudaLaunchCooperativeKernel((void*)kern, dim3(grid), dim3(kBlock), args, 0, st);
}

cudaError_t launch_iterate(int precision, int pb, int syncfree, const Batch* dB, int K, int pc, int gen,
                           cudaStream_t st)
{
    ++g_launches;
    if (precision == 0) {
        if (pb)
            return syncfree ? launch_iterate_t<double, true, true>(dB, K, pc, gen, st)
                            : launch_iterate_t<double, true, false>(dB, K, pc, gen, st);
        return syncfree ? launch_iterate_t<double, false, true>(dB, K, pc, gen, st)
                        : launch_iterate_t<double, false, false>(dB, K, pc, gen, st);
    }
    if (pb)
        return syncfree ? launch_iterate_t<float, true, true>(dB, K, pc, gen, st)
                        : launch_iterate_t<float, true, false>(dB, K, pc, gen, st);
    if (syncfree) return launch_iterate_t<float, false, true>(dB, K, pc, gen, st);
    return pc >= PC_DIC ? launch_iterate_t<float, false, false, true>(dB, K, pc, gen, st)
                        : launch_iterate_t<float, false, false>(dB, K, pc, gen, st);
}

void launch_gather_scal(const Batch* dB, Scal* out, cudaStream_t st)
{
    ++g_launches;
    k_gather_scal<<<8, 128, 0, st>>>(dB, out);
}

void launch_recount(const Batch* dB, cudaStream_t st)
{
    ++g_launches;
    k_recount<<<1, 256, 0, st>>>(dB);
}

void launch_ggi(int n_dst, const int32_t* ptr, const int32_t* addr, const double* w, const double* src, double* dst,
                int ncomp, cudaStream_t st)
{
    long long tot = (long long)n_dst * ncomp;
    if (tot <= 0) return;
    ++g_launches;
    int grid = (int)((tot + 255) / 256);
    if (grid > 4096) grid = 4096;
    k_ggi<<<grid, 256, 0, st>>>(n_dst, ptr, addr, w, src, dst, ncomp);
}

}  // namespace mrg
