// noalloc.cu -- foam-normalised residual that allocates no device memory.
//
// mrg_residual_noalloc returns the same two numbers as mrg_residual --
// lduMatrix::solver::normFactor and gSumMag(b - A x) / normFactor -- but for
// a matrix that lives in the caller's own device arrays, in foam's own LDU
// addressing (lowerAddr, upperAddr, ownerStartAddr, losortAddr,
// losortStartAddr), and it allocates nothing: no cudaMalloc, no cudaFree, no
// library routine that allocates.  It is for callers that cannot allocate
// device memory at the point where they need a residual: code that runs
// inside a host application whose allocator already owns the GPU's memory
// (a caching pool that has reserved most of HBM, or an MPS client under a
// hard memory limit, where a direct cudaMalloc fails or fragments that
// pool), and monitoring code that runs beside asynchronous solves, where
// cudaMalloc / cudaFree would synchronise the whole device and stall them.
//
// Its reduction scratch is the file-scope array g_noalloc_scratch below,
// 393,472 bytes, which every GPU that loads this library holds until the
// process exits.  It bounds the matrix at kNoAllocMaxCells = 16,777,216 cells
// (16,384 tiles of 1,024 cells, one partial pair per tile); larger matrices
// are rejected with MRG_E_INVALID before any work is queued.
//
// Every call shares that array and it keeps the last call's contents: the
// two CTA counters and the error word are cleared at the start of each call
// (every per-tile partial is rewritten before it is read).  Two calls whose
// work overlaps on the GPU -- from two host threads, or on two streams that
// do not wait for each other -- race on the array and both results are then
// undefined.  Every call looks up the array's device address in the current
// context (cudaGetSymbolAddress); the first call on a device also loads this
// library's device code there if it is not loaded yet, so make that first
// call before any stream capture on that device.
//
// The sums run in a fixed order (four rows per thread, a fixed block tree,
// tile partials summed in tile order), so the result does not depend on the
// device or on other work; per row, A x is accumulated as foam's
// lduMatrix::Amul orders it (lduMatrixATmul.C: diagonal, then faces in
// ascending face order -- for an upper-triangular face order the faces of
// losortAddr come before those of ownerStartAddr).  The kernel checks that
// order as it reads the addressing (each cell's losortAddr faces ascending
// with owners below the cell, its ownerStartAddr neighbours above it and
// ascending) and rejects a matrix that breaks it with MRG_E_INVALID.
#include <cuda_runtime.h>

#include <string>

#include "../../include/mrgpu.h"
#include "engine.h"
#include "kernels.h"
#include "noalloc.h"

namespace mrg {
namespace {

constexpr int kNaBlock = 256;
constexpr int kNaRowsPerThread = 4;
constexpr int kNaTileRows = kNaBlock * kNaRowsPerThread;   // 1024
constexpr int kNaMaxTiles = 16384;
constexpr int kNaHeadBytes = 256;

// First 256 bytes of the scratch.
struct NaHead {
    unsigned done[2];      // CTAs finished: pass 1 (sum x), pass 2 (residual)
    unsigned err;          // 1: the addressing points outside its arrays;
                           // 2: faces not in upper-triangular order
    unsigned pad;
    double xsum;           // pass 1 result
    double norm_factor;    // pass 2 results
    double residual;
};
static_assert(sizeof(NaHead) <= kNaHeadBytes, "scratch head");

constexpr size_t kNaScratchBytes = kNaHeadBytes + sizeof(double) * 3 * (size_t)kNaMaxTiles;

// The scratch: head, then the per-tile partials of sum x, of the norm factor
// and of sum |b - A x|, kNaMaxTiles doubles each.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

struct NaArgs {
    int n, nf;
    const int *lower_addr, *upper_addr, *owner_start, *losort, *losort_start;
    const double *diag, *upper, *lower, *b, *x;
};

// Sum of N values over the CTA, in a fixed order; the result is valid in
// thread 0.
template <int N>
__device__ void na_block_sum(double (&v)[N])
{
    __shared__ double sh[N][kNaBlock / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int q = 0; q < N; ++q) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < N; ++q) sh[q][w] = v[q];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < N; ++q) {
            double s = sh[q][0];
            for (int k = 1; k < kNaBlock / 32; ++k) s += sh[q][k];
            v[q] = s;
        }
}

// Store this tile's partials; the CTA that finishes last sums all tiles'
// partials in tile order.  Returns true (in every thread) for that CTA.
template <int N>
__device__ bool na_flush(double (&v)[N], double* part, unsigned* done, int tiles)
{
    __shared__ bool last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < N; ++q) part[(size_t)q * kNaMaxTiles + blockIdx.x] = v[q];
        __threadfence();
        last = atomicAdd(done, 1u) == (unsigned)(tiles - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
#pragma unroll
    for (int q = 0; q < N; ++q) {
        double s = 0.0;
        for (int j = threadIdx.x; j < tiles; j += kNaBlock) s += __ldcg(part + (size_t)q * kNaMaxTiles + j);
        v[q] = s;
    }
    na_block_sum<N>(v);
    return true;
}

__global__ void __launch_bounds__(kNaBlock) k_na_sumx(int n, const double* __restrict__ x, double* part,
                                                       NaHead* head)
{
    const int row0 = blockIdx.x * kNaTileRows;
    double v[1] = {0.0};
#pragma unroll
    for (int k = 0; k < kNaRowsPerThread; ++k) {
        const int i = row0 + k * kNaBlock + threadIdx.x;
        if (i < n) v[0] += x[i];
    }
    na_block_sum<1>(v);
    if (na_flush<1>(v, part, &head->done[0], gridDim.x) && threadIdx.x == 0) head->xsum = v[0];
}

__global__ void __launch_bounds__(kNaBlock) k_na_residual(NaArgs a, double* part, NaHead* head)
{
    const int row0 = blockIdx.x * kNaTileRows;
    const double xbar = __ldcg(&head->xsum) / (double)a.n;
    const unsigned nf = (unsigned)a.nf, n = (unsigned)a.n;
    double v[2] = {0.0, 0.0};   // norm factor, sum |b - A x|
    bool bad = false, disorder = false;
#pragma unroll 1
    for (int k = 0; k < kNaRowsPerThread; ++k) {
        const int i = row0 + k * kNaBlock + threadIdx.x;
        if (i >= a.n) break;
        const double d = a.diag[i];
        double ax = d * a.x[i];
        double sa = d;
        // faces with i as neighbour: A(i, l) = lower
        int s0 = a.losort_start[i], s1 = a.losort_start[i + 1];
        if (s0 < 0 || s1 < s0 || (unsigned)s1 > nf) {
            bad = true;
            s1 = s0;
        }
        int fprev = -1;
        for (int j = s0; j < s1; ++j) {
            const int f = a.losort[j];
            if ((unsigned)f >= nf) { bad = true; continue; }
            const int l = a.lower_addr[f];
            if ((unsigned)l >= n) { bad = true; continue; }
            // foam's order: a cell's neighbour faces ascending, owner below it
            disorder |= (f <= fprev) | (l >= i);
            fprev = f;
            const double c = a.lower[f];
            ax = fma(c, a.x[l], ax);
            sa += c;
        }
        // faces with i as owner: A(i, u) = upper
        int o0 = a.owner_start[i], o1 = a.owner_start[i + 1];
        if (o0 < 0 || o1 < o0 || (unsigned)o1 > nf) {
            bad = true;
            o1 = o0;
        }
        int uprev = i;
        for (int f = o0; f < o1; ++f) {
            const int u = a.upper_addr[f];
            if ((unsigned)u >= n) { bad = true; continue; }
            // upper-triangular order: an owner's neighbours above it, ascending
            disorder |= (u <= i) | (u < uprev);
            uprev = u;
            const double c = a.upper[f];
            ax = fma(c, a.x[u], ax);
            sa += c;
        }
        const double xr = sa * xbar, bi = a.b[i];
        v[0] += fabs(ax - xr) + fabs(bi - xr);
        v[1] += fabs(bi - ax);
    }
    if (bad) atomicOr(&head->err, 1u);
    if (disorder) atomicOr(&head->err, 2u);
    na_block_sum<2>(v);
    if (na_flush<2>(v, part + kNaMaxTiles, &head->done[1], gridDim.x) && threadIdx.x == 0) {
        const double nfac = v[0] + 1e-20;   // lduMatrix::small_
        head->norm_factor = nfac;
        head->residual = v[1] / nfac;
    }
}

// Device address of the scratch in the current context.  In host code
// g_noalloc_scratch names a host-side stand-in, not device memory, so it is
// never dereferenced or passed to a kernel here.  The address is looked up
// on every call (cudaGetSymbolAddress allocates nothing and costs far less
// than the call's own synchronisation): a cached one would be stale after a
// cudaDeviceReset, or wrong when the caller has made another context of the
// same device current.  The first lookup on a device also loads this
// library's device code there.
unsigned char* scratch_in_current_context()
{
    unsigned char* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
        throw Error(MRG_E_CUDA, std::string("mrg_residual_noalloc: cudaGetSymbolAddress of its scratch failed: ") +
                                    cudaGetErrorString(e));
    return ptr;
}

constexpr int kNoAllocMaxCells = kNaMaxTiles * kNaTileRows;

}  // namespace

void residual_noalloc(int n_cells, int n_faces, const int32_t* lower_addr, const int32_t* upper_addr,
                      const int32_t* owner_start, const int32_t* losort, const int32_t* losort_start, const double* diag,
                      const double* upper, const double* lower, const double* b, const double* x, void* stream,
                      double* residual, double* norm_factor)
{
    if (n_cells <= 0 || n_faces < 0)
        throw Error(MRG_E_INVALID, "mrg_residual_noalloc: n_cells must be > 0 and n_faces >= 0");
    if (n_cells > kNoAllocMaxCells)
        throw Error(MRG_E_INVALID, "mrg_residual_noalloc: n_cells = " + std::to_string(n_cells) +
                                       " exceeds its maximum of " + std::to_string(kNoAllocMaxCells) +
                                       " cells (fixed scratch of " + std::to_string(kNaMaxTiles) + " tiles of " +
                                       std::to_string(kNaTileRows) + " cells); use mrg_residual");
    if (!lower_addr || !upper_addr || !owner_start || !losort || !losort_start || !diag || !upper || !b || !x)
        throw Error(MRG_E_INVALID, "mrg_residual_noalloc: NULL array (only the lower coefficients may be NULL)");
    NaArgs a;
    a.n = n_cells;
    a.nf = n_faces;
    a.lower_addr = lower_addr;
    a.upper_addr = upper_addr;
    a.owner_start = owner_start;
    a.losort = losort;
    a.losort_start = losort_start;
    a.diag = diag;
    a.upper = upper;
    a.lower = lower ? lower : upper;
    a.b = b;
    a.x = x;

    unsigned char* base = scratch_in_current_context();
    NaHead* head = reinterpret_cast<NaHead*>(base);
    double* part = reinterpret_cast<double*>(base + kNaHeadBytes);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int tiles = (n_cells + kNaTileRows - 1) / kNaTileRows;

    MRG_CUDA(cudaMemsetAsync(head, 0, sizeof(NaHead), st));
    k_na_sumx<<<tiles, kNaBlock, 0, st>>>(n_cells, x, part, head);
    k_na_residual<<<tiles, kNaBlock, 0, st>>>(a, part, head);
    MRG_CUDA(cudaGetLastError());
    add_launches(2);
    NaHead h;
    MRG_CUDA(cudaMemcpyAsync(&h, head, sizeof h, cudaMemcpyDeviceToHost, st));
    MRG_CUDA(cudaStreamSynchronize(st));
    if (h.err & 1u)
        throw Error(MRG_E_INVALID, "mrg_residual_noalloc: the LDU addressing points outside its arrays");
    if (h.err & 2u)
        throw Error(MRG_E_INVALID, "mrg_residual_noalloc: faces are not in upper-triangular order (lowerAddr < "
                                   "upperAddr, ownerStartAddr neighbours and losortAddr faces ascending)");
    if (residual) *residual = h.residual;
    if (norm_factor) *norm_factor = h.norm_factor;
}

}  // namespace mrg
