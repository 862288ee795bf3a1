// ggi_build.cu -- GGI interface weights built on the device.
//
// The weights foam-extend's GGIInterpolation gives the reference's
// ggiInterfaceToInterfaceMapping (ggiInterfaceToInterfaceMapping.C:62-77:
// rescale = true, SMALL non-overlap tolerance): for every pair of faces of
// the two patches the weight is the area of their intersection divided by
// the receiving face's area, rescaled so that the weights of every covered
// face sum to one; faces that overlap nothing get no weights.  Faces are
// planar convex polygons (2-D vertex lists, counter-clockwise).  For moving
// interfaces the reference rebuilds the weights every
// interpolatorUpdateFrequency steps (regionInterfaceType.C:489-510); here
// the whole construction runs on the device:
//   1. face bounding boxes, the patches' common box and the mean B face size
//   2. B faces binned on a uniform grid of that size (count, scan, fill)
//   3. one thread per A face: candidates from its bins, sorted and
//      de-duplicated, box test, Sutherland-Hodgman clip, intersection area,
//      tolerance test -- counted, scanned, then written in candidate order
//   4. A-from-B weights per A face; the pairs transposed to B rows, each
//      sorted by A face, and B-from-A weights per B face.
// Every floating-point operation is an explicit IEEE one in the order of a
// plain sequential restatement, so the weights do not depend on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/mrgpu.h"
#include "ggi_build.h"
#include "kernels.h"

namespace mrg {
namespace {

constexpr int kMaxFaceV = 32;  // vertices of an input face
constexpr int kMaxV = 64;      // vertices of a clipped polygon (two faces' sum: never truncated)
constexpr int kMaxCand = 256;  // candidate B faces of one A face

struct GridParams {
    double gx0, gy0, cw, ch;
    int gnx, gny, nbins, pad;
};

__device__ double poly_area(const double* p, int nv)
{
    double a = 0.0;
    for (int i = 0; i < nv; ++i) {
        const int j = (i + 1) % nv;
        a = __dadd_rn(a, __dsub_rn(__dmul_rn(p[2 * i], p[2 * j + 1]), __dmul_rn(p[2 * j], p[2 * i + 1])));
    }
    return __dmul_rn(0.5, a);
}

// Clip convex polygon subj (ns vertices) by convex clip (nc vertices);
// result in out (returned count).  buf: 2 * kMaxV doubles of scratch.
__device__ int clip_convex(const double* subj, int ns, const double* clip, int nc, double* out, double* buf)
{
    double* in = out;
    double* res = buf;
    for (int i = 0; i < 2 * ns; ++i) in[i] = subj[i];
    int nin = ns;
    for (int e = 0; e < nc && nin > 0; ++e) {
        const double ax = clip[2 * e], ay = clip[2 * e + 1];
        const double bx = clip[2 * ((e + 1) % nc)], by = clip[2 * ((e + 1) % nc) + 1];
        int nout = 0;
        for (int i = 0; i < nin; ++i) {
            const double px = in[2 * i], py = in[2 * i + 1];
            const double qx = in[2 * ((i + 1) % nin)], qy = in[2 * ((i + 1) % nin) + 1];
            const double sp = __dsub_rn(__dmul_rn(__dsub_rn(bx, ax), __dsub_rn(py, ay)),
                                        __dmul_rn(__dsub_rn(by, ay), __dsub_rn(px, ax)));
            const double sq = __dsub_rn(__dmul_rn(__dsub_rn(bx, ax), __dsub_rn(qy, ay)),
                                        __dmul_rn(__dsub_rn(by, ay), __dsub_rn(qx, ax)));
            const bool pin = sp >= 0.0, qin = sq >= 0.0;
            if (pin && nout < kMaxV) {
                res[2 * nout] = px;
                res[2 * nout + 1] = py;
                ++nout;
            }
            if (pin != qin && nout < kMaxV) {
                const double t = __ddiv_rn(sp, __dsub_rn(sp, sq));
                res[2 * nout] = __dadd_rn(px, __dmul_rn(t, __dsub_rn(qx, px)));
                res[2 * nout + 1] = __dadd_rn(py, __dmul_rn(t, __dsub_rn(qy, py)));
                ++nout;
            }
        }
        double* tmp = in;
        in = res;
        res = tmp;
        nin = nout;
    }
    if (in != out)
        for (int i = 0; i < 2 * nin; ++i) out[i] = in[i];
    return nin;
}

__global__ void k_bbox(int nf, const int32_t* __restrict__ ptr, const double* __restrict__ xy, double* bb)
{
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
        for (int k = ptr[f]; k < ptr[f + 1]; ++k) {
            const double x = xy[2 * k], y = xy[2 * k + 1];
            x0 = fmin(x0, x);
            x1 = fmax(x1, x);
            y0 = fmin(y0, y);
            y1 = fmax(y1, y);
        }
        bb[4 * f] = x0;
        bb[4 * f + 1] = y0;
        bb[4 * f + 2] = x1;
        bb[4 * f + 3] = y1;
    }
}

// The grid: common box of both patches, cells of the mean B face extent.
__global__ void k_grid(int na, const double* __restrict__ bba, int nb, const double* __restrict__ bbb,
                       GridParams* gp)
{
    __shared__ double s0[256], s1[256], s2[256], s3[256], s4[256];
    double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY, mw = 0.0;
    for (int f = threadIdx.x; f < na + nb; f += blockDim.x) {
        const double* b = f < na ? bba + 4 * f : bbb + 4 * (f - na);
        x0 = fmin(x0, b[0]);
        y0 = fmin(y0, b[1]);
        x1 = fmax(x1, b[2]);
        y1 = fmax(y1, b[3]);
        if (f >= na) mw += (b[2] - b[0]) + (b[3] - b[1]);
    }
    const int t = threadIdx.x;
    s0[t] = x0;
    s1[t] = y0;
    s2[t] = x1;
    s3[t] = y1;
    s4[t] = mw;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (t < s) {
            s0[t] = fmin(s0[t], s0[t + s]);
            s1[t] = fmin(s1[t], s1[t + s]);
            s2[t] = fmax(s2[t], s2[t + s]);
            s3[t] = fmax(s3[t], s3[t + s]);
            s4[t] += s4[t + s];
        }
        __syncthreads();
    }
    if (t == 0) {
        double meanw = nb ? s4[0] / (2.0 * nb) : 1.0;
        if (!(meanw > 0.0)) meanw = 1.0;
        int gnx = (int)((s2[0] - s0[0]) / meanw) + 1, gny = (int)((s3[0] - s1[0]) / meanw) + 1;
        if (gnx < 1) gnx = 1;
        if (gny < 1) gny = 1;
        if ((long long)gnx * gny > 16LL * 1024 * 1024) gnx = gny = 4096;
        gp->gx0 = s0[0];
        gp->gy0 = s1[0];
        gp->cw = (s2[0] - s0[0]) / gnx + 1e-300;
        gp->ch = (s3[0] - s1[0]) / gny + 1e-300;
        gp->gnx = gnx;
        gp->gny = gny;
        gp->nbins = gnx * gny;
    }
}

__device__ __forceinline__ void bin_range(const GridParams& g, const double* b, int& ix0, int& ix1, int& iy0,
                                          int& iy1)
{
    ix0 = (int)((b[0] - g.gx0) / g.cw);
    ix1 = (int)((b[2] - g.gx0) / g.cw);
    iy0 = (int)((b[1] - g.gy0) / g.ch);
    iy1 = (int)((b[3] - g.gy0) / g.ch);
    if (ix1 >= g.gnx) ix1 = g.gnx - 1;
    if (iy1 >= g.gny) iy1 = g.gny - 1;
    if (ix0 < 0) ix0 = 0;
    if (iy0 < 0) iy0 = 0;
}

__global__ void k_bin_count(int nb, const double* __restrict__ bbb, const GridParams* __restrict__ gp,
                            int* __restrict__ cnt)
{
    const GridParams g = *gp;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nb; f += gridDim.x * blockDim.x) {
        int ix0, ix1, iy0, iy1;
        bin_range(g, bbb + 4 * f, ix0, ix1, iy0, iy1);
        for (int iy = iy0; iy <= iy1; ++iy)
            for (int ix = ix0; ix <= ix1; ++ix) atomicAdd(&cnt[iy * g.gnx + ix + 1], 1);
    }
}

// In-place inclusive scan of v[0..n) by one CTA (v[0] is the leading zero of
// an exclusive offset array when the caller counts into v[1..n)).
__global__ void k_scan(int* v, int n)
{
    __shared__ int carry;
    __shared__ int sh[1024];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        const int i = base + threadIdx.x;
        int x = i < n ? v[i] : 0;
        sh[threadIdx.x] = x;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const int y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += y;
            __syncthreads();
        }
        if (i < n) v[i] = sh[threadIdx.x] + carry;
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
}

__global__ void k_bin_fill(int nb, const double* __restrict__ bbb, const GridParams* __restrict__ gp,
                           const int* __restrict__ off, int* __restrict__ fill, int* __restrict__ bins)
{
    const GridParams g = *gp;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nb; f += gridDim.x * blockDim.x) {
        int ix0, ix1, iy0, iy1;
        bin_range(g, bbb + 4 * f, ix0, ix1, iy0, iy1);
        for (int iy = iy0; iy <= iy1; ++iy)
            for (int ix = ix0; ix <= ix1; ++ix) {
                const int b = iy * g.gnx + ix;
                bins[off[b] + atomicAdd(&fill[b], 1)] = f;
            }
    }
}

struct Patches {
    int na, nb;
    const int32_t *pa, *pb;
    const double *xa, *xb, *bba, *bbb;
    const GridParams* gp;
    const int *boff, *bins;
    double tol;
};

// Pass 0 counts the overlapping B faces of each A face; pass 1 writes them
// (ascending B face) with their intersection areas at out_off[fa].
__global__ void k_overlaps(Patches P, int pass, int* __restrict__ count, const int* __restrict__ out_off,
                           int* __restrict__ out_b, double* __restrict__ out_area, unsigned* __restrict__ err)
{
    const GridParams g = *P.gp;
    double pa[2 * kMaxFaceV], pb[2 * kMaxFaceV], pc[2 * kMaxV], tmp[2 * kMaxV];
    int cand[kMaxCand];
    for (int fa = blockIdx.x * blockDim.x + threadIdx.x; fa < P.na; fa += gridDim.x * blockDim.x) {
        const int nva = P.pa[fa + 1] - P.pa[fa];
        for (int i = 0; i < 2 * nva; ++i) pa[i] = P.xa[2 * P.pa[fa] + i];
        const double areaA = fabs(poly_area(pa, nva));
        const double* ba = P.bba + 4 * fa;
        int ix0, ix1, iy0, iy1;
        bin_range(g, ba, ix0, ix1, iy0, iy1);
        int nc = 0;
        for (int iy = iy0; iy <= iy1; ++iy)
            for (int ix = ix0; ix <= ix1; ++ix) {
                const int b = iy * g.gnx + ix;
                for (int k = P.boff[b]; k < P.boff[b + 1]; ++k) {
                    const int fb = P.bins[k];
                    const double* bb = P.bbb + 4 * fb;
                    if (bb[0] > ba[2] || bb[2] < ba[0] || bb[1] > ba[3] || bb[3] < ba[1]) continue;
                    if (nc < kMaxCand)
                        cand[nc++] = fb;
                    else
                        atomicOr(err, 1u);
                }
            }
        // ascending, duplicates (a face in several bins) removed
        for (int i = 1; i < nc; ++i) {
            const int v = cand[i];
            int j = i - 1;
            while (j >= 0 && cand[j] > v) {
                cand[j + 1] = cand[j];
                --j;
            }
            cand[j + 1] = v;
        }
        int w = 0;
        for (int i = 0; i < nc; ++i)
            if (i == 0 || cand[i] != cand[i - 1]) cand[w++] = cand[i];
        nc = w;
        int np = 0;
        const int o = pass ? out_off[fa] : 0;
        for (int c = 0; c < nc; ++c) {
            const int fb = cand[c];
            const int nvb = P.pb[fb + 1] - P.pb[fb];
            for (int i = 0; i < 2 * nvb; ++i) pb[i] = P.xb[2 * P.pb[fb] + i];
            const double areaB = fabs(poly_area(pb, nvb));
            const int nvc = clip_convex(pa, nva, pb, nvb, pc, tmp);
            if (nvc < 3) continue;
            const double ov = fabs(poly_area(pc, nvc));
            if (ov <= __dmul_rn(P.tol, fmin(areaA, areaB))) continue;
            if (pass) {
                out_b[o + np] = fb;
                out_area[o + np] = ov;
            }
            ++np;
        }
        if (!pass) count[fa + 1] = np;
    }
}

// Face areas (|signed area|) of one patch.
__global__ void k_face_area(int nf, const int32_t* __restrict__ ptr, const double* __restrict__ xy, double* area)
{
    double p[2 * kMaxFaceV];
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        const int nv = ptr[f + 1] - ptr[f];
        for (int i = 0; i < 2 * nv; ++i) p[i] = xy[2 * ptr[f] + i];
        area[f] = fabs(poly_area(p, nv));
    }
}

// Row r: w_k = area_k / face_area[r], then divided by the row's sum (in
// order) -- covered faces sum to one.
__global__ void k_rescale(int nrows, const int* __restrict__ ptr, const double* __restrict__ area,
                          const double* __restrict__ face_area, double* __restrict__ w)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
            w[k] = __ddiv_rn(area[k], face_area[r]);
            s = __dadd_rn(s, w[k]);
        }
        for (int k = ptr[r]; k < ptr[r + 1]; ++k) w[k] = __ddiv_rn(w[k], s);
    }
}

__global__ void k_transpose_count(int na, const int* __restrict__ aoff, const int* __restrict__ ab,
                                  int* __restrict__ bcnt)
{
    for (int fa = blockIdx.x * blockDim.x + threadIdx.x; fa < na; fa += gridDim.x * blockDim.x)
        for (int k = aoff[fa]; k < aoff[fa + 1]; ++k) atomicAdd(&bcnt[ab[k] + 1], 1);
}

__global__ void k_transpose_fill(int na, const int* __restrict__ aoff, const int* __restrict__ ab,
                                 const double* __restrict__ aarea, const int* __restrict__ boff,
                                 int* __restrict__ bfill, int* __restrict__ ba, double* __restrict__ barea)
{
    for (int fa = blockIdx.x * blockDim.x + threadIdx.x; fa < na; fa += gridDim.x * blockDim.x)
        for (int k = aoff[fa]; k < aoff[fa + 1]; ++k) {
            const int fb = ab[k];
            const int pos = boff[fb] + atomicAdd(&bfill[fb], 1);
            ba[pos] = fa;
            barea[pos] = aarea[k];
        }
}

// Each B row's (A face, area) entries in ascending A face.
__global__ void k_sort_rows(int nrows, const int* __restrict__ ptr, int* __restrict__ key,
                            double* __restrict__ val)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x)
        for (int i = ptr[r] + 1; i < ptr[r + 1]; ++i) {
            const int kv = key[i];
            const double vv = val[i];
            int j = i - 1;
            while (j >= ptr[r] && key[j] > kv) {
                key[j + 1] = key[j];
                val[j + 1] = val[j];
                --j;
            }
            key[j + 1] = kv;
            val[j + 1] = vv;
        }
}

int grid_for(int n) { return std::max(1, std::min((n + 255) / 256, 4096)); }

void check_faces(int nf, const int32_t* ptr, const char* which)
{
    if (nf < 0 || !ptr) throw Error(MRG_E_INVALID, std::string(which) + ": bad face list");
    if (ptr[0] != 0) throw Error(MRG_E_INVALID, std::string(which) + ": face pointer must start at 0");
    for (int f = 0; f < nf; ++f) {
        const int nv = ptr[f + 1] - ptr[f];
        if (nv < 3 || nv > kMaxFaceV)
            throw Error(MRG_E_INVALID, std::string(which) + ": a face needs 3 to 32 vertices");
    }
}

}  // namespace

// One warp per receiving face: the lanes test 32 source faces at a time, in
// face order, and the warp stops at the first group holding a match; the
// smallest matching index is kept (the reference's first match).  Distance
// as foam's mag: sqrt((dx dx + dy dy) + dz dz).
__global__ void k_direct_map(int n_dst, const double* __restrict__ cd, int n_src, const double* __restrict__ cs,
                             double tol, int32_t* __restrict__ map, unsigned* __restrict__ missing)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = warp; i < n_dst; i += nw) {
        const double x = cd[3 * (size_t)i], y = cd[3 * (size_t)i + 1], z = cd[3 * (size_t)i + 2];
        int found = -1;
        for (int j0 = 0; j0 < n_src && found < 0; j0 += 32) {
            const int j = j0 + lane;
            bool hit = false;
            if (j < n_src) {
                const double dx = __dsub_rn(x, cs[3 * (size_t)j]);
                const double dy = __dsub_rn(y, cs[3 * (size_t)j + 1]);
                const double dz = __dsub_rn(z, cs[3 * (size_t)j + 2]);
                const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
                hit = __dsqrt_rn(d2) < tol;
            }
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (m) found = j0 + __ffs((int)m) - 1;
        }
        if (lane == 0) {
            map[i] = found;
            if (found < 0) atomicAdd(missing, 1u);
        }
    }
}

void direct_map_build(Ctx* c, int na, const double* a_centres, int nb, const double* b_centres, double tol,
                      Ggi& a_from_b, Ggi& b_from_a)
{
    if (na <= 0 || nb <= 0 || !a_centres || !b_centres)
        throw Error(MRG_E_INVALID, "directMap: empty patch or NULL face centres");
    if (na != nb)
        throw Error(MRG_E_INVALID, "directMap: interfaces are not conformal (" + std::to_string(na) + " and " +
                                       std::to_string(nb) + " faces); directMap needs conformal interfaces");
    if (!(tol > 0.0)) throw Error(MRG_E_INVALID, "directMap: the match tolerance must be > 0");
    cudaStream_t st = c->st;
    std::vector<void*> tmp;
    auto dalloc = [&](size_t bytes) {
        void* p = c->alloc(bytes);
        tmp.push_back(p);
        return p;
    };
    try {
        double* da = (double*)dalloc(24 * (size_t)na);
        double* db = (double*)dalloc(24 * (size_t)nb);
        unsigned* miss = (unsigned*)dalloc(16);
        MRG_CUDA(cudaMemcpyAsync(da, a_centres, 24 * (size_t)na, cudaMemcpyHostToDevice, st));
        MRG_CUDA(cudaMemcpyAsync(db, b_centres, 24 * (size_t)nb, cudaMemcpyHostToDevice, st));
        for (int dir = 0; dir < 2; ++dir) {
            Ggi& g = dir == 0 ? a_from_b : b_from_a;
            const int nd = dir == 0 ? na : nb, ns = dir == 0 ? nb : na;
            g.ctx = c;
            g.n_dst = nd;
            g.n_src = ns;
            g.ptr = (int32_t*)c->alloc(4 * (size_t)(nd + 1));
            g.addr = (int32_t*)c->alloc(4 * (size_t)nd);
            g.w = (double*)c->alloc(8 * (size_t)nd);
            std::vector<int32_t> ptr(nd + 1);
            for (int i = 0; i <= nd; ++i) ptr[i] = i;
            const std::vector<double> ones(nd, 1.0);
            MRG_CUDA(cudaMemcpyAsync(g.ptr, ptr.data(), 4 * (size_t)(nd + 1), cudaMemcpyHostToDevice, st));
            MRG_CUDA(cudaMemcpyAsync(g.w, ones.data(), 8 * (size_t)nd, cudaMemcpyHostToDevice, st));
            MRG_CUDA(cudaMemsetAsync(miss, 0, 4, st));
            const int grid = std::max(1, std::min((nd + 7) / 8, 4096));
            k_direct_map<<<grid, 256, 0, st>>>(nd, dir == 0 ? da : db, ns, dir == 0 ? db : da, tol, g.addr, miss);
            MRG_CUDA(cudaGetLastError());
            add_launches(1);
            unsigned h = 0;
            MRG_CUDA(cudaMemcpyAsync(&h, miss, 4, cudaMemcpyDeviceToHost, st));
            MRG_CUDA(cudaStreamSynchronize(st));
            if (h)
                throw Error(MRG_E_INVALID, "directMap: interfaces are not conformal: " + std::to_string(h) +
                                               " faces have no partner within the tolerance");
        }
    } catch (...) {
        for (void* p : tmp) c->release(p);
        throw;
    }
    for (void* p : tmp) c->release(p);
}

void ggi_build(Ctx* c, int na, const int32_t* a_ptr, const double* a_xy, int nb, const int32_t* b_ptr,
               const double* b_xy, double tol, Ggi& a_from_b, Ggi& b_from_a)
{
    check_faces(na, a_ptr, "patch A");
    check_faces(nb, b_ptr, "patch B");
    if (na > 0 && !a_xy) throw Error(MRG_E_INVALID, "patch A: NULL vertices");
    if (nb > 0 && !b_xy) throw Error(MRG_E_INVALID, "patch B: NULL vertices");
    cudaStream_t st = c->st;
    std::vector<void*> tmp;
    auto dalloc = [&](size_t bytes) {
        void* p = c->alloc(bytes);
        tmp.push_back(p);
        return p;
    };
    auto upload = [&](const void* h, size_t bytes) {
        void* p = dalloc(std::max<size_t>(bytes, 16));
        if (bytes) MRG_CUDA(cudaMemcpyAsync(p, h, bytes, cudaMemcpyHostToDevice, st));
        return p;
    };
    try {
        auto* dpa = (int32_t*)upload(a_ptr, 4 * (size_t)(na + 1));
        auto* dpb = (int32_t*)upload(b_ptr, 4 * (size_t)(nb + 1));
        auto* dxa = (double*)upload(a_xy, 16 * (size_t)a_ptr[na]);
        auto* dxb = (double*)upload(b_xy, 16 * (size_t)b_ptr[nb]);
        auto* bba = (double*)dalloc(32 * (size_t)std::max(na, 1));
        auto* bbb = (double*)dalloc(32 * (size_t)std::max(nb, 1));
        auto* gp = (GridParams*)dalloc(sizeof(GridParams));
        auto* err = (unsigned*)dalloc(16);
        MRG_CUDA(cudaMemsetAsync(err, 0, 16, st));
        k_bbox<<<grid_for(na), 256, 0, st>>>(na, dpa, dxa, bba);
        k_bbox<<<grid_for(nb), 256, 0, st>>>(nb, dpb, dxb, bbb);
        k_grid<<<1, 256, 0, st>>>(na, bba, nb, bbb, gp);
        GridParams hg;
        MRG_CUDA(cudaMemcpyAsync(&hg, gp, sizeof hg, cudaMemcpyDeviceToHost, st));
        MRG_CUDA(cudaStreamSynchronize(st));
        auto* boff = (int*)dalloc(4 * ((size_t)hg.nbins + 1));
        auto* bfill = (int*)dalloc(4 * (size_t)hg.nbins);
        MRG_CUDA(cudaMemsetAsync(boff, 0, 4 * ((size_t)hg.nbins + 1), st));
        MRG_CUDA(cudaMemsetAsync(bfill, 0, 4 * (size_t)hg.nbins, st));
        k_bin_count<<<grid_for(nb), 256, 0, st>>>(nb, bbb, gp, boff);
        k_scan<<<1, 1024, 0, st>>>(boff, hg.nbins + 1);
        int nbinned = 0;
        MRG_CUDA(cudaMemcpyAsync(&nbinned, boff + hg.nbins, 4, cudaMemcpyDeviceToHost, st));
        MRG_CUDA(cudaStreamSynchronize(st));
        auto* bins = (int*)dalloc(4 * (size_t)std::max(nbinned, 1));
        k_bin_fill<<<grid_for(nb), 256, 0, st>>>(nb, bbb, gp, boff, bfill, bins);
        Patches P{na, nb, dpa, dpb, dxa, dxb, bba, bbb, gp, boff, bins, tol};
        auto* acnt = (int*)dalloc(4 * (size_t)(na + 1));
        MRG_CUDA(cudaMemsetAsync(acnt, 0, 4 * (size_t)(na + 1), st));
        k_overlaps<<<grid_for(na), 128, 0, st>>>(P, 0, acnt, nullptr, nullptr, nullptr, err);
        k_scan<<<1, 1024, 0, st>>>(acnt, na + 1);
        int npairs = 0;
        unsigned herr = 0;
        MRG_CUDA(cudaMemcpyAsync(&npairs, acnt + na, 4, cudaMemcpyDeviceToHost, st));
        MRG_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
        MRG_CUDA(cudaStreamSynchronize(st));
        if (herr) throw Error(MRG_E_INVALID, "a face overlaps more than 256 candidate faces");
        // A-from-B: rows = A faces, ascending B face
        a_from_b.ctx = c;
        a_from_b.n_dst = na;
        a_from_b.n_src = nb;
        tmp.erase(std::find(tmp.begin(), tmp.end(), (void*)acnt));
        a_from_b.ptr = acnt;
        a_from_b.addr = (int32_t*)c->alloc(4 * (size_t)std::max(npairs, 1));
        a_from_b.w = (double*)c->alloc(8 * (size_t)std::max(npairs, 1));
        auto* aarea = (double*)dalloc(8 * (size_t)std::max(npairs, 1));
        k_overlaps<<<grid_for(na), 128, 0, st>>>(P, 1, nullptr, acnt, a_from_b.addr, aarea, err);
        auto* fa_area = (double*)dalloc(8 * (size_t)std::max(na, 1));
        auto* fb_area = (double*)dalloc(8 * (size_t)std::max(nb, 1));
        k_face_area<<<grid_for(na), 128, 0, st>>>(na, dpa, dxa, fa_area);
        k_face_area<<<grid_for(nb), 128, 0, st>>>(nb, dpb, dxb, fb_area);
        k_rescale<<<grid_for(na), 256, 0, st>>>(na, acnt, aarea, fa_area, a_from_b.w);
        // B-from-A: the pairs transposed, each row ascending A face
        b_from_a.ctx = c;
        b_from_a.n_dst = nb;
        b_from_a.n_src = na;
        b_from_a.ptr = (int32_t*)c->alloc(4 * (size_t)(nb + 1));
        b_from_a.addr = (int32_t*)c->alloc(4 * (size_t)std::max(npairs, 1));
        b_from_a.w = (double*)c->alloc(8 * (size_t)std::max(npairs, 1));
        auto* bcnt = (int*)b_from_a.ptr;
        auto* bfil = (int*)dalloc(4 * (size_t)std::max(nb, 1));
        auto* barea = (double*)dalloc(8 * (size_t)std::max(npairs, 1));
        MRG_CUDA(cudaMemsetAsync(bcnt, 0, 4 * (size_t)(nb + 1), st));
        MRG_CUDA(cudaMemsetAsync(bfil, 0, 4 * (size_t)std::max(nb, 1), st));
        k_transpose_count<<<grid_for(na), 256, 0, st>>>(na, acnt, a_from_b.addr, bcnt);
        k_scan<<<1, 1024, 0, st>>>(bcnt, nb + 1);
        k_transpose_fill<<<grid_for(na), 256, 0, st>>>(na, acnt, a_from_b.addr, aarea, bcnt, bfil, b_from_a.addr,
                                                       barea);
        k_sort_rows<<<grid_for(nb), 256, 0, st>>>(nb, bcnt, b_from_a.addr, barea);
        k_rescale<<<grid_for(nb), 256, 0, st>>>(nb, bcnt, barea, fb_area, b_from_a.w);
        MRG_CUDA(cudaGetLastError());
        add_launches(16);
        MRG_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        cudaStreamSynchronize(st);
        for (void* p : tmp) c->release(p);
        throw;
    }
    for (void* p : tmp) c->release(p);
}

}  // namespace mrg
