/*
 * ggi_weights.c -- CPU oracle for GGI face weights (test infrastructure only).
 *
 * Restates the weight definition that foam-extend 4.1's GGIInterpolation
 * uses for the reference's ggiInterfaceToInterfaceMapping
 * (ggiInterfaceToInterfaceMapping.C:62-77: rescale = true, SMALL
 * non-overlap tolerances): for every pair (master face i, slave face j) the
 * weight is the area of the polygon intersection divided by the area of the
 * receiving face; rescaled so the weights of every covered face sum to one;
 * faces with no overlap are "uncovered" and get no weights.
 *
 * The interfaces handled here are planar (the projection onto the master
 * plane is the identity): faces are convex polygons given by their 2-D
 * vertex lists.  Intersections use Sutherland-Hodgman clipping of one convex
 * polygon against the other; candidate pairs come from a uniform bin grid
 * over face bounding boxes.  Parity against foam-extend is unpinned.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>



#define GW_MAXV 64

static double poly_area(const double* p, int nv)
{
    double a = 0.0;
    for (int i = 0; i < nv; ++i) {
        int j = (i + 1) % nv;
        a += p[2 * i] * p[2 * j + 1] - p[2 * j] * p[2 * i + 1];
    }
    return 0.5 * a;
}

/* Clip convex polygon subj (counter-clockwise) by convex clip (ccw). */
static int clip_convex(const double* subj, int ns, const double* clip, int nc,
                       double* out)
{
    double bufA[2 * GW_MAXV], bufB[2 * GW_MAXV];
    double* in = bufA;
    double* res = bufB;
    int nin = ns;
    memcpy(in, subj, sizeof(double) * 2 * (size_t)ns);
    for (int e = 0; e < nc && nin > 0; ++e) {
        double ax = clip[2 * e], ay = clip[2 * e + 1];
        double bx = clip[2 * ((e + 1) % nc)], by = clip[2 * ((e + 1) % nc) + 1];
        int nout = 0;
        for (int i = 0; i < nin; ++i) {
            double px = in[2 * i], py = in[2 * i + 1];
            double qx = in[2 * ((i + 1) % nin)], qy = in[2 * ((i + 1) % nin) + 1];
            double sp = (bx - ax) * (py - ay) - (by - ay) * (px - ax);
            double sq = (bx - ax) * (qy - ay) - (by - ay) * (qx - ax);
            int pin = sp >= 0.0, qin = sq >= 0.0;
            if (pin && nout < GW_MAXV) { res[2 * nout] = px; res[2 * nout + 1] = py; ++nout; }
            if (pin != qin && nout < GW_MAXV) {
                double t = sp / (sp - sq);
                res[2 * nout] = px + t * (qx - px);
                res[2 * nout + 1] = py + t * (qy - py);
                ++nout;
            }
        }
        double* tmp = in; in = res; res = tmp;
        nin = nout;
    }
    if (nin > 0) memcpy(out, in, sizeof(double) * 2 * (size_t)nin);
    return nin;
}

/*
 * Overlap areas between two planar face sets.
 *   A faces: fa_ptr[na+1] into fa_xy (2 doubles per vertex, ccw)
 *   B faces: fb_ptr[nb+1] into fb_xy
 * Output: the list of overlapping pairs (ia, ib, area) with area > tol *
 * min(face areas); returns the pair count, or -1 when cap is too small.
 */
long gw_overlaps(int na, const int32_t* fa_ptr, const double* fa_xy,
                 int nb, const int32_t* fb_ptr, const double* fb_xy,
                 double tol, long cap, int32_t* out_a, int32_t* out_b,
                 double* out_area)
{
    /* Bounding boxes. */
    double* bba = (double*)malloc(sizeof(double) * 4 * (size_t)(na ? na : 1));
    double* bbb = (double*)malloc(sizeof(double) * 4 * (size_t)(nb ? nb : 1));
    double gx0 = INFINITY, gy0 = INFINITY, gx1 = -INFINITY, gy1 = -INFINITY;
    double meanw = 0.0;
    for (int s = 0; s < 2; ++s) {
        int nf = s ? nb : na;
        const int32_t* ptr = s ? fb_ptr : fa_ptr;
        const double* xy = s ? fb_xy : fa_xy;
        double* bb = s ? bbb : bba;
        for (int f = 0; f < nf; ++f) {
            double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
            for (int k = ptr[f]; k < ptr[f + 1]; ++k) {
                double x = xy[2 * k], y = xy[2 * k + 1];
                x0 = fmin(x0, x); x1 = fmax(x1, x);
                y0 = fmin(y0, y); y1 = fmax(y1, y);
            }
            bb[4 * f] = x0; bb[4 * f + 1] = y0; bb[4 * f + 2] = x1; bb[4 * f + 3] = y1;
            gx0 = fmin(gx0, x0); gy0 = fmin(gy0, y0);
            gx1 = fmax(gx1, x1); gy1 = fmax(gy1, y1);
            if (s) meanw += (x1 - x0) + (y1 - y0);
        }
    }
    meanw = nb ? meanw / (2.0 * nb) : 1.0;
    if (!(meanw > 0.0)) meanw = 1.0;
    int gnx = (int)((gx1 - gx0) / meanw) + 1, gny = (int)((gy1 - gy0) / meanw) + 1;
    if (gnx < 1) gnx = 1;
    if (gny < 1) gny = 1;
    if ((long)gnx * gny > 16L * 1024 * 1024) { gnx = gny = 4096; }
    double cw = (gx1 - gx0) / gnx + 1e-300, ch = (gy1 - gy0) / gny + 1e-300;
    /* Bin B faces by bbox (CSR of bins). */
    int nbins = gnx * gny;
    int32_t* cnt = (int32_t*)calloc((size_t)nbins + 1, sizeof(int32_t));
    for (int f = 0; f < nb; ++f) {
        int ix0 = (int)((bbb[4 * f] - gx0) / cw), ix1 = (int)((bbb[4 * f + 2] - gx0) / cw);
        int iy0 = (int)((bbb[4 * f + 1] - gy0) / ch), iy1 = (int)((bbb[4 * f + 3] - gy0) / ch);
        if (ix1 >= gnx) ix1 = gnx - 1;
        if (iy1 >= gny) iy1 = gny - 1;
        for (int iy = iy0; iy <= iy1; ++iy)
            for (int ix = ix0; ix <= ix1; ++ix) cnt[iy * gnx + ix + 1]++;
    }
    for (int i = 0; i < nbins; ++i) cnt[i + 1] += cnt[i];
    int32_t* bins = (int32_t*)malloc(sizeof(int32_t) * ((size_t)(uint32_t)cnt[nbins] + 1));
    int32_t* fill = (int32_t*)malloc(sizeof(int32_t) * (size_t)nbins);
    memcpy(fill, cnt, sizeof(int32_t) * (size_t)nbins);
    for (int f = 0; f < nb; ++f) {
        int ix0 = (int)((bbb[4 * f] - gx0) / cw), ix1 = (int)((bbb[4 * f + 2] - gx0) / cw);
        int iy0 = (int)((bbb[4 * f + 1] - gy0) / ch), iy1 = (int)((bbb[4 * f + 3] - gy0) / ch);
        if (ix1 >= gnx) ix1 = gnx - 1;
        if (iy1 >= gny) iy1 = gny - 1;
        for (int iy = iy0; iy <= iy1; ++iy)
            for (int ix = ix0; ix <= ix1; ++ix) bins[fill[iy * gnx + ix]++] = f;
    }
    free(fill);

    int32_t* seen = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nb ? nb : 1));
    for (int f = 0; f < nb; ++f) seen[f] = -1;
    long npairs = 0;
    double pa[2 * GW_MAXV], pb[2 * GW_MAXV], pc[2 * GW_MAXV];
    for (int fa = 0; fa < na; ++fa) {
        int nva = fa_ptr[fa + 1] - fa_ptr[fa];
        memcpy(pa, fa_xy + 2 * (size_t)fa_ptr[fa], sizeof(double) * 2 * (size_t)nva);
        double areaA = fabs(poly_area(pa, nva));
        int ix0 = (int)((bba[4 * fa] - gx0) / cw), ix1 = (int)((bba[4 * fa + 2] - gx0) / cw);
        int iy0 = (int)((bba[4 * fa + 1] - gy0) / ch), iy1 = (int)((bba[4 * fa + 3] - gy0) / ch);
        if (ix1 >= gnx) ix1 = gnx - 1;
        if (iy1 >= gny) iy1 = gny - 1;
        /* Collect candidates, sorted ascending so output order is canonical. */
        int ncand = 0;
        int32_t cand[1024];
        for (int iy = iy0; iy <= iy1; ++iy)
            for (int ix = ix0; ix <= ix1; ++ix)
                for (int k = cnt[iy * gnx + ix]; k < cnt[iy * gnx + ix + 1]; ++k) {
                    int fb = bins[k];
                    if (seen[fb] == fa) continue;
                    seen[fb] = fa;
                    if (bbb[4 * fb] > bba[4 * fa + 2] || bbb[4 * fb + 2] < bba[4 * fa] ||
                        bbb[4 * fb + 1] > bba[4 * fa + 3] || bbb[4 * fb + 3] < bba[4 * fa + 1])
                        continue;
                    if (ncand < 1024) cand[ncand++] = fb;
                }
        for (int i = 1; i < ncand; ++i) {
            int32_t v = cand[i];
            int j = i - 1;
            while (j >= 0 && cand[j] > v) { cand[j + 1] = cand[j]; --j; }
            cand[j + 1] = v;
        }
        for (int c = 0; c < ncand; ++c) {
            int fb = cand[c];
            int nvb = fb_ptr[fb + 1] - fb_ptr[fb];
            memcpy(pb, fb_xy + 2 * (size_t)fb_ptr[fb], sizeof(double) * 2 * (size_t)nvb);
            double areaB = fabs(poly_area(pb, nvb));
            int nvc = clip_convex(pa, nva, pb, nvb, pc);
            if (nvc < 3) continue;
            double ov = fabs(poly_area(pc, nvc));
            if (ov <= tol * fmin(areaA, areaB)) continue;
            if (npairs >= cap) { npairs = -1; goto done; }
            out_a[npairs] = fa;
            out_b[npairs] = fb;
            out_area[npairs] = ov;
            ++npairs;
        }
    }
done:
    free(seen); free(bins); free(cnt); free(bba); free(bbb);
    return npairs;
}

/* Signed area of each face (ccw positive). */
void gw_face_areas(int nf, const int32_t* ptr, const double* xy, double* area)
{
    for (int f = 0; f < nf; ++f)
        area[f] = poly_area(xy + 2 * (size_t)ptr[f], ptr[f + 1] - ptr[f]);
}
