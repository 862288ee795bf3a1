// plan.cpp -- see plan.h.  O(n + F) host work per (mesh, ordering); done
// once when a mesh is uploaded, never per solve.
#include "plan.h"

#include <algorithm>
#include <cstdio>

namespace mrg {

std::string validate_addressing(int n, int nf, const int32_t* lower,
                                const int32_t* upper, const IfaceHost& ifc)
{
    char buf[256];
    if (n <= 0) return "n_cells must be positive";
    if (nf < 0) return "n_faces must be non-negative";
    if (nf > 0 && (!lower || !upper)) return "lower/upper addressing is NULL";
    for (int f = 0; f < nf; ++f) {
        int l = lower[f], u = upper[f];
        if (l < 0 || u < 0 || l >= n || u >= n) {
            snprintf(buf, sizeof buf, "face %d addresses cell out of range (%d,%d), n=%d", f, l, u, n);
            return buf;
        }
        if (l >= u) {
            snprintf(buf, sizeof buf, "face %d: lowerAddr %d must be < upperAddr %d", f, l, u);
            return buf;
        }
        if (f > 0) {
            int pl = lower[f - 1], pu = upper[f - 1];
            if (l < pl || (l == pl && u <= pu)) {
                snprintf(buf, sizeof buf,
                         "faces not in upper-triangular order at face %d ((%d,%d) after (%d,%d))",
                         f, l, u, pl, pu);
                return buf;
            }
        }
    }
    int ni = ifc.size();
    if ((int)ifc.ptr.size() != ni + 1) return "interface CSR has wrong length";
    for (int i = 0; i < ni; ++i) {
        if (ifc.cells[i] < 0 || ifc.cells[i] >= n) {
            snprintf(buf, sizeof buf, "interface face %d: faceCell %d out of range", i, ifc.cells[i]);
            return buf;
        }
        if (ifc.ptr[i + 1] < ifc.ptr[i]) return "interface CSR pointer decreases";
    }
    if (ni && ifc.ptr[0] != 0) return "interface CSR must start at 0";
    for (size_t k = 0; k < ifc.src.size(); ++k)
        if (ifc.src[k] < 0 || ifc.src[k] >= n) {
            snprintf(buf, sizeof buf, "interface source cell %d out of range", ifc.src[k]);
            return buf;
        }
    return "";
}

namespace {

// Row lists in foam face order: for cell c, faces with upperAddr==c
// (ascending), then faces with lowerAddr==c (ascending).
struct Rows {
    std::vector<int32_t> start, face;  // CSR
    std::vector<int32_t> nlow;         // # of faces with upperAddr==c (first part)
};

Rows build_rows(int n, int nf, const int32_t* lower, const int32_t* upper)
{
    Rows R;
    R.start.assign(n + 1, 0);
    R.nlow.assign(n, 0);
    for (int f = 0; f < nf; ++f) {
        R.start[lower[f] + 1]++;
        R.start[upper[f] + 1]++;
        R.nlow[upper[f]]++;
    }
    for (int c = 0; c < n; ++c) R.start[c + 1] += R.start[c];
    R.face.resize((size_t)2 * nf);
    std::vector<int32_t> lowfill(n), upfill(n);
    for (int c = 0; c < n; ++c) {
        lowfill[c] = R.start[c];
        upfill[c] = R.start[c] + R.nlow[c];
    }
    for (int f = 0; f < nf; ++f) {
        R.face[lowfill[upper[f]]++] = f;  // c = upper: neighbour-side face
        R.face[upfill[lower[f]]++] = f;   // c = lower: owner-side face
    }
    return R;
}

}  // namespace

PlanHost build_plan(int n, int nf, const int32_t* lower, const int32_t* upper,
                    const IfaceHost& ifc, int ordering)
{
    PlanHost P;
    P.n = n;
    P.nf = nf;
    P.ni = ifc.size();
    P.ordering = ordering;
    P.npad = ((n + kTileRows - 1) / kTileRows) * kTileRows;
    Rows R = build_rows(n, nf, lower, upper);
    auto other = [&](int c, int f) { return lower[f] == c ? upper[f] : lower[f]; };

    // ---- ordering ------------------------------------------------------
    std::vector<int32_t> key(n, 0);  // level (exact) or colour
    if (ordering == 0) {
        for (int c = 0; c < n; ++c) {
            int lv = 0;
            for (int k = R.start[c]; k < R.start[c] + R.nlow[c]; ++k)
                lv = std::max(lv, key[lower[R.face[k]]] + 1);
            key[c] = lv;
        }
    } else {
        std::vector<int32_t> mark;
        for (int c = 0; c < n; ++c) {
            int deg = R.start[c + 1] - R.start[c];
            if ((int)mark.size() < deg + 2) mark.resize(deg + 2);
            std::fill(mark.begin(), mark.begin() + deg + 2, 0);
            for (int k = R.start[c]; k < R.start[c + 1]; ++k) {
                int o = other(c, R.face[k]);
                if (o < c && key[o] <= deg + 1) mark[key[o]] = 1;
            }
            int col = 0;
            while (mark[col]) ++col;
            key[c] = col;
        }
    }
    int nkey = 0;
    for (int c = 0; c < n; ++c) nkey = std::max(nkey, key[c] + 1);
    {
        std::vector<int32_t> cnt(nkey + 1, 0);
        for (int c = 0; c < n; ++c) cnt[key[c] + 1]++;
        for (int k = 0; k < nkey; ++k) cnt[k + 1] += cnt[k];
        P.perm.resize(n);
        for (int c = 0; c < n; ++c) P.perm[cnt[key[c]]++] = c;  // stable
    }
    P.iperm.resize(n);
    for (int i = 0; i < n; ++i) P.iperm[P.perm[i]] = i;

    // ---- sweep levels in the internal order ----------------------------
    // Forward deps of internal row i: neighbours with smaller internal index.
    P.level_of_row.assign(n, 0);
    if (ordering == 0) {
        for (int i = 0; i < n; ++i) P.level_of_row[i] = key[P.perm[i]];
    } else {
        // Colour classes are independent sets: every dependency has a smaller
        // colour, so each colour is one level.
        for (int i = 0; i < n; ++i) P.level_of_row[i] = key[P.perm[i]];
    }
    P.nlevels = nkey;

    // ---- chunks: <= 32 consecutive rows of one level -------------------
    P.chunk_start.clear();
    P.lvl_chunk.assign(P.nlevels + 1, 0);
    {
        int i = 0;
        for (int lv = 0; lv < P.nlevels; ++lv) {
            P.lvl_chunk[lv] = (int)P.chunk_start.size();
            while (i < n && P.level_of_row[i] == lv) {
                P.chunk_start.push_back(i);
                int e = i;
                while (e < n && e - i < kSlice && P.level_of_row[e] == lv) ++e;
                i = e;
            }
        }
        P.lvl_chunk[P.nlevels] = (int)P.chunk_start.size();
        P.nchunks = (int)P.chunk_start.size();
        P.chunk_start.push_back(n);
    }

    // ---- interface bookkeeping -----------------------------------------
    int ni = P.ni;
    std::vector<int32_t> ic_start(n + 1, 0), ic_list(ni);
    for (int j = 0; j < ni; ++j) ic_start[ifc.cells[j] + 1]++;
    for (int c = 0; c < n; ++c) ic_start[c + 1] += ic_start[c];
    {
        std::vector<int32_t> fill(ic_start.begin(), ic_start.end() - 1);
        for (int j = 0; j < ni; ++j) ic_list[fill[ifc.cells[j]]++] = j;
    }
    std::vector<int32_t> gen_index(ni, -1);
    P.g_ptr.assign(1, 0);
    for (int j = 0; j < ni; ++j) {
        int k0 = ifc.ptr[j], k1 = ifc.ptr[j + 1];
        bool conformal = (k1 - k0 == 1) && ifc.w[k0] == 1.0;
        if (!conformal) {
            gen_index[j] = P.ngen++;
            for (int k = k0; k < k1; ++k) {
                P.g_src.push_back(P.iperm[ifc.src[k]]);
                P.g_w.push_back(ifc.w[k]);
            }
            P.g_ptr.push_back((int32_t)P.g_src.size());
        }
    }

    // ---- Amul sliced ELL ------------------------------------------------
    int nsl = P.npad / kSlice;
    P.a_sptr.assign(nsl + 1, 0);
    auto row_len = [&](int i) {
        if (i >= n) return 0;
        int c = P.perm[i];
        return (R.start[c + 1] - R.start[c]) + (ic_start[c + 1] - ic_start[c]);
    };
    for (int s = 0; s < nsl; ++s) {
        int w = 0;
        for (int r = 0; r < kSlice; ++r) w = std::max(w, row_len(s * kSlice + r));
        P.max_row_len = std::max(P.max_row_len, w);
        P.a_sptr[s + 1] = P.a_sptr[s] + w * kSlice;
    }
    P.a_col.assign(P.a_sptr[nsl], -1);
    P.a_src.assign(P.a_sptr[nsl], -1);
    for (int i = 0; i < n; ++i) {
        int s = i / kSlice, lane = i % kSlice, c = P.perm[i];
        int k = 0;
        for (int q = R.start[c]; q < R.start[c + 1]; ++q, ++k) {
            int f = R.face[q];
            size_t e = (size_t)P.a_sptr[s] + (size_t)k * kSlice + lane;
            P.a_col[e] = P.iperm[other(c, f)];
            P.a_src[e] = (upper[f] == c) ? nf + f : f;
        }
        for (int q = ic_start[c]; q < ic_start[c + 1]; ++q, ++k) {
            int j = ic_list[q];
            size_t e = (size_t)P.a_sptr[s] + (size_t)k * kSlice + lane;
            P.a_col[e] = gen_index[j] < 0 ? P.iperm[ifc.src[ifc.ptr[j]]] : P.npad + gen_index[j];
            P.a_src[e] = 2 * nf + j;
        }
    }

    // ---- 16-bit column offsets, per round of 8 slices -------------------
    P.a_col16.assign(P.a_sptr[nsl], (uint16_t)0xFFFF);
    P.a_cbase.assign(nsl, -1);
    for (int r = 0; r < nsl / 8; ++r) {
        int lo[8], hi[8];
        bool ok = true;
        for (int q = 0; q < 8; ++q) {
            const int sl = 8 * r + q;
            lo[q] = INT32_MAX;
            hi[q] = -1;
            for (int32_t e = P.a_sptr[sl]; e < P.a_sptr[sl + 1]; ++e) {
                const int c = P.a_col[e];
                if (c < 0) continue;
                lo[q] = std::min(lo[q], c);
                hi[q] = std::max(hi[q], c);
            }
            if (hi[q] >= 0 && (int64_t)hi[q] - lo[q] > 65534) ok = false;
        }
        if (!ok) continue;
        for (int q = 0; q < 8; ++q) {
            const int sl = 8 * r + q;
            const int base = hi[q] >= 0 ? lo[q] : 0;
            P.a_cbase[sl] = base;
            for (int32_t e = P.a_sptr[sl]; e < P.a_sptr[sl + 1]; ++e)
                if (P.a_col[e] >= 0) P.a_col16[e] = (uint16_t)(P.a_col[e] - base);
        }
    }

    // ---- sweep dependencies (per chunk sliced ELL) ---------------------
    auto build_sweep = [&](bool fwd, std::vector<int32_t>& sptr, std::vector<int32_t>& col,
                           std::vector<int32_t>& src) {
        sptr.assign(P.nchunks + 1, 0);
        std::vector<std::vector<int32_t>> tmpc, tmps;  // reused per row
        auto deps = [&](int i, std::vector<int32_t>& fc) {
            fc.clear();
            int c = P.perm[i];
            for (int q = R.start[c]; q < R.start[c + 1]; ++q) {
                int f = R.face[q];
                int oi = P.iperm[other(c, f)];
                if (fwd ? (oi < i) : (oi > i)) fc.push_back(f);
            }
            // R lists faces ascending; backward sweeps walk faces descending.
            if (!fwd) std::reverse(fc.begin(), fc.end());
        };
        std::vector<int32_t> fc;
        for (int ch = 0; ch < P.nchunks; ++ch) {
            int w = 0;
            for (int i = P.chunk_start[ch]; i < P.chunk_start[ch + 1]; ++i) {
                deps(i, fc);
                w = std::max(w, (int)fc.size());
            }
            sptr[ch + 1] = sptr[ch] + w * kSlice;
        }
        col.assign(sptr[P.nchunks], -1);
        src.assign(sptr[P.nchunks], -1);
        for (int ch = 0; ch < P.nchunks; ++ch) {
            for (int i = P.chunk_start[ch]; i < P.chunk_start[ch + 1]; ++i) {
                deps(i, fc);
                int c = P.perm[i], lane = i - P.chunk_start[ch];
                for (size_t k = 0; k < fc.size(); ++k) {
                    int f = fc[k];
                    size_t e = (size_t)sptr[ch] + k * kSlice + lane;
                    col[e] = P.iperm[other(c, f)];
                    src[e] = (upper[f] == c) ? nf + f : f;  // A[row][dep]
                }
            }
        }
    };
    build_sweep(true, P.f_sptr, P.f_col, P.f_src);
    build_sweep(false, P.b_sptr, P.b_col, P.b_src);
    return P;
}

void build_parts(PlanHost& P, int nparts)
{
    const int n = P.n;
    P.nparts = nparts;
    P.part_cells = (n + nparts - 1) / nparts;
    const int B = P.part_cells;
    // segments: runs of rows with one (level, part); rows of a level are in
    // cell order, so each run is a part's whole level
    std::vector<std::vector<std::pair<int, int>>> segs(nparts);
    for (int i = 0; i < n;) {
        const int lv = P.level_of_row[i], pt = P.perm[i] / B;
        int e = i + 1;
        while (e < n && P.level_of_row[e] == lv && P.perm[e] / B == pt) ++e;
        segs[pt].push_back({i, e});
        i = e;
    }
    P.pt_ptr.assign(1, 0);
    P.part_rows.clear();
    P.part_step.clear();
    for (int p = 0; p < nparts; ++p) {
        int step = 0;
        for (auto& sg : segs[p]) {
            for (int i = sg.first; i < sg.second; ++i) {
                P.part_rows.push_back(i);
                P.part_step.push_back(step);
            }
            ++step;
        }
        P.pt_ptr.push_back((int32_t)P.part_rows.size());
    }
    auto rows = [&](const std::vector<int32_t>& sptr, std::vector<int32_t>& row) {
        row.assign(2 * (size_t)n, 0);
        for (int c = 0; c < P.nchunks; ++c)
            for (int i = P.chunk_start[c]; i < P.chunk_start[c + 1]; ++i) {
                row[2 * (size_t)i] = sptr[c] + (i - P.chunk_start[c]);
                row[2 * (size_t)i + 1] = (sptr[c + 1] - sptr[c]) / kSlice;
            }
    };
    rows(P.f_sptr, P.f_row);
    rows(P.b_sptr, P.b_row);
    auto locs = [&](const std::vector<int32_t>& sptr, const std::vector<int32_t>& col, std::vector<int32_t>& loc) {
        loc.assign(col.size(), -1);
        for (int c = 0; c < P.nchunks; ++c) {
            const int r0 = P.chunk_start[c], r1 = P.chunk_start[c + 1];
            const int e0 = sptr[c], W = (sptr[c + 1] - e0) / kSlice;
            for (int k = 0; k < W; ++k)
                for (int l = 0; l < r1 - r0; ++l) {
                    const int e = e0 + k * kSlice + l, d = col[e];
                    if (d < 0) continue;
                    const int cell = P.perm[r0 + l], dc = P.perm[d];
                    if (dc / B == cell / B) loc[e] = dc - (cell / B) * B;
                }
        }
    };
    locs(P.f_sptr, P.f_col, P.f_loc);
    locs(P.b_sptr, P.b_col, P.b_loc);
}

}  // namespace mrg
