// api.cu -- the extern "C" boundary declared in include/mrgpu.h.
// Every entry point converts C++ exceptions into status codes; nothing
// throws across the ABI.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/mrgpu.h"
#include "engine.h"
#include "kernels.h"
#include "blockpc.h"
#include "dn.h"
#include "gamg.h"
#include "ggi_build.h"
#include "mono.h"
#include "noalloc.h"
#include "server.h"

using namespace mrg;

struct mrg_ctx {
    Ctx c;
};
struct mrg_mesh {
    Mesh m;
};
struct mrg_ggi {
    Ggi g;
};
struct mrg_server {
    std::unique_ptr<Server> s;
};
struct mrg_dn {
    std::unique_ptr<Dn> d;
};
struct mrg_mono {
    Mono m;
};
struct mrg_batch {
    Ctx* ctx = nullptr;
    int ordering = 0;
    std::vector<Mesh*> meshes;
    BatchHost bh;
    double* d_stage = nullptr;    // caller-numbered b and x of every member
    size_t stage_n = 0;
    std::vector<size_t> offset;   // member s: b at offset[s], x at stage_n + offset[s]
    ~mrg_batch()
    {
        if (ctx) ctx->release(d_stage);
    }
};

namespace {
// A plain buffer, not std::string: callers may reach the ABI from static
// destructors after thread-local objects with destructors are gone.
thread_local char g_last_error[1024];

int fail(int code, const std::string& msg)
{
    std::snprintf(g_last_error, sizeof g_last_error, "%s", msg.c_str());
    return code;
}

template <typename F>
int guard(F&& f)
{
    try {
        g_last_error[0] = '\0';
        return f();
    } catch (const Error& e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(MRG_E_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(MRG_E_INVALID, e.what());
    }
}

Controls to_controls(const mrg_controls* c)
{
    Controls k;
    if (!c) return k;
    k.tol = c->tolerance;
    k.rel_tol = c->rel_tol;
    k.min_iter = c->min_iter;
    k.max_iter = c->max_iter;
    k.solver = c->solver;
    k.pc = c->preconditioner;
    k.precision = c->precision;
    k.ordering = c->ordering;
    k.inner_rel_tol = c->inner_rel_tol > 0 ? c->inner_rel_tol : 1e-5;
    k.inner_max_iter = c->inner_max_iter;
    k.max_outer = c->max_outer > 0 ? c->max_outer : 50;
    k.k_launch = c->iters_per_launch > 0 ? c->iters_per_launch : 16;
    k.n_sweeps = c->n_sweeps > 0 ? c->n_sweeps : 1;
    if (k.solver < 0 || k.solver > 4) throw Error(MRG_E_INVALID, "unknown solver");
    if (k.solver == MRG_SOLVER_GAMG) {
        if (c->smoother != MRG_SMOOTHER_GAUSS_SEIDEL) throw Error(MRG_E_INVALID, "GAMG: smoother must be GaussSeidel");
        if (c->precision != MRG_PRECISION_FP64 || c->ordering != MRG_ORDER_EXACT)
            throw Error(MRG_E_INVALID, "GAMG runs in FP64 in foam's order (precision fp64, ordering exact)");
        k.pc = PC_NONE;
        k.gamg_coarsest = c->gamg_coarsest_cells > 0 ? c->gamg_coarsest_cells : 10;
        k.gamg_post = c->gamg_post_sweeps >= 0 ? c->gamg_post_sweeps : 2;
        k.gamg_finest = c->gamg_finest_sweeps >= 0 ? c->gamg_finest_sweeps : 2;
        k.gamg_max_post = c->gamg_max_post_sweeps;
        k.gamg_post_mult = c->gamg_post_sweeps_level_multiplier;
        k.gamg_scale = c->gamg_scale_correction != 0;
        k.gamg_agglomerator = c->gamg_agglomerator;
        if (k.gamg_coarsest > 64) throw Error(MRG_E_INVALID, "GAMG: nCellsInCoarsestLevel must be at most 64");
        if (k.gamg_max_post < 0 || k.gamg_post_mult < 0)
            throw Error(MRG_E_INVALID, "GAMG: maxPostSweeps and postSweepsLevelMultiplier must be non-negative");
        if (k.gamg_agglomerator != MRG_AGGLOMERATOR_ALGEBRAIC_PAIR &&
            k.gamg_agglomerator != MRG_AGGLOMERATOR_FACE_AREA_PAIR)
            throw Error(MRG_E_INVALID, "GAMG: unknown agglomerator");
    }
    if (k.solver == MRG_SOLVER_SMOOTH) {
        if (c->smoother < MRG_SMOOTHER_GAUSS_SEIDEL || c->smoother > MRG_SMOOTHER_DILU_GAUSS_SEIDEL)
            throw Error(MRG_E_INVALID, "unknown smoother");
        if (c->precision != MRG_PRECISION_FP64 || c->ordering != MRG_ORDER_EXACT)
            throw Error(MRG_E_INVALID, "smoothSolver runs in FP64 in foam's order (precision fp64, ordering exact)");
        k.smoother = c->smoother;
        // the factorisation the DIC / DILU smoothers apply (Gauss-Seidel needs none)
        const bool dilu = c->smoother == MRG_SMOOTHER_DILU || c->smoother == MRG_SMOOTHER_DILU_GAUSS_SEIDEL;
        k.pc = c->smoother == MRG_SMOOTHER_GAUSS_SEIDEL ? PC_NONE : (dilu ? PC_DILU : PC_DIC);
    }
    if (k.pc < 0 || k.pc > 4) throw Error(MRG_E_INVALID, "unknown preconditioner");
    if (k.pc == PC_BLOCK) {
        if (k.solver != MRG_SOLVER_PCG && k.solver != MRG_SOLVER_BICGSTAB)
            throw Error(MRG_E_INVALID, "block preconditioner: solver must be PCG or BiCGStab");
        if (k.precision != MRG_PRECISION_FP64 || k.ordering != MRG_ORDER_EXACT)
            throw Error(MRG_E_INVALID, "block preconditioner: FP64 in foam's order (precision fp64, ordering exact)");
    }
    if (k.precision < 0 || k.precision > 1) throw Error(MRG_E_INVALID, "unknown precision");
    if (k.ordering < 0 || k.ordering > 1) throw Error(MRG_E_INVALID, "unknown ordering");
    if (k.max_iter < 0 || k.min_iter < 0) throw Error(MRG_E_INVALID, "negative iteration bounds");
    return k;
}

void fill_perf(mrg_perf* p, const Perf& r)
{
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->initial_residual = r.res0;
    p->final_residual = r.res;
    p->n_iter = r.iters;
    p->converged = r.converged;
    p->singular = r.singular;
    p->status = r.status;
    p->n_outer = r.outer;
    p->fallback = r.fallback;
    p->solve_ms = r.ms;
}

// Device staging buffers of a context for the host-pointer entry points.
double* stage(Ctx* c, int k, size_t n)
{
    if (c->stage_cap < n) {
        for (auto& p : c->stage) {
            c->release(p);
            p = nullptr;
        }
        c->stage_cap = n;
    }
    if (!c->stage[k]) c->stage[k] = (double*)c->alloc(8 * c->stage_cap);
    return c->stage[k];
}

void h2d(Ctx* c, double* d, const double* h, size_t n)
{
    MRG_CUDA(cudaMemcpyAsync(d, h, 8 * n, cudaMemcpyHostToDevice, c->st));
}
void d2h(Ctx* c, double* h, const double* d, size_t n)
{
    MRG_CUDA(cudaMemcpyAsync(h, d, 8 * n, cudaMemcpyDeviceToHost, c->st));
    MRG_CUDA(cudaStreamSynchronize(c->st));
}

}  // namespace

namespace mrg {
// The calling thread's last error text, for ABI entries in other files
// (block.cpp); they clear it on entry.
void set_last_error(const std::string& msg) { std::snprintf(g_last_error, sizeof g_last_error, "%s", msg.c_str()); }
}  // namespace mrg

extern "C" {

const char* mrg_last_error(void) { return g_last_error; }

const char* mrg_version(void) { return "mrgpu 0.1 (sm_103a)"; }

void mrg_controls_default(mrg_controls* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->tolerance = 1e-6;
    c->rel_tol = 0.0;
    c->min_iter = 0;
    c->max_iter = 1000;
    c->solver = MRG_SOLVER_PCG;
    c->preconditioner = MRG_PRECOND_DIC;
    c->precision = MRG_PRECISION_FP64;
    c->ordering = MRG_ORDER_EXACT;
    c->inner_rel_tol = 1e-5;
    c->inner_max_iter = 0;
    c->max_outer = 50;
    c->iters_per_launch = 16;
    c->smoother = MRG_SMOOTHER_GAUSS_SEIDEL;
    c->n_sweeps = 1;
    c->gamg_coarsest_cells = 10;
    c->gamg_post_sweeps = 2;
    c->gamg_finest_sweeps = 2;
    c->gamg_max_post_sweeps = 4;
    c->gamg_post_sweeps_level_multiplier = 1;
    c->gamg_scale_correction = 1;
    c->gamg_agglomerator = MRG_AGGLOMERATOR_ALGEBRAIC_PAIR;
}

int mrg_ctx_create(int device, size_t hbm_budget_bytes, mrg_ctx** out)
{
    return guard([&] {
        if (!out) return fail(MRG_E_INVALID, "out is NULL");
        *out = nullptr;
        int ndev = 0;
        MRG_CUDA(cudaGetDeviceCount(&ndev));
        if (device < 0 || device >= ndev) return fail(MRG_E_INVALID, "no such CUDA device");
        MRG_CUDA(cudaSetDevice(device));
        auto* c = new mrg_ctx();
        try {
            c->c.device = device;
            c->c.budget = hbm_budget_bytes;
            MRG_CUDA(cudaDeviceGetAttribute(&c->c.nsm, cudaDevAttrMultiProcessorCount, device));
            set_device_sms(c->c.nsm);
            MRG_CUDA(cudaStreamCreateWithFlags(&c->c.st, cudaStreamNonBlocking));
            MRG_CUDA(cudaStreamSynchronize(c->c.st));
        } catch (...) {
            delete c;
            throw;
        }
        *out = c;
        return (int)MRG_OK;
    });
}

int mrg_ctx_destroy(mrg_ctx* ctx)
{
    return guard([&] {
        if (!ctx) return (int)MRG_OK;
        delete ctx;
        return (int)MRG_OK;
    });
}

int mrg_ctx_mem_used(mrg_ctx* ctx, size_t* bytes)
{
    if (!ctx || !bytes) return fail(MRG_E_INVALID, "NULL argument");
    *bytes = ctx->c.used;
    return MRG_OK;
}

int mrg_ctx_set_watchdog(mrg_ctx* ctx, long long wait_cycles, int unpublished_chunk)
{
    if (!ctx) return fail(MRG_E_INVALID, "ctx is NULL");
    if (wait_cycles < 0 || unpublished_chunk < -1) return fail(MRG_E_INVALID, "bad watchdog setting");
    ctx->c.wait_cycles = wait_cycles;
    ctx->c.unpublished1 = unpublished_chunk + 1;
    return MRG_OK;
}

int mrg_host_alloc(size_t bytes, void** out)
{
    return guard([&] {
        if (!out) return fail(MRG_E_INVALID, "out is NULL");
        MRG_CUDA(cudaMallocHost(out, bytes ? bytes : 16));
        return (int)MRG_OK;
    });
}

int mrg_host_free(void* p)
{
    return guard([&] {
        if (p) MRG_CUDA(cudaFreeHost(p));
        return (int)MRG_OK;
    });
}

int mrg_mesh_upload(mrg_ctx* ctx, int n_cells, int n_faces, const int32_t* lower_addr, const int32_t* upper_addr,
                    int n_iface, const mrg_iface_desc* ifaces, mrg_mesh** out)
{
    return guard([&] {
        if (!ctx || !out) return fail(MRG_E_INVALID, "NULL argument");
        *out = nullptr;
        if (n_iface < 0 || (n_iface > 0 && !ifaces)) return fail(MRG_E_INVALID, "bad interface list");
        MRG_CUDA(cudaSetDevice(ctx->c.device));
        IfaceHost ifc;
        ifc.ptr.push_back(0);
        for (int p = 0; p < n_iface; ++p) {
            const mrg_iface_desc& d = ifaces[p];
            if (d.n_faces < 0 || (d.n_faces > 0 && (!d.face_cells || !d.src_cell)))
                return fail(MRG_E_INVALID, "interface " + std::to_string(p) + ": NULL arrays");
            for (int i = 0; i < d.n_faces; ++i) {
                ifc.cells.push_back(d.face_cells[i]);
                const int k0 = d.src_ptr ? d.src_ptr[i] : i, k1 = d.src_ptr ? d.src_ptr[i + 1] : i + 1;
                if (k1 < k0) return fail(MRG_E_INVALID, "interface CSR pointer decreases");
                for (int k = k0; k < k1; ++k) {
                    ifc.src.push_back(d.src_cell[k]);
                    ifc.w.push_back(d.src_weight ? d.src_weight[k] : 1.0);
                }
                ifc.ptr.push_back((int32_t)ifc.src.size());
            }
        }
        std::string msg = validate_addressing(n_cells, n_faces, lower_addr, upper_addr, ifc);
        if (!msg.empty()) return fail(MRG_E_INVALID, msg);
        if ((long long)n_cells + 1024 > (1LL << 30)) return fail(MRG_E_INVALID, "mesh too large for int32 layout");
        auto* m = new mrg_mesh();
        m->m.ctx = &ctx->c;
        m->m.n = n_cells;
        m->m.nf = n_faces;
        m->m.ni = ifc.size();
        m->m.lower.assign(lower_addr, lower_addr + n_faces);
        m->m.upper.assign(upper_addr, upper_addr + n_faces);
        m->m.ifc = std::move(ifc);
        *out = m;
        return (int)MRG_OK;
    });
}

int mrg_mesh_destroy(mrg_mesh* mesh)
{
    return guard([&] {
        delete mesh;
        return (int)MRG_OK;
    });
}

int mrg_mesh_levels(mrg_mesh* mesh, int ordering, int* n_levels)
{
    return guard([&] {
        if (!mesh || !n_levels) return fail(MRG_E_INVALID, "NULL argument");
        *n_levels = mesh->m.plan(ordering).sys.nlevels;
        return (int)MRG_OK;
    });
}

int mrg_mesh_set_blocks(mrg_mesh* mesh, int bs, int n_cells, int n_faces, const int32_t* lower_addr,
                        const int32_t* upper_addr)
{
    return guard([&] {
        if (!mesh) return fail(MRG_E_INVALID, "NULL argument");
        set_blocks(mesh->m, bs, n_cells, n_faces, lower_addr, upper_addr);
        return (int)MRG_OK;
    });
}

int mrg_mesh_set_face_areas(mrg_mesh* mesh, const double* sf)
{
    return guard([&] {
        if (!mesh || (!sf && mesh->m.nf > 0)) return fail(MRG_E_INVALID, "NULL argument");
        std::vector<double> w = face_area_weights(sf, mesh->m.nf);
        for (int f = 0; f < mesh->m.nf; ++f)
            if (!std::isfinite(w[f]))
                return fail(MRG_E_INVALID, "face " + std::to_string(f) + ": zero or non-finite area vector");
        mesh->m.agglom_w = std::move(w);
        mesh->m.agglom_version += 1;
        return (int)MRG_OK;
    });
}

int mrg_coeffs_upload(mrg_mesh* mesh, const double* diag, const double* upper, const double* lower_or_null,
                      const double* iface_bou, const double* iface_int_or_null)
{
    return guard([&] {
        if (!mesh) return fail(MRG_E_INVALID, "mesh is NULL");
        upload_coeffs(mesh->m, diag, upper, lower_or_null, iface_bou, iface_int_or_null, cudaMemcpyHostToDevice, true);
        return (int)MRG_OK;
    });
}

int mrg_coeffs_upload_device(mrg_mesh* mesh, const double* diag, const double* upper, const double* lower_or_null,
                             const double* iface_bou, const double* iface_int_or_null)
{
    return guard([&] {
        if (!mesh) return fail(MRG_E_INVALID, "mesh is NULL");
        upload_coeffs(mesh->m, diag, upper, lower_or_null, iface_bou, iface_int_or_null, cudaMemcpyDeviceToDevice, false);
        return (int)MRG_OK;
    });
}

int mrg_solve(mrg_mesh* mesh, const double* b, double* x_inout, const mrg_controls* controls, mrg_perf* perf)
{
    return guard([&] {
        if (!mesh || !b || !x_inout) return fail(MRG_E_INVALID, "NULL argument");
        Controls k = to_controls(controls);
        Mesh& m = mesh->m;
        Ctx* c = m.ctx;
        double* db = stage(c, 0, m.n);
        double* dx = stage(c, 1, m.n);
        h2d(c, db, b, m.n);
        h2d(c, dx, x_inout, m.n);
        Perf r = solve_device(m, db, dx, k);
        d2h(c, x_inout, dx, m.n);
        fill_perf(perf, r);
        if (r.status != MRG_OK) return fail(r.status, "non-finite residual (breakdown)");
        return (int)MRG_OK;
    });
}

int mrg_solve_device(mrg_mesh* mesh, const double* d_b, double* d_x_inout, const mrg_controls* controls,
                     mrg_perf* perf)
{
    return guard([&] {
        if (!mesh || !d_b || !d_x_inout) return fail(MRG_E_INVALID, "NULL argument");
        Controls k = to_controls(controls);
        Perf r = solve_device(mesh->m, d_b, d_x_inout, k);
        fill_perf(perf, r);
        if (r.status != MRG_OK) return fail(r.status, "non-finite residual (breakdown)");
        return (int)MRG_OK;
    });
}

int mrg_amul(mrg_mesh* mesh, const double* x, double* y, int transpose)
{
    return guard([&] {
        if (!mesh || !x || !y) return fail(MRG_E_INVALID, "NULL argument");
        Mesh& m = mesh->m;
        Ctx* c = m.ctx;
        double* dx = stage(c, 0, m.n);
        double* dy = stage(c, 1, m.n);
        h2d(c, dx, x, m.n);
        amul_device(m, dx, dy, transpose);
        d2h(c, y, dy, m.n);
        return (int)MRG_OK;
    });
}

int mrg_residual(mrg_mesh* mesh, const double* b, const double* x, double* residual, double* norm_factor)
{
    return guard([&] {
        if (!mesh || !b || !x) return fail(MRG_E_INVALID, "NULL argument");
        Mesh& m = mesh->m;
        Ctx* c = m.ctx;
        double* db = stage(c, 0, m.n);
        double* dx = stage(c, 1, m.n);
        h2d(c, db, b, m.n);
        h2d(c, dx, x, m.n);
        residual_device(m, db, dx, residual, norm_factor);
        return (int)MRG_OK;
    });
}

int mrg_precondition(mrg_mesh* mesh, int precond, int ordering, const double* r, double* w, int transpose)
{
    return guard([&] {
        if (!mesh || !r || !w) return fail(MRG_E_INVALID, "NULL argument");
        if (precond < 0 || precond > 4) return fail(MRG_E_INVALID, "unknown preconditioner");
        if (precond == PC_BLOCK && (transpose || ordering != MRG_ORDER_EXACT))
            return fail(MRG_E_INVALID, "block preconditioner: no transpose, exact ordering only");
        Mesh& m = mesh->m;
        Ctx* c = m.ctx;
        double* dr = stage(c, 0, m.n);
        double* dw = stage(c, 1, m.n);
        h2d(c, dr, r, m.n);
        precondition_device(m, precond, ordering, dr, dw, transpose);
        d2h(c, w, dw, m.n);
        return (int)MRG_OK;
    });
}

int mrg_factor_diag(mrg_mesh* mesh, int precond, int ordering, double* rD)
{
    return guard([&] {
        if (!mesh || !rD) return fail(MRG_E_INVALID, "NULL argument");
        if (precond < 1 || precond > 3) return fail(MRG_E_INVALID, "preconditioner has no factor");
        Mesh& m = mesh->m;
        double* d = stage(m.ctx, 2, m.n);
        factor_diag_device(m, precond, ordering, d);
        d2h(m.ctx, rD, d, m.n);
        return (int)MRG_OK;
    });
}

int mrg_ggi_create(mrg_ctx* ctx, int n_dst, int n_src, const int32_t* row_ptr, const int32_t* src_addr,
                   const double* weights, mrg_ggi** out)
{
    return guard([&] {
        if (!ctx || !out || !row_ptr || n_dst < 0 || n_src < 0) return fail(MRG_E_INVALID, "bad argument");
        *out = nullptr;
        if (row_ptr[0] != 0) return fail(MRG_E_INVALID, "row_ptr must start at 0");
        for (int i = 0; i < n_dst; ++i)
            if (row_ptr[i + 1] < row_ptr[i]) return fail(MRG_E_INVALID, "row_ptr decreases");
        const int nnz = row_ptr[n_dst];
        if (nnz > 0 && (!src_addr || !weights)) return fail(MRG_E_INVALID, "NULL weights");
        for (int k = 0; k < nnz; ++k)
            if (src_addr[k] < 0 || src_addr[k] >= n_src) return fail(MRG_E_INVALID, "source face out of range");
        Ctx* c = &ctx->c;
        auto* g = new mrg_ggi();
        try {
            g->g.ctx = c;
            g->g.n_dst = n_dst;
            g->g.n_src = n_src;
            g->g.ptr = (int32_t*)c->alloc(4 * (size_t)(n_dst + 1));
            g->g.addr = (int32_t*)c->alloc(4 * (size_t)std::max(nnz, 1));
            g->g.w = (double*)c->alloc(8 * (size_t)std::max(nnz, 1));
            MRG_CUDA(cudaMemcpyAsync(g->g.ptr, row_ptr, 4 * (size_t)(n_dst + 1), cudaMemcpyHostToDevice, c->st));
            if (nnz) {
                MRG_CUDA(cudaMemcpyAsync(g->g.addr, src_addr, 4 * (size_t)nnz, cudaMemcpyHostToDevice, c->st));
                MRG_CUDA(cudaMemcpyAsync(g->g.w, weights, 8 * (size_t)nnz, cudaMemcpyHostToDevice, c->st));
            }
            MRG_CUDA(cudaStreamSynchronize(c->st));
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
        return (int)MRG_OK;
    });
}

int mrg_ggi_destroy(mrg_ggi* ggi)
{
    return guard([&] {
        delete ggi;
        return (int)MRG_OK;
    });
}

int mrg_ggi_apply_device(mrg_ggi* ggi, const double* d_src, double* d_dst, int ncomp)
{
    return guard([&] {
        if (!ggi || !d_src || !d_dst || ncomp < 1 || ncomp > 16) return fail(MRG_E_INVALID, "bad argument");
        Ggi& g = ggi->g;
        launch_ggi(g.n_dst, g.ptr, g.addr, g.w, d_src, d_dst, ncomp, g.ctx->st);
        MRG_CUDA(cudaGetLastError());
        MRG_CUDA(cudaStreamSynchronize(g.ctx->st));
        return (int)MRG_OK;
    });
}

int mrg_ggi_time(mrg_ggi* ggi, const double* d_src, double* d_dst, int ncomp, int reps, float* ms_per_apply)
{
    return guard([&] {
        if (!ggi || !d_src || !d_dst || ncomp < 1 || ncomp > 16 || reps < 1 || !ms_per_apply)
            return fail(MRG_E_INVALID, "bad argument");
        Ggi& g = ggi->g;
        cudaStream_t st = g.ctx->st;
        launch_ggi(g.n_dst, g.ptr, g.addr, g.w, d_src, d_dst, ncomp, st);   // warm-up
        cudaEvent_t e0, e1;
        MRG_CUDA(cudaEventCreate(&e0));
        MRG_CUDA(cudaEventCreate(&e1));
        MRG_CUDA(cudaEventRecord(e0, st));
        for (int i = 0; i < reps; ++i) launch_ggi(g.n_dst, g.ptr, g.addr, g.w, d_src, d_dst, ncomp, st);
        MRG_CUDA(cudaEventRecord(e1, st));
        MRG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        MRG_CUDA(cudaGetLastError());
        *ms_per_apply = ms / (float)reps;
        return (int)MRG_OK;
    });
}

int mrg_ggi_build(mrg_ctx* ctx, int na, const int32_t* a_ptr, const double* a_xy, int nb, const int32_t* b_ptr,
                  const double* b_xy, double tol, mrg_ggi** a_from_b, mrg_ggi** b_from_a)
{
    return guard([&] {
        if (!ctx || !a_from_b || !b_from_a || na < 0 || nb < 0 || !a_ptr || !b_ptr || !(tol >= 0.0))
            return fail(MRG_E_INVALID, "bad argument");
        *a_from_b = nullptr;
        *b_from_a = nullptr;
        auto* ab = new mrg_ggi();
        auto* ba = new mrg_ggi();
        try {
            ggi_build(&ctx->c, na, a_ptr, a_xy, nb, b_ptr, b_xy, tol, ab->g, ba->g);
        } catch (...) {
            delete ab;
            delete ba;
            throw;
        }
        *a_from_b = ab;
        *b_from_a = ba;
        return (int)MRG_OK;
    });
}

int mrg_direct_map_build(mrg_ctx* ctx, int na, const double* a_centres, int nb, const double* b_centres, double tol,
                         mrg_ggi** a_from_b, mrg_ggi** b_from_a)
{
    return guard([&] {
        if (!ctx || !a_from_b || !b_from_a) return fail(MRG_E_INVALID, "bad argument");
        *a_from_b = nullptr;
        *b_from_a = nullptr;
        auto* ab = new mrg_ggi();
        auto* ba = new mrg_ggi();
        try {
            direct_map_build(&ctx->c, na, a_centres, nb, b_centres, tol, ab->g, ba->g);
        } catch (...) {
            delete ab;
            delete ba;
            throw;
        }
        *a_from_b = ab;
        *b_from_a = ba;
        return (int)MRG_OK;
    });
}

int mrg_ggi_get(mrg_ggi* ggi, int* n_dst, int* n_src, int* nnz, int32_t* row_ptr, int32_t* src_addr,
                double* weights)
{
    return guard([&] {
        if (!ggi) return fail(MRG_E_INVALID, "bad argument");
        Ggi& g = ggi->g;
        Ctx* c = g.ctx;
        int32_t total = 0;
        MRG_CUDA(cudaMemcpyAsync(&total, g.ptr + g.n_dst, 4, cudaMemcpyDeviceToHost, c->st));
        MRG_CUDA(cudaStreamSynchronize(c->st));
        if (n_dst) *n_dst = g.n_dst;
        if (n_src) *n_src = g.n_src;
        if (nnz) *nnz = total;
        if (row_ptr)
            MRG_CUDA(cudaMemcpyAsync(row_ptr, g.ptr, 4 * (size_t)(g.n_dst + 1), cudaMemcpyDeviceToHost, c->st));
        if (src_addr && total)
            MRG_CUDA(cudaMemcpyAsync(src_addr, g.addr, 4 * (size_t)total, cudaMemcpyDeviceToHost, c->st));
        if (weights && total)
            MRG_CUDA(cudaMemcpyAsync(weights, g.w, 8 * (size_t)total, cudaMemcpyDeviceToHost, c->st));
        MRG_CUDA(cudaStreamSynchronize(c->st));
        return (int)MRG_OK;
    });
}

int mrg_ggi_apply(mrg_ggi* ggi, const double* src, double* dst, int ncomp)
{
    return guard([&] {
        if (!ggi || !src || !dst || ncomp < 1 || ncomp > 16) return fail(MRG_E_INVALID, "bad argument");
        Ggi& g = ggi->g;
        Ctx* c = g.ctx;
        if (g.cap_comp < ncomp) {
            c->release(g.d_src);
            c->release(g.d_dst);
            g.d_src = (double*)c->alloc(8 * (size_t)std::max(g.n_src, 1) * ncomp);
            g.d_dst = (double*)c->alloc(8 * (size_t)std::max(g.n_dst, 1) * ncomp);
            g.cap_comp = ncomp;
        }
        MRG_CUDA(cudaMemcpyAsync(g.d_src, src, 8 * (size_t)g.n_src * ncomp, cudaMemcpyHostToDevice, c->st));
        launch_ggi(g.n_dst, g.ptr, g.addr, g.w, g.d_src, g.d_dst, ncomp, c->st);
        MRG_CUDA(cudaGetLastError());
        MRG_CUDA(cudaMemcpyAsync(dst, g.d_dst, 8 * (size_t)g.n_dst * ncomp, cudaMemcpyDeviceToHost, c->st));
        MRG_CUDA(cudaStreamSynchronize(c->st));
        return (int)MRG_OK;
    });
}

int mrg_batch_create(mrg_ctx* ctx, int n_meshes, mrg_mesh* const* meshes, int ordering, mrg_batch** out)
{
    return guard([&] {
        if (!ctx || !out || n_meshes < 1 || !meshes) return fail(MRG_E_INVALID, "bad argument");
        if (ordering < 0 || ordering > 1) return fail(MRG_E_INVALID, "unknown ordering");
        *out = nullptr;
        auto* b = new mrg_batch();
        try {
            b->ctx = &ctx->c;
            b->ordering = ordering;
            std::vector<PlanState*> plans;
            size_t tot = 0;
            for (int i = 0; i < n_meshes; ++i) {
                if (!meshes[i] || meshes[i]->m.ctx != &ctx->c)
                    throw Error(MRG_E_INVALID, "batch member " + std::to_string(i) + " is NULL or in another context");
                for (int j = 0; j < i; ++j)
                    if (meshes[j] == meshes[i])
                        throw Error(MRG_E_INVALID, "a mesh appears twice in the batch");
                b->meshes.push_back(&meshes[i]->m);
                plans.push_back(&meshes[i]->m.plan(ordering));
                b->offset.push_back(tot);
                tot += (size_t)meshes[i]->m.n;
            }
            b->stage_n = tot;
            b->d_stage = (double*)ctx->c.alloc(16 * tot);
            b->bh.init(&ctx->c);
            b->bh.set(plans);
        } catch (...) {
            delete b;
            throw;
        }
        *out = b;
        return (int)MRG_OK;
    });
}

int mrg_batch_destroy(mrg_batch* batch)
{
    return guard([&] {
        delete batch;
        return (int)MRG_OK;
    });
}

// Shared by the host and device variants: d_b[s], d_x[s] are device pointers.
static int batch_solve_device(mrg_batch* batch, const double* const* d_b, double* const* d_x,
                              const mrg_controls* controls, mrg_perf* perfs)
{
    Controls k = to_controls(controls);
    if (k.ordering != batch->ordering) throw Error(MRG_E_INVALID, "controls.ordering differs from the batch's");
    prepare_batch(batch->bh, batch->meshes, k);
    for (size_t s = 0; s < batch->meshes.size(); ++s) {
        PlanState* P = batch->bh.members[s];
        P->sys.in_b = d_b[s];
        P->sys.in_x = d_x[s];
        P->sys.out_x = d_x[s];
    }
    batch->bh.sync_sys();
    std::vector<Perf> r = solve_batch(batch->bh, k);
    int status = MRG_OK;
    for (size_t s = 0; s < r.size(); ++s) {
        if (perfs) fill_perf(perfs + s, r[s]);
        if (r[s].status != MRG_OK) status = r[s].status;
    }
    if (status != MRG_OK) return fail(status, "non-finite residual in a batch member (breakdown)");
    return (int)MRG_OK;
}

int mrg_batch_solve_device(mrg_batch* batch, const double* const* d_b, double* const* d_x,
                           const mrg_controls* controls, mrg_perf* perfs)
{
    return guard([&] {
        if (!batch || !d_b || !d_x) return fail(MRG_E_INVALID, "NULL argument");
        return batch_solve_device(batch, d_b, d_x, controls, perfs);
    });
}

int mrg_batch_solve(mrg_batch* batch, const double* const* b, double* const* x, const mrg_controls* controls,
                    mrg_perf* perfs)
{
    return guard([&] {
        if (!batch || !b || !x) return fail(MRG_E_INVALID, "NULL argument");
        Ctx* c = batch->ctx;
        const size_t ns = batch->meshes.size();
        std::vector<const double*> db(ns);
        std::vector<double*> dx(ns);
        for (size_t s = 0; s < ns; ++s) {
            const size_t n = (size_t)batch->meshes[s]->n;
            double* pb = batch->d_stage + batch->offset[s];
            double* px = batch->d_stage + batch->stage_n + batch->offset[s];
            if (!b[s] || !x[s]) return fail(MRG_E_INVALID, "NULL member vector");
            MRG_CUDA(cudaMemcpyAsync(pb, b[s], 8 * n, cudaMemcpyHostToDevice, c->st));
            MRG_CUDA(cudaMemcpyAsync(px, x[s], 8 * n, cudaMemcpyHostToDevice, c->st));
            db[s] = pb;
            dx[s] = px;
        }
        int rc = batch_solve_device(batch, db.data(), dx.data(), controls, perfs);
        for (size_t s = 0; s < ns; ++s)
            MRG_CUDA(cudaMemcpyAsync(x[s], dx[s], 8 * (size_t)batch->meshes[s]->n, cudaMemcpyDeviceToHost, c->st));
        MRG_CUDA(cudaStreamSynchronize(c->st));
        return rc;
    });
}

int mrg_dev_alloc(mrg_ctx* ctx, size_t bytes, void** out)
{
    return guard([&] {
        if (!ctx || !out) return fail(MRG_E_INVALID, "NULL argument");
        *out = ctx->c.alloc(bytes);
        MRG_CUDA(cudaStreamSynchronize(ctx->c.st));
        return (int)MRG_OK;
    });
}

int mrg_dev_free(mrg_ctx* ctx, void* p)
{
    return guard([&] {
        if (!ctx) return fail(MRG_E_INVALID, "NULL context");
        MRG_CUDA(cudaStreamSynchronize(ctx->c.st));
        ctx->c.release(p);
        return (int)MRG_OK;
    });
}

int mrg_dev_copy(mrg_ctx* ctx, void* dst, const void* src, size_t bytes, int kind)
{
    return guard([&] {
        if (!ctx || (bytes && (!dst || !src))) return fail(MRG_E_INVALID, "NULL argument");
        cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice
                                     : (kind == 1 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice);
        if (kind < 0 || kind > 2) return fail(MRG_E_INVALID, "unknown copy kind");
        if (bytes) MRG_CUDA(cudaMemcpyAsync(dst, src, bytes, k, ctx->c.st));
        MRG_CUDA(cudaStreamSynchronize(ctx->c.st));
        return (int)MRG_OK;
    });
}

int mrg_event_record(mrg_ctx* ctx, int slot)
{
    return guard([&] {
        if (!ctx || slot < 0 || slot >= 64) return fail(MRG_E_INVALID, "bad event slot");
        cudaEvent_t& e = ctx->c.events[slot];
        if (!e) MRG_CUDA(cudaEventCreate(&e));
        MRG_CUDA(cudaEventRecord(e, ctx->c.st));
        return (int)MRG_OK;
    });
}

int mrg_event_elapsed(mrg_ctx* ctx, int a, int b, float* ms)
{
    return guard([&] {
        if (!ctx || !ms || a < 0 || b < 0 || a >= 64 || b >= 64) return fail(MRG_E_INVALID, "bad argument");
        if (!ctx->c.events[a] || !ctx->c.events[b]) return fail(MRG_E_INVALID, "event slot not recorded");
        MRG_CUDA(cudaEventSynchronize(ctx->c.events[b]));
        MRG_CUDA(cudaEventElapsedTime(ms, ctx->c.events[a], ctx->c.events[b]));
        return (int)MRG_OK;
    });
}

int mrg_kernel_launches(uint64_t* count)
{
    if (!count) return fail(MRG_E_INVALID, "NULL argument");
    *count = (uint64_t)launch_count();
    return MRG_OK;
}

int mrg_time_kernel(mrg_mesh* mesh, const mrg_controls* controls, int kernel, int reps, float* ms_per_launch)
{
    return guard([&] {
        if (!mesh || !ms_per_launch) return fail(MRG_E_INVALID, "NULL argument");
        Controls k = to_controls(controls);
        *ms_per_launch = time_kernel(mesh->m, k, kernel, reps);
        return (int)MRG_OK;
    });
}

static void fill_tuning(mrg_tuning* out, const Tuning& t)
{
    if (!out) return;
    std::memset(out, 0, sizeof *out);
    out->mode = t.mode;
    out->iters_per_launch = t.k;
    out->sweep_chunks_per_cta = t.sweep_div;
    // the Amul kernel: block shape (256 row threads; 288 with the streamed
    // kernel's producer warp) and rows a warp takes per step
    out->spmv_kernel = t.spmv;
    out->spmv_block_threads = t.spmv == 0 ? 0 : t.spmv >= 2 ? kBlock + 32 : kBlock;
    out->spmv_rows_per_warp_step = t.spmv == 0 ? 0 : t.spmv == 2 ? 32 : 64;
    out->candidates = t.candidates;
    out->us_per_iter = t.us_per_iter;
}

int mrg_mesh_tune(mrg_mesh* mesh, const double* d_b, const double* d_x, const mrg_controls* controls,
                  mrg_tuning* out)
{
    return guard([&] {
        if (!mesh || !d_b || !d_x) return fail(MRG_E_INVALID, "NULL argument");
        Controls k = to_controls(controls);
        PlanState& P = prepare(mesh->m, k);
        P.sys.in_b = d_b;
        P.sys.in_x = d_x;
        P.sys.out_x = nullptr;
        P.sync_sys();
        P.single.sync_sys();
        fill_tuning(out, tune_batch(P.single, k));
        MRG_CUDA(cudaStreamSynchronize(mesh->m.ctx->st));
        return (int)MRG_OK;
    });
}

int mrg_batch_tune(mrg_batch* batch, const double* const* d_b, const double* const* d_x,
                   const mrg_controls* controls, mrg_tuning* out)
{
    return guard([&] {
        if (!batch || !d_b || !d_x) return fail(MRG_E_INVALID, "NULL argument");
        Controls k = to_controls(controls);
        if (k.ordering != batch->ordering) throw Error(MRG_E_INVALID, "controls.ordering differs from the batch's");
        prepare_batch(batch->bh, batch->meshes, k);
        for (size_t s = 0; s < batch->meshes.size(); ++s) {
            PlanState* P = batch->bh.members[s];
            if (!d_b[s] || !d_x[s]) throw Error(MRG_E_INVALID, "NULL member vector");
            P->sys.in_b = d_b[s];
            P->sys.in_x = d_x[s];
            P->sys.out_x = nullptr;
        }
        batch->bh.sync_sys();
        fill_tuning(out, tune_batch(batch->bh, k));
        MRG_CUDA(cudaStreamSynchronize(batch->ctx->st));
        return (int)MRG_OK;
    });
}

int mrg_dn_create(mrg_ctx* ctx, const mrg_dn_patch* a, const mrg_dn_patch* b, const mrg_dn_config* cfg,
                  mrg_dn** out)
{
    return guard([&] {
        if (!ctx || !a || !b || !cfg || !out) return fail(MRG_E_INVALID, "NULL argument");
        *out = nullptr;
        if (!a->src_ptr || !b->src_ptr) return fail(MRG_E_INVALID, "NULL interpolation CSR");
        std::vector<double> wa, wb;
        const double* pwa = a->src_weight;
        const double* pwb = b->src_weight;
        if (!pwa) {
            wa.assign((size_t)std::max(a->src_ptr[a->n_faces], 0), 1.0);
            pwa = wa.data();
        }
        if (!pwb) {
            wb.assign((size_t)std::max(b->src_ptr[b->n_faces], 0), 1.0);
            pwb = wb.data();
        }
        auto* d = new mrg_dn();
        try {
            d->d.reset(dn_create(&ctx->c, a->n_cells, a->n_faces, a->face_cells, a->delta_coeffs, a->k, a->area,
                                 b->n_cells, b->n_faces, b->face_cells, b->delta_coeffs, b->k, b->area, a->src_ptr,
                                 a->src_face, pwa, b->src_ptr, b->src_face, pwb, cfg->K, cfg->flux_jump,
                                 cfg->relax_model, cfg->relax, cfg->coupling_reuse));
        } catch (...) {
            delete d;
            throw;
        }
        *out = d;
        return (int)MRG_OK;
    });
}

int mrg_dn_set_flux_relaxation(mrg_dn* dn, int relax_model, double relax, int coupling_reuse)
{
    return guard([&] {
        if (!dn) return fail(MRG_E_INVALID, "NULL argument");
        dn_set_flux_relaxation(*dn->d, relax_model, relax, coupling_reuse);
        return (int)MRG_OK;
    });
}

int mrg_dn_destroy(mrg_dn* dn)
{
    return guard([&] {
        delete dn;
        return (int)MRG_OK;
    });
}

int mrg_dn_set_state(mrg_dn* dn, const double* value_a, const double* grad_b)
{
    return guard([&] {
        if (!dn || !value_a || !grad_b) return fail(MRG_E_INVALID, "NULL argument");
        dn_set_state(*dn->d, value_a, grad_b);
        return (int)MRG_OK;
    });
}

int mrg_dn_new_time_step(mrg_dn* dn)
{
    return guard([&] {
        if (!dn) return fail(MRG_E_INVALID, "NULL argument");
        dn_new_time_step(*dn->d);
        return (int)MRG_OK;
    });
}

int mrg_dn_update_jump(mrg_dn* dn, const double* d_t_b)
{
    return guard([&] {
        if (!dn || !d_t_b) return fail(MRG_E_INVALID, "NULL argument");
        dn_update_a(*dn->d, d_t_b);
        return (int)MRG_OK;
    });
}

int mrg_dn_update_flux(mrg_dn* dn, const double* d_t_a)
{
    return guard([&] {
        if (!dn || !d_t_a) return fail(MRG_E_INVALID, "NULL argument");
        dn_update_b(*dn->d, d_t_a);
        return (int)MRG_OK;
    });
}

int mrg_dn_rhs(mrg_dn* dn, int side, const double* d_b0, double* d_b)
{
    return guard([&] {
        if (!dn || !d_b0 || !d_b) return fail(MRG_E_INVALID, "NULL argument");
        if (side != 0 && side != 1) return fail(MRG_E_INVALID, "side must be 0 (A) or 1 (B)");
        dn_rhs(*dn->d, side, d_b0, d_b);
        return (int)MRG_OK;
    });
}

int mrg_dn_residuals(mrg_dn* dn, const double* d_t_a, const double* d_t_b, double* jump_res, double* flux_res)
{
    return guard([&] {
        if (!dn || !d_t_a || !d_t_b) return fail(MRG_E_INVALID, "NULL argument");
        dn_residuals(*dn->d, d_t_a, d_t_b, jump_res, flux_res);
        return (int)MRG_OK;
    });
}

int mrg_dn_get_state(mrg_dn* dn, double* value_a, double* grad_b, double* aitken)
{
    return guard([&] {
        if (!dn) return fail(MRG_E_INVALID, "NULL argument");
        dn_get_state(*dn->d, value_a, grad_b, aitken);
        return (int)MRG_OK;
    });
}

int mrg_dn_criteria(int corr, double jump_res, double flux_res, double max_jump_res, double max_flux_res)
{
    if (corr == 1) return 0;
    return (jump_res <= max_jump_res && flux_res <= max_flux_res) ? 1 : 0;
}

int mrg_mono_create(mrg_ctx* ctx, const mrg_mono_patch* a, const mrg_mono_patch* b, mrg_mono** out)
{
    return guard([&] {
        if (!ctx || !a || !b || !out) return fail(MRG_E_INVALID, "NULL argument");
        *out = nullptr;
        auto host = [](const mrg_mono_patch* p) {
            return MonoPatchHost{p->n_cells,      p->n_faces,   p->face_cells, p->weights,   p->mag_long_delta,
                                 p->delta_coeffs, p->mag_sf,    p->src_ptr,    p->src_face, p->src_weight};
        };
        auto* m = new mrg_mono();
        try {
            mono_create(m->m, &ctx->c, host(a), host(b));
        } catch (...) {
            delete m;
            throw;
        }
        *out = m;
        return (int)MRG_OK;
    });
}

int mrg_mono_destroy(mrg_mono* mono)
{
    return guard([&] {
        delete mono;
        return (int)MRG_OK;
    });
}

int mrg_mono_update(mrg_mono* mono, int side, const double* T_own, const double* T_nbr, const double* f_own,
                    const double* f_nbr, const double* Qr_own, const double* Qr_nbr, double* k, double* Tw)
{
    return guard([&] {
        if (!mono || side < 0 || side > 1) return fail(MRG_E_INVALID, "bad argument");
        if (mono->m.side[side].n_faces > 0 && (!T_own || !T_nbr || !f_own || !f_nbr || !k || !Tw))
            return fail(MRG_E_INVALID, "NULL array");
        mono_update(mono->m, side, T_own, T_nbr, f_own, f_nbr, Qr_own, Qr_nbr, k, Tw);
        MRG_CUDA(cudaStreamSynchronize(mono->m.ctx->st));
        return (int)MRG_OK;
    });
}

int mrg_mono_source(mrg_mono* mono, int side, const double* T_own, const double* T_nbr, const double* Tw,
                    const double* k, const double* f_own, double* b)
{
    return guard([&] {
        if (!mono || side < 0 || side > 1) return fail(MRG_E_INVALID, "bad argument");
        if (mono->m.side[side].n_faces > 0 && (!T_own || !T_nbr || !Tw || !k || !f_own || !b))
            return fail(MRG_E_INVALID, "NULL array");
        mono_source(mono->m, side, T_own, T_nbr, Tw, k, f_own, b);
        MRG_CUDA(cudaStreamSynchronize(mono->m.ctx->st));
        return (int)MRG_OK;
    });
}

int mrg_server_create(mrg_ctx* ctx, const mrg_controls* sym_controls, const mrg_controls* asym_controls,
                      size_t hbm_budget, int max_active, mrg_server** out)
{
    return guard([&] {
        if (!ctx || !sym_controls || !out) return fail(MRG_E_INVALID, "NULL argument");
        *out = nullptr;
        Controls sym = to_controls(sym_controls), asym;
        if (asym_controls) asym = to_controls(asym_controls);
        auto* s = new mrg_server();
        try {
            s->s.reset(new Server(&ctx->c, sym, asym_controls ? &asym : nullptr, hbm_budget, max_active));
        } catch (...) {
            delete s;
            throw;
        }
        *out = s;
        return (int)MRG_OK;
    });
}

int mrg_server_destroy(mrg_server* server)
{
    return guard([&] {
        delete server;
        return (int)MRG_OK;
    });
}

int mrg_server_submit(mrg_server* server, mrg_mesh* mesh, int asym, const double* diag, const double* upper,
                      const double* lower_or_null, const double* iface_bou, const double* iface_int_or_null,
                      const double* b, const double* x0, double* x_out, uint64_t* request_id)
{
    return guard([&] {
        if (!server || !mesh || !request_id) return fail(MRG_E_INVALID, "NULL argument");
        if (mesh->m.ni > 0 && !iface_bou) return fail(MRG_E_INVALID, "interface coefficients must not be NULL");
        *request_id = server->s->submit(&mesh->m, asym, diag, upper, lower_or_null, iface_bou, iface_int_or_null, b,
                                        x0, x_out);
        return (int)MRG_OK;
    });
}

static int server_result(int status, bool done, const Perf& p, const std::string& err, int* done_out,
                         mrg_perf* perf, double lat, double* latency_ms)
{
    if (done_out) *done_out = done ? 1 : 0;
    if (!done) return (int)MRG_OK;
    fill_perf(perf, p);
    if (latency_ms) *latency_ms = lat;
    if (status != MRG_OK) return fail(status, err.empty() ? "request failed" : err);
    return (int)MRG_OK;
}

int mrg_server_poll(mrg_server* server, uint64_t request_id, int* done, mrg_perf* perf, double* latency_ms)
{
    return guard([&] {
        if (!server || !done) return fail(MRG_E_INVALID, "NULL argument");
        bool d = false;
        Perf p;
        double lat = 0;
        std::string err;
        const int st = server->s->poll(request_id, &d, &p, &lat, &err);
        return server_result(st, d, p, err, done, perf, lat, latency_ms);
    });
}

int mrg_server_wait(mrg_server* server, uint64_t request_id, double timeout_ms, int* done, mrg_perf* perf,
                    double* latency_ms)
{
    return guard([&] {
        if (!server || !done) return fail(MRG_E_INVALID, "NULL argument");
        bool d = false;
        Perf p;
        double lat = 0;
        std::string err;
        const int st = server->s->wait(request_id, timeout_ms, &d, &p, &lat, &err);
        return server_result(st, d, p, err, done, perf, lat, latency_ms);
    });
}

int mrg_server_get_stats(mrg_server* server, mrg_server_stats* out)
{
    return guard([&] {
        if (!server || !out) return fail(MRG_E_INVALID, "NULL argument");
        const ServerStats s = server->s->stats();
        std::memset(out, 0, sizeof *out);
        out->submitted = s.submitted;
        out->completed = s.completed;
        out->running = s.running;
        out->queued = s.queued;
        out->peak_running = s.peak_running;
        out->inflight_bytes = s.inflight_bytes;
        out->peak_inflight_bytes = s.peak_inflight_bytes;
        return (int)MRG_OK;
    });
}

int mrg_residual_noalloc(int n_cells, int n_faces, const int32_t* d_lower_addr, const int32_t* d_upper_addr,
                         const int32_t* d_owner_start, const int32_t* d_losort, const int32_t* d_losort_start,
                         const double* d_diag, const double* d_upper, const double* d_lower, const double* d_b,
                         const double* d_x, void* stream, double* residual, double* norm_factor)
{
    return guard([&] {
        residual_noalloc(n_cells, n_faces, d_lower_addr, d_upper_addr, d_owner_start, d_losort, d_losort_start,
                         d_diag, d_upper, d_lower, d_b, d_x, stream, residual, norm_factor);
        return (int)MRG_OK;
    });
}

}  // extern "C"

namespace mrg {
Ggi::~Ggi()
{
    if (!ctx) return;
    for (void* p : {(void*)ptr, (void*)addr, (void*)w, (void*)d_src, (void*)d_dst}) ctx->release(p);
}
}  // namespace mrg
