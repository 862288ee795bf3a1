// blockpc.cu -- host side of the block preconditioner (PC_BLOCK): the block
// structure of a block-expanded mesh and its per-plan views.  The kernels
// (gather, factor, sweeps) are in kernels.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/mrgpu.h"
#include "blockpc.h"
#include "engine.h"
#include "kernels.h"
#include "plan.h"

namespace mrg {

std::string block_expansion(int n, int nf, const int32_t* lower, const int32_t* upper, int bs,
                            std::vector<int32_t>& s_lower, std::vector<int32_t>& s_upper, std::vector<int64_t>& src);

namespace {
template <typename T>
T* upload(Ctx* c, const std::vector<T>& v)
{
    T* d = (T*)c->alloc(std::max<size_t>(sizeof(T) * v.size(), 16));
    if (!v.empty()) MRG_CUDA(cudaMemcpyAsync(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c->st));
    return d;
}
}  // namespace

BlockHost::~BlockHost()
{
    if (!ctx) return;
    for (void* p : {(void*)d_perm, (void*)chunk_start, (void*)f_sptr, (void*)f_col, (void*)f_src, (void*)b_sptr,
                    (void*)b_col, (void*)b_src, (void*)dmap, (void*)fmap, (void*)D, (void*)U, (void*)L})
        ctx->release(p);
}

BlockView::~BlockView()
{
    if (!ctx) return;
    for (void* p : {(void*)d, (void*)vmap, (void*)dD}) ctx->release(p);
}

void set_blocks(Mesh& m, int bs, int n, int nf, const int32_t* lower, const int32_t* upper)
{
    if (bs < 1 || bs > 4) throw Error(MRG_E_INVALID, "block preconditioner: block size must be 1..4");
    if (n < 1 || nf < 0 || (nf > 0 && (!lower || !upper))) throw Error(MRG_E_INVALID, "bad block addressing");
    if ((long long)n * bs != m.n) throw Error(MRG_E_INVALID, "the mesh is not the block system's expansion (cells)");
    if (m.ni > 0) throw Error(MRG_E_INVALID, "block preconditioner: the mesh has interfaces");
    std::vector<int32_t> s_lower, s_upper;
    std::vector<int64_t> src;
    const std::string msg = block_expansion(n, nf, lower, upper, bs, s_lower, s_upper, src);
    if (!msg.empty()) throw Error(MRG_E_INVALID, "block addressing: " + msg);
    if (s_lower != m.lower || s_upper != m.upper)
        throw Error(MRG_E_INVALID, "the mesh is not the block system's expansion (faces)");
    Ctx* c = m.ctx;
    auto B = std::make_unique<BlockHost>();
    B->ctx = c;
    B->bs = bs;
    B->n = n;
    B->nf = nf;
    const long long bb = (long long)bs * bs;
    std::vector<int32_t> dmap((size_t)n * bb, 0), fmap((size_t)nf * bb, 0);
    for (int cc = 0; cc < n; ++cc)
        for (int a = 0; a < bs; ++a) dmap[cc * bb + a * bs + a] = cc * bs + a;   // diagonal rows
    for (size_t k = 0; k < src.size(); ++k) {
        const int64_t s = src[k];
        if (s < 0) {   // diagonal block (a, b), a < b: upper D[a][b], lower D[b][a]
            const int64_t q = -1 - s, cc = q / bb, a = (q % bb) / bs, b = q % bs;
            dmap[cc * bb + a * bs + b] = -1 - (int32_t)k;
            dmap[cc * bb + b * bs + a] = -1 - (int32_t)k;
        } else {
            fmap[s] = (int32_t)k;
        }
    }
    IfaceHost none;
    none.ptr.assign(1, 0);
    PlanHost P = build_plan(n, nf, lower, upper, none, 0);
    B->nchunks = P.nchunks;
    B->perm = P.perm;
    B->d_perm = upload(c, P.perm);
    B->chunk_start = upload(c, P.chunk_start);
    B->f_sptr = upload(c, P.f_sptr);
    B->f_col = upload(c, P.f_col);
    B->f_src = upload(c, P.f_src);
    B->b_sptr = upload(c, P.b_sptr);
    B->b_col = upload(c, P.b_col);
    B->b_src = upload(c, P.b_src);
    B->dmap = upload(c, dmap);
    B->fmap = upload(c, fmap);
    B->D = (double*)c->alloc(8 * (size_t)std::max<long long>(n * bb, 1));
    B->U = (double*)c->alloc(8 * (size_t)std::max<long long>(nf * bb, 1));
    B->L = (double*)c->alloc(8 * (size_t)std::max<long long>(nf * bb, 1));
    MRG_CUDA(cudaStreamSynchronize(c->st));
    for (auto& v : m.bviews) v.reset();
    m.blocks = std::move(B);
}

BlockView& block_view(Mesh& m, PlanState& P)
{
    if (!m.blocks) throw Error(MRG_E_INVALID, "block preconditioner: the mesh has no block structure "
                                              "(mrg_mesh_set_blocks)");
    const int o = P.host.ordering;
    if (m.bviews[o]) return *m.bviews[o];
    BlockHost& B = *m.blocks;
    Ctx* c = m.ctx;
    auto V = std::make_unique<BlockView>();
    V->ctx = c;
    // (internal cell, component) -> the plan's internal scalar row
    std::vector<int32_t> sperm(m.n), siperm(m.n);
    MRG_CUDA(cudaMemcpy(sperm.data(), P.perm, 4 * (size_t)m.n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < m.n; ++i) siperm[sperm[i]] = i;
    std::vector<int32_t> vmap((size_t)B.n * B.bs);
    for (int i = 0; i < B.n; ++i)
        for (int a = 0; a < B.bs; ++a) vmap[(size_t)i * B.bs + a] = siperm[B.perm[i] * B.bs + a];
    V->vmap = upload(c, vmap);
    V->dD = (double*)c->alloc(8 * (size_t)B.n * B.bs * B.bs);
    BlockDev& h = V->h;
    h.bs = B.bs;
    h.n = B.n;
    h.nf = B.nf;
    h.nchunks = B.nchunks;
    h.perm = B.d_perm;
    h.chunk_start = B.chunk_start;
    h.f_sptr = B.f_sptr;
    h.f_col = B.f_col;
    h.f_src = B.f_src;
    h.b_sptr = B.b_sptr;
    h.b_col = B.b_col;
    h.b_src = B.b_src;
    h.dmap = B.dmap;
    h.fmap = B.fmap;
    h.D = B.D;
    h.U = B.U;
    h.L = B.L;
    h.dD = V->dD;
    h.vmap = V->vmap;
    h.sym = m.sym ? 1 : 0;
    V->d = (BlockDev*)c->alloc(sizeof(BlockDev));
    MRG_CUDA(cudaMemcpyAsync(V->d, &h, sizeof(BlockDev), cudaMemcpyHostToDevice, c->st));
    MRG_CUDA(cudaStreamSynchronize(c->st));
    m.bviews[o] = std::move(V);
    return *m.bviews[o];
}

}  // namespace mrg
