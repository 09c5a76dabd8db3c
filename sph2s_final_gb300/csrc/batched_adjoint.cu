// batched_adjoint.cu -- differentiable rollout of every scene of a batch at
// once (no counterpart in the reference).
//
// The single-scale rollout (adjoint.cu) restated over the batch's packed
// arrays: one forward with checkpoints every K steps, one Poly6-splat loss per
// scene on its own node grid, and one reverse pass that recomputes each
// segment into a tape and runs the adjoint kernels backwards.  Every kernel
// walks the batch's 256-particle tiles, so a block's scene constants (grid
// tables, P, viscosity) are uniform and the per-particle code is the
// single-scale adjoint's (adj_force_one, adj_density_one, splat_node,
// splat_grad_one).  The viscosity gradient is reduced per tile in the same
// fixed order as the single-scale per-block partials and summed per scene in
// tile order, so each scene's loss, field and gradients are the single-scale
// solver's bit for bit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "adjoint_kernels.cuh"
#include "batched_solver.h"
#include "errors.h"
#include "host_params.h"

using namespace sph;
using namespace sph_b;

namespace sph {

struct BRollout {
    int T = 0, K = 0;
    float dt = 0.0f;
    std::vector<void*> owned;
    std::vector<float4*> ck_pos, ck_vel;
    std::vector<uint32_t*> perm;
    std::vector<float4*> xh, vh;
    std::vector<float*> rho;
    std::vector<float2*> aux;
    std::vector<uint4*> nbr;
    std::vector<uint32_t*> cnt;
    std::vector<uint2*> cells;
    float4 *gx = nullptr, *gv = nullptr, *gx2 = nullptr, *gv2 = nullptr, *lam = nullptr;
    float4* gxT = nullptr;
    float* grho = nullptr;
    float* gmu_part = nullptr;  // one partial per 256-particle tile
    double* gmu_acc = nullptr;  // per scene
    float* mu = nullptr;        // per scene
    uint32_t *tfirst = nullptr, *tcount = nullptr;
    bool forward_done = false, have_loss = false;
};

// Node grid of one scene's density loss; off = first node in the packed field.
struct NodeRec {
    GridParams ng;
    uint32_t off, nn;
    float scale;  // 2 / nn * 6 m C6
};

}  // namespace sph

namespace {

constexpr int kTile = 256;

static __global__ void __launch_bounds__(kTile) b_adj_force_kernel(
    const uint2* __restrict__ tiles, uint32_t num_tiles, const SceneRec* __restrict__ recs,
    const float* __restrict__ mu_s, const float4* __restrict__ pos, const float4* __restrict__ vel,
    const float* __restrict__ rho, const float2* __restrict__ aux, const uint4* __restrict__ nbr4,
    const uint32_t* __restrict__ cnt, const uint2* __restrict__ cells,
    const float4* __restrict__ bpos, const uint2* __restrict__ bcells,
    const uint8_t* __restrict__ bnear, const uint32_t* __restrict__ bstart,
    const uint32_t* __restrict__ bcand, uint32_t n, uint32_t nb, float dt,
    const float4* __restrict__ lam, const float4* __restrict__ gx_in,
    const float4* __restrict__ gv_in, float4* __restrict__ gx_out, float4* __restrict__ gv_out,
    float* __restrict__ grho, float* __restrict__ gmu_tile) {
    for (uint32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
        const uint2 tile = tiles[t];
        const SceneRec& R = recs[tile.x];
        const uint32_t i = tile.y + threadIdx.x;
        float g = 0.0f;
        if (i < R.p_off + R.p_n) {
            const SimParams P = R.P;
            g = adj_force_one(i, pos, vel, rho, aux, nbr4, cnt, cells + R.c_off, bpos,
                              bcells + R.c_off, bnear + R.c_off, bstart + R.c_off, bcand, n, nb,
                              P, mu_s[tile.x], dt, lam,
                              gx_in, gv_in, gx_out, gv_out, grho);
        }
        const float s = block_sum_fixed(g);
        if (threadIdx.x == 0) gmu_tile[t] = s;
    }
}

static __global__ void __launch_bounds__(kTile) b_adj_density_kernel(
    const uint2* __restrict__ tiles, uint32_t num_tiles, const SceneRec* __restrict__ recs,
    const float4* __restrict__ pos, const uint4* __restrict__ nbr4, const uint32_t* __restrict__ cnt,
    const uint2* __restrict__ cells, uint32_t n, const float* __restrict__ grho,
    float4* __restrict__ gx) {
    for (uint32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
        const uint2 tile = tiles[t];
        const SceneRec& R = recs[tile.x];
        const uint32_t i = tile.y + threadIdx.x;
        if (i >= R.p_off + R.p_n) continue;
        const SimParams P = R.P;
        adj_density_one(i, pos, nbr4, cnt, cells + R.c_off, n, P, grho, gx);
    }
}

// d L_s / d mu_s: the scene's tile partials in tile order (the single-scale
// adj_sum_kernel's order over its blocks).
static __global__ void b_adj_sum_kernel(const float* __restrict__ part,
                                        const uint32_t* __restrict__ first,
                                        const uint32_t* __restrict__ count, uint32_t S,
                                        double* __restrict__ acc) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    double sum = 0.0;
    for (uint32_t k = 0; k < count[s]; ++k) sum += (double)part[first[s] + k];
    acc[s] += sum;
}

// tiles[t] = (scene, first node of the tile within the scene's node grid)
static __global__ void __launch_bounds__(kTile) b_splat_kernel(
    const uint2* __restrict__ tiles, uint32_t num_tiles, const SceneRec* __restrict__ recs,
    const NodeRec* __restrict__ nodes, const float4* __restrict__ pos,
    const uint2* __restrict__ cells, uint32_t n, float* __restrict__ field) {
    for (uint32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
        const uint2 tile = tiles[t];
        const NodeRec& Q = nodes[tile.x];
        const uint32_t c = tile.y + threadIdx.x;
        if (c >= Q.nn) continue;
        const SceneRec& R = recs[tile.x];
        const SimParams P = R.P;
        const GridParams ng = Q.ng;
        field[Q.off + c] = splat_node(c, pos, cells + R.c_off, n, P, ng);
    }
}

static __global__ void __launch_bounds__(kTile) b_splat_grad_kernel(
    const uint2* __restrict__ tiles, uint32_t num_tiles, const SceneRec* __restrict__ recs,
    const NodeRec* __restrict__ nodes, const float4* __restrict__ pos,
    const float* __restrict__ err, float4* __restrict__ gx) {
    for (uint32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
        const uint2 tile = tiles[t];
        const SceneRec& R = recs[tile.x];
        const uint32_t i = tile.y + threadIdx.x;
        if (i >= R.p_off + R.p_n) continue;
        const NodeRec& Q = nodes[tile.x];
        const SimParams P = R.P;
        const GridParams ng = Q.ng;
        gx[i] = splat_grad_one(i, pos, P, ng, err + Q.off, Q.scale);
    }
}

template <class T>
int ralloc(BRollout* r, T** p, size_t count) {
    SPH_CUDA(cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)));
    r->owned.push_back(*p);
    return SPH_OK;
}

void free_brollout(BRollout* r) {
    if (!r) return;
    for (void* p : r->owned) cudaFree(p);
    delete r;
}

int alloc_brollout(sph_batch* b, int T, int K, BRollout** out) {
    BRollout* r = new BRollout();
    r->T = T;
    r->K = K;
    const uint32_t N = b->N;
    const int nseg = (T + K - 1) / K;
    int rc = SPH_OK;
    r->ck_pos.resize(nseg);
    r->ck_vel.resize(nseg);
    for (int c = 0; c < nseg && rc == SPH_OK; ++c) {
        rc = ralloc(r, &r->ck_pos[c], N);
        if (rc == SPH_OK) rc = ralloc(r, &r->ck_vel[c], N);
    }
    r->perm.resize(K);
    r->xh.resize(K);
    r->vh.resize(K);
    r->rho.resize(K);
    r->aux.resize(K);
    r->nbr.resize(K);
    r->cnt.resize(K);
    r->cells.resize(K);
    for (int k = 0; k < K && rc == SPH_OK; ++k) {
        if ((rc = ralloc(r, &r->perm[k], N)) || (rc = ralloc(r, &r->xh[k], N)) ||
            (rc = ralloc(r, &r->vh[k], N)) || (rc = ralloc(r, &r->rho[k], N)) ||
            (rc = ralloc(r, &r->aux[k], N)) ||
            (rc = ralloc(r, &r->nbr[k], (size_t)N * (kMaxNbr / 4))) ||
            (rc = ralloc(r, &r->cnt[k], N)) || (rc = ralloc(r, &r->cells[k], b->NC)))
            break;
    }
    if (rc == SPH_OK &&
        ((rc = ralloc(r, &r->gx, N)) || (rc = ralloc(r, &r->gv, N)) || (rc = ralloc(r, &r->gx2, N)) ||
         (rc = ralloc(r, &r->gv2, N)) || (rc = ralloc(r, &r->lam, N)) || (rc = ralloc(r, &r->gxT, N)) ||
         (rc = ralloc(r, &r->grho, N)) || (rc = ralloc(r, &r->gmu_part, b->ntiles[1])) ||
         (rc = ralloc(r, &r->gmu_acc, b->S)) || (rc = ralloc(r, &r->mu, b->S)) ||
         (rc = ralloc(r, &r->tfirst, b->S)) || (rc = ralloc(r, &r->tcount, b->S)))) {
    }
    if (rc == SPH_OK) {
        std::vector<uint32_t> cnt(b->S);
        for (uint32_t s = 0; s < b->S; ++s) cnt[s] = (b->recs_h[s].p_n + kTile - 1) / kTile;
        cudaError_t e = cudaMemcpy(r->tfirst, b->tile_first.data(), 4 * (size_t)b->S, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(r->tcount, cnt.data(), 4 * (size_t)b->S, cudaMemcpyHostToDevice);
        rc = check_cuda(e, "rollout tables", __FILE__, __LINE__);
    }
    if (rc != SPH_OK) {
        std::string m = sph_last_error();
        free_brollout(r);
        return fail(rc, m);
    }
    *out = r;
    return SPH_OK;
}

uint32_t tile_grid(const sph_batch* b, uint32_t tiles) { return pgrid(b, tiles); }

}  // namespace

void sphb_rollout_release(sph_batch* b) {
    if (b && b->rollout) {
        free_brollout(b->rollout);
        b->rollout = nullptr;
    }
}

extern "C" {

int sphb_rollout_forward(sph_batch* b, const float* v0_xyz, const float* viscosity, float dt,
                         int32_t steps, int32_t checkpoint_every) {
    if (!b) return fail(SPH_E_INVALID, "sphb_rollout_forward: NULL handle");
    if (steps < 1 || checkpoint_every < 1 || !(dt > 0.0f))
        return fail(SPH_E_INVALID, "sphb_rollout_forward: need steps >= 1, checkpoint_every >= 1, dt > 0");
    if (b->N == 0) return fail(SPH_E_INVALID, "sphb_rollout_forward: no fluid particles");
    if (viscosity)
        for (uint32_t s = 0; s < b->S; ++s)
            if (!(viscosity[s] >= 0.0f))
                return fail(SPH_E_INVALID, "sphb_rollout_forward: viscosity must be >= 0");
    const int K = checkpoint_every > steps ? steps : checkpoint_every;
    if (b->rollout && (b->rollout->T != steps || b->rollout->K != K)) sphb_rollout_release(b);
    if (!b->rollout) {
        int rc = alloc_brollout(b, steps, K, &b->rollout);
        if (rc != SPH_OK) return rc;
    }
    BRollout* r = b->rollout;
    r->dt = dt;
    r->forward_done = r->have_loss = false;
    SPH_CUDA(cudaStreamSynchronize(b->stream));
    if (viscosity)
        for (uint32_t s = 0; s < b->S; ++s) b->cfgs[s].viscosity = viscosity[s];
    int rc = refresh_scene_params(b);
    if (rc != SPH_OK) return rc;
    std::vector<float> mu(b->S);
    for (uint32_t s = 0; s < b->S; ++s) mu[s] = b->cfgs[s].viscosity;
    SPH_CUDA(cudaMemcpy(r->mu, mu.data(), 4 * (size_t)b->S, cudaMemcpyHostToDevice));
    // restart from the creation positions with v0
    const uint32_t N = b->N;
    SPH_CUDA(cudaMemcpyAsync(b->pos, b->pos0, 16 * (size_t)N, cudaMemcpyDeviceToDevice, b->stream));
    std::vector<float4> hv(N);
    for (uint32_t i = 0; i < N; ++i)
        hv[i] = v0_xyz ? make_float4(v0_xyz[3 * (size_t)i], v0_xyz[3 * (size_t)i + 1],
                                     v0_xyz[3 * (size_t)i + 2], 0.f)
                       : make_float4(0.f, 0.f, 0.f, 0.f);
    SPH_CUDA(cudaMemcpyAsync(b->vel, hv.data(), 16 * (size_t)N, cudaMemcpyHostToDevice, b->stream));
    const int nseg = (steps + K - 1) / K;
    for (int c = 0; c < nseg; ++c) {
        SPH_CUDA(cudaMemcpyAsync(r->ck_pos[c], b->pos, 16 * (size_t)N, cudaMemcpyDeviceToDevice, b->stream));
        SPH_CUDA(cudaMemcpyAsync(r->ck_vel[c], b->vel, 16 * (size_t)N, cudaMemcpyDeviceToDevice, b->stream));
        rc = sphb_advance(b, dt, std::min(K, steps - c * K));
        if (rc != SPH_OK) return rc;
    }
    rc = sphb_sync(b);
    if (rc != SPH_OK) return rc;
    r->forward_done = true;
    return SPH_OK;
}

int sphb_rollout_density_loss(sph_batch* b, const sph_grid* nodes, const float* target,
                              float* field, double* loss) {
    if (!b || !nodes) return fail(SPH_E_INVALID, "sphb_rollout_density_loss: NULL argument");
    std::vector<NodeRec> nr(b->S);
    std::vector<uint2> ntiles;
    uint64_t total = 0;
    for (uint32_t s = 0; s < b->S; ++s) {
        int rc = validate_grid(nodes[s], "sphb_rollout_density_loss");
        if (rc != SPH_OK) return rc;
        NodeRec& Q = nr[s];
        Q.ng = make_grid_params(nodes[s]);
        Q.nn = sph_grid_num_cells(&nodes[s]);
        Q.off = (uint32_t)total;
        Q.scale = (float)(2.0 / (double)Q.nn * 6.0 * (double)b->recs_h[s].P.dens_coef);
        for (uint32_t c = 0; c < Q.nn; c += kTile) ntiles.push_back(make_uint2(s, c));
        total += Q.nn;
    }
    if (total > 0xFFFFFFF0ull) return fail(SPH_E_CAPACITY, "sphb_rollout_density_loss: too many nodes");
    const uint32_t NN = (uint32_t)total;
    SPH_CUDA(cudaStreamSynchronize(b->stream));
    NodeRec* d_nr = nullptr;
    uint2* d_nt = nullptr;
    float *d_field = nullptr, *d_err = nullptr;
    float4* d_gs = nullptr;
    cudaError_t e = cudaMalloc(&d_nr, sizeof(NodeRec) * b->S);
    if (e == cudaSuccess) e = cudaMalloc(&d_nt, sizeof(uint2) * std::max<size_t>(ntiles.size(), 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_field, 4 * (size_t)std::max(NN, 1u));
    if (e == cudaSuccess) e = cudaMalloc(&d_err, 4 * (size_t)std::max(NN, 1u));
    if (e == cudaSuccess) e = cudaMalloc(&d_gs, 16 * (size_t)std::max(b->N, 1u));
    if (e == cudaSuccess) e = cudaMemcpy(d_nr, nr.data(), sizeof(NodeRec) * b->S, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !ntiles.empty())
        e = cudaMemcpy(d_nt, ntiles.data(), sizeof(uint2) * ntiles.size(), cudaMemcpyHostToDevice);
    std::vector<float> hf(NN);
    int out = 0;
    if (e == cudaSuccess) {
        if (b->N) out = enqueue_neighborhood(b);
        const uint32_t nt = (uint32_t)ntiles.size();
        if (nt)
            b_splat_kernel<<<tile_grid(b, nt), kTile, 0, b->stream>>>(d_nt, nt, b->recs, d_nr,
                                                                    b->spos, b->cells, b->N, d_field);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && NN) e = cudaMemcpyAsync(hf.data(), d_field, 4 * (size_t)NN, cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess && field && NN) std::memcpy(field, hf.data(), 4 * (size_t)NN);
    if (e == cudaSuccess && target) {
        std::vector<float> err(NN);
        for (uint32_t s = 0; s < b->S; ++s) {
            double L = 0.0;
            for (uint32_t k = 0; k < nr[s].nn; ++k) {
                const uint32_t q = nr[s].off + k;
                const double d = (double)hf[q] - (double)target[q];
                err[q] = (float)d;
                L += d * d;
            }
            if (loss) loss[s] = nr[s].nn ? L / (double)nr[s].nn : 0.0;
        }
        if (NN) e = cudaMemcpyAsync(d_err, err.data(), 4 * (size_t)NN, cudaMemcpyHostToDevice, b->stream);
        if (e == cudaSuccess && b->rollout && b->N) {
            b_splat_grad_kernel<<<tile_grid(b, b->ntiles[1]), kTile, 0, b->stream>>>(
                b->tiles[1], b->ntiles[1], b->recs, d_nr, b->spos, d_err, d_gs);
            adj_unpermute_kernel<<<(b->N + kTile - 1) / kTile, kTile, 0, b->stream>>>(
                b->vals[out], b->N, d_gs, d_gs, b->rollout->gxT, b->rollout->gx2);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
            if (e == cudaSuccess) b->rollout->have_loss = true;
        }
    }
    cudaFree(d_nr);
    cudaFree(d_nt);
    cudaFree(d_field);
    cudaFree(d_err);
    cudaFree(d_gs);
    SPH_CUDA(e);
    return check_err(b);
}

int sphb_rollout_backward(sph_batch* b, float* grad_v0, float* grad_x0, double* grad_mu) {
    if (!b || !b->rollout) return fail(SPH_E_INVALID, "sphb_rollout_backward: no rollout");
    BRollout* r = b->rollout;
    if (!r->forward_done || !r->have_loss)
        return fail(SPH_E_INVALID, "sphb_rollout_backward: run the forward and the loss first");
    const uint32_t N = b->N;
    cudaStream_t st = b->stream;
    const int nseg = (r->T + r->K - 1) / r->K;
    SPH_CUDA(cudaMemcpyAsync(r->gx, r->gxT, 16 * (size_t)N, cudaMemcpyDeviceToDevice, st));
    SPH_CUDA(cudaMemsetAsync(r->gv, 0, 16 * (size_t)N, st));
    SPH_CUDA(cudaMemsetAsync(r->gmu_acc, 0, 8 * (size_t)b->S, st));
    // the step's own buffers, redirected into the tape while recording
    float4 *spos0 = b->spos, *svel0 = b->svel;
    float* rho0 = b->rho;
    float2* aux0 = b->aux;
    uint4* nbr0 = b->nbr;
    uint32_t* cnt0 = b->nbr_count;
    uint2* cells0 = b->cells;
    const uint32_t blocks = (N + kTile - 1) / kTile;
    const uint32_t nt = b->ntiles[1];
    const uint32_t grid = tile_grid(b, nt);
    for (int c = nseg - 1; c >= 0; --c) {
        const int t0 = c * r->K, len = std::min(r->K, r->T - t0);
        SPH_CUDA(cudaMemcpyAsync(b->pos, r->ck_pos[c], 16 * (size_t)N, cudaMemcpyDeviceToDevice, st));
        SPH_CUDA(cudaMemcpyAsync(b->vel, r->ck_vel[c], 16 * (size_t)N, cudaMemcpyDeviceToDevice, st));
        for (int k = 0; k < len; ++k) {  // recompute the segment, recording the tape
            b->spos = r->xh[k];
            b->svel = r->vh[k];
            b->cells = r->cells[k];
            b->rho = r->rho[k];
            b->aux = r->aux[k];
            b->nbr = r->nbr[k];
            b->nbr_count = r->cnt[k];
            const int out = enqueue_neighborhood(b);
            cudaMemcpyAsync(r->perm[k], b->vals[out], 4 * (size_t)N, cudaMemcpyDeviceToDevice, st);
            enqueue_density(b);
            enqueue_force(b, r->dt);
        }
        b->spos = spos0;
        b->svel = svel0;
        b->cells = cells0;
        b->rho = rho0;
        b->aux = aux0;
        b->nbr = nbr0;
        b->nbr_count = cnt0;
        for (int k = len - 1; k >= 0; --k) {  // reverse through the segment
            adj_lambda_kernel<<<blocks, kTile, 0, st>>>(r->gx, r->gv, N, r->dt, r->lam);
            b_adj_force_kernel<<<grid, kTile, 0, st>>>(
                b->tiles[1], nt, b->recs, r->mu, r->xh[k], r->vh[k], r->rho[k], r->aux[k],
                r->nbr[k], r->cnt[k], r->cells[k], b->bpos, b->bcells, b->bnear, b->bstart,
                b->bcand, N, b->NB, r->dt,
                r->lam, r->gx, r->gv, r->gx2, r->gv2, r->grho, r->gmu_part);
            b_adj_sum_kernel<<<(b->S + 127) / 128, 128, 0, st>>>(r->gmu_part, r->tfirst, r->tcount,
                                                                b->S, r->gmu_acc);
            b_adj_density_kernel<<<grid, kTile, 0, st>>>(b->tiles[1], nt, b->recs, r->xh[k],
                                                         r->nbr[k], r->cnt[k], r->cells[k], N,
                                                         r->grho, r->gx2);
            adj_unpermute_kernel<<<blocks, kTile, 0, st>>>(r->perm[k], N, r->gx2, r->gv2, r->gx, r->gv);
        }
        SPH_CUDA(cudaGetLastError());
    }
    std::vector<float4> hg(N);
    std::vector<double> gm(b->S);
    SPH_CUDA(cudaMemcpyAsync(gm.data(), r->gmu_acc, 8 * (size_t)b->S, cudaMemcpyDeviceToHost, st));
    for (int which = 0; which < 2; ++which) {
        float* dst = which == 0 ? grad_v0 : grad_x0;
        if (!dst) continue;
        SPH_CUDA(cudaMemcpyAsync(hg.data(), which == 0 ? r->gv : r->gx, 16 * (size_t)N,
                                 cudaMemcpyDeviceToHost, st));
        SPH_CUDA(cudaStreamSynchronize(st));
        for (uint32_t i = 0; i < N; ++i) {
            dst[3 * (size_t)i] = hg[i].x;
            dst[3 * (size_t)i + 1] = hg[i].y;
            dst[3 * (size_t)i + 2] = hg[i].z;
        }
    }
    SPH_CUDA(cudaStreamSynchronize(st));
    if (grad_mu) std::memcpy(grad_mu, gm.data(), 8 * (size_t)b->S);
    return check_err(b);
}

}  // extern "C"
