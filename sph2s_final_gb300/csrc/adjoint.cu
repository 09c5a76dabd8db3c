// adjoint.cu -- differentiable rollout of the single-scale step (no
// counterpart in the reference).
//
// Forward: from the creation positions and given initial velocities and
// viscosity, T steps; the state is checkpointed every K steps.
// Loss: L = mean_n (G_n - target_n)^2, G the Poly6 splat of the final
// positions on the cell centres of a node grid.
// Backward: segment by segment, latest first: the segment is recomputed from
// its checkpoint while the step's own buffers are redirected into a tape
// (sort permutation, sorted positions and velocities, densities, neighbour
// lists), then the hand-written adjoint kernels run backwards through it,
// holding the neighbour structure of every step constant.  Memory is one
// segment of tape (~310 bytes per particle per step) plus T/K checkpoints.
#include <cmath>
#include <cstring>
#include <vector>
#include "adjoint_kernels.cuh"
#include "errors.h"
#include "host_params.h"
#include "single_scale_kernels.cuh"
#include "single_scale_solver.h"

using namespace sph;
using namespace sph_ss;

namespace sph {

struct Rollout {
    int T = 0, K = 0;
    float dt = 0.0f, mu = 0.0f;
    uint32_t n = 0, ncells = 0;
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
    float* gmu_part = nullptr;
    double* gmu_acc = nullptr;
    bool forward_done = false, have_loss = false;
};

}  // namespace sph

namespace {

template <class T>
int ralloc(Rollout* r, T** p, size_t count) {
    SPH_CUDA(cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)));
    r->owned.push_back(*p);
    return SPH_OK;
}

void free_rollout(Rollout* r) {
    if (!r) return;
    for (void* p : r->owned) cudaFree(p);
    delete r;
}

int alloc_rollout(sph_solver* s, int T, int K, Rollout** out) {
    Rollout* r = new Rollout();
    r->T = T;
    r->K = K;
    r->n = s->n;
    r->ncells = s->ncells;
    const int nseg = (T + K - 1) / K;
    const uint32_t n = s->n;
    int rc = SPH_OK;
    r->ck_pos.resize(nseg);
    r->ck_vel.resize(nseg);
    for (int c = 0; c < nseg && rc == SPH_OK; ++c) {
        rc = ralloc(r, &r->ck_pos[c], n);
        if (rc == SPH_OK) rc = ralloc(r, &r->ck_vel[c], n);
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
        if ((rc = ralloc(r, &r->perm[k], n)) || (rc = ralloc(r, &r->xh[k], n)) ||
            (rc = ralloc(r, &r->vh[k], n)) || (rc = ralloc(r, &r->rho[k], n)) ||
            (rc = ralloc(r, &r->aux[k], n)) || (rc = ralloc(r, &r->nbr[k], (size_t)n * (kMaxNbr / 4))) ||
            (rc = ralloc(r, &r->cnt[k], n)) || (rc = ralloc(r, &r->cells[k], s->ncells)))
            break;
    }
    const uint32_t blocks = blocks_for(n);
    if (rc == SPH_OK &&
        ((rc = ralloc(r, &r->gx, n)) || (rc = ralloc(r, &r->gv, n)) || (rc = ralloc(r, &r->gx2, n)) ||
         (rc = ralloc(r, &r->gv2, n)) || (rc = ralloc(r, &r->lam, n)) || (rc = ralloc(r, &r->gxT, n)) ||
         (rc = ralloc(r, &r->grho, n)) || (rc = ralloc(r, &r->gmu_part, blocks)) ||
         (rc = ralloc(r, &r->gmu_acc, 1)))) {
    }
    if (rc != SPH_OK) {
        std::string m = sph_last_error();
        free_rollout(r);
        return fail(rc, m);
    }
    *out = r;
    return SPH_OK;
}

// Resets the solver to its creation positions with velocities v0 (creation
// order, host, NULL = zero).
int reset_state(sph_solver* s, const float* v0) {
    SPH_CUDA(cudaMemcpyAsync(s->pos, s->pos0, 16 * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream));
    std::vector<float4> hv(s->n);
    for (uint32_t i = 0; i < s->n; ++i)
        hv[i] = v0 ? make_float4(v0[3 * i], v0[3 * i + 1], v0[3 * i + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    SPH_CUDA(cudaMemcpyAsync(s->vel, hv.data(), 16 * (size_t)s->n, cudaMemcpyHostToDevice, s->stream));
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    return SPH_OK;
}

int set_viscosity(sph_solver* s, float mu) {
    if (s->cfg.viscosity == mu) return SPH_OK;
    sph_config c = s->cfg;
    c.viscosity = mu;
    SimParams P;
    int rc = make_sim_params(c, &P);
    if (rc != SPH_OK) return rc;
    s->cfg = c;
    s->P = P;
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    return SPH_OK;
}

}  // namespace

void sph_rollout_release(sph_solver* s) {
    if (s && s->rollout) {
        free_rollout(s->rollout);
        s->rollout = nullptr;
    }
}

extern "C" {

int sph_rollout_forward(sph_solver* s, const float* v0_xyz, float viscosity, float dt,
                        int32_t steps, int32_t checkpoint_every) {
    if (!s) return fail(SPH_E_INVALID, "sph_rollout_forward: NULL handle");
    if (steps < 1 || checkpoint_every < 1 || !(dt > 0.0f) || !(viscosity >= 0.0f))
        return fail(SPH_E_INVALID, "sph_rollout_forward: need steps >= 1, checkpoint_every >= 1, dt > 0");
    if (s->n == 0) return fail(SPH_E_INVALID, "sph_rollout_forward: no fluid particles");
    const int K = checkpoint_every > steps ? steps : checkpoint_every;
    if (s->rollout && (s->rollout->T != steps || s->rollout->K != K)) sph_rollout_release(s);
    if (!s->rollout) {
        int rc = alloc_rollout(s, steps, K, &s->rollout);
        if (rc != SPH_OK) return rc;
    }
    Rollout* r = s->rollout;
    r->dt = dt;
    r->mu = viscosity;
    r->forward_done = r->have_loss = false;
    int rc = set_viscosity(s, viscosity);
    if (rc != SPH_OK) return rc;
    rc = reset_state(s, v0_xyz);
    if (rc != SPH_OK) return rc;
    const int nseg = (steps + K - 1) / K;
    for (int c = 0; c < nseg; ++c) {
        SPH_CUDA(cudaMemcpyAsync(r->ck_pos[c], s->pos, 16 * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream));
        SPH_CUDA(cudaMemcpyAsync(r->ck_vel[c], s->vel, 16 * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream));
        const int len = std::min(K, steps - c * K);
        rc = sph_advance(s, dt, len);
        if (rc != SPH_OK) return rc;
    }
    rc = sph_sync(s);
    if (rc != SPH_OK) return rc;
    r->forward_done = true;
    return SPH_OK;
}

int sph_rollout_density_loss(sph_solver* s, const sph_grid* nodes, const float* target,
                             float* field, double* loss) {
    if (!s || !nodes) return fail(SPH_E_INVALID, "sph_rollout_density_loss: NULL argument");
    int rc = validate_grid(*nodes, "sph_rollout_density_loss");
    if (rc != SPH_OK) return rc;
    const uint32_t nn = sph_grid_num_cells(nodes);
    const GridParams ng = make_grid_params(*nodes);
    float* d_field = nullptr;
    float* d_err = nullptr;
    float4* d_gs = nullptr;
    SPH_CUDA(cudaMalloc(&d_field, 4 * (size_t)nn));
    SPH_CUDA(cudaMalloc(&d_err, 4 * (size_t)nn));
    SPH_CUDA(cudaMalloc(&d_gs, 16 * (size_t)std::max(s->n, 1u)));
    cudaError_t e = cudaSuccess;
    std::vector<float> hf(nn);
    int out = 0;
    if (s->n) out = enqueue_neighborhood(s);
    splat_kernel<<<blocks_for(nn), 256, 0, s->stream>>>(s->spos, s->cells, s->n, s->P, ng, d_field);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hf.data(), d_field, 4 * (size_t)nn, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess && field) std::memcpy(field, hf.data(), 4 * (size_t)nn);
    if (e == cudaSuccess && target) {
        double L = 0.0;
        std::vector<float> err(nn);
        for (uint32_t k = 0; k < nn; ++k) {
            const double d = (double)hf[k] - (double)target[k];
            err[k] = (float)d;
            L += d * d;
        }
        L /= (double)nn;
        if (loss) *loss = L;
        e = cudaMemcpyAsync(d_err, err.data(), 4 * (size_t)nn, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess && s->rollout && s->n) {
            const float scale = (float)(2.0 / (double)nn * 6.0 * (double)s->P.dens_coef);
            splat_grad_kernel<<<blocks_for(s->n), 256, 0, s->stream>>>(s->spos, s->n, s->P, ng,
                                                                       d_err, scale, d_gs);
            adj_unpermute_kernel<<<blocks_for(s->n), 256, 0, s->stream>>>(
                s->vals[out], s->n, d_gs, d_gs, s->rollout->gxT, s->rollout->gx2);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            if (e == cudaSuccess) s->rollout->have_loss = true;
        }
    }
    cudaFree(d_field);
    cudaFree(d_err);
    cudaFree(d_gs);
    SPH_CUDA(e);
    return check_device_error(s);
}

int sph_rollout_backward(sph_solver* s, float* grad_v0, float* grad_x0, double* grad_mu) {
    if (!s || !s->rollout) return fail(SPH_E_INVALID, "sph_rollout_backward: no rollout");
    Rollout* r = s->rollout;
    if (!r->forward_done || !r->have_loss)
        return fail(SPH_E_INVALID, "sph_rollout_backward: run the forward and the loss first");
    const uint32_t n = s->n;
    cudaStream_t st = s->stream;
    const int nseg = (r->T + r->K - 1) / r->K;
    SPH_CUDA(cudaMemcpyAsync(r->gx, r->gxT, 16 * (size_t)n, cudaMemcpyDeviceToDevice, st));
    SPH_CUDA(cudaMemsetAsync(r->gv, 0, 16 * (size_t)n, st));
    SPH_CUDA(cudaMemsetAsync(r->gmu_acc, 0, 8, st));
    // the step's own buffers, redirected into the tape while recording
    float4 *spos0 = s->spos, *svel0 = s->svel;
    float* rho0 = s->rho;
    float2* aux0 = s->aux;
    uint4* nbr0 = s->nbr;
    uint32_t* cnt0 = s->nbr_count;
    uint2* cells0 = s->cells;
    const uint32_t blocks = blocks_for(n);
    for (int c = nseg - 1; c >= 0; --c) {
        const int t0 = c * r->K, len = std::min(r->K, r->T - t0);
        SPH_CUDA(cudaMemcpyAsync(s->pos, r->ck_pos[c], 16 * (size_t)n, cudaMemcpyDeviceToDevice, st));
        SPH_CUDA(cudaMemcpyAsync(s->vel, r->ck_vel[c], 16 * (size_t)n, cudaMemcpyDeviceToDevice, st));
        for (int k = 0; k < len; ++k) {  // recompute the segment, recording the tape
            s->spos = r->xh[k];
            s->svel = r->vh[k];
            s->cells = r->cells[k];
            s->rho = r->rho[k];
            s->aux = r->aux[k];
            s->nbr = r->nbr[k];
            s->nbr_count = r->cnt[k];
            const int out = enqueue_neighborhood(s);
            cudaMemcpyAsync(r->perm[k], s->vals[out], 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
            enqueue_density(s);
            enqueue_force(s, r->dt);
        }
        s->spos = spos0;
        s->svel = svel0;
        s->cells = cells0;
        s->rho = rho0;
        s->aux = aux0;
        s->nbr = nbr0;
        s->nbr_count = cnt0;
        for (int k = len - 1; k >= 0; --k) {  // reverse through the segment
            adj_lambda_kernel<<<blocks, 256, 0, st>>>(r->gx, r->gv, n, r->dt, r->lam);
            adj_force_kernel<<<blocks, 256, 0, st>>>(
                r->xh[k], r->vh[k], r->rho[k], r->aux[k], r->nbr[k], r->cnt[k], r->cells[k], s->bpos,
                s->bcells, s->bnear, s->bstart, s->bcand, n, s->nb, s->P, r->mu, r->dt, r->lam,
                r->gx, r->gv, r->gx2,
                r->gv2, r->grho, r->gmu_part);
            adj_sum_kernel<<<1, 32, 0, st>>>(r->gmu_part, blocks, r->gmu_acc);
            adj_density_kernel<<<blocks, 256, 0, st>>>(r->xh[k], r->nbr[k], r->cnt[k], r->cells[k],
                                                       n, s->P, r->grho, r->gx2);
            adj_unpermute_kernel<<<blocks, 256, 0, st>>>(r->perm[k], n, r->gx2, r->gv2, r->gx, r->gv);
        }
        SPH_CUDA(cudaGetLastError());
    }
    // gx, gv are now the adjoints of the creation-order initial state
    std::vector<float4> hg(n);
    double gm = 0.0;
    SPH_CUDA(cudaMemcpyAsync(&gm, r->gmu_acc, 8, cudaMemcpyDeviceToHost, st));
    if (grad_v0) {
        SPH_CUDA(cudaMemcpyAsync(hg.data(), r->gv, 16 * (size_t)n, cudaMemcpyDeviceToHost, st));
        SPH_CUDA(cudaStreamSynchronize(st));
        for (uint32_t i = 0; i < n; ++i) {
            grad_v0[3 * i] = hg[i].x;
            grad_v0[3 * i + 1] = hg[i].y;
            grad_v0[3 * i + 2] = hg[i].z;
        }
    }
    if (grad_x0) {
        SPH_CUDA(cudaMemcpyAsync(hg.data(), r->gx, 16 * (size_t)n, cudaMemcpyDeviceToHost, st));
        SPH_CUDA(cudaStreamSynchronize(st));
        for (uint32_t i = 0; i < n; ++i) {
            grad_x0[3 * i] = hg[i].x;
            grad_x0[3 * i + 1] = hg[i].y;
            grad_x0[3 * i + 2] = hg[i].z;
        }
    }
    SPH_CUDA(cudaStreamSynchronize(st));
    if (grad_mu) *grad_mu = gm;
    return check_device_error(s);
}

}  // extern "C"
