// single_scale.cu -- the single-scale solver handle behind the C ABI.
//
// Replaces Solver (SPH2S_FINAL_SINGLE_SCALE/Solver.h:62-132, Solver.cu:898-1198):
// the handle owns all device memory, keeps its configuration in kernel
// parameters instead of one __constant__ symbol, runs on its own stream, and
// captures one step into a CUDA graph that is replayed by sph_advance.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "errors.h"
#include "host_params.h"
#include "boundary_tables.cuh"

using namespace sph;

#include "single_scale_solver.h"

using namespace sph_ss;

namespace {

int free_solver(sph_solver* s) {
    if (!s) return SPH_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    sph_rollout_release(s);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    void* ptrs[] = {s->pos,     s->vel,     s->spos,    s->svel,  s->rho,   s->aux,
                    s->keys[0], s->keys[1], s->vals[0], s->vals[1], s->cells, s->bcells,
                    s->bpos,    s->sort_mem, s->co_mem,  s->err,   s->stage, s->nbr, s->nbr_count,
                    s->bnear,   s->pos0, s->xacc, s->xall, s->xnb, s->xa, s->bacc, s->blist, s->bflag, s->bcount, s->bstart, s->bcand};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (s->side) cudaStreamSynchronize(s->side);
    if (s->fork) cudaEventDestroy(s->fork);
    if (s->join) cudaEventDestroy(s->join);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->copy_stream) cudaStreamSynchronize(s->copy_stream);
    for (int b = 0; b < 2; ++b) {
        if (s->astage[b]) cudaFree(s->astage[b]);
        if (s->packed[b]) cudaEventDestroy(s->packed[b]);
        if (s->copied[b]) cudaEventDestroy(s->copied[b]);
    }
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->err_host) cudaFreeHost(s->err_host);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return SPH_OK;
}

template <class T>
int dalloc(T** p, size_t count) {
    SPH_CUDA(cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)));
    return SPH_OK;
}

}  // namespace

namespace sph_ss {

// hash -> stable sort of (cell key, index) -> reorder + cell ranges
// (Solver.cu:1098-1140).  The sort is the coherent one (coherent_sort.cuh):
// the same permutation as sorting from scratch, at the cost of the particles
// that changed cell since the last step.
int enqueue_neighborhood(sph_solver* s) {
    cudaStream_t st = s->stream;
    int out = 1;
    const bool coherent = s->sort_mode == kSortCoherent ||
                          (s->sort_mode == kSortAuto && s->n >= kCoherentMinParticles);
    NearList near;  // the near-boundary particles, for the boundary force pass
    near.bnear = s->bnear;
    near.list = s->blist;
    near.count = s->bcount;
    near.flag = s->bflag;
    cudaMemsetAsync(s->bcount, 0, 4, st);
    if (!coherent || s->force_timeout) {
        const int passes = sort_passes(s->key_bits);
        sort_reset(s->sort, st);
        uint32_t hb = blocks_for(s->n);
        if (hb > 152 * 8) hb = 152 * 8;
        hash_hist_kernel<<<hb, 256, 0, st>>>(s->pos, s->n, s->P.g, passes, s->keys[0], s->sort.hist);
        sort_scan(passes, s->sort, st);
        out = sort_passes_run(s->keys, s->vals, nullptr, s->n, passes, s->sort, s->err, s->force_timeout, st);
    } else {  // sort, reorder and cell table in one sequence
        coherent_sort_cells(s->co, s->pos, s->vel, s->P.g, s->cells, s->key_bits, s->keys[0],
                            s->keys[1], s->vals[1], s->spos, s->svel, s->err, s->force_timeout, st,
                            near);
        return out;
    }
    cudaMemsetAsync(s->cells, 0xFF, sizeof(uint2) * s->ncells, st);
    gather_cells_kernel<true><<<blocks_for(s->n), 256, 0, st>>>(
        s->keys[out], s->vals[out], s->n, s->P.g, s->pos, s->vel, s->spos, s->svel, s->cells,
        s->err, 0, s->co.kprev, near);
    return out;
}

// The density pass, and beside it on the second branch (fork/join events,
// captured into the step graph as a parallel branch) the boundary force sums
// of the near-boundary particles, which need only the sorted positions.
void enqueue_density(sph_solver* s) {
    cudaEventRecord(s->fork, s->stream);
    cudaStreamWaitEvent(s->side, s->fork, 0);
    const uint32_t bgrid = std::min(blocks_for(s->n), (uint32_t)(2 * (s->sms > 0 ? s->sms : 1)));
    boundary_force_kernel<<<bgrid, 256, 0, s->side>>>(s->spos, s->bpos, s->bcells, s->bstart,
                                                      s->bcand, s->blist, s->bcount, s->n, s->nb,
                                                      s->P, s->bacc);
    cudaEventRecord(s->join, s->side);
    density_kernel<false><<<blocks_for(s->n, kDensityThreads), kDensityThreads, 0, s->stream>>>(
        s->spos, s->cells, s->n, s->P, s->rho, s->aux, s->nbr, s->nbr_count, nullptr, s->xa,
        s->svel);
}

void enqueue_force(sph_solver* s, float dt) {
    cudaStreamWaitEvent(s->stream, s->join, 0);
    force_kernel<0, true><<<blocks_for(s->n), 256, 0, s->stream>>>(
        s->spos, s->xa, s->svel, s->cells, s->nbr, s->nbr_count, s->bpos, s->bcells, s->bnear,
        s->n, s->nb, s->P, dt, s->pos, s->vel, nullptr, nullptr, s->bacc, s->bflag);
}

// One step: Solver::Advance (Solver.cu:1082-1096) with integrate fused into
// the force pass.
void enqueue_step(sph_solver* s, float dt) {
    if (s->n == 0) return;
    enqueue_neighborhood(s);
    if (s->integrator == SPH_INTEGRATOR_XSPH) {
        // density (+ full neighbour counts), accelerations, XSPH integrate
        density_kernel<true><<<blocks_for(s->n, kDensityThreads), kDensityThreads, 0, s->stream>>>(
            s->spos, s->cells, s->n, s->P, s->rho, s->aux, s->nbr, s->nbr_count, s->xall, s->xa,
            s->svel);
        force_kernel<1><<<blocks_for(s->n), 256, 0, s->stream>>>(
            s->spos, s->xa, s->svel, s->cells, s->nbr, s->nbr_count, s->bpos, s->bcells, s->bnear,
            s->n, s->nb, s->P, dt, nullptr, nullptr, s->xacc, s->xnb);
        xsph_integrate_kernel<<<blocks_for(s->n), 256, 0, s->stream>>>(
            s->spos, s->svel, s->xacc, s->aux, s->cells, s->nbr, s->nbr_count, s->xall, s->n, s->P,
            dt, s->cfg.xsph_coeff, s->pos, s->vel);
        return;
    }
    enqueue_density(s);
    enqueue_force(s, dt);
}

int set_integrator(sph_solver* s, int32_t integrator) {
    if (integrator != SPH_INTEGRATOR_SYMPLECTIC_EULER && integrator != SPH_INTEGRATOR_XSPH)
        return fail(SPH_E_INVALID, "sph_set_integrator: unknown integrator");
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    if (integrator == SPH_INTEGRATOR_XSPH && !s->xacc) {
        const size_t n = s->n ? s->n : 1;
        SPH_CUDA(cudaMalloc(&s->xacc, 12 * n));
        SPH_CUDA(cudaMalloc(&s->xall, 4 * n));
        SPH_CUDA(cudaMalloc(&s->xnb, 4 * n));
    }
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    s->integrator = integrator;
    return SPH_OK;
}

int check_device_error(sph_solver* s) {
    SPH_CUDA(cudaMemcpyAsync(s->err_host, s->err, 4, cudaMemcpyDeviceToHost, s->stream));
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    uint32_t e = *s->err_host;
    if (e) {
        SPH_CUDA(cudaMemsetAsync(s->err, 0, 4, s->stream));
        coherent_reset(s->co, s->stream);  // the stored sorted keys may be garbage now
        SPH_CUDA(cudaStreamSynchronize(s->stream));
        if (e & kErrLookbackTimeout)
            return fail(SPH_E_TIMEOUT, "radix sort look-back timed out; step results are invalid");
        return fail(SPH_E_CAPACITY, "device-side capacity check failed");
    }
    return SPH_OK;
}

int create_solver(const sph_config* config, const HostInit& init, uint32_t n_fluid,
                  uint32_t n_boundary, uint64_t step, sph_solver** out) {
    *out = nullptr;
    SimParams P;
    int rc = make_sim_params(*config, &P);
    if (rc != SPH_OK) return rc;

    sph_solver* s = new sph_solver();
    s->cfg = *config;
    s->P = P;
    s->n = n_fluid;
    s->nb = n_boundary;
    s->ncells = sph_grid_num_cells(&config->grid);
    s->key_bits = 3 * P.g.mbits;
    s->step = step;
#define TRY(x)                      \
    do {                            \
        int _r = (x);               \
        if (_r != SPH_OK) {         \
            std::string m = sph_last_error(); \
            free_solver(s);         \
            return fail(_r, m);     \
        }                           \
    } while (0)
    TRY(check_cuda(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "stream", __FILE__, __LINE__));
    TRY(check_cuda(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking), "stream", __FILE__, __LINE__));
    TRY(check_cuda(cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming), "event", __FILE__, __LINE__));
    TRY(check_cuda(cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming), "event", __FILE__, __LINE__));
    uint32_t nmax = n_fluid > n_boundary ? n_fluid : n_boundary;
    TRY(dalloc(&s->pos, n_fluid));
    TRY(dalloc(&s->vel, n_fluid));
    TRY(dalloc(&s->spos, n_fluid));
    TRY(dalloc(&s->svel, n_fluid));
    TRY(dalloc(&s->rho, n_fluid));
    TRY(dalloc(&s->aux, n_fluid));
    TRY(dalloc(&s->xa, n_fluid));
    TRY(dalloc(&s->nbr, (size_t)n_fluid * (kMaxNbr / 4)));
    TRY(dalloc(&s->nbr_count, n_fluid));
    TRY(dalloc(&s->bnear, s->ncells));
    TRY(dalloc(&s->bacc, n_fluid));
    TRY(check_cuda(cudaMemsetAsync(s->bacc, 0, sizeof(float4) * (n_fluid ? n_fluid : 1), s->stream), "memset", __FILE__, __LINE__));
    TRY(dalloc(&s->blist, n_fluid));
    TRY(dalloc(&s->bflag, n_fluid));
    TRY(dalloc(&s->bcount, 1));
    {
        int dev = 0;
        TRY(check_cuda(cudaGetDevice(&dev), "device", __FILE__, __LINE__));
        TRY(check_cuda(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev), "device", __FILE__, __LINE__));
    }
    TRY(dalloc(&s->keys[0], nmax));
    TRY(dalloc(&s->keys[1], nmax));
    TRY(dalloc(&s->vals[0], nmax));
    TRY(dalloc(&s->vals[1], nmax));
    TRY(dalloc(&s->bcells, s->ncells));
    TRY(dalloc(&s->bpos, n_boundary));
    TRY(dalloc(&s->pos0, n_fluid));
    TRY(check_cuda(cudaMalloc(&s->sort_mem, sort_scratch_bytes(nmax)), "sort scratch", __FILE__, __LINE__));
    s->sort = sort_scratch_from(s->sort_mem, nmax);
    TRY(dalloc(&s->cells, s->ncells));  // read by the first coherent sort: no stale ranges
    TRY(check_cuda(cudaMemsetAsync(s->cells, 0xFF, sizeof(uint2) * s->ncells, s->stream), "memset", __FILE__, __LINE__));
    TRY(check_cuda(cudaMalloc(&s->co_mem, coherent_bytes(n_fluid)), "sort scratch", __FILE__, __LINE__));
    s->co = coherent_from(s->co_mem, n_fluid);
    coherent_reset(s->co, s->stream);
    TRY(dalloc(&s->err, 1));
    TRY(check_cuda(cudaMallocHost((void**)&s->err_host, 4), "pinned", __FILE__, __LINE__));
    TRY(check_cuda(cudaMemsetAsync(s->err, 0, 4, s->stream), "memset", __FILE__, __LINE__));
    for (int b = 0; b < 2; ++b) {
        TRY(check_cuda(cudaMemsetAsync(s->keys[b], 0, 4 * (size_t)(nmax ? nmax : 1), s->stream), "memset", __FILE__, __LINE__));
        TRY(check_cuda(cudaMemsetAsync(s->vals[b], 0, 4 * (size_t)(nmax ? nmax : 1), s->stream), "memset", __FILE__, __LINE__));
    }
    TRY(check_cuda(cudaMemsetAsync(s->rho, 0, 4 * (size_t)(n_fluid ? n_fluid : 1), s->stream), "memset", __FILE__, __LINE__));

    // Upload the fluid state (float4, persistent id in w).  Raw caller xyz
    // arrays go up as they are (12 bytes per particle) into the step buffers,
    // which are free until the first step, and are packed on the device.
    {
        if (n_fluid && init.pos_xyz) {
            const size_t bytes = 12 * (size_t)n_fluid;
            TRY(check_cuda(cudaMemcpyAsync(s->spos, init.pos_xyz, bytes, cudaMemcpyHostToDevice, s->stream), "upload", __FILE__, __LINE__));
            unpack_xyz_kernel<<<blocks_for(n_fluid), 256, 0, s->stream>>>(
                reinterpret_cast<const float*>(s->spos), n_fluid, 1, s->pos);
            if (init.vel_xyz) {
                TRY(check_cuda(cudaMemcpyAsync(s->svel, init.vel_xyz, bytes, cudaMemcpyHostToDevice, s->stream), "upload", __FILE__, __LINE__));
                unpack_xyz_kernel<<<blocks_for(n_fluid), 256, 0, s->stream>>>(
                    reinterpret_cast<const float*>(s->svel), n_fluid, 0, s->vel);
            } else {
                TRY(check_cuda(cudaMemsetAsync(s->vel, 0, sizeof(float4) * n_fluid, s->stream), "memset", __FILE__, __LINE__));
            }
            TRY(check_cuda(cudaMemcpyAsync(s->pos0, s->pos, sizeof(float4) * n_fluid, cudaMemcpyDeviceToDevice, s->stream), "copy", __FILE__, __LINE__));
            TRY(check_cuda(cudaGetLastError(), "unpack", __FILE__, __LINE__));
        } else if (n_fluid) {
            TRY(check_cuda(cudaMemcpyAsync(s->pos, init.pos, sizeof(float4) * n_fluid, cudaMemcpyHostToDevice, s->stream), "upload", __FILE__, __LINE__));
            TRY(check_cuda(cudaMemcpyAsync(s->vel, init.vel, sizeof(float4) * n_fluid, cudaMemcpyHostToDevice, s->stream), "upload", __FILE__, __LINE__));
            TRY(check_cuda(cudaMemcpyAsync(s->pos0, init.pos0, sizeof(float4) * n_fluid, cudaMemcpyHostToDevice, s->stream), "upload", __FILE__, __LINE__));
        }
        // Boundary: hashed and sorted once on the fluid grid (Solver.cu:1013-1055).
        TRY(check_cuda(cudaMemsetAsync(s->bcells, 0xFF, sizeof(uint2) * s->ncells, s->stream), "memset", __FILE__, __LINE__));
        if (n_boundary) {
            // the unsorted boundary in float4 (input index in w): in the force
            // records' buffer when it is large enough (unused until the first
            // density pass), else a temporary allocation
            float4* braw = s->xa;
            const bool own = n_boundary > n_fluid;
            if (own) TRY(dalloc(&braw, n_boundary));
            cudaError_t e;
            if (init.bound_xyz) {  // raw xyz staged in bpos (overwritten by the presort)
                e = cudaMemcpyAsync(s->bpos, init.bound_xyz, 12 * (size_t)n_boundary,
                                    cudaMemcpyHostToDevice, s->stream);
                if (e == cudaSuccess) {
                    unpack_xyz_kernel<<<blocks_for(n_boundary), 256, 0, s->stream>>>(
                        reinterpret_cast<const float*>(s->bpos), n_boundary, 1, braw);
                    e = cudaGetLastError();
                }
            } else {
                e = cudaMemcpyAsync(braw, init.bound, sizeof(float4) * n_boundary,
                                    cudaMemcpyHostToDevice, s->stream);
            }
            if (e == cudaSuccess) {
                // keys (cell, depth class): each cell's boundary particles by
                // non-decreasing depth, the order boundary_reach's cut needs
                const int qb = boundary_depth_bits(s->P.g, s->P.h, s->key_bits);
                int passes = sort_passes(s->key_bits + qb);
                sort_reset(s->sort, s->stream);
                boundary_hash_hist_kernel<<<blocks_for(n_boundary) > 1216 ? 1216 : blocks_for(n_boundary), 256, 0, s->stream>>>(
                    braw, n_boundary, s->P.g, qb, boundary_quantum(s->P.h), passes, s->keys[0],
                    s->sort.hist);
                sort_scan(passes, s->sort, s->stream);
                int o = sort_passes_run(s->keys, s->vals, nullptr, n_boundary, passes, s->sort, s->err, 0, s->stream);
                gather_cells_kernel<false><<<blocks_for(n_boundary), 256, 0, s->stream>>>(
                    s->keys[o], s->vals[o], n_boundary, s->P.g, braw, nullptr, s->bpos, nullptr, s->bcells,
                    s->err, qb);
                e = cudaGetLastError();
                if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            }
            if (own) cudaFree(braw);
            TRY(check_cuda(e, "boundary presort", __FILE__, __LINE__));
        }
        const int reach = (int)std::ceil(config->effective_radius / config->grid.spacing) + 1;
        boundary_near_kernel<<<blocks_for(s->ncells), 256, 0, s->stream>>>(s->bcells, s->P.g, reach,
                                                                           s->bnear);
        TRY(check_cuda(cudaGetLastError(), "boundary flags", __FILE__, __LINE__));
        BoundaryTables bt;
        const cudaError_t e = build_boundary_tables(s->bcells, s->bpos, s->bnear, s->P.g, s->ncells,
                                                    n_boundary, s->P.h, s->P.bmargin, s->stream, bt);
        s->bstart = bt.start;
        s->bcand = bt.cand;
        TRY(check_cuda(e, "boundary tables", __FILE__, __LINE__));
        TRY(check_cuda(cudaStreamSynchronize(s->stream), "create sync", __FILE__, __LINE__));
    }
    TRY(check_device_error(s));
#undef TRY
    *out = s;
    return SPH_OK;
}

}  // namespace sph_ss

namespace {

// Copies xyz of a float4 device array into a host AoS array, in sorted order
// or by the persistent ids in pos.w; the packing runs on the device so the
// host only receives 12 bytes per particle.
int download_xyz(sph_solver* s, const float4* dsrc, float* dst, int32_t order) {
    if (s->n == 0) return SPH_OK;
    if (!s->stage) SPH_CUDA(cudaMalloc(&s->stage, 12 * (size_t)s->n));
    pack_xyz_kernel<<<blocks_for(s->n), 256, 0, s->stream>>>(dsrc, s->pos, s->n,
                                                             order == SPH_ORDER_BY_ID, s->stage);
    SPH_CUDA(cudaGetLastError());
    SPH_CUDA(cudaMemcpyAsync(dst, s->stage, 12 * (size_t)s->n, cudaMemcpyDeviceToHost, s->stream));
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    return SPH_OK;
}

}  // namespace

extern "C" {

int sph_create(const sph_config* config, const float* fluid_xyz, uint32_t n_fluid,
               const float* boundary_xyz, uint32_t n_boundary, const float* velocity_xyz,
               sph_solver** out) {
    if (!config || !out) return fail(SPH_E_INVALID, "sph_create: NULL config or output handle");
    *out = nullptr;
    if (n_fluid && !fluid_xyz) return fail(SPH_E_INVALID, "sph_create: NULL fluid positions");
    if (n_boundary && !boundary_xyz) return fail(SPH_E_INVALID, "sph_create: NULL boundary positions");
    if (n_fluid > kMaxParticles || n_boundary > kMaxParticles)
        return fail(SPH_E_CAPACITY, "sph_create: more than 2^30 particles");
    sph_ss::HostInit init;
    init.pos_xyz = fluid_xyz;
    init.vel_xyz = velocity_xyz;
    init.bound_xyz = boundary_xyz;
    return sph_ss::create_solver(config, init, n_fluid, n_boundary, 0, out);
}

int sph_advance(sph_solver* s, float dt, int32_t steps) {
    if (!s) return fail(SPH_E_INVALID, "sph_advance: NULL handle");
    if (steps < 0 || !std::isfinite(dt)) return fail(SPH_E_INVALID, "sph_advance: bad dt or steps");
    if (s->n == 0 || steps == 0) return SPH_OK;
    if (s->force_timeout) {
        for (int k = 0; k < steps; ++k) enqueue_step(s, dt);
        SPH_CUDA(cudaGetLastError());
        s->step += (uint64_t)steps;
        return SPH_OK;
    }
    if (!s->graph || s->graph_dt != dt) {
        if (s->graph) {
            cudaGraphExecDestroy(s->graph);
            s->graph = nullptr;
        }
        cudaGraph_t g;
        SPH_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(s, dt);
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
        SPH_CUDA(le);
        SPH_CUDA(ce);
        cudaError_t ie = cudaGraphInstantiate(&s->graph, g, 0);
        cudaGraphDestroy(g);
        SPH_CUDA(ie);
        s->graph_dt = dt;
    }
    for (int k = 0; k < steps; ++k) SPH_CUDA(cudaGraphLaunch(s->graph, s->stream));
    s->step += (uint64_t)steps;
    return SPH_OK;
}

int sph_sync(sph_solver* s) {
    if (!s) return fail(SPH_E_INVALID, "sph_sync: NULL handle");
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    if (s->copy_stream) SPH_CUDA(cudaStreamSynchronize(s->copy_stream));
    return check_device_error(s);
}

int sph_get_positions_async(sph_solver* s, float* xyz, int32_t order) {
    if (!s || (!xyz && s->n)) return fail(SPH_E_INVALID, "sph_get_positions_async: NULL argument");
    if (order != SPH_ORDER_SORTED && order != SPH_ORDER_BY_ID) return fail(SPH_E_INVALID, "bad order");
    if (s->n == 0) return SPH_OK;
    if (!s->copy_stream) {
        SPH_CUDA(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
        for (int b = 0; b < 2; ++b) {
            SPH_CUDA(cudaEventCreateWithFlags(&s->packed[b], cudaEventDisableTiming));
            SPH_CUDA(cudaEventCreateWithFlags(&s->copied[b], cudaEventDisableTiming));
            SPH_CUDA(cudaMalloc(&s->astage[b], 12 * (size_t)s->n));
        }
    }
    const int b = s->abuf;
    s->abuf ^= 1;
    // the last copy out of this staging buffer has drained before it is refilled
    SPH_CUDA(cudaStreamWaitEvent(s->stream, s->copied[b], 0));
    pack_xyz_kernel<<<blocks_for(s->n), 256, 0, s->stream>>>(s->pos, s->pos, s->n,
                                                             order == SPH_ORDER_BY_ID, s->astage[b]);
    SPH_CUDA(cudaGetLastError());
    SPH_CUDA(cudaEventRecord(s->packed[b], s->stream));
    SPH_CUDA(cudaStreamWaitEvent(s->copy_stream, s->packed[b], 0));
    SPH_CUDA(cudaMemcpyAsync(xyz, s->astage[b], 12 * (size_t)s->n, cudaMemcpyDeviceToHost,
                             s->copy_stream));
    SPH_CUDA(cudaEventRecord(s->copied[b], s->copy_stream));
    return SPH_OK;
}

int sph_get_positions(sph_solver* s, float* xyz, int32_t order) {
    if (!s || (!xyz && s->n)) return fail(SPH_E_INVALID, "sph_get_positions: NULL argument");
    if (order != SPH_ORDER_SORTED && order != SPH_ORDER_BY_ID) return fail(SPH_E_INVALID, "bad order");
    int rc = sph_sync(s);
    if (rc != SPH_OK) return rc;
    return download_xyz(s, s->pos, xyz, order);
}

int sph_get_velocities(sph_solver* s, float* xyz, int32_t order) {
    if (!s || (!xyz && s->n)) return fail(SPH_E_INVALID, "sph_get_velocities: NULL argument");
    if (order != SPH_ORDER_SORTED && order != SPH_ORDER_BY_ID) return fail(SPH_E_INVALID, "bad order");
    int rc = sph_sync(s);
    if (rc != SPH_OK) return rc;
    return download_xyz(s, s->vel, xyz, order);
}

int sph_get_densities(sph_solver* s, float* rho, int32_t order) {
    if (!s || (!rho && s->n)) return fail(SPH_E_INVALID, "sph_get_densities: NULL argument");
    if (order != SPH_ORDER_SORTED && order != SPH_ORDER_BY_ID) return fail(SPH_E_INVALID, "bad order");
    int rc = sph_sync(s);
    if (rc != SPH_OK) return rc;
    std::vector<float> h(s->n);
    std::vector<float4> p(s->n);
    SPH_CUDA(cudaMemcpy(h.data(), s->rho, 4 * (size_t)s->n, cudaMemcpyDeviceToHost));
    SPH_CUDA(cudaMemcpy(p.data(), s->pos, sizeof(float4) * s->n, cudaMemcpyDeviceToHost));
    for (uint32_t k = 0; k < s->n; ++k) {
        uint32_t d = k;
        if (order == SPH_ORDER_BY_ID) std::memcpy(&d, &p[k].w, 4);
        if (d >= s->n) return fail(SPH_E_INVALID, "corrupt persistent id");
        rho[d] = h[k];
    }
    return SPH_OK;
}

}  // extern "C"

namespace {

int device_readback(sph_solver* s, const float4* src4, const float* src1, void* dst, int32_t order,
                    const char* who) {
    if (!s || (!dst && s->n)) return fail(SPH_E_INVALID, std::string(who) + ": NULL argument");
    if (order != SPH_ORDER_SORTED && order != SPH_ORDER_BY_ID) return fail(SPH_E_INVALID, "bad order");
    if (s->n == 0) return SPH_OK;
    int rc = check_device_pointer(dst, who);
    if (rc != SPH_OK) return rc;
    if (src4)
        pack_xyz_kernel<<<blocks_for(s->n), 256, 0, s->stream>>>(src4, s->pos, s->n,
                                                                 order == SPH_ORDER_BY_ID,
                                                                 static_cast<float*>(dst));
    else
        pack_scalar_kernel<<<blocks_for(s->n), 256, 0, s->stream>>>(src1, s->pos, s->n,
                                                                    order == SPH_ORDER_BY_ID,
                                                                    static_cast<float*>(dst));
    SPH_CUDA(cudaGetLastError());
    return SPH_OK;
}

}  // namespace

extern "C" {

int sph_get_positions_device(sph_solver* s, float* d_xyz, int32_t order) {
    return device_readback(s, s ? s->pos : nullptr, nullptr, d_xyz, order, "sph_get_positions_device");
}

int sph_get_velocities_device(sph_solver* s, float* d_xyz, int32_t order) {
    return device_readback(s, s ? s->vel : nullptr, nullptr, d_xyz, order, "sph_get_velocities_device");
}

int sph_get_densities_device(sph_solver* s, float* d_rho, int32_t order) {
    return device_readback(s, nullptr, s ? s->rho : nullptr, d_rho, order, "sph_get_densities_device");
}

int sph_get_ids(sph_solver* s, uint32_t* ids) {
    if (!s || (!ids && s->n)) return fail(SPH_E_INVALID, "sph_get_ids: NULL argument");
    int rc = sph_sync(s);
    if (rc != SPH_OK) return rc;
    std::vector<float4> p(s->n);
    SPH_CUDA(cudaMemcpy(p.data(), s->pos, sizeof(float4) * s->n, cudaMemcpyDeviceToHost));
    for (uint32_t k = 0; k < s->n; ++k) std::memcpy(&ids[k], &p[k].w, 4);
    return SPH_OK;
}

int sph_set_velocities(sph_solver* s, const float* xyz, int32_t order) {
    if (!s || (!xyz && s->n)) return fail(SPH_E_INVALID, "sph_set_velocities: NULL argument");
    if (order != SPH_ORDER_SORTED && order != SPH_ORDER_BY_ID) return fail(SPH_E_INVALID, "bad order");
    int rc = sph_sync(s);
    if (rc != SPH_OK) return rc;
    std::vector<float4> p(s->n), v(s->n);
    SPH_CUDA(cudaMemcpy(p.data(), s->pos, sizeof(float4) * s->n, cudaMemcpyDeviceToHost));
    for (uint32_t k = 0; k < s->n; ++k) {
        uint32_t src = k;
        if (order == SPH_ORDER_BY_ID) std::memcpy(&src, &p[k].w, 4);
        if (src >= s->n) return fail(SPH_E_INVALID, "corrupt persistent id");
        v[k] = make_float4(xyz[3 * src], xyz[3 * src + 1], xyz[3 * src + 2], 0.0f);
    }
    SPH_CUDA(cudaMemcpy(s->vel, v.data(), sizeof(float4) * s->n, cudaMemcpyHostToDevice));
    return SPH_OK;
}

int sph_set_integrator(sph_solver* s, int32_t integrator) {
    if (!s) return fail(SPH_E_INVALID, "sph_set_integrator: NULL handle");
    return set_integrator(s, integrator);
}

int sph_counts(sph_solver* s, uint32_t* n_fluid, uint32_t* n_boundary) {
    if (!s) return fail(SPH_E_INVALID, "sph_counts: NULL handle");
    if (n_fluid) *n_fluid = s->n;
    if (n_boundary) *n_boundary = s->nb;
    return SPH_OK;
}

void* sph_stream(sph_solver* s) { return s ? (void*)s->stream : nullptr; }

int sph_destroy(sph_solver* s) { return free_solver(s); }

int sph_debug_step_fields(sph_solver* s, uint32_t* keys, uint32_t* ids, uint32_t* cell_start,
                          uint32_t* cell_end, uint32_t* nbr_fluid, uint32_t* nbr_boundary,
                          float* rho, float* acc) {
    if (!s) return fail(SPH_E_INVALID, "sph_debug_step_fields: NULL handle");
    int rc = sph_sync(s);
    if (rc != SPH_OK) return rc;
    if (s->n == 0) return SPH_OK;
    const uint32_t n = s->n;
    float* drho = nullptr;
    float2* daux = nullptr;
    float* dacc = nullptr;
    uint32_t *dnf = nullptr, *dnb = nullptr;
    SPH_CUDA(cudaMalloc(&drho, 4 * (size_t)n));
    SPH_CUDA(cudaMalloc(&daux, 8 * (size_t)n));
    SPH_CUDA(cudaMalloc(&dacc, 12 * (size_t)n));
    SPH_CUDA(cudaMalloc(&dnf, 4 * (size_t)n));
    SPH_CUDA(cudaMalloc(&dnb, 4 * (size_t)n));
    const int out = enqueue_neighborhood(s);  // buffer index holding the sorted keys
    density_kernel<true><<<blocks_for(n, kDensityThreads), kDensityThreads, 0, s->stream>>>(
        s->spos, s->cells, n, s->P, drho, daux, s->nbr, s->nbr_count, dnf, s->xa, s->svel);
    force_kernel<1><<<blocks_for(n), 256, 0, s->stream>>>(
        s->spos, s->xa, s->svel, s->cells, s->nbr, s->nbr_count, s->bpos, s->bcells, s->bnear, n,
        s->nb, s->P, 0.0f, nullptr, nullptr, dacc, dnb);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    std::vector<float4> sp;
    if (e == cudaSuccess && keys) e = cudaMemcpy(keys, s->keys[out], 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && ids) {
        sp.resize(n);
        e = cudaMemcpy(sp.data(), s->spos, sizeof(float4) * n, cudaMemcpyDeviceToHost);
        for (uint32_t k = 0; k < n && e == cudaSuccess; ++k) std::memcpy(&ids[k], &sp[k].w, 4);
    }
    if (e == cudaSuccess && (cell_start || cell_end)) {
        std::vector<uint2> c(s->ncells);
        e = cudaMemcpy(c.data(), s->cells, sizeof(uint2) * s->ncells, cudaMemcpyDeviceToHost);
        for (uint32_t k = 0; k < s->ncells && e == cudaSuccess; ++k) {
            if (cell_start) cell_start[k] = c[k].x;
            if (cell_end) cell_end[k] = c[k].y;
        }
    }
    if (e == cudaSuccess && nbr_fluid) e = cudaMemcpy(nbr_fluid, dnf, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && nbr_boundary) e = cudaMemcpy(nbr_boundary, dnb, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && rho) e = cudaMemcpy(rho, drho, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && acc) e = cudaMemcpy(acc, dacc, 12 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(drho);
    cudaFree(daux);
    cudaFree(dacc);
    cudaFree(dnf);
    cudaFree(dnb);
    SPH_CUDA(e);
    return check_device_error(s);
}

int sph_profile_phases(sph_solver* s, float dt, int32_t steps, float* ms) {
    if (!s || !ms || steps < 0) return fail(SPH_E_INVALID, "sph_profile_phases: bad argument");
    ms[0] = ms[1] = ms[2] = 0.0f;
    if (s->n == 0 || steps == 0) return SPH_OK;
    // The steps are captured into one graph with an event record node at each
    // phase boundary, so the phases are timed as the step graph runs them
    // (back to back, no host launches in between); they sum to the whole span.
    std::vector<cudaEvent_t> ev(3 * (size_t)steps + 1, nullptr);
    cudaError_t err = cudaSuccess;
    for (auto& e : ev)
        if (err == cudaSuccess) err = cudaEventCreate(&e);
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    if (err == cudaSuccess) err = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
    if (err == cudaSuccess) {
        // cudaEventRecordExternal: a real event record node (a plain record
        // during capture only orders streams)
        const unsigned fl = cudaEventRecordExternal;
        for (int k = 0; k < steps; ++k) {
            if (k == 0) cudaEventRecordWithFlags(ev[0], s->stream, fl);
            enqueue_neighborhood(s);
            cudaEventRecordWithFlags(ev[3 * k + 1], s->stream, fl);
            enqueue_density(s);
            cudaEventRecordWithFlags(ev[3 * k + 2], s->stream, fl);
            enqueue_force(s, dt);
            cudaEventRecordWithFlags(ev[3 * k + 3], s->stream, fl);
        }
        cudaError_t le = cudaGetLastError();
        err = cudaStreamEndCapture(s->stream, &g);
        if (err == cudaSuccess) err = le;
    }
    if (err == cudaSuccess) err = cudaGraphInstantiate(&ge, g, 0);
    if (err == cudaSuccess) err = cudaGraphLaunch(ge, s->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s->stream);
    double acc[3] = {0, 0, 0};
    for (int k = 0; k < steps && err == cudaSuccess; ++k)
        for (int p = 0; p < 3 && err == cudaSuccess; ++p) {
            float t = 0.0f;
            err = cudaEventElapsedTime(&t, ev[3 * k + p], ev[3 * k + p + 1]);
            acc[p] += t;
        }
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    SPH_CUDA(err);
    s->step += (uint64_t)steps;
    for (int p = 0; p < 3; ++p) ms[p] = (float)(acc[p] / steps);
    return check_device_error(s);
}

int sph_debug_force_lookback_timeout(sph_solver* s, int32_t on) {
    if (!s) return fail(SPH_E_INVALID, "NULL handle");
    s->force_timeout = on ? 1 : 0;
    return SPH_OK;
}

int sph_debug_sort_mode(sph_solver* s, int32_t mode) {
    if (!s) return fail(SPH_E_INVALID, "NULL handle");
    if (mode != kSortAuto && mode != kSortFull && mode != kSortCoherent)
        return fail(SPH_E_INVALID, "sph_debug_sort_mode: mode must be 0, 1 or 2");
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    s->sort_mode = mode;
    return SPH_OK;
}

}  // extern "C"
