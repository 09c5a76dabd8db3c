// batched.cu -- many independent single-scale scenes stepped together.
//
// The reference runs one Solver per process and binds its configuration to
// one __constant__ symbol (SPH2S_FINAL_SINGLE_SCALE/Solver.cu:12, 1068-1080),
// so several scenes can only be stepped one after another.  A batch packs the
// scenes into shared device arrays with a per-scene parameter table and steps
// all of them with one launch per kernel (hash, onesweep sort passes, reorder,
// density, force + integrate), captured as one CUDA graph per step.  Results
// per scene are those of the single-scale solver on that scene: same keys,
// same sorted order, same per-particle device code.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "batched_solver.h"
#include "errors.h"
#include "host_params.h"
#include "scan.cuh"
#include "single_scale_kernels.cuh"

using namespace sph;

namespace {

template <class T>
int dalloc(T** p, size_t count, std::vector<void*>& owned) {
    SPH_CUDA(cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)));
    owned.push_back(*p);
    return SPH_OK;
}

}  // namespace

namespace sph_b {

int free_batch(sph_batch* b) {
    if (!b) return SPH_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->side) cudaStreamSynchronize(b->side);
    sphb_rollout_release(b);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (void* p : b->owned) cudaFree(p);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->join) cudaEventDestroy(b->join);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->err_host) cudaFreeHost(b->err_host);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return SPH_OK;
}

std::vector<uint2> make_tiles(const std::vector<SceneRec>& recs, int bs, bool boundary) {
    std::vector<uint2> t;
    for (uint32_t s = 0; s < recs.size(); ++s) {
        const uint32_t beg = boundary ? recs[s].b_off : recs[s].p_off;
        const uint32_t n = boundary ? recs[s].b_n : recs[s].p_n;
        for (uint32_t k = 0; k < n; k += (uint32_t)bs) t.push_back(make_uint2(s, beg + k));
    }
    return t;
}

uint32_t pgrid(const sph_batch* b, uint32_t tiles) {
    uint32_t g = (uint32_t)(b->grid_mult * b->sms);
    return std::max(1u, std::min(g, tiles));
}

template <int BS>
void launch_density(sph_batch* b, int ti) {
    b_density_kernel<BS><<<pgrid(b, b->ntiles[ti]), BS, 0, b->stream>>>(
        b->tiles[ti], b->ntiles[ti], b->recs, b->spos, b->cells, b->N, b->rho, b->aux, b->nbr,
        b->nbr_count, b->xa, b->svel);
}

template <int BS>
void launch_force(sph_batch* b, int ti, float dt) {
    b_force_kernel<BS><<<pgrid(b, b->ntiles[ti]), BS, 0, b->stream>>>(
        b->tiles[ti], b->ntiles[ti], b->recs, b->spos, b->xa, b->svel, b->cells, b->nbr,
        b->nbr_count, b->bpos, b->bcells, b->bnear, b->N, b->NB, dt, b->pos, b->vel, b->bacc,
        b->bflag);
}

// The density pass, and beside it on the second branch (fork / join events,
// a parallel branch of the step graph) the boundary force sums.
void enqueue_density(sph_batch* b) {
    cudaEventRecord(b->fork, b->stream);
    cudaStreamWaitEvent(b->side, b->fork, 0);
    // two blocks per SM: the density blocks fit beside them (a full persistent
    // grid here would hold every SM until it drained, and density would wait)
    b_boundary_force_kernel<256><<<std::min(pgrid(b, b->ntiles[1]), 2u * (uint32_t)b->sms), 256,
                                   0, b->side>>>(
        b->tiles[1], b->ntiles[1], b->recs, b->spos, b->bpos, b->bcells, b->bnear, b->bstart,
        b->bcand, b->NB, b->bacc, b->bflag);
    cudaEventRecord(b->join, b->side);
    switch (b->bs_density) {
        case 0: launch_density<128>(b, 0); break;
        case 2: launch_density<512>(b, 2); break;
        default: launch_density<256>(b, 1); break;
    }
}

void enqueue_force(sph_batch* b, float dt) {
    cudaStreamWaitEvent(b->stream, b->join, 0);
    switch (b->bs_force) {
        case 0: launch_force<128>(b, 0, dt); break;
        case 2: launch_force<512>(b, 2, dt); break;
        default: launch_force<256>(b, 1, dt); break;
    }
}

// hash -> stable sort of (scene, cell key, index) -> reorder + cell ranges.
// From 131,072 fluid particles the sort is the coherent one (coherent_sort.cuh:
// the same permutation, radix-sorting only the particles that changed cell).
int enqueue_neighborhood(sph_batch* b) {
    cudaStream_t st = b->stream;
    cudaMemsetAsync(b->cells, 0xFF, sizeof(uint2) * b->NC, st);
    int o = 1;
    if (b->coherent) {
        b_hash_hist_kernel<256><<<pgrid(b, b->ntiles[1]), 256, 0, st>>>(
            b->tiles[1], b->ntiles[1], b->recs, b->pos, b->shift, 0, b->keys[0], b->sort.hist);
        coherent_sort_keys(b->co, b->keys[0], 8 * b->passes, b->keys[1], b->vals[1], b->err, 0,
                           st);
    } else {
        sort_reset(b->sort, st);
        b_hash_hist_kernel<256><<<pgrid(b, b->ntiles[1]), 256, 0, st>>>(
            b->tiles[1], b->ntiles[1], b->recs, b->pos, b->shift, b->passes, b->keys[0],
            b->sort.hist);
        sort_scan(b->passes, b->sort, st);
        o = sort_passes_run(b->keys, b->vals, nullptr, b->N, b->passes, b->sort, b->err, 0, st);
    }
    b_gather_cells_kernel<256, true><<<pgrid(b, b->ntiles[1]), 256, 0, st>>>(
        b->tiles[1], b->ntiles[1], b->recs, b->keys[o], b->vals[o], b->N, b->shift, false, b->pos,
        b->vel, b->spos, b->svel, b->cells, b->err, 0, b->coherent ? b->co.kprev : nullptr,
        b->bnear, b->bflag);
    return o;
}

void enqueue_step(sph_batch* b, float dt) {
    if (b->N == 0) return;
    enqueue_neighborhood(b);
    enqueue_density(b);
    enqueue_force(b, dt);
}

int refresh_scene_params(sph_batch* b) {
    for (uint32_t s = 0; s < b->S; ++s) {
        int rc = make_sim_params(b->cfgs[s], &b->recs_h[s].P);
        if (rc != SPH_OK) return rc;
    }
    SPH_CUDA(cudaMemcpyAsync(b->recs, b->recs_h.data(), sizeof(SceneRec) * b->S,
                             cudaMemcpyHostToDevice, b->stream));
    SPH_CUDA(cudaStreamSynchronize(b->stream));
    return SPH_OK;
}

int check_err(sph_batch* b) {
    SPH_CUDA(cudaMemcpyAsync(b->err_host, b->err, 4, cudaMemcpyDeviceToHost, b->stream));
    SPH_CUDA(cudaStreamSynchronize(b->stream));
    const uint32_t e = *b->err_host;
    if (e) {
        SPH_CUDA(cudaMemsetAsync(b->err, 0, 4, b->stream));
        if (b->coherent) coherent_reset(b->co, b->stream);  // the kept keys may be garbage
        SPH_CUDA(cudaStreamSynchronize(b->stream));
        if (e & kErrLookbackTimeout) return fail(SPH_E_TIMEOUT, "radix sort look-back timed out");
        return fail(SPH_E_CAPACITY, "device-side index check failed");
    }
    return SPH_OK;
}

}  // namespace sph_b

using namespace sph_b;

extern "C" {

int sphb_create(const sph_scene_desc* scenes, uint32_t num_scenes, sph_batch** out) {
    if (!scenes || !out || num_scenes == 0)
        return fail(SPH_E_INVALID, "sphb_create: need at least one scene and an output handle");
    *out = nullptr;
    sph_batch* b = new sph_batch();
    b->S = num_scenes;
    uint64_t N = 0, NB = 0, NC = 0;
    int maxbits = 1;
    for (uint32_t s = 0; s < num_scenes; ++s) {
        const sph_scene_desc& d = scenes[s];
        SceneRec R;
        int rc = make_sim_params(d.config, &R.P);
        if (rc != SPH_OK) {
            free_batch(b);
            return rc;
        }
        if ((d.n_fluid && !d.fluid_xyz) || (d.n_boundary && !d.boundary_xyz)) {
            free_batch(b);
            return fail(SPH_E_INVALID, "sphb_create: NULL particle array");
        }
        R.p_off = (uint32_t)N;
        R.p_n = d.n_fluid;
        R.c_off = (uint32_t)NC;
        R.b_off = (uint32_t)NB;
        R.b_n = d.n_boundary;
        N += d.n_fluid;
        NB += d.n_boundary;
        NC += sph_grid_num_cells(&d.config.grid);
        maxbits = std::max(maxbits, R.P.g.mbits);
        b->recs_h.push_back(R);
        b->cfgs.push_back(d.config);
        b->tile_first.push_back(0);
    }
    int sbits = 1;
    while ((1u << sbits) < num_scenes) ++sbits;
    b->shift = 3 * maxbits;
    if (b->shift + sbits > 32 || N > kMaxParticles || NB > kMaxParticles || NC > 0xFFFFFFF0ull) {
        free_batch(b);
        return fail(SPH_E_CAPACITY, "sphb_create: scenes, particles or cells beyond the ABI limits");
    }
    b->passes = sort_passes(b->shift + sbits);
    b->N = (uint32_t)N;
    b->NB = (uint32_t)NB;
    b->NC = (uint32_t)NC;
#define TRY(x)                                \
    do {                                      \
        int _r = (x);                         \
        if (_r != SPH_OK) {                   \
            std::string m = sph_last_error(); \
            free_batch(b);                    \
            return fail(_r, m);               \
        }                                     \
    } while (0)
    int dev = 0;
    TRY(check_cuda(cudaGetDevice(&dev), "device", __FILE__, __LINE__));
    TRY(check_cuda(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev), "attr", __FILE__, __LINE__));
    TRY(check_cuda(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream", __FILE__, __LINE__));
    TRY(check_cuda(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking), "stream", __FILE__, __LINE__));
    TRY(check_cuda(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "event", __FILE__, __LINE__));
    TRY(check_cuda(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming), "event", __FILE__, __LINE__));
    const uint32_t nmax = std::max(b->N, b->NB);
    TRY(dalloc(&b->recs, num_scenes, b->owned));
    TRY(dalloc(&b->pos, b->N, b->owned));
    TRY(dalloc(&b->vel, b->N, b->owned));
    TRY(dalloc(&b->spos, b->N, b->owned));
    TRY(dalloc(&b->svel, b->N, b->owned));
    TRY(dalloc(&b->rho, b->N, b->owned));
    TRY(dalloc(&b->aux, b->N, b->owned));
    TRY(dalloc(&b->xa, b->N, b->owned));
    TRY(dalloc(&b->nbr, (size_t)b->N * (kMaxNbr / 4), b->owned));
    TRY(dalloc(&b->nbr_count, b->N, b->owned));
    for (int k = 0; k < 2; ++k) {
        TRY(dalloc(&b->keys[k], nmax, b->owned));
        TRY(dalloc(&b->vals[k], nmax, b->owned));
        TRY(check_cuda(cudaMemset(b->keys[k], 0, 4 * (size_t)std::max(nmax, 1u)), "memset", __FILE__, __LINE__));
        TRY(check_cuda(cudaMemset(b->vals[k], 0, 4 * (size_t)std::max(nmax, 1u)), "memset", __FILE__, __LINE__));
    }
    TRY(dalloc(&b->cells, b->NC, b->owned));
    TRY(dalloc(&b->bcells, b->NC, b->owned));
    TRY(dalloc(&b->bnear, b->NC, b->owned));
    TRY(dalloc(&b->bstart, (size_t)b->NC + 1, b->owned));
    TRY(dalloc(&b->bacc, b->N, b->owned));
    TRY(dalloc(&b->bflag, b->N, b->owned));
    TRY(check_cuda(cudaMemset(b->bacc, 0, 16 * (size_t)std::max(b->N, 1u)), "memset", __FILE__, __LINE__));
    TRY(dalloc(&b->bpos, b->NB, b->owned));
    TRY(check_cuda(cudaMalloc(&b->sort_mem, sort_scratch_bytes(nmax)), "sort scratch", __FILE__, __LINE__));
    b->owned.push_back(b->sort_mem);
    b->sort = sort_scratch_from(b->sort_mem, nmax);
    b->coherent = b->N >= 131072u;
    if (b->coherent) {
        TRY(check_cuda(cudaMalloc(&b->co_mem, coherent_bytes(b->N)), "sort scratch", __FILE__, __LINE__));
        b->owned.push_back(b->co_mem);
        b->co = coherent_from(b->co_mem, b->N);
        TRY(check_cuda(cudaMemset(b->co.kprev, 0xFF, 4 * (size_t)b->N), "memset", __FILE__, __LINE__));
    }
    TRY(dalloc(&b->err, 1, b->owned));
    TRY(check_cuda(cudaMemset(b->err, 0, 4), "memset", __FILE__, __LINE__));
    TRY(check_cuda(cudaMallocHost((void**)&b->err_host, 4), "pinned", __FILE__, __LINE__));
    TRY(check_cuda(cudaMemcpy(b->recs, b->recs_h.data(), sizeof(SceneRec) * num_scenes, cudaMemcpyHostToDevice), "recs", __FILE__, __LINE__));
    for (uint32_t s = 1; s < num_scenes; ++s)
        b->tile_first[s] = b->tile_first[s - 1] + (b->recs_h[s - 1].p_n + 255u) / 256u;
    for (int k = 0; k < 3; ++k) {
        std::vector<uint2> t = make_tiles(b->recs_h, kBlockChoices[k], false);
        b->ntiles[k] = (uint32_t)t.size();
        TRY(dalloc(&b->tiles[k], t.size(), b->owned));
        if (!t.empty())
            TRY(check_cuda(cudaMemcpy(b->tiles[k], t.data(), 8 * t.size(), cudaMemcpyHostToDevice), "tiles", __FILE__, __LINE__));
    }
    {
        std::vector<uint2> t = make_tiles(b->recs_h, 256, true);
        b->nbtiles = (uint32_t)t.size();
        TRY(dalloc(&b->btiles, t.size(), b->owned));
        if (!t.empty())
            TRY(check_cuda(cudaMemcpy(b->btiles, t.data(), 8 * t.size(), cudaMemcpyHostToDevice), "tiles", __FILE__, __LINE__));
    }
    // upload particles: persistent id = index within the scene
    {
        std::vector<float4> hp(b->N), hv(b->N), hb(b->NB);
        for (uint32_t s = 0; s < num_scenes; ++s) {
            const sph_scene_desc& d = scenes[s];
            const SceneRec& R = b->recs_h[s];
            for (uint32_t i = 0; i < d.n_fluid; ++i) {
                float w;
                std::memcpy(&w, &i, 4);
                const float* x = d.fluid_xyz + 3 * (size_t)i;
                hp[R.p_off + i] = make_float4(x[0], x[1], x[2], w);
                const float* v = d.velocity_xyz ? d.velocity_xyz + 3 * (size_t)i : nullptr;
                hv[R.p_off + i] = v ? make_float4(v[0], v[1], v[2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            for (uint32_t i = 0; i < d.n_boundary; ++i) {
                const float* x = d.boundary_xyz + 3 * (size_t)i;
                hb[R.b_off + i] = make_float4(x[0], x[1], x[2], 0.0f);
            }
        }
        TRY(dalloc(&b->pos0, b->N, b->owned));
        if (b->N) {
            TRY(check_cuda(cudaMemcpy(b->pos0, hp.data(), 16 * (size_t)b->N, cudaMemcpyHostToDevice), "upload", __FILE__, __LINE__));
            TRY(check_cuda(cudaMemcpy(b->pos, hp.data(), 16 * (size_t)b->N, cudaMemcpyHostToDevice), "upload", __FILE__, __LINE__));
            TRY(check_cuda(cudaMemcpy(b->vel, hv.data(), 16 * (size_t)b->N, cudaMemcpyHostToDevice), "upload", __FILE__, __LINE__));
        }
        // boundaries: sorted once per scene on the scene's grid
        TRY(check_cuda(cudaMemset(b->bcells, 0xFF, sizeof(uint2) * std::max(b->NC, 1u)), "memset", __FILE__, __LINE__));
        if (b->NB) {
            float4* braw = nullptr;
            TRY(dalloc(&braw, b->NB, b->owned));
            TRY(check_cuda(cudaMemcpy(braw, hb.data(), 16 * (size_t)b->NB, cudaMemcpyHostToDevice), "upload", __FILE__, __LINE__));
            // keys (scene, cell, depth class): each cell's boundary particles by
            // non-decreasing depth, the order boundary_reach's cut needs; the
            // class bits are those every scene allows
            int sbits = 1;
            while ((1u << sbits) < num_scenes) ++sbits;
            int qb = 8;
            for (const SceneRec& R : b->recs_h)
                qb = std::min(qb, boundary_depth_bits(R.P.g, R.P.h, b->shift + sbits));
            const int bpasses = sort_passes(b->shift + sbits + qb);
            sort_reset(b->sort, b->stream);
            b_boundary_hash_hist_kernel<256><<<pgrid(b, b->nbtiles), 256, 0, b->stream>>>(
                b->btiles, b->nbtiles, b->recs, braw, b->shift, qb, bpasses, b->keys[0],
                b->sort.hist);
            sort_scan(bpasses, b->sort, b->stream);
            const int o = sort_passes_run(b->keys, b->vals, nullptr, b->NB, bpasses, b->sort,
                                          b->err, 0, b->stream);
            b_gather_cells_kernel<256, false><<<pgrid(b, b->nbtiles), 256, 0, b->stream>>>(
                b->btiles, b->nbtiles, b->recs, b->keys[o], b->vals[o], b->NB, b->shift, true, braw,
                nullptr, b->bpos, nullptr, b->bcells, b->err, qb);
            TRY(check_cuda(cudaStreamSynchronize(b->stream), "boundary presort", __FILE__, __LINE__));
            cudaFree(braw);
            b->owned.pop_back();
        }
        for (uint32_t s = 0; s < num_scenes; ++s) {
            const SceneRec& R = b->recs_h[s];
            const sph_config& c = scenes[s].config;
            const uint32_t nc = sph_grid_num_cells(&c.grid);
            const int reach = (int)std::ceil(c.effective_radius / c.grid.spacing) + 1;
            boundary_near_kernel<<<(nc + 255) / 256, 256, 0, b->stream>>>(b->bcells + R.c_off, R.P.g,
                                                                          reach, b->bnear + R.c_off);
        }
        TRY(check_cuda(cudaGetLastError(), "boundary flags", __FILE__, __LINE__));
        // static boundary tables of every scene (boundary_tables.cuh): candidate
        // counts per scene, one prefix sum over all cells, then the candidates
        // (global boundary indices)
        std::vector<float> lims(num_scenes);
        for (uint32_t s = 0; s < num_scenes; ++s) {
            const SceneRec& R = b->recs_h[s];
            const uint32_t nc = sph_grid_num_cells(&scenes[s].config.grid);
            lims[s] = R.P.h * 1.01f + 4.0f * R.P.bmargin;
            if (!nc) continue;
            boundary_cand_kernel<false><<<(nc + 255) / 256, 256, 0, b->stream>>>(
                b->bcells + R.c_off, b->bpos, b->bnear + R.c_off, R.P.g, b->NB, lims[s],
                b->bstart + R.c_off, nullptr);
        }
        TRY(check_cuda(cudaMemsetAsync(b->bstart + b->NC, 0, 4, b->stream), "memset", __FILE__, __LINE__));
        {
            const uint32_t words = (uint32_t)scan_scratch_words(b->NC + 1);
            uint32_t* scratch = nullptr;
            TRY(dalloc(&scratch, (size_t)words + 1, b->owned));
            const ScanSeg seg = {b->bstart, b->bstart, b->NC + 1, scratch + words};
            scan_exclusive_batch(&seg, 1, scratch, b->stream);
            uint32_t total = 0;
            TRY(check_cuda(cudaMemcpyAsync(&total, scratch + words, 4, cudaMemcpyDeviceToHost, b->stream), "copy", __FILE__, __LINE__));
            TRY(check_cuda(cudaStreamSynchronize(b->stream), "boundary tables", __FILE__, __LINE__));
            cudaFree(scratch);
            b->owned.pop_back();
            TRY(dalloc(&b->bcand, total, b->owned));
        }
        for (uint32_t s = 0; s < num_scenes; ++s) {
            const SceneRec& R = b->recs_h[s];
            const uint32_t nc = sph_grid_num_cells(&scenes[s].config.grid);
            if (!nc) continue;
            boundary_cand_kernel<true><<<(nc + 255) / 256, 256, 0, b->stream>>>(
                b->bcells + R.c_off, b->bpos, b->bnear + R.c_off, R.P.g, b->NB, lims[s],
                b->bstart + R.c_off, b->bcand);
        }
        TRY(check_cuda(cudaGetLastError(), "boundary tables", __FILE__, __LINE__));
        TRY(check_cuda(cudaStreamSynchronize(b->stream), "create", __FILE__, __LINE__));
    }
    TRY(check_err(b));
#undef TRY
    *out = b;
    return SPH_OK;
}

int sphb_advance(sph_batch* b, float dt, int32_t steps) {
    if (!b) return fail(SPH_E_INVALID, "sphb_advance: NULL handle");
    if (steps < 0 || !std::isfinite(dt)) return fail(SPH_E_INVALID, "sphb_advance: bad dt or steps");
    if (b->N == 0 || steps == 0) return SPH_OK;
    if (!b->graph || b->graph_dt != dt) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        cudaGraph_t g;
        SPH_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(b, dt);
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        SPH_CUDA(le);
        SPH_CUDA(ce);
        cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        SPH_CUDA(ie);
        b->graph_dt = dt;
    }
    for (int k = 0; k < steps; ++k) SPH_CUDA(cudaGraphLaunch(b->graph, b->stream));
    return SPH_OK;
}

int sphb_sync(sph_batch* b) {
    if (!b) return fail(SPH_E_INVALID, "sphb_sync: NULL handle");
    SPH_CUDA(cudaStreamSynchronize(b->stream));
    return check_err(b);
}

void* sphb_stream(sph_batch* b) { return b ? (void*)b->stream : nullptr; }

int sphb_counts(sph_batch* b, uint32_t* num_scenes, uint32_t* total_fluid,
                uint32_t* total_boundary) {
    if (!b) return fail(SPH_E_INVALID, "sphb_counts: NULL handle");
    if (num_scenes) *num_scenes = b->S;
    if (total_fluid) *total_fluid = b->N;
    if (total_boundary) *total_boundary = b->NB;
    return SPH_OK;
}

// xyz (or velocity) of one scene, sorted order or by the scene-local ids.
int sphb_get_scene(sph_batch* b, uint32_t scene, float* xyz, float* vel, float* rho,
                   int32_t order) {
    if (!b || scene >= b->S) return fail(SPH_E_INVALID, "sphb_get_scene: bad handle or scene");
    if (order != SPH_ORDER_SORTED && order != SPH_ORDER_BY_ID)
        return fail(SPH_E_INVALID, "sphb_get_scene: bad order");
    int rc = sphb_sync(b);
    if (rc != SPH_OK) return rc;
    const SceneRec& R = b->recs_h[scene];
    const uint32_t n = R.p_n;
    std::vector<float4> hp(n), hv(n);
    std::vector<float> hr(n);
    if (n) {
        SPH_CUDA(cudaMemcpy(hp.data(), b->pos + R.p_off, 16 * (size_t)n, cudaMemcpyDeviceToHost));
        SPH_CUDA(cudaMemcpy(hv.data(), b->vel + R.p_off, 16 * (size_t)n, cudaMemcpyDeviceToHost));
        SPH_CUDA(cudaMemcpy(hr.data(), b->rho + R.p_off, 4 * (size_t)n, cudaMemcpyDeviceToHost));
    }
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t d = k;
        if (order == SPH_ORDER_BY_ID) std::memcpy(&d, &hp[k].w, 4);
        if (d >= n) return fail(SPH_E_INVALID, "corrupt persistent id");
        if (xyz) {
            xyz[3 * d] = hp[k].x;
            xyz[3 * d + 1] = hp[k].y;
            xyz[3 * d + 2] = hp[k].z;
        }
        if (vel) {
            vel[3 * d] = hv[k].x;
            vel[3 * d + 1] = hv[k].y;
            vel[3 * d + 2] = hv[k].z;
        }
        if (rho) rho[d] = hr[k];
    }
    return SPH_OK;
}

// Picks the block size of the density and force passes (128, 256 or 512
// threads) and the persistent grid (2, 4 or 8 blocks per SM) by timing each
// candidate on the batch's own data; the particle state is restored after.
int sphb_autotune(sph_batch* b, float dt, int32_t* choice) {
    if (!b) return fail(SPH_E_INVALID, "sphb_autotune: NULL handle");
    if (b->N == 0) return SPH_OK;
    SPH_CUDA(cudaStreamSynchronize(b->stream));
    float4 *p0 = nullptr, *v0 = nullptr;
    SPH_CUDA(cudaMalloc(&p0, 16 * (size_t)b->N));
    SPH_CUDA(cudaMalloc(&v0, 16 * (size_t)b->N));
    cudaMemcpyAsync(p0, b->pos, 16 * (size_t)b->N, cudaMemcpyDeviceToDevice, b->stream);
    cudaMemcpyAsync(v0, b->vel, 16 * (size_t)b->N, cudaMemcpyDeviceToDevice, b->stream);
    cudaEvent_t e0, e1, e2;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&e2);
    const int mults[3] = {2, 4, 8};
    float best_d = 1e30f, best_f = 1e30f;
    int bd = 1, bf = 1, bm = 4;
    float best_total = 1e30f;
    for (int m : mults) {
        b->grid_mult = m;
        for (int k = 0; k < 3; ++k) {
            b->bs_density = b->bs_force = k;
            float td = 0.f, tf = 0.f;
            for (int rep = 0; rep < 3; ++rep) {
                enqueue_neighborhood(b);
                cudaEventRecord(e0, b->stream);
                enqueue_density(b);
                cudaEventRecord(e1, b->stream);
                enqueue_force(b, dt);
                cudaEventRecord(e2, b->stream);
                cudaEventSynchronize(e2);
                float a = 0.f, c = 0.f;
                cudaEventElapsedTime(&a, e0, e1);
                cudaEventElapsedTime(&c, e1, e2);
                if (rep > 0) {
                    td += a;
                    tf += c;
                }
                cudaMemcpyAsync(b->pos, p0, 16 * (size_t)b->N, cudaMemcpyDeviceToDevice, b->stream);
                cudaMemcpyAsync(b->vel, v0, 16 * (size_t)b->N, cudaMemcpyDeviceToDevice, b->stream);
            }
            if (td < best_d) best_d = td, bd = k;
            if (tf < best_f) best_f = tf, bf = k;
            if (td + tf < best_total) best_total = td + tf, bm = m;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    cudaStreamSynchronize(b->stream);
    cudaFree(p0);
    cudaFree(v0);
    b->bs_density = bd;
    b->bs_force = bf;
    b->grid_mult = bm;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    if (choice) {
        choice[0] = kBlockChoices[bd];
        choice[1] = kBlockChoices[bf];
        choice[2] = bm;
    }
    SPH_CUDA(cudaGetLastError());
    return check_err(b);
}

int sphb_destroy(sph_batch* b) { return free_batch(b); }

}  // extern "C"
