// two_scale.cu -- the two-scale solver handle behind the C ABI.
//
// Replaces the two-scale Solver (SPH2S_FINAL_TWO_SCALE/Solver.h:64-144,
// Solver.cu:1333-1771).  Step order follows Solver::Advance (Solver.cu:1568-1614):
// neighbourhoods of both populations, densities, accelerations, integration;
// split children and merged particles are placed by prefix-sum compaction
// instead of the reference's atomicAdd re-listing, so every step is
// deterministic.  The host reads the new population sizes back after each
// step, as the reference does (Solver.cu:1633-1638).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "errors.h"
#include "state_format.h"
#include "host_params.h"
#include "radix_sort.cuh"
#include "scan.cuh"
#include "boundary_tables.cuh"
#include "single_scale_kernels.cuh"
#include "two_scale_kernels.cuh"

using namespace sph;

namespace {

struct Pop {
    uint32_t n = 0, cap = 0, ncells = 0;
    int key_bits = 0;
    float4 *pos = nullptr, *vel = nullptr;
    int32_t* stt = nullptr;
    uint32_t* grp = nullptr;
    float4 *spos = nullptr, *svel = nullptr;
    int32_t* sstt = nullptr;
    uint32_t* sgrp = nullptr;
    float* rho = nullptr;
    float2* aux = nullptr;
    float4 *ipos = nullptr, *ivel = nullptr;
    int32_t* istt = nullptr;
    uint32_t *igrp = nullptr, *keep = nullptr, *off = nullptr, *split = nullptr, *soff = nullptr;
    uint2* cells = nullptr;
    uint4* list = nullptr;           // same-population force neighbours, kMaxNbr per particle
    uint32_t* list_count = nullptr;
    uint4* clist = nullptr;          // complementary force neighbours, ComplCap per particle
    uint32_t* clist_count = nullptr;
    float4* bacc = nullptr;          // boundary force sums of the step (boundary_force_kernel)
};

template <class T>
int dalloc(T** p, size_t count, std::vector<void*>& owned) {
    SPH_CUDA(cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)));
    owned.push_back(*p);
    return SPH_OK;
}

inline uint32_t blocks_for(uint32_t n, uint32_t t = 256) { return (n + t - 1) / t; }

}  // namespace

struct sph_solver2 {
    sph_config2 cfg;
    TSParams P;
    cudaStream_t stream = nullptr;
    Pop pop[2];
    uint32_t nb = 0;
    float4* bpos = nullptr;
    uint2* bcells = nullptr;
    uint8_t* bnear = nullptr;  // per LOW cell: a boundary particle within stencil reach
    BoundaryTables btab;       // static tables of the boundary force pass (LOW grid)
    SimParams BP;              // the boundary force's constants: LOW grid, h, threshold, weights
    int sms = 0;
    cudaStream_t side = nullptr;  // second branch of the step: the boundary force
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaStream_t lowst = nullptr;  // the LOW density and force passes, beside the HIGH ones
    cudaEvent_t pfork = nullptr, pjoin = nullptr;
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* vals[2] = {nullptr, nullptr};
    void* sort_mem = nullptr;
    SortScratch sort;
    uint32_t* scan_scratch = nullptr;
    uint32_t* tot = nullptr;
    uint32_t cap_groups = 0;
    unsigned long long* gsum = nullptr;
    uint32_t* gready = nullptr;
    uint32_t* gmerge = nullptr;
    uint32_t* moff = nullptr;
    unsigned long long* gacc = nullptr;
    uint32_t* ctl = nullptr;
    uint32_t* ctl_host = nullptr;
    uint32_t* err = nullptr;
    uint32_t group_base = 0;
    uint32_t stats[6] = {0, 0, 0, 0, 0, 0};
    uint32_t next_id[2] = {0, 0};  // persistent id of the next particle created (LOW, HIGH)
    uint64_t step = 0;             // steps advanced since creation
    float* colour[2] = {nullptr, nullptr};  // colour output of the last step
    bool colour_on = false;
    uint32_t colour_n[2] = {0, 0};          // particles of that step per population
    std::vector<void*> owned;
};

namespace {

int free_solver2(sph_solver2* s) {
    if (!s) return SPH_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->side) cudaStreamSynchronize(s->side);
    if (s->lowst) cudaStreamSynchronize(s->lowst);
    if (s->pfork) cudaEventDestroy(s->pfork);
    if (s->pjoin) cudaEventDestroy(s->pjoin);
    if (s->lowst) cudaStreamDestroy(s->lowst);
    for (void* p : s->owned) cudaFree(p);
    for (void* p : {(void*)s->btab.start, (void*)s->btab.cand})
        if (p) cudaFree(p);
    if (s->fork) cudaEventDestroy(s->fork);
    if (s->join) cudaEventDestroy(s->join);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->ctl_host) cudaFreeHost(s->ctl_host);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return SPH_OK;
}

int make_ts_params(const sph_config2& c, TSParams* out) {
    for (int r = 0; r < 2; ++r) {
        int rc = validate_grid(c.grid[r], "sph_config2");
        if (rc != SPH_OK) return rc;
        if (!(c.effective_radius[r] > 0.0f) || !(c.fluid_particle_mass[r] > 0.0f))
            return fail(SPH_E_INVALID, "sph_config2: radii and masses must be positive");
    }
    if (c.refine_axis > 2) return fail(SPH_E_INVALID, "sph_config2: refine_axis must be -1..2");
    if (c.mode != SPH2_MODE_BLENDED && c.mode != SPH2_MODE_COUPLED)
        return fail(SPH_E_INVALID, "sph_config2: unknown mode");
    if (c.split_trigger != SPH2_SPLIT_SLAB && c.split_trigger != SPH2_SPLIT_SURFACE)
        return fail(SPH_E_INVALID, "sph_config2: unknown split trigger");
    if (c.split_trigger == SPH2_SPLIT_SURFACE && !(c.surface_density > 0.0f))
        return fail(SPH_E_INVALID, "sph_config2: surface_density must be positive");
    const double pi = 3.14159265358979323846;
    TSParams P;
    for (int r = 0; r < 2; ++r) {
        const double h = c.effective_radius[r], h3 = h * h * h;
        P.g[r] = make_grid_params(c.grid[r]);
        P.h[r] = c.effective_radius[r];
        P.h2[r] = P.h[r] * P.h[r];
        P.T[r] = neighbor_threshold(P.h[r]);
        P.mass[r] = c.fluid_particle_mass[r];
        P.poly6[r] = (float)(315.0 / (64.0 * pi * h3 * h3 * h3));
        P.spiky[r] = (float)(45.0 / (pi * h3 * h3));
    }
    const double m0 = c.fluid_particle_mass[0], mb = c.boundary_particle_mass;
    P.rho0 = c.rest_density;
    P.bulk = c.bulk_modulus;
    P.mu = c.viscosity;
    P.sigma = c.tension_coefficient;
    P.bnd_coef = (float)(0.02 * (double)c.speed_sound * c.speed_sound * mb / (m0 + mb));
    P.two_over_h0 = (float)(2.0 / (double)c.effective_radius[0]);
    P.gravity = -9.81f;
    P.blend_inc = c.blend_increment;
    P.coupled = c.mode == SPH2_MODE_COUPLED ? 1 : 0;
    P.surface = (!P.coupled && c.split_trigger == SPH2_SPLIT_SURFACE) ? 1 : 0;
    P.surf_rho = c.surface_density;
    P.axis = (P.coupled || P.surface) ? -1 : c.refine_axis;
    P.lo = c.refine_lo;
    P.hi = c.refine_hi;
    P.lo43 = std::llrint((double)c.refine_lo * 8796093022208.0);
    P.hi43 = std::llrint((double)c.refine_hi * 8796093022208.0);
    P.bmargin = boundary_margin(P.g[0], P.h[0]);
    *out = P;
    return SPH_OK;
}

int alloc_pop(Pop& p, uint32_t cap, const sph_grid& g, uint32_t compl_cap, std::vector<void*>& o) {
    p.cap = cap;
    p.ncells = sph_grid_num_cells(&g);
    p.key_bits = 3 * morton_bits_for(g);
    int rc = SPH_OK;
    if ((rc = dalloc(&p.pos, cap, o)) || (rc = dalloc(&p.vel, cap, o)) ||
        (rc = dalloc(&p.stt, cap, o)) || (rc = dalloc(&p.grp, cap, o)) ||
        (rc = dalloc(&p.spos, cap, o)) || (rc = dalloc(&p.svel, cap, o)) ||
        (rc = dalloc(&p.sstt, cap, o)) || (rc = dalloc(&p.sgrp, cap, o)) ||
        (rc = dalloc(&p.rho, cap, o)) || (rc = dalloc(&p.aux, cap, o)) ||
        (rc = dalloc(&p.ipos, cap, o)) || (rc = dalloc(&p.ivel, cap, o)) ||
        (rc = dalloc(&p.istt, cap, o)) || (rc = dalloc(&p.igrp, cap, o)) ||
        (rc = dalloc(&p.keep, cap, o)) || (rc = dalloc(&p.off, cap, o)) ||
        (rc = dalloc(&p.split, cap, o)) || (rc = dalloc(&p.soff, cap, o)) ||
        (rc = dalloc(&p.cells, p.ncells, o)) ||
        (rc = dalloc(&p.list, (size_t)cap * (kMaxNbr / 4), o)) ||
        (rc = dalloc(&p.list_count, cap, o)) ||
        (rc = dalloc(&p.clist, (size_t)cap * (compl_cap / 4), o)) ||
        (rc = dalloc(&p.clist_count, cap, o)) || (rc = dalloc(&p.bacc, cap, o)))
        return rc;
    return SPH_OK;
}

TSOut outputs(Pop& p, float* acc, uint32_t* nbr_bnd, float* colour = nullptr) {
    TSOut o;
    o.colour = colour;
    o.ipos = p.ipos;
    o.ivel = p.ivel;
    o.istt = p.istt;
    o.igrp = p.igrp;
    o.keep = p.keep;
    o.split = p.split;
    o.acc = acc;
    o.nbr_bnd = nbr_bnd;
    return o;
}

// hash -> sort -> reorder + cell ranges of both populations (Solver.cu:1616-1680):
// one stable sort of (population bit, cell key) pairs gives each population the
// order of its own sort with half the sort launches.
void ts_neighborhoods(sph_solver2* s) {
    Pop &L = s->pop[0], &H = s->pop[1];
    cudaStream_t st = s->stream;
    cudaMemsetAsync(H.cells, 0xFF, sizeof(uint2) * H.ncells, st);
    cudaMemsetAsync(L.cells, 0xFF, sizeof(uint2) * L.ncells, st);
    const uint32_t n = L.n + H.n;
    if (n == 0) return;
    const int pop_bit = std::max(L.key_bits, H.key_bits);
    const int passes = sort_passes(pop_bit + 1);
    sort_reset(s->sort, st);
    uint32_t hb = blocks_for(n);
    if (hb > 1216) hb = 1216;
    ts_hash_hist_kernel<<<hb, 256, 0, st>>>(L.pos, L.n, s->P.g[0], H.pos, H.n, s->P.g[1], pop_bit,
                                            passes, s->keys[0], s->sort.hist);
    sort_scan(passes, s->sort, st);
    const int o = sort_passes_run(s->keys, s->vals, nullptr, n, passes, s->sort, s->err, 0, st);
    const uint32_t mask = (1u << pop_bit) - 1u;
    if (H.n)
        ts_gather_kernel<true><<<blocks_for(H.n), 256, 0, st>>>(
            s->keys[o] + L.n, s->vals[o] + L.n, H.n, mask, L.n, s->P.g[1], H.pos, H.vel, H.stt,
            H.grp, H.spos, H.svel, H.sstt, H.sgrp, H.cells, s->err, s->P.axis, s->P.surface,
            s->group_base, s->gsum, s->gready);
    if (L.n)
        ts_gather_kernel<false><<<blocks_for(L.n), 256, 0, st>>>(
            s->keys[o], s->vals[o], L.n, mask, 0u, s->P.g[0], L.pos, L.vel, L.stt, L.grp, L.spos,
            L.svel, L.sstt, L.sgrp, L.cells, s->err, -1, 0, 0, nullptr, nullptr);
}

// Everything up to and including the force/integrate pass; DEBUG variants
// also write accelerations and neighbour counts of population `dbg_pop`.
void ts_front(sph_solver2* s, float dt, bool debug, int dbg_pop, uint32_t* dnb_same,
              uint32_t* dnb_compl, float* dacc, uint32_t* dnb_bnd) {
    cudaStream_t st = s->stream;
    const uint32_t gb = s->group_base;
    if (gb) {
        cudaMemsetAsync(s->gsum, 0, 8 * (size_t)gb, st);
        cudaMemsetAsync(s->gready, 0, 4 * (size_t)gb, st);
        cudaMemsetAsync(s->gacc, 0, 48 * (size_t)gb, st);
    }
    cudaMemsetAsync(s->ctl + kCtlFadedL, 0, 8, st);
    ts_neighborhoods(s);
    Pop &L = s->pop[0], &H = s->pop[1];
    // the boundary force sums of both populations on the second branch, beside
    // the density passes (they need only the sorted positions)
    const bool bsep = !debug;
    if (bsep) {
        cudaEventRecord(s->fork, st);
        cudaStreamWaitEvent(s->side, s->fork, 0);
        for (Pop* p : {&H, &L})
            if (p->n)
                boundary_force_kernel<<<blocks_for(p->n), 256, 0, s->side>>>(
                    p->spos, s->bpos, s->bcells, s->btab.start, s->btab.cand, nullptr, nullptr,
                    p->n, s->nb, s->BP, p->bacc, s->bnear);
        cudaEventRecord(s->join, s->side);
    }
    // The HIGH and LOW passes read only the step's sorted copies of both
    // populations and write their own population's outputs (their shared
    // group and step counters are integer atomics, whose sums do not depend
    // on order), so the LOW passes run on a second stream beside the HIGH
    // ones and fill the SMs the smaller population's waves leave idle;
    // results are those of running them one after the other.
    cudaStream_t lo = s->lowst;
    cudaEventRecord(s->pfork, st);
    cudaStreamWaitEvent(lo, s->pfork, 0);
    if (H.n) {
        if (debug && dbg_pop == 1)
            ts_density_kernel<1, true><<<blocks_for(H.n), 256, 0, st>>>(
                H.spos, H.cells, H.n, L.spos, L.cells, L.n, s->P, H.rho, H.aux, dnb_same, dnb_compl,
                H.sgrp, gb, s->gsum, H.list, H.list_count, H.clist, H.clist_count);
        else
            ts_density_kernel<1, false><<<blocks_for(H.n), 256, 0, st>>>(
                H.spos, H.cells, H.n, L.spos, L.cells, L.n, s->P, H.rho, H.aux, nullptr, nullptr,
                H.sgrp, gb, s->gsum, H.list, H.list_count, H.clist, H.clist_count);
    }
    if (L.n) {
        if (debug && dbg_pop == 0)
            ts_density_kernel<0, true><<<blocks_for(L.n), 256, 0, lo>>>(
                L.spos, L.cells, L.n, H.spos, H.cells, H.n, s->P, L.rho, L.aux, dnb_same, dnb_compl,
                L.sgrp, gb, s->gsum, L.list, L.list_count, L.clist, L.clist_count);
        else
            ts_density_kernel<0, false><<<blocks_for(L.n), 256, 0, lo>>>(
                L.spos, L.cells, L.n, H.spos, H.cells, H.n, s->P, L.rho, L.aux, nullptr, nullptr,
                L.sgrp, gb, s->gsum, L.list, L.list_count, L.clist, L.clist_count);
    }
    cudaEventRecord(s->pjoin, lo);
    cudaStreamWaitEvent(st, s->pjoin, 0);
    // merge decisions (slab: start-of-step centroids; surface: this step's densities)
    if (gb && (s->P.axis >= 0 || s->P.surface))
        ts_group_decide_kernel<<<blocks_for(gb), 256, 0, st>>>(s->gsum, s->gready, gb, s->P.lo43,
                                                               s->P.hi43, s->P.surface, s->gmerge);
    else if (gb)
        cudaMemsetAsync(s->gmerge, 0, 4 * (size_t)gb, st);
    const uint32_t* gm = gb ? s->gmerge : nullptr;
    if (bsep) cudaStreamWaitEvent(st, s->join, 0);
    cudaEventRecord(s->pfork, st);
    cudaStreamWaitEvent(lo, s->pfork, 0);
    if (H.n) {
        TSOut o = outputs(H, dacc, dnb_bnd, (s->colour_on && !debug) ? s->colour[1] : nullptr);
        if (debug && dbg_pop == 1)
            ts_force_kernel<1, true><<<blocks_for(H.n), 256, 0, st>>>(
                H.spos, H.svel, H.sstt, H.sgrp, H.aux, H.cells, H.n, L.spos, L.svel, L.aux, L.cells,
                L.n, s->bpos, s->bcells, s->bnear, s->nb, s->P, dt, gm, gb, s->gacc, s->ctl, H.rho, H.list, H.list_count, H.clist, H.clist_count, o, nullptr);
        else
            ts_force_kernel<1, false><<<blocks_for(H.n), 256, 0, st>>>(
                H.spos, H.svel, H.sstt, H.sgrp, H.aux, H.cells, H.n, L.spos, L.svel, L.aux, L.cells,
                L.n, s->bpos, s->bcells, s->bnear, s->nb, s->P, dt, gm, gb, s->gacc, s->ctl, H.rho, H.list, H.list_count, H.clist, H.clist_count, o, bsep ? H.bacc : nullptr);
    }
    if (L.n) {
        TSOut o = outputs(L, dacc, dnb_bnd, (s->colour_on && !debug) ? s->colour[0] : nullptr);
        if (debug && dbg_pop == 0)
            ts_force_kernel<0, true><<<blocks_for(L.n), 256, 0, lo>>>(
                L.spos, L.svel, L.sstt, L.sgrp, L.aux, L.cells, L.n, H.spos, H.svel, H.aux, H.cells,
                H.n, s->bpos, s->bcells, s->bnear, s->nb, s->P, dt, gm, gb, s->gacc, s->ctl, L.rho, L.list, L.list_count, L.clist, L.clist_count, o, nullptr);
        else
            ts_force_kernel<0, false><<<blocks_for(L.n), 256, 0, lo>>>(
                L.spos, L.svel, L.sstt, L.sgrp, L.aux, L.cells, L.n, H.spos, H.svel, H.aux, H.cells,
                H.n, s->bpos, s->bcells, s->bnear, s->nb, s->P, dt, gm, gb, s->gacc, s->ctl, L.rho, L.list, L.list_count, L.clist, L.clist_count, o, bsep ? L.bacc : nullptr);
    }
    cudaEventRecord(s->pjoin, lo);
    cudaStreamWaitEvent(st, s->pjoin, 0);
}

int check_err2(sph_solver2* s) {
    uint32_t e = 0;
    SPH_CUDA(cudaMemcpyAsync(&e, s->err, 4, cudaMemcpyDeviceToHost, s->stream));
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    if (e) {
        SPH_CUDA(cudaMemsetAsync(s->err, 0, 4, s->stream));
        SPH_CUDA(cudaStreamSynchronize(s->stream));
        if (e & kErrLookbackTimeout)
            return fail(SPH_E_TIMEOUT, "radix sort look-back timed out; step results are invalid");
        if (e & 4u)
            return fail(SPH_E_CAPACITY, "two-scale step exceeded a particle or group capacity");
        return fail(SPH_E_CAPACITY, "device-side index check failed");
    }
    return SPH_OK;
}

int ts_step(sph_solver2* s, float dt) {
    cudaStream_t st = s->stream;
    Pop &L = s->pop[0], &H = s->pop[1];
    const uint32_t gb = s->group_base;
    ts_front(s, dt, false, 0, nullptr, nullptr, nullptr, nullptr);
    // compaction: the prefix sums over keep / split / merge flags, in one batch
    const ScanSeg segs[4] = {{H.keep, H.off, H.n, s->tot + 0},
                             {L.keep, L.off, L.n, s->tot + 1},
                             {L.split, L.soff, L.n, s->tot + 2},
                             {s->gmerge, s->moff, gb, s->tot + 3}};
    scan_exclusive_batch(segs, 4, s->scan_scratch, st);
    ts_totals_kernel<<<1, 1, 0, st>>>(s->tot, H.n, L.n, H.cap, L.cap, s->cap_groups, s->ctl, s->err);
    {
        const TSState hs = {H.pos, H.vel, H.stt, H.grp, H.cap};
        const TSState ls = {L.pos, L.vel, L.stt, L.grp, L.cap};
        const uint32_t work = H.n + L.n + gb;
        if (work)
            ts_finish_kernel<<<blocks_for(work), 256, 0, st>>>(
                outputs(H, nullptr, nullptr), H.off, H.n, outputs(L, nullptr, nullptr), L.off,
                L.soff, L.rho, L.n, s->P.mass[0], s->gmerge, s->moff, s->gacc, gb, s->ctl, hs, ls);
    }
    ts_advance_counters_kernel<<<1, 1, 0, st>>>(s->ctl, s->cap_groups, s->err);
    SPH_CUDA(cudaGetLastError());
    SPH_CUDA(cudaMemcpyAsync(s->ctl_host, s->ctl, 4 * kCtlWords, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(cudaStreamSynchronize(st));
    const uint32_t* c = s->ctl_host;
    s->stats[0] = c[kCtlSplits];
    s->stats[1] = c[kCtlMerges];
    s->stats[2] = L.n - c[kCtlSurvL];
    s->stats[3] = H.n - c[kCtlSurvH];
    s->stats[4] = c[kCtlFadedL];
    s->stats[5] = c[kCtlFadedH];
    s->colour_n[0] = L.n;
    s->colour_n[1] = H.n;
    H.n = c[kCtlNextH];
    L.n = c[kCtlNextL];
    s->group_base = c[kCtlGroupBase];
    s->next_id[0] = c[kCtlPidL];
    s->next_id[1] = c[kCtlPidH];
    // the error word came back with the counts: no second round trip unless set
    return c[kCtlErr] ? check_err2(s) : SPH_OK;
}

// Host copy of one population's persistent state, in the order the next
// step starts from: position (persistent id in w), velocity (blend
// coefficient lambda in w), state bits, group id.
struct HostPop {
    std::vector<float4> pos, vel;
    std::vector<int32_t> stt;
    std::vector<uint32_t> grp;
};

HostPop initial_pop(int r, const float* xyz, uint32_t n) {
    HostPop h;
    h.pos.resize(n);
    h.vel.assign(n, make_float4(0.f, 0.f, 0.f, 1.0f));  // lambda starts at 1 (Solver.cu:1371)
    h.stt.assign(n, r == 1 ? 4 : 0);  // HIGH states start at 4 (Solver.cu:1537-1543)
    h.grp.assign(n, kNoGroup);
    for (uint32_t i = 0; i < n; ++i) {
        float w;
        std::memcpy(&w, &i, 4);
        h.pos[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], w);
    }
    return h;
}

int upload_pop(sph_solver2* s, int r, const HostPop& h) {
    Pop& p = s->pop[r];
    const uint32_t n = (uint32_t)h.pos.size();
    if (n) {
        SPH_CUDA(cudaMemcpy(p.pos, h.pos.data(), 16 * (size_t)n, cudaMemcpyHostToDevice));
        SPH_CUDA(cudaMemcpy(p.vel, h.vel.data(), 16 * (size_t)n, cudaMemcpyHostToDevice));
        SPH_CUDA(cudaMemcpy(p.stt, h.stt.data(), 4 * (size_t)n, cudaMemcpyHostToDevice));
        SPH_CUDA(cudaMemcpy(p.grp, h.grp.data(), 4 * (size_t)n, cudaMemcpyHostToDevice));
    }
    p.n = n;
    return SPH_OK;
}

// Allocates a handle for capacities capL / capH, uploads both populations,
// sets the group and id counters and presorts the boundary (float4, ordered
// by depth outside the LOW grid's box with the depth in w) on the LOW grid.
int create_solver2(const sph_config2* config, const TSParams& P, uint64_t capL, uint64_t capH,
                   const HostPop* pops, const float4* hb, uint32_t n_boundary,
                   uint32_t group_base, const uint32_t next_id[2], uint64_t step,
                   sph_solver2** out) {
    // both populations share one sort, whose look-back counts hold 30 bits
    if (capL + capH > kMaxParticles || n_boundary > kMaxParticles)
        return fail(SPH_E_CAPACITY, "two-scale: more than 2^30 particles");
    sph_solver2* s = new sph_solver2();
    s->cfg = *config;
    s->P = P;
    s->nb = n_boundary;
    s->next_id[0] = next_id[0];
    s->next_id[1] = next_id[1];
    s->group_base = group_base;
    s->step = step;
    s->cap_groups = (uint32_t)(capH / 8 * 4 + 64);
#define TRY(x)                                 \
    do {                                       \
        int _r = (x);                          \
        if (_r != SPH_OK) {                    \
            std::string m = sph_last_error();  \
            free_solver2(s);                   \
            return fail(_r, m);                \
        }                                      \
    } while (0)
    if (group_base > s->cap_groups) {
        free_solver2(s);
        return fail(SPH_E_INVALID, "two-scale state: group counter beyond the group capacity");
    }
    TRY(check_cuda(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "stream", __FILE__, __LINE__));
    TRY(check_cuda(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking), "stream", __FILE__, __LINE__));
    TRY(check_cuda(cudaStreamCreateWithFlags(&s->lowst, cudaStreamNonBlocking), "stream", __FILE__, __LINE__));
    TRY(check_cuda(cudaEventCreateWithFlags(&s->pfork, cudaEventDisableTiming), "event", __FILE__, __LINE__));
    TRY(check_cuda(cudaEventCreateWithFlags(&s->pjoin, cudaEventDisableTiming), "event", __FILE__, __LINE__));
    TRY(check_cuda(cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming), "event", __FILE__, __LINE__));
    TRY(check_cuda(cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming), "event", __FILE__, __LINE__));
    {
        int dev = 0;
        TRY(check_cuda(cudaGetDevice(&dev), "device", __FILE__, __LINE__));
        TRY(check_cuda(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev), "device", __FILE__, __LINE__));
    }
    // the boundary force uses the LOW grid, radius and threshold for both populations
    s->BP = SimParams{};
    s->BP.g = P.g[0];
    s->BP.h = P.h[0];
    s->BP.h2 = P.h2[0];
    s->BP.T = P.T[0];
    s->BP.bnd_coef = P.bnd_coef;
    s->BP.two_over_h = P.two_over_h0;
    s->BP.bmargin = P.bmargin;
    TRY(alloc_pop(s->pop[0], (uint32_t)capL, config->grid[0], ComplCap<0>::value, s->owned));
    TRY(alloc_pop(s->pop[1], (uint32_t)capH, config->grid[1], ComplCap<1>::value, s->owned));
    // one sort holds both populations (ts_neighborhoods), or the boundary at creation
    const uint32_t nmax = (uint32_t)std::max<uint64_t>(capL + capH, n_boundary);
    for (int b = 0; b < 2; ++b) {
        TRY(dalloc(&s->keys[b], nmax, s->owned));
        TRY(dalloc(&s->vals[b], nmax, s->owned));
    }
    TRY(check_cuda(cudaMalloc(&s->sort_mem, sort_scratch_bytes(nmax)), "sort scratch", __FILE__, __LINE__));
    s->owned.push_back(s->sort_mem);
    s->sort = sort_scratch_from(s->sort_mem, nmax);
    TRY(dalloc(&s->scan_scratch,
               scan_scratch_words((uint32_t)capH) + 2 * scan_scratch_words((uint32_t)capL) +
                   scan_scratch_words(s->cap_groups),
               s->owned));
    TRY(dalloc(&s->tot, 4, s->owned));
    TRY(dalloc(&s->gsum, s->cap_groups, s->owned));
    TRY(dalloc(&s->gready, s->cap_groups, s->owned));
    TRY(dalloc(&s->gmerge, s->cap_groups, s->owned));
    TRY(dalloc(&s->moff, s->cap_groups, s->owned));
    TRY(dalloc(&s->gacc, 6 * (size_t)s->cap_groups, s->owned));
    TRY(dalloc(&s->ctl, kCtlWords, s->owned));
    TRY(dalloc(&s->err, 1, s->owned));
    TRY(dalloc(&s->bpos, n_boundary, s->owned));
    TRY(dalloc(&s->bcells, s->pop[0].ncells, s->owned));
    TRY(dalloc(&s->bnear, s->pop[0].ncells, s->owned));
    TRY(check_cuda(cudaMallocHost((void**)&s->ctl_host, 4 * kCtlWords), "pinned", __FILE__, __LINE__));
    TRY(check_cuda(cudaMemset(s->err, 0, 4), "memset", __FILE__, __LINE__));
    {
        uint32_t c0[kCtlWords] = {0};
        c0[kCtlPidH] = next_id[1];
        c0[kCtlPidL] = next_id[0];
        c0[kCtlGroupBase] = group_base;
        TRY(check_cuda(cudaMemcpy(s->ctl, c0, sizeof(c0), cudaMemcpyHostToDevice), "ctl", __FILE__, __LINE__));
    }
    for (int b = 0; b < 2; ++b) {
        TRY(check_cuda(cudaMemset(s->keys[b], 0, 4 * (size_t)nmax), "memset", __FILE__, __LINE__));
        TRY(check_cuda(cudaMemset(s->vals[b], 0, 4 * (size_t)nmax), "memset", __FILE__, __LINE__));
    }
    TRY(upload_pop(s, 0, pops[0]));
    TRY(upload_pop(s, 1, pops[1]));
    // boundary: sorted once on the LOW grid (SPH2S_FINAL_TWO_SCALE/Solver.cu:1469-1527)
    TRY(check_cuda(cudaMemset(s->bcells, 0xFF, sizeof(uint2) * s->pop[0].ncells), "memset", __FILE__, __LINE__));
    if (n_boundary) {
        float4* braw = nullptr;
        cudaError_t e = cudaMalloc(&braw, 16 * (size_t)n_boundary);
        if (e == cudaSuccess) e = cudaMemcpy(braw, hb, 16 * (size_t)n_boundary, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            // keys (cell, depth class): the order boundary_reach's cut needs
            const int qb = boundary_depth_bits(s->P.g[0], s->P.h[0], s->pop[0].key_bits);
            const int passes = sort_passes(s->pop[0].key_bits + qb);
            sort_reset(s->sort, s->stream);
            uint32_t hbk = blocks_for(n_boundary);
            if (hbk > 1216) hbk = 1216;
            boundary_hash_hist_kernel<<<hbk, 256, 0, s->stream>>>(
                braw, n_boundary, s->P.g[0], qb, boundary_quantum(s->P.h[0]), passes, s->keys[0],
                s->sort.hist);
            sort_scan(passes, s->sort, s->stream);
            const int o = sort_passes_run(s->keys, s->vals, nullptr, n_boundary, passes, s->sort,
                                          s->err, 0, s->stream);
            gather_cells_kernel<false><<<blocks_for(n_boundary), 256, 0, s->stream>>>(
                s->keys[o], s->vals[o], n_boundary, s->P.g[0], braw, nullptr, s->bpos, nullptr,
                s->bcells, s->err, qb);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        }
        if (braw) cudaFree(braw);
        TRY(check_cuda(e, "boundary presort", __FILE__, __LINE__));
    }
    {
        const int reach = (int)std::ceil(s->cfg.effective_radius[0] / s->cfg.grid[0].spacing) + 1;
        boundary_near_kernel<<<blocks_for(s->pop[0].ncells), 256, 0, s->stream>>>(
            s->bcells, s->P.g[0], reach, s->bnear);
        TRY(check_cuda(cudaGetLastError(), "boundary flags", __FILE__, __LINE__));
        TRY(check_cuda(build_boundary_tables(s->bcells, s->bpos, s->bnear, s->P.g[0], s->pop[0].ncells,
                                             n_boundary, s->P.h[0], s->P.bmargin, s->stream, s->btab),
                       "boundary tables", __FILE__, __LINE__));
        TRY(check_cuda(cudaStreamSynchronize(s->stream), "create sync", __FILE__, __LINE__));
    }
    TRY(check_err2(s));
#undef TRY
    *out = s;
    return SPH_OK;
}

uint64_t ts_state_bytes(uint64_t n_low, uint64_t n_high, uint64_t nb) {
    return sizeof(sph_io::StatePrefix) + sizeof(sph_config2) + 24 + 16 +
           40 * (n_low + n_high) + 16 * nb + 8;
}

}  // namespace

extern "C" {

// SolverConfiguration::MakeConfiguration of the two-scale project
// (SPH2S_FINAL_TWO_SCALE/Solver.h:16-50): h1 = h0/2, m1 = m0/8, one grid per
// radius; refinement disabled (refine_axis = -1).
int sph_make_configuration2(const float origin[3], const float end[3], float volume,
                            uint32_t num_particles, uint32_t avg_particles, float rest_density,
                            float bulk_modulus, float viscosity, float speed_sound,
                            float tension_coefficient, float blend_increment, sph_config2* out) {
    if (!out) return fail(SPH_E_INVALID, "sph_make_configuration2: NULL output");
    sph_config c1;
    int rc = sph_make_configuration(origin, end, volume, num_particles, avg_particles,
                                    rest_density, bulk_modulus, viscosity, speed_sound,
                                    tension_coefficient, 0.0f, &c1);
    if (rc != SPH_OK) return rc;
    sph_config2 c;
    std::memset(&c, 0, sizeof(c));
    c.effective_radius[0] = c1.effective_radius;
    c.effective_radius[1] = 0.5f * c1.effective_radius;
    c.fluid_particle_mass[0] = c1.fluid_particle_mass;
    c.fluid_particle_mass[1] = 1.0f / 8.0f * c1.fluid_particle_mass;
    c.boundary_particle_mass = c1.fluid_particle_mass;
    c.rest_density = rest_density;
    c.bulk_modulus = bulk_modulus;
    c.viscosity = viscosity;
    c.speed_sound = speed_sound;
    c.tension_coefficient = tension_coefficient;
    c.blend_increment = blend_increment;
    c.grid[0] = c1.grid;
    rc = sph_make_grid(origin, end, c.effective_radius[1], &c.grid[1]);
    if (rc != SPH_OK) return rc;
    c.refine_axis = -1;
    *out = c;
    return SPH_OK;
}

int sph2_create(const sph_config2* config, const float* low_xyz, uint32_t n_low,
                const float* high_xyz, uint32_t n_high, const float* boundary_xyz,
                uint32_t n_boundary, uint32_t capacity_low, uint32_t capacity_high,
                sph_solver2** out) {
    if (!config || !out) return fail(SPH_E_INVALID, "sph2_create: NULL config or output handle");
    *out = nullptr;
    if ((n_low && !low_xyz) || (n_high && !high_xyz) || (n_boundary && !boundary_xyz))
        return fail(SPH_E_INVALID, "sph2_create: NULL particle array");
    TSParams P;
    int rc = make_ts_params(*config, &P);
    if (rc != SPH_OK) return rc;
    uint64_t capL = capacity_low ? capacity_low : 2ull * n_low + 1024;
    uint64_t capH = capacity_high ? capacity_high : 8ull * (n_low + n_high) + 1024;
    if (capL < n_low || capH < n_high) return fail(SPH_E_CAPACITY, "sph2_create: capacity below the initial count");
    if (capL + capH > kMaxParticles || n_boundary > kMaxParticles)
        return fail(SPH_E_CAPACITY, "sph2_create: more than 2^30 particles");
    HostPop pops[2] = {initial_pop(0, low_xyz, n_low), initial_pop(1, high_xyz, n_high)};
    std::vector<float4> hb(n_boundary);
    for (uint32_t i = 0; i < n_boundary; ++i) {
        float w;
        std::memcpy(&w, &i, 4);
        hb[i] = make_float4(boundary_xyz[3 * i], boundary_xyz[3 * i + 1], boundary_xyz[3 * i + 2], w);
    }
    const uint32_t next_id[2] = {n_low, n_high};
    return create_solver2(config, P, capL, capH, pops, hb.data(), n_boundary, 0, next_id, 0, out);
}

int sph2_advance(sph_solver2* s, float dt, int32_t steps) {
    if (!s) return fail(SPH_E_INVALID, "sph2_advance: NULL handle");
    if (steps < 0 || !(dt > 0.0f) || !std::isfinite(dt))
        return fail(SPH_E_INVALID, "sph2_advance: bad dt or steps");
    for (int k = 0; k < steps; ++k) {
        int rc = ts_step(s, dt);
        if (rc != SPH_OK) return rc;
        ++s->step;
    }
    return SPH_OK;
}

int sph2_counts(sph_solver2* s, uint32_t* n_low, uint32_t* n_high, uint32_t* n_boundary,
                uint32_t* groups) {
    if (!s) return fail(SPH_E_INVALID, "sph2_counts: NULL handle");
    if (n_low) *n_low = s->pop[0].n;
    if (n_high) *n_high = s->pop[1].n;
    if (n_boundary) *n_boundary = s->nb;
    if (groups) *groups = s->group_base;
    return SPH_OK;
}

int sph2_next_ids(sph_solver2* s, uint32_t* next_low, uint32_t* next_high) {
    if (!s) return fail(SPH_E_INVALID, "sph2_next_ids: NULL handle");
    if (next_low) *next_low = s->next_id[0];
    if (next_high) *next_high = s->next_id[1];
    return SPH_OK;
}

int sph2_last_stats(sph_solver2* s, uint32_t* stats) {
    if (!s || !stats) return fail(SPH_E_INVALID, "sph2_last_stats: NULL argument");
    std::memcpy(stats, s->stats, sizeof(s->stats));
    return SPH_OK;
}

int sph2_get_state(sph_solver2* s, int32_t population, float* xyz, float* vel, float* lambda,
                   int32_t* state, uint32_t* group, uint32_t* ids) {
    if (!s || population < 0 || population > 1)
        return fail(SPH_E_INVALID, "sph2_get_state: bad handle or population");
    Pop& p = s->pop[population];
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    const uint32_t n = p.n;
    std::vector<float4> hp(n), hv(n);
    if (n) {
        SPH_CUDA(cudaMemcpy(hp.data(), p.pos, 16 * (size_t)n, cudaMemcpyDeviceToHost));
        SPH_CUDA(cudaMemcpy(hv.data(), p.vel, 16 * (size_t)n, cudaMemcpyDeviceToHost));
        if (state) SPH_CUDA(cudaMemcpy(state, p.stt, 4 * (size_t)n, cudaMemcpyDeviceToHost));
        if (group) SPH_CUDA(cudaMemcpy(group, p.grp, 4 * (size_t)n, cudaMemcpyDeviceToHost));
    }
    for (uint32_t i = 0; i < n; ++i) {
        if (xyz) {
            xyz[3 * i] = hp[i].x;
            xyz[3 * i + 1] = hp[i].y;
            xyz[3 * i + 2] = hp[i].z;
        }
        if (vel) {
            vel[3 * i] = hv[i].x;
            vel[3 * i + 1] = hv[i].y;
            vel[3 * i + 2] = hv[i].z;
        }
        if (lambda) lambda[i] = hv[i].w;
        if (ids) std::memcpy(&ids[i], &hp[i].w, 4);
    }
    return SPH_OK;
}

int sph2_get_positions_device(sph_solver2* s, int32_t population, float* d_xyz) {
    if (!s || population < 0 || population > 1)
        return fail(SPH_E_INVALID, "sph2_get_positions_device: bad handle or population");
    Pop& p = s->pop[population];
    if (p.n == 0) return SPH_OK;
    if (!d_xyz) return fail(SPH_E_INVALID, "sph2_get_positions_device: NULL destination");
    int rc = sph::check_device_pointer(d_xyz, "sph2_get_positions_device");
    if (rc != SPH_OK) return rc;
    pack_xyz_kernel<<<blocks_for(p.n), 256, 0, s->stream>>>(p.pos, p.pos, p.n, 0, d_xyz);
    SPH_CUDA(cudaGetLastError());
    return SPH_OK;
}

int sph2_get_states_device(sph_solver2* s, int32_t population, int32_t* d_state) {
    if (!s || population < 0 || population > 1)
        return fail(SPH_E_INVALID, "sph2_get_states_device: bad handle or population");
    Pop& p = s->pop[population];
    if (p.n == 0) return SPH_OK;
    if (!d_state) return fail(SPH_E_INVALID, "sph2_get_states_device: NULL destination");
    int rc = sph::check_device_pointer(d_state, "sph2_get_states_device");
    if (rc != SPH_OK) return rc;
    SPH_CUDA(cudaMemcpyAsync(d_state, p.stt, 4 * (size_t)p.n, cudaMemcpyDeviceToDevice, s->stream));
    return SPH_OK;
}

int sph2_debug_step_fields(sph_solver2* s, int32_t population, uint32_t* ids_sorted, float* rho,
                           float* acc, uint32_t* nbr_same, uint32_t* nbr_compl,
                           uint32_t* nbr_boundary) {
    if (!s || population < 0 || population > 1)
        return fail(SPH_E_INVALID, "sph2_debug_step_fields: bad handle or population");
    Pop& p = s->pop[population];
    const uint32_t n = p.n;
    if (n == 0) return SPH_OK;
    float* dacc = nullptr;
    uint32_t *ds = nullptr, *dc = nullptr, *db = nullptr;
    SPH_CUDA(cudaMalloc(&dacc, 12 * (size_t)n));
    SPH_CUDA(cudaMalloc(&ds, 4 * (size_t)n));
    SPH_CUDA(cudaMalloc(&dc, 4 * (size_t)n));
    SPH_CUDA(cudaMalloc(&db, 4 * (size_t)n));
    ts_front(s, 1e-6f, true, population, ds, dc, dacc, db);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    std::vector<float4> sv;
    if (e == cudaSuccess && ids_sorted) {
        sv.resize(n);
        e = cudaMemcpy(sv.data(), p.svel, 16 * (size_t)n, cudaMemcpyDeviceToHost);
        for (uint32_t i = 0; i < n && e == cudaSuccess; ++i) std::memcpy(&ids_sorted[i], &sv[i].w, 4);
    }
    if (e == cudaSuccess && rho) e = cudaMemcpy(rho, p.rho, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && acc) e = cudaMemcpy(acc, dacc, 12 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && nbr_same) e = cudaMemcpy(nbr_same, ds, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && nbr_compl) e = cudaMemcpy(nbr_compl, dc, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && nbr_boundary) e = cudaMemcpy(nbr_boundary, db, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(dacc);
    cudaFree(ds);
    cudaFree(dc);
    cudaFree(db);
    SPH_CUDA(e);
    return check_err2(s);
}

int sph2_destroy(sph_solver2* s) { return free_solver2(s); }

int sph2_set_color_output(sph_solver2* s, int32_t on) {
    if (!s) return fail(SPH_E_INVALID, "sph2_set_color_output: NULL handle");
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    if (on && !s->colour[0]) {
        for (int r = 0; r < 2; ++r) {
            int rc = dalloc(&s->colour[r], s->pop[r].cap, s->owned);
            if (rc != SPH_OK) return rc;
        }
    }
    s->colour_on = on != 0;
    s->colour_n[0] = s->colour_n[1] = 0;
    return SPH_OK;
}

int sph2_get_colors(sph_solver2* s, int32_t population, float* colour, uint32_t* ids_sorted,
                    uint32_t* count) {
    if (!s || population < 0 || population > 1)
        return fail(SPH_E_INVALID, "sph2_get_colors: bad handle or population");
    const uint32_t n = s->colour_on ? s->colour_n[population] : 0u;
    if (count) *count = n;
    if (!colour && !ids_sorted) return SPH_OK;
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    if (n && colour)
        SPH_CUDA(cudaMemcpy(colour, s->colour[population], 4 * (size_t)n, cudaMemcpyDeviceToHost));
    if (n && ids_sorted) {
        std::vector<float4> sv(n);
        SPH_CUDA(cudaMemcpy(sv.data(), s->pop[population].svel, 16 * (size_t)n, cudaMemcpyDeviceToHost));
        for (uint32_t k = 0; k < n; ++k) std::memcpy(&ids_sorted[k], &sv[k].w, 4);
    }
    return SPH_OK;
}

// ---- state I/O (formats in state_format.h) ---------------------------------
// Two-scale state body:
//   sph_config2 | u32 n_low, n_high, nb, group_base, next_low, next_high |
//   u64 cap_low, cap_high |
//   per population (LOW, HIGH): float4 pos[n] (id in w), float4 vel[n]
//   (lambda in w), i32 state[n], u32 group[n] | float4 bpos[nb]

int sph2_step_count(sph_solver2* s, uint64_t* steps) {
    if (!s || !steps) return fail(SPH_E_INVALID, "sph2_step_count: NULL argument");
    *steps = s->step;
    return SPH_OK;
}

int sph2_save_state(sph_solver2* s, void* dst, uint64_t capacity, uint64_t* bytes) {
    if (!s || !bytes) return fail(SPH_E_INVALID, "sph2_save_state: NULL handle or size output");
    const uint64_t nL = s->pop[0].n, nH = s->pop[1].n;
    const uint64_t need = ts_state_bytes(nL, nH, s->nb);
    *bytes = need;
    if (!dst) return SPH_OK;
    if (capacity < need) return fail(SPH_E_CAPACITY, "sph2_save_state: buffer smaller than the state");
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    int rc = check_err2(s);
    if (rc != SPH_OK) return rc;
    sph_io::Writer w{static_cast<unsigned char*>(dst)};
    sph_io::StatePrefix pre;
    std::memcpy(pre.magic, sph_io::kStateMagic, 8);
    pre.version = sph_io::kStateVersion;
    pre.kind = sph_io::kKindTwoScale;
    pre.step = s->step;
    w.put(&pre, sizeof(pre));
    w.put(&s->cfg, sizeof(sph_config2));
    const uint32_t counts[6] = {s->pop[0].n, s->pop[1].n, s->nb, s->group_base, s->next_id[0],
                                s->next_id[1]};
    w.put(counts, sizeof(counts));
    const uint64_t caps[2] = {s->pop[0].cap, s->pop[1].cap};
    w.put(caps, sizeof(caps));
    for (int r = 0; r < 2; ++r) {
        const Pop& p = s->pop[r];
        const size_t n = p.n;
        if (!n) continue;
        SPH_CUDA(cudaMemcpy(w.take(16 * n), p.pos, 16 * n, cudaMemcpyDeviceToHost));
        SPH_CUDA(cudaMemcpy(w.take(16 * n), p.vel, 16 * n, cudaMemcpyDeviceToHost));
        SPH_CUDA(cudaMemcpy(w.take(4 * n), p.stt, 4 * n, cudaMemcpyDeviceToHost));
        SPH_CUDA(cudaMemcpy(w.take(4 * n), p.grp, 4 * n, cudaMemcpyDeviceToHost));
    }
    if (s->nb) SPH_CUDA(cudaMemcpy(w.take(16 * (size_t)s->nb), s->bpos, 16 * (size_t)s->nb, cudaMemcpyDeviceToHost));
    const uint64_t sum = sph_io::checksum(dst, w.off);
    w.put(&sum, 8);
    return SPH_OK;
}

int sph2_create_from_state(const void* src, uint64_t bytes, sph_solver2** out) {
    if (!src || !out) return fail(SPH_E_INVALID, "sph2_create_from_state: NULL argument");
    *out = nullptr;
    sph_io::StatePrefix pre;
    if (!sph_io::check_state(src, (size_t)bytes, sph_io::kKindTwoScale, &pre))
        return fail(SPH_E_INVALID, "sph2_create_from_state: not a two-scale state, or corrupt");
    sph_io::Reader r{static_cast<const unsigned char*>(src), (size_t)bytes - 8, sizeof(pre)};
    sph_config2 cfg;
    uint32_t c[6];
    uint64_t caps[2];
    if (!r.get(&cfg, sizeof(cfg)) || !r.get(c, sizeof(c)) || !r.get(caps, sizeof(caps)))
        return fail(SPH_E_INVALID, "sph2_create_from_state: truncated header");
    const uint32_t nb = c[2], group_base = c[3];
    const uint32_t next_id[2] = {c[4], c[5]};
    if (caps[0] > kMaxParticles || caps[1] > kMaxParticles || nb > kMaxParticles ||
        c[0] > caps[0] || c[1] > caps[1])
        return fail(SPH_E_CAPACITY, "sph2_create_from_state: counts beyond capacities or 2^30");
    if (bytes != ts_state_bytes(c[0], c[1], nb))
        return fail(SPH_E_INVALID, "sph2_create_from_state: size does not match the particle counts");
    TSParams P;
    int rc = make_ts_params(cfg, &P);
    if (rc != SPH_OK) return rc;
    HostPop pops[2];
    for (int q = 0; q < 2; ++q) {
        const uint32_t n = c[q];
        HostPop& h = pops[q];
        h.pos.resize(n);
        h.vel.resize(n);
        h.stt.resize(n);
        h.grp.resize(n);
        r.get(h.pos.data(), 16 * (size_t)n);
        r.get(h.vel.data(), 16 * (size_t)n);
        r.get(h.stt.data(), 4 * (size_t)n);
        r.get(h.grp.data(), 4 * (size_t)n);
        std::vector<unsigned char> seen(next_id[q], 0);
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t id;
            std::memcpy(&id, &h.pos[i].w, 4);
            if (id >= next_id[q] || seen[id] || h.stt[i] < 0 || h.stt[i] > 15 ||
                (h.grp[i] != kNoGroup && h.grp[i] >= group_base))
                return fail(SPH_E_INVALID, "sph2_create_from_state: inconsistent ids, states or groups");
            seen[id] = 1;
        }
    }
    std::vector<float4> hb(nb);
    r.get(hb.data(), 16 * (size_t)nb);
    return create_solver2(&cfg, P, caps[0], caps[1], pops, hb.data(), nb, group_base, next_id,
                          pre.step, out);
}

int sph2_write_frame(sph_solver2* s, const char* path, uint32_t fields, int32_t append) {
    if (!s || !path) return fail(SPH_E_INVALID, "sph2_write_frame: NULL argument");
    const uint32_t known = SPH_FIELD_POSITIONS | SPH_FIELD_VELOCITIES | SPH_FIELD_BLEND;
    if (fields == 0 || (fields & ~known))
        return fail(SPH_E_INVALID, "sph2_write_frame: fields must be a non-empty mask of "
                                   "positions, velocities, blend");
    struct Arrays {
        std::vector<uint32_t> ids;
        std::vector<float> x, v, lambda;
        std::vector<int32_t> state;
    } a[2];
    for (int q = 0; q < 2; ++q) {
        const size_t n = s->pop[q].n;
        a[q].ids.resize(n);
        if (fields & SPH_FIELD_POSITIONS) a[q].x.resize(3 * n);
        if (fields & SPH_FIELD_VELOCITIES) a[q].v.resize(3 * n);
        if (fields & SPH_FIELD_BLEND) {
            a[q].lambda.resize(n);
            a[q].state.resize(n);
        }
        int rc = sph2_get_state(s, q, a[q].x.empty() ? nullptr : a[q].x.data(),
                                a[q].v.empty() ? nullptr : a[q].v.data(),
                                a[q].lambda.empty() ? nullptr : a[q].lambda.data(),
                                a[q].state.empty() ? nullptr : a[q].state.data(), nullptr,
                                a[q].ids.data());
        if (rc != SPH_OK) return rc;
    }
    FILE* f = std::fopen(path, append ? "ab" : "wb");
    if (!f) return fail(SPH_E_IO, std::string("sph2_write_frame: cannot open ") + path);
    sph_io::FramePrefix pre;
    std::memcpy(pre.magic, sph_io::kFrameMagic, 8);
    pre.kind = sph_io::kKindTwoScale;
    pre.fields = fields;
    pre.step = s->step;
    const uint32_t counts[2] = {s->pop[0].n, s->pop[1].n};
    bool ok = std::fwrite(&pre, sizeof(pre), 1, f) == 1 && std::fwrite(counts, sizeof(counts), 1, f) == 1;
    auto put = [&](const void* p, size_t n) {
        if (ok && n) ok = std::fwrite(p, 1, n, f) == n;
    };
    for (int q = 0; q < 2; ++q) {
        put(a[q].ids.data(), 4 * a[q].ids.size());
        put(a[q].x.data(), 4 * a[q].x.size());
        put(a[q].v.data(), 4 * a[q].v.size());
        put(a[q].lambda.data(), 4 * a[q].lambda.size());
        put(a[q].state.data(), 4 * a[q].state.size());
    }
    if (std::fclose(f) != 0) ok = false;
    return ok ? SPH_OK : fail(SPH_E_IO, "sph2_write_frame: write failed");
}

}  // extern "C"
