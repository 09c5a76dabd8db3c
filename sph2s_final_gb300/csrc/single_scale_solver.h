// single_scale_solver.h -- the single-scale solver handle, shared by the step
// (single_scale.cu) and the differentiable rollout (adjoint.cu).
#pragma once
#include <cuda_runtime.h>
#include "../../include/sph2s.h"
#include "common.cuh"
#include "coherent_sort.cuh"
#include "radix_sort.cuh"

namespace sph {
struct Rollout;  // tape of a differentiable rollout (adjoint.cu)
}

struct sph_solver {
    sph_config cfg;
    sph::SimParams P;
    cudaStream_t stream = nullptr;
    uint32_t n = 0, nb = 0, ncells = 0;
    int key_bits = 0;
    float4* pos = nullptr;   // state, sorted order of the last step
    float4* vel = nullptr;
    float4* spos = nullptr;  // working copies in the current step's sorted order
    float4* svel = nullptr;
    float* rho = nullptr;
    float2* aux = nullptr;
    float4* xa = nullptr;           // force-pass records (x, p/rho^2), written by the density pass
    uint4* nbr = nullptr;           // neighbour lists, kMaxNbr per particle, [group][particle]
    uint32_t* nbr_count = nullptr;  // neighbours per particle (force set, r > 0)
    uint8_t* bnear = nullptr;       // per cell: boundary particles within stencil reach
    uint32_t* bstart = nullptr;     // per cell + 1: start of its static boundary candidates ...
    uint32_t* bcand = nullptr;      // ... (boundary particle indices, boundary_cand_kernel)
    float4* bacc = nullptr;         // boundary force sums of near-boundary particles (step order)
    uint32_t* blist = nullptr;      // the step's near-boundary particles (sorted indices) ...
    uint32_t* bcount = nullptr;     // ... and their number
    uint8_t* bflag = nullptr;       // per sorted particle: 1 if in blist (read by the force pass)
    int sms = 0;                    // SM count (grid of the boundary force pass)
    cudaStream_t side = nullptr;    // second branch of the step: the boundary force
    cudaEvent_t fork = nullptr, join = nullptr;
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* vals[2] = {nullptr, nullptr};
    uint2* cells = nullptr;
    uint2* bcells = nullptr;
    float4* bpos = nullptr;
    float4* pos0 = nullptr;  // positions at creation, creation order (rollout restarts)
    float* stage = nullptr;  // device staging for packed readback
    void* sort_mem = nullptr;
    sph::SortScratch sort;
    void* co_mem = nullptr;   // scratch of the coherent sort
    sph::CoherentSort co;
    int sort_mode = 0;        // kSortAuto / kSortFull / kSortCoherent (sph_debug_sort_mode)
    uint32_t* err = nullptr;  // device error word
    uint32_t* err_host = nullptr;
    int force_timeout = 0;
    cudaGraphExec_t graph = nullptr;
    float graph_dt = 0.0f;
    uint64_t step = 0;  // steps advanced since creation (carried by saved states)
    int32_t integrator = SPH_INTEGRATOR_SYMPLECTIC_EULER;
    float* xacc = nullptr;     // XSPH integrator: accelerations of the step (3 per particle)
    uint32_t* xall = nullptr;  // XSPH integrator: neighbours incl. distance 0, per particle
    uint32_t* xnb = nullptr;   // XSPH integrator: boundary neighbour counts (unused output)
    // asynchronous position readback: two device staging buffers drained by a copy stream
    float* astage[2] = {nullptr, nullptr};
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t packed[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
    int abuf = 0;
    sph::Rollout* rollout = nullptr;
};

namespace sph_ss {
// The step's sort: automatic (coherent from kCoherentMinParticles on, where it
// is faster on GB300), from scratch, or coherent.
constexpr int kSortAuto = 0, kSortFull = 1, kSortCoherent = 2;
constexpr uint32_t kCoherentMinParticles = 131072;
// hash -> sort (coherent or from scratch, sort_mode) -> reorder + cell ranges;
// returns the index of the key/value buffers that hold the sorted keys and
// the permutation.
int enqueue_neighborhood(sph_solver* s);
void enqueue_density(sph_solver* s);
void enqueue_force(sph_solver* s, float dt);
int check_device_error(sph_solver* s);
// Selects the integrator (allocating the XSPH buffers on first use) and drops
// the captured step graph.
int set_integrator(sph_solver* s, int32_t integrator);
// Host arrays a handle is created from: either packed float4 arrays (a saved
// state: fluid positions with the persistent id in w and velocities in the
// order the next step starts from, creation-time positions for rollout
// restarts, boundary positions) or the caller's raw xyz arrays (sph_create:
// 3 floats per particle, ids = input order, velocities NULL = zero), which are
// copied as they are and packed into float4 on the device.
struct HostInit {
    const float4 *pos = nullptr, *vel = nullptr, *pos0 = nullptr, *bound = nullptr;
    const float *pos_xyz = nullptr, *vel_xyz = nullptr, *bound_xyz = nullptr;
};
// Creates a handle (boundary presorted here).
int create_solver(const sph_config* config, const HostInit& init, uint32_t n_fluid,
                  uint32_t n_boundary, uint64_t step, sph_solver** out);
inline uint32_t blocks_for(uint32_t n, uint32_t t = 256) { return (n + t - 1) / t; }
}  // namespace sph_ss

// Releases the rollout tape (adjoint.cu).
void sph_rollout_release(sph_solver* s);
