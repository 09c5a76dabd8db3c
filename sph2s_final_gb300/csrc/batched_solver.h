// batched_solver.h -- the batch handle, shared by the batched step
// (batched.cu) and the batched differentiable rollout (batched_adjoint.cu).
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include "../../include/sph2s.h"
#include "batched_kernels.cuh"
#include "coherent_sort.cuh"
#include "radix_sort.cuh"

namespace sph {
struct BRollout;
constexpr int kBlockChoices[3] = {128, 256, 512};
}  // namespace sph

using sph::SceneRec;
using sph::SortScratch;

struct sph_batch {
    uint32_t S = 0;                  // scenes
    uint32_t N = 0, NB = 0, NC = 0;  // fluid, boundary, cells (all scenes)
    int shift = 0, passes = 0;
    std::vector<SceneRec> recs_h;
    SceneRec* recs = nullptr;
    cudaStream_t stream = nullptr;
    float4 *pos = nullptr, *vel = nullptr, *spos = nullptr, *svel = nullptr;
    float* rho = nullptr;
    float2* aux = nullptr;
    float4* xa = nullptr;  // force-pass records (x, p/rho^2), written by the density pass
    uint4* nbr = nullptr;
    uint32_t* nbr_count = nullptr;
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* vals[2] = {nullptr, nullptr};
    uint2 *cells = nullptr, *bcells = nullptr;
    uint8_t* bnear = nullptr;
    uint32_t *bstart = nullptr, *bcand = nullptr;  // static boundary candidate tables
    float4* bacc = nullptr;              // the step's boundary force sums
    uint8_t* bflag = nullptr;            // per sorted particle: bnear of its cell
    cudaStream_t side = nullptr;         // second branch of the step: the boundary force
    cudaEvent_t fork = nullptr, join = nullptr;
    float4* bpos = nullptr;
    void* sort_mem = nullptr;
    SortScratch sort;
    void* co_mem = nullptr;  // the step's coherent sort (from 131,072 fluid particles on)
    sph::CoherentSort co;
    bool coherent = false;
    uint32_t* err = nullptr;
    uint32_t* err_host = nullptr;
    // tiles per block-size choice (fluid), boundary tiles at 256
    uint2* tiles[3] = {nullptr, nullptr, nullptr};
    uint32_t ntiles[3] = {0, 0, 0};
    uint2* btiles = nullptr;
    uint32_t nbtiles = 0;
    int bs_density = 1, bs_force = 1;  // index into kBlockChoices
    int grid_mult = 4;                 // persistent grid = grid_mult * SMs
    int sms = 152;
    cudaGraphExec_t graph = nullptr;
    float graph_dt = 0.0f;
    std::vector<void*> owned;
    std::vector<sph_config> cfgs;     // per-scene configuration (viscosity changes in rollouts)
    float4* pos0 = nullptr;           // creation positions, packed by scene (rollout restarts)
    std::vector<uint32_t> tile_first; // first 256-particle tile of each scene in tiles[1]
    sph::BRollout* rollout = nullptr; // tape of a batched differentiable rollout
};

namespace sph_b {
using namespace sph;
int free_batch(sph_batch* b);
uint32_t pgrid(const sph_batch* b, uint32_t tiles);
// hash -> sort -> reorder of all scenes; returns the key/value buffer index
// holding the sorted keys and the permutation.
int enqueue_neighborhood(sph_batch* b);
void enqueue_density(sph_batch* b);
void enqueue_force(sph_batch* b, float dt);
int check_err(sph_batch* b);
// Re-derives scene s's kernel constants from b->cfgs[s] and uploads the table.
int refresh_scene_params(sph_batch* b);
}  // namespace sph_b

// Releases the rollout tape (batched_adjoint.cu).
void sphb_rollout_release(sph_batch* b);
