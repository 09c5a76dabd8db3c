/*
 * sph2s.h -- C ABI of the GB300-native SPH2S particle step.
 *
 * The reference (segfault11/SPH2S_FINAL) exposes the step as C++ classes:
 *   SolverConfiguration::MakeConfiguration   SPH2S_FINAL_SINGLE_SCALE/Solver.h:15-48
 *   Grid::MakeGrid / ComputeNumGridCells      SPH2S_FINAL_SINGLE_SCALE/Grid.h:11-46
 *   ParticleData::CreateParticleBox(Canvas)   SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:129-209
 *   Solver(fluid, boundary, config)           SPH2S_FINAL_SINGLE_SCALE/Solver.h:113-118
 *   Solver::Bind / Solver::Advance(dt)        SPH2S_FINAL_SINGLE_SCALE/Solver.h:120-121
 *   ParticleData::dPositions (GL VBO)         SPH2S_FINAL_SINGLE_SCALE/ParticleData.h:38-45
 * This header replaces them with plain functions over plain pointers: a solver
 * handle owns every device buffer, host arrays are copied in, results are
 * copied out into caller buffers.  No exception crosses the ABI; every entry
 * point returns an SPH_* status and sph_last_error() describes the last
 * failure of the calling thread.
 *
 * Arrays of positions and velocities are AoS float xyz (3 floats per
 * particle), the layout of the reference's ParticleData buffers.
 */
#ifndef SPH2S_H
#define SPH2S_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (the reference throws std::runtime_error from
 * CUDA::SafeCall, SPH2S_FINAL_SINGLE_SCALE/cuda.h:115-129). */
#define SPH_OK 0
#define SPH_E_INVALID 1  /* bad argument, NULL handle, bad configuration */
#define SPH_E_CAPACITY 2 /* particle or cell count beyond what the ABI supports */
#define SPH_E_CUDA 3     /* a CUDA runtime call failed (incl. allocation) */
#define SPH_E_TIMEOUT 4  /* a bounded device-side wait gave up; results invalid */

/* Readback order. */
#define SPH_ORDER_SORTED 0 /* array order of the last step (the reference's order) */
#define SPH_ORDER_BY_ID 1  /* input order: element i is the particle created i-th */

/* Grid::Grid (SPH2S_FINAL_SINGLE_SCALE/Grid.h:55-58). */
typedef struct sph_grid {
    float origin[3];
    int32_t dims[3];
    float spacing;
} sph_grid;

/* SolverConfiguration (SPH2S_FINAL_SINGLE_SCALE/Solver.h:50-60). */
typedef struct sph_config {
    float effective_radius;       /* h */
    float fluid_particle_mass;    /* m */
    float boundary_particle_mass; /* m_b */
    float rest_density;           /* rho0 */
    float bulk_modulus;           /* K in p = K (rho - rho0) */
    float viscosity;              /* mu */
    float speed_sound;            /* c, boundary force 0.02 c^2 */
    float tension_coefficient;    /* sigma */
    float xsph_coeff;             /* epsilon (kept for layout; the step does not use it) */
    sph_grid grid;                /* uniform grid, spacing normally h */
} sph_config;

typedef struct sph_solver sph_solver;

/* ---- configuration and scene builders ---------------------------------- */

/* Grid::MakeGrid(origin, end, spacing): dims = ceil((end - origin) / spacing). */
int sph_make_grid(const float origin[3], const float end[3], float spacing, sph_grid* out);

/* Grid::ComputeNumGridCells. */
uint32_t sph_grid_num_cells(const sph_grid* grid);

/* SolverConfiguration::MakeConfiguration (SPH2S_FINAL_SINGLE_SCALE/Solver.h:15-48). */
int sph_make_configuration(const float origin[3], const float end[3], float volume,
                           uint32_t num_particles, uint32_t avg_particles, float rest_density,
                           float bulk_modulus, float viscosity, float speed_sound,
                           float tension_coefficient, float epsilon, sph_config* out);

/* ParticleData::CreateParticleBox (ParticleData.cpp:129-163): one particle at
 * origin + (i, j, k) * spacing per grid cell, x fastest.  With xyz == NULL
 * only *n_out is written. */
int sph_particle_box(const sph_grid* grid, float* xyz, uint32_t capacity, uint32_t* n_out);

/* ParticleData::CreateParticleBoxCanvas (ParticleData.cpp:165-209): the hollow
 * shell of `border` layers around the grid. */
int sph_particle_box_canvas(const sph_grid* grid, int32_t border, float* xyz, uint32_t capacity,
                            uint32_t* n_out);

/* ---- single-scale solver ---------------------------------------------- */

/* Solver::Solver(fluid, boundary, config) + Bind().  Copies the fluid and
 * boundary positions (and optional initial velocities, NULL = zero) to the
 * device, sorts the static boundary once on the fluid grid.  The handle has
 * its own stream and keeps the configuration in kernel parameters, so several
 * handles can coexist (the reference binds one __constant__ config). */
int sph_create(const sph_config* config, const float* fluid_xyz, uint32_t n_fluid,
               const float* boundary_xyz, uint32_t n_boundary, const float* velocity_xyz,
               sph_solver** out);

/* Solver::Advance(dt), `steps` times.  Asynchronous: returns after enqueueing
 * the work on the handle's stream; sph_sync waits and reports device-side
 * errors (SPH_E_TIMEOUT if a bounded wait gave up). */
int sph_advance(sph_solver* s, float dt, int32_t steps);
int sph_sync(sph_solver* s);

/* Readback into host buffers (3 floats per particle for positions and
 * velocities, 1 for densities).  Synchronises the handle's stream.  Densities
 * are those of the last step (zero before the first step). */
int sph_get_positions(sph_solver* s, float* xyz, int32_t order);
int sph_get_velocities(sph_solver* s, float* xyz, int32_t order);
int sph_get_densities(sph_solver* s, float* rho, int32_t order);
/* Persistent ids in sorted order (ids[k] = input index of the k-th particle). */
int sph_get_ids(sph_solver* s, uint32_t* ids);
/* Overwrites the velocities (3 floats per particle) in the given order. */
int sph_set_velocities(sph_solver* s, const float* xyz, int32_t order);
int sph_counts(sph_solver* s, uint32_t* n_fluid, uint32_t* n_boundary);
/* Stream the handle enqueues on (a cudaStream_t). */
void* sph_stream(sph_solver* s);
int sph_destroy(sph_solver* s);

/* Parity instrumentation for the current state, without advancing it:
 * hashes, sorts and reorders exactly as the next step will, and returns, each
 * pointer optional (NULL = skip), in the sorted order of that step:
 *   keys[n]       Morton cell keys (ascending)
 *   ids[n]        persistent id of each sorted particle
 *   cell_start/cell_end[cells]  per linear cell cx + Dx (cy + Dy cz), 0xFFFFFFFF when empty
 *   nbr_fluid[n]  fluid neighbours with r < h (self included)
 *   nbr_boundary[n] boundary neighbours with r < h
 *   rho[n], acc[3n] density and acceleration (before integration). */
int sph_debug_step_fields(sph_solver* s, uint32_t* keys, uint32_t* ids, uint32_t* cell_start,
                          uint32_t* cell_end, uint32_t* nbr_fluid, uint32_t* nbr_boundary,
                          float* rho, float* acc);

/* Advances `steps` steps outside the step graph, timing each phase with CUDA
 * events on the handle's stream; ms[0..2] receive the mean milliseconds per
 * step of (hash + sort + reorder + cell ranges), density, force + integrate.
 * (The reference only times the whole Advance, SPH2S_FINAL_SINGLE_SCALE/Solver.cu:1084-1095.) */
int sph_profile_phases(sph_solver* s, float dt, int32_t steps, float* ms);

/* Test hook for the bounded-wait path: while `on` is non-zero the radix sort's
 * look-back treats every predecessor as not ready and gives up after a short
 * bounded spin, so the next sph_sync returns SPH_E_TIMEOUT without hanging. */
int sph_debug_force_lookback_timeout(sph_solver* s, int32_t on);

/* ---- key-value sort ------------------------------------------------------ */

/* Stable ascending sort of n (uint32 key, uint32 value) pairs in device
 * memory by the low `key_bits` bits of the key (the higher bits must be 0):
 * the hand-written onesweep radix sort the step uses, replacing
 * thrust::sort_by_key (SPH2S_FINAL_SINGLE_SCALE/Solver.cu:1110-1115).
 * vals_in may be NULL (values are then 0..n-1).  Inputs are not modified; the
 * outputs must not overlap them.  Enqueues on `stream` (a cudaStream_t, NULL
 * = legacy default stream), allocates its scratch with cudaMalloc, and
 * returns after the sort completed. */
int sph_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                   uint32_t* vals_out, uint32_t n, int32_t key_bits, void* stream);

/* sph_sort_pairs for callers that cannot allocate device memory (no
 * counterpart in the reference): hosts that own a fixed device-memory budget
 * and pass only their own buffers, code running while a global-mode stream
 * capture is open elsewhere (cudaMalloc is illegal then), or loops that must
 * not risk an allocation's implicit synchronisation.  Same arguments and
 * results as sph_sort_pairs; calls no cudaMalloc/cudaFree.  Its scratch is one
 * static device array of about 10 MB that each GPU loading the library holds
 * until exit, which limits n to 1,048,576 pairs (larger n: SPH_E_CAPACITY).
 * The first call on a device looks the array up (make it before any stream
 * capture); all calls share the array, so calls that overlap on the GPU race
 * and must be serialised by the caller. */
int sph_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                           uint32_t* vals_out, uint32_t n, int32_t key_bits, void* stream);

/* Description of the last failure on the calling thread ("" if none). */
const char* sph_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SPH2S_H */
