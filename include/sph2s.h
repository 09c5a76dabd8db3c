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
#define SPH_E_IO 5       /* a file could not be opened or written */

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
    float xsph_coeff;             /* epsilon of the XSPH integrator (SPH_INTEGRATOR_XSPH) */
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
/* Enqueues a readback of the current positions (3 floats per particle) into
 * xyz and returns at once: the positions are packed into one of two device
 * staging buffers on the handle's stream and copied out on a second stream,
 * so the copy of step k overlaps the computation of step k+1.  xyz must stay
 * valid, and should be pinned host memory for the copy to be asynchronous,
 * until sph_sync; at most two readbacks are in flight (a third waits for the
 * first). */
int sph_get_positions_async(sph_solver* s, float* xyz, int32_t order);
/* Device-resident readback (the reference's own consumers read
 * ParticleData::dPositions in device memory every frame, the renderer through
 * the mapped VBO, SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:47-66,
 * main.cpp:79): the same arrays as sph_get_positions / _velocities /
 * _densities, written into caller-owned device memory (3 floats per particle,
 * 1 for densities) by a kernel on the handle's stream.  Asynchronous: order
 * later work after sph_stream(s) or call sph_sync.  A destination that is not
 * device or managed memory of the current device: SPH_E_INVALID. */
int sph_get_positions_device(sph_solver* s, float* d_xyz, int32_t order);
int sph_get_velocities_device(sph_solver* s, float* d_xyz, int32_t order);
int sph_get_densities_device(sph_solver* s, float* d_rho, int32_t order);
/* Persistent ids in sorted order (ids[k] = input index of the k-th particle). */
int sph_get_ids(sph_solver* s, uint32_t* ids);
/* Overwrites the velocities (3 floats per particle) in the given order. */
int sph_set_velocities(sph_solver* s, const float* xyz, int32_t order);
int sph_counts(sph_solver* s, uint32_t* n_fluid, uint32_t* n_boundary);
/* Stream the handle enqueues on (a cudaStream_t). */
void* sph_stream(sph_solver* s);
int sph_destroy(sph_solver* s);

/* ---- headless state I/O ---------------------------------------------------
 * Replaces the reference's only output path, the GL vertex buffer mapped by
 * ParticleData::Map/Unmap (SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:47-66)
 * and the rendered frames of VideoWriter::CaptureFrame
 * (SPH2S_FINAL_SINGLE_SCALE/VideoWriter/VideoWriter.cpp:41-49). */

/* Field mask of frame records. */
#define SPH_FIELD_POSITIONS 1u
#define SPH_FIELD_VELOCITIES 2u
#define SPH_FIELD_DENSITIES 4u /* single scale only */
#define SPH_FIELD_BLEND 8u     /* two scale only: blend coefficient and state bits */

/* Integrators.  SYMPLECTIC_EULER is the reference's integrateD
 * (SPH2S_FINAL_SINGLE_SCALE/Solver.cu:713-755), the default.  XSPH is its
 * integrateXSPHD (Solver.cu:757-853, launch commented out at 1185-1196):
 * v' = v + dt a; v'' = v' + eps sum_j (v'_j - v'_i) m/rho_j W_poly6; x' = x + dt v''
 * with eps = sph_config.xsph_coeff, the correction applied per component (the
 * reference adds its x component to all three).  The differentiable rollout
 * always uses SYMPLECTIC_EULER. */
#define SPH_INTEGRATOR_SYMPLECTIC_EULER 0
#define SPH_INTEGRATOR_XSPH 1
int sph_set_integrator(sph_solver* s, int32_t integrator);

/* Steps advanced since creation (a state carries it across save / resume). */
int sph_step_count(sph_solver* s, uint64_t* steps);
/* Serialises the complete solver state into dst (host memory).  With dst ==
 * NULL only *bytes (the size needed) is written.  A solver created from the
 * state continues bit for bit like this one.  Waits for queued steps. */
int sph_save_state(sph_solver* s, void* dst, uint64_t capacity, uint64_t* bytes);
/* Creates a solver from a buffer written by sph_save_state; SPH_E_INVALID if
 * the buffer is not a single-scale state or fails its checksum. */
int sph_create_from_state(const void* src, uint64_t bytes, sph_solver** out);
/* Appends (append != 0) or writes one frame record to path: the current step
 * number and the requested fields, in input (persistent id) order. */
int sph_write_frame(sph_solver* s, const char* path, uint32_t fields, int32_t append);

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

/* Advances `steps` steps as one CUDA graph with an event record node at every
 * phase boundary (the phases run back to back as in the step graph, so they
 * sum to the span of the steps); ms[0..2] receive the mean milliseconds per
 * step of (hash + sort + reorder + cell ranges), density, force + integrate.
 * (The reference only times the whole Advance, SPH2S_FINAL_SINGLE_SCALE/Solver.cu:1084-1095.) */
int sph_profile_phases(sph_solver* s, float dt, int32_t steps, float* ms);

/* Test hook for the bounded-wait path: while `on` is non-zero the radix sort's
 * look-back treats every predecessor as not ready and gives up after a short
 * bounded spin, so the next sph_sync returns SPH_E_TIMEOUT without hanging. */
int sph_debug_force_lookback_timeout(sph_solver* s, int32_t on);

/* Test hook selecting how each step sorts its (cell key, index) pairs; both
 * ways give the same permutation.  0 (default): automatic -- coherent from
 * 131,072 particles on, from scratch below (where the radix sort alone is
 * faster); 1: from scratch (sph_sort_pairs' onesweep sort); 2: coherent
 * (sph_sort_keys_coherent's scheme: only the particles that changed cell
 * since the last step are radix-sorted, the rest merged around them). */
int sph_debug_sort_mode(sph_solver* s, int32_t mode);

/* ---- differentiable rollout (no counterpart in the reference) ------------ */

/* Restarts the solver from its creation positions with initial velocities
 * v0 (3 floats per particle in creation order, NULL = zero) and viscosity
 * `viscosity`, and runs `steps` steps of dt, checkpointing the state every
 * `checkpoint_every` steps for the backward pass. */
int sph_rollout_forward(sph_solver* s, const float* v0_xyz, float viscosity, float dt,
                        int32_t steps, int32_t checkpoint_every);
/* Poly6 splat G of the current particles on the cell centres of `nodes`
 * (G_n = m sum_i W(|y_n - x_i|), the density pass's kernel and stencil rule);
 * `field` (optional) receives G.  With a target (one value per node),
 * *loss = mean_n (G_n - target_n)^2 and, after sph_rollout_forward, its
 * gradient with respect to the final positions is kept for the backward. */
int sph_rollout_density_loss(sph_solver* s, const sph_grid* nodes, const float* target,
                             float* field, double* loss);
/* Reverse pass of the last forward + loss: hand-written adjoints of
 * integrate, force and density, recomputing each checkpoint segment and
 * holding every step's neighbour structure constant.  Gradients with respect
 * to the initial velocities and positions (3 floats per particle, creation
 * order; each optional) and the viscosity. */
int sph_rollout_backward(sph_solver* s, float* grad_v0, float* grad_x0, double* grad_mu);

/* ---- two-scale solver -------------------------------------------------- */

#define SPH_LOW 0  /* coarse population: support h, mass m */
#define SPH_HIGH 1 /* fine population: support h/2, mass m/8 */

/* SolverConfiguration of the two-scale project (SPH2S_FINAL_TWO_SCALE/Solver.h:52-61)
 * plus the refinement slab that drives splitting and merging (not in the
 * reference, whose split trigger is commented out, Solver.cu:1077-1082):
 * a LOW particle in state 0 strictly inside refine_lo < x[refine_axis] <
 * refine_hi at the start of a step splits into 8 HIGH children; a group of
 * 8 children, all fully blended in, whose centroid is outside the slab
 * merges back into one LOW particle.  refine_axis = -1 disables both. */
typedef struct sph_config2 {
    float effective_radius[2];    /* [SPH_LOW] h, [SPH_HIGH] h/2 */
    float fluid_particle_mass[2]; /* m, m/8 */
    float boundary_particle_mass; /* used with the LOW radius for both populations */
    float rest_density;
    float bulk_modulus;
    float viscosity;
    float speed_sound;
    float tension_coefficient;
    float blend_increment;        /* lambda change per step (BlendIncrement) */
    sph_grid grid[2];             /* one grid per population, spacing = its support */
    int32_t refine_axis;          /* slab trigger: 0, 1, 2 or -1 (no slab) */
    float refine_lo, refine_hi;
    int32_t mode;                 /* SPH2_MODE_BLENDED or SPH2_MODE_COUPLED */
    int32_t split_trigger;        /* SPH2_SPLIT_SLAB or SPH2_SPLIT_SURFACE */
    float surface_density;        /* SPH2_SPLIT_SURFACE: a particle with rho < this is at the surface */
} sph_config2;

/* Modes.  BLENDED is SPH2S_FINAL_TWO_SCALE: lambda-weighted sums, velocity
 * clamp, fade / split / merge state machine.  COUPLED is
 * SPH2S_FINAL_TWO_SCALE_COUPLED (Solver.cu:648-1015): two fixed populations,
 * unweighted sums, no clamp, no state changes, and its complementary tension
 * weight W_{h_c}(r) of the neighbour's own support (Solver.cu:448-460). */
#define SPH2_MODE_BLENDED 0
#define SPH2_MODE_COUPLED 1
/* Split triggers (BLENDED).  SLAB: a LOW particle whose start-of-step
 * position lies inside refine_lo < x[refine_axis] < refine_hi splits; a group
 * whose centroid leaves the slab merges.  SURFACE replaces the reference's
 * render-pass surface flag (getSurfaceIDs, SPH2S_FINAL_TWO_SCALE/SSFRenderer.cu:
 * 196-218, which sets state bit 8) and its commented-out split marking
 * (Solver.cu:1077-1082) by a density deficit computed in the step: a normal
 * LOW particle with rho < surface_density splits; a group whose 8 members
 * are fully blended in and all have rho >= surface_density merges. */
#define SPH2_SPLIT_SLAB 0
#define SPH2_SPLIT_SURFACE 1

typedef struct sph_solver2 sph_solver2;

/* SolverConfiguration::MakeConfiguration of the two-scale project
 * (SPH2S_FINAL_TWO_SCALE/Solver.h:16-50); refinement disabled. */
int sph_make_configuration2(const float origin[3], const float end[3], float volume,
                            uint32_t num_particles, uint32_t avg_particles, float rest_density,
                            float bulk_modulus, float viscosity, float speed_sound,
                            float tension_coefficient, float blend_increment, sph_config2* out);

/* Solver(low, high, boundary, config) + Bind() (SPH2S_FINAL_TWO_SCALE/Solver.h:121-130,
 * Solver.cu:1444-1544): LOW particles start in state 0, HIGH in state 4, all
 * with lambda 1 and zero velocity; the boundary is sorted once on the LOW
 * grid.  Capacities bound the populations (0 = 2 n_low + 1024 and
 * 8 (n_low + n_high) + 1024; the reference allocates 8 x LOW for HIGH). */
int sph2_create(const sph_config2* config, const float* low_xyz, uint32_t n_low,
                const float* high_xyz, uint32_t n_high, const float* boundary_xyz,
                uint32_t n_boundary, uint32_t capacity_low, uint32_t capacity_high,
                sph_solver2** out);
/* Solver::Advance (SPH2S_FINAL_TWO_SCALE/Solver.cu:1568-1614), `steps` times;
 * synchronous (the population sizes are read back after every step, like
 * the reference's per-step count read, Solver.cu:1633-1638). */
int sph2_advance(sph_solver2* s, float dt, int32_t steps);
int sph2_counts(sph_solver2* s, uint32_t* n_low, uint32_t* n_high, uint32_t* n_boundary,
                uint32_t* groups);
/* Persistent id the next particle created in each population will get
 * (children and merged particles receive consecutive ids). */
int sph2_next_ids(sph_solver2* s, uint32_t* next_low, uint32_t* next_high);
/* Counters of the last step: splits, merges, removed LOW, removed HIGH,
 * fade-in completions LOW, HIGH. */
int sph2_last_stats(sph_solver2* s, uint32_t* stats6);
/* State of one population in its current order (each pointer optional):
 * positions, velocities (3 floats each), blend coefficients, state bits,
 * group ids (0xFFFFFFFF = none) and persistent ids. */
int sph2_get_state(sph_solver2* s, int32_t population, float* xyz, float* vel, float* lambda,
                   int32_t* state, uint32_t* group, uint32_t* ids);
/* Positions of one population in its current order (3 floats per particle)
 * written into caller-owned device memory by a kernel on the handle's stream,
 * as sph_get_positions_device: the two-scale renderer's read of
 * ParticleData::dPositions (SPH2S_FINAL_TWO_SCALE/ParticleData.h:38-43).
 * Asynchronous; a destination that is not device memory: SPH_E_INVALID. */
int sph2_get_positions_device(sph_solver2* s, int32_t population, float* d_xyz);
/* State bits of one population in its current order (one int32 per
 * particle) copied into caller-owned device memory on the handle's stream:
 * the two-scale ParticleData::dStates the reference's renderer reads
 * (SPH2S_FINAL_TWO_SCALE/ParticleData.h:43).  Asynchronous; a destination
 * that is not device memory: SPH_E_INVALID. */
int sph2_get_states_device(sph_solver2* s, int32_t population, int32_t* d_state);
/* Parity instrumentation: for the current state, without advancing, the
 * sorted persistent ids, densities, accelerations and neighbour counts (same
 * population, complementary population, boundary) of one population, in the
 * sorted order of the next step. */
int sph2_debug_step_fields(sph_solver2* s, int32_t population, uint32_t* ids_sorted, float* rho,
                           float* acc, uint32_t* nbr_same, uint32_t* nbr_compl,
                           uint32_t* nbr_boundary);
int sph2_destroy(sph_solver2* s);
/* Colour / energy output of the two-scale force pass (dColorValues,
 * SPH2S_FINAL_TWO_SCALE/Solver.cu:206-213, 378-387, 897-907, 1050-1070): per
 * particle, over its own population, e = |sum_j psi_ij v_j|^2 / ((sum_j psi_ij)^2 h)
 * with the Mexican-hat wavelet psi (self included), colour = 0.3 if the
 * particle is within 0.0025 of its neighbours' mass centre, else min(e, 300)/300.
 * Off by default; when on, every step writes it.  sph2_get_colors returns the
 * last step's values in that step's sorted order with the persistent ids
 * (*count = particles of that step; any pointer may be NULL). */
int sph2_set_color_output(sph_solver2* s, int32_t on);
int sph2_get_colors(sph_solver2* s, int32_t population, float* colour, uint32_t* ids_sorted,
                    uint32_t* count);
/* Two-scale state I/O, as sph_save_state / sph_create_from_state: both
 * populations with blend coefficients, state bits and group ids, the group
 * and id counters, capacities and the presorted boundary. */
int sph2_step_count(sph_solver2* s, uint64_t* steps);
int sph2_save_state(sph_solver2* s, void* dst, uint64_t capacity, uint64_t* bytes);
int sph2_create_from_state(const void* src, uint64_t bytes, sph_solver2** out);
/* Frame record of both populations in their current order, each preceded by
 * its persistent ids; fields: positions, velocities, blend. */
int sph2_write_frame(sph_solver2* s, const char* path, uint32_t fields, int32_t append);

/* ---- batched single-scale scenes --------------------------------------- */

/* One scene of a batch: its own particles, boundary and configuration (grid,
 * h, masses, viscosity, stiffness may all differ between scenes). */
typedef struct sph_scene_desc {
    const float* fluid_xyz;
    uint32_t n_fluid;
    const float* boundary_xyz;
    uint32_t n_boundary;
    const float* velocity_xyz; /* NULL = zero */
    sph_config config;
} sph_scene_desc;

typedef struct sph_batch sph_batch;

/* Many independent Solver instances stepped together.  The reference can
 * step only one solver at a time (one bound __constant__ configuration,
 * SPH2S_FINAL_SINGLE_SCALE/Solver.cu:12, 1068-1080); a batch packs the
 * scenes and advances all of them with one launch per kernel, each step one
 * CUDA graph.  Every scene evolves exactly as sph_create/sph_advance would
 * evolve it alone. */
int sphb_create(const sph_scene_desc* scenes, uint32_t num_scenes, sph_batch** out);
int sphb_advance(sph_batch* b, float dt, int32_t steps);
int sphb_sync(sph_batch* b);
void* sphb_stream(sph_batch* b);
int sphb_counts(sph_batch* b, uint32_t* num_scenes, uint32_t* total_fluid,
                uint32_t* total_boundary);
/* Positions, velocities (3 floats per particle) and densities of one scene,
 * sorted order or by the scene-local creation index; each pointer optional. */
int sphb_get_scene(sph_batch* b, uint32_t scene, float* xyz, float* vel, float* rho,
                   int32_t order);
/* Times block sizes 128/256/512 for the density and force passes and 2/4/8
 * resident blocks per SM for the persistent grid on the batch's own data,
 * keeps the fastest (choice3 = density block, force block, blocks per SM),
 * and restores the particle state. */
int sphb_autotune(sph_batch* b, float dt, int32_t* choice3);
int sphb_destroy(sph_batch* b);

/* Batched differentiable rollout (no counterpart in the reference): the
 * sph_rollout_* sequence for every scene of the batch at once, through the
 * batch's packed arrays and one launch per kernel.  Arrays are packed by
 * scene in scene order, each scene's particles in creation order:
 *   v0_xyz, grad_v0, grad_x0   3 floats per particle (all scenes)
 *   viscosity, loss, grad_mu   one value per scene (viscosity NULL = keep)
 *   nodes                      one node grid per scene
 *   target, field              the scenes' node values, concatenated
 * Each scene's loss, fields and gradients equal those of a single-scale
 * solver on that scene. */
int sphb_rollout_forward(sph_batch* b, const float* v0_xyz, const float* viscosity, float dt,
                         int32_t steps, int32_t checkpoint_every);
int sphb_rollout_density_loss(sph_batch* b, const sph_grid* nodes, const float* target,
                              float* field, double* loss);
int sphb_rollout_backward(sph_batch* b, float* grad_v0, float* grad_x0, double* grad_mu);

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
 * and pass only their own buffers (an engine whose memory manager owns every
 * device allocation), or loops that must not risk an allocation's implicit
 * synchronisation.  Same arguments and results as sph_sort_pairs; calls no
 * cudaMalloc/cudaFree.  Its scratch is one static device array of about 10 MB
 * that each GPU loading the library holds until exit, which limits n to
 * 1,048,576 pairs (larger n: SPH_E_CAPACITY).  The first call on a device
 * looks the array up (make it before any stream capture; the lookup is
 * repeated after the device's context is recreated); all calls share the
 * array, so calls that overlap on the GPU race and must be serialised by the
 * caller. */
int sph_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                           uint32_t* vals_out, uint32_t n, int32_t key_bits, void* stream);

/* The step's coherent sort on keys in device memory (no counterpart in the
 * reference): the stable ascending order of n keys (low `key_bits` bits, the
 * others 0), given `hint`, any non-decreasing array of n uint32 in device
 * memory -- typically the same objects' sorted keys of a moment earlier.
 * keys_out = the sorted keys and perm_out[i] = the input index of the i-th
 * of them, exactly sph_sort_pairs with values 0..n-1, for every hint; the
 * hint sets only the cost: keys that differ from the hint at their own index
 * are radix-sorted, the others merged around them in one pass.  A hint that
 * decreases anywhere: SPH_E_INVALID, outputs untouched.  Enqueues on
 * `stream`, allocates its scratch with cudaMalloc, and returns after the sort
 * completed. */
int sph_sort_keys_coherent(const uint32_t* keys_in, const uint32_t* hint, uint32_t* keys_out,
                           uint32_t* perm_out, uint32_t n, int32_t key_bits, void* stream);

/* Description of the last failure on the calling thread ("" if none). */
const char* sph_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SPH2S_H */
