// sph2s_solver2.hpp -- header-only drop-in for the two-scale project's Grid,
// SolverConfiguration, ParticleData and Solver classes
// (SPH2S_FINAL_TWO_SCALE/Grid.h:9-58, Solver.h:14-144, ParticleData.h:9-54),
// forwarding to the two-scale entry points of include/sph2s.h.  The two-scale
// host program -- initSim in SPH2S_FINAL_TWO_SCALE/main.cpp:149-258, a LOW
// ParticleData from CreateParticleBox, an empty HIGH one of eight times its
// capacity, a boundary from Union, MakeConfiguration with a blend increment,
// new Solver(low, high, boundary, &config), Advance(dt) once per frame --
// compiles against this header unchanged apart from its GL and video code.
//
// ParticleData keeps public NumParticles, MaxParticles and device arrays
// dPositions (3 floats per particle), dColorValues and dStates (one int32 per
// particle), in plain device memory instead of GL vertex buffers (Map / Unmap
// are no-ops).  Solver copies both populations and the boundary into its
// handle at construction, with each population's MaxParticles as its
// capacity; every Advance runs one step and writes the new positions and
// state bits of both populations back into their ParticleData (in the order
// the next step starts from) and sets their NumParticles, then returns, like
// the reference's Advance, which reads the counts back every step
// (SPH2S_FINAL_TWO_SCALE/Solver.cu:1633-1638).  A population that outgrows its
// MaxParticles makes Advance throw.  The colour / energy values stay with the
// solver (sph2_get_colors, by persistent id); dColorValues is left as it was.
// SolverConfiguration carries the reference's members first and then this
// build's refinement controls (RefineAxis = -1: no slab, as the reference,
// whose own split marking is commented out, Solver.cu:1077-1082).  Errors
// throw std::runtime_error with sph_last_error(), as CUDA::SafeCall does.
// Needs the CUDA runtime (cudaMalloc for ParticleData).
#pragma once
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "sph2s.h"

namespace sph2s_compat2 {

inline void check(int rc) {
    if (rc != SPH_OK) throw std::runtime_error(sph_last_error());
}

inline void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace sph2s_compat2

// Grid (SPH2S_FINAL_TWO_SCALE/Grid.h:9-58); same layout as sph_grid.
struct Grid {
    static unsigned int ComputeNumGridCells(const Grid& grid) {
        return grid.Dimensions.x * grid.Dimensions.y * grid.Dimensions.z;
    }

    static Grid MakeGrid(float3 origin, float3 end, float spacing) {
        const float o[3] = {origin.x, origin.y, origin.z};
        const float e[3] = {end.x, end.y, end.z};
        sph_grid g;
        sph2s_compat2::check(sph_make_grid(o, e, spacing, &g));
        return FromABI(g);
    }

    static Grid MakeGrid(float3 origin, int3 dimensions, float spacing) {
        Grid grid;
        grid.Origin = origin;
        grid.Dimensions = dimensions;
        grid.Spacing = spacing;
        return grid;
    }

    static float ComputeVolume(const Grid& grid) {
        return grid.Dimensions.x * grid.Dimensions.y * grid.Dimensions.z * grid.Spacing *
               grid.Spacing * grid.Spacing;
    }

    static Grid FromABI(const sph_grid& g) {
        return MakeGrid(make_float3(g.origin[0], g.origin[1], g.origin[2]),
                        make_int3(g.dims[0], g.dims[1], g.dims[2]), g.spacing);
    }

    sph_grid ToABI() const {
        sph_grid g;
        g.origin[0] = Origin.x;
        g.origin[1] = Origin.y;
        g.origin[2] = Origin.z;
        g.dims[0] = Dimensions.x;
        g.dims[1] = Dimensions.y;
        g.dims[2] = Dimensions.z;
        g.spacing = Spacing;
        return g;
    }

    float3 Origin;
    int3 Dimensions;
    float Spacing;
};
static_assert(sizeof(Grid) == sizeof(sph_grid), "Grid mirrors sph_grid");

// SolverConfiguration (SPH2S_FINAL_TWO_SCALE/Solver.h:14-61) + refinement controls.
struct SolverConfiguration {
    static SolverConfiguration MakeConfiguration(float3 origin, float3 end, float volume,
                                                 unsigned int numParticles, unsigned int avgParticles,
                                                 float restDensity, float bulkModulus, float viscosity,
                                                 float speedSound, float tensionCoefficient,
                                                 float blendIncrement) {
        const float o[3] = {origin.x, origin.y, origin.z};
        const float e[3] = {end.x, end.y, end.z};
        sph_config2 c;
        sph2s_compat2::check(sph_make_configuration2(o, e, volume, numParticles, avgParticles,
                                                     restDensity, bulkModulus, viscosity, speedSound,
                                                     tensionCoefficient, blendIncrement, &c));
        return FromABI(c);
    }

    static SolverConfiguration FromABI(const sph_config2& c) {
        SolverConfiguration s;
        for (int r = 0; r < 2; ++r) {
            s.EffectiveRadius[r] = c.effective_radius[r];
            s.FluidParticleMass[r] = c.fluid_particle_mass[r];
            s.Grid[r] = ::Grid::FromABI(c.grid[r]);
        }
        s.BoundaryParticleMass = c.boundary_particle_mass;
        s.RestDensity = c.rest_density;
        s.BulkModulus = c.bulk_modulus;
        s.Viscosity = c.viscosity;
        s.SpeedSound = c.speed_sound;
        s.TensionCoefficient = c.tension_coefficient;
        s.BlendIncrement = c.blend_increment;
        s.RefineAxis = c.refine_axis;
        s.RefineLo = c.refine_lo;
        s.RefineHi = c.refine_hi;
        s.Mode = c.mode;
        s.SplitTrigger = c.split_trigger;
        s.SurfaceDensity = c.surface_density;
        return s;
    }

    sph_config2 ToABI() const {
        sph_config2 c;
        for (int r = 0; r < 2; ++r) {
            c.effective_radius[r] = EffectiveRadius[r];
            c.fluid_particle_mass[r] = FluidParticleMass[r];
            c.grid[r] = Grid[r].ToABI();
        }
        c.boundary_particle_mass = BoundaryParticleMass;
        c.rest_density = RestDensity;
        c.bulk_modulus = BulkModulus;
        c.viscosity = Viscosity;
        c.speed_sound = SpeedSound;
        c.tension_coefficient = TensionCoefficient;
        c.blend_increment = BlendIncrement;
        c.refine_axis = RefineAxis;
        c.refine_lo = RefineLo;
        c.refine_hi = RefineHi;
        c.mode = Mode;
        c.split_trigger = SplitTrigger;
        c.surface_density = SurfaceDensity;
        return c;
    }

    // the reference's members (Solver.h:52-61)
    float EffectiveRadius[2];
    float FluidParticleMass[2];
    float BoundaryParticleMass;
    float RestDensity;
    float BulkModulus;
    float Viscosity;
    float SpeedSound;
    float TensionCoefficient;
    float BlendIncrement;
    ::Grid Grid[2];
    // refinement controls of this build (sph_config2): slab split / merge,
    // coupled mode, surface trigger
    int RefineAxis = -1;
    float RefineLo = 0.0f, RefineHi = 0.0f;
    int Mode = SPH2_MODE_BLENDED;
    int SplitTrigger = SPH2_SPLIT_SLAB;
    float SurfaceDensity = 0.0f;
};

// ParticleData (SPH2S_FINAL_TWO_SCALE/ParticleData.h:9-54) without OpenGL.
class ParticleData {
public:
    explicit ParticleData(unsigned int maxParticles)
        : NumParticles(maxParticles), MaxParticles(maxParticles) {  // all particles active
        const size_t n = maxParticles ? maxParticles : 1;
        sph2s_compat2::check_cuda(cudaMalloc(&dPositions, sizeof(float) * 3 * n), "ParticleData");
        sph2s_compat2::check_cuda(cudaMalloc(&dColorValues, sizeof(float) * n), "ParticleData");
        sph2s_compat2::check_cuda(cudaMalloc(&dStates, sizeof(int) * n), "ParticleData");
        sph2s_compat2::check_cuda(cudaMemset(dColorValues, 0, sizeof(float) * n), "ParticleData");
        sph2s_compat2::check_cuda(cudaMemset(dStates, 0, sizeof(int) * n), "ParticleData");
    }
    ~ParticleData() {
        cudaFree(dPositions);
        cudaFree(dColorValues);
        cudaFree(dStates);
    }
    ParticleData(const ParticleData&) = delete;
    ParticleData& operator=(const ParticleData&) = delete;

    void Map() {}
    void Unmap() {}

    static ParticleData* CreateParticleBox(const Grid& grid) {
        const sph_grid g = grid.ToABI();
        uint32_t n = 0;
        sph2s_compat2::check(sph_particle_box(&g, nullptr, 0, &n));
        std::vector<float> xyz(3 * (size_t)n);
        sph2s_compat2::check(sph_particle_box(&g, xyz.data(), n, &n));
        return FromHost(xyz, n);
    }

    static ParticleData* CreateParticleBoxCanvas(const Grid& grid, int border) {
        const sph_grid g = grid.ToABI();
        uint32_t n = 0;
        sph2s_compat2::check(sph_particle_box_canvas(&g, border, nullptr, 0, &n));
        std::vector<float> xyz(3 * (size_t)n);
        sph2s_compat2::check(sph_particle_box_canvas(&g, border, xyz.data(), n, &n));
        return FromHost(xyz, n);
    }

    // ParticleData::Union: a's particles, then b's; NULL if either is NULL.
    static ParticleData* Union(const ParticleData* a, const ParticleData* b) {
        if (!a || !b) return nullptr;
        ParticleData* r = new ParticleData(a->MaxParticles + b->MaxParticles);
        sph2s_compat2::check_cuda(cudaMemcpy(r->dPositions, a->dPositions, 12 * (size_t)a->NumParticles,
                                             cudaMemcpyDeviceToDevice), "Union");
        sph2s_compat2::check_cuda(cudaMemcpy(r->dPositions + 3 * (size_t)a->NumParticles, b->dPositions,
                                             12 * (size_t)b->NumParticles, cudaMemcpyDeviceToDevice),
                                  "Union");
        return r;
    }

    static ParticleData* FromHost(const std::vector<float>& xyz, unsigned int n) {
        ParticleData* p = new ParticleData(n);
        if (n)
            sph2s_compat2::check_cuda(cudaMemcpy(p->dPositions, xyz.data(), 12 * (size_t)n,
                                                 cudaMemcpyHostToDevice), "ParticleData");
        return p;
    }

    std::vector<float> PositionsToHost() const {
        std::vector<float> xyz(3 * (size_t)NumParticles);
        if (NumParticles)
            sph2s_compat2::check_cuda(cudaMemcpy(xyz.data(), dPositions, xyz.size() * 4,
                                                 cudaMemcpyDeviceToHost), "ParticleData");
        return xyz;
    }

    std::vector<int> StatesToHost() const {
        std::vector<int> st(NumParticles);
        if (NumParticles)
            sph2s_compat2::check_cuda(cudaMemcpy(st.data(), dStates, st.size() * 4,
                                                 cudaMemcpyDeviceToHost), "ParticleData");
        return st;
    }

    unsigned int NumParticles;
    unsigned int MaxParticles;
    float* dPositions = nullptr;
    float* dColorValues = nullptr;
    int* dStates = nullptr;
};

// Solver (SPH2S_FINAL_TWO_SCALE/Solver.h:64-144).
class Solver {
public:
    Solver(ParticleData* fluidData, ParticleData* fluidDataHigh, ParticleData* boundaryData,
           const SolverConfiguration* configuration)
        : mPop{fluidData, fluidDataHigh} {
        if (!fluidData || !fluidDataHigh || !boundaryData || !configuration)
            throw std::runtime_error("Solver: NULL particle data or configuration");
        const sph_config2 c = configuration->ToABI();
        const std::vector<float> low = fluidData->PositionsToHost();
        const std::vector<float> high = fluidDataHigh->PositionsToHost();
        const std::vector<float> boundary = boundaryData->PositionsToHost();
        sph2s_compat2::check(sph2_create(&c, low.data(), fluidData->NumParticles, high.data(),
                                         fluidDataHigh->NumParticles, boundary.data(),
                                         boundaryData->NumParticles, fluidData->MaxParticles,
                                         fluidDataHigh->MaxParticles, &mHandle));
        WriteBack();  // states 0 (LOW) and 4 (HIGH), as the reference's constructor sets them
    }
    ~Solver() { sph2_destroy(mHandle); }
    Solver(const Solver&) = delete;
    Solver& operator=(const Solver&) = delete;

    void Bind() const {}  // the configuration lives in the handle

    void Advance(float dt) {
        sph2s_compat2::check(sph2_advance(mHandle, dt, 1));
        WriteBack();
    }

    // The handle, for the ABI's further reads (velocities, blend values, colours, ids).
    sph_solver2* Handle() const { return mHandle; }

private:
    void WriteBack() {
        uint32_t n[2] = {0, 0}, nb = 0, groups = 0;
        sph2s_compat2::check(sph2_counts(mHandle, &n[0], &n[1], &nb, &groups));
        for (int r = 0; r < 2; ++r) {
            if (n[r] > mPop[r]->MaxParticles)
                throw std::runtime_error("Solver: a population outgrew its ParticleData");
            sph2s_compat2::check(sph2_get_positions_device(mHandle, r, mPop[r]->dPositions));
            sph2s_compat2::check(sph2_get_states_device(mHandle, r, mPop[r]->dStates));
            mPop[r]->NumParticles = n[r];
        }
        sph2s_compat2::check_cuda(cudaDeviceSynchronize(), "Advance");
    }

    ParticleData* mPop[2];
    sph_solver2* mHandle = nullptr;
};
