// sph2s_solver.hpp -- header-only drop-in for the single-scale project's
// Grid, SolverConfiguration, ParticleData and Solver classes
// (SPH2S_FINAL_SINGLE_SCALE/Grid.h:9-58, Solver.h:13-132, ParticleData.h:9-51),
// forwarding to the C ABI of include/sph2s.h.  A host program written against
// the reference -- initSim / display / tearDownSim in
// SPH2S_FINAL_SINGLE_SCALE/main.cpp:161-267 -- compiles against this header
// unchanged apart from its GL and video code:
//
//   ParticleData* fluid = ParticleData::CreateParticleBox(particleGrid);
//   ParticleData* boundary = ParticleData::Union(a, b);
//   SolverConfiguration config = SolverConfiguration::MakeConfiguration(...);
//   Solver* solver = new Solver(fluid, boundary, &config);
//   solver->Bind();
//   solver->Advance(dt);            // fluid->dPositions now holds the new positions
//
// ParticleData keeps public device arrays dPositions (3 floats per particle)
// and dColorValues, but in plain device memory instead of a GL vertex buffer,
// so Map / Unmap are no-ops.  Solver copies the particles into its own handle
// at construction; each Advance runs one step and writes the positions back
// into the fluid ParticleData's dPositions in the step's sorted order (the
// reference's integrate writes them there in sorted order,
// SPH2S_FINAL_SINGLE_SCALE/Solver.cu:713-755) and returns after the step
// finished, like the reference's Advance.  The reference also rewrites the
// boundary ParticleData in its presorted order (Solver.cu:1055); here the
// caller's boundary array is left as it was.  Errors throw std::runtime_error
// with sph_last_error(), as CUDA::SafeCall does (SPH2S_FINAL_SINGLE_SCALE/
// cuda.h:115-129).  Needs the CUDA runtime (cudaMalloc for ParticleData).
#pragma once
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "sph2s.h"

namespace sph2s_compat {

inline void check(int rc) {
    if (rc != SPH_OK) throw std::runtime_error(sph_last_error());
}

inline void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace sph2s_compat

// Grid (SPH2S_FINAL_SINGLE_SCALE/Grid.h:9-58); same layout as sph_grid.
struct Grid {
    static unsigned int ComputeNumGridCells(const Grid& grid) {
        return grid.Dimensions.x * grid.Dimensions.y * grid.Dimensions.z;
    }

    static Grid MakeGrid(float3 origin, float3 end, float spacing) {
        const float o[3] = {origin.x, origin.y, origin.z};
        const float e[3] = {end.x, end.y, end.z};
        sph_grid g;
        sph2s_compat::check(sph_make_grid(o, e, spacing, &g));
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

// SolverConfiguration (SPH2S_FINAL_SINGLE_SCALE/Solver.h:13-60); same layout as sph_config.
struct SolverConfiguration {
    static SolverConfiguration MakeConfiguration(float3 origin, float3 end, float volume,
                                                 unsigned int numParticles, unsigned int avgParticles,
                                                 float restDensity, float bulkModulus, float viscosity,
                                                 float speedSound, float tensionCoefficient,
                                                 float epsilon) {
        const float o[3] = {origin.x, origin.y, origin.z};
        const float e[3] = {end.x, end.y, end.z};
        sph_config c;
        sph2s_compat::check(sph_make_configuration(o, e, volume, numParticles, avgParticles,
                                                   restDensity, bulkModulus, viscosity, speedSound,
                                                   tensionCoefficient, epsilon, &c));
        return FromABI(c);
    }

    static SolverConfiguration FromABI(const sph_config& c) {
        SolverConfiguration s;
        s.EffectiveRadius = c.effective_radius;
        s.FluidParticleMass = c.fluid_particle_mass;
        s.BoundaryParticleMass = c.boundary_particle_mass;
        s.RestDensity = c.rest_density;
        s.BulkModulus = c.bulk_modulus;
        s.Viscosity = c.viscosity;
        s.SpeedSound = c.speed_sound;
        s.TensionCoefficient = c.tension_coefficient;
        s.XSPHCoeff = c.xsph_coeff;
        s.Grid = ::Grid::FromABI(c.grid);
        return s;
    }

    sph_config ToABI() const {
        sph_config c;
        c.effective_radius = EffectiveRadius;
        c.fluid_particle_mass = FluidParticleMass;
        c.boundary_particle_mass = BoundaryParticleMass;
        c.rest_density = RestDensity;
        c.bulk_modulus = BulkModulus;
        c.viscosity = Viscosity;
        c.speed_sound = SpeedSound;
        c.tension_coefficient = TensionCoefficient;
        c.xsph_coeff = XSPHCoeff;
        c.grid = Grid.ToABI();
        return c;
    }

    float EffectiveRadius;
    float FluidParticleMass;
    float BoundaryParticleMass;
    float RestDensity;
    float BulkModulus;
    float Viscosity;
    float SpeedSound;
    float TensionCoefficient;
    float XSPHCoeff;
    ::Grid Grid;
};
static_assert(sizeof(SolverConfiguration) == sizeof(sph_config), "mirrors sph_config");

// ParticleData (SPH2S_FINAL_SINGLE_SCALE/ParticleData.h:9-51) without OpenGL:
// the arrays are device memory owned by the object.
class ParticleData {
public:
    explicit ParticleData(unsigned int maxParticles)
        : NumParticles(maxParticles), MaxParticles(maxParticles) {  // all particles active
        const size_t n = maxParticles ? maxParticles : 1;
        sph2s_compat::check_cuda(cudaMalloc(&dPositions, sizeof(float) * 3 * n), "ParticleData");
        sph2s_compat::check_cuda(cudaMalloc(&dColorValues, sizeof(float) * n), "ParticleData");
        sph2s_compat::check_cuda(cudaMemset(dColorValues, 0, sizeof(float) * n), "ParticleData");
    }
    ~ParticleData() {
        cudaFree(dPositions);
        cudaFree(dColorValues);
    }
    ParticleData(const ParticleData&) = delete;
    ParticleData& operator=(const ParticleData&) = delete;

    void Map() {}
    void Unmap() {}

    static ParticleData* CreateParticleBox(const Grid& grid) {
        const sph_grid g = grid.ToABI();
        uint32_t n = 0;
        sph2s_compat::check(sph_particle_box(&g, nullptr, 0, &n));
        std::vector<float> xyz(3 * (size_t)n);
        sph2s_compat::check(sph_particle_box(&g, xyz.data(), n, &n));
        return FromHost(xyz, n);
    }

    static ParticleData* CreateParticleBoxCanvas(const Grid& grid, int border) {
        const sph_grid g = grid.ToABI();
        uint32_t n = 0;
        sph2s_compat::check(sph_particle_box_canvas(&g, border, nullptr, 0, &n));
        std::vector<float> xyz(3 * (size_t)n);
        sph2s_compat::check(sph_particle_box_canvas(&g, border, xyz.data(), n, &n));
        return FromHost(xyz, n);
    }

    // ParticleData::Union (SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:68-126): a's
    // particles, then b's; NULL if either is NULL.
    static ParticleData* Union(const ParticleData* a, const ParticleData* b) {
        if (!a || !b) return nullptr;
        ParticleData* r = new ParticleData(a->MaxParticles + b->MaxParticles);
        sph2s_compat::check_cuda(cudaMemcpy(r->dPositions, a->dPositions, 12 * (size_t)a->NumParticles,
                                            cudaMemcpyDeviceToDevice), "Union");
        sph2s_compat::check_cuda(cudaMemcpy(r->dPositions + 3 * (size_t)a->NumParticles, b->dPositions,
                                            12 * (size_t)b->NumParticles, cudaMemcpyDeviceToDevice),
                                 "Union");
        return r;
    }

    static ParticleData* FromHost(const std::vector<float>& xyz, unsigned int n) {
        ParticleData* p = new ParticleData(n);
        if (n)
            sph2s_compat::check_cuda(cudaMemcpy(p->dPositions, xyz.data(), 12 * (size_t)n,
                                                cudaMemcpyHostToDevice), "ParticleData");
        return p;
    }

    std::vector<float> PositionsToHost() const {
        std::vector<float> xyz(3 * (size_t)NumParticles);
        if (NumParticles)
            sph2s_compat::check_cuda(cudaMemcpy(xyz.data(), dPositions, xyz.size() * 4,
                                                cudaMemcpyDeviceToHost), "ParticleData");
        return xyz;
    }

    unsigned int NumParticles;
    unsigned int MaxParticles;
    float* dPositions = nullptr;
    float* dColorValues = nullptr;
};

// Solver (SPH2S_FINAL_SINGLE_SCALE/Solver.h:62-132).
class Solver {
public:
    Solver(ParticleData* fluidData, ParticleData* boundaryData,
           const SolverConfiguration* configuration)
        : mFluid(fluidData) {
        if (!fluidData || !boundaryData || !configuration)
            throw std::runtime_error("Solver: NULL particle data or configuration");
        const sph_config c = configuration->ToABI();
        const std::vector<float> fluid = fluidData->PositionsToHost();
        const std::vector<float> boundary = boundaryData->PositionsToHost();
        sph2s_compat::check(sph_create(&c, fluid.data(), fluidData->NumParticles, boundary.data(),
                                       boundaryData->NumParticles, nullptr, &mHandle));
    }
    ~Solver() { sph_destroy(mHandle); }
    Solver(const Solver&) = delete;
    Solver& operator=(const Solver&) = delete;

    void Bind() const {}  // the configuration lives in the handle, not in __constant__ memory

    void Advance(float dt) {
        sph2s_compat::check(sph_advance(mHandle, dt, 1));
        sph2s_compat::check(sph_get_positions_device(mHandle, mFluid->dPositions, SPH_ORDER_SORTED));
        sph2s_compat::check(sph_sync(mHandle));
    }

    // The handle, for the ABI's further reads (velocities, densities, ids, state I/O).
    sph_solver* Handle() const { return mHandle; }

private:
    ParticleData* mFluid;
    sph_solver* mHandle = nullptr;
};
