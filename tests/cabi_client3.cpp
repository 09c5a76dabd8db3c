// cabi_client3.cpp -- the reference's single-scale host program flow
// (initSim / display / tearDownSim, SPH2S_FINAL_SINGLE_SCALE/main.cpp:79,
// 161-267) written against include/sph2s_solver.hpp, the header-only drop-in
// for its Grid, SolverConfiguration, ParticleData and Solver classes.  The
// scene is initSim's (fluid box, two boundary canvases joined by Union, the
// same MakeConfiguration arguments) at a coarser spacing of 0.02 so the test
// runs in seconds; display()'s Advance(0.001f) is called once per step and
// the positions are read from the fluid ParticleData's device array, as the
// reference's renderer reads them.
//
// usage: cabi_client3 <out.bin> <steps>
// Writes: u32 n_fluid, n_boundary, steps | f32 dt | sph_config | fluid xyz |
// boundary xyz (as created) | fluid->dPositions after the steps (sorted
// order) | persistent ids of that order.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sph2s_solver.hpp"

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: cabi_client3 <out.bin> <steps>\n");
        return 1;
    }
    const int steps = std::atoi(argv[2]);
    const float spacing = 0.02f;
    const float dt = 0.001f;
    try {
        // INIT PARTICLE DATA
        Grid particleGrid = Grid::MakeGrid(make_float3(0.04f, 0.04f, -0.0f),
                                           make_float3(0.35f, 0.75f, 0.4f), spacing);
        ParticleData* fluid = ParticleData::CreateParticleBox(particleGrid);
        // INIT BOUNDARY PARTICLES
        Grid boundaryGridA = Grid::MakeGrid(make_float3(0.0f, 0.0f, -0.1f),
                                            make_float3(1.6f, 1.5f, 0.5f), spacing);
        Grid boundaryGridB = Grid::MakeGrid(make_float3(0.7f, 0.0f, 0.22f),
                                            make_float3(0.75f, 1.5f, 0.25f), spacing);
        ParticleData* boundaryA = ParticleData::CreateParticleBoxCanvas(boundaryGridA, 5);
        ParticleData* boundaryB = ParticleData::CreateParticleBoxCanvas(boundaryGridB, 5);
        ParticleData* boundary = ParticleData::Union(boundaryA, boundaryB);
        delete boundaryA;
        delete boundaryB;
        // INIT SOLVER
        SolverConfiguration config = SolverConfiguration::MakeConfiguration(
            make_float3(-0.1f, -0.1f, -0.2f), make_float3(1.7f, 1.6f, 0.6f),
            Grid::ComputeVolume(particleGrid), fluid->MaxParticles,
            35,        // avg. particle neighbors
            1000.0f,   // rest density
            30.0f,     // bulk modulus
            5.0f,      // viscosity
            88.1472f,  // speed of sound in fluid
            0.8f,      // tension coefficient
            0.05f);
        const std::vector<float> fluid0 = fluid->PositionsToHost();
        const std::vector<float> boundary0 = boundary->PositionsToHost();
        Solver* solver = new Solver(fluid, boundary, &config);
        solver->Bind();
        for (int k = 0; k < steps; ++k) solver->Advance(dt);  // display()
        const std::vector<float> x = fluid->PositionsToHost();
        std::vector<uint32_t> ids(fluid->NumParticles);
        sph2s_compat::check(sph_get_ids(solver->Handle(), ids.data()));

        FILE* f = std::fopen(argv[1], "wb");
        if (!f) return 2;
        const uint32_t hdr[3] = {fluid->NumParticles, boundary->NumParticles, (uint32_t)steps};
        const sph_config c = config.ToABI();
        std::fwrite(hdr, 4, 3, f);
        std::fwrite(&dt, 4, 1, f);
        std::fwrite(&c, sizeof(c), 1, f);
        std::fwrite(fluid0.data(), 4, fluid0.size(), f);
        std::fwrite(boundary0.data(), 4, boundary0.size(), f);
        std::fwrite(x.data(), 4, x.size(), f);
        std::fwrite(ids.data(), 4, ids.size(), f);
        std::fclose(f);
        // tearDownSim
        delete fluid;
        delete boundary;
        delete solver;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "cabi_client3: %s\n", e.what());
        return 3;
    }
    return 0;
}
