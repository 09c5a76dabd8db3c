// cabi_client4.cpp -- the reference's two-scale host program flow (initSim /
// display, SPH2S_FINAL_TWO_SCALE/main.cpp:68, 149-258) written against
// include/sph2s_solver2.hpp, the header-only drop-in for its Grid,
// SolverConfiguration, ParticleData and Solver classes.  initSim's scene
// (fluid box, an empty HIGH ParticleData of eight times the LOW capacity, two
// boundary canvases joined by Union, MakeConfiguration with the blend
// increment 0.0125) at a coarser spacing of 0.02 so the test runs in seconds;
// the refinement slab 0.1 < x < 0.2 is switched on through the configuration's
// refinement members so that HIGH particles appear.  display()'s
// Advance(0.001f) is called once per step and both populations are read from
// their ParticleData's device arrays, as the reference's renderers read them.
//
// usage: cabi_client4 <out.bin> <steps>
// Writes: u32 n_low, n_boundary, steps | f32 dt | sph_config2 | LOW xyz and
// boundary xyz (as created) | per population (LOW, HIGH): u32 NumParticles |
// dPositions xyz | dStates | persistent ids (sph2_get_state).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sph2s_solver2.hpp"

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: cabi_client4 <out.bin> <steps>\n");
        return 1;
    }
    const int steps = std::atoi(argv[2]);
    const float dt = 0.001f;
    try {
        // INIT PARTICLE DATA
        Grid particleGrid = Grid::MakeGrid(make_float3(0.02f, 0.04f, -0.05f),
                                           make_float3(0.35f, 0.75f, 0.45f), 0.02f);
        ParticleData* low = ParticleData::CreateParticleBox(particleGrid);
        ParticleData* high = new ParticleData(low->MaxParticles * 8);
        high->NumParticles = 0;
        // INIT BOUNDARY PARTICLES
        Grid boundaryGridA = Grid::MakeGrid(make_float3(0.0f, 0.0f, -0.1f),
                                            make_float3(1.6f, 1.5f, 0.5f), 0.03f);
        Grid boundaryGridB = Grid::MakeGrid(make_float3(0.7f, 0.0f, 0.22f),
                                            make_float3(0.75f, 1.5f, 0.25f), 0.03f);
        ParticleData* boundaryA = ParticleData::CreateParticleBoxCanvas(boundaryGridA, 5);
        ParticleData* boundaryB = ParticleData::CreateParticleBoxCanvas(boundaryGridB, 5);
        ParticleData* boundary = ParticleData::Union(boundaryA, boundaryB);
        delete boundaryA;
        delete boundaryB;
        // INIT SOLVER
        SolverConfiguration config = SolverConfiguration::MakeConfiguration(
            make_float3(-0.1f, -0.1f, -0.2f), make_float3(1.7f, 1.6f, 0.6f),
            Grid::ComputeVolume(particleGrid), low->MaxParticles,
            35,        // avg. particle neighbors
            1000.0f,   // rest density
            30.0f,     // bulk modulus
            5.0f,      // viscosity
            88.1472f,  // speed of sound in fluid
            0.8f,      // tension coefficient
            0.0125f);  // blend increment
        config.RefineAxis = 0;  // this build's slab trigger
        config.RefineLo = 0.1f;
        config.RefineHi = 0.2f;
        const std::vector<float> low0 = low->PositionsToHost();
        const std::vector<float> boundary0 = boundary->PositionsToHost();
        Solver* solver = new Solver(low, high, boundary, &config);
        solver->Bind();
        for (int k = 0; k < steps; ++k) solver->Advance(dt);  // display()

        FILE* f = std::fopen(argv[1], "wb");
        if (!f) return 2;
        const uint32_t hdr[3] = {(uint32_t)(low0.size() / 3), boundary->NumParticles, (uint32_t)steps};
        const sph_config2 c = config.ToABI();
        std::fwrite(hdr, 4, 3, f);
        std::fwrite(&dt, 4, 1, f);
        std::fwrite(&c, sizeof(c), 1, f);
        std::fwrite(low0.data(), 4, low0.size(), f);
        std::fwrite(boundary0.data(), 4, boundary0.size(), f);
        ParticleData* pops[2] = {low, high};
        for (int r = 0; r < 2; ++r) {
            const uint32_t n = pops[r]->NumParticles;
            const std::vector<float> x = pops[r]->PositionsToHost();
            const std::vector<int> st = pops[r]->StatesToHost();
            std::vector<uint32_t> ids(n);
            sph2s_compat2::check(sph2_get_state(solver->Handle(), r, nullptr, nullptr, nullptr,
                                                nullptr, nullptr, ids.data()));
            std::fwrite(&n, 4, 1, f);
            std::fwrite(x.data(), 4, x.size(), f);
            std::fwrite(st.data(), 4, st.size(), f);
            std::fwrite(ids.data(), 4, ids.size(), f);
        }
        std::fclose(f);
        // tearDownSim
        delete low;
        delete high;
        delete boundary;
        delete solver;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "cabi_client4: %s\n", e.what());
        return 3;
    }
    return 0;
}
