// cabi_client.cpp -- a C++ client of include/sph2s.h written the way the
// reference's host code would drive its solver: the adapter class keeps the
// reference's `Solver` name and constructor shape (SPH2S_FINAL_SINGLE_SCALE/
// Solver.h:113-121) and forwards to the C ABI; the scene is built with the
// replacements of Grid::MakeGrid, ParticleData::CreateParticleBox(Canvas) and
// SolverConfiguration::MakeConfiguration, as initSim does
// (SPH2S_FINAL_SINGLE_SCALE/main.cpp:161-258).
//
// usage: cabi_client <out.bin> <steps>
// Writes: u32 n_fluid, n_boundary, steps | f32 dt | sph_config | fluid xyz |
// boundary xyz | positions after the steps (by id) | densities (by id).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "sph2s.h"

namespace {

void check(int rc) {
    if (rc != SPH_OK) throw std::runtime_error(sph_last_error());  // CUDA::SafeCall's behaviour
}

class Solver {
public:
    Solver(const std::vector<float>& fluid, const std::vector<float>& boundary,
           const sph_config* configuration) {
        check(sph_create(configuration, fluid.data(), (uint32_t)(fluid.size() / 3), boundary.data(),
                         (uint32_t)(boundary.size() / 3), nullptr, &handle_));
        n_ = (uint32_t)(fluid.size() / 3);
    }
    ~Solver() { sph_destroy(handle_); }
    Solver(const Solver&) = delete;
    Solver& operator=(const Solver&) = delete;
    void Bind() const {}
    void Advance(float dt) { check(sph_advance(handle_, dt, 1)); }
    std::vector<float> Positions(int32_t order) {
        std::vector<float> xyz(3 * (size_t)n_);
        check(sph_get_positions(handle_, xyz.data(), order));
        return xyz;
    }
    std::vector<float> Densities(int32_t order) {
        std::vector<float> rho(n_);
        check(sph_get_densities(handle_, rho.data(), order));
        return rho;
    }

private:
    sph_solver* handle_ = nullptr;
    uint32_t n_ = 0;
};

std::vector<float> particle_box(const sph_grid& g) {
    uint32_t n = 0;
    check(sph_particle_box(&g, nullptr, 0, &n));
    std::vector<float> xyz(3 * (size_t)n);
    check(sph_particle_box(&g, xyz.data(), n, &n));
    return xyz;
}

std::vector<float> particle_box_canvas(const sph_grid& g, int32_t border) {
    uint32_t n = 0;
    check(sph_particle_box_canvas(&g, border, nullptr, 0, &n));
    std::vector<float> xyz(3 * (size_t)n);
    check(sph_particle_box_canvas(&g, border, xyz.data(), n, &n));
    return xyz;
}

void put(FILE* f, const void* p, size_t bytes) {
    if (bytes && std::fwrite(p, 1, bytes, f) != bytes) throw std::runtime_error("short write");
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s <out.bin> <steps>\n", argv[0]);
        return 2;
    }
    try {
        const uint32_t steps = (uint32_t)std::strtoul(argv[2], nullptr, 10);
        const float s = 1.0f / 32.0f, dt = 1e-4f;
        const float origin[3] = {0.0f, 0.0f, 0.0f}, block_end[3] = {0.5f, 0.5f, 0.5f},
                    box_end[3] = {1.0f, 1.0f, 1.0f};
        // fluid block [0, 0.5)^3 on a lattice of spacing s, boundary shell of the unit box
        sph_grid block, box;
        check(sph_make_grid(origin, block_end, s, &block));
        check(sph_make_grid(origin, box_end, s, &box));
        const std::vector<float> fluid = particle_box(block);
        const std::vector<float> boundary = particle_box_canvas(box, 3);
        // h from the average neighbour count over the fluid volume, grid of spacing h
        sph_config cfg;
        check(sph_make_configuration(origin, box_end, 0.125f, (uint32_t)(fluid.size() / 3), 35,
                                     1000.0f, 30.0f, 5.0f, 88.1472f, 0.8f, 0.0f, &cfg));
        Solver solver(fluid, boundary, &cfg);
        solver.Bind();
        for (uint32_t k = 0; k < steps; ++k) solver.Advance(dt);
        const std::vector<float> x = solver.Positions(SPH_ORDER_BY_ID);
        const std::vector<float> rho = solver.Densities(SPH_ORDER_BY_ID);

        FILE* f = std::fopen(argv[1], "wb");
        if (!f) throw std::runtime_error(std::string("cannot open ") + argv[1]);
        const uint32_t head[3] = {(uint32_t)(fluid.size() / 3), (uint32_t)(boundary.size() / 3),
                                  steps};
        put(f, head, sizeof(head));
        put(f, &dt, sizeof(dt));
        put(f, &cfg, sizeof(cfg));
        put(f, fluid.data(), 4 * fluid.size());
        put(f, boundary.data(), 4 * boundary.size());
        put(f, x.data(), 4 * x.size());
        put(f, rho.data(), 4 * rho.size());
        std::fclose(f);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "cabi_client: %s\n", e.what());
        return 1;
    }
    return 0;
}
