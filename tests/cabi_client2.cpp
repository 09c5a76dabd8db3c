// cabi_client2.cpp -- a C++ client of the two-scale half of include/sph2s.h,
// written the way the reference's two-scale host code drives its solver: the
// adapter keeps the shape of Solver(low, high, boundary, config) + Bind() +
// Advance(dt) (SPH2S_FINAL_TWO_SCALE/Solver.h:121-130) and forwards to the C
// ABI; the scene comes from the ABI's grid, particle-box and configuration
// builders (SolverConfiguration::MakeConfiguration, Solver.h:16-50), with a
// refinement slab so that particles split, fade and merge.
//
// usage: cabi_client2 <out.bin> <steps>
// Writes: u32 n_low, n_boundary, steps | f32 dt | sph_config2 | low xyz |
// boundary xyz | u32 stats[6] of the last step | then per population (LOW,
// HIGH): u32 n | ids | xyz | vel | lambda | state | group.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "sph2s.h"

namespace {

void check(int rc) {
    if (rc != SPH_OK) throw std::runtime_error(sph_last_error());
}

struct Population {
    std::vector<uint32_t> ids, group;
    std::vector<float> xyz, vel, lambda;
    std::vector<int32_t> state;
};

class Solver {
public:
    Solver(const std::vector<float>& low, const std::vector<float>& high,
           const std::vector<float>& boundary, const sph_config2* configuration) {
        check(sph2_create(configuration, low.data(), (uint32_t)(low.size() / 3),
                          high.empty() ? nullptr : high.data(), (uint32_t)(high.size() / 3),
                          boundary.data(), (uint32_t)(boundary.size() / 3), 0, 0, &handle_));
    }
    ~Solver() { sph2_destroy(handle_); }
    Solver(const Solver&) = delete;
    Solver& operator=(const Solver&) = delete;
    void Bind() const {}
    void Advance(float dt) { check(sph2_advance(handle_, dt, 1)); }
    void LastStats(uint32_t stats[6]) { check(sph2_last_stats(handle_, stats)); }
    Population State(int32_t population) {
        uint32_t nl = 0, nh = 0;
        check(sph2_counts(handle_, &nl, &nh, nullptr, nullptr));
        const uint32_t n = population == SPH_LOW ? nl : nh;
        Population p;
        p.ids.resize(n);
        p.group.resize(n);
        p.xyz.resize(3 * (size_t)n);
        p.vel.resize(3 * (size_t)n);
        p.lambda.resize(n);
        p.state.resize(n);
        check(sph2_get_state(handle_, population, p.xyz.data(), p.vel.data(), p.lambda.data(),
                             p.state.data(), p.group.data(), p.ids.data()));
        return p;
    }

private:
    sph_solver2* handle_ = nullptr;
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

template <class T>
void put(FILE* f, const std::vector<T>& v) {
    const size_t bytes = sizeof(T) * v.size();
    if (bytes && std::fwrite(v.data(), 1, bytes, f) != bytes) throw std::runtime_error("short write");
}

void put_raw(FILE* f, const void* p, size_t bytes) {
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
        sph_grid block, box;
        check(sph_make_grid(origin, block_end, s, &block));
        check(sph_make_grid(origin, box_end, s, &box));
        const std::vector<float> low = particle_box(block);
        const std::vector<float> boundary = particle_box_canvas(box, 3);
        sph_config2 cfg;
        check(sph_make_configuration2(origin, box_end, 0.125f, (uint32_t)(low.size() / 3), 35,
                                      1000.0f, 30.0f, 5.0f, 88.1472f, 0.8f, 0.0125f, &cfg));
        cfg.refine_axis = 0;  // the slab 0.35 < x < 0.65 refines the block's far side
        cfg.refine_lo = 0.35f;
        cfg.refine_hi = 0.65f;
        Solver solver(low, {}, boundary, &cfg);
        solver.Bind();
        for (uint32_t k = 0; k < steps; ++k) solver.Advance(dt);
        uint32_t stats[6];
        solver.LastStats(stats);

        FILE* f = std::fopen(argv[1], "wb");
        if (!f) throw std::runtime_error(std::string("cannot open ") + argv[1]);
        const uint32_t head[3] = {(uint32_t)(low.size() / 3), (uint32_t)(boundary.size() / 3),
                                  steps};
        put_raw(f, head, sizeof(head));
        put_raw(f, &dt, sizeof(dt));
        put_raw(f, &cfg, sizeof(cfg));
        put(f, low);
        put(f, boundary);
        put_raw(f, stats, sizeof(stats));
        for (int32_t r : {SPH_LOW, SPH_HIGH}) {
            const Population p = solver.State(r);
            const uint32_t n = (uint32_t)p.ids.size();
            put_raw(f, &n, sizeof(n));
            put(f, p.ids);
            put(f, p.xyz);
            put(f, p.vel);
            put(f, p.lambda);
            put(f, p.state);
            put(f, p.group);
        }
        std::fclose(f);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "cabi_client2: %s\n", e.what());
        return 1;
    }
    return 0;
}
