// state_io.cu -- headless state save / resume and frame records of the
// single-scale handle (formats in state_format.h).
//
// Single-scale state body:
//   sph_config (64 B) | u32 n | u32 nb | u32 integrator | u32 reserved (0) |
//   float4 pos[n]   positions in the sorted order of the last step, persistent id in w
//   float4 vel[n]   velocities, same order
//   float4 pos0[n]  positions at creation, creation order (rollout restarts)
//   float4 bpos[nb] boundary positions, presorted on the fluid grid, depth outside the
//                   grid's box in w (the order boundary_reach's cut relies on)
// The next step's sort is stable with respect to the stored order, which is
// why the order itself is part of the state.  Re-presorting the stored
// (already sorted) boundary reproduces it exactly.
#include <cstdio>
#include <string>
#include <vector>
#include "errors.h"
#include "host_params.h"
#include "single_scale_solver.h"
#include "state_format.h"

using namespace sph;
using namespace sph_io;

namespace {

uint64_t ss_state_bytes(uint64_t n, uint64_t nb) {
    return sizeof(StatePrefix) + sizeof(sph_config) + 16 + 16 * (3 * n + nb) + 8;
}

// Every w of pos must be a distinct id below n.
bool ids_are_permutation(const std::vector<float4>& pos) {
    std::vector<unsigned char> seen(pos.size(), 0);
    for (const float4& p : pos) {
        uint32_t id;
        std::memcpy(&id, &p.w, 4);
        if (id >= pos.size() || seen[id]) return false;
        seen[id] = 1;
    }
    return true;
}

int write_all(FILE* f, const void* p, size_t n) {
    return (n == 0 || std::fwrite(p, 1, n, f) == n) ? SPH_OK : fail(SPH_E_IO, "frame write failed");
}

}  // namespace

extern "C" {

int sph_step_count(sph_solver* s, uint64_t* steps) {
    if (!s || !steps) return fail(SPH_E_INVALID, "sph_step_count: NULL argument");
    *steps = s->step;
    return SPH_OK;
}

int sph_save_state(sph_solver* s, void* dst, uint64_t capacity, uint64_t* bytes) {
    if (!s || !bytes) return fail(SPH_E_INVALID, "sph_save_state: NULL handle or size output");
    const uint64_t need = ss_state_bytes(s->n, s->nb);
    *bytes = need;
    if (!dst) return SPH_OK;
    if (capacity < need) return fail(SPH_E_CAPACITY, "sph_save_state: buffer smaller than the state");
    int rc = sph_sync(s);
    if (rc != SPH_OK) return rc;
    Writer w{static_cast<unsigned char*>(dst)};
    StatePrefix pre;
    std::memcpy(pre.magic, kStateMagic, 8);
    pre.version = kStateVersion;
    pre.kind = kKindSingleScale;
    pre.step = s->step;
    w.put(&pre, sizeof(pre));
    w.put(&s->cfg, sizeof(sph_config));
    const uint32_t counts[4] = {s->n, s->nb, (uint32_t)s->integrator, 0u};
    w.put(counts, sizeof(counts));
    const float4* src[3] = {s->pos, s->vel, s->pos0};
    for (const float4* a : src)
        if (s->n) SPH_CUDA(cudaMemcpy(w.take(16 * (size_t)s->n), a, 16 * (size_t)s->n, cudaMemcpyDeviceToHost));
    if (s->nb) SPH_CUDA(cudaMemcpy(w.take(16 * (size_t)s->nb), s->bpos, 16 * (size_t)s->nb, cudaMemcpyDeviceToHost));
    const uint64_t sum = checksum(dst, w.off);
    w.put(&sum, 8);
    return SPH_OK;
}

int sph_create_from_state(const void* src, uint64_t bytes, sph_solver** out) {
    if (!src || !out) return fail(SPH_E_INVALID, "sph_create_from_state: NULL argument");
    *out = nullptr;
    StatePrefix pre;
    if (!check_state(src, (size_t)bytes, kKindSingleScale, &pre))
        return fail(SPH_E_INVALID, "sph_create_from_state: not a single-scale state, or corrupt");
    Reader r{static_cast<const unsigned char*>(src), (size_t)bytes - 8, sizeof(StatePrefix)};
    sph_config cfg;
    uint32_t c[4];
    if (!r.get(&cfg, sizeof(cfg)) || !r.get(c, sizeof(c)))
        return fail(SPH_E_INVALID, "sph_create_from_state: truncated header");
    const uint32_t n = c[0], nb = c[1];
    const int32_t integrator = (int32_t)c[2];
    if (integrator != SPH_INTEGRATOR_SYMPLECTIC_EULER && integrator != SPH_INTEGRATOR_XSPH)
        return fail(SPH_E_INVALID, "sph_create_from_state: unknown integrator");
    if (n > kMaxParticles || nb > kMaxParticles)
        return fail(SPH_E_CAPACITY, "sph_create_from_state: more than 2^30 particles");
    if (bytes != ss_state_bytes(n, nb))
        return fail(SPH_E_INVALID, "sph_create_from_state: size does not match the particle counts");
    std::vector<float4> pos(n), vel(n), pos0(n), bpos(nb);
    r.get(pos.data(), 16 * (size_t)n);
    r.get(vel.data(), 16 * (size_t)n);
    r.get(pos0.data(), 16 * (size_t)n);
    r.get(bpos.data(), 16 * (size_t)nb);
    if (!ids_are_permutation(pos))
        return fail(SPH_E_INVALID, "sph_create_from_state: persistent ids are not a permutation");
    sph_ss::HostInit init;
    init.pos = pos.data();
    init.vel = vel.data();
    init.pos0 = pos0.data();
    init.bound = bpos.data();
    int rc = sph_ss::create_solver(&cfg, init, n, nb, pre.step, out);
    if (rc == SPH_OK && integrator != SPH_INTEGRATOR_SYMPLECTIC_EULER) {
        rc = sph_ss::set_integrator(*out, integrator);
        if (rc != SPH_OK) {
            sph_destroy(*out);
            *out = nullptr;
        }
    }
    return rc;
}

int sph_write_frame(sph_solver* s, const char* path, uint32_t fields, int32_t append) {
    if (!s || !path) return fail(SPH_E_INVALID, "sph_write_frame: NULL argument");
    const uint32_t known = SPH_FIELD_POSITIONS | SPH_FIELD_VELOCITIES | SPH_FIELD_DENSITIES;
    if (fields == 0 || (fields & ~known))
        return fail(SPH_E_INVALID, "sph_write_frame: fields must be a non-empty mask of "
                                   "positions, velocities, densities");
    std::vector<float> pos, vel, rho;
    int rc = SPH_OK;
    if (fields & SPH_FIELD_POSITIONS) {
        pos.resize(3 * (size_t)s->n);
        rc = sph_get_positions(s, pos.data(), SPH_ORDER_BY_ID);
    }
    if (rc == SPH_OK && (fields & SPH_FIELD_VELOCITIES)) {
        vel.resize(3 * (size_t)s->n);
        rc = sph_get_velocities(s, vel.data(), SPH_ORDER_BY_ID);
    }
    if (rc == SPH_OK && (fields & SPH_FIELD_DENSITIES)) {
        rho.resize(s->n);
        rc = sph_get_densities(s, rho.data(), SPH_ORDER_BY_ID);
    }
    if (rc != SPH_OK) return rc;
    FILE* f = std::fopen(path, append ? "ab" : "wb");
    if (!f) return fail(SPH_E_IO, std::string("sph_write_frame: cannot open ") + path);
    FramePrefix pre;
    std::memcpy(pre.magic, kFrameMagic, 8);
    pre.kind = kKindSingleScale;
    pre.fields = fields;
    pre.step = s->step;
    const uint32_t counts[2] = {s->n, 0u};
    rc = write_all(f, &pre, sizeof(pre));
    if (rc == SPH_OK) rc = write_all(f, counts, sizeof(counts));
    if (rc == SPH_OK) rc = write_all(f, pos.data(), 4 * pos.size());
    if (rc == SPH_OK) rc = write_all(f, vel.data(), 4 * vel.size());
    if (rc == SPH_OK) rc = write_all(f, rho.data(), 4 * rho.size());
    if (std::fclose(f) != 0 && rc == SPH_OK) rc = fail(SPH_E_IO, "sph_write_frame: close failed");
    return rc;
}

}  // extern "C"
