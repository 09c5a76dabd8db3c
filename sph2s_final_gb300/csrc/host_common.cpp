// host_common.cpp -- configuration, grid and scene builders of the C ABI,
// plus the thread-local error state.  Pure host C++ (no kernels).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include "errors.h"

namespace sph {

thread_local std::string g_last_error;
const double kPi = 3.14159265358979323846;  // M_PI, SPH2S_FINAL_SINGLE_SCALE/Solver.h:11

void set_last_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int check_cuda(cudaError_t e, const char* what, const char* file, int line) {
    if (e == cudaSuccess) return SPH_OK;
    char buf[512];
    std::snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s at %s:%d", (int)e,
                  cudaGetErrorString(e), what, file, line);
    g_last_error = buf;
    cudaGetLastError();  // clear the sticky-free error so later calls can proceed
    return SPH_E_CUDA;
}

int check_device_pointer(const void* p, const char* who) {
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(SPH_E_INVALID, std::string(who) + ": not a CUDA pointer");
    }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
        return fail(SPH_E_INVALID, std::string(who) + ": destination is not device memory");
    int dev = -1;
    int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice", __FILE__, __LINE__);
    if (rc != SPH_OK) return rc;
    if (a.type == cudaMemoryTypeDevice && a.device != dev)
        return fail(SPH_E_INVALID, std::string(who) + ": destination is on another device");
    return SPH_OK;
}

}  // namespace sph

using sph::fail;

extern "C" {

const char* sph_last_error(void) { return sph::g_last_error.c_str(); }

// Grid::MakeGrid(origin, end, spacing), SPH2S_FINAL_SINGLE_SCALE/Grid.h:16-35.
int sph_make_grid(const float origin[3], const float end[3], float spacing, sph_grid* out) {
    if (!origin || !end || !out) return fail(SPH_E_INVALID, "sph_make_grid: NULL argument");
    if (!(spacing > 0.0f) || !std::isfinite(spacing))
        return fail(SPH_E_INVALID, "sph_make_grid: spacing must be positive and finite");
    for (int a = 0; a < 3; ++a) {
        float d = std::ceil((end[a] - origin[a]) / spacing);
        if (!(d >= 1.0f) || d > 1024.0f)
            return fail(SPH_E_INVALID, "sph_make_grid: every axis needs 1..1024 cells");
        out->origin[a] = origin[a];
        out->dims[a] = (int32_t)d;
    }
    out->spacing = spacing;
    return SPH_OK;
}

// Grid::ComputeNumGridCells, SPH2S_FINAL_SINGLE_SCALE/Grid.h:11-14.
uint32_t sph_grid_num_cells(const sph_grid* g) {
    if (!g) return 0;
    return (uint32_t)g->dims[0] * (uint32_t)g->dims[1] * (uint32_t)g->dims[2];
}

// SolverConfiguration::MakeConfiguration, SPH2S_FINAL_SINGLE_SCALE/Solver.h:15-48:
// h = (0.75 V n / (pi N))^(1/3), m = rho0 V / N, m_b = m, grid spacing h.
int sph_make_configuration(const float origin[3], const float end[3], float volume,
                           uint32_t num_particles, uint32_t avg_particles, float rest_density,
                           float bulk_modulus, float viscosity, float speed_sound,
                           float tension_coefficient, float epsilon, sph_config* out) {
    if (!origin || !end || !out)
        return fail(SPH_E_INVALID, "sph_make_configuration: NULL argument");
    if (num_particles == 0 || !(volume > 0.0f))
        return fail(SPH_E_INVALID, "sph_make_configuration: need particles and a positive volume");
    float num = 0.75f * volume * static_cast<float>(avg_particles);
    double q = (double)num / (sph::kPi * (double)static_cast<float>(num_particles));
    float h = std::pow((float)q, 1.0f / 3.0f);
    sph_config c;
    std::memset(&c, 0, sizeof(c));
    c.effective_radius = h;
    c.fluid_particle_mass = rest_density * volume / static_cast<float>(num_particles);
    c.boundary_particle_mass = c.fluid_particle_mass;
    c.rest_density = rest_density;
    c.bulk_modulus = bulk_modulus;
    c.viscosity = viscosity;
    c.speed_sound = speed_sound;
    c.tension_coefficient = tension_coefficient;
    c.xsph_coeff = epsilon;
    int rc = sph_make_grid(origin, end, h, &c.grid);
    if (rc != SPH_OK) return rc;
    *out = c;
    return SPH_OK;
}

// ParticleData::CreateParticleBox, SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:129-163.
int sph_particle_box(const sph_grid* g, float* xyz, uint32_t capacity, uint32_t* n_out) {
    if (!g || !n_out) return fail(SPH_E_INVALID, "sph_particle_box: NULL argument");
    uint64_t n = (uint64_t)g->dims[0] * g->dims[1] * g->dims[2];
    *n_out = (uint32_t)n;
    if (!xyz) return SPH_OK;
    if (n > capacity) return fail(SPH_E_CAPACITY, "sph_particle_box: output too small");
    uint64_t c = 0;
    for (int k = 0; k < g->dims[2]; ++k)
        for (int j = 0; j < g->dims[1]; ++j)
            for (int i = 0; i < g->dims[0]; ++i) {
                xyz[c + 0] = g->origin[0] + (float)i * g->spacing;
                xyz[c + 1] = g->origin[1] + (float)j * g->spacing;
                xyz[c + 2] = g->origin[2] + (float)k * g->spacing;
                c += 3;
            }
    return SPH_OK;
}

// ParticleData::CreateParticleBoxCanvas, SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:165-209.
int sph_particle_box_canvas(const sph_grid* g, int32_t border, float* xyz, uint32_t capacity,
                            uint32_t* n_out) {
    if (!g || !n_out) return fail(SPH_E_INVALID, "sph_particle_box_canvas: NULL argument");
    if (border < 0) return fail(SPH_E_INVALID, "sph_particle_box_canvas: negative border");
    uint64_t outer = (uint64_t)(g->dims[0] + 2 * border) * (g->dims[1] + 2 * border) *
                     (g->dims[2] + 2 * border);
    uint64_t n = outer - (uint64_t)g->dims[0] * g->dims[1] * g->dims[2];
    *n_out = (uint32_t)n;
    if (!xyz) return SPH_OK;
    if (n > capacity) return fail(SPH_E_CAPACITY, "sph_particle_box_canvas: output too small");
    uint64_t c = 0;
    for (int k = -border; k < g->dims[2] + border; ++k)
        for (int j = -border; j < g->dims[1] + border; ++j)
            for (int i = -border; i < g->dims[0] + border; ++i) {
                bool inside = (i >= 0 && i < g->dims[0]) && (j >= 0 && j < g->dims[1]) &&
                              (k >= 0 && k < g->dims[2]);
                if (inside) continue;
                xyz[c + 0] = g->origin[0] + (float)i * g->spacing;
                xyz[c + 1] = g->origin[1] + (float)j * g->spacing;
                xyz[c + 2] = g->origin[2] + (float)k * g->spacing;
                c += 3;
            }
    return SPH_OK;
}

}  // extern "C"
