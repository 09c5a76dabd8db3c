// ref_harness_ts.cu -- runs the reference's own two-scale kernels on a GPU.
//
// TEST INFRASTRUCTURE ONLY.  Loads a cubin of the reference's
//   SPH2S_FINAL_TWO_SCALE/Solver.cu          (mode 0, "blended": lambda, states, split)
//   SPH2S_FINAL_TWO_SCALE_COUPLED/Solver.cu  (mode 1, "coupled": two fixed populations)
// compiled unmodified by oracle/ref_build.py, and replays the host side of the
// reference's Solver around those kernels with the driver API:
//   constructor (buffers, fills, boundary presort on Grid[LOW], states 0 / 4)
//                                           TS Solver.cu:1331-1544, CP Solver.cu:1017-1193
//   Advance                                 TS Solver.cu:1568-1614, CP Solver.cu:1216-1236
//     TS: neighbourhoods HIGH, LOW (count read back, 0xFF cell memsets, hash of the
//         active ids, thrust::sort_by_key, reorder), densities HIGH, LOW,
//         accelerations HIGH, LOW, count := 0 + integrate HIGH, count := 0 +
//         integrate LOW (survivors re-listed by atomicAdd, split children
//         inserted into HIGH)            TS Solver.cu:1618-1771
//     CP: the same phases LOW before HIGH, ids reset to 0..n-1 by the hash
//         kernel, plain integration    CP Solver.cu:1238-1339
// with the reference's launch shape (256 threads, ceil(MaxParticles/256)
// blocks for fluid kernels, (256+1)*4 bytes of shared memory for the cell-range
// kernels).  What the harness adds, none of which the kernels see:
//   * the initial velocities, blend coefficients and state bits of the input
//     are written over the constructor's fills (the reference's own states can
//     only come from its renderer; its split marking is commented out,
//     TS Solver.cu:1077-1082), so split, fade-out and fade-in run from step 1;
//   * a persistent id per storage slot, gathered through each sort's
//     permutation and copied to the slot integrate writes; split children
//     (inserted at atomicAdd slots, TS Solver.cu:564-585) get fresh ids in slot
//     order, which the reader matches to their parents geometrically;
//   * per step, readback of what the phases produced.
//
// usage: ref_harness_ts <cubin> <input.bin> <output.bin> [--time W]
//   --time W: W untimed steps, then the input's steps timed with CUDA events
//             around each whole Advance (the reference's CUDA::Timer, TS
//             Solver.cu:1574-1593); only the final state is written then and
//             the harness-only id tracking is skipped in the timed steps.
//   input : "SPHTSI01" | u32 mode | u32 config_bytes | config | u32 nL, nH, nB,
//           capL, capH, steps | f32 dt | per population (LOW, HIGH): f32 x[3n],
//           f32 v[3n], f32 lambda[n], i32 state[n] | f32 boundary[3nB]
//   output: "SPHTSO01" | u32 mode, steps_recorded | per recorded step, per
//           population (LOW, HIGH):
//             u32 n | sorted order of the step: u32 pid[n], u32 hash[n],
//             f32 rho[n], f32 p[n], f32 acc[3n], f32 colour[n] (0 in mode 1),
//             i32 state[n], f32 lambda[n] (the reorder's copies)
//           then per population: u32 count, u32 slots | u32 active[count] |
//             f32 x[3 slots], f32 v[3 slots], i32 state[slots], f32 lambda[slots],
//             u32 pid[slots]
//           then u32 high_survivors (before children), u32 slot_overlap
//           (children written over slots of HIGH survivors: a reference
//           hazard, TS Solver.cu:566 vs 1287; 0 in every fixture).
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/gather.h>
#include <thrust/sort.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

void die(const char* what, int code) {
    std::fprintf(stderr, "ref_harness_ts: %s failed (%d)\n", what, code);
    std::exit(2);
}

#define CU(x)                                     \
    do {                                          \
        CUresult _r = (x);                        \
        if (_r != CUDA_SUCCESS) die(#x, (int)_r); \
    } while (0)
#define RT(x)                                    \
    do {                                         \
        cudaError_t _r = (x);                    \
        if (_r != cudaSuccess) die(#x, (int)_r); \
    } while (0)

constexpr uint32_t kLow = 0, kHigh = 1;
constexpr uint32_t kChildPidBase = 0x40000000u;  // ids of children born in the harness run

struct Grid {  // Grid (TS Grid.h:55-58)
    float origin[3];
    int32_t dims[3];
    float spacing;
};
static_assert(sizeof(Grid) == 28, "Grid layout");

// SolverConfiguration: TS Solver.h:52-61 (100 bytes), CP Solver.h:50-58 (96 bytes,
// no BlendIncrement).  Both end with Grid[2]; the cell counts are read from there.
struct ConfigBytes {
    uint32_t size = 0;
    unsigned char raw[128];
    const Grid* grids() const { return reinterpret_cast<const Grid*>(raw + size - 2 * sizeof(Grid)); }
};

// Itanium names of the reference kernels (TS Solver.cu:594-1289, CP Solver.cu:515-968);
// `int resID` in the two-scale project, `unsigned char resID` in the coupled one.
const char* kBoundaryReorder = "_Z35reorderComputeCellStartEndBoundaryDPjS_PfPKfPKjS4_j";
const char* kTSHash = "_Z12computeHashsPjS_PKfji";
const char* kTSReorder = "_Z30reorderAndComputeCellStartEndDPjS_PfS0_PiS0_PKjPKfS5_PKiS5_S3_j";
const char* kTSDensity = "_Z26computeDensitiesPressuresDPfS_PKfS1_PKjS3_S1_S1_S3_S3_ji";
const char* kTSAccel = "_Z21computeAccelerationsDPfS_PKfS1_S1_S1_S1_PiPKjS4_S1_S1_S1_S1_S1_S4_S4_S1_S4_S4_ji";
const char* kTSIntegrate = "_Z10integrateDPfS_S_PiS_PjS1_S_S_S0_S_S1_S1_PKfS3_S3_PKiS3_fji";
const char* kCPHash = "_Z12computeHashsPjS_PKfjh";
const char* kCPReorder = "_Z30reorderAndComputeCellStartEndDPjS_PfS0_S_PKfS2_PKjj";
const char* kCPDensity = "_Z26computeDensitiesPressuresDPfS_PKfPKjS3_S1_S3_S3_jh";
const char* kCPAccel = "_Z21computeAccelerationsDPfPKfS1_S1_S1_PKjS3_S1_S1_S1_S1_S3_S3_S1_S3_S3_jh";
const char* kCPIntegrate = "_Z10integrateDPfS_S_PKfS1_fj";

CUfunction fn(CUmodule m, const char* name) {
    CUfunction f;
    CU(cuModuleGetFunction(&f, m, name));
    return f;
}

unsigned blocks_for(uint32_t n) { return n % 256 == 0 ? n / 256 : n / 256 + 1; }  // computeGridDimensions

void launch(CUfunction f, unsigned blocks, void** args, unsigned smem = 0) {
    if (blocks == 0) return;
    CU(cuLaunchKernel(f, blocks, 1, 1, 256, 1, 1, smem, 0, args, nullptr));
}

template <class T>
T* dalloc(size_t count) {
    T* p = nullptr;
    RT(cudaMalloc(&p, sizeof(T) * (count ? count : 1)));
    return p;
}

template <class T>
void fill(T* d, size_t count, T start, T inc) {  // CUDA::Fill (TS cuda.h:62-89)
    std::vector<T> h(count);
    for (size_t i = 0; i < count; ++i) h[i] = start + static_cast<T>(i) * inc;
    if (count) RT(cudaMemcpy(d, h.data(), sizeof(T) * count, cudaMemcpyHostToDevice));
}

template <class T>
void rd(FILE* f, T* dst, size_t count) {
    if (count && std::fread(dst, sizeof(T), count, f) != count) die("read input", 0);
}

template <class T>
void wr(FILE* f, const T* src, size_t count) {
    if (count) std::fwrite(src, sizeof(T), count, f);
}

template <class T>
std::vector<T> down(const T* d, size_t count) {
    std::vector<T> h(count);
    if (count) RT(cudaMemcpy(h.data(), d, sizeof(T) * count, cudaMemcpyDeviceToHost));
    return h;
}

// SPHParticleData (TS Solver.cu:1331-1386): buffers sized by MaxParticles.
struct Pop {
    uint32_t n = 0, cap = 0, cells = 0;
    float *pos, *vel, *dens, *pres, *acc, *tpos, *tvel, *blend, *tblend, *colour;
    int *states, *tstates;
    unsigned *ids, *hashs, *cs, *ce, *dnum;
    unsigned *pid, *pid_sorted;  // harness-side persistent ids (storage slot / sorted order)

    void create(uint32_t n_, uint32_t cap_, uint32_t cells_, int init_state) {
        n = n_;
        cap = cap_;
        cells = cells_;
        pos = dalloc<float>(3 * (size_t)cap);
        vel = dalloc<float>(3 * (size_t)cap);
        dens = dalloc<float>(cap);
        pres = dalloc<float>(cap);
        acc = dalloc<float>(3 * (size_t)cap);
        tpos = dalloc<float>(3 * (size_t)cap);
        tvel = dalloc<float>(3 * (size_t)cap);
        blend = dalloc<float>(cap);
        tblend = dalloc<float>(cap);
        colour = dalloc<float>(cap);
        states = dalloc<int>(cap);
        tstates = dalloc<int>(cap);
        ids = dalloc<unsigned>(cap);
        hashs = dalloc<unsigned>(cap);
        cs = dalloc<unsigned>(cells);
        ce = dalloc<unsigned>(cells);
        dnum = dalloc<unsigned>(1);
        pid = dalloc<unsigned>(cap);
        pid_sorted = dalloc<unsigned>(cap);
        fill<float>(pos, 3 * (size_t)cap, 0.f, 0.f);
        fill<float>(dens, cap, 0.f, 0.f);
        fill<float>(pres, cap, 0.f, 0.f);
        fill<float>(acc, 3 * (size_t)cap, 0.f, 0.f);
        fill<float>(vel, 3 * (size_t)cap, 0.f, 0.f);
        fill<float>(tpos, 3 * (size_t)cap, 0.f, 0.f);
        fill<float>(tvel, 3 * (size_t)cap, 0.f, 0.f);
        fill<float>(colour, cap, 0.f, 0.f);
        fill<unsigned>(ids, cap, 0u, 1u);
        fill<unsigned>(hashs, cap, 0u, 0u);
        fill<unsigned>(cs, cells, 0u, 0u);
        fill<unsigned>(ce, cells, 0u, 0u);
        fill<int>(tstates, cap, 0, 0);
        fill<float>(blend, cap, 1.f, 0.f);
        fill<float>(tblend, cap, 1.f, 0.f);
        fill<int>(states, cap, init_state, 0);  // Solver.cu:1530-1543
        fill<unsigned>(pid, cap, 0u, 1u);
        RT(cudaMemcpy(dnum, &n, 4, cudaMemcpyHostToDevice));
    }
};

struct Kernels {
    CUfunction hash, reorder, density, accel, integrate, breorder;
};

struct Run {
    uint32_t mode;
    Pop p[2];
    float* bpos;
    unsigned *bcs, *bce;
    uint32_t nb;
    Kernels k;
    bool track = true;  // harness-only id tracking
    uint32_t next_child = kChildPidBase;
    uint32_t high_survivors = 0, overlap = 0;
    const unsigned smem = sizeof(int) * (256 + 1);

    void neighbourhood(uint32_t r) {
        Pop& P = p[r];
        int res_i = (int)r;
        unsigned char res_c = (unsigned char)r;
        if (mode == 0) {  // TS Solver.cu:1618-1682
            RT(cudaMemset(P.cs, 0xFF, 4 * (size_t)P.cells));
            RT(cudaMemset(P.ce, 0xFF, 4 * (size_t)P.cells));
            RT(cudaMemcpy(&P.n, P.dnum, 4, cudaMemcpyDeviceToHost));
            if (!P.n) return;
            void* h[] = {&P.hashs, &P.ids, &P.pos, &P.n, &res_i};
            launch(k.hash, blocks_for(P.cap), h);
        } else {  // CP Solver.cu:1238-1282
            void* h[] = {&P.hashs, &P.ids, &P.pos, &P.n, &res_c};
            launch(k.hash, blocks_for(P.cap), h);
        }
        if (P.n)
            thrust::sort_by_key(thrust::device_ptr<unsigned>(P.hashs),
                                thrust::device_ptr<unsigned>(P.hashs + P.n),
                                thrust::device_ptr<unsigned>(P.ids));
        if (track && P.n)
            thrust::gather(thrust::device_ptr<unsigned>(P.ids), thrust::device_ptr<unsigned>(P.ids + P.n),
                           thrust::device_ptr<unsigned>(P.pid), thrust::device_ptr<unsigned>(P.pid_sorted));
        if (mode == 0) {
            void* a[] = {&P.cs, &P.ce, &P.tpos, &P.tvel, &P.tstates, &P.tblend, &P.ids,
                         &P.pos, &P.vel, &P.states, &P.blend, &P.hashs, &P.n};
            launch(k.reorder, blocks_for(P.cap), a, smem);
        } else {
            RT(cudaMemset(P.cs, 0xFF, 4 * (size_t)P.cells));
            RT(cudaMemset(P.ce, 0xFF, 4 * (size_t)P.cells));
            void* a[] = {&P.cs, &P.ce, &P.tpos, &P.tvel, &P.ids, &P.pos, &P.vel, &P.hashs, &P.n};
            launch(k.reorder, blocks_for(P.cap), a, smem);
        }
    }

    void density(uint32_t r) {
        Pop& P = p[r];
        Pop& Q = p[1 - r];
        if (mode == 0) {  // TS Solver.cu:1685-1707
            if (!P.n) return;
            int res = (int)r;
            void* a[] = {&P.dens, &P.pres, &P.tpos, &P.tblend, &P.cs, &P.ce,
                         &Q.tpos, &Q.tblend, &Q.cs, &Q.ce, &P.n, &res};
            launch(k.density, blocks_for(P.cap), a);
        } else {  // CP Solver.cu:1284-1299
            unsigned char res = (unsigned char)r;
            void* a[] = {&P.dens, &P.pres, &P.tpos, &P.cs, &P.ce, &Q.tpos, &Q.cs, &Q.ce, &P.n, &res};
            launch(k.density, blocks_for(P.cap), a);
        }
    }

    void accel(uint32_t r) {
        Pop& P = p[r];
        Pop& Q = p[1 - r];
        if (mode == 0) {  // TS Solver.cu:1709-1742
            if (!P.n) return;
            int res = (int)r;
            void* a[] = {&P.acc, &P.colour, &P.dens, &P.pres, &P.tpos, &P.tvel, &P.tblend,
                         &P.tstates, &P.cs, &P.ce, &Q.dens, &Q.pres, &Q.tpos, &Q.tvel,
                         &Q.tblend, &Q.cs, &Q.ce, &bpos, &bcs, &bce, &P.n, &res};
            launch(k.accel, blocks_for(P.cap), a);
        } else {  // CP Solver.cu:1301-1324
            unsigned char res = (unsigned char)r;
            void* a[] = {&P.acc, &P.dens, &P.pres, &P.tpos, &P.tvel, &P.cs, &P.ce, &Q.dens,
                         &Q.pres, &Q.tpos, &Q.tvel, &Q.cs, &Q.ce, &bpos, &bcs, &bce, &P.n, &res};
            launch(k.accel, blocks_for(P.cap), a);
        }
    }

    void integrate(uint32_t r, float dt) {
        Pop& P = p[r];
        Pop& Q = p[1 - r];
        const uint32_t n_before = P.n;
        if (mode == 0) {  // TS Solver.cu:1600-1603, 1744-1771
            RT(cudaMemset(P.dnum, 0, 4));
            if (P.n) {
                int res = (int)r;
                void* a[] = {&P.pos, &P.vel, &P.acc, &P.states, &P.blend, &P.ids, &P.dnum,
                             &Q.pos, &Q.vel, &Q.states, &Q.blend, &Q.ids, &Q.dnum,
                             &P.tpos, &P.tvel, &P.dens, &P.tstates, &P.tblend, &dt, &P.n, &res};
                launch(k.integrate, blocks_for(P.cap), a);
            }
        } else {  // CP Solver.cu:1326-1339
            void* a[] = {&P.pos, &P.vel, &P.acc, &P.tpos, &P.tvel, &dt, &P.n};
            launch(k.integrate, blocks_for(P.cap), a);
        }
        if (!track) return;
        // the particle at sorted index i now lives in storage slot i
        if (n_before)
            RT(cudaMemcpy(P.pid, P.pid_sorted, 4 * (size_t)n_before, cudaMemcpyDeviceToDevice));
        if (mode == 0 && r == kHigh) {
            RT(cudaMemcpy(&high_survivors, P.dnum, 4, cudaMemcpyDeviceToHost));
            overlap = 0;
        }
        if (mode == 0 && r == kLow) {  // children were appended to HIGH from high_survivors on
            uint32_t nh = 0;
            RT(cudaMemcpy(&nh, Q.dnum, 4, cudaMemcpyDeviceToHost));
            if (nh > high_survivors) {
                if (high_survivors < Q.n) overlap = 1;
                std::vector<unsigned> ids(nh - high_survivors);
                for (auto& v : ids) v = next_child++;
                RT(cudaMemcpy(Q.pid + high_survivors, ids.data(), 4 * ids.size(), cudaMemcpyHostToDevice));
            }
        }
    }

    void step(float dt, FILE* rec) {
        const uint32_t order[2] = {mode == 0 ? kHigh : kLow, mode == 0 ? kLow : kHigh};
        for (uint32_t r : order) neighbourhood(r);
        for (uint32_t r : order) density(r);
        for (uint32_t r : order) accel(r);
        if (rec) {
            RT(cudaDeviceSynchronize());
            for (uint32_t r = 0; r < 2; ++r) {
                const Pop& P = p[r];
                const size_t n = P.n;
                wr(rec, &P.n, 1);
                wr(rec, down(P.pid_sorted, n).data(), n);
                wr(rec, down(P.hashs, n).data(), n);
                wr(rec, down(P.dens, n).data(), n);
                wr(rec, down(P.pres, n).data(), n);
                wr(rec, down(P.acc, 3 * n).data(), 3 * n);
                wr(rec, down(P.colour, n).data(), n);
                if (mode == 0) {
                    wr(rec, down(P.tstates, n).data(), n);
                    wr(rec, down(P.tblend, n).data(), n);
                } else {
                    std::vector<int> z(n, r == kHigh ? 4 : 0);
                    std::vector<float> one(n, 1.0f);
                    wr(rec, z.data(), n);
                    wr(rec, one.data(), n);
                }
            }
        }
        for (uint32_t r : order) integrate(r, dt);
        if (rec) write_state(rec);
    }

    void write_state(FILE* rec) {
        RT(cudaDeviceSynchronize());
        for (uint32_t r = 0; r < 2; ++r) {
            Pop& P = p[r];
            uint32_t count = P.n;
            std::vector<unsigned> active;
            if (mode == 0) {
                RT(cudaMemcpy(&count, P.dnum, 4, cudaMemcpyDeviceToHost));
                active = down(P.ids, count);
            } else {
                active.resize(count);
                for (uint32_t i = 0; i < count; ++i) active[i] = i;
            }
            uint32_t slots = 0;
            for (unsigned a : active) slots = std::max(slots, a + 1);
            wr(rec, &count, 1);
            wr(rec, &slots, 1);
            wr(rec, active.data(), count);
            wr(rec, down(P.pos, 3 * (size_t)slots).data(), 3 * (size_t)slots);
            wr(rec, down(P.vel, 3 * (size_t)slots).data(), 3 * (size_t)slots);
            if (mode == 0) {
                wr(rec, down(P.states, slots).data(), slots);
                wr(rec, down(P.blend, slots).data(), slots);
            } else {
                std::vector<int> z(slots, r == kHigh ? 4 : 0);
                std::vector<float> one(slots, 1.0f);
                wr(rec, z.data(), slots);
                wr(rec, one.data(), slots);
            }
            wr(rec, down(P.pid, slots).data(), slots);
        }
        wr(rec, &high_survivors, 1);
        wr(rec, &overlap, 1);
    }
};

}  // namespace

int main(int argc, char** argv) {
    if (argc != 4 && !(argc == 6 && std::strcmp(argv[4], "--time") == 0)) {
        std::fprintf(stderr, "usage: ref_harness_ts <cubin> <input.bin> <output.bin> [--time W]\n");
        return 1;
    }
    const int warm = argc == 6 ? std::atoi(argv[5]) : -1;
    if (argc == 6 && warm < 1) {
        std::fprintf(stderr, "ref_harness_ts: --time needs at least one warm-up step\n");
        return 1;
    }
    FILE* in = std::fopen(argv[2], "rb");
    if (!in) die("open input", 0);
    char magic[8];
    rd(in, magic, 8);
    if (std::memcmp(magic, "SPHTSI01", 8) != 0) die("input magic", 0);
    Run run;
    rd(in, &run.mode, 1);
    ConfigBytes cfg;
    rd(in, &cfg.size, 1);
    const uint32_t want = run.mode == 0 ? 100u : 96u;
    if (run.mode > 1 || cfg.size != want) die("config size for the mode", (int)cfg.size);
    rd(in, cfg.raw, cfg.size);
    uint32_t hdr[6];
    rd(in, hdr, 6);
    float dt;
    rd(in, &dt, 1);
    const uint32_t nL = hdr[0], nH = hdr[1], nB = hdr[2], capL = hdr[3], capH = hdr[4], steps = hdr[5];
    if (capL < nL || capH < nH || capL == 0 || capH == 0) die("capacities", 0);
    std::vector<float> hx[2], hv[2], hl[2];
    std::vector<int> hs[2];
    const uint32_t ns[2] = {nL, nH};
    for (int r = 0; r < 2; ++r) {
        hx[r].resize(3 * (size_t)ns[r]);
        hv[r].resize(3 * (size_t)ns[r]);
        hl[r].resize(ns[r]);
        hs[r].resize(ns[r]);
        rd(in, hx[r].data(), hx[r].size());
        rd(in, hv[r].data(), hv[r].size());
        rd(in, hl[r].data(), hl[r].size());
        rd(in, hs[r].data(), hs[r].size());
    }
    std::vector<float> hb(3 * (size_t)nB);
    rd(in, hb.data(), hb.size());
    std::fclose(in);

    RT(cudaFree(nullptr));  // primary context shared by the runtime (thrust) and the driver API
    CUmodule mod;
    CU(cuModuleLoad(&mod, argv[1]));
    CUdeviceptr gconf;
    size_t gsize = 0;
    CU(cuModuleGetGlobal(&gconf, &gsize, mod, "gConfiguration"));
    if (gsize != cfg.size) die("gConfiguration size", (int)gsize);
    CU(cuMemcpyHtoD(gconf, cfg.raw, cfg.size));  // Solver::Bind
    if (run.mode == 0)
        run.k = {fn(mod, kTSHash), fn(mod, kTSReorder), fn(mod, kTSDensity), fn(mod, kTSAccel),
                 fn(mod, kTSIntegrate), fn(mod, kBoundaryReorder)};
    else
        run.k = {fn(mod, kCPHash), fn(mod, kCPReorder), fn(mod, kCPDensity), fn(mod, kCPAccel),
                 fn(mod, kCPIntegrate), fn(mod, kBoundaryReorder)};

    const Grid* g = cfg.grids();
    uint32_t cells[2];
    for (int r = 0; r < 2; ++r) cells[r] = (uint32_t)g[r].dims[0] * g[r].dims[1] * g[r].dims[2];
    run.p[kLow].create(nL, capL, cells[0], 0);
    run.p[kHigh].create(nH, capH, cells[1], run.mode == 0 ? 4 : 0);
    for (int r = 0; r < 2; ++r) {  // the harness's initial state over the constructor's fills
        Pop& P = run.p[r];
        const size_t n = ns[r];
        if (!n) continue;
        RT(cudaMemcpy(P.pos, hx[r].data(), 12 * n, cudaMemcpyHostToDevice));
        RT(cudaMemcpy(P.vel, hv[r].data(), 12 * n, cudaMemcpyHostToDevice));
        RT(cudaMemcpy(P.blend, hl[r].data(), 4 * n, cudaMemcpyHostToDevice));
        RT(cudaMemcpy(P.states, hs[r].data(), 4 * n, cudaMemcpyHostToDevice));
    }

    // BoundaryParticleData + constructor presort on Grid[LOW] (TS Solver.cu:1403-1529)
    run.nb = nB;
    run.bpos = dalloc<float>(3 * (size_t)nB);
    float* btmp = dalloc<float>(3 * (size_t)nB);
    unsigned* bids = dalloc<unsigned>(nB);
    unsigned* bhash = dalloc<unsigned>(nB);
    run.bcs = dalloc<unsigned>(cells[0]);
    run.bce = dalloc<unsigned>(cells[0]);
    fill<unsigned>(bids, nB, 0u, 1u);
    if (nB) RT(cudaMemcpy(run.bpos, hb.data(), 4 * hb.size(), cudaMemcpyHostToDevice));
    {
        int res_i = 0;
        unsigned char res_c = 0;
        void* h[] = {&bhash, &bids, &run.bpos, &run.nb, run.mode == 0 ? (void*)&res_i : (void*)&res_c};
        launch(run.k.hash, blocks_for(nB), h);
        if (nB)
            thrust::sort_by_key(thrust::device_ptr<unsigned>(bhash), thrust::device_ptr<unsigned>(bhash + nB),
                                thrust::device_ptr<unsigned>(bids));
        RT(cudaMemset(run.bcs, 0xFF, 4 * (size_t)cells[0]));
        RT(cudaMemset(run.bce, 0xFF, 4 * (size_t)cells[0]));
        void* a[] = {&run.bcs, &run.bce, &btmp, &run.bpos, &bids, &bhash, &run.nb};
        launch(run.k.breorder, blocks_for(nB), a, run.smem);
        if (nB) RT(cudaMemcpy(run.bpos, btmp, 12 * (size_t)nB, cudaMemcpyDeviceToDevice));
    }

    FILE* out = std::fopen(argv[3], "wb");
    if (!out) die("open output", 0);
    wr(out, "SPHTSO01", 8);
    wr(out, &run.mode, 1);
    const uint32_t recorded = warm >= 0 ? 0u : steps;
    wr(out, &recorded, 1);
    if (warm < 0) {
        for (uint32_t s = 0; s < steps; ++s) run.step(dt, out);
    } else {
        for (int s = 0; s < warm; ++s) run.step(dt, nullptr);
        run.track = false;
        cudaEvent_t ev0, ev1;
        RT(cudaEventCreate(&ev0));
        RT(cudaEventCreate(&ev1));
        RT(cudaDeviceSynchronize());
        RT(cudaEventRecord(ev0));
        for (uint32_t s = 0; s < steps; ++s) run.step(dt, nullptr);
        RT(cudaEventRecord(ev1));
        RT(cudaEventSynchronize(ev1));
        float ms = 0.0f;
        RT(cudaEventElapsedTime(&ms, ev0, ev1));
        uint32_t n_end[2];
        for (int r = 0; r < 2; ++r) {
            n_end[r] = run.p[r].n;
            if (run.mode == 0) RT(cudaMemcpy(&n_end[r], run.p[r].dnum, 4, cudaMemcpyDeviceToHost));
        }
        std::printf("ref_harness_ms_per_step %.6f\n", steps ? ms / (float)steps : 0.0f);
        std::printf("ref_harness_counts %u %u\n", n_end[0], n_end[1]);
    }
    std::fclose(out);
    std::printf("ref_harness_ts: mode %u, %u low, %u high, %u boundary, %u steps\n", run.mode, nL, nH,
                nB, steps);
    return 0;
}
