// ============================================================================
// sph_oracle_ts.cpp -- FP64 CPU restatement of the two-scale SPH2S step.
// TEST INFRASTRUCTURE ONLY (the product never loads this library).
//
// What it restates (file:line within segfault11/SPH2S_FINAL):
//   * configuration, two grids, LOW/HIGH         SPH2S_FINAL_TWO_SCALE/Solver.h:16-61
//   * state bits, COMPL, blend coefficient       SPH2S_FINAL_TWO_SCALE/Solver.cu:14-20, 1367-1372, 1529-1543
//   * density: same population weighted by
//     lambda_j, complementary population with
//     averaged kernels on the other grid         SPH2S_FINAL_TWO_SCALE/Solver.cu:215-290, 732-845
//   * accelerations: same + complementary +
//     boundary (LOW radius and LOW mass)          SPH2S_FINAL_TWO_SCALE/Solver.cu:292-539, 847-1048
//   * integrate: velocity clamp, blend update,
//     fade-out removal, fade-in completion,
//     split into 8 children                       SPH2S_FINAL_TWO_SCALE/Solver.cu:541-586, 1163-1289
//   * step order: neighbourhoods, densities,
//     accelerations, integrate HIGH then LOW      SPH2S_FINAL_TWO_SCALE/Solver.cu:1568-1614
//
// Defined here, not in the reference (the reference's split trigger is
// commented out, Solver.cu:1077-1082, and it has no merge):
//   * split: a LOW particle in state 0 whose position at the start of the step
//     lies strictly inside the refinement slab lo < x[axis] < hi (FP32 compare)
//     is marked 3 and split in that step's integration, as the reference's
//     commented-out marking in the force pass would do;
//   * group: the 8 children of one split form a group with a new group id;
//   * merge: a group whose 8 members are all in state 4 (fine, fully blended
//     in) at the start of the step and whose centroid then lies outside the
//     slab merges: its members fade out (state 5) and one LOW particle fades in
//     (state 2, lambda 0) at the members' mean position and velocity after
//     integration.  The centroid test uses a fixed-point sum
//     sum_k llrint(x_k * 2^40) against llrint(lo * 2^43), llrint(hi * 2^43),
//     which is exact and order independent, so GPU and oracle agree bit for bit;
//   * compaction replaces the reference's atomicAdd re-listing (whose order is
//     not deterministic, Solver.cu:1287-1288): next HIGH = HIGH survivors in
//     sorted order, then children in the sorted order of their parents; next
//     LOW = LOW survivors in sorted order, then merged particles by group id;
//   * the velocity clamp skips |v| = 0 (the reference divides 0 by 0 there).
// Blend coefficients and the state machine run in FP32 like the GPU (the
// increments are exact, so removal/completion counts match bit for bit).
//
// Also restated: the coupled fixed-population solver
// (SPH2S_FINAL_TWO_SCALE_COUPLED/Solver.cu:648-1015: unit weights, its
// complementary tension with the neighbour's own support, no clamp, no state
// changes) and the colour / energy output (SPH2S_FINAL_TWO_SCALE/Solver.cu:
// 206-213, 378-387, 897-907, 1050-1070).  Defined here, replacing the
// reference's render-pass surface flag (SSFRenderer.cu:196-218) and its
// commented-out split marking (Solver.cu:1077-1082): the surface trigger
// splits a normal LOW particle with rho < surface_density and merges a group
// whose 8 members are fully blended in and all have rho >= surface_density,
// both on the densities of the current step.
// ============================================================================
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_common.h"

namespace {

using namespace oracle;

constexpr uint32_t kNoGroup = 0xFFFFFFFFu;
constexpr int LOW = 0, HIGH = 1;

// Same layout as sph_config2 in include/sph2s.h.
struct OConfig2 {
    float effective_radius[2];
    float fluid_particle_mass[2];
    float boundary_particle_mass;
    float rest_density;
    float bulk_modulus;
    float viscosity;
    float speed_sound;
    float tension_coefficient;
    float blend_increment;
    OGrid grid[2];
    int32_t refine_axis;
    float refine_lo, refine_hi;
    int32_t mode;           // 0 blended, 1 coupled
    int32_t split_trigger;  // 0 slab, 1 surface
    float surface_density;
};

struct TPop {
    std::vector<double> x, v;  // 3 per particle
    std::vector<float> lam;
    std::vector<int32_t> state;
    std::vector<uint32_t> group, ids;
    size_t size() const { return lam.size(); }
    void resize(size_t n) {
        x.resize(3 * n);
        v.resize(3 * n);
        lam.resize(n);
        state.resize(n);
        group.resize(n);
        ids.resize(n);
    }
    void push(const double* xx, const double* vv, float l, int32_t s, uint32_t g, uint32_t id) {
        for (int a = 0; a < 3; ++a) {
            x.push_back(xx[a]);
            v.push_back(vv[a]);
        }
        lam.push_back(l);
        state.push_back(s);
        group.push_back(g);
        ids.push_back(id);
    }
};

struct TBoundary {
    std::vector<float> xf;
    std::vector<double> xd;
    SortedSet set;
};

struct StepStats {
    uint32_t splits, merges, removed[2], faded_in[2];
};

inline int64_t fixed40(float x) { return (int64_t)std::llrint((double)x * 1099511627776.0); }
inline int64_t fixed43(float x) { return (int64_t)std::llrint((double)x * 8796093022208.0); }

// Sorted copy of one population (Morton order on its own grid, stable).
struct SortedPop {
    TPop p;                 // sorted
    std::vector<float> xf;  // sorted float positions
    SortedSet set;
};

void sort_pop(const OGrid& g, const TPop& in, SortedPop& out) {
    const size_t n = in.size();
    std::vector<float> xf(3 * n);
    for (size_t i = 0; i < 3 * n; ++i) xf[i] = (float)in.x[i];
    sort_set(g, xf.data(), n, out.set);
    out.p.resize(n);
    out.xf.resize(3 * n);
    for (size_t k = 0; k < n; ++k) {
        const uint32_t q = out.set.perm[k];
        for (int a = 0; a < 3; ++a) {
            out.p.x[3 * k + a] = in.x[3 * q + a];
            out.p.v[3 * k + a] = in.v[3 * q + a];
            out.xf[3 * k + a] = xf[3 * q + a];
        }
        out.p.lam[k] = in.lam[q];
        out.p.state[k] = in.state[q];
        out.p.group[k] = in.group[q];
        out.p.ids[k] = in.ids[q];
    }
}

struct Fields {
    std::vector<double> rho, p, acc, colour, dist_cm;
    std::vector<uint32_t> nbr_same, nbr_compl, nbr_bnd;
};

inline double dist(const double* a, const double* b, double* d) {
    for (int k = 0; k < 3; ++k) d[k] = a[k] - b[k];
    return std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

// Densities of population r (SPH2S_FINAL_TWO_SCALE/Solver.cu:732-845).
void ts_density(const OConfig2& C, int r, const SortedPop* P, Fields& F) {
    const int c = 1 - r;
    const SortedPop& S = P[r];
    const SortedPop& O = P[c];
    const size_t n = S.p.size();
    const float hr = C.effective_radius[r], h0 = C.effective_radius[LOW];
    const float Tr = thresh_sq(hr), T0 = thresh_sq(h0);
    const Kern Kr(hr), K0(C.effective_radius[LOW]), K1(C.effective_radius[HIGH]);
    const double mr = C.fluid_particle_mass[r], mc = C.fluid_particle_mass[c];
    const bool coupled = C.mode == 1;
    F.rho.assign(n, 0.0);
    F.p.assign(n, 0.0);
    F.nbr_same.assign(n, 0);
    F.nbr_compl.assign(n, 0);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        const float* xi = &S.xf[3 * i];
        const double* xd = &S.p.x[3 * i];
        double s = 0.0, sc = 0.0, d[3];
        uint32_t ns = 0, nc = 0;
        for_stencil(C.grid[r], S.set.cells, xi, hr, [&](uint32_t j) {
            if (r2_f32(xi, &S.xf[3 * j]) < Tr) {
                s += (coupled ? 1.0 : S.p.lam[j]) * Kr.W(dist(xd, &S.p.x[3 * j], d));
                ++ns;
            }
        });
        for_stencil(C.grid[c], O.set.cells, xi, h0, [&](uint32_t j) {
            if (r2_f32(xi, &O.xf[3 * j]) < T0) {
                const double rr = dist(xd, &O.p.x[3 * j], d);
                const double w1 = rr < K1.h ? K1.W(rr) : 0.0;
                sc += (coupled ? 1.0 : O.p.lam[j]) * 0.5 * (K0.W(rr) + w1);
                ++nc;
            }
        });
        F.rho[i] = s * mr + sc * mc;
        F.p[i] = C.bulk_modulus * (F.rho[i] - C.rest_density);
        F.nbr_same[i] = ns;
        F.nbr_compl[i] = nc;
    }
}

// Accelerations of population r (SPH2S_FINAL_TWO_SCALE/Solver.cu:847-1048).
void ts_accel(const OConfig2& C, int r, const SortedPop* P, const Fields* F, const TBoundary& B,
              Fields& out) {
    const int c = 1 - r;
    const SortedPop& S = P[r];
    const SortedPop& O = P[c];
    const size_t n = S.p.size();
    const float hr = C.effective_radius[r], h0 = C.effective_radius[LOW];
    const float Tr = thresh_sq(hr), T0 = thresh_sq(h0);
    const Kern Kr(hr), K0(C.effective_radius[LOW]), K1(C.effective_radius[HIGH]);
    const double mr = C.fluid_particle_mass[r], mc = C.fluid_particle_mass[c];
    const double mb = C.boundary_particle_mass, m0 = C.fluid_particle_mass[LOW];
    const double mu = C.viscosity, sigma = C.tension_coefficient;
    const bool coupled = C.mode == 1;
    const double hmc = 0.8673250705840776;  // Mexican hat 2 / (sqrt(3) pi^(1/4))
    out.acc.assign(3 * n, 0.0);
    out.nbr_bnd.assign(n, 0);
    out.colour.assign(n, 0.0);
    out.dist_cm.assign(n, 0.0);
    const std::vector<double>& rho = F[r].rho;
    const std::vector<double>& pr = F[r].p;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        const float* xi = &S.xf[3 * i];
        const double* xd = &S.p.x[3 * i];
        const double* vi = &S.p.v[3 * i];
        const double ri = rho[i], pi = pr[i];
        double f[3] = {0, 0, 0}, b[3] = {0, 0, 0}, d[3];
        const double psi0 = -3.0 * hmc;
        double psum = psi0, cw[3] = {vi[0] * psi0, vi[1] * psi0, vi[2] * psi0};
        double cs[3] = {xd[0], xd[1], xd[2]}, ccnt = 1.0;
        for_stencil(C.grid[r], S.set.cells, xi, hr, [&](uint32_t j) {
            const float r2 = r2_f32(xi, &S.xf[3 * j]);
            if (r2 != 0.0f && r2 < Tr) {
                const double rr = dist(xd, &S.p.x[3 * j], d);
                const double q2 = rr * rr / ((double)hr * (double)hr);
                const double psi = hmc * (q2 - 3.0) * std::exp(-0.5 * q2);
                psum += psi;
                for (int a = 0; a < 3; ++a) {
                    cw[a] += S.p.v[3 * j + a] * psi;
                    cs[a] += S.p.x[3 * j + a];
                }
                ccnt += 1.0;
                const double lj = coupled ? 1.0 : S.p.lam[j];
                const double coeffP = -ri * mr * (pi / (ri * ri) + pr[j] / (rho[j] * rho[j]));
                const double gw = Kr.gradW_factor(rr);
                const double coeffV = mu * mr / rho[j] * Kr.lapl(rr);
                const double coeffT = -Kr.W(rr) * mr * sigma;
                for (int a = 0; a < 3; ++a)
                    f[a] += lj * (coeffP * gw * d[a] + coeffV * (S.p.v[3 * j + a] - vi[a]) +
                                  coeffT * d[a]);
            }
        });
        const std::vector<double>& rho_c = F[c].rho;
        const std::vector<double>& p_c = F[c].p;
        for_stencil(C.grid[c], O.set.cells, xi, h0, [&](uint32_t j) {
            const float r2 = r2_f32(xi, &O.xf[3 * j]);
            if (r2 != 0.0f && r2 < T0) {
                const double rr = dist(xd, &O.p.x[3 * j], d);
                const double lj = coupled ? 1.0 : O.p.lam[j];
                const double coeffP = -ri * mc * (pi / (ri * ri) + p_c[j] / (rho_c[j] * rho_c[j]));
                const double g1 = rr <= K1.h ? K1.gradW_factor(rr) : 0.0;
                const double gw = 0.5 * (K0.gradW_factor(rr) + g1);
                const double l1 = rr < K1.h ? K1.lapl(rr) : 0.0;
                const double coeffV = mu * mc / rho_c[j] * 0.5 * (K0.lapl(rr) + l1);
                const double w1 = rr < K1.h ? K1.W(rr) : 0.0;
                // coupled: Poly6 of the neighbour's own support (COUPLED/Solver.cu:448-460)
                const double wt = !coupled ? 0.5 * (K0.W(rr) + w1) : (c == LOW ? K0.W(rr) : w1);
                const double coeffT = -wt * mc * sigma;
                for (int a = 0; a < 3; ++a)
                    f[a] += lj * (coeffP * gw * d[a] + coeffV * (O.p.v[3 * j + a] - vi[a]) +
                                  coeffT * d[a]);
            }
        });
        uint32_t bc = 0;
        for_stencil(C.grid[LOW], B.set.cells, xi, h0, [&](uint32_t j) {
            if (r2_f32(xi, &B.xf[3 * j]) < T0) {
                const double rr = dist(xd, &B.xd[3 * j], d);
                const double w = boundary_weight(rr, (double)h0, C.speed_sound) * mb / (m0 + mb);
                for (int a = 0; a < 3; ++a) b[a] += w * d[a] / rr;
                ++bc;
            }
        });
        out.acc[3 * i + 0] = f[0] / ri + b[0];
        out.acc[3 * i + 1] = f[1] / ri - 9.81 + b[1];
        out.acc[3 * i + 2] = f[2] / ri + b[2];
        out.nbr_bnd[i] = bc;
        double e2 = 0.0, ene = 0.0;
        for (int a = 0; a < 3; ++a) {
            const double da = xd[a] - cs[a] / ccnt;
            e2 += da * da;
            ene += cw[a] * cw[a];
        }
        ene = std::min(ene / (psum * psum * (double)hr), 300.0);
        out.dist_cm[i] = std::sqrt(e2);
        out.colour[i] = out.dist_cm[i] < 0.0025 ? 0.3 : ene / 300.0;
    }
}

struct TSState {
    OConfig2 C;
    TBoundary B;
    TPop pop[2];
    uint32_t group_base = 0;
    uint32_t pid_base[2] = {0, 0};
    StepStats last = {};
};

void make_tboundary(const OGrid& g, const float* bxyz, size_t nb, TBoundary& B) {
    sort_set(g, bxyz, nb, B.set);
    B.xf.resize(3 * nb);
    B.xd.resize(3 * nb);
    for (size_t k = 0; k < nb; ++k)
        for (int a = 0; a < 3; ++a) {
            B.xf[3 * k + a] = bxyz[3 * B.set.perm[k] + a];
            B.xd[3 * k + a] = B.xf[3 * k + a];
        }
}

// One step; fills fields of the sorted populations if requested.
void ts_step(TSState& S, double dt, SortedPop* keep_sorted, Fields* keep_fields) {
    const OConfig2& C = S.C;
    SortedPop P[2];
    sort_pop(C.grid[LOW], S.pop[LOW], P[LOW]);
    sort_pop(C.grid[HIGH], S.pop[HIGH], P[HIGH]);

    Fields F[2], A[2];
    ts_density(C, HIGH, P, F[HIGH]);
    ts_density(C, LOW, P, F[LOW]);

    // groups: slab trigger on the start-of-step centroid (fixed point along the
    // axis), surface trigger on this step's member densities
    const bool coupled = C.mode == 1;
    const bool surface = !coupled && C.split_trigger == 1;
    const bool refine = !coupled && !surface && C.refine_axis >= 0 && C.refine_axis < 3;
    const float surf_rho = C.surface_density;
    const int ax = refine ? C.refine_axis : 0;
    std::vector<int64_t> gsum(S.group_base, 0);
    std::vector<uint32_t> gready(S.group_base, 0), gsurf(S.group_base, 0);
    for (size_t k = 0; k < P[HIGH].p.size(); ++k) {
        const uint32_t g = P[HIGH].p.group[k];
        if (g == kNoGroup || g >= S.group_base) continue;
        gsum[g] += fixed40(P[HIGH].xf[3 * k + ax]);
        gready[g] += P[HIGH].p.state[k] == 4 ? 1u : 0u;
        gsurf[g] += F[HIGH].rho[k] < (double)surf_rho ? 1u : 0u;
    }
    const int64_t L = fixed43(C.refine_lo), H = fixed43(C.refine_hi);
    std::vector<uint8_t> merge(S.group_base, 0);
    for (uint32_t g = 0; g < S.group_base; ++g)
        merge[g] = gready[g] == 8 &&
                   ((refine && !(L < gsum[g] && gsum[g] < H)) || (surface && gsurf[g] == 0));
    ts_accel(C, HIGH, P, F, S.B, A[HIGH]);
    ts_accel(C, LOW, P, F, S.B, A[LOW]);

    StepStats st = {};
    TPop next[2];
    std::vector<double> msum(6 * (size_t)S.group_base, 0.0);
    const float cblend[4] = {0.0f, -1.0f, 1.0f, 0.0f};
    struct Child {
        double x[3], v[3];
    };
    std::vector<Child> children;
    // SQRT3INV, SPH2S_FINAL_TWO_SCALE/Solver.cu:541-563
    const double s3 = 0.57735026919;
    const double dir[8][3] = {{s3, s3, s3},   {s3, s3, -s3},  {s3, -s3, s3},  {s3, -s3, -s3},
                              {-s3, s3, s3},  {-s3, s3, -s3}, {-s3, -s3, s3}, {-s3, -s3, -s3}};
    for (int r = HIGH; r >= LOW; --r) {  // integrate HIGH before LOW (Solver.cu:1592-1595)
        const SortedPop& Q = P[r];
        const double vmax = 0.8 * (double)C.effective_radius[r] / dt;
        for (size_t i = 0; i < Q.p.size(); ++i) {
            double v[3], x[3];
            for (int a = 0; a < 3; ++a) v[a] = Q.p.v[3 * i + a] + dt * A[r].acc[3 * i + a];
            const double nv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            if (!coupled && nv > vmax && nv > 0.0)
                for (int a = 0; a < 3; ++a) v[a] *= vmax / nv;
            for (int a = 0; a < 3; ++a) x[a] = Q.p.x[3 * i + a] + dt * v[a];
            int32_t state = Q.p.state[i];
            uint32_t group = Q.p.group[i];
            const float xa = Q.xf[3 * i + ax];
            if (r == LOW && refine && (state & 3) == 0 && C.refine_lo < xa && xa < C.refine_hi)
                state = (state & 4) | 3;
            if (r == LOW && surface && (state & 3) == 0 && F[LOW].rho[i] < (double)surf_rho)
                state = (state & 4) | 3;
            if (coupled) {  // fixed populations: no blend, no state changes
                next[r].push(x, v, Q.p.lam[i], state, group, Q.p.ids[i]);
                continue;
            }
            float lam = Q.p.lam[i] + cblend[state & 3] * C.blend_increment;
            if (lam <= 0.0f && (state & 3) == 1) {
                st.removed[r]++;
                continue;
            }
            if (lam >= 1.0f && (state & 3) == 2) {
                state &= 4;
                lam = 1.0f;
                st.faded_in[r]++;
            }
            if (r == LOW && (state & 3) == 3) {
                const double rs = 0.5 * std::cbrt(3.0 / (4.0 * kPi) * C.fluid_particle_mass[LOW] /
                                                  F[LOW].rho[i]);
                for (int k = 0; k < 8; ++k) {
                    Child ch;
                    for (int a = 0; a < 3; ++a) {
                        ch.x[a] = x[a] + rs * dir[k][a];
                        ch.v[a] = v[a];
                    }
                    children.push_back(ch);
                }
                st.splits++;
                state = 1;
            }
            if (r == HIGH && group != kNoGroup && group < S.group_base && merge[group]) {
                for (int a = 0; a < 3; ++a) {
                    msum[6 * group + a] += x[a];
                    msum[6 * group + 3 + a] += v[a];
                }
                state = 5;
                group = kNoGroup;
            }
            next[r].push(x, v, lam, state, group, Q.p.ids[i]);
        }
    }
    // children appended to HIGH, merged particles to LOW
    const uint32_t gb = S.group_base;
    for (size_t c = 0; c < children.size(); ++c) {
        const uint32_t q = (uint32_t)(c / 8);
        next[HIGH].push(children[c].x, children[c].v, 0.0f, 6, gb + q,
                        S.pid_base[HIGH] + (uint32_t)c);
    }
    S.pid_base[HIGH] += (uint32_t)children.size();
    for (uint32_t g = 0; g < gb; ++g) {
        if (!merge[g]) continue;
        double x[3], v[3];
        for (int a = 0; a < 3; ++a) {
            x[a] = msum[6 * g + a] / 8.0;
            v[a] = msum[6 * g + 3 + a] / 8.0;
        }
        next[LOW].push(x, v, 0.0f, 2, kNoGroup, S.pid_base[LOW]++);
        st.merges++;
    }
    S.group_base += st.splits;
    if (keep_sorted) {
        keep_sorted[LOW] = P[LOW];
        keep_sorted[HIGH] = P[HIGH];
    }
    if (keep_fields) {
        for (int r = 0; r < 2; ++r) {
            keep_fields[r] = F[r];
            keep_fields[r].acc = A[r].acc;
            keep_fields[r].nbr_bnd = A[r].nbr_bnd;
            keep_fields[r].colour = A[r].colour;
            keep_fields[r].dist_cm = A[r].dist_cm;
        }
    }
    S.pop[LOW] = std::move(next[LOW]);
    S.pop[HIGH] = std::move(next[HIGH]);
    S.last = st;
}

void load_pop(TPop& p, uint32_t n, const float* x, const float* v, const float* lam,
              const int32_t* state, const uint32_t* group, const uint32_t* ids, int default_state) {
    p.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) {
            p.x[3 * i + a] = x[3 * i + a];
            p.v[3 * i + a] = v ? v[3 * i + a] : 0.0;
        }
        p.lam[i] = lam ? lam[i] : 1.0f;
        p.state[i] = state ? state[i] : default_state;
        p.group[i] = group ? group[i] : kNoGroup;
        p.ids[i] = ids ? ids[i] : i;
    }
}

}  // namespace

extern "C" {

// Creates a two-scale rollout.  Per population (0 = LOW, 1 = HIGH): float
// positions/velocities (3 per particle), blend coefficients, states, group
// ids and persistent ids; any of v/lam/state/group/ids may be NULL (defaults:
// 0, 1, 0 for LOW and 4 for HIGH, no group, 0..n-1).
void* or_ts_create(const OConfig2* C, const float* bxyz, uint32_t nb, const uint32_t* n,
                   const float* const* x, const float* const* v, const float* const* lam,
                   const int32_t* const* state, const uint32_t* const* group,
                   const uint32_t* const* ids, uint32_t group_base, const uint32_t* pid_base) {
    TSState* S = new TSState();
    S->C = *C;
    make_tboundary(C->grid[LOW], bxyz, nb, S->B);
    for (int r = 0; r < 2; ++r)
        load_pop(S->pop[r], n[r], x[r], v ? v[r] : nullptr, lam ? lam[r] : nullptr,
                 state ? state[r] : nullptr, group ? group[r] : nullptr, ids ? ids[r] : nullptr,
                 r == HIGH ? 4 : 0);
    S->group_base = group_base;
    S->pid_base[LOW] = pid_base ? pid_base[LOW] : n[LOW];
    S->pid_base[HIGH] = pid_base ? pid_base[HIGH] : n[HIGH];
    return S;
}

void or_ts_advance(void* h, double dt, int steps) {
    TSState* S = (TSState*)h;
    for (int s = 0; s < steps; ++s) ts_step(*S, dt, nullptr, nullptr);
}

// Advances one step and returns, for the SORTED populations of that step
// (the order the GPU's per-step fields use), density, acceleration and
// neighbour counts (same population, complementary, boundary), plus the
// sorted persistent ids.  Arrays per population r sized by the pre-step count.
void or_ts_step_fields(void* h, double dt, double* const* rho, double* const* acc,
                       uint32_t* const* nbr_same, uint32_t* const* nbr_compl,
                       uint32_t* const* nbr_bnd, uint32_t* const* ids_sorted,
                       double* const* colour, double* const* dist_cm) {
    TSState* S = (TSState*)h;
    SortedPop P[2];
    Fields F[2];
    ts_step(*S, dt, P, F);
    for (int r = 0; r < 2; ++r) {
        const size_t n = P[r].p.size();
        if (rho && rho[r]) std::memcpy(rho[r], F[r].rho.data(), n * 8);
        if (acc && acc[r]) std::memcpy(acc[r], F[r].acc.data(), 3 * n * 8);
        if (nbr_same && nbr_same[r]) std::memcpy(nbr_same[r], F[r].nbr_same.data(), n * 4);
        if (nbr_compl && nbr_compl[r]) std::memcpy(nbr_compl[r], F[r].nbr_compl.data(), n * 4);
        if (nbr_bnd && nbr_bnd[r]) std::memcpy(nbr_bnd[r], F[r].nbr_bnd.data(), n * 4);
        if (ids_sorted && ids_sorted[r]) std::memcpy(ids_sorted[r], P[r].p.ids.data(), n * 4);
        if (colour && colour[r]) std::memcpy(colour[r], F[r].colour.data(), n * 8);
        if (dist_cm && dist_cm[r]) std::memcpy(dist_cm[r], F[r].dist_cm.data(), n * 8);
    }
}

void or_ts_counts(void* h, uint32_t* n_low, uint32_t* n_high, uint32_t* group_base) {
    TSState* S = (TSState*)h;
    if (n_low) *n_low = (uint32_t)S->pop[LOW].size();
    if (n_high) *n_high = (uint32_t)S->pop[HIGH].size();
    if (group_base) *group_base = S->group_base;
}

// stats[6] = splits, merges, removed LOW, removed HIGH, faded-in LOW, faded-in HIGH
void or_ts_last_stats(void* h, uint32_t* stats) {
    TSState* S = (TSState*)h;
    stats[0] = S->last.splits;
    stats[1] = S->last.merges;
    stats[2] = S->last.removed[LOW];
    stats[3] = S->last.removed[HIGH];
    stats[4] = S->last.faded_in[LOW];
    stats[5] = S->last.faded_in[HIGH];
}

void or_ts_get(void* h, int r, double* x, double* v, float* lam, int32_t* state, uint32_t* group,
               uint32_t* ids) {
    TSState* S = (TSState*)h;
    const TPop& p = S->pop[r];
    const size_t n = p.size();
    if (x) std::memcpy(x, p.x.data(), 3 * n * 8);
    if (v) std::memcpy(v, p.v.data(), 3 * n * 8);
    if (lam) std::memcpy(lam, p.lam.data(), n * 4);
    if (state) std::memcpy(state, p.state.data(), n * 4);
    if (group) std::memcpy(group, p.group.data(), n * 4);
    if (ids) std::memcpy(ids, p.ids.data(), n * 4);
}

// The blend / state-machine decisions of one slab-trigger step
// (SPH2S_FINAL_TWO_SCALE/Solver.cu:1229-1289 plus the slab split and group
// merge rules of ts_step above) from the start-of-step state alone: they
// depend on positions only through the slab test of each LOW particle and of
// each group's fixed-point centroid, never on the step's physics.  stats =
// splits, merges, removed LOW, removed HIGH, faded-in LOW, faded-in HIGH;
// per particle (each output optional): keep (survives the step), the state
// bits, blend coefficient and group id it leaves the step with.  Blended mode
// with the slab trigger only.
void or_ts_decide(const OConfig2* C, const uint32_t* n, const float* const* x,
                  const float* const* lam, const int32_t* const* state,
                  const uint32_t* const* group, uint32_t group_base, uint32_t* stats,
                  uint8_t* const* keep, int32_t* const* next_state, float* const* next_lam,
                  uint32_t* const* next_group) {
    const bool refine = C->refine_axis >= 0 && C->refine_axis < 3;
    const int ax = refine ? C->refine_axis : 0;
    std::vector<int64_t> gsum(group_base, 0);
    std::vector<uint32_t> gready(group_base, 0);
    for (uint32_t k = 0; k < n[HIGH]; ++k) {
        const uint32_t g = group[HIGH][k];
        if (g == kNoGroup || g >= group_base) continue;
        gsum[g] += fixed40(x[HIGH][3 * k + ax]);
        gready[g] += state[HIGH][k] == 4 ? 1u : 0u;
    }
    const int64_t L = fixed43(C->refine_lo), H = fixed43(C->refine_hi);
    std::vector<uint8_t> merge(group_base, 0);
    uint32_t merges = 0;
    for (uint32_t g = 0; g < group_base; ++g) {
        merge[g] = refine && gready[g] == 8 && !(L < gsum[g] && gsum[g] < H);
        merges += merge[g];
    }
    const float cblend[4] = {0.0f, -1.0f, 1.0f, 0.0f};
    uint32_t st[6] = {0, merges, 0, 0, 0, 0};
    for (int r = HIGH; r >= LOW; --r)
        for (uint32_t i = 0; i < n[r]; ++i) {
            int32_t s = state[r][i];
            uint32_t g = group[r][i];
            const float xa = x[r][3 * i + ax];
            if (r == LOW && refine && (s & 3) == 0 && C->refine_lo < xa && xa < C->refine_hi)
                s = (s & 4) | 3;
            float l = lam[r][i] + cblend[s & 3] * C->blend_increment;
            uint8_t kp = 1;
            if (l <= 0.0f && (s & 3) == 1) {
                st[2 + r]++;
                kp = 0;
            } else {
                if (l >= 1.0f && (s & 3) == 2) {
                    s &= 4;
                    l = 1.0f;
                    st[4 + r]++;
                }
                if (r == LOW && (s & 3) == 3) {
                    st[0]++;
                    s = 1;
                }
                if (r == HIGH && g != kNoGroup && g < group_base && merge[g]) {
                    s = 5;
                    g = kNoGroup;
                }
            }
            if (keep && keep[r]) keep[r][i] = kp;
            if (next_state && next_state[r]) next_state[r][i] = s;
            if (next_lam && next_lam[r]) next_lam[r][i] = l;
            if (next_group && next_group[r]) next_group[r][i] = g;
        }
    for (int k = 0; k < 6; ++k) stats[k] = st[k];
}

void or_ts_destroy(void* h) { delete (TSState*)h; }

}  // extern "C"
