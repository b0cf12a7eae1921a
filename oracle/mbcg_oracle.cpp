// mbcg_oracle.cpp -- CPU oracle for the moment-based colour-gradient LBM step.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / reference legs may load it.  The product path never calls it.
//
// It restates, loop for loop, the reference's pull-stream time step
//   RCS                       lbm.cuh:20-262
//   feq / fneqr / guo_force   pdf.cuh:16-79, 94-136
//   Omega2 / cosphi / recolorDelta          collisionOperators.cuh:16-80
//   force_outlet_limited / cos2rule / A_calculation / preOmega2_outlet_limited
//                             forces.cuh:20-60, 66-95, 114-137
//   psi / force_y_outlet_limited / isJet / clamp01 / convective_outlet_value
//                             utilities/mathUtilities.cuh:12-63
//   wrapx/y/z, pullx/y/z      utilities/bounds.cuh:34-103
//   inlet / outlet functors   jet/boundary_conditions.cuh:16-109
//   case initial conditions   jet/jetIn.cuh, bubble/bubbleIn.cuh, rti/rtiIn.cuh
// with the same expression order, so that in FP32 it reproduces the reference's own host
// build bit for bit (pinned by tests/test_oracle_golden.py against fixtures generated from
// the reference headers), and in FP64 it is the high-precision oracle.
//
// Extensions the reference lacks (all off by default, each a documented model choice):
//   * any axis periodic / inlet-outlet / wall, wall = halfway bounce-back;
//   * Guo body force F = rho g (stored Pi carries +1/2 (uF + Fu), u = (j + F/2)/rho);
//   * density ratio via a phase-dependent rest population K (w_i - delta_i0),
//     K = rho_r kappa_r + rho_b kappa_b, kappa_k = rho_min / rho_k0 - 1;
//   * zero-gradient outlet; counter-based inlet noise; tanh bubble profile.
//
// Build: see oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <vector>

#include "../include/mbcg.h"

namespace {

// ---------------------------------------------------------------- lattice tables
// Direction order of stencil_ct.cuh:16-23 (D3Q27) and :227-234 (D3Q19, a prefix of it).
const int CX[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
const int CY[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1};
const int CZ[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1};

template <typename R>
struct Consts {
    // constants.cuh:56-69, evaluated in R exactly as the reference's constexpr chain
    R cs2, cs4, cs6, inv_cs2, inv_cs4, inv_cs6, inv_2cs2, inv_2cs4, inv_6cs6, inv_2cs6, half;
    R taub, oms, sigma, sigma_over_4cs4, beta, rhor0, rhob0, kappa_r, kappa_b;
    R tau_r, tau_b; // extension: phase-dependent relaxation (forces.cuh:101-108)
    bool tau_var;
    R g[3];
    bool forced, ratio;
    // per-direction tables (stencil_ct.cuh)
    R w[27], B[27], invc[27], c[3][27];
    R Hxx[27], Hxy[27], Hyy[27], Hyz[27], Hzz[27], Hxz[27];
    R Hxxy[27], Hxxz[27], Hxyy[27], Hxzz[27], Hyyz[27], Hyzz[27], Hxyz[27];
    int opp[27];

    void build(const mbcg_params &p) {
        cs2 = static_cast<R>(1.0 / 3.0);
        cs4 = cs2 * cs2;
        cs6 = cs4 * cs2;
        inv_cs2 = static_cast<R>(1) / cs2;
        inv_cs4 = static_cast<R>(1) / cs4;
        inv_cs6 = static_cast<R>(1) / cs6;
        inv_2cs2 = static_cast<R>(1) / (static_cast<R>(2) * cs2);
        inv_2cs4 = static_cast<R>(1) / (static_cast<R>(2) * cs4);
        inv_6cs6 = static_cast<R>(1.0) / (static_cast<R>(6.0) * cs6);
        inv_2cs6 = static_cast<R>(1.0) / (static_cast<R>(2.0) * cs6);
        half = static_cast<R>(0.5);
        taub = static_cast<R>(p.tau);
        const R omegab = static_cast<R>(1) / taub;
        oms = static_cast<R>(1) - omegab;
        tau_var = p.tau_b > 0.0 && p.tau_b != p.tau;
        tau_r = taub;
        tau_b = p.tau_b > 0.0 ? static_cast<R>(p.tau_b) : taub;
        sigma = static_cast<R>(p.sigma);
        sigma_over_4cs4 = sigma / (static_cast<R>(4) * cs4);
        beta = static_cast<R>(p.beta);
        rhor0 = static_cast<R>(p.rho_r0);
        rhob0 = static_cast<R>(p.rho_b0);
        const double rmin = std::min(p.rho_r0, p.rho_b0);
        kappa_r = static_cast<R>(rmin / p.rho_r0 - 1.0);
        kappa_b = static_cast<R>(rmin / p.rho_b0 - 1.0);
        ratio = (p.rho_r0 != p.rho_b0);
        for (int a = 0; a < 3; ++a) g[a] = static_cast<R>(p.gravity[a]);
        forced = (p.gravity[0] != 0.0 || p.gravity[1] != 0.0 || p.gravity[2] != 0.0);
        const bool q27 = (p.q == 27);
        for (int i = 0; i < 27; ++i) {
            const int cx = CX[i], cy = CY[i], cz = CZ[i];
            const int s = cx * cx + cy * cy + cz * cz;
            c[0][i] = static_cast<R>(cx);
            c[1][i] = static_cast<R>(cy);
            c[2][i] = static_cast<R>(cz);
            if (q27) {
                w[i] = s == 0 ? R(8.0 / 27.0) : s == 1 ? R(2.0 / 27.0) : s == 2 ? R(1.0 / 54.0) : R(1.0 / 216.0);
                B[i] = i == 0 ? R(-10.0 / 27.0) : w[i];
            } else {
                w[i] = s == 0 ? R(1.0 / 3.0) : s == 1 ? R(1.0 / 18.0) : R(1.0 / 36.0);
                B[i] = i == 0 ? R(-1.0 / 3.0) : w[i];
            }
            invc[i] = s == 0 ? R(0) : s == 1 ? R(1) : s == 2 ? R(0.7071067811865475) : R(0.5773502691896258);
            Hxx[i] = R(cx * cx) - cs2;
            Hxy[i] = R(cx * cy);
            Hyy[i] = R(cy * cy) - cs2;
            Hyz[i] = R(cy * cz);
            Hzz[i] = R(cz * cz) - cs2;
            Hxz[i] = R(cx * cz);
            Hxxy[i] = R(cx * cx * cy) - cs2 * R(cy);
            Hxxz[i] = R(cx * cx * cz) - cs2 * R(cz);
            Hxyy[i] = R(cx * cy * cy) - cs2 * R(cx);
            Hxzz[i] = R(cx * cz * cz) - cs2 * R(cx);
            Hyyz[i] = R(cy * cy * cz) - cs2 * R(cz);
            Hyzz[i] = R(cy * cz * cz) - cs2 * R(cy);
            Hxyz[i] = R(cx * cy * cz);
            for (int j = 0; j < 27; ++j)
                if (CX[j] == -cx && CY[j] == -cy && CZ[j] == -cz) opp[i] = j;
        }
    }
};

inline float my_sqrt(float v) { return sqrtf(v); }
inline double my_sqrt(double v) { return std::sqrt(v); }
inline float my_cos(float v) { return cosf(v); }
inline double my_cos(double v) { return std::cos(v); }
inline float my_tanh(float v) { return tanhf(v); }
inline double my_tanh(double v) { return std::tanh(v); }

// Counter-based inlet-noise generator: SplitMix64 finaliser (Steele, Lea & Flood 2014)
// applied to (seed, step) and then to (node, component).  Identical integer arithmetic in
// the CUDA library; returns a value in [-1, 1) with 24 random bits.
inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
template <typename R>
inline R noise_xi(uint64_t seed, int64_t step, uint64_t node, int comp) {
    uint64_t h = mix64(seed + 0x9E3779B97F4A7C15ULL * static_cast<uint64_t>(step + 1));
    h = mix64(h ^ (node * 4ULL + static_cast<uint64_t>(comp)));
    return static_cast<R>(static_cast<double>(h >> 40) * (1.0 / 8388608.0) - 1.0);
}

template <typename R>
struct Oracle {
    const mbcg_params &p;
    Consts<R> k;
    int N[3];
    int Q;
    int64_t sx, sy, sz; // dense strides
    R *const *A;
    R *const *B;
    // Per-step caches of psi at every node and of the colour gradient F at every interface node
    // of state A (filled by rcs before the node loop).  The reference recomputes F of a source
    // for each direction that pulls from it; both caches hold the same numbers, computed by the
    // same expressions in the same order, so the results are the same bits at a fraction of the
    // cost on interface-heavy lattices.
    // The storage lives per calling thread across steps (no allocation per step); only the
    // entries rcs fills are read.
    static std::vector<R> &cache_store(int which) {
        thread_local std::vector<R> store[2];
        return store[which];
    }
    std::vector<R> &psi_c = cache_store(0);
    std::vector<R> &F_c = cache_store(1);
    mutable bool psi_ready = false, F_ready = false;

    Oracle(const mbcg_params &pp, R *const *a, R *const *b) : p(pp), A(a), B(b) {
        k.build(p);
        N[0] = p.nx; N[1] = p.ny; N[2] = p.nz;
        Q = p.q;
        sx = 1; sy = p.nx; sz = int64_t(p.nx) * p.ny;
    }

    int64_t id(int x, int y, int z) const { return x * sx + y * sy + z * sz; }
    int64_t id3(const int *v) const { return id(v[0], v[1], v[2]); }

    // bounds.cuh:34-77
    int wrap(int a, int v) const {
        if (v == 0) return N[a] - 2;
        if (v == N[a] - 1) return 1;
        return v;
    }

    // pdf.cuh:16-36
    R feq(int i, R rho, R ux, R uy, R uz) const {
        const R cx = k.c[0][i], cy = k.c[1][i], cz = k.c[2][i];
        const R wi = k.w[i];
        const R cu = ux * cx + uy * cy + uz * cz;
        const R usq = ux * ux + uy * uy + uz * uz;
        const R cu2 = cu * cu;
        const R A2eq = (cu * k.inv_cs2) - (usq * k.inv_2cs2) + (cu * cu) * k.inv_2cs4;
        const R A3eq = cu * (cu2 * k.inv_6cs6 - usq * k.inv_2cs4);
        return wi * rho * (static_cast<R>(1.0) + A2eq + A3eq);
    }

    // pdf.cuh:38-79
    R fneqr(int i, R Pixx, R Pixy, R Piyy, R Piyz, R Pizz, R Pixz, R ux, R uy, R uz) const {
        const R two = static_cast<R>(2.0);
        const R A2neq = (Pixx * k.Hxx[i] + two * Pixy * k.Hxy[i] + Piyy * k.Hyy[i] + two * Piyz * k.Hyz[i] +
                         Pizz * k.Hzz[i] + two * Pixz * k.Hxz[i]) * k.inv_2cs4;
        const R a3xxy = Pixx * uy + two * Pixy * ux;
        const R a3xxz = Pixx * uz + two * Pixz * ux;
        const R a3xyy = Piyy * ux + two * Pixy * uy;
        const R a3xzz = Pizz * ux + two * Pixz * uz;
        const R a3yyz = Piyy * uz + two * Piyz * uy;
        const R a3yzz = Pizz * uy + two * Piyz * uz;
        const R a3xyz = Pixy * uz + Pixz * uy + Piyz * ux;
        const R A3neq = (a3xxy * k.Hxxy[i] + a3xxz * k.Hxxz[i] + a3xyy * k.Hxyy[i] + a3xzz * k.Hxzz[i] +
                         a3yyz * k.Hyyz[i] + a3yzz * k.Hyzz[i] + two * a3xyz * k.Hxyz[i]) * k.inv_2cs6;
        return k.w[i] * (A2neq + A3neq);
    }

    // pdf.cuh:94-136 (Guo forcing term, third-order Hermite form)
    R guo(int i, R Fx, R Fy, R Fz, R ux, R uy, R uz) const {
        const R cx = k.c[0][i], cy = k.c[1][i], cz = k.c[2][i];
        const R h = k.half;
        const R A1 = (Fx * cx + Fy * cy + Fz * cz) * k.inv_cs2;
        const R A2 = (Fx * ux * k.Hxx[i] + Fy * uy * k.Hyy[i] + Fz * uz * k.Hzz[i] + (Fx * uy + Fy * ux) * k.Hxy[i] +
                      (Fy * uz + Fz * uy) * k.Hyz[i] + (Fx * uz + Fz * ux) * k.Hxz[i]) * k.inv_cs4;
        const R A3 = ((Fx * ux * uy + h * Fy * ux * ux) * k.Hxxy[i] + (Fx * ux * uz + h * Fz * ux * ux) * k.Hxxz[i] +
                      (Fy * ux * uy + h * Fx * uy * uy) * k.Hxyy[i] + (Fz * ux * uz + h * Fx * uz * uz) * k.Hxzz[i] +
                      (Fy * uy * uz + h * Fz * uy * uy) * k.Hyyz[i] + (Fz * uy * uz + h * Fy * uz * uz) * k.Hyzz[i] +
                      (Fx * uy * uz + Fy * ux * uz + Fz * ux * uy) * k.Hxyz[i]) * k.inv_cs6;
        return k.w[i] * (A1 + A2 + A3);
    }

    // extension: phase-dependent rest population, K (w_i - delta_i0)
    R ratio_term(int i, R rr, R rb) const {
        const R K = rr * k.kappa_r + rb * k.kappa_b;
        return K * (k.w[i] - (i == 0 ? static_cast<R>(1) : static_cast<R>(0)));
    }

    // utilities/mathUtilities.cuh:12-19
    static R psi(R self, R other) {
        const R s = self + other;
        const R d = self - other;
        return d / s;
    }

    // neighbour coordinate rule of the colour gradient (forces.cuh:28-31,
    // mathUtilities.cuh:25-33): periodic axes wrap, the inlet/outlet axis clamps only at the
    // outlet side, wall axes clamp on both sides (extension: neutral wetting).
    int force_coord(int a, int v) const {
        switch (p.bc[a]) {
        case MBCG_BC_PERIODIC: return wrap(a, v);
        case MBCG_BC_INOUT: return v >= N[a] - 1 ? N[a] - 2 : v;
        default: return v <= 0 ? 1 : (v >= N[a] - 1 ? N[a] - 2 : v);
        }
    }

    // forces.cuh:20-60
    void force(const int *n, R &Fx, R &Fy, R &Fz) const {
        R sx_ = 0, sy_ = 0, sz_ = 0;
        for (int i = 1; i < Q; ++i) {
            int v[3];
            v[0] = force_coord(0, n[0] + CX[i]);
            v[1] = force_coord(1, n[1] + CY[i]);
            v[2] = force_coord(2, n[2] + CZ[i]);
            const int64_t idn = id3(v);
            const R psi_n = psi_ready ? psi_c[idn] : psi(A[0][idn], A[1][idn]);
            sx_ += k.w[i] * psi_n * k.c[0][i];
            sy_ += k.w[i] * psi_n * k.c[1][i];
            sz_ += k.w[i] * psi_n * k.c[2][i];
        }
        Fx = k.inv_cs2 * sx_;
        Fy = k.inv_cs2 * sy_;
        Fz = k.inv_cs2 * sz_;
    }

    // forces.cuh:75-95
    R cos2rule(int i, R Fx, R Fy, R Fz, R absF) const {
        if (i == 0) return 0;
        if (absF <= static_cast<R>(1.0e-4)) return 0;
        const R Fici = Fx * k.c[0][i] + Fy * k.c[1][i] + Fz * k.c[2][i];
        return (Fici * Fici) / (absF * absF);
    }
    // collisionOperators.cuh:16-25
    R omega2(int i, R Fx, R Fy, R Fz, R absF, R Acoef) const {
        const R c2 = cos2rule(i, Fx, Fy, Fz, absF);
        return static_cast<R>(0.5) * Acoef * absF * (k.w[i] * c2 - k.B[i]);
    }
    // collisionOperators.cuh:31-53
    R cosphi(int i, R Fx, R Fy, R Fz, R absF) const {
        if (i == 0) return 0;
        if (absF <= static_cast<R>(1.0e-4)) return 0;
        const R dot = Fx * k.c[0][i] + Fy * k.c[1][i] + Fz * k.c[2][i];
        return dot * k.invc[i] / absF;
    }
    // collisionOperators.cuh:60-80.  With a density ratio the rest-state equilibrium of a
    // moving direction is w_i (rho + K) (extension), so the recolouring uses that weight.
    R recolor(int i, R rr, R rb, R Fx, R Fy, R Fz, R absF) const {
        if (i == 0) return 0;
        const R rho = rr + rb;
        const R cos_i = cosphi(i, Fx, Fy, Fz, absF);
        const R coeff = k.beta * (rr * rb) / (rho * rho);
        const R fieq = k.ratio ? k.w[i] * (rho + rr * k.kappa_r + rb * k.kappa_b) : k.w[i] * rho;
        return coeff * cos_i * fieq;
    }

    // extension: tau_interface (forces.cuh:101-108) with the red phase as "self"
    R tau_eff(R rr, R rb) const {
        const R psix = psi(rr, rb);
        return static_cast<R>(0.5) * (static_cast<R>(1) + psix) * k.tau_r +
               static_cast<R>(0.5) * (static_cast<R>(1) - psix) * k.tau_b;
    }
    R oms_of(R rr, R rb) const { return k.tau_var ? static_cast<R>(1) - static_cast<R>(1) / tau_eff(rr, rb) : k.oms; }

    // Bulk branch of lbm.cuh:153-208 for source node n and direction i.
    void bulk(const int *n, int i, R &fr, R &fb) const {
        const int64_t src = id3(n);
        const R rhor_s = A[0][src], rhob_s = A[1][src];
        const R rho_s = rhor_s + rhob_s;
        const R inv_rhos = static_cast<R>(1) / (rhor_s + rhob_s);
        const R aR = rhor_s * inv_rhos;
        const R aB = rhob_s * inv_rhos;
        const R ux_s = A[2][src], uy_s = A[3][src], uz_s = A[4][src];
        const R gieq = feq(i, rho_s, ux_s, uy_s, uz_s);
        const R gineqr = fneqr(i, A[5][src], A[6][src], A[7][src], A[8][src], A[9][src], A[10][src], ux_s, uy_s, uz_s);
        const R omega1 = gieq + oms_of(rhor_s, rhob_s) * gineqr;
        const R interface_indicator = static_cast<R>(4) * rhor_s * rhob_s * inv_rhos * inv_rhos;
        R gi = omega1;
        if (k.ratio) gi += ratio_term(i, rhor_s, rhob_s);
        if (k.forced) gi += k.half * guo(i, rho_s * k.g[0], rho_s * k.g[1], rho_s * k.g[2], ux_s, uy_s, uz_s);
        R Deltai = 0;
        if (interface_indicator > static_cast<R>(1.0e-4)) {
            R Fx, Fy, Fz;
            if (!F_ready) {
                force(n, Fx, Fy, Fz);
            } else {
                Fx = F_c[3 * src];
                Fy = F_c[3 * src + 1];
                Fz = F_c[3 * src + 2];
            }
            const R Acoef = k.sigma_over_4cs4 / (k.tau_var ? tau_eff(rhor_s, rhob_s) : k.taub);
            const R absF = my_sqrt(Fx * Fx + Fy * Fy + Fz * Fz);
            if (!p.omega2_conservative || absF > static_cast<R>(1.0e-4)) gi += omega2(i, Fx, Fy, Fz, absF, Acoef);
            Deltai = recolor(i, rhor_s, rhob_s, Fx, Fy, Fz, absF);
        }
        fr = aR * gi + Deltai;
        fb = aB * gi - Deltai;
    }

    // Ghost branch of lbm.cuh:83-151 (inlet/outlet ghost source s, first fluid node f).
    void ghost(const int *s, const int *f, int i, R &fr, R &fb) const {
        const int64_t src = id3(s);
        const int64_t idF = id3(f);
        const R rrB = A[0][src], rbB = A[1][src];
        const R rhoB = rrB + rbB;
        const R inv_rhoB = static_cast<R>(1) / rhoB;
        const R aR = rrB * inv_rhoB;
        const R aB = rbB * inv_rhoB;
        const R uxB = A[2][src], uyB = A[3][src], uzB = A[4][src];
        const R gieq = feq(i, rhoB, uxB, uyB, uzB);
        const R gineqr = fneqr(i, A[5][idF], A[6][idF], A[7][idF], A[8][idF], A[9][idF], A[10][idF], A[2][idF],
                               A[3][idF], A[4][idF]);
        R gi = gieq + oms_of(rrB, rbB) * gineqr;
        if (k.ratio) gi += ratio_term(i, rrB, rbB);
        if (k.forced) gi += k.half * guo(i, rhoB * k.g[0], rhoB * k.g[1], rhoB * k.g[2], uxB, uyB, uzB);
        fr = aR * gi;
        fb = aB * gi;
    }

    // One destination node (lbm.cuh:20-262 with the source classification generalised).
    void rcs_node(int x, int y, int z) const {
        const int pos[3] = {x, y, z};
        R sumr = 0, sumb = 0, jx = 0, jy = 0, jz = 0;
        R Axx = 0, Axy = 0, Ayy = 0, Ayz = 0, Azz = 0, Axz = 0;
        for (int i = 0; i < Q; ++i) {
            const int c[3] = {CX[i], CY[i], CZ[i]};
            int s[3];
            int ghost_axis = -1;
            bool wall_hit = false;
            for (int a = 0; a < 3; ++a) {
                s[a] = pos[a] - c[a];
                if (p.bc[a] == MBCG_BC_PERIODIC) {
                    s[a] = wrap(a, s[a]);
                } else if (s[a] == 0 || s[a] == N[a] - 1) {
                    if (p.bc[a] == MBCG_BC_WALL) wall_hit = true;
                    else ghost_axis = a;
                }
            }
            R fr_i, fb_i;
            if (wall_hit) {
                bulk(pos, k.opp[i], fr_i, fb_i); // halfway bounce-back
            } else if (ghost_axis >= 0) {
                int f[3] = {s[0], s[1], s[2]};
                f[ghost_axis] = (s[ghost_axis] == 0) ? 1 : N[ghost_axis] - 2;
                ghost(s, f, i, fr_i, fb_i);
            } else {
                bulk(s, i, fr_i, fb_i);
            }
            sumr += fr_i;
            sumb += fb_i;
            const R g_i = fr_i + fb_i;
            jx += g_i * k.c[0][i];
            jy += g_i * k.c[1][i];
            jz += g_i * k.c[2][i];
            Axx += g_i * k.Hxx[i];
            Axy += g_i * k.Hxy[i];
            Ayy += g_i * k.Hyy[i];
            Ayz += g_i * k.Hyz[i];
            Azz += g_i * k.Hzz[i];
            Axz += g_i * k.Hxz[i];
        }
        const R rhor_t = sumr, rhob_t = sumb;
        const R rho_t = rhor_t + rhob_t;
        const R inv_rho = static_cast<R>(1) / rho_t;
        R vx, vy, vz, Fx = 0, Fy = 0, Fz = 0;
        if (k.forced) {
            Fx = rho_t * k.g[0];
            Fy = rho_t * k.g[1];
            Fz = rho_t * k.g[2];
            vx = (jx + k.half * Fx) * inv_rho;
            vy = (jy + k.half * Fy) * inv_rho;
            vz = (jz + k.half * Fz) * inv_rho;
        } else {
            vx = jx * inv_rho;
            vy = jy * inv_rho;
            vz = jz * inv_rho;
        }
        const int64_t o = id(x, y, z);
        B[0][o] = rhor_t;
        B[1][o] = rhob_t;
        B[2][o] = vx;
        B[3][o] = vy;
        B[4][o] = vz;
        R Pxx = Axx - rho_t * vx * vx;
        R Pxy = Axy - rho_t * vx * vy;
        R Pyy = Ayy - rho_t * vy * vy;
        R Pyz = Ayz - rho_t * vy * vz;
        R Pzz = Azz - rho_t * vz * vz;
        R Pxz = Axz - rho_t * vx * vz;
        if (k.forced) {
            Pxx += vx * Fx;
            Pxy += k.half * (vx * Fy + vy * Fx);
            Pyy += vy * Fy;
            Pyz += k.half * (vy * Fz + vz * Fy);
            Pzz += vz * Fz;
            Pxz += k.half * (vx * Fz + vz * Fx);
        }
        if (k.ratio) {
            const R Kc = (rhor_t * k.kappa_r + rhob_t * k.kappa_b) * k.cs2;
            Pxx -= Kc;
            Pyy -= Kc;
            Pzz -= Kc;
        }
        B[5][o] = Pxx;
        B[6][o] = Pxy;
        B[7][o] = Pyy;
        B[8][o] = Pyz;
        B[9][o] = Pzz;
        B[10][o] = Pxz;
    }

    // the interface test of bulk() (lbm.cuh:181,187) at node o of state A
    bool interface_node(int64_t o) const {
        const R rhor_s = A[0][o], rhob_s = A[1][o];
        const R inv_rhos = static_cast<R>(1) / (rhor_s + rhob_s);
        return static_cast<R>(4) * rhor_s * rhob_s * inv_rhos * inv_rhos > static_cast<R>(1.0e-4);
    }

    // cached: the colour gradient once per interface node (the default); otherwise once per
    // (destination, direction) as the reference computes it (the timed CPU baseline)
    void rcs(int threads, bool cached) const {
        const int z0 = 1, z1 = N[2] - 1;
        psi_ready = F_ready = false;
        if (cached) {
            const int64_t n_all = int64_t(N[0]) * N[1] * N[2];
            if (static_cast<int64_t>(psi_c.size()) < n_all) psi_c.resize(n_all);
            if (static_cast<int64_t>(F_c.size()) < 3 * n_all) F_c.resize(3 * n_all);
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
            for (int64_t o = 0; o < n_all; ++o) psi_c[o] = psi(A[0][o], A[1][o]);
            psi_ready = true;
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
            for (int z = 0; z < N[2]; ++z)
                for (int y = 0; y < N[1]; ++y)
                    for (int x = 0; x < N[0]; ++x) {
                        const int64_t o = id(x, y, z);
                        if (!interface_node(o)) continue;
                        const int n[3] = {x, y, z};
                        force(n, F_c[3 * o], F_c[3 * o + 1], F_c[3 * o + 2]);
                    }
            F_ready = true;
        }
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
        for (int z = z0; z < z1; ++z)
            for (int y = 1; y < N[1] - 1; ++y)
                for (int x = 1; x < N[0] - 1; ++x) rcs_node(x, y, z);
    }

    int inout_axis() const {
        for (int a = 0; a < 3; ++a)
            if (p.bc[a] == MBCG_BC_INOUT) return a;
        return -1;
    }

    // isJet (mathUtilities.cuh:39-45) on the two transverse coordinates
    R jet_mask(int u, int v) const {
        const R dx = static_cast<R>(u) - static_cast<R>(p.jet_center[0]);
        const R dz = static_cast<R>(v) - static_cast<R>(p.jet_center[1]);
        const R rad = static_cast<R>(p.jet_radius);
        return (dx * dx + dz * dz) <= (rad * rad) ? static_cast<R>(1) : static_cast<R>(0);
    }

    // Inlet functor (jet/boundary_conditions.cuh:16-39, jet/jetIn.cuh:39-60) on state T.
    // copy_pi: take Pi from the first fluid layer (boundary pass) or zero it (initial state).
    void inlet(R *const *T, int a, int u, int v, bool copy_pi, int64_t step) const {
        const int ta = (a + 1) % 3, tb = (a + 2) % 3;
        const int b0 = std::min(ta, tb), b1 = std::max(ta, tb);
        int nb[3], nf[3];
        nb[a] = 0; nf[a] = 1;
        nb[b0] = nf[b0] = u;
        nb[b1] = nf[b1] = v;
        const int64_t idB = id3(nb), idF = id3(nf);
        const R jetMask = jet_mask(u, v);
        if (p.jet_phase < 0) {
            T[0][idB] = (static_cast<R>(1) - jetMask) * k.rhor0;
            T[1][idB] = jetMask * k.rhob0;
        } else {
            T[0][idB] = jetMask * k.rhor0;
            T[1][idB] = (static_cast<R>(1) - jetMask) * k.rhob0;
        }
        R uu[3] = {0, 0, 0};
        uu[a] = jetMask * static_cast<R>(p.jet_velocity);
        if (p.inlet_noise != 0.0 && copy_pi) {
            const R amp = static_cast<R>(p.jet_velocity * p.inlet_noise);
            for (int cmp = 0; cmp < 3; ++cmp)
                uu[cmp] += jetMask * amp * noise_xi<R>(p.seed, step, static_cast<uint64_t>(idB), cmp);
        }
        T[2][idB] = uu[0];
        T[3][idB] = uu[1];
        T[4][idB] = uu[2];
        for (int f = 5; f < 11; ++f) T[f][idB] = copy_pi ? T[f][idF] : static_cast<R>(0);
    }

    // Outlet functor (jet/boundary_conditions.cuh:45-109) on B using old state O.
    void outlet(R *const *Bn, R *const *O, int a, int u, int v) const {
        const int ta = (a + 1) % 3, tb = (a + 2) % 3;
        const int b0 = std::min(ta, tb), b1 = std::max(ta, tb);
        int nb[3], nf[3];
        nb[a] = N[a] - 1; nf[a] = N[a] - 2;
        nb[b0] = nf[b0] = u;
        nb[b1] = nf[b1] = v;
        const int64_t idB = id3(nb), idF = id3(nf);
        if (p.outlet == MBCG_OUTLET_ZERO_GRADIENT) {
            for (int f = 0; f < 11; ++f) Bn[f][idB] = Bn[f][idF];
            return;
        }
        const R rrF = Bn[0][idF], rbF = Bn[1][idF];
        const R uF[3] = {Bn[2][idF], Bn[3][idF], Bn[4][idF]};
        const R rrB_old = O[0][idB], rbB_old = O[1][idB];
        const R uB_old[3] = {O[2][idB], O[3][idB], O[4][idB]};
        R ucomp = uF[a];
        const R uc = ucomp < static_cast<R>(0) ? static_cast<R>(0) : (ucomp > static_cast<R>(1) ? static_cast<R>(1) : ucomp);
        const R rhoB_old = rrB_old + rbB_old;
        R out[5];
        if (rhoB_old <= static_cast<R>(1.0e-20)) {
            out[0] = rrF; out[1] = rbF;
            for (int c = 0; c < 3; ++c) out[2 + c] = uF[c];
        } else {
            out[0] = rrB_old - uc * (rrB_old - rrF);
            out[1] = rbB_old - uc * (rbB_old - rbF);
            for (int c = 0; c < 3; ++c) out[2 + c] = uB_old[c] - uc * (uB_old[c] - uF[c]);
        }
        for (int f = 0; f < 5; ++f) Bn[f][idB] = out[f];
        for (int f = 5; f < 11; ++f) Bn[f][idB] = Bn[f][idF];
    }

    // kernels.cu:102-114 on B with old state O
    void bc(R *const *Bn, R *const *O, int64_t step) const {
        const int a = inout_axis();
        if (a < 0) return;
        const int ta = (a + 1) % 3, tb = (a + 2) % 3;
        const int b0 = std::min(ta, tb), b1 = std::max(ta, tb);
        for (int v = 1; v < N[b1] - 1; ++v)
            for (int u = 1; u < N[b0] - 1; ++u) {
                inlet(Bn, a, u, v, true, step);
                outlet(Bn, O, a, u, v);
            }
    }

    // ---------------------------------------------------------------- initial conditions
    void init_jet(R *const *T) const {
        const int a = inout_axis();
        const int64_t n = int64_t(N[0]) * N[1] * N[2];
        for (int64_t i = 0; i < n; ++i) {
            if (p.jet_phase < 0) {
                T[0][i] = k.rhor0;
                T[1][i] = static_cast<R>(0);
            } else {
                T[0][i] = static_cast<R>(0);
                T[1][i] = k.rhob0;
            }
            for (int f = 2; f < 11; ++f) T[f][i] = static_cast<R>(0);
        }
        if (a < 0) return;
        const int ta = (a + 1) % 3, tb = (a + 2) % 3;
        const int b0 = std::min(ta, tb), b1 = std::max(ta, tb);
        for (int v = 1; v < N[b1] - 1; ++v)
            for (int u = 1; u < N[b0] - 1; ++u) inlet(T, a, u, v, false, 0);
        bc(T, T, 0);
    }

    void init_bubble(R *const *T) const {
        const R x0 = static_cast<R>(p.bubble_center[0]);
        const R y0 = static_cast<R>(p.bubble_center[1]);
        const R z0 = static_cast<R>(p.bubble_center[2]);
        const R rad = static_cast<R>(p.bubble_radius);
        const R width = static_cast<R>(p.bubble_width);
        for (int z = 1; z < N[2] - 1; ++z)
            for (int y = 1; y < N[1] - 1; ++y)
                for (int x = 1; x < N[0] - 1; ++x) {
                    const int64_t o = id(x, y, z);
                    const R dx = static_cast<R>(x) - x0;
                    const R dy = static_cast<R>(y) - y0;
                    const R dz = static_cast<R>(z) - z0;
                    const R r2 = dx * dx + dy * dy + dz * dz;
                    if (p.bubble_width <= 0.0) {
                        const R R2 = rad * rad;
                        const R in = static_cast<R>(r2 <= R2);
                        if (p.bubble_phase < 0) {
                            T[0][o] = (static_cast<R>(1) - in) * k.rhor0;
                            T[1][o] = in * k.rhob0;
                        } else {
                            T[0][o] = in * k.rhor0;
                            T[1][o] = (static_cast<R>(1) - in) * k.rhob0;
                        }
                    } else {
                        const R ps = static_cast<R>(p.bubble_phase) * my_tanh((rad - my_sqrt(r2)) / width);
                        T[0][o] = static_cast<R>(0.5) * (static_cast<R>(1) + ps) * k.rhor0;
                        T[1][o] = static_cast<R>(0.5) * (static_cast<R>(1) - ps) * k.rhob0;
                    }
                    for (int f = 2; f < 11; ++f) T[f][o] = static_cast<R>(0);
                }
    }

    int rti_axis() const {
        for (int a = 0; a < 3; ++a)
            if (p.bc[a] == MBCG_BC_WALL) return a;
        return 1;
    }

    void init_rti(R *const *T) const {
        const int h = rti_axis();
        const int ta = (h + 1) % 3, tb = (h + 2) % 3;
        const int t0 = std::min(ta, tb), t1 = std::max(ta, tb);
        const R pi = static_cast<R>(3.141592653589793);
        const R L0 = static_cast<R>(N[t0] - 2), L1 = static_cast<R>(N[t1] - 2);
        const R k0 = static_cast<R>(2.0) * pi * static_cast<R>(p.rti_mode[0]) / L0;
        const R k1 = static_cast<R>(2.0) * pi * static_cast<R>(p.rti_mode[1]) / L1;
        const R pos0 = static_cast<R>(p.rti_position), amp = static_cast<R>(p.rti_amplitude);
        const R width = static_cast<R>(p.rti_width);
        for (int z = 0; z < N[2]; ++z)
            for (int y = 0; y < N[1]; ++y)
                for (int x = 0; x < N[0]; ++x) {
                    const int c[3] = {x, y, z};
                    const R pos = pos0 + amp * my_cos(k0 * static_cast<R>(c[t0])) * my_cos(k1 * static_cast<R>(c[t1]));
                    const R eta = (static_cast<R>(c[h]) - pos) / width;
                    const R phi = my_tanh(eta);
                    const int64_t o = id(x, y, z);
                    if (p.rti_phase_above < 0) {
                        T[0][o] = static_cast<R>(0.5) * (static_cast<R>(1) - phi) * k.rhor0;
                        T[1][o] = static_cast<R>(0.5) * (static_cast<R>(1) + phi) * k.rhob0;
                    } else {
                        T[0][o] = static_cast<R>(0.5) * (static_cast<R>(1) + phi) * k.rhor0;
                        T[1][o] = static_cast<R>(0.5) * (static_cast<R>(1) - phi) * k.rhob0;
                    }
                    for (int f = 2; f < 11; ++f) T[f][o] = static_cast<R>(0);
                }
        // rtiIn.cuh:76-119: wall ghost layers copy the neighbour with u = 0
        for (int v = 1; v < N[t1] - 1; ++v)
            for (int u = 1; u < N[t0] - 1; ++u) {
                for (int side = 0; side < 2; ++side) {
                    int nb[3], nf[3];
                    nb[h] = side == 0 ? 0 : N[h] - 1;
                    nf[h] = side == 0 ? 1 : N[h] - 2;
                    nb[t0] = nf[t0] = u;
                    nb[t1] = nf[t1] = v;
                    const int64_t idB = id3(nb), idF = id3(nf);
                    T[0][idB] = T[0][idF];
                    T[1][idB] = T[1][idF];
                    T[2][idB] = T[3][idB] = T[4][idB] = static_cast<R>(0);
                    for (int f = 5; f < 11; ++f) T[f][idB] = T[f][idF];
                }
            }
    }

    void init(R *const *T) const {
        switch (p.ic) {
        case MBCG_IC_JET: init_jet(T); break;
        case MBCG_IC_BUBBLE: init_bubble(T); break;
        case MBCG_IC_RTI: init_rti(T); break;
        default: break;
        }
    }
};

int check(const mbcg_params *p) {
    if (!p) return -1;
    if (p->q != 19 && p->q != 27) return -1;
    if (p->nx < 3 || p->ny < 3 || p->nz < 3) return -1;
    int np = 0;
    for (int a = 0; a < 3; ++a) {
        if (p->bc[a] < 0 || p->bc[a] > 2) return -1;
        if (p->bc[a] != MBCG_BC_PERIODIC) ++np;
    }
    if (np > 1) return -1;
    return 0;
}

template <typename R>
int step_impl(const mbcg_params *p, void *const *a, void *const *b, int64_t step, int do_rcs, int do_bc,
              int threads) {
    R *A[11], *B[11];
    for (int f = 0; f < 11; ++f) {
        A[f] = static_cast<R *>(a[f]);
        B[f] = static_cast<R *>(b[f]);
    }
    Oracle<R> o(*p, A, B);
    if (do_rcs) o.rcs(threads, do_rcs != 2);
    if (do_bc) o.bc(B, A, step);
    return 0;
}

template <typename R>
int init_impl(const mbcg_params *p, void *const *a) {
    R *A[11];
    for (int f = 0; f < 11; ++f) A[f] = static_cast<R *>(a[f]);
    Oracle<R> o(*p, A, A);
    o.init(A);
    return 0;
}

} // namespace

extern "C" {

// One time step on dense (pitch = nx) host arrays of 4-byte (float) or 8-byte (double)
// reals: RCS A -> B over the fluid nodes (if do_rcs; 2: with the colour gradient recomputed for
// every direction as the reference does, same results), then the inlet/outlet functors on B
// reading the old state A (if do_bc).  step = index of the state B holds.
int oracle_step(const mbcg_params *p, int real_bytes, void *const *a, void *const *b, int64_t step, int do_rcs,
                int do_bc, int threads) {
    if (check(p)) return -1;
    if (real_bytes == 4) return step_impl<float>(p, a, b, step, do_rcs, do_bc, threads);
    if (real_bytes == 8) return step_impl<double>(p, a, b, step, do_rcs, do_bc, threads);
    return -1;
}

// Initial condition p->ic on state a (plus the jet's initial boundary pass).
int oracle_init(const mbcg_params *p, int real_bytes, void *const *a) {
    if (check(p)) return -1;
    if (real_bytes == 4) return init_impl<float>(p, a);
    if (real_bytes == 8) return init_impl<double>(p, a);
    return -1;
}

// Inlet noise sample, exported so tests can compare it with the CUDA library's generator.
double oracle_noise(uint64_t seed, int64_t step, uint64_t node, int comp) {
    return noise_xi<double>(seed, step, node, comp);
}

} // extern "C"
