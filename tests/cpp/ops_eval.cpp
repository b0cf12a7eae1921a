// ops_eval.cpp -- evaluates the lattice and operator surface on seeded inputs and writes every
// result as raw float32, in a fixed order.  Compiled two ways from this one source:
//   -DOPS_REFERENCE  against the reference's own headers (force-included prelude with one
//                    configuration's constants): produces the golden output, where the reference
//                    sources are mounted (tests/golden/make_golden.py);
//   default          against include/mbcg_operators.cuh with the same configuration as run-time
//                    parameters (tests/test_operators.py compares the two outputs bit for bit).
//   ops_eval <in.raw> <out.raw> [<nx> <ny> <nz> <tau> <sigma> <beta> <jet_radius> <jet_velocity>
//            <bubble_radius> <rti_amplitude> <rti_width> <q>]   (the bracket only without OPS_REFERENCE)
// in.raw: NS samples x 15 floats (rho, ux, uy, uz, Pi x6, Fx, Fy, Fz, rhor, rhob), then two lattice
// states of 11 x NX*NY*NZ floats.
#include <cstdio>
#include <cstdlib>
#include <utility>
#include <vector>

#ifdef OPS_REFERENCE
#include "bubble/bubbleIn.cuh"
#include "collisionOperators.cuh"
#include "forces.cuh"
#include "jet/boundary_conditions.cuh"
#include "jet/jetIn.cuh"
#include "pdf.cuh"
#include "rti/rtiIn.cuh"
#include "stencil_ct.cuh"
#include "utilities/mathUtilities.cuh"
using Moments = MomentsDevice;
#define K_
#define QQ Q
static constexpr label_t LX = NX, LY = NY, LZ = NZ;
#else
#include "mbcg_operators.cuh"
using namespace mbcg::ops;
struct Moments {
    float *rhor, *rhob, *ux, *uy, *uz, *Pixx, *Pixy, *Piyy, *Piyz, *Pizz, *Pixz;
};
static OpParams<float> k;
#define K_ , k
#define QQ (LbmStencil::q)
static label_t LX, LY, LZ;
using real_t = float;
#endif

static std::vector<float> out;
static void put(float v) { out.push_back(v); }

template <label_t I>
static void tables() {
    put(static_cast<float>(LbmStencil::cx<I>()));
    put(static_cast<float>(LbmStencil::cy<I>()));
    put(static_cast<float>(LbmStencil::cz<I>()));
    put(LbmStencil::w<I>());
    put(LbmStencil::B<I>());
    put(LbmStencil::Hxx<I>());
    put(LbmStencil::Hxy<I>());
    put(LbmStencil::Hyy<I>());
    put(LbmStencil::Hyz<I>());
    put(LbmStencil::Hzz<I>());
    put(LbmStencil::Hxz<I>());
    put(LbmStencil::Hxxy<I>());
    put(LbmStencil::Hxxz<I>());
    put(LbmStencil::Hxyy<I>());
    put(LbmStencil::Hxzz<I>());
    put(LbmStencil::Hyyz<I>());
    put(LbmStencil::Hyzz<I>());
    put(LbmStencil::Hxyz<I>());
    put(LbmStencil::invcnorm<I>());
}

template <label_t I>
static void per_direction(const float* s) {
    const float rho = s[0], ux = s[1], uy = s[2], uz = s[3];
    const float Pxx = s[4], Pxy = s[5], Pyy = s[6], Pyz = s[7], Pzz = s[8], Pxz = s[9];
    const float Fx = s[10], Fy = s[11], Fz = s[12], rr = s[13], rb = s[14];
    const float absF = absforce_calcul(Fx, Fy, Fz);
    const float A = A_calculation(static_cast<float>(0.8) K_);
    put(feq<I>(rho, ux, uy, uz));
    put(fneqr<I>(Pxx, Pxy, Pyy, Pyz, Pzz, Pxz, ux, uy, uz));
    put(fpost<I>(rho, ux, uy, uz, Pxx, Pxy, Pyy, Pyz, Pzz, Pxz K_));
    put(guo_force<I>(Fx, Fy, Fz, ux, uy, uz));
    put(fneqr_forced<I>(Pxx, Pxy, Pyy, Pyz, Pzz, Pxz, ux, uy, uz, Fx, Fy, Fz));
    put(cos2rule<I>(Fx, Fy, Fz, absF));
    put(Omega2<I>(Fx, Fy, Fz, absF, A));
    put(cosphi<I>(Fx, Fy, Fz, absF));
    put(recolorDelta<I>(rr, rb, Fx, Fy, Fz, absF K_));
}

template <label_t... Is>
static void all_tables(std::integer_sequence<label_t, Is...>) {
    (tables<Is>(), ...);
}
template <label_t... Is>
static void all_directions(const float* s, std::integer_sequence<label_t, Is...>) {
    (per_direction<Is>(s), ...);
}

static Moments view(std::vector<float>& st, size_t n) {
    float* b = st.data();
    return Moments{b, b + n, b + 2 * n, b + 3 * n, b + 4 * n, b + 5 * n, b + 6 * n, b + 7 * n, b + 8 * n, b + 9 * n, b + 10 * n};
}

int main(int argc, char** argv) {
#ifdef OPS_REFERENCE
    if (argc != 3) return 2;
#else
    if (argc != 15) return 2;
    mbcg_params p{};
    p.nx = std::atoi(argv[3]);
    p.ny = std::atoi(argv[4]);
    p.nz = std::atoi(argv[5]);
    p.tau = std::atof(argv[6]);
    p.sigma = std::atof(argv[7]);
    p.beta = std::atof(argv[8]);
    p.jet_radius = std::atof(argv[9]);
    p.jet_velocity = std::atof(argv[10]);
    p.bubble_radius = std::atof(argv[11]);
    p.rti_amplitude = std::atof(argv[12]);
    p.rti_width = std::atof(argv[13]);
    if (std::atoi(argv[14]) != LbmStencil::q) return 5;
    // the reference's derived geometry (constants.cuh): centres at (N - 1) / 2, unit densities,
    // interface mode 1 x 1
    p.rho_r0 = p.rho_b0 = 1.0;
    p.jet_center[0] = (p.nx - 1) / 2.0;
    p.jet_center[1] = (p.nz - 1) / 2.0;
    p.bubble_center[0] = (p.nx - 1) / 2.0;
    p.bubble_center[1] = (p.ny - 1) / 2.0;
    p.bubble_center[2] = (p.nz - 1) / 2.0;
    p.rti_position = (p.ny - 1) / 2.0;
    p.rti_mode[0] = p.rti_mode[1] = 1;
    k = OpParams<float>::from(p);
    LX = k.NX;
    LY = k.NY;
    LZ = k.NZ;
#endif
    const size_t n = static_cast<size_t>(LX) * LY * LZ;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    std::vector<float> in;
    {
        float buf[4096];
        size_t got;
        while ((got = std::fread(buf, sizeof(float), 4096, f)) > 0) in.insert(in.end(), buf, buf + got);
        std::fclose(f);
    }
    const size_t lattice = 2 * 11 * n;
    if (in.size() < lattice || (in.size() - lattice) % 15 != 0) return 4;
    const size_t ns = (in.size() - lattice) / 15;
    const float* samples = in.data();
    std::vector<float> s1(in.end() - lattice, in.end() - lattice / 2), s2(in.end() - lattice / 2, in.end());

    all_tables(std::make_integer_sequence<label_t, QQ>{});
    for (size_t i = 0; i < ns; ++i) all_directions(samples + 15 * i, std::make_integer_sequence<label_t, QQ>{});
    for (size_t i = 0; i < ns; ++i) {
        const float* s = samples + 15 * i;
        put(psi(s[13], s[14]));
        put(absforce_calcul(s[10], s[11], s[12]));
        put(tau_interface(s[13], static_cast<float>(0.7), s[14], static_cast<float>(0.9)));
        put(clamp01(static_cast<float>(20) * s[1]));
        put(convective_outlet_value(s[13], s[14], clamp01(static_cast<float>(10) * s[2])));
    }
    // colour gradient and Omega2 pre-computation at every fluid node of state 1
    {
        Moments A = view(s1, n);
        for (label_t z = 1; z + 1 < LZ; ++z)
            for (label_t y = 1; y + 1 < LY; ++y)
                for (label_t x = 1; x + 1 < LX; ++x) {
                    float Fx, Fy, Fz, absF, Acoef;
                    force_outlet_limited(A.rhor, A.rhob, x, y, z, Fx, Fy, Fz K_);
                    put(Fx);
                    put(Fy);
                    put(Fz);
                    preOmega2_outlet_limited(A.rhor, A.rhob, x, y, z, Fx, Fy, Fz, absF, Acoef K_);
                    put(absF);
                    put(Acoef);
                }
    }
    auto dump = [&](const std::vector<float>& st) { out.insert(out.end(), st.begin(), st.end()); };
    // jet initial condition (jetIn.cuh: bulk everywhere, then the inlet layer)
    {
        std::vector<float> st(s1);
        Moments A = view(st, n);
        for (label_t z = 0; z < LZ; ++z)
            for (label_t y = 0; y < LY; ++y)
                for (label_t x = 0; x < LX; ++x) init_jet_bulk(A, x, y, z K_);
        for (label_t z = 0; z < LZ; ++z)
            for (label_t x = 0; x < LX; ++x) init_jet_inlet(A, x, z K_);
        dump(st);
    }
    // static bubble on the fluid nodes
    {
        std::vector<float> st(s1);
        Moments A = view(st, n);
        for (label_t z = 1; z + 1 < LZ; ++z)
            for (label_t y = 1; y + 1 < LY; ++y)
                for (label_t x = 1; x + 1 < LX; ++x) init_static_bubble(A, x, y, z K_);
        dump(st);
    }
    // Rayleigh-Taylor domain and wall layers, and the interface functions
    {
        std::vector<float> st(s1);
        Moments A = view(st, n);
        for (label_t z = 0; z < LZ; ++z)
            for (label_t y = 0; y < LY; ++y)
                for (label_t x = 0; x < LX; ++x) init_rti_domain(A, x, y, z K_);
        for (label_t z = 1; z + 1 < LZ; ++z)
            for (label_t x = 1; x + 1 < LX; ++x) init_rti_y_walls(A, x, z K_);
        dump(st);
        for (label_t z = 0; z < LZ; ++z)
            for (label_t x = 0; x < LX; ++x) {
                put(rti_interface_position(x, z K_));
                put(rti_phase_field(x, LY / 2, z K_));
            }
    }
    // jet inlet and convective outlet functors (state 2 new, state 1 old)
    {
        std::vector<float> b(s2);
        Moments B = view(b, n), Aold = view(s1, n);
        for (label_t z = 1; z + 1 < LZ; ++z)
            for (label_t x = 1; x + 1 < LX; ++x) {
                inlet_bc_calculation(B, x, z K_);
                outlet_neumann_bc_calculation(B, Aold, x, z K_);
            }
        dump(b);
    }
    FILE* g = std::fopen(argv[2], "wb");
    if (!g) return 6;
    const bool ok = std::fwrite(out.data(), sizeof(float), out.size(), g) == out.size();
    return (std::fclose(g) == 0 && ok) ? 0 : 7;
}
