// mbcg_operators.cuh -- the reference's lattice and operator surface as __host__ __device__
// templates, for code written against its headers (custom kernels, post-processing, tests):
//
//   stencil_ct.cuh                 D3Q27 / D3Q19 and the alias LbmStencil: cx<I>(), cy<I>(),
//                                  cz<I>(), s<I>(), w<I>(), B<I>(), the second- and third-order
//                                  Hermite polynomials, invcnorm<I>(), offset<I>(), offset_xz<I>()
//   pdf.cuh                        feq<I>, fneqr<I>, fpost<I>, guo_force<I>, fneqr_forced<I>
//   collisionOperators.cuh         Omega2<I>, cosphi<I>, recolorDelta<I>
//   forces.cuh                     force_outlet_limited, absforce_calcul, cos2rule<I>,
//                                  tau_interface, A_calculation, preOmega2_outlet_limited
//   utilities/mathUtilities.cuh    psi, force_y_outlet_limited, isJet, clamp01,
//                                  convective_outlet_value
//   utilities/bounds.cuh           wrapx, wrapz (periodic wrap over the fluid nodes)
//   case headers                   init_jet_bulk, init_jet_inlet (jet/jetIn.cuh),
//                                  inlet_bc_calculation, outlet_neumann_bc_calculation
//                                  (jet/boundary_conditions.cuh), bubble_mask, init_static_bubble
//                                  (bubble/bubbleIn.cuh), rti_interface_position, rti_phase_field,
//                                  init_rti_domain, init_rti_y_walls (rti/rtiIn.cuh)
//
// Names, argument order and expression order are the reference's, so FP32 results agree with
// its headers bit for bit (when both are compiled without multiply-add contraction).  The one
// difference: what the reference fixes at compile time in constants.cuh (lattice size, tau,
// sigma, beta, phase densities, case geometry) is a run-time OpParams built from an
// mbcg_params, passed as the last argument of the functions that read it.  Per-direction
// operators take the lattice as an optional second template argument (LbmStencil by default, as
// in the reference), so both lattices can be used in one program.  The lattice is the
// reference's dense layout (index x + NX (y + NY z)); the moments argument of the case functors
// is any struct with the reference's MomentsDevice members (rhor, rhob, ux, ..., Pixz).
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <utility>

#include "mbcg.h"

#if defined(__CUDACC__)
#define MBCG_OPS_HD __host__ __device__
#else
#define MBCG_OPS_HD
#endif
#define MBCG_OPS_FN MBCG_OPS_HD inline

namespace mbcg {
namespace ops {

using label_t = uint32_t;

// constants.cuh:56-69, the same constexpr chain in the real type R
template <typename R = float>
struct Lattice {
    static constexpr R cs2 = static_cast<R>(1.0 / 3.0);
    static constexpr R cs4 = cs2 * cs2;
    static constexpr R cs6 = cs4 * cs2;
    static constexpr R inv_cs2 = static_cast<R>(1) / cs2;
    static constexpr R inv_cs4 = static_cast<R>(1) / cs4;
    static constexpr R inv_cs6 = static_cast<R>(1) / cs6;
    static constexpr R inv_2cs2 = static_cast<R>(1) / (static_cast<R>(2) * cs2);
    static constexpr R inv_2cs4 = static_cast<R>(1) / (static_cast<R>(2) * cs4);
    static constexpr R inv_6cs6 = static_cast<R>(1.0) / (static_cast<R>(6.0) * cs6);
    static constexpr R inv_2cs6 = static_cast<R>(1.0) / (static_cast<R>(2.0) * cs6);
    static constexpr R half = static_cast<R>(0.5);
};

// The run-time part of constants.cuh (constants.cuh:9-93), derived as the reference derives it.
template <typename R = float>
struct OpParams {
    label_t NX, NY, NZ;
    R taub, oms, beta_recolor, sigma, sigma_over_4cs4;
    R rhor0, rhob0;
    R jet_x0, jet_z0, jet_radius, jet_velocity;
    R bubble_x0, bubble_y0, bubble_z0, bubble_radius;
    R rti_y0, rti_amplitude, rti_interface_width;
    int rti_mode_x, rti_mode_z;

    static OpParams from(const mbcg_params& p) {
        OpParams k{};
        k.NX = static_cast<label_t>(p.nx);
        k.NY = static_cast<label_t>(p.ny);
        k.NZ = static_cast<label_t>(p.nz);
        k.taub = static_cast<R>(p.tau);
        k.oms = static_cast<R>(1) - static_cast<R>(1) / k.taub;
        k.beta_recolor = static_cast<R>(p.beta);
        k.sigma = static_cast<R>(p.sigma);
        k.sigma_over_4cs4 = k.sigma / (static_cast<R>(4) * Lattice<R>::cs4);
        k.rhor0 = static_cast<R>(p.rho_r0);
        k.rhob0 = static_cast<R>(p.rho_b0);
        k.jet_x0 = static_cast<R>(p.jet_center[0]);
        k.jet_z0 = static_cast<R>(p.jet_center[1]);
        k.jet_radius = static_cast<R>(p.jet_radius);
        k.jet_velocity = static_cast<R>(p.jet_velocity);
        k.bubble_x0 = static_cast<R>(p.bubble_center[0]);
        k.bubble_y0 = static_cast<R>(p.bubble_center[1]);
        k.bubble_z0 = static_cast<R>(p.bubble_center[2]);
        k.bubble_radius = static_cast<R>(p.bubble_radius);
        k.rti_y0 = static_cast<R>(p.rti_position);
        k.rti_amplitude = static_cast<R>(p.rti_amplitude);
        k.rti_interface_width = static_cast<R>(p.rti_width);
        k.rti_mode_x = p.rti_mode[0];
        k.rti_mode_z = p.rti_mode[1];
        return k;
    }
};

// ---------------------------------------------------------------- lattices (stencil_ct.cuh)
// Tables D (velocities, weights by |c|^2, rest-population B) in the reference's direction order.
template <typename D>
struct Stencil {
    static constexpr int q = D::q;
    template <label_t I>
    MBCG_OPS_HD static constexpr int cx() noexcept { return D::cx_ct[I]; }
    template <label_t I>
    MBCG_OPS_HD static constexpr int cy() noexcept { return D::cy_ct[I]; }
    template <label_t I>
    MBCG_OPS_HD static constexpr int cz() noexcept { return D::cz_ct[I]; }
    template <label_t I>
    MBCG_OPS_HD static constexpr int s() noexcept { return cx<I>() * cx<I>() + cy<I>() * cy<I>() + cz<I>() * cz<I>(); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R w() noexcept { return static_cast<R>(D::weight(s<I>())); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R B() noexcept { return I == 0 ? static_cast<R>(D::b0) : w<I, R>(); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hxx() noexcept { return R(cx<I>() * cx<I>()) - Lattice<R>::cs2; }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hxy() noexcept { return R(cx<I>() * cy<I>()); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hyy() noexcept { return R(cy<I>() * cy<I>()) - Lattice<R>::cs2; }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hyz() noexcept { return R(cy<I>() * cz<I>()); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hzz() noexcept { return R(cz<I>() * cz<I>()) - Lattice<R>::cs2; }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hxz() noexcept { return R(cx<I>() * cz<I>()); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hxxy() noexcept { return R(cx<I>() * cx<I>() * cy<I>()) - Lattice<R>::cs2 * R(cy<I>()); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hxxz() noexcept { return R(cx<I>() * cx<I>() * cz<I>()) - Lattice<R>::cs2 * R(cz<I>()); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hxyy() noexcept { return R(cx<I>() * cy<I>() * cy<I>()) - Lattice<R>::cs2 * R(cx<I>()); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hxzz() noexcept { return R(cx<I>() * cz<I>() * cz<I>()) - Lattice<R>::cs2 * R(cx<I>()); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hyyz() noexcept { return R(cy<I>() * cy<I>() * cz<I>()) - Lattice<R>::cs2 * R(cz<I>()); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hyzz() noexcept { return R(cy<I>() * cz<I>() * cz<I>()) - Lattice<R>::cs2 * R(cy<I>()); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R Hxyz() noexcept { return R(cx<I>() * cy<I>() * cz<I>()); }
    template <label_t I, typename R = float>
    MBCG_OPS_HD static constexpr R invcnorm() noexcept {
        return s<I>() == 0 ? R(0) : s<I>() == 1 ? R(1) : s<I>() == 2 ? R(0.7071067811865475) : R(0.5773502691896258);
    }
    // linear offset of the direction in the dense layout (stencil_ct.cuh:203-214)
    template <label_t I>
    MBCG_OPS_HD static constexpr int offset(label_t NX, label_t NXNY) noexcept {
        return cx<I>() + static_cast<int>(NX) * cy<I>() + static_cast<int>(NXNY) * cz<I>();
    }
    template <label_t I>
    MBCG_OPS_HD static constexpr int offset_xz(label_t NX, label_t NY) noexcept {
        return cx<I>() + static_cast<int>(NX) * static_cast<int>(NY) * cz<I>();
    }
};

struct D3Q27Table {
    static constexpr int q = 27;
    static constexpr int cx_ct[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
    static constexpr int cy_ct[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1};
    static constexpr int cz_ct[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1};
    static constexpr double b0 = -10.0 / 27.0;
    MBCG_OPS_HD static constexpr double weight(int s) {
        return s == 0 ? 8.0 / 27.0 : s == 1 ? 2.0 / 27.0 : s == 2 ? 1.0 / 54.0 : 1.0 / 216.0;
    }
};
struct D3Q19Table {
    static constexpr int q = 19;
    static constexpr int cx_ct[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
    static constexpr int cy_ct[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
    static constexpr int cz_ct[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
    static constexpr double b0 = -1.0 / 3.0;
    MBCG_OPS_HD static constexpr double weight(int s) { return s == 0 ? 1.0 / 3.0 : s == 1 ? 1.0 / 18.0 : 1.0 / 36.0; }
};

using D3Q27 = Stencil<D3Q27Table>;
using D3Q19 = Stencil<D3Q19Table>;
#if defined(MBCG_D3Q19) || defined(LBM_D3Q19)
using LbmStencil = D3Q19;
#else
using LbmStencil = D3Q27;
#endif

// compile-time loop over the directions [B, E)
template <label_t B, label_t E, typename F>
MBCG_OPS_FN void constexpr_for(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<label_t, B>{});
        constexpr_for<B + 1, E>(static_cast<F&&>(f));
    }
}

// ---------------------------------------------------------------- pdf.cuh
// pdf.cuh:16-36
template <label_t I, typename L = LbmStencil, typename R>
MBCG_OPS_FN R feq(const R rho, const R ux, const R uy, const R uz) noexcept {
    using C = Lattice<R>;
    constexpr R cx = static_cast<R>(L::template cx<I>());
    constexpr R cy = static_cast<R>(L::template cy<I>());
    constexpr R cz = static_cast<R>(L::template cz<I>());
    constexpr R wi = L::template w<I, R>();
    const R cu = ux * cx + uy * cy + uz * cz;
    const R usq = ux * ux + uy * uy + uz * uz;
    const R cu2 = cu * cu;
    const R A2eq = (cu * C::inv_cs2) - (usq * C::inv_2cs2) + (cu * cu) * C::inv_2cs4;
    const R A3eq = cu * (cu2 * C::inv_6cs6 - usq * C::inv_2cs4);
    return wi * rho * (static_cast<R>(1.0) + A2eq + A3eq);
}

// pdf.cuh:38-79: regularised non-equilibrium (second- and third-order Hermite projection)
template <label_t I, typename L = LbmStencil, typename R>
MBCG_OPS_FN R fneqr(const R Pixx, const R Pixy, const R Piyy, const R Piyz, const R Pizz, const R Pixz, const R ux,
                    const R uy, const R uz) noexcept {
    using C = Lattice<R>;
    constexpr R wi = L::template w<I, R>();
    const R two = static_cast<R>(2.0);
    const R A2neq = (Pixx * L::template Hxx<I, R>() + two * Pixy * L::template Hxy<I, R>() +
                     Piyy * L::template Hyy<I, R>() + two * Piyz * L::template Hyz<I, R>() +
                     Pizz * L::template Hzz<I, R>() + two * Pixz * L::template Hxz<I, R>()) *
                    C::inv_2cs4;
    const R a3xxy = Pixx * uy + two * Pixy * ux;
    const R a3xxz = Pixx * uz + two * Pixz * ux;
    const R a3xyy = Piyy * ux + two * Pixy * uy;
    const R a3xzz = Pizz * ux + two * Pixz * uz;
    const R a3yyz = Piyy * uz + two * Piyz * uy;
    const R a3yzz = Pizz * uy + two * Piyz * uz;
    const R a3xyz = Pixy * uz + Pixz * uy + Piyz * ux;
    const R A3neq = (a3xxy * L::template Hxxy<I, R>() + a3xxz * L::template Hxxz<I, R>() +
                     a3xyy * L::template Hxyy<I, R>() + a3xzz * L::template Hxzz<I, R>() +
                     a3yyz * L::template Hyyz<I, R>() + a3yzz * L::template Hyzz<I, R>() +
                     two * a3xyz * L::template Hxyz<I, R>()) *
                    C::inv_2cs6;
    return wi * (A2neq + A3neq);
}

// pdf.cuh:81-88: BGK-regularised post-collision population
template <label_t I, typename L = LbmStencil, typename R>
MBCG_OPS_FN R fpost(const R rho, const R ux, const R uy, const R uz, const R Pixx, const R Pixy, const R Piyy,
                    const R Piyz, const R Pizz, const R Pixz, const OpParams<R>& k) noexcept {
    return feq<I, L>(rho, ux, uy, uz) + k.oms * fneqr<I, L>(Pixx, Pixy, Piyy, Piyz, Pizz, Pixz, ux, uy, uz);
}

// pdf.cuh:94-136: Guo forcing term (third-order Hermite form)
template <label_t I, typename L = LbmStencil, typename R>
MBCG_OPS_FN R guo_force(const R Fx, const R Fy, const R Fz, const R ux, const R uy, const R uz) noexcept {
    using C = Lattice<R>;
    constexpr R wi = L::template w<I, R>();
    constexpr R cx = static_cast<R>(L::template cx<I>());
    constexpr R cy = static_cast<R>(L::template cy<I>());
    constexpr R cz = static_cast<R>(L::template cz<I>());
    constexpr R Hxx = L::template Hxx<I, R>(), Hxy = L::template Hxy<I, R>(), Hyy = L::template Hyy<I, R>();
    constexpr R Hyz = L::template Hyz<I, R>(), Hzz = L::template Hzz<I, R>(), Hxz = L::template Hxz<I, R>();
    constexpr R Hxxy = L::template Hxxy<I, R>(), Hxxz = L::template Hxxz<I, R>(), Hxyy = L::template Hxyy<I, R>();
    constexpr R Hxzz = L::template Hxzz<I, R>(), Hyyz = L::template Hyyz<I, R>(), Hyzz = L::template Hyzz<I, R>();
    constexpr R Hxyz = L::template Hxyz<I, R>();
    const R h = C::half;
    const R A1 = (Fx * cx + Fy * cy + Fz * cz) * C::inv_cs2;
    const R A2 = (Fx * ux * Hxx + Fy * uy * Hyy + Fz * uz * Hzz + (Fx * uy + Fy * ux) * Hxy + (Fy * uz + Fz * uy) * Hyz +
                  (Fx * uz + Fz * ux) * Hxz) *
                 C::inv_cs4;
    const R A3 = ((Fx * ux * uy + h * Fy * ux * ux) * Hxxy + (Fx * ux * uz + h * Fz * ux * ux) * Hxxz +
                  (Fy * ux * uy + h * Fx * uy * uy) * Hxyy + (Fz * ux * uz + h * Fx * uz * uz) * Hxzz +
                  (Fy * uy * uz + h * Fz * uy * uy) * Hyyz + (Fz * uy * uz + h * Fy * uz * uz) * Hyzz +
                  (Fx * uy * uz + Fy * ux * uz + Fz * ux * uy) * Hxyz) *
                 C::inv_cs6;
    return wi * (A1 + A2 + A3);
}

// pdf.cuh:144-163: fneq_regularized - F_i / 2
template <label_t I, typename L = LbmStencil, typename R>
MBCG_OPS_FN R fneqr_forced(const R Pixx, const R Pixy, const R Piyy, const R Piyz, const R Pizz, const R Pixz,
                           const R ux, const R uy, const R uz, const R Fx, const R Fy, const R Fz) noexcept {
    const R fneq_regularized = fneqr<I, L>(Pixx, Pixy, Piyy, Piyz, Pizz, Pixz, ux, uy, uz);
    const R Fi = guo_force<I, L>(Fx, Fy, Fz, ux, uy, uz);
    return fneq_regularized - Lattice<R>::half * Fi;
}

// ---------------------------------------------------------------- mathUtilities.cuh, bounds.cuh
// mathUtilities.cuh:12-19
template <typename R>
MBCG_OPS_FN R psi(const R rho_self, const R rho_other) noexcept {
    const R rho_sum = rho_self + rho_other;
    const R rho_diff = rho_self - rho_other;
    return rho_diff / rho_sum;
}
// mathUtilities.cuh:25-33: the colour-gradient y index, clamped below the outlet ghost layer
template <typename R>
MBCG_OPS_FN label_t force_y_outlet_limited(const int y, const OpParams<R>& k) noexcept {
    if (y >= static_cast<int>(k.NY - static_cast<label_t>(1))) return k.NY - static_cast<label_t>(2);
    return static_cast<label_t>(y);
}
// mathUtilities.cuh:39-45
template <typename R>
MBCG_OPS_FN bool isJet(const label_t x, const label_t z, const OpParams<R>& k) noexcept {
    const R dx = static_cast<R>(x) - k.jet_x0;
    const R dz = static_cast<R>(z) - k.jet_z0;
    return (dx * dx + dz * dz) <= (k.jet_radius * k.jet_radius) ? 1 : 0;
}
// mathUtilities.cuh:51-58
template <typename R>
MBCG_OPS_FN R clamp01(const R x) noexcept {
    return x < static_cast<R>(0) ? static_cast<R>(0) : (x > static_cast<R>(1) ? static_cast<R>(1) : x);
}
// mathUtilities.cuh:60-63
template <typename R>
MBCG_OPS_FN R convective_outlet_value(const R phiB_old, const R phiF, const R uc) noexcept {
    return phiB_old - uc * (phiB_old - phiF);
}
// bounds.cuh:34-77: periodic image over the fluid nodes 1..N-2
MBCG_OPS_FN label_t wrap_axis(const label_t v, const label_t N) noexcept {
    if (v == static_cast<label_t>(0)) return N - static_cast<label_t>(2);
    if (v == N - static_cast<label_t>(1)) return static_cast<label_t>(1);
    return v;
}
template <typename R>
MBCG_OPS_FN label_t wrapx(const label_t x, const OpParams<R>& k) noexcept { return wrap_axis(x, k.NX); }
template <typename R>
MBCG_OPS_FN label_t wrapz(const label_t z, const OpParams<R>& k) noexcept { return wrap_axis(z, k.NZ); }

template <typename R>
MBCG_OPS_FN std::size_t idx(const label_t x, const label_t y, const label_t z, const OpParams<R>& k) noexcept {
    return static_cast<std::size_t>(x) + static_cast<std::size_t>(k.NX) * (y + static_cast<std::size_t>(k.NY) * z);
}

// ---------------------------------------------------------------- forces.cuh
// forces.cuh:20-60: F = (1/cs^2) sum_i w_i psi(x + c_i) c_i, x / z wrapped, y clamped at the outlet
template <typename L = LbmStencil, typename R>
MBCG_OPS_FN void force_outlet_limited(const R* __restrict__ rho_self, const R* __restrict__ rho_other, const label_t x,
                                      const label_t y, const label_t z, R& Fx_component, R& Fy_component,
                                      R& Fz_component, const OpParams<R>& k) noexcept {
    R sx = static_cast<R>(0), sy = static_cast<R>(0), sz = static_cast<R>(0);
    constexpr_for<1, L::q>([&](auto Ic) {
        constexpr label_t i = decltype(Ic)::value;
        constexpr int cx_i = L::template cx<i>(), cy_i = L::template cy<i>(), cz_i = L::template cz<i>();
        constexpr R cx = static_cast<R>(cx_i), cy = static_cast<R>(cy_i), cz = static_cast<R>(cz_i);
        constexpr R wi = L::template w<i, R>();
        const label_t xn = wrapx(static_cast<label_t>(static_cast<int>(x) + cx_i), k);
        const label_t zn = wrapz(static_cast<label_t>(static_cast<int>(z) + cz_i), k);
        const label_t yn = force_y_outlet_limited(static_cast<int>(y) + cy_i, k);
        const std::size_t idn = idx(xn, yn, zn, k);
        const R psi_n = psi(rho_self[idn], rho_other[idn]);
        sx += wi * psi_n * cx;
        sy += wi * psi_n * cy;
        sz += wi * psi_n * cz;
    });
    Fx_component = Lattice<R>::inv_cs2 * sx;
    Fy_component = Lattice<R>::inv_cs2 * sy;
    Fz_component = Lattice<R>::inv_cs2 * sz;
}

// forces.cuh:66-69 (single-precision square root, as the reference)
MBCG_OPS_FN float absforce_calcul(const float Fx, const float Fy, const float Fz) noexcept {
    return sqrtf(Fx * Fx + Fy * Fy + Fz * Fz);
}
MBCG_OPS_FN double absforce_calcul(const double Fx, const double Fy, const double Fz) noexcept {
    return sqrt(Fx * Fx + Fy * Fy + Fz * Fz);
}

// forces.cuh:75-95: (F . c_i)^2 / |F|^2, 0 for the rest direction and below |F| = 1e-4
template <label_t I, typename L = LbmStencil, typename R>
MBCG_OPS_FN R cos2rule(const R Fx, const R Fy, const R Fz, const R absF) noexcept {
    if constexpr (I == 0) {
        return static_cast<R>(0);
    } else {
        if (absF <= static_cast<R>(1.0e-4)) return static_cast<R>(0);
        constexpr R cx = static_cast<R>(L::template cx<I>());
        constexpr R cy = static_cast<R>(L::template cy<I>());
        constexpr R cz = static_cast<R>(L::template cz<I>());
        const R Fici = Fx * cx + Fy * cy + Fz * cz;
        return (Fici * Fici) / (absF * absF);
    }
}

// forces.cuh:101-108
template <typename R>
MBCG_OPS_FN R tau_interface(const R rho_self, const R tau_self, const R rho_other, const R tau_other) noexcept {
    const R psix = psi(rho_self, rho_other);
    return static_cast<R>(0.5) * (static_cast<R>(1) + psix) * tau_self +
           static_cast<R>(0.5) * (static_cast<R>(1) - psix) * tau_other;
}

// forces.cuh:114-117
template <typename R>
MBCG_OPS_FN R A_calculation(const R tau_eff, const OpParams<R>& k) noexcept {
    return k.sigma_over_4cs4 / tau_eff;
}

// forces.cuh:124-137
template <typename L = LbmStencil, typename R>
MBCG_OPS_FN void preOmega2_outlet_limited(const R* __restrict__ rho_self, const R* __restrict__ rho_other,
                                          const label_t x, const label_t y, const label_t z, R& Fx, R& Fy, R& Fz,
                                          R& absF, R& A, const OpParams<R>& k) noexcept {
    force_outlet_limited<L>(rho_self, rho_other, x, y, z, Fx, Fy, Fz, k);
    const R tau_eff = k.taub;
    A = A_calculation(tau_eff, k);
    absF = absforce_calcul(Fx, Fy, Fz);
}

// ---------------------------------------------------------------- collisionOperators.cuh
// collisionOperators.cuh:16-25: surface-tension perturbation A |F| / 2 (w_i cos2rule_i - B_i)
template <label_t I, typename L = LbmStencil, typename R>
MBCG_OPS_FN R Omega2(const R Fx, const R Fy, const R Fz, const R absF, const R A) noexcept {
    const R cos2rule_i = cos2rule<I, L>(Fx, Fy, Fz, absF);
    constexpr R wi = L::template w<I, R>();
    constexpr R Bi = L::template B<I, R>();
    return static_cast<R>(0.5) * A * absF * (wi * cos2rule_i - Bi);
}

// collisionOperators.cuh:31-53: cosine between F and c_i
template <label_t I, typename L = LbmStencil, typename R>
MBCG_OPS_FN R cosphi(const R Fx, const R Fy, const R Fz, const R absF) noexcept {
    if constexpr (I == 0) {
        return static_cast<R>(0);
    } else {
        if (absF <= static_cast<R>(1.0e-4)) return static_cast<R>(0);
        constexpr R cx = static_cast<R>(L::template cx<I>());
        constexpr R cy = static_cast<R>(L::template cy<I>());
        constexpr R cz = static_cast<R>(L::template cz<I>());
        constexpr R invc = L::template invcnorm<I, R>();
        const R dot = Fx * cx + Fy * cy + Fz * cz;
        return dot * invc / absF;
    }
}

// collisionOperators.cuh:60-80: recolouring Delta_i = beta (rho_r rho_b / rho^2) cos(phi_i) w_i rho
template <label_t I, typename L = LbmStencil, typename R>
MBCG_OPS_FN R recolorDelta(const R rhor, const R rhob, const R Fx, const R Fy, const R Fz, const R absF,
                           const OpParams<R>& k) noexcept {
    if constexpr (I == 0) {
        return static_cast<R>(0);
    } else {
        const R rho = rhor + rhob;
        constexpr R wi = L::template w<I, R>();
        const R cos_i = cosphi<I, L>(Fx, Fy, Fz, absF);
        const R coeff = k.beta_recolor * (rhor * rhob) / (rho * rho);
        const R fieq = wi * rho;
        return coeff * cos_i * fieq;
    }
}

// ---------------------------------------------------------------- case functors
// jet/jetIn.cuh:16-33: ambient fluid at rest
template <typename M, typename R>
MBCG_OPS_FN void init_jet_bulk(M A, const label_t x, const label_t y, const label_t z, const OpParams<R>& k) noexcept {
    const std::size_t id = idx(x, y, z, k);
    A.rhor[id] = k.rhor0;
    A.rhob[id] = static_cast<R>(0);
    A.ux[id] = A.uy[id] = A.uz[id] = static_cast<R>(0);
    A.Pixx[id] = A.Pixy[id] = A.Piyy[id] = A.Piyz[id] = A.Pizz[id] = A.Pixz[id] = static_cast<R>(0);
}

// jet/jetIn.cuh:39-60: inlet ghost layer y = 0 with the jet disc
template <typename M, typename R>
MBCG_OPS_FN void init_jet_inlet(M A, const label_t x, const label_t z, const OpParams<R>& k) noexcept {
    const std::size_t id = idx(x, static_cast<label_t>(0), z, k);
    const R jetMask = static_cast<R>(isJet(x, z, k));
    A.rhor[id] = (static_cast<R>(1) - jetMask) * k.rhor0;
    A.rhob[id] = jetMask * k.rhob0;
    A.ux[id] = static_cast<R>(0);
    A.uy[id] = jetMask * k.jet_velocity;
    A.uz[id] = static_cast<R>(0);
    A.Pixx[id] = A.Pixy[id] = A.Piyy[id] = A.Piyz[id] = A.Pizz[id] = A.Pixz[id] = static_cast<R>(0);
}

// jet/boundary_conditions.cuh:16-39: inlet functor, Pi copied from the first fluid layer
template <typename M, typename R>
MBCG_OPS_FN void inlet_bc_calculation(M A, const label_t x, const label_t z, const OpParams<R>& k) noexcept {
    const std::size_t idB = idx(x, static_cast<label_t>(0), z, k);
    const std::size_t idF = idx(x, static_cast<label_t>(1), z, k);
    const R jetMask = static_cast<R>(isJet(x, z, k));
    A.rhor[idB] = (static_cast<R>(1) - jetMask) * k.rhor0;
    A.rhob[idB] = jetMask * k.rhob0;
    A.ux[idB] = static_cast<R>(0);
    A.uy[idB] = jetMask * k.jet_velocity;
    A.uz[idB] = static_cast<R>(0);
    A.Pixx[idB] = A.Pixx[idF];
    A.Pixy[idB] = A.Pixy[idF];
    A.Piyy[idB] = A.Piyy[idF];
    A.Piyz[idB] = A.Piyz[idF];
    A.Pizz[idB] = A.Pizz[idF];
    A.Pixz[idB] = A.Pixz[idF];
}

// jet/boundary_conditions.cuh:45-109: convective outlet from the old ghost layer
template <typename M, typename R>
MBCG_OPS_FN void outlet_neumann_bc_calculation(M B, const M Aold, const label_t x, const label_t z,
                                               const OpParams<R>& k) noexcept {
    const std::size_t idB = idx(x, k.NY - static_cast<label_t>(1), z, k);
    const std::size_t idF = idx(x, k.NY - static_cast<label_t>(2), z, k);
    const R rrF = B.rhor[idF], rbF = B.rhob[idF];
    const R uxF = B.ux[idF], uyF = B.uy[idF], uzF = B.uz[idF];
    const R rrB_old = Aold.rhor[idB], rbB_old = Aold.rhob[idB];
    const R uxB_old = Aold.ux[idB], uyB_old = Aold.uy[idB], uzB_old = Aold.uz[idB];
    const R uc = clamp01(uyF);
    const R rhoB_old = rrB_old + rbB_old;
    R rrB, rbB, uxB, uyB, uzB;
    if (rhoB_old <= static_cast<R>(1.0e-20)) {
        rrB = rrF;
        rbB = rbF;
        uxB = uxF;
        uyB = uyF;
        uzB = uzF;
    } else {
        rrB = convective_outlet_value(rrB_old, rrF, uc);
        rbB = convective_outlet_value(rbB_old, rbF, uc);
        uxB = convective_outlet_value(uxB_old, uxF, uc);
        uyB = convective_outlet_value(uyB_old, uyF, uc);
        uzB = convective_outlet_value(uzB_old, uzF, uc);
    }
    B.rhor[idB] = rrB;
    B.rhob[idB] = rbB;
    B.ux[idB] = uxB;
    B.uy[idB] = uyB;
    B.uz[idB] = uzB;
    B.Pixx[idB] = B.Pixx[idF];
    B.Pixy[idB] = B.Pixy[idF];
    B.Piyy[idB] = B.Piyy[idF];
    B.Piyz[idB] = B.Piyz[idF];
    B.Pizz[idB] = B.Pizz[idF];
    B.Pixz[idB] = B.Pixz[idF];
}

// bubble/bubbleIn.cuh:15-30: sharp sphere, blue inside
template <typename M, typename R>
MBCG_OPS_FN void bubble_mask(M A, const label_t x, const label_t y, const label_t z, const OpParams<R>& k) noexcept {
    const std::size_t id = idx(x, y, z, k);
    const R dx = static_cast<R>(x) - k.bubble_x0;
    const R dy = static_cast<R>(y) - k.bubble_y0;
    const R dz = static_cast<R>(z) - k.bubble_z0;
    const R r2 = dx * dx + dy * dy + dz * dz;
    const R R2 = k.bubble_radius * k.bubble_radius;
    const R is_bubble = static_cast<R>(r2 <= R2);
    A.rhor[id] = (static_cast<R>(1) - is_bubble) * k.rhor0;
    A.rhob[id] = is_bubble * k.rhob0;
}

// bubble/bubbleIn.cuh:36-52
template <typename M, typename R>
MBCG_OPS_FN void init_static_bubble(M A, const label_t x, const label_t y, const label_t z,
                                    const OpParams<R>& k) noexcept {
    const std::size_t id = idx(x, y, z, k);
    bubble_mask(A, x, y, z, k);
    A.ux[id] = A.uy[id] = A.uz[id] = static_cast<R>(0);
    A.Pixx[id] = A.Pixy[id] = A.Piyy[id] = A.Piyz[id] = A.Pizz[id] = A.Pixz[id] = static_cast<R>(0);
}

// rti/rtiIn.cuh:18-31: y0 + a cos(kx x) cos(kz z) (single-precision cosine, as the reference)
template <typename R>
MBCG_OPS_FN R rti_interface_position(const label_t x, const label_t z, const OpParams<R>& k) noexcept {
    const R x_real = static_cast<R>(x);
    const R z_real = static_cast<R>(z);
    const R Lx = static_cast<R>(k.NX - static_cast<label_t>(2));
    const R Lz = static_cast<R>(k.NZ - static_cast<label_t>(2));
    const R pi = static_cast<R>(3.141592653589793);
    const R kx = static_cast<R>(2.0) * pi * static_cast<R>(k.rti_mode_x) / Lx;
    const R kz = static_cast<R>(2.0) * pi * static_cast<R>(k.rti_mode_z) / Lz;
    return k.rti_y0 + k.rti_amplitude * cosf(kx * x_real) * cosf(kz * z_real);
}

// rti/rtiIn.cuh:33-40
template <typename R>
MBCG_OPS_FN R rti_phase_field(const label_t x, const label_t y, const label_t z, const OpParams<R>& k) noexcept {
    const R y_real = static_cast<R>(y);
    const R y_interface = rti_interface_position(x, z, k);
    const R eta = (y_real - y_interface) / k.rti_interface_width;
    return tanhf(eta);
}

// rti/rtiIn.cuh:47-70: blue phase above the interface, fluid at rest
template <typename M, typename R>
MBCG_OPS_FN void init_rti_domain(M A, const label_t x, const label_t y, const label_t z, const OpParams<R>& k) noexcept {
    const std::size_t id = idx(x, y, z, k);
    const R phi = rti_phase_field(x, y, z, k);
    A.rhor[id] = static_cast<R>(0.5) * (static_cast<R>(1) - phi) * k.rhor0;
    A.rhob[id] = static_cast<R>(0.5) * (static_cast<R>(1) + phi) * k.rhob0;
    A.ux[id] = A.uy[id] = A.uz[id] = static_cast<R>(0);
    A.Pixx[id] = A.Pixy[id] = A.Piyy[id] = A.Piyz[id] = A.Pizz[id] = A.Pixz[id] = static_cast<R>(0);
}

// rti/rtiIn.cuh:76-119: the wall ghost layers y = 0 and NY-1 copy their neighbour, u = 0
template <typename M, typename R>
MBCG_OPS_FN void init_rti_y_walls(M A, const label_t x, const label_t z, const OpParams<R>& k) noexcept {
    const label_t ys[2][2] = {{static_cast<label_t>(0), static_cast<label_t>(1)},
                              {k.NY - static_cast<label_t>(1), k.NY - static_cast<label_t>(2)}};
    for (int side = 0; side < 2; ++side) {
        const std::size_t idB = idx(x, ys[side][0], z, k);
        const std::size_t idF = idx(x, ys[side][1], z, k);
        A.rhor[idB] = A.rhor[idF];
        A.rhob[idB] = A.rhob[idF];
        A.ux[idB] = A.uy[idB] = A.uz[idB] = static_cast<R>(0);
        A.Pixx[idB] = A.Pixx[idF];
        A.Pixy[idB] = A.Pixy[idF];
        A.Piyy[idB] = A.Piyy[idF];
        A.Piyz[idB] = A.Piyz[idF];
        A.Pizz[idB] = A.Pizz[idF];
        A.Pixz[idB] = A.Pixz[idF];
    }
}

} // namespace ops
} // namespace mbcg
