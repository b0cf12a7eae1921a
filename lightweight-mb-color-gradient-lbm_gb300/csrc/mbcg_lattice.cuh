// mbcg_lattice.cuh -- lattice tables, storage codecs and the device parameter block of the
// GB300 moment-based colour-gradient step.
//
// Stencil<Q> keeps the reference's lattice (stencil_ct.cuh:7-425): velocities in the same
// direction order, weights w, the perturbation constants B (B_0 differs from w_0), and
// 1/|c| (invcnorm).  Everything here is __host__ __device__ constexpr so the host library
// and the kernels share one table.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include "mbcg.h"

namespace mbcg {

#define MBCG_HD __host__ __device__ __forceinline__

// ------------------------------------------------------------------ lattice
template <int Q>
struct Stencil;

template <>
struct Stencil<27> {
    static constexpr int q = 27;
    // stencil_ct.cuh:16-23
    static constexpr int cx[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
    static constexpr int cy[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1};
    static constexpr int cz[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1};
    // weight by |c|^2 = 0, 1, 2, 3 (stencil_ct.cuh:53-75)
    static MBCG_HD constexpr float wk(int s) {
        return s == 0 ? 8.0f / 27.0f : s == 1 ? 2.0f / 27.0f : s == 2 ? 1.0f / 54.0f : 1.0f / 216.0f;
    }
    static constexpr float B0 = -10.0f / 27.0f; // stencil_ct.cuh:77-89
    static MBCG_HD constexpr bool has(int x, int y, int z) { return true; }
};

template <>
struct Stencil<19> {
    static constexpr int q = 19;
    // stencil_ct.cuh:227-234
    static constexpr int cx[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
    static constexpr int cy[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
    static constexpr int cz[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
    // stencil_ct.cuh:264-281
    static MBCG_HD constexpr float wk(int s) {
        return s == 0 ? 1.0f / 3.0f : s == 1 ? 1.0f / 18.0f : s == 2 ? 1.0f / 36.0f : 0.0f;
    }
    static constexpr float B0 = -1.0f / 3.0f; // stencil_ct.cuh:283-295
    static MBCG_HD constexpr bool has(int x, int y, int z) { return x * x + y * y + z * z < 3; }
};

// weight of velocity (x, y, z) in {-1,0,1}^3 (0 for D3Q19 corners)
template <int Q>
MBCG_HD constexpr float weight(int x, int y, int z) {
    return Stencil<Q>::has(x, y, z) ? Stencil<Q>::wk(x * x + y * y + z * z) : 0.0f;
}
// 1/|c| (stencil_ct.cuh:178-200)
MBCG_HD constexpr float inv_cnorm(int x, int y, int z) {
    return (x * x + y * y + z * z) == 0 ? 0.0f
         : (x * x + y * y + z * z) == 1 ? 1.0f
         : (x * x + y * y + z * z) == 2 ? 0.7071067811865475f
                                        : 0.5773502691896258f;
}

// ------------------------------------------------------------------ field slots
enum Field : int { RHOR = 0, RHOB, UX, UY, UZ, PXX, PXY, PYY, PYZ, PZZ, PXZ, NF };

// ------------------------------------------------------------------ storage codecs
// FP32 stores the reference's moments as they are.  FP16 / BF16 store scaled deviations:
// slot 0 (rho - rho_nominal(phi)) / rho_scale, slot 1 the colour complement c (colour_slot),
// 2..4 u / u_ref, 5..10 Pi / pi_scale, with rho_nominal(phi) = (rho_r0 + rho_b0)/2 +
// phi (rho_r0 - rho_b0)/2 evaluated at the stored (rounded) phi.
template <typename S>
struct Codec;

template <>
struct Codec<float> {
    static constexpr int bytes = 4;
    static MBCG_HD float to_f(float v) { return v; }
    static MBCG_HD float from_f(float v) { return v; }
};
// from_f rounds to nearest; from_f_sr rounds a pair stochastically (cvt.rs, sm_100 and later:
// up with probability equal to the distance from the lower neighbour in ulps, drawing on 32
// random bits; exact values, +-0 included, are unchanged).  The instruction packs a into the
// upper half of the result and b into the lower half.
template <>
struct Codec<__half> {
    static constexpr int bytes = 2;
    static __device__ __forceinline__ float to_f(__half v) { return __half2float(v); }
    static __device__ __forceinline__ __half from_f(float v) { return __float2half_rn(v); }
    static __device__ __forceinline__ void from_f_sr(float a, float b, unsigned bits, __half& ha, __half& hb) {
        unsigned d;
        asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(a), "f"(b), "r"(bits));
        ha = __ushort_as_half(static_cast<unsigned short>(d >> 16));
        hb = __ushort_as_half(static_cast<unsigned short>(d & 0xffffU));
    }
};
template <>
struct Codec<__nv_bfloat16> {
    static constexpr int bytes = 2;
    static __device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
    static __device__ __forceinline__ __nv_bfloat16 from_f(float v) { return __float2bfloat16_rn(v); }
    static __device__ __forceinline__ void from_f_sr(float a, float b, unsigned bits, __nv_bfloat16& ha,
                                                     __nv_bfloat16& hb) {
        unsigned d;
        asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(a), "f"(b), "r"(bits));
        ha = __ushort_as_bfloat16(static_cast<unsigned short>(d >> 16));
        hb = __ushort_as_bfloat16(static_cast<unsigned short>(d & 0xffffU));
    }
};

// Colour slot of the 16-bit forms.  It holds the complement of the colour field,
// c = sign(phi) (1 - |phi|) = +2 rho_b / rho (phi >= 0) or -2 rho_r / rho (phi < 0), not phi
// itself: near the pure phases phi rounds to +-1 in 16 bits (resolution 2^-11) and the minority
// colour would vanish, while c keeps its full relative precision there.  Pure red is c = +0,
// pure blue c = -0.
MBCG_HD float colour_slot(float rr, float rb, float rho) {
#ifdef __CUDA_ARCH__
    // a 2-ulp quotient is ample for a 16-bit slot
    return rr >= rb ? __fdividef(2.0f * rb, rho) : -__fdividef(2.0f * rr, rho);
#else
    return rr >= rb ? 2.0f * rb / rho : -(2.0f * rr / rho);
#endif
}
MBCG_HD float phi_of_slot(float c) { return copysignf(1.0f - fabsf(c), c); }
// colour densities from rho and the slot: the minority colour is rho |c| / 2 directly (forming
// 1 + phi in FP32 would cancel away the digits c keeps), the majority the rest
MBCG_HD void colour_split(float c, float rho, float& rr, float& rb) {
    const float minor = 0.5f * rho * fabsf(c);
    const float major = rho - minor;
    const bool red_major = !signbit(c);
    rr = red_major ? major : minor;
    rb = red_major ? minor : major;
}

// ------------------------------------------------------------------ parameter block
struct StepParams {
    int nx, ny, nz;
    int bc[3];          // MBCG_BC_* per axis
    int inout_axis;     // -1 if none
    int outlet;         // MBCG_OUTLET_*
    long long pitch;    // elements between rows
    long long plane;    // elements between planes (pitch * ny)
    // collision
    float oms;          // 1 - 1/tau (constants.cuh:85)
    float A;            // sigma / (4 cs^4 tau) (forces.cuh:114-117, 132-134)
    int tau_var;        // phase-dependent relaxation: tau_eff = (1+psi)/2 tau_r + (1-psi)/2 tau_b
    float tau_r, tau_b, s4; // s4 = sigma / (4 cs^4), so A = s4 / tau_eff
    float beta;
    int omega2_conservative; // Omega2 = 0 below |F| = 1e-4 (mass conserving option)
    int ratio;          // density-ratio rest population on
    float kappa_r, kappa_b;
    int forced;         // body force on
    float g[3];
    // jet inlet (jet/boundary_conditions.cuh:16-39)
    float jet_c0, jet_c1, jet_radius, jet_velocity, noise_amp;
    int jet_blue;       // injected fluid is blue (reference) or red
    float rho_r0, rho_b0;
    unsigned long long seed;
    long long step;     // index of the state being written
    // scaled-deviation storage
    float rho_scale, inv_rho_scale, u_ref, inv_u_ref, pi_scale, inv_pi_scale;
    float rho_mean, rho_half_diff; // rho_nominal = rho_mean + phi * rho_half_diff
    // launch geometry
    int zchunk;         // destination planes per CTA
    int do_bc;          // fuse the inlet/outlet functors into the step
    int ghost_images;   // the ghost frame of periodic x / y axes holds the periodic images of
                        // the opposite fluid layer (read by the step, written through on store)
    int* status;        // device status word (bounded-wait failures); may be null
    int wait_test_cycles; // testing only: > 0 makes the first plane wait of a tile wait on a
                          // barrier nothing completes, with this limit (exercises the bail path)
    const void* a[NF];  // current state
    void* b[NF];        // next state
};

// Optional parts of the step a lattice needs: bounce-back walls, a body force, density-ratio rest
// term or phase-dependent relaxation time (F_FORCE), an inlet/outlet axis.  Kernels are instantiated per feature set.
constexpr int F_WALL = 1, F_FORCE = 2, F_INOUT = 4, F_ALL = 7;

MBCG_HD int features_of(const StepParams& P) {
    int f = 0;
    for (int a = 0; a < 3; ++a)
        if (P.bc[a] == MBCG_BC_WALL) f |= F_WALL;
    if (P.forced || P.ratio || P.tau_var) f |= F_FORCE;
    if (P.inout_axis >= 0) f |= F_INOUT;
    return f;
}

// Random bits for the stochastic rounding of the 16-bit forms: Chris Wellons' "lowbias32"
// integer hash (public domain, github.com/skeeto/hash-prospector), keyed by (seed, step, node,
// slot pair), so a run is reproducible and a restart continues bit for bit.
MBCG_HD unsigned lowbias32(unsigned x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}
// per (seed, step): the base every node's key is offset from
MBCG_HD unsigned round_key_base(unsigned long long seed, long long step) {
    return lowbias32(static_cast<unsigned>(step) ^ lowbias32(static_cast<unsigned>(seed) + 0x632BE5ABU));
}

// Counter-based inlet-noise generator: SplitMix64 finaliser (Steele, Lea & Flood 2014) on
// (seed, step) and then on (dense node index, component).  Uniform in [-1, 1), 24 bits.
MBCG_HD unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
MBCG_HD float noise_xi(unsigned long long seed, long long step, unsigned long long node, int comp) {
    unsigned long long h = mix64(seed + 0x9E3779B97F4A7C15ULL * static_cast<unsigned long long>(step + 1));
    h = mix64(h ^ (node * 4ULL + static_cast<unsigned long long>(comp)));
    return static_cast<float>(static_cast<double>(h >> 40) * (1.0 / 8388608.0) - 1.0);
}

// Periodic image of a coordinate p in [-1, n] on an axis with fluid nodes 1..n-2
// (bounds.cuh:34-77 generalised to the halo of width 2 the colour gradient needs).
MBCG_HD int periodic_image(int p, int n) {
    const int L = n - 2;
    while (p < 1) p += L;
    while (p > n - 2) p -= L;
    return p;
}

} // namespace mbcg
