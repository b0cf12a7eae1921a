// mbcg_step.cuh -- fused moment-based colour-gradient time step for sm_103a (GB300).
//
// step_tile() advances one tile (30 columns x (W-2) rows x zchunk planes) of one lattice by one
// time step of the reference's main loop (main.cu:41-45):
//   RCS (lbm.cuh:20-262)  +  jet inlet/outlet functors (kernels.cu:102-114)  [+ swap by the host]
// The plain step kernel runs one tile per CTA over a grid covering the lattice; the batch
// kernel (mbcg_batch.cu) runs tiles of many lattices from a queue in persistent CTAs.  The
// translation units mbcg_step_q{19,27}_{f32,f16,bf16}.cu instantiate the plain kernel.
//
// Formulation.  The reference pulls, for every destination node and direction i, the post-
// collision population of the source node x - c_i and rebuilds it from the source's 11
// moments (feq + oms*fneqr, Omega2 and recolouring at interfaces).  Every one of those
// populations is a polynomial in c_i whose coefficients depend only on the source node, so
// here each source node is visited once:
//   1. its coefficient tensor p_abc (monomials cx^a cy^b cz^c, a,b,c <= 2; 17 non-zero) is
//      built from the moments (equilibrium, regularised non-equilibrium, Guo force,
//      density-ratio rest term, Omega2), plus the rest-population correction r0;
//   2. a separable inverse transform over x, y, z evaluates all Q populations g_i = w_i V(c_i)
//      (+ r0 at i = 0); red populations are fr_i = aR g_i + Delta_i (recolouring);
//   3. populations are streamed and projected onto the destination's moments by the
//      separable forward transform, one axis at a time:
//        z: the CTA marches along z; class cz of source plane k feeds destination plane k+cz,
//        x: warp lanes are consecutive x nodes; neighbours exchange by __shfl_up/down_sync,
//        y: warps are consecutive y rows; neighbours exchange through shared memory.
// The colour gradient F (forces.cuh:20-60) is evaluated once per interface source node from a
// ring of psi = (rhor - rhob)/rho planes kept in shared memory.
//
// Tiling.  A CTA is 32 lanes (x) x W warps (y).  Lanes 0 and 31 and warps 0 and W-1 are
// halo sources; the CTA writes the 30 x (W-2) destination columns in between, for a chunk of
// zchunk planes.  Each source plane arrives in shared memory through TMA
// (cp.async.bulk.tensor.3d, one box per field, 4-slot ring tracked by mbarriers).  The ghost
// frame of a periodic x / y axis holds the periodic image of the opposite fluid layer (every
// store writes it through), so every source a tile needs is inside its staged box
// (bounds.cuh:34-77 wraps on read instead); the periodic images two layers out that the colour
// gradient needs come from global memory one plane ahead.
//
// Boundary kinds: periodic; inlet/outlet (the reference's ghost-source branch,
// lbm.cuh:79-151, plus the inlet and outlet functors fused into the store of the first and
// last fluid layer); wall (halfway bounce-back).
//
// Feature sets.  kFeat selects at compile time which optional parts a kernel carries:
// F_WALL (bounce-back walls), F_FORCE (body force and density-ratio rest term), F_INOUT (an
// inlet/outlet axis).  A lattice runs on any instantiation whose set covers its parameters;
// the smaller sets leave out code, registers and branches the lattice never uses.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "mbcg_lattice.cuh"
#include "mbcg_internal.h"

namespace mbcg {

namespace {

constexpr int kTX = kStepTileX; // destination columns per CTA (30)
constexpr int kRBX = kStepRBX;   // staged width of rhor/rhob rows (34 needed + 16-byte alignment slack)
constexpr int kMX = kStepMX;     // staged width of the other 9 fields (32 needed + slack)
constexpr int kPSX = 34;   // psi ring width (32 sources + 1 on each side)
constexpr int kNSTAGE = 4; // planes staged: k, k+1, and k+2, k+3 in flight
constexpr unsigned kFull = 0xffffffffu;

constexpr int align128(int b) { return (b + 127) / 128 * 128; }

// Shared-memory carve-up of one tile: the mbarriers in the first 128 bytes, then the staged
// planes, the psi ring and the y-exchange buffer.  `smem` is the dynamic size to request (it
// includes 128 bytes of slack for aligning the base).
template <typename S, int W>
struct Geo {
    static constexpr int RBY = W + 2;
    static constexpr int MY = W;
    static constexpr int rb_field = align128(RBY * kRBX * (int)sizeof(S));
    static constexpr int m_field = align128(MY * kMX * (int)sizeof(S));
    static constexpr int stage = 2 * rb_field + 9 * m_field;
    static constexpr int tx = 2 * RBY * kRBX * (int)sizeof(S) + 9 * MY * kMX * (int)sizeof(S);
    static constexpr int psi_plane = RBY * kPSX;           // floats
    static constexpr int psi = kNSTAGE * psi_plane * 4;    // bytes (ring slot = stage slot)
    static constexpr int xbuf_floats = 3 * 2 * 4 * W * 32; // float4 [class][slot][row][lane]
    static constexpr int xbuf = xbuf_floats * 4;
    static constexpr int off_bar = 0;
    static constexpr int off_stage = 128;
    static constexpr int off_psi = off_stage + kNSTAGE * stage;
    static constexpr int off_xbuf = off_psi + psi;
    static constexpr int smem = off_xbuf + xbuf + 128;
};

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after ~limit clock cycles instead of spinning forever.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit) {
    if (mbar_try_wait(bar, parity)) return true; // the usual case: the plane is already there
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > limit) return false;
    }
    return true;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ int floor8(int v) { return v & ~7; }

// ------------------------------------------------------------------ coordinate roles
enum Role : int { R_FLUID = 0, R_IMAGE = 1, R_GHOST = 2, R_WALL = 3, R_OUT = 4 };

template <int kFeat>
__device__ __forceinline__ int axis_role(const StepParams& P, int a, int p, int n) {
    if (p < 0 || p > n - 1) return R_OUT;
    if (p == 0 || p == n - 1) {
        if constexpr ((kFeat & (F_WALL | F_INOUT)) == 0) return R_IMAGE;
        const int k = P.bc[a];
        return k == MBCG_BC_PERIODIC ? R_IMAGE : (k == MBCG_BC_INOUT ? R_GHOST : R_WALL);
    }
    return R_FLUID;
}
__device__ __forceinline__ int data_coord(const StepParams& P, int a, int p, int n) {
    return (P.bc[a] == MBCG_BC_PERIODIC) ? periodic_image(p, n) : min(max(p, 0), n - 1);
}
// neighbour rule of the colour gradient (forces.cuh:28-31, mathUtilities.cuh:25-33)
__device__ __forceinline__ int psi_coord(const StepParams& P, int a, int p, int n) {
    const int k = P.bc[a];
    if (k == MBCG_BC_PERIODIC) return periodic_image(p, n);
    if (k == MBCG_BC_INOUT) return p >= n - 1 ? n - 2 : max(p, 0);
    return min(max(p, 1), n - 2);
}

// ------------------------------------------------------------------ state access
template <typename S>
struct Node {
    float rr, rb, ux, uy, uz, pxx, pxy, pyy, pyz, pzz, pxz;
};

template <typename S>
__device__ __forceinline__ float psi_of(const StepParams& P, S s0, S s1) {
    if constexpr (std::is_same<S, float>::value) {
        const float r = Codec<S>::to_f(s0), b = Codec<S>::to_f(s1);
        return __fdividef(r - b, r + b);
    } else {
        (void)P;
        (void)s0;
        return phi_of_slot(Codec<S>::to_f(s1));
    }
}

// psi from the two stored slots already widened to float
template <typename S>
__device__ __forceinline__ float psi_of_slots(float v0, float v1) {
    if constexpr (std::is_same<S, float>::value) return __fdividef(v0 - v1, v0 + v1);
    else return phi_of_slot(v1);
}

// decode the 11 stored slots into the reference's moments
template <typename S>
__device__ __forceinline__ void decode(const StepParams& P, const float (&v)[NF], Node<S>& n) {
    if constexpr (sizeof(S) == 4) {
        n.rr = v[0]; n.rb = v[1]; n.ux = v[2]; n.uy = v[3]; n.uz = v[4];
        n.pxx = v[5]; n.pxy = v[6]; n.pyy = v[7]; n.pyz = v[8]; n.pzz = v[9]; n.pxz = v[10];
    } else {
        const float phi = phi_of_slot(v[1]);
        const float rho = P.rho_mean + phi * P.rho_half_diff + P.rho_scale * v[0];
        colour_split(v[1], rho, n.rr, n.rb);
        n.ux = P.u_ref * v[2]; n.uy = P.u_ref * v[3]; n.uz = P.u_ref * v[4];
        n.pxx = P.pi_scale * v[5]; n.pxy = P.pi_scale * v[6]; n.pyy = P.pi_scale * v[7];
        n.pyz = P.pi_scale * v[8]; n.pzz = P.pi_scale * v[9]; n.pxz = P.pi_scale * v[10];
    }
}

// The 16-bit forms round every stored slot stochastically (`key`: the node's random stream).
// Rounded to nearest, a slowly changing state is rounded the same way step after step and the
// errors add up (field error growing in proportion to the step count); rounded stochastically
// they are unbiased and independent from step to step.
template <typename S>
__device__ __forceinline__ void encode(const StepParams& P, float rr, float rb, const float (&u)[3],
                                       const float (&pi)[6], S (&out)[NF], unsigned key) {
    if constexpr (sizeof(S) == 4) {
        (void)key;
        out[0] = rr; out[1] = rb; out[2] = u[0]; out[3] = u[1]; out[4] = u[2];
        for (int i = 0; i < 6; ++i) out[5 + i] = pi[i];
    } else {
        const float rho = rr + rb;
        S unused;
        Codec<S>::from_f_sr(colour_slot(rr, rb, rho), 0.0f, lowbias32(key), out[1], unused);
        const float phi = phi_of_slot(Codec<S>::to_f(out[1])); // the phi a reader decodes
        Codec<S>::from_f_sr((rho - (P.rho_mean + phi * P.rho_half_diff)) * P.inv_rho_scale, u[0] * P.inv_u_ref,
                            lowbias32(key + 1), out[0], out[2]);
        Codec<S>::from_f_sr(u[1] * P.inv_u_ref, u[2] * P.inv_u_ref, lowbias32(key + 2), out[3], out[4]);
        Codec<S>::from_f_sr(pi[0] * P.inv_pi_scale, pi[1] * P.inv_pi_scale, lowbias32(key + 3), out[5], out[6]);
        Codec<S>::from_f_sr(pi[2] * P.inv_pi_scale, pi[3] * P.inv_pi_scale, lowbias32(key + 4), out[7], out[8]);
        Codec<S>::from_f_sr(pi[4] * P.inv_pi_scale, pi[5] * P.inv_pi_scale, lowbias32(key + 5), out[9], out[10]);
    }
}

// random stream of node (x, y, z) given the step's key base: six consecutive keys per node
__device__ __forceinline__ unsigned node_round_key(const StepParams& P, unsigned base, int x, int y, int z) {
    // unsigned arithmetic: the index wraps (harmlessly) on lattices beyond 2^32 nodes
    const unsigned node = (static_cast<unsigned>(z) * static_cast<unsigned>(P.ny) + static_cast<unsigned>(y)) *
                              static_cast<unsigned>(P.nx) +
                          static_cast<unsigned>(x);
    return base + 6U * node;
}

template <typename S>
__device__ __forceinline__ void store_node(const StepParams& P, long long o, const S (&v)[NF]) {
#pragma unroll
    for (int f = 0; f < NF; ++f) static_cast<S*>(P.b[f])[o] = v[f];
}

template <typename S>
__device__ __forceinline__ void load_global(const StepParams& P, long long o, float (&v)[NF]) {
#pragma unroll
    for (int f = 0; f < NF; ++f) v[f] = Codec<S>::to_f(static_cast<const S*>(P.a[f])[o]);
}

// ------------------------------------------------------------------ coefficient tensor
struct Coef {
    float p000, p100, p010, p001, p200, p020, p002, p110, p101, p011;
    float p210, p201, p120, p102, p021, p012, p111, r0;
};

// Equilibrium (pdf.cuh:16-36) at (rho, u) + oms * regularised non-equilibrium (pdf.cuh:38-79)
// from (Pi, v) + 1/2 Guo force (pdf.cuh:94-136) + density-ratio rest term, as the
// coefficients of a polynomial in c (w_i factored out).
// Phase-dependent relaxation (forces.cuh:101-108): tau_eff = (1 + psi)/2 tau_r + (1 - psi)/2 tau_b
__device__ __forceinline__ float tau_eff_of(const StepParams& P, float rr, float rb) {
    const float psix = (rr - rb) / (rr + rb);
    return 0.5f * (1.0f + psix) * P.tau_r + 0.5f * (1.0f - psix) * P.tau_b;
}

template <int kFeat>
__device__ __forceinline__ void build_coef(const StepParams& P, Coef& c, float rho, float rr, float rb, float ux,
                                           float uy, float uz, float vx, float vy, float vz, float pxx, float pxy,
                                           float pyy, float pyz, float pzz, float pxz) {
    float oms = P.oms;
    if constexpr ((kFeat & F_FORCE) != 0)
        if (P.tau_var) oms = 1.0f - 1.0f / tau_eff_of(P, rr, rb);
    const float usq = ux * ux + uy * uy + uz * uz;
    const float rux = rho * ux, ruy = rho * uy, ruz = rho * uz;
    const float t1 = 3.0f - 4.5f * usq;
    const float a3xxy = pxx * vy + 2.0f * pxy * vx;
    const float a3xxz = pxx * vz + 2.0f * pxz * vx;
    const float a3xyy = pyy * vx + 2.0f * pxy * vy;
    const float a3xzz = pzz * vx + 2.0f * pxz * vz;
    const float a3yyz = pyy * vz + 2.0f * pyz * vy;
    const float a3yzz = pzz * vy + 2.0f * pyz * vz;
    const float a3xyz = pxy * vz + pxz * vy + pyz * vx;
    const float o45 = 4.5f * oms, o9 = 9.0f * oms, o135 = 13.5f * oms;
    // p000 holds only the small isotropic part; rho itself is added to every direction last
    // (see emit), so the rounding of rho + small treats rest and moving populations alike
    c.p000 = -1.5f * (rho * usq + oms * (pxx + pyy + pzz));
    c.p100 = rux * t1 + 4.5f * rux * ux * ux - o45 * (a3xyy + a3xzz);
    c.p010 = ruy * t1 + 4.5f * ruy * uy * uy - o45 * (a3xxy + a3yzz);
    c.p001 = ruz * t1 + 4.5f * ruz * uz * uz - o45 * (a3xxz + a3yyz);
    c.p200 = 4.5f * rux * ux + o45 * pxx;
    c.p020 = 4.5f * ruy * uy + o45 * pyy;
    c.p002 = 4.5f * ruz * uz + o45 * pzz;
    c.p110 = 9.0f * rux * uy + o9 * pxy;
    c.p101 = 9.0f * rux * uz + o9 * pxz;
    c.p011 = 9.0f * ruy * uz + o9 * pyz;
    c.p210 = 13.5f * rux * ux * uy + o135 * a3xxy;
    c.p201 = 13.5f * rux * ux * uz + o135 * a3xxz;
    c.p120 = 13.5f * rux * uy * uy + o135 * a3xyy;
    c.p102 = 13.5f * rux * uz * uz + o135 * a3xzz;
    c.p021 = 13.5f * ruy * uy * uz + o135 * a3yyz;
    c.p012 = 13.5f * ruy * uz * uz + o135 * a3yzz;
    c.p111 = 27.0f * rux * uy * uz + 2.0f * o135 * a3xyz;
    c.r0 = 0.0f;
    if constexpr ((kFeat & F_FORCE) == 0) return;
    if (P.forced) {
        const float Fx = rho * P.g[0], Fy = rho * P.g[1], Fz = rho * P.g[2];
        const float Gxxy = Fx * ux * uy + 0.5f * Fy * ux * ux;
        const float Gxxz = Fx * ux * uz + 0.5f * Fz * ux * ux;
        const float Gxyy = Fy * ux * uy + 0.5f * Fx * uy * uy;
        const float Gxzz = Fz * ux * uz + 0.5f * Fx * uz * uz;
        const float Gyyz = Fy * uy * uz + 0.5f * Fz * uy * uy;
        const float Gyzz = Fz * uy * uz + 0.5f * Fy * uz * uz;
        const float Gxyz = Fx * uy * uz + Fy * ux * uz + Fz * ux * uy;
        c.p000 -= 1.5f * (Fx * ux + Fy * uy + Fz * uz);
        c.p100 += 1.5f * Fx - 4.5f * (Gxyy + Gxzz);
        c.p010 += 1.5f * Fy - 4.5f * (Gxxy + Gyzz);
        c.p001 += 1.5f * Fz - 4.5f * (Gxxz + Gyyz);
        c.p200 += 4.5f * Fx * ux;
        c.p020 += 4.5f * Fy * uy;
        c.p002 += 4.5f * Fz * uz;
        c.p110 += 4.5f * (Fx * uy + Fy * ux);
        c.p101 += 4.5f * (Fx * uz + Fz * ux);
        c.p011 += 4.5f * (Fy * uz + Fz * uy);
        c.p210 += 13.5f * Gxxy;
        c.p201 += 13.5f * Gxxz;
        c.p120 += 13.5f * Gxyy;
        c.p102 += 13.5f * Gxzz;
        c.p021 += 13.5f * Gyyz;
        c.p012 += 13.5f * Gyzz;
        c.p111 += 13.5f * Gxyz;
    }
    if (P.ratio) {
        const float K = rr * P.kappa_r + rb * P.kappa_b;
        c.p000 += K;
        c.r0 -= K;
    }
}

// ------------------------------------------------------------------ accumulators
// (rho, red) and (jx, xx) are packed pairs: they always take the same operations, which then
// issue as one f32x2 instruction (add/fma.f32x2, sm_100 and later) instead of two.
struct Acc {
    float2 rr, jxx;
    float jy, jz, xy, yy, yz, zz, xz;
    __device__ __forceinline__ void zero() {
        rr = jxx = make_float2(0.0f, 0.0f);
        jy = jz = xy = yy = yz = zz = xz = 0.0f;
    }
};

__device__ __forceinline__ float2 pair(float v) { return make_float2(v, v); }
// a + f b on both halves (f = 1: a plain add, as fmaf(1, b, a) would round)
template <int F>
__device__ __forceinline__ float2 acc2(float2 a, float2 b) {
    if constexpr (F == 1) return __fadd2_rn(a, b);
    else return __ffma2_rn(pair(static_cast<float>(F)), b, a);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    float2 r;
    asm("{.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

// A quantity over the three x velocities of one (cy, cz): `o` = (cx = -1, cx = +1) as an f32x2
// pair, `c` = cx = 0.  The two outer values always take the same operations.
struct Tri {
    float2 o;
    float c;
};
__device__ __forceinline__ Tri tri(float base, float odd, float centre) {
    return Tri{make_float2(base - odd, base + odd), centre};
}
__device__ __forceinline__ Tri operator+(Tri a, Tri b) { return Tri{__fadd2_rn(a.o, b.o), a.c + b.c}; }
__device__ __forceinline__ Tri operator-(Tri a, Tri b) { return Tri{sub2(a.o, b.o), a.c - b.c}; }
__device__ __forceinline__ Tri operator+(Tri a, float s) { return Tri{__fadd2_rn(a.o, pair(s)), a.c + s}; }

// add one population of velocity (ex, ey, ez) to a destination's moment sums
__device__ __forceinline__ void add_pop(Acc& a, float g, float r, int ex, int ey, int ez) {
    a.rr.x += g;
    a.rr.y += r;
    if (ex) { a.jxx.x += ex * g; a.jxx.y += g; }
    if (ey) { a.jy += ey * g; a.yy += g; }
    if (ez) { a.jz += ez * g; a.zz += g; }
    if (ex && ey) a.xy += ex * ey * g;
    if (ey && ez) a.yz += ey * ez * g;
    if (ex && ez) a.xz += ex * ez * g;
}

// ------------------------------------------------------------------ the kernel
// fast reciprocal (MUFU-based, <= 2 ulp); the colour fraction of a pure node stays exact
__device__ __forceinline__ float fast_rcp(float v) { return __fdividef(1.0f, v); }

// Store one node at (x, y, z); on periodic x / y axes the first and last fluid layers are also
// written to their image in the opposite ghost layer, so the next step reads every source
// (including wrapped ones) from the staged box (bounds.cuh:34-77 wraps on read instead).
// ix / iy: the column's periodic image in x / y (-1: none).
template <typename S>
__device__ __forceinline__ void finalize_store(const StepParams& P, int x, int y, int z, float rr, float rb,
                                               float ux, float uy, float uz, const float (&pi)[6], int ix, int iy,
                                               unsigned key_base) {
    const float u[3] = {ux, uy, uz};
    S out[NF];
    encode<S>(P, rr, rb, u, pi, out, sizeof(S) == 4 ? 0U : node_round_key(P, key_base, x, y, z));
    const long long zo = static_cast<long long>(z) * P.plane;
    store_node<S>(P, zo + static_cast<long long>(y) * P.pitch + x, out);
    if ((ix & iy) != -1) { // either is >= 0: the faces of a periodic x / y axis only
        if (ix >= 0) store_node<S>(P, zo + static_cast<long long>(y) * P.pitch + ix, out);
        if (iy >= 0) store_node<S>(P, zo + static_cast<long long>(iy) * P.pitch + x, out);
        if (ix >= 0 && iy >= 0) store_node<S>(P, zo + static_cast<long long>(iy) * P.pitch + ix, out);
    }
}

// 128-byte aligned base of the dynamic shared memory (TMA destinations need it; every Geo
// size carries the slack)
__device__ __forceinline__ unsigned char* aligned_smem_base() {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    return reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
}

// Initialise the stage mbarriers (one elected thread) before the first tile of a CTA.  One more
// barrier after them is never arrived at: the bounded-wait test hook waits on it.
__device__ __forceinline__ void init_stage_barriers(unsigned char* smem) {
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        for (int s = 0; s <= kNSTAGE; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
}

// One tile of one time step.  (bx, by, bz) index the tile in the lattice's tile grid; `step`
// is the index of the state being written (keys the inlet noise); `phase` carries the parity
// of the stage mbarriers from one tile of a CTA to the next (0 before the first tile).
// Returns false if a staged plane never arrived (the status word is set and the CTA must stop).
// kLeanZ: compile the steady-state body for an inlet/outlet z axis (the batch kernel, whose
// lattices never have one, leaves it out).
template <int Q, typename S, int W, bool kTMA, int kFeat, bool kLeanZ = true>
__device__ __forceinline__ bool step_tile(const StepParams& P, const CUtensorMap* maps, int bx, int by, int bz,
                                          long long step, unsigned char* smem, uint32_t& phase) {
    using G = Geo<S, W>;
    float* psi_ring = reinterpret_cast<float*>(smem + G::off_psi);
    float4* xbuf = reinterpret_cast<float4*>(smem + G::off_xbuf);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + G::off_bar);

    const int lane = threadIdx.x;
    const int w = threadIdx.y;
    const int tid = w * 32 + lane;
    const int nx = P.nx, ny = P.ny, nz = P.nz;

    const int xb = kTX * bx;     // source column of lane 0
    const int yb = (W - 2) * by; // source row of warp 0
    const int xs = xb + lane, ys = yb + w;
    const int zd0 = 1 + P.zchunk * bz;
    const int zd1 = min(zd0 + P.zchunk, nz - 1);
    const int kfirst = zd0 - 2;

    const int xr0 = floor8(xb - 1); // first staged column of rhor/rhob
    const int xm0 = floor8(xb);     // first staged column of the other fields
    const int offRB = xb - xr0;
    const int offM = xb - xm0;
    const int bR = (w + 1) * kRBX + lane + offRB; // this node in the rhor/rhob boxes
    const int bM = w * kMX + lane + offM;         // this node in the other boxes

    const bool dest_thread = lane >= 1 && lane <= kTX && w >= 1 && w <= W - 2 && xs <= nx - 2 && ys <= ny - 2;
    const int rx = axis_role<kFeat>(P, 0, xs, nx);
    const int ry = axis_role<kFeat>(P, 1, ys, ny);
    const bool in_xy = rx != R_OUT && ry != R_OUT;
    const int ia = P.inout_axis;
    // the node's role, given the role of its plane
    auto role_of = [&](int rz) -> int {
        if (rx == R_OUT || ry == R_OUT || rz == R_OUT) return R_OUT;
        if ((kFeat & F_WALL) && (rx == R_WALL || ry == R_WALL || rz == R_WALL)) return R_WALL;
        if ((kFeat & F_INOUT) && (rx == R_GHOST || ry == R_GHOST || rz == R_GHOST)) return R_GHOST;
        return R_FLUID;
    };
    const int role_xy = role_of(R_FLUID); // on fluid planes
    // stochastic rounding of the 16-bit stores: key base of this step
    const unsigned key_base = sizeof(S) == 4 ? 0U : round_key_base(P.seed, step);
    // the inlet / outlet functors run at this column (x or y axis) or on planes 1 and nz-2 (z)
    const bool bc_xy = (kFeat & F_INOUT) && P.do_bc && (ia == 0 || ia == 1) &&
                       ((ia == 0 ? xs : ys) == 1 || (ia == 0 ? xs : ys) == (ia == 0 ? nx : ny) - 2);
    const bool bc_z = (kFeat & F_INOUT) && P.do_bc && ia == 2;
    // periodic images of this column's store (x = 1 / nx-2, y = 1 / ny-2 on a periodic axis)
    const int img_x = P.bc[0] == MBCG_BC_PERIODIC ? (xs == 1 ? nx - 1 : (xs == nx - 2 ? 0 : -1)) : -1;
    const int img_y = P.bc[1] == MBCG_BC_PERIODIC ? (ys == 1 ? ny - 1 : (ys == ny - 2 ? 0 : -1)) : -1;

    // psi fill: each thread owns <= kPsiPer ring elements; their mapping never changes along z.
    // Each element reads the staged box at the node whose stored value equals psi there (the
    // periodic ghost frame holds images), or, for the periodic images two layers out that the
    // box cannot hold, a global load issued one plane ahead into registers.
    constexpr int kPsiPer = (G::psi_plane + 32 * W - 1) / (32 * W);
    int psi_box[kPsiPer];      // box index, -1: prefetched global load, -2: no element
    long long psi_g[kPsiPer];  // mapped (x, y) offset in global memory
    float pf0[kPsiPer], pf1[kPsiPer];
#pragma unroll
    for (int j = 0; j < kPsiPer; ++j) {
        const int e = tid + j * 32 * W;
        psi_box[j] = -2;
        psi_g[j] = 0;
        pf0[j] = pf1[j] = 0.0f;
        if (e < G::psi_plane) {
            const int r = e / kPSX, c = e % kPSX;
            const int gx = xb - 1 + c, gy = yb - 1 + r;
            if (gx < -1 || gx > nx || gy < -1 || gy > ny) {
                // beyond the ghost frame and its one-node halo: read only by the colour gradient of
                // sources outside the lattice, whose populations reach no destination of the tile,
                // so any staged element serves (no global load)
                psi_box[j] = 0;
                continue;
            }
            const int mx = psi_coord(P, 0, gx, nx), my = psi_coord(P, 1, gy, ny);
            const bool px = P.bc[0] == MBCG_BC_PERIODIC, py = P.bc[1] == MBCG_BC_PERIODIC;
            const int dx = (px && gx >= 0 && gx <= nx - 1) ? gx : mx;
            const int dy = (py && gy >= 0 && gy <= ny - 1) ? gy : my;
            const int bc_ = dx - xr0, br_ = dy - (yb - 1);
            psi_box[j] = (bc_ >= 0 && bc_ < kRBX && br_ >= 0 && br_ < G::RBY) ? br_ * kRBX + bc_ : -1;
            psi_g[j] = static_cast<long long>(my) * P.pitch + mx;
        }
    }

    // periodic images two layers out are read from global memory; most tiles have none
    bool far_any = false;
#pragma unroll
    for (int j = 0; j < kPsiPer; ++j) far_any = far_any || psi_box[j] == -1;
    far_any = __syncthreads_or(far_any) != 0;

    // Plane k lives in stage slot (k - kfirst) mod 3, and its psi in the ring slot of the same
    // index; the z loop advances the slot incrementally.
    auto nxt = [](int sl) -> int { return sl == kNSTAGE - 1 ? 0 : sl + 1; };
    auto prv = [](int sl) -> int { return sl == 0 ? kNSTAGE - 1 : sl - 1; };
    auto stage_at = [&](int sl) -> unsigned char* { return smem + G::off_stage + sl * G::stage; };
    auto rb_box = [&](unsigned char* st, int f) -> S* { return reinterpret_cast<S*>(st + f * G::rb_field); };
    auto m_box = [&](unsigned char* st, int f) -> S* {
        return reinterpret_cast<S*>(st + 2 * G::rb_field + (f - 2) * G::m_field);
    };
    auto zload = [&](int k) -> int { return data_coord(P, 2, k, nz); };

    // ---- stage loader -------------------------------------------------------------
    auto issue = [&](int k, int sl) {
        unsigned char* st = stage_at(sl);
        const int kz = zload(k);
        if constexpr (kTMA) {
            if (tid == 0) {
                uint64_t* bar = &bars[sl];
                fence_proxy_async();
                mbar_expect_tx(bar, G::tx);
                tma_load_3d(rb_box(st, 0), &maps[0], xr0, yb - 1, kz, bar);
                tma_load_3d(rb_box(st, 1), &maps[1], xr0, yb - 1, kz, bar);
#pragma unroll
                for (int f = 2; f < NF; ++f) tma_load_3d(m_box(st, f), &maps[f], xm0, yb, kz, bar);
            }
        } else {
            // plain-load path for layouts TMA cannot describe (row pitch not 16-byte aligned)
            const long long zo = static_cast<long long>(kz) * P.plane;
            for (int e = tid; e < 2 * G::RBY * kRBX; e += 32 * W) {
                const int f = e / (G::RBY * kRBX), r = (e / kRBX) % G::RBY, c = e % kRBX;
                const int gx = xr0 + c, gy = yb - 1 + r;
                S v = Codec<S>::from_f(0.0f);
                if (gx >= 0 && gx < nx && gy >= 0 && gy < ny)
                    v = static_cast<const S*>(P.a[f])[zo + gy * P.pitch + gx];
                rb_box(st, f)[r * kRBX + c] = v;
            }
            for (int e = tid; e < 9 * G::MY * kMX; e += 32 * W) {
                const int f = 2 + e / (G::MY * kMX), r = (e / kMX) % G::MY, c = e % kMX;
                const int gx = xm0 + c, gy = yb + r;
                S v = Codec<S>::from_f(0.0f);
                if (gx >= 0 && gx < nx && gy >= 0 && gy < ny)
                    v = static_cast<const S*>(P.a[f])[zo + gy * P.pitch + gx];
                m_box(st, f)[r * kMX + c] = v;
            }
        }
    };
    constexpr long long kWaitLimit = 4000000000LL; // ~2 s at 2 GHz
    // Expected parity of the next phase of each slot's mbarrier; every completed wait flips it.
    // It starts from the parities the previous tile of this CTA left.
    uint32_t par = phase;
    int k_waited = kfirst - 1; // last plane whose load was waited for
    auto wait_slot = [&](int k, int sl) -> bool {
        if constexpr (kTMA) {
            const bool ok = mbar_wait_bounded(&bars[sl], (par >> sl) & 1u, kWaitLimit);
            if (ok) {
                par ^= 1u << sl;
                k_waited = k;
            }
            return ok;
        } else {
            k_waited = k;
            return true;
        }
    };
    // On a failed wait: flag it, drain the copies still in flight (bounded) and leave.  If the drain
    // gives up too, copies may still land in this block's shared memory after it exits, which the
    // status cannot tell apart (a flag for it cost the ten-body batch kernel 3-5 %): the host treats
    // any non-zero status as a poisoned context.
    auto bail = [&](int k_issued) {
        if (tid == 0 && P.status) atomicOr(P.status, 1);
        if constexpr (kTMA) {
            for (int k = k_waited + 1; k <= k_issued; ++k) {
                const int sl = (k - kfirst) % kNSTAGE;
                mbar_wait_bounded(&bars[sl], (par >> sl) & 1u, kWaitLimit / 4);
            }
        }
    };

    // ---- psi ring: psi = (rhor - rhob)/rho (mathUtilities.cuh:12-19) of plane k over
    // columns xb-1..xb+32 and rows yb-1..yb+W, colour-gradient neighbour rule applied
    auto prefetch_psi = [&](int mz) {
        const long long zo = static_cast<long long>(mz) * P.plane;
#pragma unroll
        for (int j = 0; j < kPsiPer; ++j)
            if (psi_box[j] == -1) {
                pf0[j] = Codec<S>::to_f(static_cast<const S*>(P.a[0])[zo + psi_g[j]]);
                pf1[j] = Codec<S>::to_f(static_cast<const S*>(P.a[1])[zo + psi_g[j]]);
            }
    };
    // mz: the plane the colour-gradient rule maps k to; plane_in_box: it is the staged plane
    auto fill_psi = [&](int mz, bool plane_in_box, int sl, bool prefetched) {
        float* ring = psi_ring + sl * G::psi_plane;
        if (plane_in_box && !far_any) {
            // every element of this tile is in the staged box (the first one of each thread
            // always exists: the ring plane has at least 32 W elements)
            unsigned char* st = stage_at(sl);
            const S* r0b = rb_box(st, 0);
            const S* r1b = rb_box(st, 1);
            ring[tid] = psi_of<S>(P, r0b[psi_box[0]], r1b[psi_box[0]]);
#pragma unroll
            for (int j = 1; j < kPsiPer; ++j)
                if (psi_box[j] >= 0) ring[tid + j * 32 * W] = psi_of<S>(P, r0b[psi_box[j]], r1b[psi_box[j]]);
            return;
        }
        const long long zo = static_cast<long long>(mz) * P.plane;
        unsigned char* st = stage_at(sl);
        const S* r0b = rb_box(st, 0);
        const S* r1b = rb_box(st, 1);
#pragma unroll
        for (int j = 0; j < kPsiPer; ++j) {
            if (psi_box[j] == -2) continue;
            float v;
            if (plane_in_box && psi_box[j] >= 0) {
                v = psi_of<S>(P, r0b[psi_box[j]], r1b[psi_box[j]]);
            } else if (prefetched && psi_box[j] == -1) {
                v = psi_of_slots<S>(pf0[j], pf1[j]);
            } else {
                const long long o = zo + psi_g[j];
                v = psi_of<S>(P, static_cast<const S*>(P.a[0])[o], static_cast<const S*>(P.a[1])[o]);
            }
            ring[tid + j * 32 * W] = v;
        }
    };

    // ---- set-up ------------------------------------------------------------------
    // every thread is done with the previous tile's shared memory before it is refilled
    __syncthreads();
    int k_issued = kfirst + kNSTAGE - 1;
    for (int k = kfirst; k <= k_issued; ++k) issue(k, k - kfirst);
    if constexpr (!kTMA) __syncthreads();
    {
        // The first wait.  Testing only (wait_test_cycles > 0): it waits on the barrier nothing
        // completes, with that limit, so it runs out and the tile takes the bail path with all its
        // planes in flight.  (Folded into the one wait: a second wait-and-bail path at the tile
        // start cost the ten-body batch kernel ~20 %.)
        bool ok = true;
        if constexpr (kTMA) {
            const bool test = P.wait_test_cycles > 0;
            ok = mbar_wait_bounded(test ? &bars[kNSTAGE] : &bars[0], test ? 0u : (par & 1u),
                                   test ? static_cast<long long>(P.wait_test_cycles) : kWaitLimit);
            if (ok) {
                par ^= 1u;
                k_waited = kfirst;
            }
        }
        ok = ok && wait_slot(kfirst + 1, 1);
        if (__syncthreads_or(!ok)) {
            bail(k_issued);
            return false;
        }
    }
    {
        const int m0 = psi_coord(P, 2, kfirst, nz), m1 = psi_coord(P, 2, kfirst + 1, nz);
        fill_psi(m0, m0 == zload(kfirst), 0, false);
        fill_psi(m1, m1 == zload(kfirst + 1), 1, false);
    }
    if (far_any) prefetch_psi(psi_coord(P, 2, kfirst + 2, nz));

    Acc accP, accC, accN; // destination planes k-1, k, k+1
    accP.zero();
    accC.zero();
    accN.zero();

    constexpr float cs2 = 1.0f / 3.0f;
    float4* xb_self = xbuf + w * 32 + lane; // (X0, XR, X1, X2) of one exported row

    int sl = 1; // slot of plane k (k starts at kfirst + 1)
    int k = zd0 - 1;
    // One plane of the z-march with the feature set kFB: the tile's own, or, on the steady-state
    // planes of an inlet/outlet z axis, the same set without the inlet/outlet parts.  Returns false
    // after a bail.
    auto plane = [&](auto featc) -> bool {
        constexpr int kFB = decltype(featc)::value;
        const int sl_next = nxt(sl), sl_prev = prv(sl);
        // (1) psi of plane k+1; one barrier both publishes the ring and makes the bail decision
        // uniform (a plane that never arrived leaves garbage in the ring, which nobody reads)
        // Plane coordinates: every mapping (staging, colour-gradient rule, node role) is the
        // identity while planes k .. k+3 are fluid planes, which is almost every plane.
        const bool zid = k >= 1 && k + kNSTAGE - 1 <= nz - 2;
        int mz1 = k + 1, mz2 = k + 2, rz = R_FLUID;
        bool inbox1 = true;
        if (!zid) {
            mz1 = psi_coord(P, 2, k + 1, nz);
            inbox1 = mz1 == zload(k + 1);
            mz2 = psi_coord(P, 2, k + 2, nz);
            rz = axis_role<kFB>(P, 2, k, nz);
        }
        {
            const bool ok = wait_slot(k + 1, sl_next);
            if (ok) fill_psi(mz1, inbox1, sl_next, true);
            if (__syncthreads_or(!ok)) {
                bail(k_issued);
                return false;
            }
        }
        if (far_any && k + 2 <= zd1 + 1) prefetch_psi(mz2);
        // (2) prefetch plane k+3 into the slot plane k-1 used
        if (k + kNSTAGE - 1 <= zd1 + 1 && k + kNSTAGE - 1 > k_issued) {
            issue(k + kNSTAGE - 1, sl_prev);
            k_issued = k + kNSTAGE - 1;
        }

        // (3) this thread's source node at plane k
        const int role = zid ? role_xy : role_of(rz);
        // Sources outside the lattice (lanes / rows past the last ghost layer) only ever stream
        // into nodes that are not destinations of this tile, so without walls every source is
        // processed branch-free; wall ghost layers hold data and must not emit.
        const bool active = ((kFB & F_WALL) == 0) || (role == R_FLUID || role == R_GHOST);

        unsigned char* st = stage_at(sl);
        Node<S> nd{};
        Node<S> fn{}; // first-fluid node of a ghost source (lbm.cuh:85-89)
        if (active) {
            float v[NF];
            v[0] = Codec<S>::to_f(rb_box(st, 0)[bR]);
            v[1] = Codec<S>::to_f(rb_box(st, 1)[bR]);
#pragma unroll
            for (int f = 2; f < NF; ++f) v[f] = Codec<S>::to_f(m_box(st, f)[bM]);
            decode<S>(P, v, nd);
            if constexpr ((kFB & F_INOUT) != 0) {
                if (role == R_GHOST) {
                    // the first fluid node behind the ghost: plane 1 or nz-2 (still staged: the
                    // slot of plane nz-2 is not refilled in the chunk that ends at nz-1), or the
                    // neighbouring column / row of the staged plane
                    const unsigned char* sf = st;
                    int b2 = bM;
                    if (rz == R_GHOST) {
                        sf = stage_at(k == 0 ? sl_next : sl_prev);
                    } else {
                        const int dx = (rx == R_GHOST) ? (xs == 0 ? 1 : -1) : 0;
                        const int dy = (ry == R_GHOST) ? (ys == 0 ? 1 : -1) : 0;
                        b2 = bM + dy * kMX + dx;
                    }
                    float u[NF];
#pragma unroll
                    for (int f = 2; f < NF; ++f)
                        u[f] = Codec<S>::to_f(reinterpret_cast<const S*>(sf + 2 * G::rb_field + (f - 2) * G::m_field)[b2]);
                    u[0] = u[1] = 1.0f;
                    decode<S>(P, u, fn);
                }
            }
        }

        // coefficient tensor and colour split; inactive sources keep all-zero coefficients
        Coef cf{};
        float aR = 0.0f, dcoef = 0.0f, Fx = 0.0f, Fy = 0.0f, Fz = 0.0f, omega2_rest = 0.0f;
        bool iface = false;
        if (active) {
            const float rho = nd.rr + nd.rb;
            const float inv = fast_rcp(rho);
            // colour fraction as a correctly rounded quotient (one residual correction): a
            // product with a rounded reciprocal is biased (aR rho - rr averages +2.5e-10 per
            // mixed node), which would move colour mass the same way every step
            const float q0 = nd.rr * inv;
            const float q1 = fmaf(fmaf(-q0, rho, nd.rr), inv, q0);
            aR = nd.rb == 0.0f ? 1.0f : (nd.rr == 0.0f ? 0.0f : q1);
            if (!(kFB & F_INOUT) || role == R_FLUID) {
                iface = (4.0f * nd.rr * nd.rb * inv * inv) > 1.0e-4f; // lbm.cuh:181,187
                // zero-filled staging outside the lattice decodes to a mixed node in the 16-bit
                // forms; keep those (never written) sources off the interface path
                if constexpr (sizeof(S) != 4) iface = iface && in_xy;
                build_coef<kFB>(P, cf, rho, nd.rr, nd.rb, nd.ux, nd.uy, nd.uz, nd.ux, nd.uy, nd.uz, nd.pxx, nd.pxy,
                                  nd.pyy, nd.pyz, nd.pzz, nd.pxz);
            } else {
                build_coef<kFB>(P, cf, rho, nd.rr, nd.rb, nd.ux, nd.uy, nd.uz, fn.ux, fn.uy, fn.uz, fn.pxx, fn.pxy,
                                  fn.pyy, fn.pyz, fn.pzz, fn.pxz);
            }
        }
        const bool any_iface = __any_sync(kFull, iface);
        if (any_iface && iface) {
            // colour gradient at the source (forces.cuh:20-60) from the psi ring
            const float* rm = psi_ring + sl_prev * G::psi_plane;
            const float* r0p = psi_ring + sl * G::psi_plane;
            const float* rp = psi_ring + sl_next * G::psi_plane;
            float sx = 0.0f, sy = 0.0f, sz = 0.0f;
#pragma unroll
            for (int dz = -1; dz <= 1; ++dz) {
                const float* ring = dz < 0 ? rm : (dz == 0 ? r0p : rp);
#pragma unroll
                for (int dy = -1; dy <= 1; ++dy) {
#pragma unroll
                    for (int dx = -1; dx <= 1; ++dx) {
                        if (dx == 0 && dy == 0 && dz == 0) continue;
                        if (!Stencil<Q>::has(dx, dy, dz)) continue;
                        const float ps = ring[(w + 1 + dy) * kPSX + lane + 1 + dx];
                        const float wp = weight<Q>(dx, dy, dz) * ps;
                        if (dx) sx += dx * wp;
                        if (dy) sy += dy * wp;
                        if (dz) sz += dz * wp;
                    }
                }
            }
            Fx = 3.0f * sx;
            Fy = 3.0f * sy;
            Fz = 3.0f * sz;
            const float absF = sqrtf(Fx * Fx + Fy * Fy + Fz * Fz);
            // Omega2 (collisionOperators.cuh:16-25) folded into the coefficients
            float Aeff = P.A; // A_calculation (forces.cuh:114-117) at the node's relaxation time
            if constexpr ((kFB & F_FORCE) != 0)
                if (P.tau_var) Aeff = P.s4 / tau_eff_of(P, nd.rr, nd.rb);
            float hA = (P.omega2_conservative && !(absF > 1.0e-4f)) ? 0.0f : 0.5f * Aeff * absF;
            if (absF > 1.0e-4f) {
                const float ia_ = fast_rcp(absF);
                const float qf = 0.5f * Aeff * ia_;
                // isotropic part from the same q |F|^2 as the anisotropic part, so Omega2 sums
                // to zero over the directions in floating point too
                hA = qf * (Fx * Fx + Fy * Fy + Fz * Fz);
                cf.p200 += qf * Fx * Fx;
                cf.p020 += qf * Fy * Fy;
                cf.p002 += qf * Fz * Fz;
                cf.p110 += 2.0f * qf * Fx * Fy;
                cf.p101 += 2.0f * qf * Fx * Fz;
                cf.p011 += 2.0f * qf * Fy * Fz;
                // recolouring (collisionOperators.cuh:60-80): beta rr rb / (rho^2 |F|) * feq0, where
                // the rest equilibrium of moving directions is w rho (w (rho + K) with a density ratio)
                const float rho = nd.rr + nd.rb;
                const float feq0 = ((kFB & F_FORCE) && P.ratio) ? rho + nd.rr * P.kappa_r + nd.rb * P.kappa_b : rho;
                const float irho = fast_rcp(rho);
                dcoef = P.beta * (nd.rr * nd.rb) * irho * irho * ia_ * feq0;
            }
            cf.p000 -= hA;
            omega2_rest = hA; // rest-population part, -hA (B0 - w0) = +2/3 hA, added below in exact units
        }
        const float rho_src = active ? nd.rr + nd.rb : 0.0f;
        const float rr_src = active ? nd.rr : 0.0f;
        // colour fractions of the x neighbours (lane -1 and lane +1)
        float2 aRlr;
        aRlr.x = __shfl_up_sync(kFull, aR, 1);
        aRlr.y = __shfl_down_sync(kFull, aR, 1);

        // separable inverse transform, x-pass: t_bc(cx) for the monomials cy^b cz^c
        const Tri t00 = tri(cf.p000 + cf.p200, cf.p100, cf.p000);
        const Tri t10 = tri(cf.p010 + cf.p210, cf.p110, cf.p010);
        const Tri t01 = tri(cf.p001 + cf.p201, cf.p101, cf.p001);
        const Tri t20 = tri(cf.p020, cf.p120, cf.p020);
        const Tri t02 = tri(cf.p002, cf.p102, cf.p002);
        const Tri t11 = tri(cf.p011, cf.p111, cf.p011);
        const float2 rho2 = pair(rho_src);
        // Populations are carried scaled by S = 216 (D3Q27) or 36 (D3Q19), where the weights
        // are small integers that sum to S exactly: float-rounded weights do not sum to 1, and
        // that error would scale every node's mass each step (about 1.5e-8 per step for D3Q19).
        // D3Q27 weights are also separable, S w(c) = prod over axes of (4 if c_a = 0 else 1):
        // populations are carried unweighted and the factors 4 are applied inside the forward
        // passes.  D3Q19 weights 12, 2, 1 are applied per population.  Each destination
        // divides its sums by S once, the mass sums with a correctly rounded quotient.
        constexpr bool kSepW = (Q == 27);
        const float dk1 = kSepW ? dcoef : 2.0f * dcoef;
        const float dk2 = dcoef * 0.7071067811865475f;
        const float dk3 = kSepW ? dcoef * 0.5773502691896258f : 0.0f;
        // rest-population correction (density-ratio K and the Omega2 rest term), with the Omega2
        // part in exact units so that Omega2 sums to zero over the directions (B0 - w0 = -2/3
        // for both lattices)
        // in value units before the rest weight (64 of 216, or 12 of 36): S r0 / W_0 and
        // S (w0 - B0) hA / W_0 = (2/3) S hA / W_0, i.e. 3.375 r0 + 2.25 hA or 3 r0 + 2 hA
        const float rc0 = kSepW ? fmaf(cf.r0, 3.375f, 2.25f * omega2_rest) : fmaf(cf.r0, 3.0f, 2.0f * omega2_rest);

        // wall bounce-back of this node's own populations (destination = this node, plane k)
        const bool wx0 = P.bc[0] == MBCG_BC_WALL && xs == 1, wx1 = P.bc[0] == MBCG_BC_WALL && xs == nx - 2;
        const bool wy0 = P.bc[1] == MBCG_BC_WALL && ys == 1, wy1 = P.bc[1] == MBCG_BC_WALL && ys == ny - 2;
        const bool wz0 = P.bc[2] == MBCG_BC_WALL && k == 1, wz1 = P.bc[2] == MBCG_BC_WALL && k == nz - 2;
        const bool reflect = (kFB & F_WALL) && role == R_FLUID && dest_thread && (wx0 | wx1 | wy0 | wy1 | wz0 | wz1);
        const bool any_reflect = (kFB & F_WALL) ? __any_sync(kFull, reflect) : false;

        // ---- emit: populations of the rows this warp exports, x streaming, own-row moments,
        // y exchange.  Halo rows export one population row (cy = +1 for warp 0, -1 for warp W-1).
        auto emit = [&](auto rowsc) {
            constexpr int ROWS = decltype(rowsc)::value;
            // y-pass per exported row j (cy = j - 1): s0 (cz^0), s1 (cz^1), e2 (cz^0 + cz^2)
            Tri s0[3], s1[3], e2[3];
            {
                const Tri e0 = t00 + t20;
                const Tri e1 = t01 + cf.p021;
                if (ROWS & 2) {
                    s0[1] = t00;
                    s1[1] = t01;
                    e2[1] = t00 + t02;
                }
                if (ROWS & 4) {
                    s0[2] = e0 + t10;
                    s1[2] = e1 + t11;
                    e2[2] = s0[2] + (t02 + cf.p012);
                }
                if (ROWS & 1) {
                    s0[0] = e0 - t10;
                    s1[0] = e1 - t11;
                    e2[0] = s0[0] + (t02 + (-cf.p012));
                }
            }
            auto do_class = [&](auto czc, Acc& acc) {
                constexpr int cz = decltype(czc)::value;
                // populations of row j: rho + the small part (rho last, see above); sm keeps the
                // small parts (value units, before the D3Q19 weight) for the red populations
                Tri g[3], sm[3];
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const int cy = j - 1;
                    g[j].o = sm[j].o = make_float2(0.0f, 0.0f);
                    g[j].c = sm[j].c = 0.0f;
                    if (!(ROWS & (1 << j))) continue;
                    Tri small = cz == 0 ? s0[j] : (cz > 0 ? e2[j] + s1[j] : e2[j] - s1[j]);
                    if (cy == 0 && cz == 0) small.c += rc0;
                    const int shc = cy * cy + cz * cz; // |c|^2 of the centre; the outer ones have shc + 1
                    if (Stencil<Q>::has(1, cy, cz)) {
                        sm[j].o = small.o;
                        const float2 vv = __fadd2_rn(rho2, small.o);
                        g[j].o = (kSepW || shc != 0) ? vv : __fadd2_rn(vv, vv);
                    }
                    if (Stencil<Q>::has(0, cy, cz)) {
                        sm[j].c = small.c;
                        const float vv = rho_src + small.c;
                        g[j].c = kSepW ? vv : (shc == 0 ? 12.0f * vv : (shc == 1 ? vv + vv : vv));
                    }
                }
                // recolouring part Delta_i of the red populations (interface sources only; the
                // red population is aR g_i + Delta_i, collisionOperators.cuh:60-80)
                auto delta = [&](int i, int j) -> float {
                    const int cx = i - 1, cy = j - 1, sh = cx * cx + cy * cy + cz * cz;
                    if (!(ROWS & (1 << j)) || !Stencil<Q>::has(cx, cy, cz) || sh == 0) return 0.0f;
                    const float dks = sh == 1 ? dk1 : (sh == 2 ? dk2 : dk3);
                    const float fc = (cx ? cx * Fx : 0.0f) + (cy ? cy * Fy : 0.0f) + (cz ? cz * Fz : 0.0f);
                    return dks * fc;
                };
                // Red population of direction (cx, cy, cz) = (i - 1, j - 1, cz) of a source with
                // density rho, red density rr, colour fraction aR = rr / rho, population
                // g = W (rho + sm) and recolouring part Delta.  On interface warps it is formed
                // as W (rr + aR sm) + Delta, which is aR g + Delta in exact arithmetic, but the
                // red populations of a source then sum to S rr + aR sum(W sm) (sm sums to zero)
                // whatever the rounding of aR, where aR g emits S aR rho: in a near-steady state
                // the quotient's rounding error repeats step after step and its sum over the
                // interface moved the 64^3 D3Q19 bubble's red mass by 7e-6 in 10^4 steps
                // (3.5e-7 with this form).  Elsewhere aR is within 2.5e-5 of 0 or 1 and the
                // populations are aR g.
                auto red_pop = [&](float rr_, float smv, float gv, float dl, int i, int j, bool withd) -> float {
                    if (!withd) return aR * gv;
                    const int cy = j - 1, shc = cy * cy + cz * cz + (i != 1 ? 1 : 0);
                    const float b = fmaf(aR, smv, rr_);
                    // D3Q19 weight of the population: 12 (rest), 2 (|c|^2 = 1), 1 (|c|^2 = 2)
                    if (kSepW || shc == 2) return b + dl;
                    if (shc == 1) return fmaf(2.0f, b, dl);
                    return fmaf(12.0f, b, dl);
                };
                if constexpr (ROWS == 7 && (kFB & F_WALL) != 0) {
                    if (any_reflect && reflect) {
#pragma unroll
                        for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int j = 0; j < 3; ++j) {
                                const int cx = i - 1, cy = j - 1;
                                if (!Stencil<Q>::has(cx, cy, cz)) continue;
                                const bool into = (wx0 && cx < 0) || (wx1 && cx > 0) || (wy0 && cy < 0) ||
                                                  (wy1 && cy > 0) || (wz0 && cz < 0) || (wz1 && cz > 0);
                                if (!into) continue;
                                const float f = kSepW ? static_cast<float>((cx == 0 ? 4 : 1) * (cy == 0 ? 4 : 1) *
                                                                           (cz == 0 ? 4 : 1))
                                                      : 1.0f;
                                const float gv = i == 0 ? g[j].o.x : (i == 2 ? g[j].o.y : g[j].c);
                                const float smv = i == 0 ? sm[j].o.x : (i == 2 ? sm[j].o.y : sm[j].c);
                                const float rr_ = red_pop(rr_src, smv, gv, any_iface ? delta(i, j) : 0.0f, i, j, any_iface);
                                add_pop(accC, f * gv, f * rr_, -cx, -cy, -cz);
                            }
                    }
                }
                // x streaming: destination x receives cx=+1 from lane-1 and cx=-1 from lane+1.
                // The populations cross lanes; on interface warps the source forms its red
                // populations (red_pop) and they cross too, elsewhere the destination forms them
                // as aR g from the source's colour fraction (shuffled once per plane).
                float X0[3], X1[3], X2[3], XR[3];
                auto xstream = [&](auto ifc) {
                    constexpr bool kIf = decltype(ifc)::value;
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        const int cy = j - 1;
                        X0[j] = X1[j] = X2[j] = XR[j] = 0.0f;
                        if (!(ROWS & (1 << j))) continue;
                        const float r1 = red_pop(rr_src, sm[j].c, g[j].c, kIf ? delta(1, j) : 0.0f, 1, j, kIf);
                        if (Stencil<Q>::has(1, cy, cz)) {
                            float2 glr; // (from lane - 1, from lane + 1)
                            glr.x = __shfl_up_sync(kFull, g[j].o.y, 1);
                            glr.y = __shfl_down_sync(kFull, g[j].o.x, 1);
                            X2[j] = glr.x + glr.y;
                            X0[j] = kSepW ? fmaf(4.0f, g[j].c, X2[j]) : X2[j] + g[j].c;
                            X1[j] = glr.x - glr.y;
                            float2 rlr;
                            if constexpr (kIf) {
                                // red_pop of this lane's cx = -1 / +1 populations, paired
                                const bool w2 = !kSepW && cy == 0 && cz == 0; // D3Q19 weight 2
                                float2 ro = __ffma2_rn(pair(aR), sm[j].o, pair(rr_src));
                                const float2 dl = make_float2(delta(0, j), delta(2, j));
                                ro = w2 ? __ffma2_rn(pair(2.0f), ro, dl) : __fadd2_rn(ro, dl);
                                rlr.x = __shfl_up_sync(kFull, ro.y, 1);
                                rlr.y = __shfl_down_sync(kFull, ro.x, 1);
                            } else {
                                rlr = __fmul2_rn(aRlr, glr);
                            }
                            XR[j] = kSepW ? fmaf(4.0f, r1, rlr.x + rlr.y) : (rlr.x + rlr.y) + r1;
                        } else {
                            X0[j] = g[j].c;
                            XR[j] = r1;
                        }
                    }
                };
                if (any_iface) xstream(std::true_type{});
                else xstream(std::false_type{});
                if constexpr ((ROWS & 2) != 0) {
                    // cy = 0 row stays in this column: add to the destination's sums now.  Plane
                    // k+1 (cz = +1) receives its first contributions here: they are assigned, so
                    // its sums need no clearing.
                    constexpr int fi = kSepW ? (cz == 0 ? 16 : 4) : 1;
                    constexpr float f = static_cast<float>(fi);
                    if constexpr (cz == 1) {
                        acc.rr = fi == 1 ? make_float2(X0[1], XR[1]) : __fmul2_rn(pair(f), make_float2(X0[1], XR[1]));
                        acc.jxx = fi == 1 ? make_float2(X1[1], X2[1]) : __fmul2_rn(pair(f), make_float2(X1[1], X2[1]));
                        acc.jz = f * X0[1];
                        acc.xz = f * X1[1];
                        acc.zz = f * X0[1];
                    } else {
                        acc.rr = acc2<fi>(acc.rr, make_float2(X0[1], XR[1]));
                        acc.jxx = acc2<fi>(acc.jxx, make_float2(X1[1], X2[1]));
                        if (cz != 0) {
                            acc.jz = fmaf(cz * f, X0[1], acc.jz);
                            acc.xz = fmaf(cz * f, X1[1], acc.xz);
                            acc.zz = fmaf(f, X0[1], acc.zz);
                        }
                    }
                }
                // cy = +1 goes to row w+1 (slot 0), cy = -1 to row w-1 (slot 1)
                constexpr int cls = cz + 1;
                if constexpr ((ROWS & 4) != 0) {
                    xb_self[(cls * 2 + 0) * (W * 32)] = make_float4(X0[2], XR[2], X1[2], X2[2]);
                }
                if constexpr ((ROWS & 1) != 0) {
                    xb_self[(cls * 2 + 1) * (W * 32)] = make_float4(X0[0], XR[0], X1[0], X2[0]);
                }
            };
            do_class(std::integral_constant<int, -1>{}, accP);
            do_class(std::integral_constant<int, 0>{}, accC);
            do_class(std::integral_constant<int, 1>{}, accN);
        };
        if (w == 0) emit(std::integral_constant<int, 4>{});
        else if (w == W - 1) emit(std::integral_constant<int, 1>{});
        else emit(std::integral_constant<int, 7>{});
        __syncthreads();

        // (4) y streaming into destination rows
        auto gather = [&](auto czc, Acc& acc) {
            constexpr int cz = decltype(czc)::value;
            constexpr int cls = cz + 1;
            constexpr int fi = (kSepW && cz == 0) ? 4 : 1;
            constexpr float f = static_cast<float>(fi);
            const float4 pv = xb_self[(cls * 2 + 0) * (W * 32) - 32]; // row w-1 exported cy = +1
            const float4 mv = xb_self[(cls * 2 + 1) * (W * 32) + 32]; // row w+1 exported cy = -1
            // slots (X0, XR, X1, X2)
            const float2 s0r = __fadd2_rn(make_float2(pv.x, pv.y), make_float2(mv.x, mv.y)); // (s00, red)
            const float2 s12 = __fadd2_rn(make_float2(pv.z, pv.w), make_float2(mv.z, mv.w)); // (s10, s20)
            const float d00 = pv.x - mv.x;
            acc.rr = acc2<fi>(acc.rr, s0r);
            acc.jxx = acc2<fi>(acc.jxx, s12);
            if constexpr (cz == 1) {
                // first contributions to jy, xy, yy, yz of plane k+1 (f = 1)
                acc.jy = d00;
                acc.xy = pv.z - mv.z;
                acc.yy = s0r.x;
                acc.yz = d00;
            } else {
                acc.jy = fmaf(f, d00, acc.jy);
                acc.xy = fmaf(f, pv.z - mv.z, acc.xy);
                acc.yy = fmaf(f, s0r.x, acc.yy);
                if (cz != 0) acc.yz += cz * d00;
            }
            if (cz != 0) {
                acc.jz += cz * s0r.x;
                acc.xz += cz * s12.x;
                acc.zz += s0r.x;
            }
        };
        const bool dest_row = (w >= 1 && w <= W - 2);
        if (dest_row) gather(std::integral_constant<int, -1>{}, accP);

        // (5) destination plane k-1 is complete: moments (lbm.cuh:239-261), store, boundary
        const int d = k - 1;
        if (dest_thread && d >= zd0 && d < zd1) {
            {
                constexpr float kS = kSepW ? 216.0f : 36.0f;
                constexpr float sc = 1.0f / kS;
                // correctly rounded mass quotients (no systematic bias), plain scaling for the rest
                const float2 q = __fmul2_rn(accP.rr, pair(sc));
                const float2 e = __ffma2_rn(make_float2(-q.x, -q.y), pair(kS), accP.rr);
                accP.rr = __ffma2_rn(e, pair(sc), q);
                // xx stays a scalar here: xx sc - rho/3 below then contracts to one fma, which
                // keeps Pi's bits through the cancellation
                accP.jxx.x *= sc; accP.jxx.y *= sc;
                accP.jy *= sc; accP.jz *= sc;
                accP.xy *= sc; accP.yy *= sc; accP.yz *= sc; accP.zz *= sc; accP.xz *= sc;
            }
            const float rho = accP.rr.x;
            const float rr = accP.rr.y;
            const float rb = rho - rr;
            const float inv = fast_rcp(rho);
            float Fbx = 0.0f, Fby = 0.0f, Fbz = 0.0f;
            constexpr bool kF = (kFB & F_FORCE) != 0;
            if (kF && P.forced) {
                Fbx = rho * P.g[0];
                Fby = rho * P.g[1];
                Fbz = rho * P.g[2];
            }
            const float ux = (accP.jxx.x + 0.5f * Fbx) * inv;
            const float uy = (accP.jy + 0.5f * Fby) * inv;
            const float uz = (accP.jz + 0.5f * Fbz) * inv;
            const float ctr = cs2 * rho;
            float pi[6];
            pi[0] = (accP.jxx.y - ctr) - rho * ux * ux;
            pi[1] = accP.xy - rho * ux * uy;
            pi[2] = (accP.yy - ctr) - rho * uy * uy;
            pi[3] = accP.yz - rho * uy * uz;
            pi[4] = (accP.zz - ctr) - rho * uz * uz;
            pi[5] = accP.xz - rho * ux * uz;
            if (kF && P.forced) {
                pi[0] += ux * Fbx;
                pi[1] += 0.5f * (ux * Fby + uy * Fbx);
                pi[2] += uy * Fby;
                pi[3] += 0.5f * (uy * Fbz + uz * Fby);
                pi[4] += uz * Fbz;
                pi[5] += 0.5f * (ux * Fbz + uz * Fbx);
            }
            if (kF && P.ratio) {
                const float Kc = (rr * P.kappa_r + rb * P.kappa_b) * cs2;
                pi[0] -= Kc;
                pi[2] -= Kc;
                pi[4] -= Kc;
            }
            finalize_store<S>(P, xs, ys, d, rr, rb, ux, uy, uz, pi, img_x, img_y, key_base);

            if ((kFB & F_INOUT) && (bc_xy || (bc_z && (d == 1 || d == nz - 2)))) {
                // inlet / outlet functors fused into the first and last fluid layer
                const int pa = ia == 0 ? xs : (ia == 1 ? ys : d);
                {
                    const bool inlet = pa == 1;
                    const int gx = ia == 0 ? (inlet ? 0 : nx - 1) : xs;
                    const int gy = ia == 1 ? (inlet ? 0 : ny - 1) : ys;
                    const int gz = ia == 2 ? (inlet ? 0 : nz - 1) : d;
                    const long long og = static_cast<long long>(gz) * P.plane + static_cast<long long>(gy) * P.pitch + gx;
                    float orr, orb, oux, ouy, ouz;
                    if (inlet) {
                        // jet/boundary_conditions.cuh:16-39 (+ seeded per-node noise)
                        const int t0 = ia == 0 ? ys : xs;
                        const int t1 = ia == 2 ? ys : d;
                        const float du = static_cast<float>(t0) - P.jet_c0;
                        const float dv = static_cast<float>(t1) - P.jet_c1;
                        const float m = (du * du + dv * dv) <= (P.jet_radius * P.jet_radius) ? 1.0f : 0.0f;
                        orr = P.jet_blue ? (1.0f - m) * P.rho_r0 : m * P.rho_r0;
                        orb = P.jet_blue ? m * P.rho_b0 : (1.0f - m) * P.rho_b0;
                        float gu[3] = {0.0f, 0.0f, 0.0f};
                        if (m != 0.0f) {
                            if (P.noise_amp != 0.0f) {
                                const unsigned long long node = static_cast<unsigned long long>(gx) +
                                                                static_cast<unsigned long long>(gy) * nx +
                                                                static_cast<unsigned long long>(gz) * nx * ny;
                                gu[0] = m * P.noise_amp * noise_xi(P.seed, step, node, 0);
                                gu[1] = m * P.noise_amp * noise_xi(P.seed, step, node, 1);
                                gu[2] = m * P.noise_amp * noise_xi(P.seed, step, node, 2);
                            }
                        }
                        oux = gu[0] + (ia == 0 ? m * P.jet_velocity : 0.0f);
                        ouy = gu[1] + (ia == 1 ? m * P.jet_velocity : 0.0f);
                        ouz = gu[2] + (ia == 2 ? m * P.jet_velocity : 0.0f);
                    } else if (P.outlet == MBCG_OUTLET_ZERO_GRADIENT) {
                        orr = rr; orb = rb; oux = ux; ouy = uy; ouz = uz;
                    } else {
                        // convective outlet (jet/boundary_conditions.cuh:45-109), old ghost from A
                        float ov[NF];
                        if (ia == 2) {
                            ov[0] = Codec<S>::to_f(rb_box(st, 0)[bR]);
                            ov[1] = Codec<S>::to_f(rb_box(st, 1)[bR]);
#pragma unroll
                            for (int f = 2; f < NF; ++f) ov[f] = Codec<S>::to_f(m_box(st, f)[bM]);
                        } else {
                            load_global<S>(P, og, ov);
                        }
                        Node<S> on{};
                        decode<S>(P, ov, on);
                        const float ua = ia == 0 ? ux : (ia == 1 ? uy : uz);
                        const float uc = fminf(fmaxf(ua, 0.0f), 1.0f);
                        if (on.rr + on.rb <= 1.0e-20f) {
                            orr = rr; orb = rb; oux = ux; ouy = uy; ouz = uz;
                        } else {
                            orr = on.rr - uc * (on.rr - rr);
                            orb = on.rb - uc * (on.rb - rb);
                            oux = on.ux - uc * (on.ux - ux);
                            ouy = on.uy - uc * (on.uy - uy);
                            ouz = on.uz - uc * (on.uz - uz);
                        }
                    }
                    const int gix = P.bc[0] == MBCG_BC_PERIODIC ? (gx == 1 ? nx - 1 : (gx == nx - 2 ? 0 : -1)) : -1;
                    const int giy = P.bc[1] == MBCG_BC_PERIODIC ? (gy == 1 ? ny - 1 : (gy == ny - 2 ? 0 : -1)) : -1;
                    finalize_store<S>(P, gx, gy, gz, orr, orb, oux, ouy, ouz, pi, gix, giy, key_base);
                }
            }
        }
        if (dest_row) {
            gather(std::integral_constant<int, 0>{}, accC);
            gather(std::integral_constant<int, 1>{}, accN);
        }
        accP = accC;
        accC = accN; // accN is assigned before it is added to again
            return true;
    };
    auto run = [&](auto featc, int kend) -> bool {
        for (; k <= kend; ++k, sl = nxt(sl))
            if (!plane(featc)) return false;
        return true;
    };
    if constexpr ((kFeat & (F_INOUT | F_WALL)) != 0 && kLeanZ) {
        // The inlet/outlet or wall axis along z: planes 3 (walls: 2) .. nz-5 need none of its parts
        // (fluid sources with identity mappings, no wall-adjacent source, no functor store).
        const bool zin = ia == 2, zwall = P.bc[2] == MBCG_BC_WALL;
        if (zin || zwall) {
            const int k0 = max(zd0 - 1, zin ? 3 : 2), k1 = min(zd1, nz - 5);
            if (k1 >= k0) {
                if (!run(std::integral_constant<int, kFeat>{}, k0 - 1)) return false;
                if (!run(std::integral_constant<int, kFeat & ~(F_INOUT | F_WALL)>{}, k1)) return false;
            }
        }
    }
    if (!run(std::integral_constant<int, kFeat>{}, zd1)) return false;
    // every load of this tile was waited for: carry the parities over to the next tile
    phase = par;
    return true;
}

// ------------------------------------------------------------------ plain step kernel
// One tile per CTA over the grid ((nx-2)/30, (ny-2)/(W-2), (nz-2)/zchunk), rounded up.
template <int Q, typename S, int W, bool kTMA, int kFeat>
__global__ void __launch_bounds__(32 * W, W <= 8 ? 2 : 1) step_kernel(const __grid_constant__ StepParams P,
                                                                      const __grid_constant__ TensorMaps T) {
    unsigned char* smem = aligned_smem_base();
    if constexpr (kTMA) init_stage_barriers(smem);
    uint32_t phase = 0;
    step_tile<Q, S, W, kTMA, kFeat>(P, T.m, blockIdx.x, blockIdx.y, blockIdx.z, P.step, smem, phase);
}

// Opt a kernel into its dynamic shared memory once per device; `done` is the kernel's own
// per-device bit set.
template <typename K>
cudaError_t configure_once(K kern, int smem, std::atomic<unsigned long long>& done) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_acq_rel);
    return e;
}

template <int Q, typename S, int W, bool kTMA, int kFeat>
cudaError_t launch_one(const StepParams& P, const TensorMaps& T, cudaStream_t s) {
    using G = Geo<S, W>;
    auto kern = step_kernel<Q, S, W, kTMA, kFeat>;
    static std::atomic<unsigned long long> configured{0};
    if (cudaError_t e = configure_once(kern, G::smem, configured)) return e;
    dim3 block(32, W, 1);
    dim3 grid((P.nx - 2 + kTX - 1) / kTX, (P.ny - 2 + W - 3) / (W - 2), (P.nz - 2 + P.zchunk - 1) / P.zchunk);
    kern<<<grid, block, G::smem, s>>>(P, T);
    return cudaGetLastError();
}

// Feature set: the smallest instantiation covering the lattice (TMA path); the plain-load
// path, for layouts TMA cannot describe, carries every feature.
template <int Q, typename S, int W>
cudaError_t launch_w(bool tma, const StepParams& P, const TensorMaps& T, cudaStream_t s) {
    if (!tma) return launch_one<Q, S, W, false, F_ALL>(P, T, s);
    if (std::getenv("MBCG_ALL_FEATURES")) return launch_one<Q, S, W, true, F_ALL>(P, T, s); // (parity tests)
    const int f = features_of(P);
    if (f == 0) return launch_one<Q, S, W, true, 0>(P, T, s);
    if (f == F_INOUT) return launch_one<Q, S, W, true, F_INOUT>(P, T, s);
    if ((f & F_INOUT) == 0) return launch_one<Q, S, W, true, F_WALL | F_FORCE>(P, T, s); // walls, force
    return launch_one<Q, S, W, true, F_ALL>(P, T, s);
}

template <int Q, typename S>
cudaError_t launch_qs(bool tma, int w, const StepParams& P, const TensorMaps& T, cudaStream_t s) {
    if (w == 8) return launch_w<Q, S, 8>(tma, P, T, s);
    return launch_w<Q, S, 16>(tma, P, T, s);
}

} // namespace

} // namespace mbcg
