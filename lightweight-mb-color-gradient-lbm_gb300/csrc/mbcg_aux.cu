// mbcg_aux.cu -- the small kernels around the fused step: the standalone inlet/outlet pass
// (the reference's split launch_JetBoundaryConditions), the case initial conditions, the
// FP64 conservation / Laplace diagnostics and the dense-layout conversions used by
// copy-in / copy-out.  None of these is on the per-step hot path of mbcg_step().
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mbcg_internal.h"

namespace mbcg {

namespace {

template <typename S>
__device__ __forceinline__ void load_node(const StepParams& P, const void* const* f, long long o, float (&v)[NF]) {
#pragma unroll
    for (int i = 0; i < NF; ++i) v[i] = Codec<S>::to_f(static_cast<const S*>(f[i])[o]);
}

// stored slots -> reference moments (rhor, rhob, u, Pi)
template <typename S>
__device__ __forceinline__ void to_moments(const StepParams& P, float (&v)[NF]) {
    if constexpr (sizeof(S) != 4) {
        const float phi = phi_of_slot(v[1]);
        const float rho = P.rho_mean + phi * P.rho_half_diff + P.rho_scale * v[0];
        colour_split(v[1], rho, v[0], v[1]);
        for (int i = 2; i < 5; ++i) v[i] *= P.u_ref;
        for (int i = 5; i < NF; ++i) v[i] *= P.pi_scale;
    }
}

// reference moments -> stored slots
template <typename S>
__device__ __forceinline__ void store_moments(const StepParams& P, void* const* f, long long o, const float (&m)[NF]) {
    if constexpr (sizeof(S) == 4) {
#pragma unroll
        for (int i = 0; i < NF; ++i) static_cast<float*>(f[i])[o] = m[i];
    } else {
        const float rho = m[0] + m[1];
        const S c = Codec<S>::from_f(colour_slot(m[0], m[1], rho));
        const float phi = phi_of_slot(Codec<S>::to_f(c)); // the phi a reader decodes
        static_cast<S*>(f[0])[o] = Codec<S>::from_f((rho - (P.rho_mean + phi * P.rho_half_diff)) * P.inv_rho_scale);
        static_cast<S*>(f[1])[o] = c;
        for (int i = 2; i < 5; ++i) static_cast<S*>(f[i])[o] = Codec<S>::from_f(m[i] * P.inv_u_ref);
        for (int i = 5; i < NF; ++i) static_cast<S*>(f[i])[o] = Codec<S>::from_f(m[i] * P.inv_pi_scale);
    }
}

__device__ __forceinline__ long long lin(const StepParams& P, int x, int y, int z) {
    return static_cast<long long>(z) * P.plane + static_cast<long long>(y) * P.pitch + x;
}

// store reference moments at (x, y, z) and, on periodic x / y axes, at the ghost-layer image
// of a first / last fluid layer (the step kernel reads wrapped sources from the ghost frame)
template <typename S>
__device__ __forceinline__ void store_with_images(const StepParams& P, int x, int y, int z, const float (&m)[NF]);

__device__ __forceinline__ void transverse(int a, int& t0, int& t1) {
    t0 = a == 0 ? 1 : 0;
    t1 = a == 2 ? 1 : 2;
}

// isJet (utilities/mathUtilities.cuh:39-45), no fused multiply-adds so the mask matches the
// reference's float arithmetic exactly
__device__ __forceinline__ float jet_mask(const StepParams& P, int u, int v) {
    const float du = __fsub_rn(static_cast<float>(u), P.jet_c0);
    const float dv = __fsub_rn(static_cast<float>(v), P.jet_c1);
    return __fadd_rn(__fmul_rn(du, du), __fmul_rn(dv, dv)) <= __fmul_rn(P.jet_radius, P.jet_radius) ? 1.0f : 0.0f;
}

template <typename S>
__device__ __forceinline__ void store_with_images(const StepParams& P, int x, int y, int z, const float (&m)[NF]) {
    store_moments<S>(P, P.b, lin(P, x, y, z), m);
    if (!P.ghost_images) return;
    const int ix = P.bc[0] == MBCG_BC_PERIODIC ? (x == 1 ? P.nx - 1 : (x == P.nx - 2 ? 0 : -1)) : -1;
    const int iy = P.bc[1] == MBCG_BC_PERIODIC ? (y == 1 ? P.ny - 1 : (y == P.ny - 2 ? 0 : -1)) : -1;
    if (ix >= 0) store_moments<S>(P, P.b, lin(P, ix, y, z), m);
    if (iy >= 0) store_moments<S>(P, P.b, lin(P, x, iy, z), m);
    if (ix >= 0 && iy >= 0) store_moments<S>(P, P.b, lin(P, ix, iy, z), m);
}

// Fill the ghost frame of periodic x (axis 0) or y (axis 1) with the images of the opposite
// fluid layer, on the state P.b: x first over every row, then y over every column, so the
// corners hold the doubly wrapped node.
template <typename S>
__global__ void fill_ghosts_kernel(const StepParams P, int axis) {
    const int n = axis == 0 ? P.nx : P.ny;
    const int m = axis == 0 ? P.ny : P.nx; // the other in-plane axis, full extent
    const long long total = static_cast<long long>(m) * P.nz * 2;
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int side = static_cast<int>(e & 1);
        const long long r = e >> 1;
        const int t = static_cast<int>(r % m);
        const int z = static_cast<int>(r / m);
        const int dst = side == 0 ? 0 : n - 1;
        const int src = side == 0 ? n - 2 : 1;
        const long long od = axis == 0 ? lin(P, dst, t, z) : lin(P, t, dst, z);
        const long long os = axis == 0 ? lin(P, src, t, z) : lin(P, t, src, z);
        for (int f = 0; f < NF; ++f) static_cast<S*>(P.b[f])[od] = static_cast<const S*>(P.b[f])[os];
    }
}

// ---------------------------------------------------------------- inlet / outlet functors
// kernels.cu:102-114 on B with the old state Aold (P.a = Aold, P.b = B); jet/
// boundary_conditions.cuh:16-109.  noise: apply the per-step inlet perturbation.
template <typename S>
__global__ void bc_kernel(const StepParams P, int init_inlet) {
    const int a = P.inout_axis;
    int t0, t1;
    transverse(a, t0, t1);
    const int n3[3] = {P.nx, P.ny, P.nz};
    const int n0 = n3[t0] - 2, n1 = n3[t1] - 2;
    const long long total = static_cast<long long>(n0) * n1;
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int u = 1 + static_cast<int>(e % n0), v = 1 + static_cast<int>(e / n0);
        int pb[3], pf[3];
        pb[t0] = pf[t0] = u;
        pb[t1] = pf[t1] = v;
        // inlet
        pb[a] = 0;
        pf[a] = 1;
        {
            const long long ob = lin(P, pb[0], pb[1], pb[2]), of = lin(P, pf[0], pf[1], pf[2]);
            float fv[NF];
            load_node<S>(P, P.b, of, fv);
            to_moments<S>(P, fv);
            const float m = jet_mask(P, u, v);
            float g[NF];
            g[0] = P.jet_blue ? (1.0f - m) * P.rho_r0 : m * P.rho_r0;
            g[1] = P.jet_blue ? m * P.rho_b0 : (1.0f - m) * P.rho_b0;
            g[2] = g[3] = g[4] = 0.0f;
            g[2 + a] = m * P.jet_velocity;
            if (!init_inlet && P.noise_amp != 0.0f && m != 0.0f) {
                const unsigned long long node = static_cast<unsigned long long>(pb[0]) +
                                                static_cast<unsigned long long>(pb[1]) * P.nx +
                                                static_cast<unsigned long long>(pb[2]) * P.nx * P.ny;
                for (int c = 0; c < 3; ++c) g[2 + c] += m * P.noise_amp * noise_xi(P.seed, P.step, node, c);
            }
            for (int i = 5; i < NF; ++i) g[i] = init_inlet ? 0.0f : fv[i];
            store_with_images<S>(P, pb[0], pb[1], pb[2], g);
        }
        if (init_inlet) continue;
        // outlet
        pb[a] = n3[a] - 1;
        pf[a] = n3[a] - 2;
        {
            const long long ob = lin(P, pb[0], pb[1], pb[2]), of = lin(P, pf[0], pf[1], pf[2]);
            float fv[NF];
            load_node<S>(P, P.b, of, fv);
            to_moments<S>(P, fv);
            float g[NF];
            if (P.outlet == MBCG_OUTLET_ZERO_GRADIENT) {
                for (int i = 0; i < NF; ++i) g[i] = fv[i];
            } else {
                float ov[NF];
                load_node<S>(P, P.a, ob, ov);
                to_moments<S>(P, ov);
                const float uc = fminf(fmaxf(fv[2 + a], 0.0f), 1.0f);
                if (ov[0] + ov[1] <= 1.0e-20f) {
                    for (int i = 0; i < 5; ++i) g[i] = fv[i];
                } else {
                    for (int i = 0; i < 5; ++i) g[i] = ov[i] - uc * (ov[i] - fv[i]);
                }
                for (int i = 5; i < NF; ++i) g[i] = fv[i];
            }
            store_with_images<S>(P, pb[0], pb[1], pb[2], g);
        }
    }
}

// ---------------------------------------------------------------- initial conditions
struct ICParams {
    int kind;
    int h;         // rti interface-normal axis
    float bc0, bc1, bc2, brad, bwidth, bphase;
    float rpos, ramp, rwidth, rphase, rk0, rk1;
};

template <typename S>
__global__ void init_kernel(const StepParams P, const ICParams I) {
    const long long total = static_cast<long long>(P.nx) * P.ny * P.nz;
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int x = static_cast<int>(e % P.nx);
        const int y = static_cast<int>((e / P.nx) % P.ny);
        const int z = static_cast<int>(e / (static_cast<long long>(P.nx) * P.ny));
        const long long o = lin(P, x, y, z);
        float m[NF];
        for (int i = 0; i < NF; ++i) m[i] = 0.0f;
        if (I.kind == MBCG_IC_JET) {
            // jet/jetIn.cuh:16-33: ambient fluid at rest everywhere
            if (P.jet_blue) m[0] = P.rho_r0;
            else m[1] = P.rho_b0;
        } else if (I.kind == MBCG_IC_BUBBLE) {
            // bubble/bubbleIn.cuh:15-52, fluid nodes only
            if (x == 0 || y == 0 || z == 0 || x == P.nx - 1 || y == P.ny - 1 || z == P.nz - 1) continue;
            const float dx = __fsub_rn(static_cast<float>(x), I.bc0);
            const float dy = __fsub_rn(static_cast<float>(y), I.bc1);
            const float dz = __fsub_rn(static_cast<float>(z), I.bc2);
            const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            if (I.bwidth <= 0.0f) {
                const float in = r2 <= __fmul_rn(I.brad, I.brad) ? 1.0f : 0.0f;
                if (I.bphase < 0.0f) {
                    m[0] = (1.0f - in) * P.rho_r0;
                    m[1] = in * P.rho_b0;
                } else {
                    m[0] = in * P.rho_r0;
                    m[1] = (1.0f - in) * P.rho_b0;
                }
            } else {
                const float ps = I.bphase * tanhf((I.brad - sqrtf(r2)) / I.bwidth);
                m[0] = 0.5f * (1.0f + ps) * P.rho_r0;
                m[1] = 0.5f * (1.0f - ps) * P.rho_b0;
            }
        } else if (I.kind == MBCG_IC_RTI) {
            // rti/rtiIn.cuh:18-70
            const int c3[3] = {x, y, z};
            int t0, t1;
            transverse(I.h, t0, t1);
            const float pos = __fadd_rn(I.rpos, __fmul_rn(__fmul_rn(I.ramp, cosf(__fmul_rn(I.rk0, static_cast<float>(c3[t0])))),
                                                          cosf(__fmul_rn(I.rk1, static_cast<float>(c3[t1])))));
            const float phi = tanhf(__fdiv_rn(__fsub_rn(static_cast<float>(c3[I.h]), pos), I.rwidth));
            if (I.rphase < 0.0f) {
                m[0] = 0.5f * (1.0f - phi) * P.rho_r0;
                m[1] = 0.5f * (1.0f + phi) * P.rho_b0;
            } else {
                m[0] = 0.5f * (1.0f + phi) * P.rho_r0;
                m[1] = 0.5f * (1.0f - phi) * P.rho_b0;
            }
        } else {
            continue;
        }
        store_moments<S>(P, P.b, o, m);
    }
}

// rtiIn.cuh:76-119: the interface-normal ghost layers copy their neighbour, u = 0
template <typename S>
__global__ void rti_walls_kernel(const StepParams P, int h) {
    int t0, t1;
    transverse(h, t0, t1);
    const int n3[3] = {P.nx, P.ny, P.nz};
    const int n0 = n3[t0] - 2, n1 = n3[t1] - 2;
    const long long total = static_cast<long long>(n0) * n1;
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int u = 1 + static_cast<int>(e % n0), v = 1 + static_cast<int>(e / n0);
        for (int side = 0; side < 2; ++side) {
            int pb[3], pf[3];
            pb[t0] = pf[t0] = u;
            pb[t1] = pf[t1] = v;
            pb[h] = side == 0 ? 0 : n3[h] - 1;
            pf[h] = side == 0 ? 1 : n3[h] - 2;
            float fv[NF];
            load_node<S>(P, P.b, lin(P, pf[0], pf[1], pf[2]), fv);
            to_moments<S>(P, fv);
            fv[2] = fv[3] = fv[4] = 0.0f;
            store_moments<S>(P, P.b, lin(P, pb[0], pb[1], pb[2]), fv);
        }
    }
}

// ---------------------------------------------------------------- diagnostics
struct DiagParams {
    int bubble;
    float c0, c1, c2, r_in2, r_out2;
    float kappa_r, kappa_b;
};

template <typename S>
__global__ void diag_kernel(const StepParams P, const DiagParams D, double* partials) {
    const long long n0 = P.nx - 2, n1 = P.ny - 2, n2 = P.nz - 2;
    const long long total = n0 * n1 * n2;
    double acc[kDiagSlots];
    for (int i = 0; i < kDiagSlots; ++i) acc[i] = 0.0;
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int x = 1 + static_cast<int>(e % n0);
        const int y = 1 + static_cast<int>((e / n0) % n1);
        const int z = 1 + static_cast<int>(e / (n0 * n1));
        float v[NF];
        load_node<S>(P, P.a, lin(P, x, y, z), v);
        to_moments<S>(P, v);
        const double rr = v[0], rb = v[1], rho = rr + rb;
        bool bad = !(rho > 0.0);
        for (int i = 0; i < NF; ++i) bad |= !isfinite(v[i]);
        acc[0] += rr;
        acc[1] += rb;
        acc[2] += rho * v[2];
        acc[3] += rho * v[3];
        acc[4] += rho * v[4];
        if (D.bubble) {
            const float dx = x - D.c0, dy = y - D.c1, dz = z - D.c2;
            const float r2 = dx * dx + dy * dy + dz * dz;
            const double p = (rho + rr * D.kappa_r + rb * D.kappa_b) / 3.0;
            if (r2 <= D.r_in2) { acc[5] += p; acc[6] += 1.0; }
            if (r2 >= D.r_out2) { acc[7] += p; acc[8] += 1.0; }
        }
        acc[9] += bad ? 1.0 : 0.0;
        acc[10] += 1.0;
    }
    // block reduction (fixed order: warp shuffles, then warps in index order)
    __shared__ double red[32][kDiagSlots];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = 0; i < kDiagSlots; ++i) {
        double s = acc[i];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) red[wid][i] = s;
    }
    __syncthreads();
    if (threadIdx.x < kDiagSlots) {
        double s = 0.0;
        for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) s += red[wv][threadIdx.x];
        partials[blockIdx.x * kDiagSlots + threadIdx.x] = s;
    }
}

__global__ void diag_final_kernel(const double* partials, int nparts, double* result) {
    const int i = threadIdx.x;
    if (i < kDiagSlots) {
        double s = 0.0;
        for (int b = 0; b < nparts; ++b) s += partials[b * kDiagSlots + i];
        result[i] = s;
    }
}

// ---------------------------------------------------------------- dense conversions
// One field between the library layout (padded pitch, 16-bit slots) and the reference's dense
// FP32 layout (pitch nx).  A block walks whole rows, so the index arithmetic is per row.
template <typename S>
__global__ void to_dense_kernel(const StepParams P, int field, float* __restrict__ dst) {
    const long long rows = static_cast<long long>(P.ny) * P.nz;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const long long o0 = (r / P.ny) * P.plane + (r % P.ny) * P.pitch;
        float* d = dst + r * P.nx;
        for (int x = threadIdx.x; x < P.nx; x += blockDim.x) {
            const long long o = o0 + x;
            float v;
            if constexpr (sizeof(S) == 4) {
                v = static_cast<const float*>(P.a[field])[o];
            } else if (field <= 1) {
                const float s0 = Codec<S>::to_f(static_cast<const S*>(P.a[0])[o]);
                const float c = Codec<S>::to_f(static_cast<const S*>(P.a[1])[o]);
                const float rho = P.rho_mean + phi_of_slot(c) * P.rho_half_diff + P.rho_scale * s0;
                float rr, rb;
                colour_split(c, rho, rr, rb);
                v = field == 0 ? rr : rb;
            } else {
                v = Codec<S>::to_f(static_cast<const S*>(P.a[field])[o]) * (field < 5 ? P.u_ref : P.pi_scale);
            }
            d[x] = v;
        }
    }
}

// Dense FP32 field(s) -> the state P.b.  The 16-bit forms store rho and the colour slot from
// rhor and rhob together: field 0 there takes src (rhor) and src_b (rhob) and field 1 is empty.
template <typename S>
__global__ void from_dense_kernel(const StepParams P, int field, const float* __restrict__ src,
                                  const float* __restrict__ src_b) {
    const long long rows = static_cast<long long>(P.ny) * P.nz;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const long long o0 = (r / P.ny) * P.plane + (r % P.ny) * P.pitch;
        const float* a = src + r * P.nx;
        for (int x = threadIdx.x; x < P.nx; x += blockDim.x) {
            const long long o = o0 + x;
            if constexpr (sizeof(S) == 4) {
                static_cast<float*>(P.b[field])[o] = a[x];
            } else if (field == 0) {
                const float rr = a[x], rb = src_b[r * P.nx + x];
                const float rho = rr + rb;
                if (rho == 0.0f) {
                    // unused ghost node with no fluid: zeros rather than 0/0
                    static_cast<S*>(P.b[0])[o] = Codec<S>::from_f(0.0f);
                    static_cast<S*>(P.b[1])[o] = Codec<S>::from_f(0.0f);
                    continue;
                }
                const S c = Codec<S>::from_f(colour_slot(rr, rb, rho));
                const float phi = phi_of_slot(Codec<S>::to_f(c)); // the phi a reader decodes
                static_cast<S*>(P.b[0])[o] = Codec<S>::from_f((rho - (P.rho_mean + phi * P.rho_half_diff)) * P.inv_rho_scale);
                static_cast<S*>(P.b[1])[o] = c;
            } else if (field >= 2) {
                static_cast<S*>(P.b[field])[o] = Codec<S>::from_f(a[x] * (field < 5 ? P.inv_u_ref : P.inv_pi_scale));
            }
        }
    }
}

// All 11 fields between the state and the reference's dense FP32 layout in host memory that
// the device reads or writes directly (pinned, mapped).  blockIdx.y is the field.  Over the host
// link a warp access costs a whole 128-byte line, so each field's element mapping is shifted to
// start at a line boundary of its own host array (fields of the reference's dense layout are
// not line-aligned): every warp then moves exactly one line (measured 209 / 190 GB/s read /
// write against 160 / 136 unaligned).  The conversions are those of to_dense / from_dense.
struct HostFields {
    float* f[NF];
};

template <bool k32>
__device__ __forceinline__ long long dense_to_state(const StepParams& P, long long i) {
    if constexpr (k32) {
        const unsigned ui = static_cast<unsigned>(i), nx = static_cast<unsigned>(P.nx), ny = static_cast<unsigned>(P.ny);
        const unsigned r = ui / nx, x = ui - r * nx;
        const unsigned z = r / ny, y = r - z * ny;
        return static_cast<long long>(z) * P.plane + static_cast<long long>(y) * P.pitch + x;
    } else {
        const long long r = i / P.nx, x = i - r * P.nx;
        const long long z = r / P.ny, y = r - z * P.ny;
        return z * P.plane + y * P.pitch + x;
    }
}

// elements of a host field before its first 128-byte line boundary
__device__ __forceinline__ int line_shift(const float* p) {
    return static_cast<int>(((128u - (reinterpret_cast<uintptr_t>(p) & 127u)) & 127u) >> 2);
}

template <typename S, bool k32>
__global__ void state_to_host_kernel(const StepParams P, HostFields h, long long n) {
    const int f = blockIdx.y;
    float* dst = h.f[f];
    // thread t handles element t - (32 - shift) mod 32, so element `shift` starts a warp
    const int lead = (32 - line_shift(dst)) & 31;
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < n + lead; t += stride) {
        const long long i = t - lead;
        if (i < 0) continue;
        const long long o = dense_to_state<k32>(P, i);
        float v;
        if constexpr (sizeof(S) == 4) {
            v = static_cast<const float*>(P.a[f])[o];
        } else if (f <= 1) {
            const float s0 = Codec<S>::to_f(static_cast<const S*>(P.a[0])[o]);
            const float c = Codec<S>::to_f(static_cast<const S*>(P.a[1])[o]);
            const float rho = P.rho_mean + phi_of_slot(c) * P.rho_half_diff + P.rho_scale * s0;
            float rr, rb;
            colour_split(c, rho, rr, rb);
            v = f == 0 ? rr : rb;
        } else {
            v = Codec<S>::to_f(static_cast<const S*>(P.a[f])[o]) * (f < 5 ? P.u_ref : P.pi_scale);
        }
        dst[i] = v;
    }
}

template <typename S, bool k32>
__global__ void host_to_state_kernel(const StepParams P, HostFields h, long long n) {
    const int f = blockIdx.y;
    if (sizeof(S) != 4 && f == 1) return; // the 16-bit forms store rhor and rhob together (f = 0)
    const float* src = h.f[f];
    const int lead = (32 - line_shift(src)) & 31;
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < n + lead; t += stride) {
        const long long i = t - lead;
        if (i < 0) continue;
        const long long o = dense_to_state<k32>(P, i);
        if constexpr (sizeof(S) == 4) {
            static_cast<float*>(P.b[f])[o] = src[i];
        } else if (f == 0) {
            const float rr = src[i], rb = h.f[1][i], rho = rr + rb;
            if (rho == 0.0f) {
                // unused ghost node with no fluid: zeros rather than 0/0
                static_cast<S*>(P.b[0])[o] = Codec<S>::from_f(0.0f);
                static_cast<S*>(P.b[1])[o] = Codec<S>::from_f(0.0f);
            } else {
                const S c = Codec<S>::from_f(colour_slot(rr, rb, rho));
                const float phi = phi_of_slot(Codec<S>::to_f(c)); // the phi a reader decodes
                static_cast<S*>(P.b[0])[o] =
                    Codec<S>::from_f((rho - (P.rho_mean + phi * P.rho_half_diff)) * P.inv_rho_scale);
                static_cast<S*>(P.b[1])[o] = c;
            }
        } else {
            static_cast<S*>(P.b[f])[o] = Codec<S>::from_f(src[i] * (f < 5 ? P.inv_u_ref : P.inv_pi_scale));
        }
    }
}

int rows_grid(const StepParams& P) {
    const long long rows = static_cast<long long>(P.ny) * P.nz;
    return static_cast<int>(std::min<long long>(rows, 65535));
}

template <typename S>
cudaError_t bc_t(const StepParams& P, int init_inlet, cudaStream_t s) {
    bc_kernel<S><<<256, 256, 0, s>>>(P, init_inlet);
    return cudaGetLastError();
}

int grid_for(long long n) {
    long long g = (n + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    if (g < 1) g = 1;
    return static_cast<int>(g);
}

} // namespace

template <typename S>
static cudaError_t fill_ghosts_t(const StepParams& P, cudaStream_t s) {
    for (int axis = 0; axis < 2; ++axis) {
        if (P.bc[axis] != MBCG_BC_PERIODIC) continue;
        const long long n = static_cast<long long>(axis == 0 ? P.ny : P.nx) * P.nz * 2;
        fill_ghosts_kernel<S><<<grid_for(n), 256, 0, s>>>(P, axis);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_fill_ghosts(int precision, const StepParams& P, cudaStream_t s) {
    switch (precision) {
    case MBCG_FP16: return fill_ghosts_t<__half>(P, s);
    case MBCG_BF16: return fill_ghosts_t<__nv_bfloat16>(P, s);
    default: return fill_ghosts_t<float>(P, s);
    }
}

cudaError_t launch_bc(int precision, const StepParams& P, cudaStream_t s) {
    if (P.inout_axis < 0) return cudaSuccess;
    switch (precision) {
    case MBCG_FP16: return bc_t<__half>(P, 0, s);
    case MBCG_BF16: return bc_t<__nv_bfloat16>(P, 0, s);
    default: return bc_t<float>(P, 0, s);
    }
}

template <typename S>
static cudaError_t init_t(const StepParams& P, const mbcg_params& p, cudaStream_t s) {
    ICParams I{};
    I.kind = p.ic;
    I.h = 1;
    for (int a = 0; a < 3; ++a)
        if (p.bc[a] == MBCG_BC_WALL) I.h = a;
    I.bc0 = static_cast<float>(p.bubble_center[0]);
    I.bc1 = static_cast<float>(p.bubble_center[1]);
    I.bc2 = static_cast<float>(p.bubble_center[2]);
    I.brad = static_cast<float>(p.bubble_radius);
    I.bwidth = static_cast<float>(p.bubble_width);
    I.bphase = static_cast<float>(p.bubble_phase);
    I.rpos = static_cast<float>(p.rti_position);
    I.ramp = static_cast<float>(p.rti_amplitude);
    I.rwidth = static_cast<float>(p.rti_width);
    I.rphase = static_cast<float>(p.rti_phase_above);
    {
        const int n3[3] = {p.nx, p.ny, p.nz};
        const int t0 = I.h == 0 ? 1 : 0, t1 = I.h == 2 ? 1 : 2;
        // rtiIn.cuh:71-84: k = 2 pi mode / (N - 2), evaluated in float as the reference does
        const float pi = 3.141592653589793f;
        I.rk0 = 2.0f * pi * static_cast<float>(p.rti_mode[0]) / static_cast<float>(n3[t0] - 2);
        I.rk1 = 2.0f * pi * static_cast<float>(p.rti_mode[1]) / static_cast<float>(n3[t1] - 2);
    }
    const long long n = static_cast<long long>(P.nx) * P.ny * P.nz;
    init_kernel<S><<<grid_for(n), 256, 0, s>>>(P, I);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (p.ic == MBCG_IC_RTI) {
        rti_walls_kernel<S><<<256, 256, 0, s>>>(P, I.h);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (p.ic == MBCG_IC_JET && P.inout_axis >= 0) {
        // jet/jetIn.cuh:39-60 then the initial boundary pass with B = A (main.cu:25-26)
        StepParams Q = P;
        Q.a[0] = nullptr;
        for (int i = 0; i < NF; ++i) Q.a[i] = P.b[i];
        Q.step = 0;
        e = bc_t<S>(Q, 1, s);
        if (e != cudaSuccess) return e;
        e = bc_t<S>(Q, 0, s);
        if (e != cudaSuccess) return e;
    }
    return P.ghost_images ? fill_ghosts_t<S>(P, s) : e;
}

cudaError_t launch_init(int precision, const StepParams& P, const mbcg_params& p, cudaStream_t s) {
    switch (precision) {
    case MBCG_FP16: return init_t<__half>(P, p, s);
    case MBCG_BF16: return init_t<__nv_bfloat16>(P, p, s);
    default: return init_t<float>(P, p, s);
    }
}

int diag_partials_needed(const StepParams& P) {
    return grid_for(static_cast<long long>(P.nx - 2) * (P.ny - 2) * (P.nz - 2));
}

template <typename S>
static cudaError_t diag_t(const StepParams& P, const mbcg_params& p, double* partials, int nparts, double* result,
                          cudaStream_t s) {
    DiagParams D{};
    D.bubble = p.ic == MBCG_IC_BUBBLE;
    D.c0 = static_cast<float>(p.bubble_center[0]);
    D.c1 = static_cast<float>(p.bubble_center[1]);
    D.c2 = static_cast<float>(p.bubble_center[2]);
    const float rin = 0.5f * static_cast<float>(p.bubble_radius);
    const float rout = static_cast<float>(p.bubble_radius + 2.0 * p.bubble_width + 4.0);
    D.r_in2 = rin * rin;
    D.r_out2 = rout * rout;
    D.kappa_r = P.ratio ? P.kappa_r : 0.0f;
    D.kappa_b = P.ratio ? P.kappa_b : 0.0f;
    diag_kernel<S><<<nparts, 256, 0, s>>>(P, D, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    diag_final_kernel<<<1, 32, 0, s>>>(partials, nparts, result);
    return cudaGetLastError();
}

cudaError_t launch_diag(int precision, const StepParams& P, const mbcg_params& p, double* partials, int nparts,
                        double* result, cudaStream_t s) {
    switch (precision) {
    case MBCG_FP16: return diag_t<__half>(P, p, partials, nparts, result, s);
    case MBCG_BF16: return diag_t<__nv_bfloat16>(P, p, partials, nparts, result, s);
    default: return diag_t<float>(P, p, partials, nparts, result, s);
    }
}

cudaError_t launch_to_dense(int precision, const StepParams& P, int field, float* dst, cudaStream_t s) {
    switch (precision) {
    case MBCG_FP16: to_dense_kernel<__half><<<rows_grid(P), 256, 0, s>>>(P, field, dst); break;
    case MBCG_BF16: to_dense_kernel<__nv_bfloat16><<<rows_grid(P), 256, 0, s>>>(P, field, dst); break;
    default: to_dense_kernel<float><<<rows_grid(P), 256, 0, s>>>(P, field, dst); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_from_dense(int precision, const StepParams& P, int field, const float* src, const float* src_b,
                              cudaStream_t s) {
    switch (precision) {
    case MBCG_FP16: from_dense_kernel<__half><<<rows_grid(P), 256, 0, s>>>(P, field, src, src_b); break;
    case MBCG_BF16: from_dense_kernel<__nv_bfloat16><<<rows_grid(P), 256, 0, s>>>(P, field, src, src_b); break;
    default: from_dense_kernel<float><<<rows_grid(P), 256, 0, s>>>(P, field, src, src_b); break;
    }
    return cudaGetLastError();
}

// grid: 4 CTAs per SM along x, one row of CTAs per field along y
static dim3 host_grid() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return dim3(4 * (sms > 0 ? sms : 1), NF);
}

template <typename S>
static void state_to_host_t(const StepParams& P, const HostFields& h, long long n, cudaStream_t s) {
    if (n + 32 < (1ll << 31)) state_to_host_kernel<S, true><<<host_grid(), 256, 0, s>>>(P, h, n);
    else state_to_host_kernel<S, false><<<host_grid(), 256, 0, s>>>(P, h, n);
}
template <typename S>
static void host_to_state_t(const StepParams& P, const HostFields& h, long long n, cudaStream_t s) {
    if (n + 32 < (1ll << 31)) host_to_state_kernel<S, true><<<host_grid(), 256, 0, s>>>(P, h, n);
    else host_to_state_kernel<S, false><<<host_grid(), 256, 0, s>>>(P, h, n);
}

cudaError_t launch_state_to_host(int precision, const StepParams& P, float* const host[NF], cudaStream_t s) {
    HostFields h;
    for (int f = 0; f < NF; ++f) h.f[f] = host[f];
    const long long n = static_cast<long long>(P.nx) * P.ny * P.nz;
    switch (precision) {
    case MBCG_FP16: state_to_host_t<__half>(P, h, n, s); break;
    case MBCG_BF16: state_to_host_t<__nv_bfloat16>(P, h, n, s); break;
    default: state_to_host_t<float>(P, h, n, s); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_host_to_state(int precision, const StepParams& P, const float* const host[NF], cudaStream_t s) {
    HostFields h;
    for (int f = 0; f < NF; ++f) h.f[f] = const_cast<float*>(host[f]);
    const long long n = static_cast<long long>(P.nx) * P.ny * P.nz;
    switch (precision) {
    case MBCG_FP16: host_to_state_t<__half>(P, h, n, s); break;
    case MBCG_BF16: host_to_state_t<__nv_bfloat16>(P, h, n, s); break;
    default: host_to_state_t<float>(P, h, n, s); break;
    }
    return cudaGetLastError();
}

} // namespace mbcg
