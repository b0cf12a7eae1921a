// mbcg_phase.cu -- in-situ phase statistics of a case's current state (declared in
// include/mbcg.h, mbcg_phase_statistics): phase volumes, diffuse-interface area, interface node
// count, jet penetration and centroid as deterministic FP64 reductions, and optionally the
// connected regions of the tracked phase (droplets) by a lock-free union-find over the fluid
// nodes.  No counterpart in the reference, which declares a jet-breakup statistics sampler
// (constants.cuh:11,53) but never implements it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "mbcg_internal.h"

using namespace mbcg;

namespace {

int fail(int code, const std::string& msg) {
    set_last_error(msg);
    return code;
}

constexpr int kSlots = 8; // tracked volume, other volume, area, interface nodes, centroid x/y/z, penetration (max)
constexpr int kBlock = 256;
constexpr int kLoopCap = 1 << 22; // union-find iterations before a loop gives up

struct PhaseArgs {
    StepParams P;
    int sign;    // +1: red tracked, -1: blue tracked
    int ia;      // inlet/outlet axis, -1 if none
    int nf[3];   // fluid nodes per axis
    int* labels; // per fluid node, or null
    int* status;
};

template <typename S>
__device__ __forceinline__ float phi_at(const StepParams& P, long long o) {
    float rr, rb;
    if constexpr (sizeof(S) == 4) {
        rr = static_cast<const float*>(P.a[0])[o];
        rb = static_cast<const float*>(P.a[1])[o];
    } else {
        const float c = Codec<S>::to_f(static_cast<const S*>(P.a[1])[o]);
        const float s0 = Codec<S>::to_f(static_cast<const S*>(P.a[0])[o]);
        const float rho = P.rho_mean + phi_of_slot(c) * P.rho_half_diff + P.rho_scale * s0;
        colour_split(c, rho, rr, rb);
    }
    return (rr - rb) / (rr + rb);
}

// neighbour coordinate along an axis: periodic axes wrap over the fluid nodes 1..n-2, the others
// stay inside them (one-sided difference at the first and last fluid layer)
__device__ __forceinline__ int nb_coord(const StepParams& P, int a, int c, int n) {
    if (P.bc[a] == MBCG_BC_PERIODIC) return periodic_image(c, n);
    return min(max(c, 1), n - 2);
}

__device__ __forceinline__ long long lin3(const StepParams& P, int x, int y, int z) {
    return static_cast<long long>(z) * P.plane + static_cast<long long>(y) * P.pitch + x;
}

template <typename S>
__global__ void phase_sums_kernel(const PhaseArgs A, double* partials) {
    const StepParams& P = A.P;
    __shared__ double sh[kSlots][kBlock];
    double acc[kSlots] = {0, 0, 0, 0, 0, 0, 0, -1.0};
    const long long total = static_cast<long long>(A.nf[0]) * A.nf[1] * A.nf[2];
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int x = 1 + static_cast<int>(e % A.nf[0]);
        const int y = 1 + static_cast<int>((e / A.nf[0]) % A.nf[1]);
        const int z = 1 + static_cast<int>(e / (static_cast<long long>(A.nf[0]) * A.nf[1]));
        const int c[3] = {x, y, z}, n[3] = {P.nx, P.ny, P.nz};
        const float phi = phi_at<S>(P, lin3(P, x, y, z));
        const bool tracked = A.sign * phi > 0.0f;
        acc[tracked ? 0 : 1] += 1.0;
        // 4 rho_r rho_b / rho^2 = 1 - phi^2 (lbm.cuh:181)
        if (1.0f - phi * phi > 1.0e-4f) acc[3] += 1.0;
        double g2 = 0.0;
        for (int a = 0; a < 3; ++a) {
            int lo[3] = {x, y, z}, hi[3] = {x, y, z};
            lo[a] = nb_coord(P, a, c[a] - 1, n[a]);
            hi[a] = nb_coord(P, a, c[a] + 1, n[a]);
            const int span = (P.bc[a] == MBCG_BC_PERIODIC) ? 2 : (min(c[a] + 1, n[a] - 2) - max(c[a] - 1, 1));
            if (span <= 0) continue;
            const double d = (static_cast<double>(phi_at<S>(P, lin3(P, hi[0], hi[1], hi[2]))) -
                              static_cast<double>(phi_at<S>(P, lin3(P, lo[0], lo[1], lo[2])))) /
                             span;
            g2 += d * d;
        }
        acc[2] += 0.5 * sqrt(g2);
        if (tracked) {
            acc[4] += x;
            acc[5] += y;
            acc[6] += z;
            if (A.ia >= 0) acc[7] = fmax(acc[7], static_cast<double>(c[A.ia]));
        }
        if (A.labels) A.labels[e] = tracked ? static_cast<int>(e) : -1;
    }
    for (int s = 0; s < kSlots; ++s) sh[s][threadIdx.x] = acc[s];
    __syncthreads();
    for (int stride = kBlock / 2; stride > 0; stride >>= 1) {
        if (threadIdx.x < stride)
            for (int s = 0; s < kSlots; ++s)
                sh[s][threadIdx.x] = s == 7 ? fmax(sh[s][threadIdx.x], sh[s][threadIdx.x + stride])
                                            : sh[s][threadIdx.x] + sh[s][threadIdx.x + stride];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int s = 0; s < kSlots; ++s) partials[blockIdx.x * kSlots + s] = sh[s][0];
}

// fixed-order sum of the block partials (deterministic)
__global__ void phase_final_kernel(const double* partials, int nparts, double* result) {
    const int s = threadIdx.x;
    if (s >= kSlots) return;
    double v = s == 7 ? -1.0 : 0.0;
    for (int b = 0; b < nparts; ++b) v = s == 7 ? fmax(v, partials[b * kSlots + s]) : v + partials[b * kSlots + s];
    result[s] = v;
}

// ---------------------------------------------------------------- connected regions
// Lock-free union-find (labels only ever decrease towards a root); every loop is capped and
// reports through the status word instead of spinning on.
__device__ __forceinline__ int find_root(int* L, int i, int* status) {
    for (int it = 0; it < kLoopCap; ++it) {
        const int p = L[i];
        if (p == i) return i;
        const int gp = L[p];
        if (gp != p) L[i] = gp; // path halving (benign race: any value on the path is valid)
        i = gp;
    }
    atomicOr(status, 4);
    return i;
}

__device__ __forceinline__ void unite(int* L, int a, int b, int* status) {
    for (int it = 0; it < kLoopCap; ++it) {
        a = find_root(L, a, status);
        b = find_root(L, b, status);
        if (a == b) return;
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicCAS(&L[b], b, a); // link the larger root under the smaller
        if (old == b) return;
        b = old;
    }
    atomicOr(status, 4);
}

__global__ void merge_kernel(const PhaseArgs A) {
    const long long total = static_cast<long long>(A.nf[0]) * A.nf[1] * A.nf[2];
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (A.labels[e] < 0) continue;
        int c[3] = {static_cast<int>(e % A.nf[0]), static_cast<int>((e / A.nf[0]) % A.nf[1]),
                    static_cast<int>(e / (static_cast<long long>(A.nf[0]) * A.nf[1]))};
        for (int a = 0; a < 3; ++a) {
            int d[3] = {c[0], c[1], c[2]};
            d[a] += 1;
            if (d[a] == A.nf[a]) {
                if (A.P.bc[a] != MBCG_BC_PERIODIC) continue;
                d[a] = 0;
            }
            const long long f = d[0] + static_cast<long long>(A.nf[0]) * (d[1] + static_cast<long long>(A.nf[1]) * d[2]);
            if (f != e && A.labels[f] >= 0) unite(A.labels, static_cast<int>(e), static_cast<int>(f), A.status);
        }
    }
}

__global__ void region_kernel(const PhaseArgs A, int* volume, unsigned char* touches) {
    const long long total = static_cast<long long>(A.nf[0]) * A.nf[1] * A.nf[2];
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (A.labels[e] < 0) continue;
        const int r = find_root(A.labels, static_cast<int>(e), A.status);
        atomicAdd(&volume[r], 1);
        if (A.ia >= 0) {
            const int c[3] = {static_cast<int>(e % A.nf[0]), static_cast<int>((e / A.nf[0]) % A.nf[1]),
                              static_cast<int>(e / (static_cast<long long>(A.nf[0]) * A.nf[1]))};
            if (c[A.ia] == 0) touches[r] = 1;
        }
    }
}

// per root: count, largest, detached count and volume (integer atomics: order-independent)
__global__ void region_stats_kernel(const PhaseArgs A, const int* volume, const unsigned char* touches,
                                    unsigned long long* out) {
    const long long total = static_cast<long long>(A.nf[0]) * A.nf[1] * A.nf[2];
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (A.labels[e] != static_cast<int>(e)) continue; // roots only
        const unsigned long long v = static_cast<unsigned long long>(volume[e]);
        atomicAdd(&out[0], 1ULL);
        atomicMax(&out[1], v);
        if (!touches[e]) {
            atomicAdd(&out[2], 1ULL);
            atomicAdd(&out[3], v);
        }
    }
}

template <typename S>
cudaError_t sums(const PhaseArgs& A, double* partials, int nparts, double* result, cudaStream_t s) {
    phase_sums_kernel<S><<<nparts, kBlock, 0, s>>>(A, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    phase_final_kernel<<<1, 32, 0, s>>>(partials, nparts, result);
    return cudaGetLastError();
}

int phase_statistics(const mbcg_params& p, const StepParams& P, int32_t flags, mbcg_phase_stats* out, mbcg_stream_t s) {
    PhaseArgs A;
    std::memset(&A, 0, sizeof(A));
    A.P = P;
    A.ia = A.P.inout_axis;
    A.sign = (A.ia >= 0 && p.ic == MBCG_IC_JET && p.jet_phase < 0.0) ? -1 : 1;
    A.nf[0] = p.nx - 2;
    A.nf[1] = p.ny - 2;
    A.nf[2] = p.nz - 2;
    const long long nodes = static_cast<long long>(A.nf[0]) * A.nf[1] * A.nf[2];
    const bool comps = (flags & MBCG_STATS_COMPONENTS) != 0;
    if (comps && nodes >= (1LL << 31)) return fail(MBCG_E_UNSUPPORTED, "region labels need fewer than 2^31 fluid nodes");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    const int nparts = static_cast<int>(std::min<long long>((nodes + kBlock - 1) / kBlock, 1184));
    // one scratch allocation: partials, results, status, region counters, then the labels
    const size_t small = sizeof(double) * (kSlots * (nparts + 1)) + 64 + 4 * sizeof(unsigned long long);
    const size_t big = comps ? static_cast<size_t>(nodes) * (2 * sizeof(int) + 1) : 0;
    unsigned char* scratch = nullptr;
    cudaError_t e = cudaMalloc(&scratch, small + big + 256);
    if (e != cudaSuccess) return fail(MBCG_E_NOMEM, "phase statistics scratch allocation failed");
    double* partials = reinterpret_cast<double*>(scratch);
    double* result = partials + kSlots * nparts;
    int* status = reinterpret_cast<int*>(result + kSlots);
    unsigned long long* counters = reinterpret_cast<unsigned long long*>(scratch + sizeof(double) * kSlots * (nparts + 1) + 64);
    int* labels = nullptr;
    int* volume = nullptr;
    unsigned char* touches = nullptr;
    if (comps) {
        unsigned char* b = scratch + ((small + 255) / 256) * 256;
        labels = reinterpret_cast<int*>(b);
        volume = labels + nodes;
        touches = reinterpret_cast<unsigned char*>(volume + nodes);
    }
    A.labels = labels;
    A.status = status;
    e = cudaMemsetAsync(scratch, 0, small + big + 256, st);
    if (e == cudaSuccess) {
        switch (p.precision) {
        case MBCG_FP16: e = sums<__half>(A, partials, nparts, result, st); break;
        case MBCG_BF16: e = sums<__nv_bfloat16>(A, partials, nparts, result, st); break;
        default: e = sums<float>(A, partials, nparts, result, st); break;
        }
    }
    const int grid = static_cast<int>(std::min<long long>((nodes + kBlock - 1) / kBlock, 4 * 1184));
    if (comps && e == cudaSuccess) {
        merge_kernel<<<grid, kBlock, 0, st>>>(A);
        e = cudaGetLastError();
        if (e == cudaSuccess) {
            region_kernel<<<grid, kBlock, 0, st>>>(A, volume, touches);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            region_stats_kernel<<<grid, kBlock, 0, st>>>(A, volume, touches, counters);
            e = cudaGetLastError();
        }
    }
    double r[kSlots];
    int stat = 0;
    unsigned long long cnt[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(r, result, sizeof(r), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&stat, status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, counters, sizeof(cnt), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(scratch);
    if (e != cudaSuccess) return fail(MBCG_E_CUDA, std::string("phase statistics: ") + cudaGetErrorString(e));
    std::memset(out, 0, sizeof(*out));
    out->volume_tracked = r[0];
    out->volume_other = r[1];
    out->interface_area = r[2];
    out->interface_nodes = static_cast<int64_t>(r[3]);
    for (int a = 0; a < 3; ++a) out->centroid[a] = r[0] > 0 ? r[4 + a] / r[0] : 0.0;
    out->penetration = A.ia >= 0 ? r[7] : -1.0; // fluid coordinate = distance from the inlet ghost layer
    out->components = comps ? static_cast<int64_t>(cnt[0]) : -1;
    out->largest_component = comps ? static_cast<int64_t>(cnt[1]) : -1;
    out->detached = comps ? static_cast<int64_t>(cnt[2]) : -1;
    out->detached_volume = comps ? static_cast<int64_t>(cnt[3]) : -1;
    out->status = stat;
    return MBCG_OK;
}

} // namespace

extern "C" {

int mbcg_phase_statistics(mbcg_case* c, int32_t flags, mbcg_phase_stats* out, mbcg_stream_t s) {
    if (!c || !out) return fail(MBCG_E_INVALID, "null argument");
    mbcg_params p;
    if (int rc = mbcg_case_params(c, &p)) return rc;
    StepParams P;
    if (int rc = case_state_params(c, &P)) return rc;
    return phase_statistics(p, P, flags, out, s);
}

int mbcg_phase_statistics_moments(const mbcg_params* p, const mbcg_moments* a, int32_t flags, mbcg_phase_stats* out,
                                  mbcg_stream_t s) {
    if (!p || !a || !out) return fail(MBCG_E_INVALID, "null argument");
    if (int rc = validate_params(p)) return rc;
    if (a->precision != p->precision || a->pitch < p->nx) return fail(MBCG_E_INVALID, "moments do not match params");
    for (int i = 0; i < NF; ++i)
        if (!a->f[i]) return fail(MBCG_E_INVALID, "null field pointer");
    StepParams P;
    fill_step_physics(*p, P);
    P.pitch = a->pitch;
    P.plane = a->pitch * p->ny;
    for (int i = 0; i < NF; ++i) P.a[i] = a->f[i];
    return phase_statistics(*p, P, flags, out, s);
}

} // extern "C"
