// mbcg_noalloc.cu -- FP64 diagnostics of caller-owned moment arrays that allocate no memory.
//
// mbcg_diagnostics() keeps its per-block partial sums in device memory the case handle
// allocated at creation.  Some callers cannot allocate at the point where they want the
// numbers: a solver loop whose device memory is entirely reserved for resident states, a host
// program embedded in a framework whose own allocator owns the GPU (a cudaMalloc there can
// synchronise the device or fail under memory pressure), or code that only holds the
// reference-style MomentsDevice arrays and no case handle.  mbcg_diagnostics_static() gives
// them the same reductions with the scratch in a fixed array compiled into this library.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <string>

#include "mbcg_internal.h"

using namespace mbcg;

namespace {

// Fixed scratch: up to kMaxParts block partials plus the final slots.  Every GPU that loads the
// library holds it (about 385 KB) until the process exits.
constexpr int kMaxParts = 4096;
constexpr long long kNodesPerBlock = 256LL * 128LL; // 256 threads, 128 fluid nodes each
static __device__ __align__(256) double g_diag_scratch[(kMaxParts + 1) * kDiagSlots];

int fail(int code, const std::string& msg) {
    set_last_error(msg); // reported by mbcg_last_error()
    return code;
}

// Device address of the scratch array on the current device.  The host-side symbol is only a
// stand-in; the address is looked up on every call, with the calling thread's device current,
// so it stays valid after a cudaDeviceReset reloads the module at another address (the lookup
// allocates nothing).
int scratch_on_current_device(double** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_diag_scratch);
    if (e != cudaSuccess || !p)
        return fail(MBCG_E_CUDA, std::string("cudaGetSymbolAddress of the diagnostics scratch: ") +
                                     cudaGetErrorString(e));
    *out = static_cast<double*>(p);
    return MBCG_OK;
}

} // namespace

extern "C" {

// Diagnostics of the state `a` (reference layout, any pitch >= nx) without any device or host
// allocation; see include/mbcg.h for the contract.
int mbcg_diagnostics_static(const mbcg_params* p, const mbcg_moments* a, mbcg_diag* out, mbcg_stream_t s) {
    if (!p || !a || !out) return fail(MBCG_E_INVALID, "null argument");
    // precision tag, densities and sizes as every other entry point checks them (an unknown
    // precision would otherwise read the fields with the wrong element size)
    if (int rc = validate_params(p)) return rc;
    if (a->precision != p->precision) return fail(MBCG_E_INVALID, "moments precision differs from params");
    if (a->pitch < p->nx || p->nx < 3 || p->ny < 3 || p->nz < 3)
        return fail(MBCG_E_INVALID, "bad lattice size or pitch");
    for (int i = 0; i < NF; ++i)
        if (!a->f[i]) return fail(MBCG_E_INVALID, "null field pointer");
    const long long nodes = static_cast<long long>(p->nx - 2) * (p->ny - 2) * (p->nz - 2);
    const long long parts = (nodes + kNodesPerBlock - 1) / kNodesPerBlock;
    if (parts > kMaxParts)
        return fail(MBCG_E_UNSUPPORTED,
                    "lattice has " + std::to_string(nodes) + " fluid nodes; the allocation-free diagnostics handle at most " +
                        std::to_string(static_cast<long long>(kMaxParts) * kNodesPerBlock));
    double* scratch = nullptr;
    if (int rc = scratch_on_current_device(&scratch)) return rc;

    StepParams P;
    std::memset(&P, 0, sizeof(P));
    P.nx = p->nx;
    P.ny = p->ny;
    P.nz = p->nz;
    for (int k = 0; k < 3; ++k) P.bc[k] = p->bc[k];
    P.pitch = a->pitch;
    P.plane = a->pitch * p->ny;
    P.ratio = p->rho_r0 != p->rho_b0;
    const double rmin = p->rho_r0 < p->rho_b0 ? p->rho_r0 : p->rho_b0;
    P.kappa_r = static_cast<float>(rmin / p->rho_r0 - 1.0);
    P.kappa_b = static_cast<float>(rmin / p->rho_b0 - 1.0);
    P.rho_scale = static_cast<float>(p->rho_scale);
    P.u_ref = static_cast<float>(p->u_ref);
    P.pi_scale = static_cast<float>(p->pi_scale);
    P.rho_mean = static_cast<float>(0.5 * (p->rho_r0 + p->rho_b0));
    P.rho_half_diff = static_cast<float>(0.5 * (p->rho_r0 - p->rho_b0));
    for (int i = 0; i < NF; ++i) P.a[i] = a->f[i];

    // every partial slot the launch uses is written by its block and the final slots are fully
    // overwritten, so nothing left by an earlier call is read
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    double* partials = scratch + kDiagSlots;
    double* result = scratch;
    cudaError_t e = launch_diag(p->precision, P, *p, partials, static_cast<int>(parts), result, st);
    if (e != cudaSuccess) return fail(MBCG_E_CUDA, std::string("diagnostics kernel: ") + cudaGetErrorString(e));
    double r[kDiagSlots];
    e = cudaMemcpyAsync(r, result, sizeof(r), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(MBCG_E_CUDA, std::string("diagnostics copy: ") + cudaGetErrorString(e));
    out->mass_r = r[0];
    out->mass_b = r[1];
    out->momentum[0] = r[2];
    out->momentum[1] = r[3];
    out->momentum[2] = r[4];
    out->p_in = r[6] > 0 ? r[5] / r[6] : 0.0;
    out->p_out = r[8] > 0 ? r[7] / r[8] : 0.0;
    out->dp = out->p_in - out->p_out;
    out->nonfinite = static_cast<int64_t>(r[9]);
    out->nodes = static_cast<int64_t>(r[10]);
    return MBCG_OK;
}

} // extern "C"
