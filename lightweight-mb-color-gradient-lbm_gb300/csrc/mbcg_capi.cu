// mbcg_capi.cu -- the extern "C" boundary of libmbcg.so (declared in include/mbcg.h).
//
// Replaces the reference's host layer: allocate_device_memory / free_device_memory
// (memory.cuh:153-194), launch_RCS / launch_JetBoundaryConditions / launch_Init*
// (launch.cuh:14-94), swap_moments (memory.cuh:200-203) and copy_out_D2H
// (memory.cuh:209-217).  Errors are returned as status codes with a per-thread message,
// never by exit() (utilities/cudaUtilities.cuh:9-19).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "mbcg_internal.h"

using namespace mbcg;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    return fail(MBCG_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define MBCG_TRY(call, what)                          \
    do {                                              \
        cudaError_t e__ = (call);                     \
        if (e__ != cudaSuccess) return cuda_fail(e__, what); \
    } while (0)

int elem_bytes(int precision) { return precision == MBCG_FP32 ? 4 : 2; }

int validate(const mbcg_params* p) {
    if (!p) return fail(MBCG_E_INVALID, "null parameters");
    if (p->q != 19 && p->q != 27) return fail(MBCG_E_INVALID, "q must be 19 or 27");
    if (p->nx < 4 || p->ny < 4 || p->nz < 4) return fail(MBCG_E_INVALID, "each lattice axis needs >= 4 nodes");
    if (static_cast<long long>(p->nx) * p->ny * p->nz >= (1LL << 40))
        return fail(MBCG_E_INVALID, "lattice too large");
    int nonper = 0;
    for (int a = 0; a < 3; ++a) {
        if (p->bc[a] < MBCG_BC_PERIODIC || p->bc[a] > MBCG_BC_WALL) return fail(MBCG_E_INVALID, "unknown boundary kind");
        if (p->bc[a] != MBCG_BC_PERIODIC) ++nonper;
    }
    if (nonper > 1) return fail(MBCG_E_INVALID, "at most one axis may be non-periodic");
    if (p->precision < MBCG_FP32 || p->precision > MBCG_BF16) return fail(MBCG_E_INVALID, "unknown precision");
    if (!(p->tau > 0.5)) return fail(MBCG_E_INVALID, "tau must exceed 1/2");
    if (p->tau_b != 0.0 && !(p->tau_b > 0.5)) return fail(MBCG_E_INVALID, "tau_b must be 0 or exceed 1/2");
    if (!(p->rho_r0 > 0.0) || !(p->rho_b0 > 0.0)) return fail(MBCG_E_INVALID, "phase densities must be positive");
    if (p->precision != MBCG_FP32 && (!(p->rho_scale > 0) || !(p->u_ref > 0) || !(p->pi_scale > 0)))
        return fail(MBCG_E_INVALID, "FP16/BF16 storage needs positive rho_scale, u_ref and pi_scale");
    return MBCG_OK;
}

int inout_axis(const mbcg_params& p) {
    for (int a = 0; a < 3; ++a)
        if (p.bc[a] == MBCG_BC_INOUT) return a;
    return -1;
}

// the reference's float constant chain (constants.cuh:56-93, forces.cuh:114-117)
void fill_physics(const mbcg_params& p, StepParams& P) {
    std::memset(&P, 0, sizeof(P));
    P.nx = p.nx;
    P.ny = p.ny;
    P.nz = p.nz;
    for (int a = 0; a < 3; ++a) P.bc[a] = p.bc[a];
    P.inout_axis = inout_axis(p);
    P.outlet = p.outlet;
    const float taub = static_cast<float>(p.tau);
    P.oms = 1.0f - 1.0f / taub;
    const float cs2 = static_cast<float>(1.0 / 3.0);
    const float cs4 = cs2 * cs2;
    const float s4 = static_cast<float>(p.sigma) / (4.0f * cs4);
    P.A = s4 / taub;
    P.s4 = s4;
    P.tau_var = p.tau_b > 0.0 && p.tau_b != p.tau;
    P.tau_r = taub;
    P.tau_b = p.tau_b > 0.0 ? static_cast<float>(p.tau_b) : taub;
    P.beta = static_cast<float>(p.beta);
    P.omega2_conservative = p.omega2_conservative != 0;
    P.wait_test_cycles = p.wait_test_cycles > 0 ? p.wait_test_cycles : 0;
    P.ratio = p.rho_r0 != p.rho_b0;
    const double rmin = std::min(p.rho_r0, p.rho_b0);
    P.kappa_r = static_cast<float>(rmin / p.rho_r0 - 1.0);
    P.kappa_b = static_cast<float>(rmin / p.rho_b0 - 1.0);
    P.forced = p.gravity[0] != 0.0 || p.gravity[1] != 0.0 || p.gravity[2] != 0.0;
    for (int a = 0; a < 3; ++a) P.g[a] = static_cast<float>(p.gravity[a]);
    P.jet_c0 = static_cast<float>(p.jet_center[0]);
    P.jet_c1 = static_cast<float>(p.jet_center[1]);
    P.jet_radius = static_cast<float>(p.jet_radius);
    P.jet_velocity = static_cast<float>(p.jet_velocity);
    P.noise_amp = static_cast<float>(p.jet_velocity * p.inlet_noise);
    P.jet_blue = p.jet_phase < 0.0;
    P.rho_r0 = static_cast<float>(p.rho_r0);
    P.rho_b0 = static_cast<float>(p.rho_b0);
    P.seed = p.seed;
    P.rho_scale = static_cast<float>(p.rho_scale);
    P.inv_rho_scale = p.rho_scale > 0 ? static_cast<float>(1.0 / p.rho_scale) : 0.0f;
    P.u_ref = static_cast<float>(p.u_ref);
    P.inv_u_ref = p.u_ref > 0 ? static_cast<float>(1.0 / p.u_ref) : 0.0f;
    P.pi_scale = static_cast<float>(p.pi_scale);
    P.inv_pi_scale = p.pi_scale > 0 ? static_cast<float>(1.0 / p.pi_scale) : 0.0f;
    P.rho_mean = static_cast<float>(0.5 * (p.rho_r0 + p.rho_b0));
    P.rho_half_diff = static_cast<float>(0.5 * (p.rho_r0 - p.rho_b0));
    P.do_bc = 1;
    P.ghost_images = 1;
}

int choose_zchunk(const mbcg_params& p, int W) {
    if (const char* env = std::getenv("MBCG_ZCHUNK")) {
        const int v = std::atoi(env);
        if (v > 0) return v;
    }
    const long long gx = (p.nx - 2 + kStepTileX - 1) / kStepTileX;
    const long long gy = (p.ny - 2 + W - 3) / (W - 2);
    const int nzf = p.nz - 2;
    int sms = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // W = 16: one CTA per SM (W = 8: two).  Pick the number of z chunks that best fills whole
    // waves, charging each chunk the three extra planes it stages before its first destination
    // plane.
    sms *= W == kStepWSmall ? 2 : 1;
    double best = -1.0;
    int best_chunk = nzf;
    for (long long gz = 1; gz <= std::max(1, nzf / 8); ++gz) {
        const long long chunk = (nzf + gz - 1) / gz;
        const long long gzr = (nzf + chunk - 1) / chunk;
        const long long ctas = gx * gy * gzr;
        const long long waves = (ctas + sms - 1) / sms;
        const double fill = static_cast<double>(ctas) / static_cast<double>(waves * sms);
        const double eff = fill * static_cast<double>(chunk) / static_cast<double>(chunk + 3);
        if (eff > best + 1e-9) {
            best = eff;
            best_chunk = static_cast<int>(chunk);
        }
    }
    return best_chunk;
}

// ---------------------------------------------------------------- tensor maps
using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                              const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn get_encode() {
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(ptr);
    });
    return fn;
}

bool tma_capable(const mbcg_params& p, const void* const* f, long long pitch, int precision) {
    if (std::getenv("MBCG_NO_TMA")) return false;
    const int es = elem_bytes(precision);
    if ((pitch * es) % 16 != 0) return false;
    for (int i = 0; i < NF; ++i)
        if (reinterpret_cast<uintptr_t>(f[i]) % 16 != 0) return false;
    return get_encode() != nullptr;
}

// TMA descriptors of one state for step CTAs of W rows: rhor / rhob boxes kStepRBX x (W+2),
// the other fields kStepMX x W, one plane deep
int encode_maps(const mbcg_params& p, const void* const* f, long long pitch, int precision, int W, TensorMaps& T) {
    EncodeFn enc = get_encode();
    if (!enc) return fail(MBCG_E_CUDA, "cuTensorMapEncodeTiled unavailable");
    const int es = elem_bytes(precision);
    for (int i = 0; i < NF; ++i) {
        const cuuint64_t dims[3] = {static_cast<cuuint64_t>(p.nx), static_cast<cuuint64_t>(p.ny),
                                    static_cast<cuuint64_t>(p.nz)};
        const cuuint64_t strides[2] = {static_cast<cuuint64_t>(pitch * es),
                                       static_cast<cuuint64_t>(pitch * p.ny * es)};
        const cuuint32_t box[3] = {static_cast<cuuint32_t>(i < 2 ? kStepRBX : kStepMX),
                                   static_cast<cuuint32_t>(i < 2 ? W + 2 : W), 1u};
        const cuuint32_t estr[3] = {1u, 1u, 1u};
        const CUresult r = enc(&T.m[i], es == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 3,
                               const_cast<void*>(f[i]), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(MBCG_E_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(r) + ")");
    }
    return MBCG_OK;
}

// ---------------------------------------------------------------- tuned shapes
// Process-wide table of the shapes mbcg_autotune() measured, keyed by everything that changes
// the kernel's work per node: lattice, storage precision, sizes and feature set.
struct ShapeKey {
    int q, precision, nx, ny, nz, features;
    bool operator<(const ShapeKey& o) const {
        return std::tie(q, precision, nx, ny, nz, features) < std::tie(o.q, o.precision, o.nx, o.ny, o.nz, o.features);
    }
};
std::mutex g_tune_mu;
std::map<ShapeKey, std::pair<int, int>> g_tuned;

ShapeKey shape_key(const mbcg_params& p) {
    StepParams P;
    fill_physics(p, P);
    return ShapeKey{p.q, p.precision, p.nx, p.ny, p.nz, features_of(P)};
}

bool tuned_shape(const mbcg_params& p, int* w, int* zchunk) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(shape_key(p));
    if (it == g_tuned.end()) return false;
    *w = it->second.first;
    *zchunk = it->second.second;
    return true;
}

} // namespace

void mbcg::set_last_error(const std::string& msg) { g_err = msg; }
int mbcg::validate_params(const mbcg_params* p) { return validate(p); }
void mbcg::fill_step_physics(const mbcg_params& p, StepParams& P) { fill_physics(p, P); }
bool mbcg::state_tma_capable(const mbcg_params& p, const void* const* f, long long pitch) {
    return tma_capable(p, f, pitch, p.precision);
}
int mbcg::encode_state_maps(const mbcg_params& p, const void* const* f, long long pitch, int W, TensorMaps& T) {
    return encode_maps(p, f, pitch, p.precision, W, T);
}

struct mbcg_case {
    mbcg_params p;
    int es = 4;
    long long pitch = 0, plane = 0, fstride = 0;
    void* buf[2] = {nullptr, nullptr};
    void* fields[2][NF] = {};
    int cur = 0;
    bool tma = false;
    TensorMaps tm[2];
    int* status = nullptr;
    double* diag_partials = nullptr;
    double* diag_result = nullptr;
    int nparts = 0;
    long long steps = 0;
    int w = kStepW;   // step CTA rows
    int zchunk = 16;  // destination planes per step CTA
    float* stage = nullptr; // two dense FP32 fields for host copies, allocated on first use
    // mbcg_run_host: dense FP32 images of input and output states (two of each, or one where
    // the device has no room for two), the two copy streams and the images' events (allocated
    // on first use)
    float* dense_in[2] = {nullptr, nullptr};
    float* dense_out[2] = {nullptr, nullptr};
    int images = 0;
    cudaStream_t s_h2d = nullptr, s_d2h = nullptr;
    cudaEvent_t ev_in_ready[2] = {}, ev_in_free[2] = {}, ev_out_ready[2] = {}, ev_out_free[2] = {};
};

namespace {

StepParams make_params(const mbcg_case* c, int from, long long step) {
    StepParams P;
    fill_physics(c->p, P);
    P.pitch = c->pitch;
    P.plane = c->plane;
    P.zchunk = c->zchunk;
    P.status = c->status;
    P.step = step;
    for (int i = 0; i < NF; ++i) {
        P.a[i] = c->fields[from][i];
        P.b[i] = c->fields[from ^ 1][i];
    }
    return P;
}

void free_case(mbcg_case* c) {
    if (!c) return;
    for (int s = 0; s < 2; ++s)
        if (c->buf[s]) cudaFree(c->buf[s]);
    if (c->status) cudaFree(c->status);
    if (c->diag_partials) cudaFree(c->diag_partials);
    if (c->diag_result) cudaFree(c->diag_result);
    if (c->stage) cudaFree(c->stage);
    for (int b = 0; b < 2; ++b) {
        if (c->dense_in[b]) cudaFree(c->dense_in[b]);
        if (c->dense_out[b]) cudaFree(c->dense_out[b]);
        for (cudaEvent_t e : {c->ev_in_ready[b], c->ev_in_free[b], c->ev_out_ready[b], c->ev_out_free[b]})
            if (e) cudaEventDestroy(e);
    }
    if (c->s_h2d) cudaStreamDestroy(c->s_h2d);
    if (c->s_d2h) cudaStreamDestroy(c->s_d2h);
    delete c;
}

int* g_raw_status = nullptr; // status word of the raw entry points, allocated once per process
std::mutex g_raw_mu;

int* raw_status() {
    std::lock_guard<std::mutex> lk(g_raw_mu);
    if (!g_raw_status) {
        if (cudaMalloc(&g_raw_status, sizeof(int)) != cudaSuccess) {
            g_raw_status = nullptr;
            return nullptr;
        }
        cudaMemset(g_raw_status, 0, sizeof(int));
    }
    return g_raw_status;
}

int check_view(const mbcg_params* p, const mbcg_moments* m) {
    if (!m) return fail(MBCG_E_INVALID, "null moments view");
    if (m->precision != p->precision) return fail(MBCG_E_INVALID, "moments precision differs from params");
    if (m->pitch < p->nx) return fail(MBCG_E_INVALID, "pitch smaller than nx");
    for (int i = 0; i < NF; ++i)
        if (!m->f[i]) return fail(MBCG_E_INVALID, "null field pointer");
    return MBCG_OK;
}

StepParams raw_params(const mbcg_params* p, const mbcg_moments* a, const mbcg_moments* b, long long step) {
    StepParams P;
    fill_physics(*p, P);
    P.pitch = b ? b->pitch : a->pitch;
    P.plane = P.pitch * p->ny;
    P.zchunk = choose_zchunk(*p, kStepW);
    P.step = step;
    P.status = raw_status();
    for (int i = 0; i < NF; ++i) {
        P.a[i] = a ? a->f[i] : nullptr;
        P.b[i] = b ? b->f[i] : nullptr;
    }
    return P;
}

} // namespace

// Copies the current state into the other one.  A step never writes the wall ghost layers (or
// nodes outside every boundary rule), so after this both states agree there for good and the
// full box read back does not depend on the parity of the step count.
int mbcg::mirror_state(mbcg_case* c, cudaStream_t s) {
    const size_t bytes = static_cast<size_t>(c->fstride) * NF * c->es;
    MBCG_TRY(cudaMemcpyAsync(c->buf[c->cur ^ 1], c->buf[c->cur], bytes, cudaMemcpyDeviceToDevice, s), "state mirror");
    return MBCG_OK;
}

int mbcg::case_state_params(mbcg_case* c, StepParams* out) {
    if (!c || !out) return fail(MBCG_E_INVALID, "null argument");
    *out = make_params(c, c->cur, c->steps); // P.a = current state
    return MBCG_OK;
}

int mbcg::case_field_to_dense(mbcg_case* c, int field, float* dst, cudaStream_t s) {
    if (!c || !dst || field < 0 || field >= NF) return fail(MBCG_E_INVALID, "bad field snapshot request");
    StepParams P = make_params(c, c->cur, c->steps); // P.a = current state
    MBCG_TRY(launch_to_dense(c->p.precision, P, field, dst, s), "field snapshot");
    return MBCG_OK;
}
void mbcg::case_set_steps(mbcg_case* c, long long steps) {
    if (c) c->steps = steps;
}

extern "C" {

void mbcg_params_default(mbcg_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->q = 27;
    p->nx = p->ny = p->nz = 128;
    p->bc[0] = MBCG_BC_PERIODIC;
    p->bc[1] = MBCG_BC_INOUT;
    p->bc[2] = MBCG_BC_PERIODIC;
    p->outlet = MBCG_OUTLET_CONVECTIVE;
    p->precision = MBCG_FP32;
    p->ic = MBCG_IC_JET;
    p->tau = 1.0;
    p->sigma = 0.1;
    p->beta = 0.9;
    p->rho_r0 = p->rho_b0 = 1.0;
    p->jet_radius = 12.0;
    p->jet_velocity = 0.05;
    p->jet_center[0] = (p->nx - 1) / 2.0;
    p->jet_center[1] = (p->nz - 1) / 2.0;
    p->jet_phase = -1.0;
    p->seed = 12345;
    p->bubble_radius = 30.0;
    for (int a = 0; a < 3; ++a) p->bubble_center[a] = (127) / 2.0;
    p->bubble_phase = -1.0;
    p->rti_position = (p->ny - 1) / 2.0;
    p->rti_amplitude = 4.0;
    p->rti_width = 4.0;
    p->rti_phase_above = -1.0;
    p->rti_mode[0] = p->rti_mode[1] = 1;
    p->rho_scale = 0.01;
    p->u_ref = 0.05;
    p->pi_scale = 0.05 * 0.05;
}

int mbcg_create(const mbcg_params* p, mbcg_case** out) {
    if (!out) return fail(MBCG_E_INVALID, "null output handle");
    *out = nullptr;
    if (int rc = validate(p)) return rc;
    mbcg_case* c = new mbcg_case();
    c->p = *p;
    c->es = elem_bytes(p->precision);
    c->pitch = (p->nx + 7) / 8 * 8;
    c->plane = c->pitch * p->ny;
    const long long per_field = c->plane * p->nz;
    c->fstride = (per_field * c->es + 255) / 256 * 256 / c->es;
    const size_t bytes = static_cast<size_t>(c->fstride) * NF * c->es;
    for (int s = 0; s < 2; ++s) {
        cudaError_t e = cudaMalloc(&c->buf[s], bytes);
        if (e != cudaSuccess) {
            free_case(c);
            return fail(MBCG_E_NOMEM, std::string("cudaMalloc of a moment state failed: ") + cudaGetErrorString(e));
        }
        cudaMemset(c->buf[s], 0, bytes);
        for (int i = 0; i < NF; ++i)
            c->fields[s][i] = static_cast<unsigned char*>(c->buf[s]) + static_cast<size_t>(i) * c->fstride * c->es;
    }
    if (cudaMalloc(&c->status, sizeof(int)) != cudaSuccess) {
        free_case(c);
        return fail(MBCG_E_NOMEM, "cudaMalloc of the status word failed");
    }
    cudaMemset(c->status, 0, sizeof(int));
    if (!tuned_shape(*p, &c->w, &c->zchunk)) {
        c->w = kStepW;
        c->zchunk = choose_zchunk(*p, c->w);
    }
    {
        StepParams P = make_params(c, 0, 0);
        c->nparts = diag_partials_needed(P);
    }
    if (cudaMalloc(&c->diag_partials, sizeof(double) * kDiagSlots * c->nparts) != cudaSuccess ||
        cudaMalloc(&c->diag_result, sizeof(double) * kDiagSlots) != cudaSuccess) {
        free_case(c);
        return fail(MBCG_E_NOMEM, "cudaMalloc of the diagnostics buffers failed");
    }
    c->tma = tma_capable(*p, c->fields[0], c->pitch, p->precision) &&
             tma_capable(*p, c->fields[1], c->pitch, p->precision);
    if (c->tma) {
        for (int s = 0; s < 2; ++s)
            if (int rc = encode_maps(*p, c->fields[s], c->pitch, p->precision, c->w, c->tm[s])) {
                free_case(c);
                return rc;
            }
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        free_case(c);
        return cuda_fail(e, "mbcg_create");
    }
    *out = c;
    return MBCG_OK;
}

int mbcg_destroy(mbcg_case* c) {
    if (!c) return MBCG_OK;
    cudaDeviceSynchronize();
    free_case(c);
    return MBCG_OK;
}

int mbcg_init(mbcg_case* c, mbcg_stream_t s) {
    if (!c) return fail(MBCG_E_INVALID, "null case");
    StepParams P = make_params(c, c->cur ^ 1, 0); // P.b = current state A
    MBCG_TRY(launch_init(c->p.precision, P, c->p, reinterpret_cast<cudaStream_t>(s)), "initial condition");
    if (int rc = mirror_state(c, reinterpret_cast<cudaStream_t>(s))) return rc;
    c->steps = 0;
    return MBCG_OK;
}

int mbcg_step(mbcg_case* c, int32_t nsteps, mbcg_stream_t s) {
    if (!c) return fail(MBCG_E_INVALID, "null case");
    if (nsteps < 0) return fail(MBCG_E_INVALID, "negative step count");
    for (int n = 0; n < nsteps; ++n) {
        StepParams P = make_params(c, c->cur, c->steps + 1);
        MBCG_TRY(launch_step(c->p.q, c->p.precision, c->tma, c->w, P, c->tm[c->cur], reinterpret_cast<cudaStream_t>(s)),
                 "step kernel");
        c->cur ^= 1;
        c->steps += 1;
    }
    return MBCG_OK;
}

int mbcg_rcs(mbcg_case* c, mbcg_stream_t s) {
    if (!c) return fail(MBCG_E_INVALID, "null case");
    StepParams P = make_params(c, c->cur, c->steps + 1);
    P.do_bc = 0;
    MBCG_TRY(launch_step(c->p.q, c->p.precision, c->tma, c->w, P, c->tm[c->cur], reinterpret_cast<cudaStream_t>(s)),
             "RCS kernel");
    return MBCG_OK;
}

int mbcg_bc(mbcg_case* c, mbcg_stream_t s) {
    if (!c) return fail(MBCG_E_INVALID, "null case");
    StepParams P = make_params(c, c->cur, c->steps + 1); // a = old state, b = new state
    MBCG_TRY(launch_bc(c->p.precision, P, reinterpret_cast<cudaStream_t>(s)), "boundary kernel");
    return MBCG_OK;
}

int mbcg_swap(mbcg_case* c) {
    if (!c) return fail(MBCG_E_INVALID, "null case");
    c->cur ^= 1;
    c->steps += 1;
    return MBCG_OK;
}

int mbcg_fields(const mbcg_case* c, mbcg_moments* a, mbcg_moments* b) {
    if (!c) return fail(MBCG_E_INVALID, "null case");
    for (int w = 0; w < 2; ++w) {
        mbcg_moments* m = w == 0 ? a : b;
        if (!m) continue;
        const int s = w == 0 ? c->cur : (c->cur ^ 1);
        for (int i = 0; i < NF; ++i) m->f[i] = c->fields[s][i];
        m->pitch = c->pitch;
        m->precision = c->p.precision;
        m->reserved = 0;
    }
    return MBCG_OK;
}

int64_t mbcg_steps_done(const mbcg_case* c) { return c ? c->steps : -1; }

int mbcg_case_params(const mbcg_case* c, mbcg_params* out) {
    if (!c || !out) return fail(MBCG_E_INVALID, "null argument");
    *out = c->p;
    return MBCG_OK;
}

// Device pointers of the host fields when every one is pinned host memory the device can
// access directly; false for pageable memory.
static bool host_fields_on_device(const float* const host[MBCG_NFIELDS], float* dev[MBCG_NFIELDS]) {
    for (int i = 0; i < NF; ++i) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, host[i]) != cudaSuccess) {
            cudaGetLastError(); // clear it: not an error of the copy
            return false;
        }
        if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr) return false;
        dev[i] = static_cast<float*>(a.devicePointer);
    }
    return true;
}

// Host copies.  Pinned host fields are read or written by one kernel that also converts the
// layout (all 11 fields, at the host link's bandwidth, no staging).  Pageable fields move one
// whole dense field per transfer (one contiguous copy: the reference's dense rows of nx floats
// would otherwise be copied row by row as a pitched 2-D transfer) through a pair of dense device
// fields, converted on the device.
int mbcg_copy_out(mbcg_case* c, float* const host[MBCG_NFIELDS], mbcg_stream_t s) {
    if (!c || !host) return fail(MBCG_E_INVALID, "null argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    const mbcg_params& p = c->p;
    const size_t n = static_cast<size_t>(p.nx) * p.ny * p.nz;
    StepParams P = make_params(c, c->cur, c->steps); // P.a = current state
    float* dev[MBCG_NFIELDS];
    if (host_fields_on_device(host, dev)) {
        MBCG_TRY(launch_state_to_host(p.precision, P, dev, st), "copy out");
        MBCG_TRY(cudaStreamSynchronize(st), "copy out");
        return MBCG_OK;
    }
    if (!c->stage) MBCG_TRY(cudaMalloc(&c->stage, 2 * n * sizeof(float)), "staging allocation");
    for (int i = 0; i < NF; ++i) {
        float* buf = c->stage + (i & 1) * n; // reused two fields later, in stream order
        MBCG_TRY(launch_to_dense(p.precision, P, i, buf, st), "copy out");
        MBCG_TRY(cudaMemcpyAsync(host[i], buf, n * sizeof(float), cudaMemcpyDeviceToHost, st), "copy out");
    }
    MBCG_TRY(cudaStreamSynchronize(st), "copy out");
    return MBCG_OK;
}

int mbcg_copy_in(mbcg_case* c, const float* const host[MBCG_NFIELDS], mbcg_stream_t s) {
    if (!c || !host) return fail(MBCG_E_INVALID, "null argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    const mbcg_params& p = c->p;
    const size_t n = static_cast<size_t>(p.nx) * p.ny * p.nz;
    StepParams P = make_params(c, c->cur ^ 1, c->steps); // P.b = current state
    float* dev[MBCG_NFIELDS];
    if (host_fields_on_device(host, dev)) {
        MBCG_TRY(launch_host_to_state(p.precision, P, dev, st), "copy in");
        MBCG_TRY(launch_fill_ghosts(p.precision, P, st), "ghost images");
        MBCG_TRY(cudaStreamSynchronize(st), "copy in");
        return MBCG_OK;
    }
    if (!c->stage) MBCG_TRY(cudaMalloc(&c->stage, 2 * n * sizeof(float)), "staging allocation");
    const bool pair = p.precision != MBCG_FP32; // rhor and rhob convert together
    for (int i = 0; i < NF; ++i) {
        float* buf = c->stage + (i & 1) * n;
        MBCG_TRY(cudaMemcpyAsync(buf, host[i], n * sizeof(float), cudaMemcpyHostToDevice, st), "copy in");
        if (pair && i == 0) continue; // converted with field 1
        if (pair && i == 1) MBCG_TRY(launch_from_dense(p.precision, P, 0, c->stage, c->stage + n, st), "copy in");
        else MBCG_TRY(launch_from_dense(p.precision, P, i, buf, nullptr, st), "copy in");
    }
    MBCG_TRY(launch_fill_ghosts(p.precision, P, st), "ghost images");
    MBCG_TRY(cudaStreamSynchronize(st), "copy in");
    return MBCG_OK;
}

// mbcg_run_host: for j = 0..count-1 the same bits as copy_in(in[j]); step(nsteps);
// copy_out(out[j]).  Host arrays move by the copy engines between pinned host memory and dense
// device images of the input and output states, on two streams of their own; the layout
// conversions and the steps run on the caller's stream.  With two images each way, state j+1
// moves in while state j is stepped and state j-1 moves out, so the host link carries both
// directions at once and the copies never wait for a conversion.  Dependencies (events per
// image b): an input image is refilled only after its conversion into the state (in_free[b]),
// the conversion waits for the fill (in_ready[b]); an output image is rewritten only after its
// copy to the host (out_free[b]), the copy waits for the conversion (out_ready[b]).
// the 11 host fields follow one another in one array (field f at field 0 + f n)
static bool contiguous(const float* const* h, size_t n) {
    for (int f = 1; f < NF; ++f)
        if (h[f] != h[0] + f * n) return false;
    return true;
}

static int host_run_images(mbcg_case* c, size_t bytes) {
    if (c->images) return MBCG_OK;
    MBCG_TRY(cudaStreamCreateWithFlags(&c->s_h2d, cudaStreamNonBlocking), "host-run stream");
    MBCG_TRY(cudaStreamCreateWithFlags(&c->s_d2h, cudaStreamNonBlocking), "host-run stream");
    for (int b = 0; b < 2; ++b)
        for (cudaEvent_t* e : {&c->ev_in_ready[b], &c->ev_in_free[b], &c->ev_out_ready[b], &c->ev_out_free[b]})
            MBCG_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "host-run event");
    for (int want = 2; want >= 1; --want) {
        bool ok = true;
        for (int b = 0; b < want && ok; ++b)
            ok = cudaMalloc(&c->dense_in[b], bytes) == cudaSuccess && cudaMalloc(&c->dense_out[b], bytes) == cudaSuccess;
        if (ok) {
            c->images = want;
            return MBCG_OK;
        }
        cudaGetLastError(); // out of memory: try one image each way
        for (int b = 0; b < 2; ++b) {
            if (c->dense_in[b]) cudaFree(c->dense_in[b]);
            if (c->dense_out[b]) cudaFree(c->dense_out[b]);
            c->dense_in[b] = c->dense_out[b] = nullptr;
        }
    }
    return fail(MBCG_E_NOMEM, "no device memory for the host-run images");
}

int mbcg_run_host(mbcg_case* c, int32_t count, const float* const* in, float* const* out, int32_t nsteps,
                  mbcg_stream_t s) {
    if (!c || (count > 0 && (!in || !out))) return fail(MBCG_E_INVALID, "null argument");
    if (count < 0 || nsteps < 0) return fail(MBCG_E_INVALID, "negative count");
    if (count == 0) return MBCG_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    const mbcg_params& p = c->p;
    const size_t n = static_cast<size_t>(p.nx) * p.ny * p.nz;
    const size_t field_bytes = n * sizeof(float);
    if (int e = host_run_images(c, NF * field_bytes)) return e;
    // the images are free once everything the caller queued before is done
    for (int b = 0; b < c->images; ++b) {
        MBCG_TRY(cudaEventRecord(c->ev_in_free[b], st), "host-run event");
        MBCG_TRY(cudaEventRecord(c->ev_out_free[b], st), "host-run event");
    }
    for (int j = 0; j < count; ++j) {
        const int b = j % c->images;
        const float* const* hin = in + static_cast<size_t>(j) * NF;
        float* const* hout = out + static_cast<size_t>(j) * NF;
        float* din[MBCG_NFIELDS];
        float* dout[MBCG_NFIELDS];
        for (int f = 0; f < NF; ++f) {
            din[f] = c->dense_in[b] + f * n;
            dout[f] = c->dense_out[b] + f * n;
        }
        // host -> input image (one transfer when the host fields are one contiguous array)
        MBCG_TRY(cudaStreamWaitEvent(c->s_h2d, c->ev_in_free[b], 0), "host-run order");
        if (contiguous(hin, n))
            MBCG_TRY(cudaMemcpyAsync(din[0], hin[0], NF * field_bytes, cudaMemcpyHostToDevice, c->s_h2d), "host-run copy in");
        else
            for (int f = 0; f < NF; ++f)
                MBCG_TRY(cudaMemcpyAsync(din[f], hin[f], field_bytes, cudaMemcpyHostToDevice, c->s_h2d), "host-run copy in");
        MBCG_TRY(cudaEventRecord(c->ev_in_ready[b], c->s_h2d), "host-run event");
        // input image -> state (as mbcg_copy_in), steps
        MBCG_TRY(cudaStreamWaitEvent(st, c->ev_in_ready[b], 0), "host-run order");
        {
            StepParams P = make_params(c, c->cur ^ 1, c->steps); // P.b = current state
            MBCG_TRY(launch_host_to_state(p.precision, P, din, st), "host-run copy in");
            MBCG_TRY(launch_fill_ghosts(p.precision, P, st), "ghost images");
        }
        MBCG_TRY(cudaEventRecord(c->ev_in_free[b], st), "host-run event");
        if (int e = mbcg_step(c, nsteps, s)) return e;
        // state -> output image (as mbcg_copy_out) -> host
        MBCG_TRY(cudaStreamWaitEvent(st, c->ev_out_free[b], 0), "host-run order");
        {
            StepParams P = make_params(c, c->cur, c->steps); // P.a = current state
            MBCG_TRY(launch_state_to_host(p.precision, P, dout, st), "host-run copy out");
        }
        MBCG_TRY(cudaEventRecord(c->ev_out_ready[b], st), "host-run event");
        MBCG_TRY(cudaStreamWaitEvent(c->s_d2h, c->ev_out_ready[b], 0), "host-run order");
        if (contiguous(hout, n))
            MBCG_TRY(cudaMemcpyAsync(hout[0], dout[0], NF * field_bytes, cudaMemcpyDeviceToHost, c->s_d2h), "host-run copy out");
        else
            for (int f = 0; f < NF; ++f)
                MBCG_TRY(cudaMemcpyAsync(hout[f], dout[f], field_bytes, cudaMemcpyDeviceToHost, c->s_d2h), "host-run copy out");
        MBCG_TRY(cudaEventRecord(c->ev_out_free[b], c->s_d2h), "host-run event");
    }
    MBCG_TRY(cudaStreamSynchronize(c->s_d2h), "host-run copy out");
    MBCG_TRY(cudaStreamSynchronize(st), "host-run");
    return MBCG_OK;
}

int mbcg_diagnostics(mbcg_case* c, mbcg_diag* out, mbcg_stream_t s) {
    if (!c || !out) return fail(MBCG_E_INVALID, "null argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    StepParams P = make_params(c, c->cur, c->steps);
    MBCG_TRY(launch_diag(c->p.precision, P, c->p, c->diag_partials, c->nparts, c->diag_result, st), "diagnostics");
    double r[kDiagSlots];
    MBCG_TRY(cudaMemcpyAsync(r, c->diag_result, sizeof(r), cudaMemcpyDeviceToHost, st), "diagnostics copy");
    MBCG_TRY(cudaStreamSynchronize(st), "diagnostics");
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

int mbcg_status(mbcg_case* c, int32_t* status) {
    if (!c || !status) return fail(MBCG_E_INVALID, "null argument");
    int v = 0;
    MBCG_TRY(cudaMemcpy(&v, c->status, sizeof(int), cudaMemcpyDeviceToHost), "status read");
    MBCG_TRY(cudaMemset(c->status, 0, sizeof(int)), "status clear");
    *status = v;
    return MBCG_OK;
}

int mbcg_rcs_moments(const mbcg_params* p, const mbcg_moments* a, const mbcg_moments* b, int64_t step,
                     mbcg_stream_t s) {
    if (int rc = validate(p)) return rc;
    if (int rc = check_view(p, a)) return rc;
    if (int rc = check_view(p, b)) return rc;
    if (a->pitch != b->pitch) return fail(MBCG_E_INVALID, "A and B must share a pitch");
    StepParams P = raw_params(p, a, b, step);
    P.do_bc = 0;
    {
        // the step reads wrapped sources from the ghost frame: fill it on the caller's state A
        // (the reference never reads its periodic ghost layers, so this changes none of its data)
        StepParams G = raw_params(p, nullptr, a, step);
        MBCG_TRY(launch_fill_ghosts(p->precision, G, reinterpret_cast<cudaStream_t>(s)), "ghost images");
    }
    TensorMaps T;
    std::memset(&T, 0, sizeof(T));
    const bool tma = tma_capable(*p, a->f, a->pitch, p->precision);
    if (tma)
        if (int rc = encode_maps(*p, a->f, a->pitch, p->precision, kStepW, T)) return rc;
    MBCG_TRY(launch_step(p->q, p->precision, tma, kStepW, P, T, reinterpret_cast<cudaStream_t>(s)), "RCS kernel");
    return MBCG_OK;
}

int mbcg_bc_moments(const mbcg_params* p, const mbcg_moments* b, const mbcg_moments* a_old, int64_t step,
                    mbcg_stream_t s) {
    if (int rc = validate(p)) return rc;
    if (int rc = check_view(p, b)) return rc;
    if (int rc = check_view(p, a_old)) return rc;
    if (a_old->pitch != b->pitch) return fail(MBCG_E_INVALID, "A and B must share a pitch");
    StepParams P = raw_params(p, a_old, b, step);
    MBCG_TRY(launch_bc(p->precision, P, reinterpret_cast<cudaStream_t>(s)), "boundary kernel");
    return MBCG_OK;
}

int mbcg_init_moments(const mbcg_params* p, const mbcg_moments* a, mbcg_stream_t s) {
    if (int rc = validate(p)) return rc;
    if (int rc = check_view(p, a)) return rc;
    StepParams P = raw_params(p, nullptr, a, 0);
    MBCG_TRY(launch_init(p->precision, P, *p, reinterpret_cast<cudaStream_t>(s)), "initial condition");
    return MBCG_OK;
}

int mbcg_get_shape(const mbcg_case* c, int32_t* block_rows, int32_t* zchunk) {
    if (!c || !block_rows || !zchunk) return fail(MBCG_E_INVALID, "null argument");
    *block_rows = c->w;
    *zchunk = c->zchunk;
    return MBCG_OK;
}

int mbcg_set_shape(mbcg_case* c, int32_t block_rows, int32_t zchunk) {
    if (!c) return fail(MBCG_E_INVALID, "null case");
    if (block_rows != kStepW && block_rows != kStepWSmall) return fail(MBCG_E_INVALID, "block_rows must be 8 or 16");
    if (zchunk < 1) return fail(MBCG_E_INVALID, "zchunk must be positive");
    if (block_rows != c->w && c->tma) {
        TensorMaps t[2];
        for (int s = 0; s < 2; ++s)
            if (int rc = encode_maps(c->p, c->fields[s], c->pitch, c->p.precision, block_rows, t[s])) return rc;
        c->tm[0] = t[0];
        c->tm[1] = t[1];
    }
    c->w = block_rows;
    c->zchunk = std::min<int>(zchunk, c->p.nz - 2);
    return MBCG_OK;
}

// Times the step for each candidate shape on this case and keeps the fastest.  Every timed
// launch reads the current state and writes the other one (the state a step would overwrite
// anyway), so the current state is unchanged.
int mbcg_autotune(mbcg_case* c, int32_t repeats, double* best_ms, mbcg_stream_t s) {
    if (!c) return fail(MBCG_E_INVALID, "null case");
    if (repeats < 1) repeats = 3;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    const int nzf = c->p.nz - 2;
    std::vector<std::pair<int, int>> cands;
    for (int w : {kStepW, kStepWSmall}) {
        std::vector<int> zs = {choose_zchunk(c->p, w), 4, 8, 16, 32, 64, nzf};
        for (int z : zs) {
            z = std::max(1, std::min(z, nzf));
            if (std::find(cands.begin(), cands.end(), std::make_pair(w, z)) == cands.end()) cands.emplace_back(w, z);
        }
    }
    cudaEvent_t e0, e1;
    MBCG_TRY(cudaEventCreate(&e0), "event");
    MBCG_TRY(cudaEventCreate(&e1), "event");
    double best = 1e300;
    std::pair<int, int> pick(c->w, c->zchunk);
    int rc = MBCG_OK;
    for (const auto& cand : cands) {
        TensorMaps T;
        std::memset(&T, 0, sizeof(T));
        if (c->tma && (rc = encode_maps(c->p, c->fields[c->cur], c->pitch, c->p.precision, cand.first, T))) break;
        StepParams P = make_params(c, c->cur, c->steps + 1);
        P.zchunk = cand.second;
        cudaError_t e = launch_step(c->p.q, c->p.precision, c->tma, cand.first, P, T, st);
        if (e == cudaSuccess) e = cudaEventRecord(e0, st);
        for (int r = 0; r < repeats && e == cudaSuccess; ++r)
            e = launch_step(c->p.q, c->p.precision, c->tma, cand.first, P, T, st);
        if (e == cudaSuccess) e = cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "autotune");
            break;
        }
        const double per = ms / repeats;
        if (per < best) {
            best = per;
            pick = cand;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (int r2 = mbcg_set_shape(c, pick.first, pick.second)) return r2;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tuned[shape_key(c->p)] = pick;
    }
    if (best_ms) *best_ms = best;
    return MBCG_OK;
}

int64_t mbcg_active_nodes(const mbcg_params* p) {
    if (!p) return -1;
    return static_cast<int64_t>(p->nx - 2) * (p->ny - 2) * (p->nz - 2);
}

int32_t mbcg_launches_per_step(const mbcg_case* c) { return c ? 1 : 0; }

const char* mbcg_last_error(void) { return g_err.c_str(); }

const char* mbcg_version(void) { return "mbcg 0.1 (sm_103a)"; }

} // extern "C"
