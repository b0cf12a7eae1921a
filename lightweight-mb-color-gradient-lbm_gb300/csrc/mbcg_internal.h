// mbcg_internal.h -- declarations shared by the translation units of libmbcg.so.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <string>

#include "mbcg.h"
#include "mbcg_lattice.cuh"

namespace mbcg {

// Step CTA shapes: W warps = W source rows (W-2 destination rows plus a halo row on each
// side) by 32 lanes (30 destination columns plus halo).  The plain step is built for both.
constexpr int kStepW = 16;     // default
constexpr int kStepWSmall = 8; // two CTAs per SM
constexpr int kStepTileX = 30; // destination columns per tile
constexpr int kStepRBX = 48;   // staged width of the rhor / rhob boxes
constexpr int kStepMX = 40;    // staged width of the other nine boxes

struct TensorMaps {
    CUtensorMap m[NF];
};

// fused step (mbcg_step.cu; instantiations in mbcg_step_q{19,27}_{f32,f16,bf16}.cu)
cudaError_t launch_step(int q, int precision, bool tma, int w, const StepParams& P, const TensorMaps& T,
                        cudaStream_t s);
cudaError_t launch_step_q19_f32(bool tma, int w, const StepParams& P, const TensorMaps& T, cudaStream_t s);
cudaError_t launch_step_q19_f16(bool tma, int w, const StepParams& P, const TensorMaps& T, cudaStream_t s);
cudaError_t launch_step_q19_bf16(bool tma, int w, const StepParams& P, const TensorMaps& T, cudaStream_t s);
cudaError_t launch_step_q27_f32(bool tma, int w, const StepParams& P, const TensorMaps& T, cudaStream_t s);
cudaError_t launch_step_q27_f16(bool tma, int w, const StepParams& P, const TensorMaps& T, cudaStream_t s);
cudaError_t launch_step_q27_bf16(bool tma, int w, const StepParams& P, const TensorMaps& T, cudaStream_t s);
int step_smem_bytes(int precision, int w);
inline int step_tile_rows(int w) { return w - 2; }

// boundary functors, initial conditions, diagnostics, layout conversion (mbcg_aux.cu)
cudaError_t launch_bc(int precision, const StepParams& P, cudaStream_t s);
cudaError_t launch_fill_ghosts(int precision, const StepParams& P, cudaStream_t s); // on P.b
cudaError_t launch_init(int precision, const StepParams& P, const mbcg_params& p, cudaStream_t s);
cudaError_t launch_diag(int precision, const StepParams& P, const mbcg_params& p, double* partials, int nparts,
                        double* result, cudaStream_t s);
int diag_partials_needed(const StepParams& P);
// one field between the state and the reference's dense FP32 layout (P.a -> dst; src -> P.b,
// where the 16-bit forms take rhor and rhob together as field 0 and skip field 1)
cudaError_t launch_to_dense(int precision, const StepParams& P, int field, float* dst, cudaStream_t s);
// all fields between the state (P.a for the read, P.b for the write) and dense FP32 fields in
// host memory the device accesses directly (device pointers of pinned host memory)
cudaError_t launch_state_to_host(int precision, const StepParams& P, float* const host[NF], cudaStream_t s);
cudaError_t launch_host_to_state(int precision, const StepParams& P, const float* const host[NF], cudaStream_t s);
cudaError_t launch_from_dense(int precision, const StepParams& P, int field, const float* src, const float* src_b,
                              cudaStream_t s);

// sets the message mbcg_last_error() returns on the calling thread (mbcg_capi.cu)
void set_last_error(const std::string& msg);
// one field of a case's current state as dense FP32 (reference layout) into dst, on stream s;
// the step counter of a case (restart from a checkpoint) (mbcg_capi.cu)
int case_field_to_dense(mbcg_case* c, int field, float* dst, cudaStream_t s);
int case_state_params(mbcg_case* c, StepParams* out); // parameter block with P.a = current state
int mirror_state(mbcg_case* c, cudaStream_t s); // current state -> the other (never-written layers agree)
void case_set_steps(mbcg_case* c, long long steps);
// parameter checks, the step's constant chain and TMA descriptors, shared by the case API and
// the server (mbcg_capi.cu); validate_params sets the last-error message on failure
int validate_params(const mbcg_params* p);
void fill_step_physics(const mbcg_params& p, StepParams& P);
bool state_tma_capable(const mbcg_params& p, const void* const* f, long long pitch);
int encode_state_maps(const mbcg_params& p, const void* const* f, long long pitch, int W, TensorMaps& T);

constexpr int kDiagSlots = 12; // mass_r, mass_b, mom x/y/z, p_in sum, n_in, p_out sum, n_out, nonfinite, nodes, spare

} // namespace mbcg
