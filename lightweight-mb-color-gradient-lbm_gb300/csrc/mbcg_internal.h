// mbcg_internal.h -- declarations shared by the translation units of libmbcg.so.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <string>

#include "mbcg.h"
#include "mbcg_lattice.cuh"

namespace mbcg {

constexpr int kStepW = 16; // warps (rows) per step CTA: 14 destination rows + 2 halo rows

struct TensorMaps {
    CUtensorMap m[NF];
};

// fused step (mbcg_step.cu)
cudaError_t launch_step(int q, int precision, bool tma, const StepParams& P, const TensorMaps& T, cudaStream_t s);
int step_smem_bytes(int precision);
int step_box_rows();
int step_tile_x();
int step_rb_box_x();
int step_m_box_x();

// boundary functors, initial conditions, diagnostics, layout conversion (mbcg_aux.cu)
cudaError_t launch_bc(int precision, const StepParams& P, cudaStream_t s);
cudaError_t launch_fill_ghosts(int precision, const StepParams& P, cudaStream_t s); // on P.b
cudaError_t launch_init(int precision, const StepParams& P, const mbcg_params& p, cudaStream_t s);
cudaError_t launch_diag(int precision, const StepParams& P, const mbcg_params& p, double* partials, int nparts,
                        double* result, cudaStream_t s);
int diag_partials_needed(const StepParams& P);
cudaError_t launch_to_dense(int precision, const StepParams& P, int field, const void* src, float* dst,
                            cudaStream_t s);
cudaError_t launch_from_dense(int precision, const StepParams& P, int field, const float* src, void* dst,
                              cudaStream_t s);

// sets the message mbcg_last_error() returns on the calling thread (mbcg_capi.cu)
void set_last_error(const std::string& msg);

constexpr int kDiagSlots = 12; // mass_r, mass_b, mom x/y/z, p_in sum, n_in, p_out sum, n_out, nonfinite, nodes, spare

} // namespace mbcg
