// Plain step kernels for D3Q27 with float storage: block shapes W = 8 and 16, feature sets
// {none, inlet/outlet, all} on the TMA path and all features on the plain-load path.
#include "mbcg_step.cuh"

namespace mbcg {

cudaError_t launch_step_q27_f32(bool tma, int w, const StepParams& P, const TensorMaps& T, cudaStream_t s) {
    return launch_qs<27, float>(tma, w, P, T, s);
}

} // namespace mbcg
