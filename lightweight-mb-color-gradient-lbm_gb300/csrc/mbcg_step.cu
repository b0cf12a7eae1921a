// mbcg_step.cu -- dispatch of the plain fused step to its (lattice, storage) instantiation.
#include "mbcg_step.cuh"

namespace mbcg {

cudaError_t launch_step(int q, int precision, bool tma, int w, const StepParams& P, const TensorMaps& T,
                        cudaStream_t s) {
    if (w != kStepW && w != kStepWSmall) return cudaErrorInvalidValue;
    if (q == 27) {
        switch (precision) {
        case MBCG_FP16: return launch_step_q27_f16(tma, w, P, T, s);
        case MBCG_BF16: return launch_step_q27_bf16(tma, w, P, T, s);
        default: return launch_step_q27_f32(tma, w, P, T, s);
        }
    }
    switch (precision) {
    case MBCG_FP16: return launch_step_q19_f16(tma, w, P, T, s);
    case MBCG_BF16: return launch_step_q19_bf16(tma, w, P, T, s);
    default: return launch_step_q19_f32(tma, w, P, T, s);
    }
}

int step_smem_bytes(int precision, int w) {
    if (precision == MBCG_FP32) return w == kStepWSmall ? Geo<float, kStepWSmall>::smem : Geo<float, kStepW>::smem;
    return w == kStepWSmall ? Geo<__half, kStepWSmall>::smem : Geo<__half, kStepW>::smem;
}

} // namespace mbcg
