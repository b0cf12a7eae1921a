// mbcg_batch.cu -- persistent batch step: one launch advances every live lattice of the server
// by one time step.
//
// The work is a flat queue of tiles (BatchTile) over all live lattices, sorted by the host
// (largest tiles first, grouped by body).  Each CTA of a grid of at most one CTA per SM takes
// the next tile with an atomic counter and runs the same step_tile() as the plain kernel,
// instantiated for the lattice's (Q, storage, feature set), on that lattice's step parameters in
// a constant-memory table indexed by slot.  The stage mbarriers are initialised once per CTA; their phase
// carries from tile to tile.
#include "mbcg_batch.h"
#include "mbcg_step.cuh"

namespace mbcg {

namespace {

__constant__ StepParams c_batch_params[kBatchParamSlots * 2]; // [slot][parity]

template <int W>
__global__ void __launch_bounds__(32 * W, 1)
    batch_kernel(const BatchCase* __restrict__ cases, const BatchTile* __restrict__ tiles, int ntiles,
                 const ChunkState* __restrict__ chunk, int* __restrict__ counters, int j) {
    __shared__ int s_tile;
    unsigned char* smem = aligned_smem_base();
    init_stage_barriers(smem);
    uint32_t phase = 0;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    for (;;) {
        __syncthreads(); // everyone is done with the previous tile's s_tile
        if (tid == 0) s_tile = atomicAdd(&counters[j], 1);
        __syncthreads();
        const int t = s_tile;
        if (t >= ntiles) return;
        const BatchTile bt = tiles[t];
        const ChunkState cs = chunk[bt.slot];
        if (j >= cs.nsteps) continue;
        const int par = cs.parity0 ^ (j & 1);
        const BatchCase& C = cases[bt.slot];
        const StepParams& sP = c_batch_params[bt.slot * 2 + par]; // this lattice, this parity
        const CUtensorMap* maps = C.maps[par];
        const long long step = cs.step0 + j + 1;
        bool ok = true;
        switch (C.kind) {
        case BK_Q19_F32: ok = step_tile<19, float, W, true, F_ALL, false>(sP, maps, bt.bx, bt.by, bt.bz, step, smem, phase); break;
        case BK_Q19_F16: ok = step_tile<19, __half, W, true, F_ALL, false>(sP, maps, bt.bx, bt.by, bt.bz, step, smem, phase); break;
        case BK_Q19_BF16: ok = step_tile<19, __nv_bfloat16, W, true, F_ALL, false>(sP, maps, bt.bx, bt.by, bt.bz, step, smem, phase); break;
        case BK_Q27_F32: ok = step_tile<27, float, W, true, F_ALL, false>(sP, maps, bt.bx, bt.by, bt.bz, step, smem, phase); break;
        case BK_Q27_F16: ok = step_tile<27, __half, W, true, F_ALL, false>(sP, maps, bt.bx, bt.by, bt.bz, step, smem, phase); break;
        case BK_Q27_BF16: ok = step_tile<27, __nv_bfloat16, W, true, F_ALL, false>(sP, maps, bt.bx, bt.by, bt.bz, step, smem, phase); break;
        case BK_Q19_F32_P: ok = step_tile<19, float, W, true, 0>(sP, maps, bt.bx, bt.by, bt.bz, step, smem, phase); break;
        case BK_Q19_F16_P: ok = step_tile<19, __half, W, true, 0>(sP, maps, bt.bx, bt.by, bt.bz, step, smem, phase); break;
        case BK_Q27_F32_P: ok = step_tile<27, float, W, true, 0>(sP, maps, bt.bx, bt.by, bt.bz, step, smem, phase); break;
        case BK_Q27_F16_P: ok = step_tile<27, __half, W, true, 0>(sP, maps, bt.bx, bt.by, bt.bz, step, smem, phase); break;
        default: ok = false; break;
        }
        if (!ok) return; // step_tile has set the lattice's status word
    }
}

// order-independent: sum over nodes of mix64(field, index, bits), wrapping
template <typename S>
__global__ void state_hash_kernel(const StepParams P, unsigned long long* out) {
    const long long nxf = P.nx - 2, nyf = P.ny - 2, nzf = P.nz - 2;
    const long long total = nxf * nyf * nzf;
    unsigned long long acc = 0;
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long x = 1 + e % nxf, y = 1 + (e / nxf) % nyf, z = 1 + e / (nxf * nyf);
        const long long o = z * P.plane + y * P.pitch + x;
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            unsigned long long bits;
            if constexpr (sizeof(S) == 4) bits = __float_as_uint(static_cast<const float*>(P.a[f])[o]);
            else bits = *reinterpret_cast<const unsigned short*>(static_cast<const S*>(P.a[f]) + o);
            acc += mix64((static_cast<unsigned long long>(e) * 16ULL + f) * 0x9E3779B97F4A7C15ULL ^ (bits << 1));
        }
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

} // namespace

int batch_smem_bytes() { return Geo<float, kBatchW>::smem; }

cudaError_t upload_batch_params(const StepParams* params, int n, cudaStream_t s) {
    if (n < 0 || n > kBatchParamSlots) return cudaErrorInvalidValue;
    return cudaMemcpyToSymbolAsync(c_batch_params, params, sizeof(StepParams) * 2 * n, 0, cudaMemcpyHostToDevice, s);
}

cudaError_t launch_batch(const BatchCase* cases, const BatchTile* tiles, int ntiles, const ChunkState* chunk,
                         int* counters, int j, int grid, cudaStream_t s) {
    auto kern = batch_kernel<kBatchW>;
    static std::atomic<unsigned long long> configured{0};
    if (cudaError_t e = configure_once(kern, batch_smem_bytes(), configured)) return e;
    if (grid < 1 || ntiles < 1) return cudaSuccess;
    kern<<<grid, dim3(32, kBatchW, 1), batch_smem_bytes(), s>>>(cases, tiles, ntiles, chunk, counters, j);
    return cudaGetLastError();
}

cudaError_t launch_state_hash(int precision, const StepParams& P, unsigned long long* out, cudaStream_t s) {
    const long long n = static_cast<long long>(P.nx - 2) * (P.ny - 2) * (P.nz - 2);
    const int grid = static_cast<int>(std::min<long long>((n + 255) / 256, 1184));
    switch (precision) {
    case MBCG_FP16: state_hash_kernel<__half><<<grid, 256, 0, s>>>(P, out); break;
    case MBCG_BF16: state_hash_kernel<__nv_bfloat16><<<grid, 256, 0, s>>>(P, out); break;
    default: state_hash_kernel<float><<<grid, 256, 0, s>>>(P, out); break;
    }
    return cudaGetLastError();
}

} // namespace mbcg
