// mbcg_batch.h -- device-side tables of the batch step (mbcg_batch.cu), shared with the server.
#pragma once

#include <cstdint>

#include "mbcg_internal.h"

namespace mbcg {

// Body of the batch kernel a lattice runs on: lattice, storage precision and feature set.
enum BatchKind : int {
    BK_Q19_F32 = 0, BK_Q19_F16, BK_Q19_BF16, BK_Q27_F32, BK_Q27_F16, BK_Q27_BF16, // every feature
    BK_Q19_F32_P, BK_Q19_F16_P, BK_Q27_F32_P, BK_Q27_F16_P,                      // fully periodic, unforced
    BK_COUNT
};

inline int batch_kind(int q, int precision, int features) {
    const bool lean = features == 0 && precision != MBCG_BF16;
    if (lean) return (q == 27 ? BK_Q27_F32_P : BK_Q19_F32_P) + (precision == MBCG_FP16 ? 1 : 0);
    return (q == 27 ? BK_Q27_F32 : BK_Q19_F32) + precision;
}

// One resident lattice: TMA descriptors and step parameters for both directions
// (parity s reads state s and writes state s^1).
struct BatchCase {
    CUtensorMap maps[2][NF];
    StepParams P[2];
    int kind;
    int pad[15];
};

// One unit of the flat tile queue: a (30 x 14 x zchunk) tile of the lattice in slot `slot`.
struct BatchTile {
    uint16_t slot, bx, by, bz;
};

// Per-slot progress for one graph replay: launch j of the replay advances the slot iff
// j < nsteps, reading state parity0 ^ (j & 1) and writing the state of index step0 + j + 1.
struct ChunkState {
    long long step0;
    int parity0;
    int nsteps;
};

constexpr int kBatchW = kStepW; // rows of the batch kernel's CTAs
// Lattices resident at once: the batch kernel reads each one's step parameters (both parities)
// from a constant-memory table of this many slots (2 x 64 x 392 bytes), as uniform loads the
// instructions take as operands, where a copy in shared memory costs a load into a register per use.
constexpr int kBatchParamSlots = 64;
// Copies n slots' parameters (StepParams[n][2], host memory valid until the copy has executed)
// into that table, in stream order.
cudaError_t upload_batch_params(const StepParams* params, int n, cudaStream_t s);

cudaError_t launch_batch(const BatchCase* cases, const BatchTile* tiles, int ntiles, const ChunkState* chunk,
                         int* counters, int j, int grid, cudaStream_t s);
int batch_smem_bytes();

// 64-bit order-independent hash of the fluid nodes (1..n-2 on every axis) of a state, added
// into *out (mbcg_batch.cu)
cudaError_t launch_state_hash(int precision, const StepParams& P, unsigned long long* out, cudaStream_t s);

} // namespace mbcg
