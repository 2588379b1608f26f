// Launchers of the Cholesky kernels with BF16-split tensor-core updates
// (k_chol_tc.cu).
#pragma once
#include <cuda.h>
#include <cstdint>
#include "kernels.cuh"

namespace uhm_gpu {

// 2D map over the chunk-major operand workspace: rows of 64 BF16 (128 bytes),
// box 64 x 128 rows, 128-byte swizzle
bool tcc_encode(CUtensorMap* map, void* base, int64_t rows);
// one outer panel of W1 (256 or 512) columns of every front in the item list
// (item: front, a = K0, b = row block relative to the panel, c = flag offset)
void launch_chol_panel(const DevCtx& c, const Item* items, int n_items, int w1, int* ticket, int* flags, int* err,
                       void* ws, const int64_t* ws_row0, cudaStream_t s);
// C -= P P^T over 128 x 256 tiles (item: front, a = r0, b = c0, c = kc0 | kc1 << 16)
void launch_tc_chol(const DevCtx& c, const CUtensorMap& map, const int64_t* ws_row0, const Item* items, int n_items,
                    int* err, cudaStream_t s);
constexpr int TCC_TILE_M = 128, TCC_TILE_N = 256;
constexpr int CP_FLAGS_PER_FRONT = 72;   // D[8] + R[8][8] of one front in one panel launch

}  // namespace uhm_gpu
