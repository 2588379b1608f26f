// Tensor-core (tcgen05) Schur update: operand maps and launchers.
#pragma once
#include <cuda.h>
#include <cstdint>
#include "kernels.cuh"

namespace uhm_gpu {

constexpr int TC_NBO = 256;   // default outer panel width of fronts updated on tensor cores

bool tc_encode_part(CUtensorMap* map, void* base, int64_t rows, int nbo);
// trans = 0: the panel rows below the outer panel (A operand, parts poff..);
// trans = 1: the LU panel's U block right of it, transposed (B operand)
void launch_tc_pack(const DevCtx& c, const Item* items, int n_items, int nbo, int nparts, void* ws,
                    const int64_t* ws_off, const int64_t* ws_stride, int trans, int poff, cudaStream_t s);
void launch_tc_syrk(const DevCtx& c, const CUtensorMap& wsmap, const int64_t* ws_off,
                    const int64_t* ws_stride, const Item* items, int n_items, int nbo, int nterms,
                    uint32_t term_code, int lower_only, int* err, cudaStream_t s);
int tc_tile();

// term codes: 4 bits per term = (A part) | (B part) << 2
constexpr uint32_t TC_TERMS_BF16X3 = (0u | 0u << 2) | ((0u | 1u << 2) << 4) | ((1u | 0u << 2) << 8);
constexpr uint32_t TC_TERMS_BF16X6 = (0u | 0u << 2) | ((0u | 1u << 2) << 4) | ((1u | 0u << 2) << 8) |
                                     ((0u | 2u << 2) << 12) | ((1u | 1u << 2) << 16) |
                                     ((2u | 0u << 2) << 20);
// LU trailing update C -= L21 U12 in BF16X3: A parts 0-1 (L21), B parts 2-3 (U12^T)
constexpr uint32_t TC_TERMS_LU_BF16X3 = (0u | 2u << 2) | ((0u | 3u << 2) << 4) | ((1u | 2u << 2) << 8);

}  // namespace uhm_gpu
