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
// mode 0: C -= P P^T over 128 x 256 tiles (item: front, a = r0, b = c0, c = kc0 | kc1 << 16);
// mode 1: X = A Linv^T below a 256-column panel's diagonal block (item: front, a = r0, b = c0, c = K0)
// (reserve: SMs the persistent grid leaves free for a concurrent launch)
void launch_tc_chol(const DevCtx& c, const CUtensorMap& map, const int64_t* ws_row0, const Item* items, int n_items,
                    int* err, cudaStream_t s, int mode = 0, const int64_t* row0b = nullptr,
                    const int64_t* linv_row0 = nullptr, void* ws = nullptr, int reserve = 0, int pair = 0);
// a 256-column panel's diagonal block and its inverse as BF16 parts (item:
// front, a = K0, b = diagonal block, c = the front's slot of CD_HAND_WORDS
// hand-off words at hand; seq < CD_MAX_SEQ: the launch's number in its
// program, epoch: the factorisation count)
void launch_chol_diag(const DevCtx& c, const Item* items, int n_items, int* ticket, uint64_t* hand,
                      const unsigned* epoch, int seq, int* err, void* ws, const int64_t* linv_row0, cudaStream_t s);
// flags[0 .. n) = 0 and, when epoch is not null, *epoch += 1
void launch_clear_flags(int* flags, int n, unsigned* epoch, cudaStream_t s);
// BF16 parts of a 256-column panel's rows below its diagonal block (item:
// front, a = K0, b = first row, c = chunk of the panel)
void launch_chol_pack(const DevCtx& c, const Item* items, int n_items, void* ws, const int64_t* row0b,
                      cudaStream_t s);
constexpr int TCC_TILE_M = 128, TCC_TILE_N = 256;
constexpr int CP_FLAGS_PER_FRONT = 80;   // D[8] + R[8][8] (+ 8 spare) of one front in one panel launch
constexpr int CD_PANEL = 256;            // panel width of the TRSM-on-tensor-cores path
constexpr int CD_LINV_ROWS = 2 * 4 * 256;   // B-operand rows of one front's Linv parts
constexpr int64_t CD_HAND_WORDS = 10 * 64 * 64;   // hand-off words of one front in one diagonal launch
constexpr int64_t CD_HAND_HEAD = 16;      // words before the first slot (the factorisation count)
constexpr int CD_MAX_SEQ = 1024;           // diagonal launches one factor program may hold

}  // namespace uhm_gpu
