// Tensor-core Schur update for FP32 fronts: C -= A21 * A21^T (Cholesky) with
// BF16-split operands on the 5th-generation tensor cores (tcgen05).
//
// The update restates the trailing SYRK of the front's blocked Cholesky
// (LINAL/src/dense/chol.cxx:78-82 and the front-level syrk of
// UHM/src/matrix/uhm/fla/chol/decompose.cxx:94-95).
//
// Split precision: every FP32 entry a = hi + lo + (mid) with hi, lo (, mid)
// BF16 (round to nearest); the product a*b is taken as the sum of BF16
// products hi*hi + hi*lo + lo*hi ("bf16x3", ~2^-17 relative) or, with three
// parts, the six terms of order <= 2^-16 ("bf16x6", FP32-class).  Terms are
// laid end to end along K, so one GEMM with K' = terms * KB accumulates them
// all in FP32 in tensor memory.
//
// Kernel: one persistent CTA per SM walks the 128 x 128 output tiles; warp 8
// issues TMA loads (128-byte swizzle) into a 4-stage shared-memory ring
// guarded by mbarriers, one thread of warp 9 issues tcgen05.mma (M=128,
// N=128, K=16) into one of two 128-column TMEM accumulators, warps 0-7 read
// TMEM back (tcgen05.ld; two warps per 32-lane quarter, one per column half)
// and apply C -= acc to the FP32 panel while the next tile accumulates in
// the other buffer.  Every wait is bounded: a wait that
// gives up records an error flag and the CTA skips its stores.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cstdio>

#include "k_common.cuh"
#include "k_tc.cuh"
#include "k_tc_ptx.cuh"

namespace uhm_gpu {

constexpr int TC_BM = 128, TC_BN = 128, TC_BK = 64, TC_STAGES = 4;
constexpr int TC_THREADS = 320;     // warps 0-7 epilogue, 8 TMA producer, 9 MMA issuer
constexpr int TC_EPI_THREADS = 256;
constexpr uint32_t TC_TILE_BYTES = TC_BM * TC_BK * 2;   // 16 KB (A and B tiles alike)
constexpr uint32_t TC_CPAD = TC_BN + 1;                 // padded row of the staged C tile
constexpr uint32_t TC_CTILE_BYTES = TC_BM * TC_CPAD * 4;
constexpr uint32_t TC_SMEM = 1024 + TC_STAGES * 2 * TC_TILE_BYTES + 256 + TC_CTILE_BYTES;

UHM_DEFINE_WAIT_LIMIT(set_wait_limit_tc, 1u << 24)

// bounded wait: false (and error flag) when the barrier never completes
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                          int* err) {
  return mbar_wait_lim(bar, parity, abort_flag, err, 1, g_wait_limit);
}

// item: front, a = K0 (outer step start), b = tile row, c = tile col
// (tiles counted from the trailing block's first row K0 + KB).
// term_code: 2 bits per part index, 4 bits per term (A part, B part).
//
// Persistent: one CTA per SM walks the tile list with stride gridDim.x.  The
// TMA ring (full / empty barriers) runs continuously across tiles; TMEM holds
// two 128-column accumulators, so the epilogue of tile i (TMEM -> registers
// -> C in global memory) overlaps the mainloop of tile i + 1.  acc_full[b]
// is committed by the MMA thread when accumulator b holds a finished tile;
// acc_empty[b] collects the 256 epilogue threads once they have read it.
__global__ void __launch_bounds__(TC_THREADS, 1)
k_tc_syrk(DevCtx c, const __grid_constant__ CUtensorMap wsmap, const int64_t* __restrict__ ws_off,
          const int64_t* __restrict__ ws_stride, const Item* __restrict__ items, int n_items, int nbo,
          int nterms, uint32_t term_code, int lower_only, int* err) {
  extern __shared__ __align__(1024) uint8_t tc_smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* tilesA = smem;
  uint8_t* tilesB = smem + TC_STAGES * TC_TILE_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + 2 * TC_STAGES * TC_TILE_BYTES);
  // bars[0..S) full, bars[S..2S) empty, bars[2S..2S+2) acc_full, bars[2S+2..2S+4) acc_empty
  uint64_t* acc_full = bars + 2 * TC_STAGES;
  uint64_t* acc_empty = bars + 2 * TC_STAGES + 2;
  volatile int* s_abort = reinterpret_cast<volatile int*>(bars + 2 * TC_STAGES + 4);
  uint32_t* s_tmem = reinterpret_cast<uint32_t*>(bars + 2 * TC_STAGES + 5);
  uint64_t* drain_bar = bars + 2 * TC_STAGES + 6;
  float* s_c = reinterpret_cast<float*>(smem + 2 * TC_STAGES * TC_TILE_BYTES + 256);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(smem_u32(&bars[s]), 1);
      mbar_init(smem_u32(&bars[TC_STAGES + s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&acc_full[b]), 1);
      mbar_init(smem_u32(&acc_empty[b]), TC_EPI_THREADS);
    }
    mbar_init(smem_u32(drain_bar), 1);
    *s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                 "r"(2 * TC_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *s_tmem;

  // per-tile geometry, identical in every role
  struct Tile {
    int front, n, base, R0, C0, row0, prow, kpt, nk, off;
  };
  auto tile_of = [&](int t) {
    const Item it = items[t];
    const FrontDev f = c.fronts[it.front];
    Tile T;
    T.front = it.front;
    T.n = f.n;
    const int KB = min(nbo, f.fs - it.a);
    T.base = it.a + KB;
    T.R0 = T.base + it.b * TC_BM;
    T.C0 = T.base + it.c * TC_BN;
    // the whole BF16 workspace is one 2D tensor of rows of nbo elements;
    // part p of this front starts at row (ws_off + p * ws_stride) / nbo
    T.row0 = (int)(ws_off[it.front] / nbo);
    T.prow = (int)(ws_stride[it.front] / nbo);
    T.kpt = (KB + TC_BK - 1) / TC_BK;
    T.nk = T.kpt * nterms;
    T.off = (int)0;
    (void)f;
    return T;
  };

  if (warp == 8) {
    if (lane == 0) {
      // TMA producer
      uint32_t g = 0;       // chunks issued by this CTA so far
      bool live = true;
      for (int t = blockIdx.x; t < n_items && live; t += gridDim.x) {
        const Tile T = tile_of(t);
        for (int kc = 0; kc < T.nk; ++kc, ++g) {
          const uint32_t s = g % TC_STAGES;
          if (g >= TC_STAGES &&
              !mbar_wait(smem_u32(&bars[TC_STAGES + s]), ((g / TC_STAGES) + 1) & 1, s_abort, err)) {
            live = false;
            break;
          }
          const int term = kc / T.kpt, kk = kc % T.kpt;
          const int pa = (term_code >> (4 * term)) & 3, pb = (term_code >> (4 * term + 2)) & 3;
          const uint32_t fb = smem_u32(&bars[s]);
          mbar_expect_tx(fb, 2 * TC_TILE_BYTES);
          tma_load_2d(smem_u32(tilesA + s * TC_TILE_BYTES), &wsmap, kk * TC_BK,
                      T.row0 + pa * T.prow + (T.R0 - T.base), fb);
          tma_load_2d(smem_u32(tilesB + s * TC_TILE_BYTES), &wsmap, kk * TC_BK,
                      T.row0 + pb * T.prow + (T.C0 - T.base), fb);
        }
      }
      // the last loads issued (one per stage at most) have landed before the
      // CTA exits, whether or not the MMA thread consumed them
      for (uint32_t g2 = g > TC_STAGES ? g - TC_STAGES : 0; g2 < g; ++g2)
        mbar_drain(smem_u32(&bars[g2 % TC_STAGES]), (g2 / TC_STAGES) & 1);
    }
  } else if (warp == 9) {
    if (lane == 0) {
      // MMA issuer
      const uint32_t idesc = idesc_bf16_f32(TC_BM, TC_BN);
      uint32_t g = 0;
      int i = 0;            // tiles processed by this CTA
      bool live = true;
      for (int t = blockIdx.x; t < n_items && live; t += gridDim.x, ++i) {
        const Tile T = tile_of(t);
        const int b = i & 1, u = i >> 1;
        if (u >= 1 && !mbar_wait(smem_u32(&acc_empty[b]), (u - 1) & 1, s_abort, err)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t acc = tmem + b * TC_BN;
        for (int kc = 0; kc < T.nk; ++kc, ++g) {
          const uint32_t s = g % TC_STAGES;
          if (!mbar_wait(smem_u32(&bars[s]), (g / TC_STAGES) & 1, s_abort, err)) {
            live = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t a0 = smem_u32(tilesA + s * TC_TILE_BYTES);
          const uint32_t b0 = smem_u32(tilesB + s * TC_TILE_BYTES);
#pragma unroll
          for (int k = 0; k < TC_BK / 16; ++k)
            umma_bf16(acc, sdesc_sw128(a0 + k * 32), sdesc_sw128(b0 + k * 32), idesc, (kc | k) != 0);
          umma_commit(smem_u32(&bars[TC_STAGES + s]));
        }
        if (live) umma_commit(smem_u32(&acc_full[b]));
      }
      // every MMA this thread issued has completed before TMEM is freed
      umma_commit(smem_u32(drain_bar));
      mbar_drain(smem_u32(drain_bar), 0);
    }
  } else {
    // epilogue warps 0-7: warp w reads TMEM lanes [32 (w % 4), +32) (its
    // lane quarter = tile rows) and handles the columns [64 (w / 4), +64).
    // The thread's half-row of the next C tile is staged in shared memory
    // while the mainloop runs (independent, coalesced loads); each thread
    // reads back only what it staged, so no barrier is needed for s_c.
    const int quarter = warp & 3, half = warp >> 2;
    const int rl = quarter * 32 + lane;
    constexpr int HW = TC_BN / 2;
    float* crow = s_c + rl * TC_CPAD + half * HW;
    int i = 0;
    for (int t = blockIdx.x; t < n_items; t += gridDim.x, ++i) {
      const Tile T = tile_of(t);
      const FrontDev f = c.fronts[T.front];
      float* __restrict__ G = c.a32 + f.off;
      const int n = T.n;
      const int row = T.R0 + rl;
      const int cbase = T.C0 + half * HW;
      const int jmax = lower_only ? min(n, row + 1) : n;     // columns < jmax are stored
#pragma unroll 1
      for (int j0 = 0; j0 < HW; j0 += 16) {
        float v[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int col = cbase + j0 + q;
          v[q] = (row < n && col < jmax) ? __ldcg(G + row + (int64_t)col * n) : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) crow[j0 + q] = v[q];
      }
      const int b = i & 1, u = i >> 1;
      const bool ok = mbar_wait(smem_u32(&acc_full[b]), u & 1, s_abort, err);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      float outv[HW / 32][32];
#pragma unroll
      for (int cc = 0; cc < HW / 32; ++cc) {
        uint32_t v[32];
        TC_LD32(tmem + ((uint32_t)(quarter * 32) << 16) + b * TC_BN + half * HW + cc * 32, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 32; ++j) outv[cc][j] = crow[cc * 32 + j] - __uint_as_float(v[j]);
      }
      // accumulator b may be overwritten from here on
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(smem_u32(&acc_empty[b]));
      if (!*s_abort && row < n) {
#pragma unroll
        for (int cc = 0; cc < HW / 32; ++cc)
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int col = cbase + cc * 32 + j;
            if (col < jmax) G[row + (int64_t)col * n] = outv[cc][j];
          }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_BN));
  }
}

// Split the panel A[K0+KB : n, K0 : K0+KB] (FP32, column-major, ld n) into
// BF16 parts stored row-major with row length nbo (zero beyond KB):
// part p row r = round-to-nearest BF16 of the p-th residual.
// item: front, a = K0, b = row block (64 rows)
// trans = 1 packs U12^T instead: row r is column base + r of the front, rows
// K0..K0+KB (the LU panel's U block right of the outer panel), into parts
// poff.. (the B operand of the LU trailing update).
__global__ void __launch_bounds__(256) k_tc_pack(DevCtx c, const Item* __restrict__ items, int nbo,
                                                 int nparts, __nv_bfloat16* __restrict__ ws,
                                                 const int64_t* __restrict__ ws_off,
                                                 const int64_t* __restrict__ ws_stride, int trans, int poff) {
  __shared__ float tile[64][65];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, K0 = it.a;
  const int KB = min(nbo, f.fs - K0);
  const int base = K0 + KB;
  const int r0 = it.b * 64;
  const float* __restrict__ G = c.a32 + f.off;
  __nv_bfloat16* __restrict__ W = ws + ws_off[it.front];
  const int64_t pstride = ws_stride[it.front];
  for (int k0 = 0; k0 < nbo; k0 += 64) {
    // one batch of 16 independent loads per thread (coalesced along the
    // column), then the shared-memory transpose
    float v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int idx = threadIdx.x + 256 * u;
      const int r = trans ? idx / 64 : idx % 64, k = trans ? idx % 64 : idx / 64;
      const int gr = base + r0 + r, gk = k0 + k;
      v[u] = (gr < n && gk < KB) ? (trans ? G[(K0 + gk) + (int64_t)gr * n] : G[gr + (int64_t)(K0 + gk) * n])
                                 : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int idx = threadIdx.x + 256 * u;
      const int r = trans ? idx / 64 : idx % 64, k = trans ? idx % 64 : idx / 64;
      tile[r][k] = v[u];
    }
    __syncthreads();
    // each thread converts 8 consecutive k of one row and writes every part
    // as one 16-byte store
#pragma unroll
    for (int h2 = 0; h2 < 2; ++h2) {
      const int idx = threadIdx.x + 256 * h2, r = idx / 8, k8 = (idx % 8) * 8;
      if (base + r0 + r >= n) continue;
      float x[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) x[q] = tile[r][k8 + q];
      for (int p = 0; p < nparts; ++p) {
        __align__(16) __nv_bfloat16 hb[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          hb[q] = __float2bfloat16_rn(x[q]);
          x[q] -= __bfloat162float(hb[q]);
        }
        *reinterpret_cast<uint4*>(W + (p + poff) * pstride + (int64_t)(r0 + r) * nbo + k0 + k8) =
            *reinterpret_cast<const uint4*>(hb);
      }
    }
  }
}

// ---- host side ---------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static bool get_encoder() {
  if (g_encode) return true;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
          cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn) {
    cudaGetLastError();
    return false;
  }
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return true;
}

// 2D map over a row-major rows x nbo BF16 matrix, box 64 (K) x 128 (rows)
bool tc_encode_part(CUtensorMap* map, void* base, int64_t rows, int nbo) {
  if (!get_encoder()) return false;
  cuuint64_t dims[2] = {(cuuint64_t)nbo, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)nbo * 2};
  cuuint32_t box[2] = {TC_BK, TC_BM};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

void launch_tc_pack(const DevCtx& c, const Item* items, int n_items, int nbo, int nparts, void* ws,
                    const int64_t* ws_off, const int64_t* ws_stride, int trans, int poff, cudaStream_t s) {
  if (!n_items) return;
  k_tc_pack<<<n_items, 256, 0, s>>>(c, items, nbo, nparts, (__nv_bfloat16*)ws, ws_off, ws_stride, trans, poff);
}

void launch_tc_syrk(const DevCtx& c, const CUtensorMap& wsmap, const int64_t* ws_off,
                    const int64_t* ws_stride, const Item* items, int n_items, int nbo, int nterms,
                    uint32_t term_code, int lower_only, int* err, cudaStream_t s) {
  if (!n_items) return;
  static int n_sm = 0;
  if (!n_sm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (n_sm <= 0) n_sm = 1;
  }
  cudaFuncSetAttribute(k_tc_syrk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
  const int grid = n_items < n_sm ? n_items : n_sm;   // one persistent CTA per SM
  k_tc_syrk<<<grid, TC_THREADS, TC_SMEM, s>>>(c, wsmap, ws_off, ws_stride, items, n_items, nbo, nterms,
                                              term_code, lower_only, err);
}

int tc_tile() { return TC_BM; }

}  // namespace uhm_gpu
