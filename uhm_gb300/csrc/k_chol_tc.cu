// Cholesky fronts factored with BF16-split tensor-core updates.
//
// Restates, for one front, the reference's partial factorisation
// chol(ATL); ABL <- ABL L^{-T}; ABR <- ABR - ABL ABL^T
// (UHM/src/matrix/uhm/fla/chol/decompose.cxx:50-98, with the blocked
// right-looking Cholesky of LINAL/src/dense/chol.cxx:46-92 inside ATL) in
// three kinds of launch per level of the tree:
//
//  1. k_chol_panel, once per outer panel of W1 columns [K0, K0 + W1) of the
//     factor block: the whole panel, all rows K0..n-1 of every front of the
//     level, is factored in one launch.  One CTA per 64-row block holds its
//     rows of the panel in shared memory.  The CTAs of the panel's first
//     rows own its 64 x 64 diagonal blocks; the owner of block j factors it
//     (and forms its inverse) once the updates of the steps before have
//     reached it, publishes the inverse and raises a flag; every CTA below
//     multiplies its block column j by the inverse (TRSM), the owners of
//     later diagonal blocks publish that product, and every CTA applies the
//     rank-64 updates of step j to its rows of the panel's later columns.
//     CTAs wait only on CTAs with smaller tickets (tickets are handed out in
//     order of the diagonal distance, then front), so the launch needs no
//     co-residency.  The CTAs below the panel then write their rows back and
//     split them into BF16 parts (hi + lo) for the tensor cores.
//  2. k_tc_chol over the trailing columns of the factor block, after every
//     panel: C[rows >= K0+W, K0+W <= cols < fs] -= P P^T (lower part), with
//     P the panel's rows below it and K = W.
//  3. k_tc_chol over ABR once per level, after the last panel:
//     ABR -= ABL ABL^T with K = fs in one pass, so every 128 x 256 tile of
//     the Schur complement accumulates the whole contraction in tensor
//     memory and is read and written once.
//
// BF16-split products (the "bf16x3" of k_tc_gemm.cu): a = hi + lo with hi,
// lo BF16 (round to nearest), a b ~ hi_a hi_b + hi_a lo_b + lo_a hi_b,
// accumulated in FP32 in tensor memory.
//
// Operand workspace, chunk-major: per front and part p, per 64-column chunk
// kc of the factor block, the n rows of that chunk as rows of 64 BF16
// (128 bytes): row index row0[front] + (p * nch + kc) * n + r.  One 2D
// tensor map of 128-byte rows covers all of it.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <stdexcept>
#include <string>

#include "k_common.cuh"
#include "k_potrf.cuh"
#include "k_tc_ptx.cuh"
#include "k_chol_tc.cuh"

namespace uhm_gpu {

UHM_DEFINE_WAIT_LIMIT(set_wait_limit_chol_tc, 1u << 22)

// ---------------------------------------------------------------------------
// 1. the cooperative panel kernel
// ---------------------------------------------------------------------------
constexpr int CP_THREADS = 256;
constexpr int CP_LT = 68;          // row of a transposed 64 x 64 operand in shared memory (16-byte rows)
constexpr int CP_ERR = 5;          // error word value of a panel wait that gave up

template <int W1>
struct CpSmem {
  float P[64 * W1];                // the CTA's 64 rows of the panel, column-major (leading dimension 64)
  union {
    PotrfShared<float> sh;         // diagonal owner: the block's factorisation
    struct {
      float Lt[64 * CP_LT];        // inverse of the step's diagonal block, transposed
      float Bt[64 * CP_LT];        // the update operand L[block jp, block j], transposed
    } t;
  } u;
  int s_t, s_ok;
};

__device__ __forceinline__ int cp_ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void cp_st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// thread 0 waits (bounded) for *flag; every thread learns whether it came.
// The leading barrier keeps thread 0 from overwriting *s_ok before a slower
// warp has read the previous answer.  A wait gives up at once when another
// CTA has already given up (the error word is set).
__device__ bool cp_wait(const int* flag, int* err, int* s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    bool ok = cp_ld_acquire(err) == 0;
    if (ok) {
      ok = false;
      const uint32_t lim = g_wait_limit;
      for (uint32_t i = 0; i < lim; ++i) {
        if (cp_ld_acquire(flag) != 0) {
          ok = true;
          break;
        }
        if ((i & 255) == 255 && cp_ld_acquire(err) != 0) break;
        __nanosleep(32);
      }
      if (!ok) atomicExch(err, CP_ERR);
    }
    __threadfence();
    *s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  return *s_ok != 0;
}

// every thread's stores to global memory are visible before thread 0 raises *flag
__device__ __forceinline__ void cp_publish(int* flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) cp_st_release(flag, 1);
}

// acc (this thread's 4 x 4 tile: rows 4 ti .., columns 4 tj .., ti = tid % 16,
// tj = tid / 16) += X * B, X = 64 x kb column-major (leading dimension 64),
// B = kb x 64 row-major with rows of CP_LT (zero where unused): two 128-bit
// shared loads per 16 FMAs.
__device__ __forceinline__ void cp_mma_tile(const float* __restrict__ X, const float* __restrict__ B, int kb,
                                            float (&acc)[4][4]) {
  const int ti = threadIdx.x & 15, tj = threadIdx.x >> 4;
#pragma unroll 4
  for (int t = 0; t < kb; ++t) {
    const float4 x4 = *reinterpret_cast<const float4*>(&X[4 * ti + t * 64]);
    const float4 b4 = *reinterpret_cast<const float4*>(&B[t * CP_LT + 4 * tj]);
    const float xv[4] = {x4.x, x4.y, x4.z, x4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] += xv[u] * bv[v];
  }
}

// P[:, dst .. dst+63] (the CTA's 64 rows) = or -= P[:, src .. src+kb-1] * T^T,
// T given transposed in Tt (Tt[t * CP_LT + jj] = T[jj][t], zero where unused).
// The destination is written only after every thread has read its source
// (src may equal dst).
__device__ __forceinline__ void cp_gemm64(float* __restrict__ P, int src, int dst, const float* __restrict__ Tt,
                                          int kb, bool sub) {
  const int ti = threadIdx.x & 15, tj = threadIdx.x >> 4;
  float acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
  cp_mma_tile(P + src * 64, Tt, kb, acc);
  __syncthreads();
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    float4* d = reinterpret_cast<float4*>(&P[4 * ti + (dst + 4 * tj + v) * 64]);
    float4 o = *d;
    if (sub) {
      o.x -= acc[0][v]; o.y -= acc[1][v]; o.z -= acc[2][v]; o.w -= acc[3][v];
    } else {
      o = make_float4(acc[0][v], acc[1][v], acc[2][v], acc[3][v]);
    }
    *d = o;
  }
  __syncthreads();
}

// item: front, a = K0 (first column of the panel), b = rel, the CTA's
// block of rows: rel < nd is the panel's diagonal block rel (rows
// K0 + 64 rel .., as many as the block has columns), rel >= nd the 64 rows
// from K0 + W + 64 (rel - nd) (W = the panel's width, nd = its diagonal
// blocks); c = offset of the front's flags in this launch (D[j] at c + j,
// R[jp][j] at c + 8 + 8 jp + j).  Tickets are taken in item order.
template <int W1>
__global__ void __launch_bounds__(CP_THREADS, W1 <= 256 ? 2 : 1)
k_chol_panel(DevCtx c, const Item* __restrict__ items, int* ticket, int* flags, int* err,
             __nv_bfloat16* __restrict__ ws, const int64_t* __restrict__ ws_row0) {
  extern __shared__ __align__(16) unsigned char cp_raw[];
  CpSmem<W1>& S = *reinterpret_cast<CpSmem<W1>*>(cp_raw);
  const int tid = threadIdx.x;
  if (tid == 0) S.s_t = atomicAdd(ticket, 1);
  __syncthreads();
  const Item it = items[S.s_t];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, K0 = it.a, rel = it.b;
  const int W = min(W1, fs - K0), nd = (W + 63) / 64;
  const int r0 = rel < nd ? K0 + 64 * rel : K0 + W + 64 * (rel - nd);
  const int rows = rel < nd ? min(64, W - 64 * rel) : min(64, n - r0);
  int* D = flags + it.c;
  int* R = D + 8;
  float* __restrict__ G = c.a32 + f.off;
  // the CTA's rows of the panel (a diagonal owner needs only its columns up to
  // and including its diagonal block)
  const int ncol = rel < nd ? min(W, 64 * (rel + 1)) : W;
  for (int idx = tid; idx < 64 * ncol; idx += CP_THREADS) {
    const int i = idx & 63, col = idx >> 6;
    S.P[idx] = i < rows ? G[(r0 + i) + (int64_t)(K0 + col) * n] : 0.f;
  }
  __syncthreads();
  auto write_back = [&](int ncols) {
    for (int idx = tid; idx < 64 * ncols; idx += CP_THREADS) {
      const int i = idx & 63, col = idx >> 6;
      if (i < rows) G[(r0 + i) + (int64_t)(K0 + col) * n] = S.P[idx];
    }
  };
  for (int j = 0; j < nd; ++j) {
    const int cj = 64 * j, kbj = min(64, W - cj);
    if (rel == j) {
      // diagonal owner: every update of steps < j has been applied to this
      // block; factor it in place and publish its inverse
      float x[4][4];
      bool bad;
      potrf_block<float>(S.P + cj * 64, 64, kbj, S.u.sh, x, bad, S.P + cj * 64);
      if (bad && tid == 0) set_status(c, it.front, ST_NOT_SPD);
      potrf_store_inverse<float>(kbj, x, c.dinv32 + f.dinv_off + (int64_t)(K0 / 64 + j) * 4096);
      // the CTAs below need only the inverse: raise the flag before the
      // write-back of this CTA's rows, which nothing in this launch reads
      cp_publish(D + j);
      write_back(cj + kbj);
      return;
    }
    // rel > j: X_j = A[rows, block j] L_jj^{-T}
    cp_wait(D + j, err, &S.s_ok);
    {
      const float* Di = c.dinv32 + f.dinv_off + (int64_t)(K0 / 64 + j) * 4096;
      for (int idx = tid; idx < 4096; idx += CP_THREADS) {
        const int t = idx >> 6, jj = idx & 63;   // Di[t * 64 + jj] = Linv[jj][t]
        S.u.t.Lt[t * CP_LT + jj] = (t < kbj && jj < kbj) ? __ldcg(Di + idx) : 0.f;
      }
    }
    __syncthreads();
    cp_gemm64(S.P, cj, cj, S.u.t.Lt, kbj, false);
    if (rel < nd) {
      // a later diagonal owner: its block of L in column block j is an
      // operand of every CTA below it
      for (int idx = tid; idx < 64 * kbj; idx += CP_THREADS) {
        const int i = idx & 63, col = idx >> 6;
        if (i < rows) G[(r0 + i) + (int64_t)(K0 + cj + col) * n] = S.P[i + (cj + col) * 64];
      }
      cp_publish(R + rel * 8 + j);
    }
    // rank-kbj updates of this CTA's later column blocks (a diagonal owner
    // stops at its own block: columns right of it are above the diagonal)
    const int jlast = rel < nd ? rel : nd - 1;
    for (int jp = j + 1; jp <= jlast; ++jp) {
      const int cjp = 64 * jp, kbp = min(64, W - cjp);
      if (jp == rel) {
        for (int idx = tid; idx < 4096; idx += CP_THREADS) {
          const int t = idx >> 6, jj = idx & 63;
          S.u.t.Bt[t * CP_LT + jj] = (t < kbj && jj < kbp) ? S.P[jj + (cj + t) * 64] : 0.f;
        }
      } else {
        cp_wait(R + jp * 8 + j, err, &S.s_ok);
        const int rjp = K0 + cjp;
        for (int idx = tid; idx < 4096; idx += CP_THREADS) {
          const int t = idx >> 6, jj = idx & 63;
          S.u.t.Bt[t * CP_LT + jj] =
              (t < kbj && jj < kbp) ? __ldcg(G + (rjp + jj) + (int64_t)(K0 + cj + t) * n) : 0.f;
        }
      }
      __syncthreads();
      cp_gemm64(S.P, cj, cjp, S.u.t.Bt, kbj, true);
    }
  }
  // below the panel's diagonal blocks: the finished rows back to the front,
  // and their BF16 parts into the operand workspace (chunks K0/64 ..)
  write_back(W);
  const int nch = (fs + 63) / 64;
  const int64_t row0 = ws_row0[it.front];
  for (int cc = 0; cc < nd; ++cc) {
    const int kc = K0 / 64 + cc;
    __nv_bfloat16* w0 = ws + (row0 + (int64_t)kc * n + r0) * 64;
    __nv_bfloat16* w1 = ws + (row0 + (int64_t)(nch + kc) * n + r0) * 64;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int idx = tid + CP_THREADS * h, i = idx & 63, g8 = idx >> 6;
      if (i >= rows) continue;
      __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int col = 64 * cc + 8 * g8 + q;
        const float xv = col < W ? S.P[i + col * 64] : 0.f;
        hi[q] = __float2bfloat16_rn(xv);
        lo[q] = __float2bfloat16_rn(xv - __bfloat162float(hi[q]));
      }
      *reinterpret_cast<uint4*>(w0 + (int64_t)i * 64 + 8 * g8) = *reinterpret_cast<const uint4*>(hi);
      *reinterpret_cast<uint4*>(w1 + (int64_t)i * 64 + 8 * g8) = *reinterpret_cast<const uint4*>(lo);
    }
  }
}

// ---------------------------------------------------------------------------
// 1b. the panel's diagonal block and its inverse (panels of 256 columns whose
//     rows below are solved on the tensor cores)
// ---------------------------------------------------------------------------
// The panel's W x W diagonal block (W <= 256, nd <= 4 blocks of 64) is
// factored by nd CTAs exactly as in k_chol_panel (CTA j owns block row j).
// Each then forms block COLUMN j of the inverse Linv of the factored block:
//   Linv[j][j] = L_jj^{-1},
//   Linv[r][j] = -L_rr^{-1} sum_{k=j}^{r-1} L[r][k] Linv[k][j]      (r > j),
// keeping its column in shared memory.  The sum for row r needs only the
// rows of L that CTA r has solved, so it is formed while CTA r still
// factors; only the product with L_rr^{-1} waits for CTA r's diagonal block.
// (By rows instead, row r needed every earlier row of Linv in turn and the
// last row finished 40 us after the last diagonal block.)  The blocks are
// written, split into BF16 hi / lo, as the B operand of the TRSM on the
// tensor cores (X = A Linv^T for the rows below the block): row c of Linv =
// row c of B, chunk i = columns 64 i .. 64 i + 63.
//
// Hand-offs between the CTAs of a front are self-validating words: each
// 64 x 64 block a CTA passes on (the inverse L_jj^{-1} of its diagonal
// block, D_j, and each solved block L[r][k], R_rk) is written as 4096 8-byte
// words (tag << 32 | the FP32 bits), one relaxed store per word, single-copy
// atomic.  The tag is unique to the launch (the engine's factorisation count
// and the launch's sequence number in its program), so a reader polls the
// words themselves until every one carries it: no flag, no fence on the
// writer's side and no second round trip for the data on the reader's.
// Word e = 64 t + i holds entry (i, t) of the block (column-major).
constexpr int CD_W = 256;
constexpr int CD_BLOCK_WORDS = 64 * 64;

struct CdSmem {
  float P[64 * CD_W];              // the CTA's rows of the diagonal block (columns 0 .. 64 j + 63 used)
  union {
    PotrfLaShared<float> sh;
    struct {
      float Lt[64 * CP_LT];
      float Bt[64 * CP_LT];
    } t;
  } u;
  float Dm[64 * 64];               // a 64 x 64 left operand, column-major (L_rk, then Dinv_r)
  float Lc[4][64 * CP_LT];         // this CTA's column block of Linv, one 64 x 64 block per row block
  int s_t;
  uint32_t s_tag;
};

__device__ __forceinline__ uint32_t cd_tag(const unsigned* epoch, int seq) {
  const uint32_t e = *reinterpret_cast<const volatile unsigned*>(epoch);
  return 0x80000000u | ((e & 0x1FFFFFu) << 10) | ((uint32_t)seq & 0x3FFu);
}

__device__ __forceinline__ void cd_put2(uint64_t* p, uint32_t tag, float a, float b) {
  const uint64_t w0 = ((uint64_t)tag << 32) | __float_as_uint(a);
  const uint64_t w1 = ((uint64_t)tag << 32) | __float_as_uint(b);
  asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(p), "l"(w0), "l"(w1) : "memory");
}

__device__ __forceinline__ void cd_get2(const uint64_t* p, uint64_t& w0, uint64_t& w1) {
  asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(w0), "=l"(w1) : "l"(p) : "memory");
}

// publish a 64 x 64 block held column-major in shared memory (leading
// dimension 64): this thread's words e = 512 m + 2 tid, + 1
__device__ __forceinline__ void cd_publish_smem(uint64_t* H, uint32_t tag, const float* __restrict__ B) {
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const int e = 512 * m + 2 * threadIdx.x;
    const float2 v = *reinterpret_cast<const float2*>(&B[e]);
    cd_put2(H + e, tag, v.x, v.y);
  }
}

// this thread's words e = 512 m + 2 tid, + 1 (m = 0 .. 7) of the block at H,
// all eight pairs polled together until each carries tag (one round trip
// once they are written).  False (and the error word set) when the wait
// gives up; a wait gives up within 256 polls when another CTA has already
// given up.
__device__ bool cd_fetch(const uint64_t* H, uint32_t tag, float2 (&v)[8], int* err) {
  const uint32_t lim = g_wait_limit;
  const uint64_t* p = H + 2 * threadIdx.x;
  for (uint32_t i = 0;; ++i) {
    uint64_t w[8][2];
#pragma unroll
    for (int m = 0; m < 8; ++m) cd_get2(p + 512 * m, w[m][0], w[m][1]);
    bool all = true;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      all = all && (uint32_t)(w[m][0] >> 32) == tag && (uint32_t)(w[m][1] >> 32) == tag;
      v[m] = make_float2(__uint_as_float((uint32_t)w[m][0]), __uint_as_float((uint32_t)w[m][1]));
    }
    if (all) return true;
    if (i >= lim || ((i & 255) == 0 && cp_ld_acquire(err) != 0)) {
      atomicExch(err, CP_ERR);
      return false;
    }
    __nanosleep(32);
  }
}

// the fetched words into a row-major operand with rows of CP_LT: entry
// (i, t) of the block to row t, column i (the transpose of the block)
__device__ __forceinline__ void cd_to_rows(const float2 (&v)[8], float* __restrict__ B) {
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const int e = 512 * m + 2 * threadIdx.x, t = e >> 6, i = e & 63;
    *reinterpret_cast<float2*>(&B[t * CP_LT + i]) = v[m];
  }
}

// ... into a column-major operand (leading dimension 64)
__device__ __forceinline__ void cd_to_cols(const float2 (&v)[8], float* __restrict__ B) {
#pragma unroll
  for (int m = 0; m < 8; ++m) *reinterpret_cast<float2*>(&B[512 * m + 2 * threadIdx.x]) = v[m];
}

// P[:, c .. c+63] = P[:, c .. c+63] T^T for the lower-triangular T given
// transposed in Tt (Tt[t * CP_LT + jj] = T[jj][t], zero for t > jj): column
// jj needs only t <= jj.  Warp w takes column group g = w (w < 4) or 11 - w,
// 8 g .. 8 g + 7, and stops at t = 8 g + 8, so the two warps of each
// scheduler (w, w + 4) run 72 steps together instead of 128.
__device__ __forceinline__ void cd_trsm64(float* __restrict__ P, int c, const float* __restrict__ Tt) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = w < 4 ? w : 11 - w;
  const int ti = lane & 15, tj = 2 * g + (lane >> 4);
  float acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
  const float* X = P + c * 64;
  const int kt = 8 * g + 8;
#pragma unroll 4
  for (int t = 0; t < kt; ++t) {
    const float4 x4 = *reinterpret_cast<const float4*>(&X[4 * ti + t * 64]);
    const float4 b4 = *reinterpret_cast<const float4*>(&Tt[t * CP_LT + 4 * tj]);
    const float xv[4] = {x4.x, x4.y, x4.z, x4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] += xv[u] * bv[v];
  }
  __syncthreads();
#pragma unroll
  for (int v = 0; v < 4; ++v)
    *reinterpret_cast<float4*>(&P[4 * ti + (c + 4 * tj + v) * 64]) =
        make_float4(acc[0][v], acc[1][v], acc[2][v], acc[3][v]);
  __syncthreads();
}

// item: front, a = K0, b = j (diagonal block), c = the front's slot in this
// launch (its hand-off words at hand + c * CD_HAND_WORDS: D_k at block k,
// R_rk at block 4 + r (r - 1) / 2 + k); seq: the launch's number in its
// program; epoch: the engine's factorisation count; linv_row0: first
// B-operand row of the front's Linv parts.  Items come front by front, and a
// CTA waits only on CTAs of its own front (the factorisation on smaller
// block rows, the inverse's column on larger ones): the lowest unfinished
// front's CTAs have all started, so every wait ends once a front's CTAs fit
// on the GPU together.
__global__ void __launch_bounds__(CP_THREADS, 1)
k_chol_diag(DevCtx c, const Item* __restrict__ items, int* ticket, uint64_t* __restrict__ hand,
            const unsigned* __restrict__ epoch, int seq, int* err, __nv_bfloat16* __restrict__ ws,
            const int64_t* __restrict__ linv_row0) {
  extern __shared__ __align__(16) unsigned char cd_raw[];
  CdSmem& S = *reinterpret_cast<CdSmem*>(cd_raw);
  const int tid = threadIdx.x;
  const int ti = tid & 15, tj = tid >> 4;
  if (tid == 0) {
    S.s_t = atomicAdd(ticket, 1);
    S.s_tag = cd_tag(epoch, seq);
  }
  __syncthreads();
  const Item it = items[S.s_t];
  const uint32_t tag = S.s_tag;
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, fs = f.fs, K0 = it.a, rel = it.b;
  const int W = min(CD_W, fs - K0);
  const int r0 = K0 + 64 * rel, rows = min(64, W - 64 * rel);
  uint64_t* __restrict__ H = hand + (int64_t)it.c * CD_HAND_WORDS;
  auto Dh = [&](int k) { return H + (int64_t)k * CD_BLOCK_WORDS; };
  auto Rh = [&](int r, int k) { return H + (int64_t)(4 + r * (r - 1) / 2 + k) * CD_BLOCK_WORDS; };
  float* __restrict__ G = c.a32 + f.off;
  const int ncol = min(W, 64 * (rel + 1));
  for (int idx = tid; idx < 64 * ncol; idx += CP_THREADS) {
    const int i = idx & 63, col = idx >> 6;
    S.P[idx] = i < rows ? G[(r0 + i) + (int64_t)(K0 + col) * n] : 0.f;
  }
  __syncthreads();
  // steps j < rel: as the diagonal owners of k_chol_panel (every block j < rel
  // is a full 64 x 64 block; rows of a ragged last block are zero)
  for (int j = 0; j < rel; ++j) {
    const int cj = 64 * j;
    {
      float2 v[8];
      const bool ok = cd_fetch(Dh(j), tag, v, err);
      if (__syncthreads_or(!ok)) return;
      cd_to_rows(v, S.u.t.Lt);
    }
    __syncthreads();
    cd_trsm64(S.P, cj, S.u.t.Lt);
    // block j of this row block, solved: for the CTAs below and the
    // inverse's columns
    cd_publish_smem(Rh(rel, j), tag, S.P + cj * 64);
    for (int jp = j + 1; jp <= rel; ++jp) {
      const int cjp = 64 * jp, kbp = min(64, W - cjp);
      if (jp == rel) {
        for (int idx = tid; idx < 4096; idx += CP_THREADS) {
          const int t = idx >> 6, jj = idx & 63;
          S.u.t.Bt[t * CP_LT + jj] = jj < kbp ? S.P[jj + (cj + t) * 64] : 0.f;
        }
      } else {
        float2 v[8];
        const bool ok = cd_fetch(Rh(jp, j), tag, v, err);
        if (__syncthreads_or(!ok)) return;
        cd_to_rows(v, S.u.t.Bt);
      }
      __syncthreads();
      cp_gemm64(S.P, cj, cjp, S.u.t.Bt, 64, true);
    }
  }
  // the diagonal block itself
  const int cr = 64 * rel, kbr = rows;
  float x[4][4];
  {
    bool bad;
    potrf_block_la<float>(S.P + cr * 64, 64, kbr, S.u.sh, x, bad, S.P + cr * 64);
    if (bad && tid == 0) set_status(c, it.front, ST_NOT_SPD);
  }
  // its inverse (zero outside the block's kbr rows and columns): to the CTAs
  // of this front first, then for the solves and into this CTA's column
  // block of Linv, row-major with rows of CP_LT
  float out[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int r = 4 * ti + u, cc = 4 * tj + v;
      out[u][v] = (r < kbr && cc < kbr) ? x[u][v] : 0.f;
    }
  {
    uint64_t* Dr = Dh(rel);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int e = (4 * tj + v) * 64 + 4 * ti;
      cd_put2(Dr + e, tag, out[0][v], out[1][v]);
      cd_put2(Dr + e + 2, tag, out[2][v], out[3][v]);
    }
  }
  potrf_store_inverse<float>(kbr, x, c.dinv32 + f.dinv_off + (int64_t)(K0 / 64 + rel) * 4096);
  for (int idx = tid; idx < 64 * (cr + kbr); idx += CP_THREADS) {
    const int i = idx & 63, col = idx >> 6;
    if (i < rows) G[(r0 + i) + (int64_t)(K0 + col) * n] = S.P[idx];
  }
  const int64_t lrow0 = linv_row0[it.front];
  const int nd = (W + 63) / 64;
  auto store_b = [&](int r, const float (&o)[4][4]) {
    // rows 64 r + 4 ti .. of Linv, chunk rel: BF16 parts as the B operand
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int rr = 4 * ti + u;
      __align__(8) __nv_bfloat16 hi[4], lo[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        hi[v] = __float2bfloat16_rn(o[u][v]);
        lo[v] = __float2bfloat16_rn(o[u][v] - __bfloat162float(hi[v]));
      }
      const int64_t rh = lrow0 + (int64_t)(0 * 4 + rel) * CD_W + 64 * r + rr;
      const int64_t rl = lrow0 + (int64_t)(1 * 4 + rel) * CD_W + 64 * r + rr;
      *reinterpret_cast<uint2*>(ws + rh * 64 + 4 * tj) = *reinterpret_cast<const uint2*>(hi);
      *reinterpret_cast<uint2*>(ws + rl * 64 + 4 * tj) = *reinterpret_cast<const uint2*>(lo);
    }
  };
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) S.Lc[rel][(4 * ti + u) * CP_LT + 4 * tj + v] = out[u][v];
  store_b(rel, out);
  for (int r = rel + 1; r < nd; ++r) {
    // T = sum_{k=rel}^{r-1} L[r][k] Linv[k][rel], each L[r][k] once CTA r has solved it
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
    for (int k = rel; k < r; ++k) {
      float2 v[8];
      const bool ok = cd_fetch(Rh(r, k), tag, v, err);
      if (__syncthreads_or(!ok)) return;   // also: the previous product has read Dm
      cd_to_cols(v, S.Dm);
      __syncthreads();
      cp_mma_tile(S.Dm, S.Lc[k], 64, acc);
    }
    // T as the row-major right operand, then Linv[r][rel] = -Dinv_r T
    {
      float2 v[8];
      const bool ok = cd_fetch(Dh(r), tag, v, err);
      if (__syncthreads_or(!ok)) return;
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int w = 0; w < 4; ++w) S.u.t.Bt[(4 * ti + u) * CP_LT + 4 * tj + w] = acc[u][w];
      cd_to_cols(v, S.Dm);
    }
    __syncthreads();
    float o[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) o[u][v] = 0.f;
    cp_mma_tile(S.Dm, S.u.t.Bt, 64, o);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        o[u][v] = -o[u][v];
        S.Lc[r][(4 * ti + u) * CP_LT + 4 * tj + v] = o[u][v];
      }
    store_b(r, o);
  }
  // chunks right of the diagonal block are zero (Linv is lower triangular)
  for (int i = rel + 1; i < 4; ++i)
    for (int idx = tid; idx < 64 * 8; idx += CP_THREADS) {
      const int r = idx >> 3, q = idx & 7;
      const int64_t rh = lrow0 + (int64_t)(0 * 4 + i) * CD_W + 64 * rel + r;
      const int64_t rl = lrow0 + (int64_t)(1 * 4 + i) * CD_W + 64 * rel + r;
      *reinterpret_cast<uint4*>(ws + rh * 64 + 8 * q) = make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(ws + rl * 64 + 8 * q) = make_uint4(0, 0, 0, 0);
    }
}

// the panel launches' tickets and flags to zero, and the factorisation count
// that tags the diagonal kernels' hand-off words one up (epoch may be null)
__global__ void k_clear_flags(int* __restrict__ flags, int n, unsigned* __restrict__ epoch) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) flags[i] = 0;
  if (epoch && blockIdx.x == 0 && threadIdx.x == 0) *epoch += 1;
}

// BF16 parts (hi, lo) of the panel's rows below its diagonal block, the A
// operand of the TRSM on the tensor cores: item front, a = K0, b = first row
// (64 rows), c = chunk of the panel (0 .. nd-1); written chunk-major at
// row0b[front] + (p * nch + K0 / 64 + c) * n + r.
__global__ void __launch_bounds__(256) k_chol_pack(DevCtx c, const Item* __restrict__ items,
                                                   __nv_bfloat16* __restrict__ ws,
                                                   const int64_t* __restrict__ row0b) {
  __shared__ float tile[64][65];
  const Item it = items[blockIdx.x];
  const FrontDev f = c.fronts[it.front];
  const int n = f.n, K0 = it.a, r0 = it.b, cc = it.c;
  const int W = min(CD_W, f.fs - K0);
  const int col0 = K0 + 64 * cc, kb = min(64, W - 64 * cc);
  const float* __restrict__ G = c.a32 + f.off;
  float v[16];
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    const int idx = threadIdx.x + 256 * u, i = idx & 63, k = idx >> 6;
    v[u] = (r0 + i < n && k < kb) ? G[(r0 + i) + (int64_t)(col0 + k) * n] : 0.f;
  }
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    const int idx = threadIdx.x + 256 * u;
    tile[idx & 63][idx >> 6] = v[u];
  }
  __syncthreads();
  const int nch = (f.fs + 63) / 64, kc = K0 / 64 + cc;
  const int64_t b0 = row0b[it.front];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int idx = threadIdx.x + 256 * h, i = idx >> 3, k8 = (idx & 7) * 8;
    if (r0 + i >= n) continue;
    __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float xv = tile[i][k8 + q];
      hi[q] = __float2bfloat16_rn(xv);
      lo[q] = __float2bfloat16_rn(xv - __bfloat162float(hi[q]));
    }
    *reinterpret_cast<uint4*>(ws + (b0 + (int64_t)kc * n + r0 + i) * 64 + k8) = *reinterpret_cast<const uint4*>(hi);
    *reinterpret_cast<uint4*>(ws + (b0 + (int64_t)(nch + kc) * n + r0 + i) * 64 + k8) =
        *reinterpret_cast<const uint4*>(lo);
  }
}

// ---------------------------------------------------------------------------
// 2./3. tensor-core update over 128 x 256 tiles
// ---------------------------------------------------------------------------
constexpr int TCC_BM = 128, TCC_BN = 256, TCC_STAGES = 4;
constexpr int TCC_KSUB = 2;                  // stages per 64-column chunk: 32 columns (64 bytes) each
constexpr int TCC_THREADS = 320;             // warps 0-7 epilogue, 8 TMA producer, 9 MMA issuer
constexpr int TCC_EPI_THREADS = 256;
constexpr uint32_t TCC_BOX = 128 * 64;       // one TMA box: 128 rows of 32 BF16 = 8 KB
constexpr uint32_t TCC_STAGE = 6 * TCC_BOX;  // A hi, A lo (128 rows), B hi, B lo (256 rows each): 48 KB
constexpr uint32_t TCC_SMEM = 1024 + TCC_STAGES * TCC_STAGE + 256;
constexpr int TCC_ERR = 6;

// mode 0 items may stand for half a tile (bits 30-31 of c: 0 the whole
// 128 x 256 tile, 1 / 2 its first / second 128 columns), so that the last
// round of a launch can be spread over twice as many CTAs
__device__ __forceinline__ int tcc_half(const Item& it) { return (int)(((unsigned)it.c >> 30) & 3u); }
// a filler item of a pair (bit 29): computed with its partner's rows, stored nowhere
__device__ __forceinline__ bool tcc_dummy(const Item& it) { return ((unsigned)it.c >> 29) & 1u; }

// Two modes.
// mode 0 (update): item front, a = first row r0, b = first column c0,
// c = kc0 | kc1 << 16 (chunks [kc0, kc1) of the factor block); C -= A B^T
// with A rows r0.. and B rows c0.. of the packed factor (ws_row0).  Columns
// stop at fs for tiles of the factor block (c0 < fs) and at n for tiles of
// ABR (c0 >= fs); only entries with col <= row are stored (Cholesky keeps
// the lower triangle).
// Paired (pair = 1, mode 0, launched in clusters of 2): items 2p and 2p + 1
// share front, columns and chunks (two row tiles of one column of tiles, or
// a tile and a filler), and CTA rank r of a cluster takes the items with
// index = r mod 2.  Each CTA loads its own A and half of the shared B, sent
// to both CTAs of the cluster (TMA multicast); a stage is reused once both
// CTAs' MMAs have released it (the MMA completion arrives on the empty
// barrier of both).  Operand traffic per tile falls from 1.5 to 1 KB per K.
// mode 1 (TRSM below a panel's diagonal block): item front, a = r0, b = c0
// (column within the panel), c = K0; X = A Linv^T with A the panel's rows
// r0.. packed at row0b and B the packed rows c0.. of Linv (linv_row0), K =
// the panel's width; X is stored over the panel's columns K0 + c0 .. and its
// BF16 parts into the packed factor (ws_row0) for the updates that follow.
__global__ void __launch_bounds__(TCC_THREADS, 1)
k_tc_chol(DevCtx c, const __grid_constant__ CUtensorMap wsmap, const int64_t* __restrict__ ws_row0,
          const Item* __restrict__ items, int n_items, int* err, int mode, const int64_t* __restrict__ row0b,
          const int64_t* __restrict__ linv_row0, __nv_bfloat16* __restrict__ ws, int pair) {
  extern __shared__ __align__(1024) uint8_t tcc_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tcc_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + TCC_STAGES * TCC_STAGE);
  // bars: [0, S) full, [S, 2S) empty, then acc_full[2], acc_empty[2], drain
  uint64_t* acc_full = bars + 2 * TCC_STAGES;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* drain_bar = acc_full + 4;
  volatile int* s_abort = reinterpret_cast<volatile int*>(acc_full + 5);
  uint32_t* s_tmem = reinterpret_cast<uint32_t*>(acc_full + 6);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TCC_STAGES; ++s) {
      mbar_init(smem_u32(&bars[s]), 1);
      mbar_init(smem_u32(&bars[TCC_STAGES + s]), pair ? 2 : 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&acc_full[b]), 1);
      mbar_init(smem_u32(&acc_empty[b]), TCC_EPI_THREADS);
    }
    mbar_init(smem_u32(drain_bar), 1);
    *s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                 "r"(2 * TCC_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // the peer's barriers are initialised before any multicast reaches them
  if (pair) cluster_sync_all();
  const uint32_t tmem = *s_tmem;
  const uint32_t lim = g_wait_limit;
  const uint32_t rank = pair ? cluster_rank() : 0;

  if (warp == 8) {
    if (lane == 0) {
      // TMA producer: per chunk one stage holding both parts of A and of B
      uint32_t g = 0;
      bool live = true;
      for (int t = blockIdx.x; t < n_items && live; t += gridDim.x) {
        const Item it = items[t];
        const FrontDev f = c.fronts[it.front];
        const int n = f.n, nch = (f.fs + 63) / 64;
        int kc0, kc1;
        int64_t ya_h, ya_l, yb_h, yb_l, ya_step, yb_step;   // rows of chunk kc0 and the step per chunk
        const int hsel = mode == 0 ? tcc_half(it) : 0;
        if (mode == 0) {
          kc0 = it.c & 0xFFFF;
          kc1 = (it.c >> 16) & 0x1FFF;
          const int64_t row0 = ws_row0[it.front];
          const int cb = it.b + (hsel == 2 ? 128 : 0);
          ya_h = row0 + (int64_t)kc0 * n + it.a;
          ya_l = row0 + (int64_t)(nch + kc0) * n + it.a;
          yb_h = row0 + (int64_t)kc0 * n + cb;
          yb_l = row0 + (int64_t)(nch + kc0) * n + cb;
          ya_step = yb_step = n;
        } else {
          const int K0 = it.c;
          kc0 = 0;
          kc1 = (min(CD_W, f.fs - K0) + 63) / 64;
          const int64_t rb = row0b[it.front], rl = linv_row0[it.front];
          ya_h = rb + (int64_t)(K0 / 64) * n + it.a;
          ya_l = rb + (int64_t)(nch + K0 / 64) * n + it.a;
          yb_h = rl + it.b;
          yb_l = rl + 4 * CD_W + it.b;
          ya_step = n;
          yb_step = CD_W;
        }
        for (int kq = TCC_KSUB * kc0; kq < TCC_KSUB * kc1; ++kq, ++g) {
          const int kc = kq / TCC_KSUB, xq = 32 * (kq % TCC_KSUB);   // chunk and its first column
          const uint32_t s = g % TCC_STAGES;
          if (g >= TCC_STAGES &&
              !mbar_wait_lim(smem_u32(&bars[TCC_STAGES + s]), ((g / TCC_STAGES) + 1) & 1, s_abort, err, TCC_ERR,
                             lim)) {
            live = false;
            break;
          }
          const uint32_t fb = smem_u32(&bars[s]);
          const uint32_t st = smem_u32(smem + s * TCC_STAGE);
          // a half tile (128 columns) takes one box of each B part
          mbar_expect_tx(fb, hsel ? 4 * TCC_BOX : TCC_STAGE);
          const int64_t da = (int64_t)(kc - kc0) * ya_step, db = (int64_t)(kc - kc0) * yb_step;
          tma_load_2d(st + 0 * TCC_BOX, &wsmap, xq, (int)(ya_h + da), fb);
          tma_load_2d(st + 1 * TCC_BOX, &wsmap, xq, (int)(ya_l + da), fb);
          if (!pair) {
            tma_load_2d(st + 2 * TCC_BOX, &wsmap, xq, (int)(yb_h + db), fb);
            if (!hsel) tma_load_2d(st + 3 * TCC_BOX, &wsmap, xq, (int)(yb_h + db + 128), fb);
            tma_load_2d(st + 4 * TCC_BOX, &wsmap, xq, (int)(yb_l + db), fb);
            if (!hsel) tma_load_2d(st + 5 * TCC_BOX, &wsmap, xq, (int)(yb_l + db + 128), fb);
          } else if (hsel) {
            // half tiles: rank 0 sends the hi box, rank 1 the lo box
            if (rank == 0) tma_load_2d_mc(st + 2 * TCC_BOX, &wsmap, xq, (int)(yb_h + db), fb, 3);
            else tma_load_2d_mc(st + 4 * TCC_BOX, &wsmap, xq, (int)(yb_l + db), fb, 3);
          } else {
            // rank r sends rows 128 r .. 128 r + 127 of both B parts
            const int off = (int)rank * 128;
            tma_load_2d_mc(st + (2 + rank) * TCC_BOX, &wsmap, xq, (int)(yb_h + db + off), fb, 3);
            tma_load_2d_mc(st + (4 + rank) * TCC_BOX, &wsmap, xq, (int)(yb_l + db + off), fb, 3);
          }
        }
      }
      // the last loads issued (one per stage at most) land before the CTA exits
      for (uint32_t g2 = g > TCC_STAGES ? g - TCC_STAGES : 0; g2 < g; ++g2)
        mbar_drain(smem_u32(&bars[g2 % TCC_STAGES]), (g2 / TCC_STAGES) & 1);
    }
  } else if (warp == 9) {
    if (lane == 0) {
      // MMA issuer: per chunk hi*hi, hi*lo, lo*hi, 4 K=16 steps each
      const uint32_t idesc_full = idesc_bf16_f32(TCC_BM, TCC_BN), idesc_half = idesc_bf16_f32(TCC_BM, 128);
      uint32_t g = 0;
      int i = 0;
      bool live = true;
      for (int t = blockIdx.x; t < n_items && live; t += gridDim.x, ++i) {
        const Item it = items[t];
        int kc0, kc1;
        const uint32_t idesc = (mode == 0 && tcc_half(it)) ? idesc_half : idesc_full;
        if (mode == 0) {
          kc0 = it.c & 0xFFFF;
          kc1 = (it.c >> 16) & 0x1FFF;
        } else {
          kc0 = 0;
          kc1 = (min(CD_W, c.fronts[it.front].fs - it.c) + 63) / 64;
        }
        const int b = i & 1, u = i >> 1;
        if (u >= 1 && !mbar_wait_lim(smem_u32(&acc_empty[b]), (u - 1) & 1, s_abort, err, TCC_ERR, lim)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t acc = tmem + b * TCC_BN;
        for (int kq = TCC_KSUB * kc0; kq < TCC_KSUB * kc1; ++kq, ++g) {
          const uint32_t s = g % TCC_STAGES;
          if (!mbar_wait_lim(smem_u32(&bars[s]), (g / TCC_STAGES) & 1, s_abort, err, TCC_ERR, lim)) {
            live = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = smem_u32(smem + s * TCC_STAGE);
          const uint32_t ah = st, al = st + TCC_BOX, bh = st + 2 * TCC_BOX, bl = st + 4 * TCC_BOX;
#pragma unroll
          for (int k = 0; k < 2; ++k)
            umma_bf16(acc, sdesc_sw64(ah + k * 32), sdesc_sw64(bh + k * 32), idesc,
                      (kq > TCC_KSUB * kc0 || k > 0) ? 1u : 0u);
#pragma unroll
          for (int k = 0; k < 2; ++k) umma_bf16(acc, sdesc_sw64(ah + k * 32), sdesc_sw64(bl + k * 32), idesc, 1u);
#pragma unroll
          for (int k = 0; k < 2; ++k) umma_bf16(acc, sdesc_sw64(al + k * 32), sdesc_sw64(bh + k * 32), idesc, 1u);
          if (pair) umma_commit_mc(smem_u32(&bars[TCC_STAGES + s]), 3);
          else umma_commit(smem_u32(&bars[TCC_STAGES + s]));
        }
        if (live) umma_commit(smem_u32(&acc_full[b]));
      }
      // every MMA issued has completed before tensor memory is freed
      umma_commit(smem_u32(drain_bar));
      mbar_drain(smem_u32(drain_bar), 0);
    }
  } else {
    // epilogue warps 0-7: warp w reads tensor-memory lanes 32 (w % 4) .. +31
    // (tile rows) and columns 128 (w / 4) .. +127; C -= acc column by
    // column, 32 columns at a time (a warp's loads and stores of one column
    // are 32 consecutive rows: 128 contiguous bytes)
    const int quarter = warp & 3, half = warp >> 2;
    int i = 0;
    for (int t = blockIdx.x; t < n_items; t += gridDim.x, ++i) {
      const Item it = items[t];
      const FrontDev f = c.fronts[it.front];
      float* __restrict__ G = c.a32 + f.off;
      const int n = f.n;
      const int cmax = it.b >= f.fs ? n : f.fs;
      const int row = it.a + quarter * 32 + lane;
      const int b = i & 1, u = i >> 1;
      if (!mbar_wait_lim(smem_u32(&acc_full[b]), u & 1, s_abort, err, TCC_ERR, lim)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (mode == 1) {
        // X = acc over the panel's columns, and its BF16 parts (zero beyond
        // the panel's width W) for the updates that follow
        const int K0 = it.c, W = min(CD_W, f.fs - K0), nch = (f.fs + 63) / 64;
        const int64_t row0 = ws_row0[it.front];
        const bool rok = row < n && !*s_abort;
#pragma unroll 1
        for (int cc = 0; cc < 4; ++cc) {
          uint32_t v[32];
          TC_LD32(tmem + ((uint32_t)(quarter * 32) << 16) + b * TCC_BN + half * 128 + cc * 32, v);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          const int cb = it.b + half * 128 + cc * 32;     // panel column of v[0]
          if (!rok || cb >= 64 * ((W + 63) / 64)) continue;
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (cb + j < W) G[row + (int64_t)(K0 + cb + j) * n] = __uint_as_float(v[j]);
          const int kc = K0 / 64 + cb / 64, e0 = cb & 63;
          __nv_bfloat16* wh = ws + (row0 + (int64_t)kc * n + row) * 64 + e0;
          __nv_bfloat16* wl = ws + (row0 + (int64_t)(nch + kc) * n + row) * 64 + e0;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
              const float xv = cb + 8 * q + e < W ? __uint_as_float(v[8 * q + e]) : 0.f;
              hi[e] = __float2bfloat16_rn(xv);
              lo[e] = __float2bfloat16_rn(xv - __bfloat162float(hi[e]));
            }
            *reinterpret_cast<uint4*>(wh + 8 * q) = *reinterpret_cast<const uint4*>(hi);
            *reinterpret_cast<uint4*>(wl + 8 * q) = *reinterpret_cast<const uint4*>(lo);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        mbar_arrive(smem_u32(&acc_empty[b]));
        continue;
      }
      // a half tile's 128 columns sit in tensor-memory columns 0..127 (warps 0-3)
      const int hsel = tcc_half(it);
      const int cbase = it.b + (hsel == 2 ? 128 : 0);
#pragma unroll 1
      for (int cc = 0; cc < 4 && !(hsel && half); ++cc) {
        uint32_t v[32];
        TC_LD32(tmem + ((uint32_t)(quarter * 32) << 16) + b * TCC_BN + half * 128 + cc * 32, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        const int cb = cbase + half * 128 + cc * 32;
        const bool rok = row < n && !*s_abort && !tcc_dummy(it);
        float cv[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = cb + j;
          cv[j] = (rok && col < cmax && col <= row) ? __ldcg(G + row + (int64_t)col * n) : 0.f;
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = cb + j;
          if (rok && col < cmax && col <= row) G[row + (int64_t)col * n] = cv[j] - __uint_as_float(v[j]);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(smem_u32(&acc_empty[b]));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  // neither CTA of a pair leaves while the other may still send it operands
  if (pair) cluster_sync_all();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TCC_BN));
  }
}

// ---- host side ---------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 g_encode_cc = nullptr;

bool tcc_encode(CUtensorMap* map, void* base, int64_t rows) {
  if (!g_encode_cc) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      cudaGetLastError();
      return false;
    }
    g_encode_cc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  cuuint64_t dims[2] = {64, (cuuint64_t)rows};
  cuuint64_t strides[1] = {128};
  cuuint32_t box[2] = {32, 128};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode_cc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <int W1>
static void launch_panel_w(const DevCtx& c, const Item* items, int n_items, int* ticket, int* flags, int* err,
                           void* ws, const int64_t* ws_row0, cudaStream_t s) {
  const int sm = (int)sizeof(CpSmem<W1>);
  cudaFuncSetAttribute(k_chol_panel<W1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  k_chol_panel<W1><<<n_items, CP_THREADS, sm, s>>>(c, items, ticket, flags, err, (__nv_bfloat16*)ws, ws_row0);
}

void launch_chol_panel(const DevCtx& c, const Item* items, int n_items, int w1, int* ticket, int* flags, int* err,
                       void* ws, const int64_t* ws_row0, cudaStream_t s) {
  if (!n_items) return;
  if (w1 == 256) launch_panel_w<256>(c, items, n_items, ticket, flags, err, ws, ws_row0, s);
  else if (w1 == 512) launch_panel_w<512>(c, items, n_items, ticket, flags, err, ws, ws_row0, s);
  else throw std::invalid_argument("chol_panel: panel width must be 256 or 512, got " + std::to_string(w1));
}

void launch_chol_diag(const DevCtx& c, const Item* items, int n_items, int* ticket, uint64_t* hand,
                      const unsigned* epoch, int seq, int* err, void* ws, const int64_t* linv_row0, cudaStream_t s) {
  if (!n_items) return;
  const int sm = (int)sizeof(CdSmem);
  cudaFuncSetAttribute(k_chol_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  k_chol_diag<<<n_items, CP_THREADS, sm, s>>>(c, items, ticket, hand, epoch, seq, err, (__nv_bfloat16*)ws,
                                              linv_row0);
}

void launch_clear_flags(int* flags, int n, unsigned* epoch, cudaStream_t s) {
  const int blocks = n > 0 ? (n + 255) / 256 < 64 ? (n + 255) / 256 : 64 : 1;
  k_clear_flags<<<blocks, 256, 0, s>>>(flags, n, epoch);
}

void launch_chol_pack(const DevCtx& c, const Item* items, int n_items, void* ws, const int64_t* row0b,
                      cudaStream_t s) {
  if (!n_items) return;
  k_chol_pack<<<n_items, 256, 0, s>>>(c, items, (__nv_bfloat16*)ws, row0b);
}

void launch_tc_chol(const DevCtx& c, const CUtensorMap& map, const int64_t* ws_row0, const Item* items, int n_items,
                    int* err, cudaStream_t s, int mode, const int64_t* row0b, const int64_t* linv_row0, void* ws,
                    int reserve, int pair) {
  if (!n_items) return;
  static int n_sm = 0;
  if (!n_sm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (n_sm <= 0) n_sm = 1;
  }
  cudaFuncSetAttribute(k_tc_chol, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TCC_SMEM);
  const int slots = n_sm - reserve > 1 ? n_sm - reserve : 1;
  if (pair) {
    // clusters of two CTAs (items come in pairs, n_items even)
    const int clusters = n_items / 2 < slots / 2 ? n_items / 2 : slots / 2;
    if (clusters < 1) return;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * clusters);
    cfg.blockDim = dim3(TCC_THREADS);
    cfg.dynamicSmemBytes = TCC_SMEM;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_tc_chol, c, map, ws_row0, items, n_items, err, mode, row0b, linv_row0,
                       (__nv_bfloat16*)ws, 1);
    return;
  }
  const int grid = n_items < slots ? n_items : slots;
  k_tc_chol<<<grid, TCC_THREADS, TCC_SMEM, s>>>(c, map, ws_row0, items, n_items, err, mode, row0b, linv_row0,
                                                (__nv_bfloat16*)ws, 0);
}

int chol_panel_max_w1() { return 512; }

}  // namespace uhm_gpu
