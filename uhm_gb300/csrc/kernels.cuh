// Device data layout shared by the host engine and the CUDA kernels.
//
// One front = one column-major n x n panel (n = fs + ss, ld = n) holding
//   [ ATL ATR ]      ATL fs x fs  (factor block)
//   [ ABL ABR ]      ABR ss x ss  (Schur complement after the partial factor)
// which restates Matrix_FLA_'s four buffers (UHM/include/uhm/matrix/uhm/fla.hxx:59-63)
// as one contiguous panel in HBM.  Fronts live in one arena per storage type
// (FP64 or FP32).  Right-hand sides travel in a global vector in elimination
// order (dofs eliminated at front f are the contiguous range g0..g0+fs), plus
// per-front vector slabs of n x n_rhs for the tree sweeps (z, y, w).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace uhm_gpu {

enum DType : int { F64 = 0, F32 = 1 };
enum Method : int { M_CHOL = 1, M_LU_NOPIV = 2, M_LU_PIV = 3 };

struct FrontDev {
  int64_t off;        // element offset of the panel in its arena
  int64_t voff;       // element offset of the front's three n x n_rhs vector slabs z, y, w (FP64)
  int64_t inv_off;    // offset of this front's inverse maps (nsrc x n int32)
  int64_t colptr_off; // offset of this front's n+1 column-source pointers
  int64_t sgi_off;    // offset of the ss global dof indices of the schur rows
  int64_t piv_off;    // offset of the fs pivot entries (LU)
  int n, fs, ss;
  int dtype;          // storage/compute type of the panel
  int g0;             // first global dof eliminated here
  int src0, nsrc;     // assembly sources [src0, src0 + nsrc)
  int status_slot;
  int flag_off;       // first per-block flag of the flag-driven solves
  int64_t dinv_off;   // inverses of the 64 x 64 diagonal blocks (element offset)
};

// An assembly source: an element matrix (full, FP64) or a child front's ABR.
struct SrcDev {
  int64_t off;        // offset of entry (0,0) of the source block in its arena
  int ld;
  int dtype;          // F64 / F32 (element matrices are F64)
  int is_child;       // 1: child ABR (lower triangle valid when symmetric)
  int slot;           // child front slot (or element index)
  int m;              // rows (= columns) of the source block
  int64_t fwd_off;    // its row map: source row -> parent position (DevCtx::fwd)
};

// Work item for per-front launches: front slot + tile / step data.
struct Item {
  int front;
  int a, b, c;        // kernel-specific (tile row, tile col, step start ...)
};

// Status words written by kernels (breakdown detection): per front.
enum Status : int { ST_OK = 0, ST_NOT_SPD = 1, ST_ZERO_PIVOT = 2, ST_NAN = 3, ST_WAIT = 4 };

struct DevCtx {
  FrontDev* fronts;
  SrcDev* srcs;
  int32_t* inv;       // inverse maps
  int32_t* fwd;       // forward maps (source row -> parent position)
  int64_t* colptr;    // per front: n+1 offsets into colsrc
  int2* colsrc;       // (source local index, source column)
  int32_t* sgi;       // schur-row global dofs
  int32_t* piv;       // pivots (LU), relative to the front's first row
  double* a64;        // FP64 panel arena
  float* a32;         // FP32 panel arena
  double* emat;       // element matrices (FP64, retained for the residual)
  double* vec;        // per-front vector slabs
  int* status;        // per-front status
  double* dinv64;     // inverted diagonal blocks of the factor (FP64 fronts)
  float* dinv32;      // ... (FP32 fronts)
  int* flags;         // per-block completion flags of the flag-driven solves
  int n_rhs;
  int symmetric;      // Cholesky: lower triangles only
};

// ---- kernel launchers (implemented in the .cu files) ----------------------
// extend-add of large fronts: one parent column per CTA, accumulated in
// shared memory (item: front, a = column)
void launch_assemble_scatter(const DevCtx& c, const Item* items, int n_items, int dtype, int lower,
                             int n_max, cudaStream_t s);
void launch_assemble(const DevCtx& c, const Item* items, int n_items, int dtype, int lower,
                     cudaStream_t s);
void launch_small_factor(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                         int max_n, cudaStream_t s);
// diagonal block + panel TRSM of one 64-column step (every CTA factors the
// block; item: front, a = k0, b = first row of the panel block, c = 1 writer)
void launch_potrf_trsm(const DevCtx& c, const Item* items, int n_items, int dtype, cudaStream_t s);
void launch_potrf_diag(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                       cudaStream_t s);
void launch_trsm_panel(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                       cudaStream_t s);
void launch_syrk_update(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                        int nbo, cudaStream_t s);
// LU (partial pivoting restricted to the factor rows, or none)
// LU panel of tall fronts on many CTAs (cooperative launch of n_ctas CTAs;
// item: front, a = k0, b = first CTA, c = CTAs; rmax = rows per CTA, at
// most GC_RMAX_F64 / GC_RMAX_F32), then the panel's row interchanges on the
// other columns (item: front, a = k0, b = first column of 256)
constexpr int GC_RMAX_F64 = 384, GC_RMAX_F32 = 768;
void launch_getrf_coop(const DevCtx& c, const Item* items, int n_items, int n_ctas, int dtype, int nb, int pivot,
                       int rmax, double* xbuf, unsigned int* ctr, int* err, cudaStream_t s);
void launch_laswp(const DevCtx& c, const Item* items, int n_items, int dtype, int nb, cudaStream_t s);
void launch_getrf_panel(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                        int pivot, cudaStream_t s);
void launch_lu_row_update(const DevCtx& c, const Item* items, int n_items, int dtype, int nb,
                          int pivot, cudaStream_t s);
// LU trailing GEMM tiles; nbo / region as for k_tile_update (0 / 0: every entry)
void launch_gemm_update(const DevCtx& c, const Item* items, int n_items, int dtype, int nb, int nbo,
                        int region, cudaStream_t s);

// tree solves over the global vector g (N x n_rhs, column-major, ld N)
void launch_fwd_gather(const DevCtx& c, const Item* items, int n_items, const double* g,
                       int64_t ldg, int method, cudaStream_t s);
void launch_fwd_small(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                      int staged_bytes, cudaStream_t s);
void launch_bwd_small(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                      double* g, int64_t ldg, int staged_bytes, cudaStream_t s);
// flag-driven level solves of large Cholesky fronts (one launch per level and
// group of FLAG_NR right-hand sides, starting at column q0): items ordered so
// that every CTA waits only on CTAs with smaller tickets
constexpr int FLAG_NR = 4;
constexpr int FLAG_NR_BWD_F64 = 2;   // backward FP64 launches take two
void launch_fwd_flags(const DevCtx& c, const Item* items, int n_items, int dtype, int* ticket,
                      int* flag_base, int n_flags, int* err, int q0, cudaStream_t s);
// the same with 256-row CTAs (item a: 256-row block of the factor rows, then
// of ABL), each solving its own four 64-row blocks in turn; the same
// hand-off words in and out
void launch_fwd_flags4(const DevCtx& c, const Item* items, int n_items, int dtype, int* ticket, int* err, int q0,
                       cudaStream_t s);
void launch_bwd_flags(const DevCtx& c, const Item* items, int n_items, int dtype, int* ticket,
                      int* flag_base, int n_flags, int* err, int q0, cudaStream_t s);
// chain solves of large FP32 Cholesky fronts (one launch per level and group
// of FLAG_NR right-hand sides).  Items: front, a = block, b = role: CH_CHAIN
// (one per front, first), CH_HELPER (forward: row blocks b > CH_K in
// ascending b; backward: column blocks b with ABL rows or b + CH_K + 1 < nfb,
// in descending b), CH_ABL (forward only: the ABL row blocks a >= nfb, last)
constexpr int CH_K = 3;
constexpr int CH_CHAIN = 0, CH_HELPER = 1, CH_ABL = 2;
// A chain waits on helpers with larger tickets, so every chain of a launch
// and at least one helper must be resident together (one CTA per SM: the
// chain's shared memory): levels with more large fronts take the
// flag-driven kernels.
constexpr int CH_MAX_CHAINS = 64;
void launch_fwd_chain(const DevCtx& c, const Item* items, int n_items, int* ticket, int* err, int q0,
                      cudaStream_t s);
void launch_bwd_chain(const DevCtx& c, const Item* items, int n_items, int* ticket, int* err, int q0,
                      cudaStream_t s);
// where the first hand-off wait of the solves gave up (0: none; kind * 10^8 +
// awaited block * 10^4 + waiting block), cleared when read
int solve_wait_where();
// blocked solve steps of large fronts (64-column diagonal blocks)
void launch_fwd_step(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                     cudaStream_t s);
void launch_bwd_step(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                     double* scratch, const int64_t* scr_off, int* counters, cudaStream_t s);
void launch_bwd_prepare(const DevCtx& c, const Item* items, int n_items, int dtype, int method,
                        const double* g, int64_t ldg, cudaStream_t s);
void launch_bwd_store(const DevCtx& c, const Item* items, int n_items, double* g, int64_t ldg,
                      cudaStream_t s);

// element-wise residual r = b - sum_e P_e^T A_e P_e x, deterministic gather
// hp-FEM element matrices generated on the device (k_elements.cu); hh = h/2,
// cmass / cconv the mass and convection scale factors as the host computes them
int64_t gen_table_doubles(int p, int dim, int has_react, int has_beta);
void launch_gen_tables(double* tab, const double* ref_p, int p, int dim, double hh, double cmass, double cconv,
                       int has_react, int has_beta, cudaStream_t s);
void launch_gen_lobatto(double* emat, const int64_t* emat_off, int n_el, const int* p_el, const double* kappa,
                        const double* react, const double* beta, const int64_t* sel_ptr, const int32_t* sel,
                        const double* tab, const int64_t* tab_off, int dim, cudaStream_t s);
void launch_elem_gemv(const double* emat, const int64_t* emat_off, const int* elem_m,
                      const int64_t* emap_off, const int32_t* emap, const double* x, int64_t ldx,
                      double* y, const int64_t* y_off, int n_elem, int n_rhs, cudaStream_t s);
void launch_dof_gather(const int64_t* ptr, const int64_t* idx, const double* y, const double* b,
                       int64_t ldb, double* r, int64_t N, int n_rhs, int sub_from_b,
                       cudaStream_t s);
void launch_absmax(const double* v, int64_t n, double* out, cudaStream_t s);
// per-tree max |v| (forest of independent meshes); out: n_trees bit patterns
void launch_absmax_tree(const double* v, int64_t nv, int64_t ng, const int* tree, int n_trees,
                        unsigned long long* out, cudaStream_t s);
void launch_axpy(double* y, const double* x, int64_t n, double alpha, cudaStream_t s);
void launch_anorm_partial(const double* emat, const int64_t* emat_off, const int* elem_m,
                          const int64_t* emap_off, const int32_t* emap, const int64_t* dof_ptr,
                          const int2* dof_el, double* part, const int64_t* y_off, int n_elem,
                          cudaStream_t s);
void launch_convert_panels(const DevCtx& c, const Item* items, int n_items, int to_f32,
                           cudaStream_t s);

}  // namespace uhm_gpu
