// Device engine behind Mesh_: one HBM arena for all fronts, precomputed
// extend-add maps, and a level-by-level program of batched kernel launches.
//
// Replaces, for the hot path, the reference's per-front OpenMP task tree
// (Scheduler_::execute_tree, UHM/src/operation/scheduler.cxx:210-258) and
// the per-front Matrix_FLA_ buffers (UHM/src/matrix/uhm/fla/matrix.cxx:75-164):
// all fronts of one generation are processed by the same launches.
#pragma once

#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "k_tc.cuh"
#include "k_chol_tc.cuh"
#include "mesh.hpp"

namespace uhm {

// precision of a front's factorisation; PREC_LEARNED (a default policy only)
// lets the learned selector pick FP64 / FP32 / BF16X3 per front
enum FrontPrec : int { PREC_FP64 = 0, PREC_FP32 = 1, PREC_BF16X3 = 2, PREC_BF16X6 = 3, PREC_LEARNED = 4 };

struct HostFront {
  Element e = nullptr;
  int slot = 0, level = 0;
  int n = 0, fs = 0, ss = 0, g0 = 0;
  int parent = -1;
  std::vector<int> children;       // slots, in child order
  int prec = PREC_FP64;
  bool tc = false;                 // trailing updates on tensor cores (BF16-split)
  bool tcc = false;                // ... through the cooperative panel kernel (BF16X3 Cholesky, k_chol_tc.cu)
  int64_t ws_off = 0, ws_stride = 0;
  int64_t ws2_row0 = 0;            // first 128-byte row of its parts in the chunk-major workspace
  int64_t ws2b_row0 = 0;           // ... of the panel rows before their TRSM (tc_panel 256)
  int64_t linv_row0 = 0;           // ... of the current panel's Linv parts (tc_panel 256)
  bool blocked = false;            // large front: blocked kernels, 64-col diagonal blocks
  int flag_off = 0;
  int64_t dinv_off = 0;
  int64_t off = 0, voff = 0, inv_off = 0, colptr_off = 0, sgi_off = 0, piv_off = 0;
  int src0 = 0, nsrc = 0;
};

struct ElemSource {                // a copy_in'd element matrix / rhs
  Element e = nullptr;
  int slot = -1;                   // front it scatters into
  int m = 0;
  std::vector<int> pos;            // user row -> front position
  std::vector<int32_t> gdof;       // user row -> global dof (elimination order)
  std::vector<std::pair<int, int>> node_order;  // node ids in user order (for reuse check)
  int64_t mat_off = -1;            // element arena offset (doubles)
  int64_t rhs_off = -1;            // element rhs staging offset (doubles)
  bool has_lhs = false, has_rhs = false;
};

struct Op {
  int kind;
  int dtype;
  int nb;
  int param;
  int64_t item_off;
  int n_items;
  double flops = 0;   // algorithmic flops of this launch (LAWN-41 terms)
  double bytes = 0;   // algorithmic HBM bytes of this launch
  int q0 = 0;         // first right-hand side (flag-driven solves) / CTAs (cooperative LU panel) /
                      // SMs left free for a concurrent launch (tensor-core Cholesky update)
  int aux = 0;        // rows per CTA (cooperative LU panel, flag-driven solves)
  int strm = 0;       // 0: the engine's stream, 1: its side stream (panel lookahead)
};

constexpr int N_OP_KINDS = 40;
struct OpProfile {
  double ms[N_OP_KINDS] = {0}, flops[N_OP_KINDS] = {0}, bytes[N_OP_KINDS] = {0};
  int64_t launches[N_OP_KINDS] = {0};
};

enum OpKind : int {
  OP_ASSEMBLE, OP_SMALL_FACTOR, OP_POTRF, OP_TRSM, OP_SYRK, OP_GETRF, OP_LUROW, OP_GEMM,
  OP_FWD_GATHER, OP_FWD_SMALL, OP_TRSV_F, OP_GEMV_F, OP_BWD_PREP, OP_BWD_SMALL, OP_GEMV_B,
  OP_TRSV_B, OP_BWD_STORE, OP_TC_PACK, OP_TC_SYRK, OP_FWD_FLAGS, OP_BWD_FLAGS, OP_GETRF_COOP,
  OP_LASWP, OP_POTRF_TRSM, OP_ASSEMBLE_SCATTER, OP_TC_GEMM, OP_CHOL_PANEL, OP_TC_CHOL_TRAIL,
  OP_TC_CHOL_SCHUR, OP_CLEAR_FLAGS, OP_CHOL_DIAG, OP_CHOL_PACK, OP_TC_CHOL_TRSM, OP_EV_RECORD, OP_EV_WAIT,
  OP_FWD_CHAIN, OP_BWD_CHAIN, OP_KIND_END
};
static_assert(OP_KIND_END <= N_OP_KINDS, "profile arrays hold N_OP_KINDS op kinds");

struct Timing {
  double upload_ms = 0, factor_ms = 0, solve_ms = 0, refine_ms = 0, total_ms = 0;
  int ir_iters = 0;
  double berr = -1, berr_first = -1;
  int64_t kernel_launches = 0;
};

// Sizes at which the engine switches kernels for a front.  The defaults suit
// the GB300 in general; Engine::autotune picks them per mesh by timing.
struct Tunables {
  int small_max_f64 = 160;   // whole front in shared memory up to this n (FP64; kernel limit 160)
  int small_max_f32 = 224;   // same for FP32 fronts (kernel limit 224)
  int tc_min_n = 512;        // BF16-split Cholesky fronts use the tensor cores from this n
  int gc_min_rows = 512;     // LU panels with this many rows below the diagonal use many CTAs
  int fuse_potrf_trsm = 2;   // Cholesky step: diagonal block + panel TRSM in one launch when it
                             // has at most this many CTAs per SM (0: never)
  int tc_nbo = 256;          // outer panel width of tensor-core fronts (128, 256 or 512)
  int tc_panel = 256;        // BF16X3 Cholesky fronts: 256 = panels of 256 columns, diagonal block
                             // and its inverse by a cooperative kernel, the rows below solved on
                             // the tensor cores; 512 = panels of 512 columns factored whole by the
                             // cooperative kernel (SIMT in-panel work); 0 = the step-by-step path
                             // of the other tensor-core fronts
  int solve_rows = 64;       // rows (columns) per CTA of the flag-driven forward (backward) solves of
                             // large Cholesky fronts (64 or 256)
  int lookahead = 1;         // panels of 256: the next panel's diagonal kernel overlaps the update
  int solve_chain = 0;       // 1: 64-row solves of FP32 fronts as chains (one CTA per front solves
                             // the diagonal blocks, helper CTAs the rest); 0: the flag-driven
                             // kernels, faster on the meshes measured (the chain CTA's per-step
                             // block loads from one SM bound it)
};
constexpr int N_TUNABLES = 10;

class Engine {
 public:
  explicit Engine(Mesh_* m);
  ~Engine();

  // --- set-up -----------------------------------------------------------
  void invalidate_plan() { plan_ok = false; }
  void invalidate_precision() { prec_dirty = true; }
  void copy_in(Element e, int m, int n, int nod_disp, const int* nods, int side,
               const double* buf);
  void copy_out(Element e, int m, int n, int nod_disp, const int* nods, int side, double* buf);
  // bulk: element matrices of all leaves, in leaf order (Mesh_::leaves), each
  // m_e x m_e column-major in the element's own node order, back to back
  void copy_in_leaves(int side, const double* buf, int64_t n_values);
  void copy_out_leaves(double* buf, int64_t n_values);
  // element matrices of all leaves generated on the device (hp-FEM Lobatto
  // modes, k_elements.cu) instead of copied in; leaf order as copy_in_leaves
  void generate_lobatto_elements(int method, int dim, double hh, double cmass, double cconv, int n_el,
                                 const double* ref, const int64_t* ref_off, int n_ref_off, const int* p_el,
                                 const double* kappa, const double* react, const double* beta,
                                 const int64_t* sel_ptr, const int32_t* sel);
  // element maps of all leaves from their node lists (leaf order, single physics)
  void set_leaf_nodes(const int* nods_all);
  // The assembled operator and right-hand sides as a sparse matrix, the
  // reference's DSparse_ (UHM/src/interf/sparse.cxx:188-460): every leaf's
  // element matrix added in leaf order into entries keyed by global
  // (row, col) -- (col, row) when cs -- then listed in key order as
  // triplets or compressed rows (columns when cs); is_sym keeps col >= row
  // of the key; fort adds 1 to every index.  sparse.cpp.
  struct SparseOut {
    int n_dof = 0, n_rhs = 0;
    std::vector<int> ia, ja;
    std::vector<double> a, b;
  };
  void export_sparse(int is_sym, int fort, int cs, int compress, int axpy, SparseOut& out);
  // Mesh_::random_spd_matrix / random_matrix (UHM/src/mesh/matrix.cxx:
  // 155-170,295-310): every leaf gets a pseudo-random element matrix and
  // right-hand sides (fill.cpp)
  void random_elements(int spd);
  uint64_t random_calls = 0;
  void node_solution(int n_nodes, const int* ids, double* out, int64_t n_values);
  // one block of a front (uhm::Matrix_::copy_out): UHM_ATL / ATR / ABL / ABR
  // after a factorisation, UHM_P (int pivots, LU), UHM_XT / XB after a solve;
  // column-major, leading dimension = the block's rows
  bool front_block_ready(Element e, int mat) const;
  void front_block(Element e, int mat, void* out);

  // --- numerics -----------------------------------------------------------
  void factor(int method);
  void solve(int method, int phase);          // 1 forward, 2 backward, 3 both
  double residual_norm1();                    // sum |b - A x| (unassembled A)
  double backward_error();                    // ||b-Ax||/(||A|| ||x|| + ||b||), inf-norms

  // --- configuration ------------------------------------------------------
  int mode = 0;            // 0 plain FP64, 1 mixed (per-front precision + IR)
  int default_prec = PREC_FP32;
  double ir_tol = 1e-12;
  int ir_max = 10;
  std::vector<int> front_prec_override;       // by slot, -1 = default
  std::vector<float> selector_params;         // MLP parameters for PREC_LEARNED
  std::vector<int> learned_class;             // by slot: 0 FP64, 1 FP32, 2 BF16-split
  void set_selector(const float* params, int n);
  Tunables tune;
  void set_tunables(const int* v);            // N_TUNABLES values, checked against the kernel limits
  void get_tunables(int* v) const;
  // coordinate descent over candidate values of every tunable: each candidate
  // whose launch programs differ from one already timed is timed over `reps`
  // factor+solve(+refine) runs (minimum kept); the fastest is kept.  Element
  // matrices and right-hand sides must have been copied in.  Returns the
  // number of timed candidates; the mesh is left factored and solved with
  // the chosen values.
  int autotune(int method, int reps);
  // device buffers for the current plan and precisions (no factorisation)
  void prepare_device(int method);
  // per-front selector features (slot order, SEL_F floats each); element
  // matrices must have been copied in
  void front_features(std::vector<float>& feat);
  int status = 0;
  int n_refactored = 0;         // fronts the last factorisation redid (the rest were kept)
  std::string last_error;
  Timing timing;
  bool profiling = false;       // per-op CUDA events (outside timed regions)
  struct OpRecord {
    int kind, n_items;
    float ms;
  };
  std::vector<OpRecord> op_log;  // every profiled launch, in launch order
  bool use_graphs = true;       // replay factor / solve programs as CUDA graphs
  OpProfile profile;

  // --- introspection ------------------------------------------------------
  std::vector<HostFront> fronts;              // by slot (leaf -> root order)
  std::vector<std::vector<int>> levels;       // slots per generation, leaf -> root
  int64_t n_global = 0;
  void ensure_plan();
  int method_built = 0;

 private:
  Mesh_* mesh;
  bool plan_ok = false;
  bool prec_dirty = false;
  bool learned_valid = false;
  void apply_selector(int method);
  bool emat_device_only = false, erhs_device_only = false;
  bool anorm_valid = false;
  bool dev_ok = false;
  bool factored = false;
  bool solved = false;          // the solution slabs hold the last solve's rows
  int factored_method = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;    // side stream of the panel lookahead
  cudaStream_t stream3 = nullptr;    // side stream of ||A||_inf, beside the factorisation
  cudaEvent_t ev_up = nullptr, ev_anorm = nullptr;
  bool anorm_pending = false;        // ||A||_inf enqueued on stream3, not yet joined into stream
  void sync_anorm();                 // stream waits for it (it writes d_y, d_r and d_red[1536..])
  std::vector<cudaEvent_t> evpool;   // events ordering the two streams (by id)
  static bool is_kernel_op(int kind) {
    return kind != OP_CLEAR_FLAGS && kind != OP_EV_RECORD && kind != OP_EV_WAIT;
  }
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_mid = nullptr;
  int* h_words = nullptr;            // pinned: the fronts' status words and the wait error word, read back together
  size_t h_words_n = 0;
  double* h_red = nullptr;           // pinned: scalars the refinement reads back (8)
  void read_status_words(const char* where);   // after the stream sync that follows the copies of enqueue_status_words
  void enqueue_status_words();

  // element sources
  std::vector<ElemSource> esrc;
  std::vector<int> esrc_of_slot;              // slot -> index in esrc (or -1)
  std::vector<double> h_emat;                 // staged element matrices (host)
  std::vector<double> h_erhs;                 // staged element rhs
  int64_t emat_total = 0, erhs_total = 0;
  bool emat_dirty = true, erhs_dirty = true;
  double* h_pinned = nullptr;
  bool h_pinned_is_malloc = false;
  size_t h_pinned_bytes = 0;

  // host-side device images
  std::vector<uhm_gpu::FrontDev> h_fronts;
  std::vector<uhm_gpu::SrcDev> h_srcs;
  std::vector<int32_t> h_inv, h_sgi, h_fwd;
  std::vector<int64_t> h_colptr;
  std::vector<int2> h_colsrc;
  std::vector<uhm_gpu::Item> h_items;
  std::vector<Op> fac_ops, fwd_ops, bwd_ops;
  // factor reuse: fronts whose factor from the last factorisation of this
  // plan is held (by slot), leaves whose element matrix changed since (by
  // element source), and the factor program over the fronts to redo
  std::vector<char> front_kept, leaf_changed;
  std::vector<Op> fac_ops_part;
  std::vector<char> part_mask;
  const std::vector<char>* fac_mask = nullptr;   // build_programs: factor only these slots
  uhm_gpu::Item* d_items_part = nullptr;
  size_t d_items_part_cap = 0;
  void build_partial(int method, const std::vector<char>& act);
  int64_t arena64_n = 0, arena32_n = 0, vec_n = 0, piv_n = 0;
  int64_t dinv64_n = 0, dinv32_n = 0, flags_n = 0;
  int* d_ticket = nullptr;

  // device memory
  uhm_gpu::DevCtx ctx{};
  uhm_gpu::Item* d_items = nullptr;
  double* d_b = nullptr;        // assembled rhs (elimination order)
  double* d_x = nullptr;        // solution
  double* d_r = nullptr;        // residual / correction rhs
  double* d_d = nullptr;        // correction
  double* d_erhs = nullptr;     // element rhs (FP64)
  double* d_y = nullptr;        // per-element A_e x_e
  double* d_red = nullptr;      // reduction scratch
  double* d_scratch = nullptr;  // backward-solve partial sums
  float* d_sel = nullptr;       // selector scratch: element statistics, features, parameters, probabilities
  int64_t* d_scr_off = nullptr;
  int* d_counters = nullptr;
  void* d_ws2 = nullptr;             // chunk-major BF16 parts of the cooperative-panel fronts
  int64_t ws2_rows = 0;              // its size in rows of 64 BF16
  int64_t* d_ws2_row0 = nullptr;     // per front: first row of its parts
  CUtensorMap ws2_map;
  int* d_pflags = nullptr;           // tickets and flags of the panel launches (cleared per factorisation)
  int64_t* d_ws2b_row0 = nullptr;
  int64_t* d_linv_row0 = nullptr;
  int64_t pflags_n = 0;
  uint64_t* d_hand = nullptr;        // the factorisation count (first word), then the diagonal-block
                                     // launches' hand-off words, CD_HAND_WORDS per front slot
  int64_t hand_n = 0;                // front slots of d_hand
  int64_t hand_factorisations = 0;   // factorisations run (the clearing of d_hand's words)
  void* d_ws = nullptr;              // BF16 operand parts of tensor-core fronts
  int64_t* d_ws_off = nullptr;
  int64_t* d_ws_stride = nullptr;
  CUtensorMap ws_map;                // one map over the whole BF16 workspace
  int* d_err = nullptr;              // bounded-wait error flag of device kernels
  unsigned char* d_gen = nullptr;    // recipe of the element generator (one block)
  size_t d_gen_bytes = 0;
  double* d_gc_xbuf = nullptr;       // exchange buffer of the cooperative LU panel
  unsigned int* d_gc_ctr = nullptr;  // its grid-barrier counter and abort word
  int n_sm = 0;
  int64_t ws_total = 0;
  int64_t* d_emat_off = nullptr;
  int* d_elem_m = nullptr;
  int64_t* d_emap_off = nullptr;
  int32_t* d_emap = nullptr;
  int64_t* d_y_off = nullptr;
  int64_t* d_dof_ptr = nullptr;
  int64_t* d_dof_idx = nullptr;
  int2* d_dof_el = nullptr;
  std::vector<int64_t> h_emat_off, h_emap_off, h_y_off;
  std::vector<int> h_elem_m;
  std::vector<int32_t> h_emap;
  int64_t y_total = 0;
  std::vector<void*> allocations;
  double anorm_inf = -1.0;
  std::vector<double> h_x;      // cached solution on host
  bool h_x_valid = false;

  void build_plan(int method);
  void build_programs(int method);
  void alloc_device(int method);
  void free_device();
  void upload_elements();
  void assemble_rhs();
  void run_ops(const std::vector<Op>& ops, double* g_in, double* g_out);
  // items of the ops at base (d_items when null)
  void launch_ops(const std::vector<Op>& ops, double* g_in, double* g_out, const uhm_gpu::Item* base = nullptr);
  struct GraphEntry {
    const std::vector<Op>* ops;
    double* gin;
    double* gout;
    int eager_runs;
    cudaGraphExec_t exec;
  };
  std::vector<GraphEntry> graphs;
  void clear_graphs();
  void solve_into(int method, double* rhs, double* out, int phase);
  void compute_residual(const double* x, double* r);
  double operator_norm_inf();
  void enqueue_anorm();
  double read_scalar(const double* d);
  // forests (several independent trees, e.g. a batch of meshes): the
  // backward error is taken per tree and the worst one is reported, so that
  // every mesh of a batch meets the tolerance on its own operator
  int n_trees = 1;
  int* d_dof_tree = nullptr;                  // tree of each global dof
  unsigned long long* d_tree_red = nullptr;   // 4 slots x n_trees: r, x, b, A maxima
  std::vector<double> tree_bnorm, tree_anorm;
  void tree_max_async(const double* v, int64_t nv, int64_t ng, int slot);
  std::vector<double> read_tree_slot(int slot);
  double forest_berr(const std::vector<double>& rn, const std::vector<double>& xn);
  void refine(int method);
  void check_device_error(const char* where);
  void* dmalloc(size_t bytes);
  int64_t add_items(const std::vector<uhm_gpu::Item>& it);
  void fail(const std::string& msg, int code);
  // A status left by an earlier solve (refinement redone in FP64, a bad
  // right-hand side, a device wait that gave up) does not carry over to the
  // next solve or to new right-hand sides.
  void clear_solve_status() {
    if (status == 20 || status == 13 || status == 14) {
      status = 0;
      last_error.clear();
    }
  }
  void element_map(Element e, int nod_disp, const int* nods, std::vector<std::pair<int, int>>& order,
                   std::vector<int>& pos, std::vector<int32_t>& gd);
  void fetch_x();
  void release_staging();
};

}  // namespace uhm
