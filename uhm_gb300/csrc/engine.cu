// Host side of the device engine: plan (front table, extend-add maps, launch
// program), HBM arenas, element staging, factor / solve / residual drivers.
#include "engine.hpp"
#include "selector.hpp"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <unordered_map>

namespace uhm {
using namespace uhm_gpu;

static constexpr int SMALL_MAX_F64 = 160;   // whole front in shared memory (200 KB)
static constexpr int SMALL_MAX_F32 = 224;
static constexpr int NB = 64;               // panel width of the blocked kernels
static constexpr int ASM_TJ = 16;           // assembly column tile (k_factor.cu)
static constexpr int ASM_SCATTER_MIN = 2048;  // fronts this large: one column per CTA, shared-memory scatter
static constexpr int ASM_SCATTER_MAX = 26624; // the FP64 column fits 208 KB of shared memory
static constexpr int TRSM_RB = 64;
static constexpr int FWD_RB = 256;            // k_solve.cu
static constexpr int BWD_RB = 512;
static constexpr int LUROW_CB = 64;
static constexpr int TILE = 64;             // trailing-update tile (k_tile_update)

#define CK(x)                                                                          \
  do {                                                                                 \
    cudaError_t e_ = (x);                                                              \
    if (e_ != cudaSuccess)                                                             \
      throw std::runtime_error(std::string(#x) + ": " + cudaGetErrorString(e_));       \
  } while (0)

Engine::Engine(Mesh_* m) : mesh(m) {}

Engine::~Engine() {
  try {
    free_device();
  } catch (...) {
  }
  release_staging();
  for (cudaEvent_t e : evpool) cudaEventDestroy(e);
  if (stream2) cudaStreamDestroy(stream2);
  if (stream3) cudaStreamDestroy(stream3);
  if (ev_up) cudaEventDestroy(ev_up);
  if (ev_anorm) cudaEventDestroy(ev_anorm);
  if (stream) cudaStreamDestroy(stream);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (ev_mid) cudaEventDestroy(ev_mid);
  if (h_words) cudaFreeHost(h_words);
  if (h_red) cudaFreeHost(h_red);
}

void Engine::fail(const std::string& msg, int code) {
  status = code;
  last_error = msg;
  throw std::runtime_error(msg);
}

void* Engine::dmalloc(size_t bytes) {
  void* p = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail("device allocation of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e), 4);
  }
  allocations.push_back(p);
  return p;
}

void Engine::free_device() {
  if (stream) cudaStreamSynchronize(stream);
  if (stream3) cudaStreamSynchronize(stream3);
  anorm_pending = false;
  clear_graphs();
  for (void* p : allocations) cudaFree(p);
  allocations.clear();
  dev_ok = false;
  ctx = DevCtx{};
  d_items = nullptr;
  d_b = d_x = d_r = d_d = d_erhs = d_y = d_red = d_scratch = nullptr;
  d_sel = nullptr;
  d_ws = nullptr;
  d_ws_off = d_ws_stride = nullptr;
  d_ws2 = nullptr;
  d_ws2_row0 = nullptr;
  d_ws2b_row0 = d_linv_row0 = nullptr;
  d_pflags = nullptr;
  d_hand = nullptr;
  d_err = nullptr;
  d_dof_tree = nullptr;
  d_tree_red = nullptr;
  d_gc_xbuf = nullptr;
  d_gc_ctr = nullptr;
  d_gen = nullptr;
  d_gen_bytes = 0;
  d_items_part = nullptr;
  d_items_part_cap = 0;
  fac_ops_part.clear();
  part_mask.clear();
  front_kept.clear();
  tree_bnorm.clear();
  tree_anorm.clear();
}

// ---------------------------------------------------------------------------
// plan: fronts in leaf -> root order, grouped by generation
// ---------------------------------------------------------------------------
void Engine::ensure_plan() {
  if (plan_ok) return;
  if (!mesh->is_locked()) fail("mesh is not locked", 5);
  fronts.clear();
  levels.clear();
  int slot = 0;
  for (auto& kv : mesh->by_generation) {
    levels.emplace_back();
    for (Element e : kv.second) {
      if (!e->is_matrix_created()) fail("create_matrix_without_buffer has not been called", 5);
      HostFront hf;
      hf.e = e;
      hf.slot = slot;
      e->slot = slot;
      hf.level = (int)levels.size() - 1;
      std::pair<int, int> d = e->get_n_dof();
      hf.fs = d.first;
      hf.ss = d.second;
      hf.n = hf.fs + hf.ss;
      hf.g0 = e->factor.empty() ? 0 : e->factor[0].first->get_offset();
      int o = hf.g0;
      for (auto& pr : e->factor) {
        if (pr.first->get_offset() != o) fail("factor dofs of a front are not contiguous", 6);
        o += pr.first->get_n_dof();
      }
      fronts.push_back(hf);
      levels.back().push_back(slot);
      ++slot;
    }
  }
  n_global = 0;
  for (auto& f : fronts) {
    f.parent = f.e->parent ? f.e->parent->slot : -1;
    f.children.clear();
    for (Element c : f.e->children) f.children.push_back(c->slot);
    n_global += f.fs;
  }
  // element staging: one slot per leaf (matrix m*m and rhs m*n_rhs)
  esrc.clear();
  esrc_of_slot.assign(fronts.size(), -1);
  emat_total = erhs_total = 0;
  const int nr = mesh->n_rhs;
  for (Element e : mesh->leaves) {
    ElemSource es;
    es.e = e;
    es.slot = e->slot;
    int m = 0;
    for (auto& kv : e->nodes) m += kv.first->get_n_dof();
    es.m = m;
    es.mat_off = emat_total;
    es.rhs_off = erhs_total;
    emat_total += (int64_t)m * m;
    erhs_total += (int64_t)m * nr;
    esrc_of_slot[e->slot] = (int)esrc.size();
    esrc.push_back(std::move(es));
  }
  leaf_changed.assign(esrc.size(), 1);
  front_kept.assign(fronts.size(), 0);
  size_t need = (size_t)(emat_total + erhs_total) * sizeof(double);
  if (need > h_pinned_bytes || !h_pinned) {
    release_staging();
    // page-locked staging; plain host memory when no device is present
    // (symbolic analysis and structure queries need no GPU)
    if (cudaMallocHost((void**)&h_pinned, std::max<size_t>(need, 64)) != cudaSuccess) {
      cudaGetLastError();
      h_pinned = (double*)std::malloc(std::max<size_t>(need, 64));
      h_pinned_is_malloc = true;
      if (!h_pinned) fail("host allocation failed", 4);
    }
    h_pinned_bytes = need;
  }
  emat_dirty = erhs_dirty = true;
  learned_valid = false;
  anorm_inf = -1.0;
  plan_ok = true;
  dev_ok = false;
  factored = false;
  h_x_valid = false;
}

void Engine::release_staging() {
  if (!h_pinned) return;
  if (h_pinned_is_malloc) std::free(h_pinned);
  else cudaFreeHost(h_pinned);
  h_pinned = nullptr;
  h_pinned_is_malloc = false;
  h_pinned_bytes = 0;
}

static std::unordered_map<Node, int> front_positions(Element e) {
  std::unordered_map<Node, int> pos;
  int fs = 0;
  for (auto& pr : e->factor) { pos[pr.first] = pr.second; fs += pr.first->get_n_dof(); }
  for (auto& pr : e->schur) pos[pr.first] = fs + pr.second;
  return pos;
}

// ---------------------------------------------------------------------------
// copy_in / copy_out  (Mesh_::copy_in / copy_out, UHM/src/mesh/interf.cxx:108-204)
// ---------------------------------------------------------------------------
void Engine::element_map(Element e, int nod_disp, const int* nods,
                         std::vector<std::pair<int, int>>& order, std::vector<int>& pos,
                         std::vector<int32_t>& gd) {
  order.clear();
  pos.clear();
  gd.clear();
  auto fpos = front_positions(e);
  for (int i = 0; i < e->get_n_nodes(); ++i) {
    std::pair<int, int> id = nod_disp == UHM_PHYSICS_MULTI ? std::make_pair(nods[2 * i], nods[2 * i + 1])
                                                           : std::make_pair(nods[i], 0);
    Node nd = mesh->find_node(id);
    if (!nd) fail("copy_in: cannot find node in the mesh", 7);
    order.push_back(id);
    if (!nd->get_n_dof()) continue;
    auto it = fpos.find(nd);
    if (it == fpos.end()) fail("copy_in: node does not belong to the element", 7);
    for (int k = 0; k < nd->get_n_dof(); ++k) {
      pos.push_back(it->second + k);
      gd.push_back(nd->get_offset() + k);
    }
  }
}

void Engine::set_leaf_nodes(const int* nods_all) {
  ensure_plan();
  int64_t k = 0;
  for (auto& es : esrc) {
    std::vector<std::pair<int, int>> order;
    std::vector<int> pos;
    std::vector<int32_t> gd;
    element_map(es.e, UHM_PHYSICS_SINGLE, nods_all + k, order, pos, gd);
    k += es.e->get_n_nodes();
    if ((int)pos.size() != es.m) fail("set_leaf_nodes: element size mismatch", 7);
    if (!es.node_order.empty() && es.node_order != order)
      fail("set_leaf_nodes: node order differs from an earlier copy_in", 7);
    if (es.node_order.empty()) dev_ok = false;
    es.node_order = order;
    es.pos = pos;
    es.gdof = gd;
  }
}

void Engine::fetch_x() {
  if (h_x_valid) return;
  h_x.resize((size_t)n_global * mesh->n_rhs);
  CK(cudaMemcpyAsync(h_x.data(), d_x, sizeof(double) * h_x.size(), cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  h_x_valid = true;
}

void Engine::node_solution(int n_nodes, const int* ids, double* out, int64_t n_values) {
  ensure_plan();
  if (!factored) fail("node_solution: nothing solved", 9);
  fetch_x();
  const int nr = mesh->n_rhs;
  int64_t rows = 0;
  for (int i = 0; i < n_nodes; ++i) {
    Node nd = mesh->find_node(ids[i]);
    if (!nd) fail("node_solution: unknown node", 7);
    rows += nd->get_n_dof();
  }
  if (rows * nr != n_values) fail("node_solution: size mismatch", 7);
  int64_t r = 0;
  for (int i = 0; i < n_nodes; ++i) {
    Node nd = mesh->find_node(ids[i]);
    for (int k = 0; k < nd->get_n_dof(); ++k, ++r)
      for (int q = 0; q < nr; ++q) out[r + q * rows] = h_x[(size_t)(nd->get_offset() + k) + (size_t)q * n_global];
  }
}

void Engine::copy_in(Element e, int m, int n, int nod_disp, const int* nods, int side,
                     const double* buf) {
  ensure_plan();
  if (side != UHM_LHS) clear_solve_status();
  if (m <= 0 || n <= 0) fail("copy_in: dimension is null", 7);
  std::vector<std::pair<int, int>> order;
  std::vector<int> pos;
  std::vector<int32_t> gd;
  element_map(e, nod_disp, nods, order, pos, gd);
  if ((int)pos.size() != m) fail("copy_in: m does not match the element's dofs", 7);
  int ei = esrc_of_slot[e->slot];
  if (ei < 0) fail("copy_in: only leaf elements carry element matrices in this engine", 7);
  ElemSource& es = esrc[ei];
  if (es.m != m) fail("copy_in: size mismatch", 7);
  bool first = es.node_order.empty();
  std::vector<int> perm;   // user row -> stored row
  if (first) {
    es.node_order = order;
    es.pos = pos;
    es.gdof = gd;
  } else if (order != es.node_order) {
    std::unordered_map<int, int> row_of;
    for (int r = 0; r < m; ++r) row_of[es.pos[r]] = r;
    perm.resize(m);
    for (int r = 0; r < m; ++r) perm[r] = row_of[pos[r]];
  }
  auto rowmap = [&](int r) { return perm.empty() ? r : perm[r]; };
  // copy_in adds into the host staging copy: fetch it first when the
  // current data only exist on the device (bulk device copy, generated)
  if (dev_ok && side == UHM_LHS && emat_device_only) {
    CK(cudaStreamSynchronize(stream));
    CK(cudaMemcpy(h_pinned, ctx.emat, sizeof(double) * (size_t)emat_total, cudaMemcpyDeviceToHost));
    emat_device_only = false;
  }
  if (dev_ok && side != UHM_LHS && erhs_device_only) {
    CK(cudaStreamSynchronize(stream));
    CK(cudaMemcpy(h_pinned + emat_total, d_erhs, sizeof(double) * (size_t)erhs_total, cudaMemcpyDeviceToHost));
    erhs_device_only = false;
  }
  if (side == UHM_LHS) {
    double* dst = h_pinned + es.mat_off;
    if (!es.has_lhs) std::memset(dst, 0, sizeof(double) * (size_t)m * m);
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) dst[rowmap(i) + (int64_t)rowmap(j) * m] += buf[i + (int64_t)j * m];
    es.has_lhs = true;
    emat_dirty = true;
    leaf_changed[ei] = 1;
    learned_valid = false;
    anorm_valid = false;
    anorm_inf = -1.0;
    dev_ok = dev_ok && !first;   // maps change when an element appears
    factored = false;
  } else {
    if (n != mesh->n_rhs) fail("copy_in: n_rhs mismatch", 7);
    double* dst = h_pinned + emat_total + es.rhs_off;
    if (!es.has_rhs) std::memset(dst, 0, sizeof(double) * (size_t)m * n);
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < m; ++i) dst[rowmap(i) + (int64_t)q * m] += buf[i + (int64_t)q * m];
    es.has_rhs = true;
    erhs_dirty = true;
    if (first) dev_ok = false;
  }
}

void Engine::copy_in_leaves(int side, const double* buf, int64_t n_values) {
  ensure_plan();
  for (auto& es : esrc)
    if (es.node_order.empty()) fail("copy_in_leaves: element maps unknown (call uhm_gpu_set_leaf_nodes first)", 7);
  if (side == UHM_LHS) {
    if (n_values != emat_total) fail("copy_in_leaves: size mismatch", 7);
    std::fill(leaf_changed.begin(), leaf_changed.end(), 1);
    if (!dev_ok) {
      std::memcpy(h_pinned, buf, sizeof(double) * (size_t)emat_total);
      for (auto& es : esrc) es.has_lhs = true;
      emat_dirty = true;
      anorm_valid = false;
    } else {
      CK(cudaMemcpyAsync(ctx.emat, buf, sizeof(double) * (size_t)emat_total, cudaMemcpyHostToDevice, stream));
      emat_dirty = false;
      emat_device_only = true;
      anorm_valid = false;
    }
    learned_valid = false;
    factored = false;
    anorm_inf = -1.0;
  } else {
    clear_solve_status();
    if (n_values != erhs_total) fail("copy_in_leaves: size mismatch", 7);
    if (!dev_ok) {
      std::memcpy(h_pinned + emat_total, buf, sizeof(double) * (size_t)erhs_total);
      for (auto& es : esrc) es.has_rhs = true;
      erhs_dirty = true;
    } else {
      CK(cudaMemcpyAsync(d_erhs, buf, sizeof(double) * (size_t)erhs_total, cudaMemcpyHostToDevice, stream));
      erhs_dirty = false;
      erhs_device_only = true;
    }
  }
}

void Engine::generate_lobatto_elements(int method, int dim, double hh, double cmass, double cconv, int n_el,
                                       const double* ref, const int64_t* ref_off, int n_ref_off, const int* p_el,
                                       const double* kappa, const double* react, const double* beta,
                                       const int64_t* sel_ptr, const int32_t* sel) {
  ensure_plan();
  if (dim != 2 && dim != 3) fail("generate_lobatto_elements: dim must be 2 or 3", 7);
  if (n_el != (int)esrc.size()) fail("generate_lobatto_elements: element count differs from the mesh's leaves", 7);
  // every index the kernel derives from the recipe is checked here: modes
  // inside the (p+1)^dim tensor grid, each order's 1D matrices inside ref
  int64_t n_ref = 0;
  if (sel_ptr[0] != 0) fail("generate_lobatto_elements: sel_ptr[0] must be 0", 7);
  for (int e = 0; e < n_el; ++e) {
    const int64_t m = sel_ptr[e + 1] - sel_ptr[e];
    const int p = p_el[e];
    if (p < 1 || p > 7 || p >= n_ref_off) fail("generate_lobatto_elements: order outside 1..7", 7);
    if (esrc[e].node_order.empty())
      fail("generate_lobatto_elements: element node lists unknown (copy_in_leaves with node lists first)", 7);
    if (m != esrc[e].m) fail("generate_lobatto_elements: retained modes differ from the element's dofs", 7);
    const int q = p + 1;
    const int64_t grid = dim == 3 ? (int64_t)q * q * q : (int64_t)q * q;
    if (m > grid) fail("generate_lobatto_elements: more retained modes than the element has", 7);
    for (int64_t k = sel_ptr[e]; k < sel_ptr[e + 1]; ++k)
      if (sel[k] < 0 || sel[k] >= grid) fail("generate_lobatto_elements: retained mode outside the tensor grid", 7);
    if (ref_off[p] < 0) fail("generate_lobatto_elements: negative ref_off", 7);
    n_ref = std::max<int64_t>(n_ref, ref_off[p] + 3 * (int64_t)q * q);
  }
  // the assembly programs list an element source only for leaves that carry a
  // matrix, so mark them before the programs are built
  for (auto& es : esrc) es.has_lhs = true;
  std::fill(leaf_changed.begin(), leaf_changed.end(), 1);
  prepare_device(method);
  const int64_t n_sel = sel_ptr[n_el];
  std::vector<int64_t> off(n_el);
  for (int e = 0; e < n_el; ++e) off[e] = esrc[e].mat_off;
  // the recipe in one device buffer (kept with the plan's allocations):
  // each array at a 16-byte-aligned offset of one host staging block
  std::vector<unsigned char> stage;
  auto place = [&](const void* src, size_t bytes) -> size_t {
    const size_t o = (stage.size() + 15) & ~size_t(15);
    stage.resize(o + bytes);
    if (bytes) std::memcpy(stage.data() + o, src, bytes);
    return o;
  };
  const size_t o_off = place(off.data(), sizeof(int64_t) * n_el);
  const size_t o_p = place(p_el, sizeof(int) * n_el);
  const size_t o_kap = place(kappa, sizeof(double) * n_el);
  const size_t o_rea = react ? place(react, sizeof(double) * n_el) : 0;
  const size_t o_beta = beta ? place(beta, sizeof(double) * dim) : 0;
  const size_t o_sp = place(sel_ptr, sizeof(int64_t) * (n_el + 1));
  const size_t o_sel = place(sel, sizeof(int32_t) * n_sel);
  const size_t o_ref = place(ref, sizeof(double) * n_ref);
  // per-order tables (device only) after the staged arrays
  bool used[8] = {};
  for (int e = 0; e < n_el; ++e) used[p_el[e]] = true;
  int64_t tab_off[8] = {}, n_tab = 0;
  for (int p = 1; p <= 7; ++p)
    if (used[p]) {
      tab_off[p] = n_tab;
      n_tab += uhm_gpu::gen_table_doubles(p, dim, react != nullptr, beta != nullptr);
    }
  const size_t o_toff = place(tab_off, sizeof(tab_off));
  const size_t o_tab = (stage.size() + 15) & ~size_t(15);
  const size_t need = o_tab + sizeof(double) * (size_t)n_tab;
  if (need > d_gen_bytes) {
    d_gen = (unsigned char*)dmalloc(need);
    d_gen_bytes = need;
  }
  CK(cudaMemcpyAsync(d_gen, stage.data(), stage.size(), cudaMemcpyHostToDevice, stream));
  unsigned char* g = d_gen;
  auto* d_tab = (double*)(g + o_tab);
  CK(cudaEventRecord(ev0, stream));
  for (int p = 1; p <= 7; ++p)
    if (used[p])
      uhm_gpu::launch_gen_tables(d_tab + tab_off[p], (const double*)(g + o_ref) + ref_off[p], p, dim, hh, cmass,
                                 cconv, react != nullptr, beta != nullptr, stream);
  uhm_gpu::launch_gen_lobatto(ctx.emat, (const int64_t*)(g + o_off), n_el, (const int*)(g + o_p),
                              (const double*)(g + o_kap), react ? (const double*)(g + o_rea) : nullptr,
                              beta ? (const double*)(g + o_beta) : nullptr, (const int64_t*)(g + o_sp),
                              (const int32_t*)(g + o_sel), d_tab, (const int64_t*)(g + o_toff), dim, stream);
  CK(cudaGetLastError());
  CK(cudaEventRecord(ev1, stream));
  CK(cudaStreamSynchronize(stream));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, ev0, ev1));
  timing = Timing{};
  timing.upload_ms = ms;   // the generation kernels' device time
  int n_launch = 1;
  for (int p = 1; p <= 7; ++p) n_launch += used[p];
  timing.kernel_launches = n_launch;
  emat_dirty = false;
  emat_device_only = true;
  anorm_valid = false;
  learned_valid = false;
  factored = false;
  anorm_inf = -1.0;
}

bool Engine::front_block_ready(Element e, int mat) const {
  if (!e || e->slot < 0 || e->slot >= (int)fronts.size() || fronts[e->slot].e != e) return false;
  if (mat == UHM_XT || mat == UHM_XB) return solved;
  if (mat == UHM_P) return factored && factored_method != UHM_CHOL;
  return factored && (mat == UHM_ATL || mat == UHM_ATR || mat == UHM_ABL || mat == UHM_ABR);
}

void Engine::front_block(Element e, int mat, void* out) {
  if (!front_block_ready(e, mat)) fail("front_block: block not available", 9);
  const HostFront& f = fronts[e->slot];
  const int n = f.n, fs = f.fs, nr = mesh->n_rhs;
  CK(cudaStreamSynchronize(stream));
  if (mat == UHM_P) {
    if (fs) CK(cudaMemcpy(out, ctx.piv + f.piv_off, sizeof(int32_t) * fs, cudaMemcpyDeviceToHost));
    return;
  }
  double* o = static_cast<double*>(out);
  if (mat == UHM_XT || mat == UHM_XB) {
    const int r0 = mat == UHM_XT ? 0 : fs, m = mat == UHM_XT ? fs : f.ss;
    std::vector<double> y((size_t)n * nr);
    CK(cudaMemcpy(y.data(), ctx.vec + f.voff + (int64_t)n * nr, sizeof(double) * y.size(), cudaMemcpyDeviceToHost));
    for (int q = 0; q < nr; ++q)
      for (int i = 0; i < m; ++i) o[(size_t)q * m + i] = y[(size_t)q * n + r0 + i];
    return;
  }
  const int r0 = (mat == UHM_ATL || mat == UHM_ATR) ? 0 : fs, c0 = (mat == UHM_ATL || mat == UHM_ABL) ? 0 : fs;
  const int m = r0 == 0 ? fs : f.ss, nc = c0 == 0 ? fs : f.ss;
  if (!m || !nc) return;
  const bool f64 = h_fronts[f.slot].dtype == F64;
  if (f64) {
    CK(cudaMemcpy2D(o, sizeof(double) * m, ctx.a64 + f.off + r0 + (int64_t)c0 * n, sizeof(double) * n,
                    sizeof(double) * m, nc, cudaMemcpyDeviceToHost));
  } else {
    std::vector<float> t((size_t)m * nc);
    CK(cudaMemcpy2D(t.data(), sizeof(float) * m, ctx.a32 + f.off + r0 + (int64_t)c0 * n, sizeof(float) * n,
                    sizeof(float) * m, nc, cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < t.size(); ++k) o[k] = t[k];
  }
  if (factored_method != UHM_CHOL) return;
  // Cholesky keeps the lower triangles; the 64 x 64 diagonal blocks of a
  // blocked front are held by their inverses (the solves use those), so L
  // there is the inverse of the inverse, by forward substitution
  if (mat == UHM_ATL || mat == UHM_ABR)
    for (int j = 0; j < nc; ++j)
      for (int i = 0; i < std::min(j, m); ++i) o[(size_t)j * m + i] = 0.0;
  if (mat == UHM_ATL && f.blocked) {
    const int nfb = (fs + NB - 1) / NB;
    std::vector<double> di((size_t)NB * NB);
    for (int b = 0; b < nfb; ++b) {
      const int kb = std::min(NB, fs - NB * b);
      if (f64) {
        CK(cudaMemcpy(di.data(), ctx.dinv64 + f.dinv_off + (int64_t)b * NB * NB, sizeof(double) * NB * NB,
                      cudaMemcpyDeviceToHost));
      } else {
        std::vector<float> t((size_t)NB * NB);
        CK(cudaMemcpy(t.data(), ctx.dinv32 + f.dinv_off + (int64_t)b * NB * NB, sizeof(float) * NB * NB,
                      cudaMemcpyDeviceToHost));
        for (int k = 0; k < NB * NB; ++k) di[k] = t[k];
      }
      // X = dinv (lower, column-major); L = X^{-1}: solve X L = I column by column
      for (int c = 0; c < kb; ++c)
        for (int i = 0; i < kb; ++i) {
          double v = 0.0;
          if (i >= c) {
            double t = i == c ? 1.0 : 0.0;
            for (int k = c; k < i; ++k) t -= di[(size_t)k * NB + i] * o[(size_t)(NB * b + c) * m + NB * b + k];
            v = t / di[(size_t)i * NB + i];
          }
          o[(size_t)(NB * b + c) * m + NB * b + i] = v;
        }
    }
  }
}

void Engine::copy_out(Element e, int m, int n, int nod_disp, const int* nods, int side, double* buf) {
  ensure_plan();
  if (side != UHM_RHS) fail("copy_out: only the solution (UHM_RHS) is supported", 7);
  if (!factored) fail("copy_out: nothing solved", 9);
  fetch_x();
  int r = 0;
  for (int i = 0; i < e->get_n_nodes(); ++i) {
    std::pair<int, int> id = nod_disp == UHM_PHYSICS_MULTI ? std::make_pair(nods[2 * i], nods[2 * i + 1])
                                                           : std::make_pair(nods[i], 0);
    Node nd = mesh->find_node(id);
    if (!nd) fail("copy_out: cannot find node in the mesh", 7);
    for (int k = 0; k < nd->get_n_dof(); ++k, ++r) {
      if (r >= m) fail("copy_out: m too small", 7);
      for (int q = 0; q < n && q < mesh->n_rhs; ++q)
        buf[r + (int64_t)q * m] = h_x[(size_t)(nd->get_offset() + k) + (size_t)q * n_global];
    }
  }
}

void Engine::copy_out_leaves(double* buf, int64_t n_values) {
  ensure_plan();
  if (n_values != erhs_total) fail("copy_out_leaves: size mismatch", 7);
  const int nr = mesh->n_rhs;
  if (!factored) fail("copy_out_leaves: nothing solved", 9);
  fetch_x();
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)esrc.size(); ++k) {
    const ElemSource& es = esrc[k];
    double* dst = buf + es.rhs_off;
    for (int q = 0; q < nr; ++q)
      for (int r = 0; r < es.m; ++r) dst[r + (int64_t)q * es.m] = h_x[(size_t)es.gdof[r] + (size_t)q * n_global];
  }
}

// ---------------------------------------------------------------------------
// sources, maps and launch programs
// ---------------------------------------------------------------------------
int64_t Engine::add_items(const std::vector<Item>& it) {
  int64_t off = (int64_t)h_items.size();
  h_items.insert(h_items.end(), it.begin(), it.end());
  return off;
}

void Engine::build_plan(int method) {
  const int nr = mesh->n_rhs;
  // precision per front
  for (auto& f : fronts) {
    int p = PREC_FP64;
    if (mode == 1) {
      p = default_prec;
      if (p == PREC_LEARNED) {
        static const int cls2prec[3] = {PREC_FP64, PREC_FP32, PREC_BF16X3};
        const int c = (int)learned_class.size() > f.slot ? learned_class[f.slot] : 1;
        p = cls2prec[c >= 0 && c < 3 ? c : 1];
      }
      if ((int)front_prec_override.size() > f.slot && front_prec_override[f.slot] >= 0)
        p = front_prec_override[f.slot];
    }
    f.prec = p;
    // tensor-core Schur updates: Cholesky in BF16X3 / BF16X6, LU in BF16X3
    // (its two operands take four packed parts)
    f.tc = f.n >= tune.tc_min_n &&
           (method == UHM_CHOL ? (p == PREC_BF16X3 || p == PREC_BF16X6) : p == PREC_BF16X3);
    // BF16X3 Cholesky fronts: cooperative panels + one deep tensor-core pass over ABR
    f.tcc = f.tc && method == UHM_CHOL && p == PREC_BF16X3 && tune.tc_panel > 0;
  }
  arena64_n = arena32_n = vec_n = piv_n = 0;
  ws_total = 0;
  ws2_rows = 0;
  for (auto& f : fronts) {
    if (!f.tcc) continue;
    // two parts (hi, lo) of every 64-column chunk of the factor block, all n rows
    f.ws2_row0 = ws2_rows;
    ws2_rows += 2 * (int64_t)((f.fs + 63) / 64) * f.n;
  }
  if (tune.tc_panel == CD_PANEL) {
    // the panel rows before their TRSM (same layout), then per front the
    // current panel's Linv parts
    const int64_t r2 = ws2_rows;
    for (auto& f : fronts) {
      if (!f.tcc) continue;
      f.ws2b_row0 = f.ws2_row0 + r2;
    }
    ws2_rows += r2;
    for (auto& f : fronts) {
      if (!f.tcc) continue;
      f.linv_row0 = ws2_rows;
      ws2_rows += CD_LINV_ROWS;
    }
  }
  if (ws2_rows + 512 > ((int64_t)1 << 31) - 1) fail("operand workspace beyond the tensor map's row range", 4);
  for (auto& f : fronts) {
    if (!f.tc || f.tcc) continue;
    const int64_t mmax = f.n - std::min(tune.tc_nbo, f.fs);
    f.ws_off = ws_total;
    f.ws_stride = mmax * tune.tc_nbo;
    ws_total += (method == UHM_CHOL ? 3 : 4) * f.ws_stride;
  }
  h_fronts.assign(fronts.size(), FrontDev{});
  h_srcs.clear();
  h_inv.clear();
  h_fwd.clear();
  h_colptr.clear();
  h_colsrc.clear();
  h_sgi.clear();
  std::vector<std::unordered_map<Node, int>> fpos(fronts.size());
  for (auto& f : fronts) fpos[f.slot] = front_positions(f.e);
  // arena and slab offsets
  for (auto& f : fronts) {
    const int n = f.n;
    const int dt = f.prec == PREC_FP64 ? F64 : F32;
    int64_t& an = dt == F64 ? arena64_n : arena32_n;
    f.off = an;
    an += ((int64_t)n * n + 63) / 64 * 64;
    f.voff = vec_n;
    vec_n += 3 * (int64_t)n * nr;          // z slab (forward), y slab (solution), w slab (chain partial sums)
    f.piv_off = piv_n;
    piv_n += f.fs;
  }
  // large Cholesky fronts: inverses of their 64 x 64 diagonal blocks and one
  // completion flag per block for the flag-driven solves
  dinv64_n = dinv32_n = flags_n = 0;
  {
    const int small_max_f[2] = {tune.small_max_f64, tune.small_max_f32};
    for (auto& f : fronts) {
      const int dt = f.prec == PREC_FP64 ? F64 : F32;
      f.blocked = f.tc || f.n > small_max_f[dt];
      f.flag_off = (int)flags_n;
      f.dinv_off = 0;
      if (!f.blocked || method != UHM_CHOL) continue;
      const int nfb = (f.fs + NB - 1) / NB;
      int64_t& dn = dt == F64 ? dinv64_n : dinv32_n;
      f.dinv_off = dn;
      dn += (int64_t)nfb * NB * NB;
      flags_n += nfb;
    }
  }
  // assembly sources in summation order: the element matrix (copy_in), then
  // the children in child order (op_merge, UHM/src/operation/element.cxx:150-162)
  for (auto& f : fronts) {
    const int n = f.n;
    f.src0 = (int)h_srcs.size();
    std::vector<std::vector<int32_t>> invs;
    const int ei = esrc_of_slot[f.slot];
    if (ei >= 0 && esrc[ei].has_lhs) {
      const ElemSource& es = esrc[ei];
      SrcDev sd{};
      sd.off = es.mat_off;
      sd.ld = es.m;
      sd.dtype = F64;
      sd.is_child = 0;
      sd.slot = ei;
      sd.m = es.m;
      sd.fwd_off = (int64_t)h_fwd.size();
      for (int r = 0; r < es.m; ++r) h_fwd.push_back(es.pos[r]);
      h_srcs.push_back(sd);
      std::vector<int32_t> inv(n, -1);
      for (int r = 0; r < es.m; ++r) inv[es.pos[r]] = r;
      invs.push_back(std::move(inv));
    }
    for (int cs : f.children) {
      const HostFront& c = fronts[cs];
      SrcDev sd{};
      sd.off = c.off + c.fs + (int64_t)c.fs * c.n;
      sd.ld = c.n;
      sd.dtype = c.prec == PREC_FP64 ? F64 : F32;
      sd.is_child = 1;
      sd.slot = cs;
      sd.m = c.ss;
      sd.fwd_off = (int64_t)h_fwd.size();
      std::vector<int32_t> inv(n, -1);
      int r = 0;
      for (auto& pr : c.e->schur) {
        auto it = fpos[f.slot].find(pr.first);
        if (it == fpos[f.slot].end()) fail("child schur node missing in parent", 6);
        for (int k = 0; k < pr.first->get_n_dof(); ++k, ++r) {
          inv[it->second + k] = r;
          h_fwd.push_back(it->second + k);
        }
      }
      if (r != c.ss) fail("child schur rows do not match its schur size", 6);
      h_srcs.push_back(sd);
      invs.push_back(std::move(inv));
    }
    f.nsrc = (int)invs.size();
    f.inv_off = (int64_t)h_inv.size();
    for (auto& v : invs) h_inv.insert(h_inv.end(), v.begin(), v.end());
    f.colptr_off = (int64_t)h_colptr.size();
    for (int J = 0; J < n; ++J) {
      h_colptr.push_back((int64_t)h_colsrc.size());
      for (int s2 = 0; s2 < (int)invs.size(); ++s2)
        if (invs[s2][J] >= 0) h_colsrc.push_back(make_int2(s2, invs[s2][J]));
    }
    h_colptr.push_back((int64_t)h_colsrc.size());
    f.sgi_off = (int64_t)h_sgi.size();
    for (auto& pr : f.e->schur)
      for (int k = 0; k < pr.first->get_n_dof(); ++k) h_sgi.push_back(pr.first->get_offset() + k);
  }
  for (auto& f : fronts) {
    FrontDev& d = h_fronts[f.slot];
    d.off = f.off;
    d.voff = f.voff;
    d.inv_off = f.inv_off;
    d.colptr_off = f.colptr_off;
    d.sgi_off = f.sgi_off;
    d.piv_off = f.piv_off;
    d.n = f.n;
    d.fs = f.fs;
    d.ss = f.ss;
    d.dtype = f.prec == PREC_FP64 ? F64 : F32;
    d.g0 = f.g0;
    d.src0 = f.src0;
    d.nsrc = f.nsrc;
    d.status_slot = f.slot;
    d.flag_off = f.flag_off;
    d.dinv_off = f.dinv_off;
  }
  // element residual tables (elements with a matrix, in leaf order)
  h_emat_off.clear();
  h_elem_m.clear();
  h_emap_off.clear();
  h_emap.clear();
  h_y_off.clear();
  y_total = 0;
  for (auto& es : esrc) {
    h_emat_off.push_back(es.mat_off);
    h_elem_m.push_back(es.m);
    h_emap_off.push_back((int64_t)h_emap.size());
    if ((int)es.gdof.size() == es.m) h_emap.insert(h_emap.end(), es.gdof.begin(), es.gdof.end());
    else h_emap.insert(h_emap.end(), es.m, 0);
    h_y_off.push_back(es.rhs_off);
  }
  y_total = erhs_total;
}

// Every tile as two half tiles of 128 columns, halves wholly above the
// diagonal left out: the next diagonal block's update is on the critical
// path of the panel chain and has two tiles only, so half the operand
// traffic per CTA (and three CTAs instead of two) shortens it.
static void split_halves(std::vector<uhm_gpu::Item>& tt) {
  std::vector<uhm_gpu::Item> out;
  for (const uhm_gpu::Item& t : tt)
    for (unsigned h = 1; h <= 2; ++h) {
      const int cb = t.b + (h == 2 ? 128 : 0);
      if (cb > t.a + 127) continue;
      uhm_gpu::Item x = t;
      x.c = (int)((unsigned)x.c | (h << 30));
      out.push_back(x);
    }
  tt.swap(out);
}

void Engine::build_programs(int method) {
  const bool chol = method == UHM_CHOL;
  const int nr = mesh->n_rhs;
  if (!n_sm) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    n_sm = std::max(1, n_sm);
  }
  h_items.clear();
  fac_ops.clear();
  fwd_ops.clear();
  bwd_ops.clear();
  int64_t pf = 0;   // tickets and flags of the cooperative panel launches
  int64_t hand_slots = 0;   // fronts of the largest diagonal-block launch
  int diag_seq = 0;         // diagonal-block launches so far (their tags)
  auto push = [&](std::vector<Op>& ops, int kind, int dtype, int nb, int param, const std::vector<Item>& it,
                  double flops = 0, double bytes = 0) {
    if (it.empty()) return;
    Op op{kind, dtype, nb, param, add_items(it), (int)it.size()};
    op.flops = flops;
    op.bytes = bytes;
    ops.push_back(op);
  };
  // The Schur pass of the tensor-core Cholesky fronts of a level, ABR -=
  // ABL ABL^T with K = fs: 128 x 256 tiles of the lower triangle, launched in
  // clusters of two whose CTAs take the two row tiles of one column pair (a
  // filler where a column has an odd count) and share the column's B
  // operand; the last partial round of pairs is spread over half tiles.
  auto push_schur = [&](std::vector<Op>& ops, const std::vector<int>& tccf) {
    const int TM = TCC_TILE_M, TN = TCC_TILE_N;
    std::vector<Item> tt;
    double ft = 0, bt = 0;
    for (int sl : tccf) {
      const HostFront& f = fronts[sl];
      if (f.ss <= 0) continue;
      const int nch = (f.fs + 63) / 64;
      for (int c0 = f.fs; c0 < f.n; c0 += TN) {
        std::vector<int> rows;
        for (int r0 = f.fs; r0 < f.n; r0 += TM)
          if (c0 <= r0 + TM - 1) rows.push_back(r0);
        for (size_t k = 0; k < rows.size(); k += 2) {
          const Item a{sl, rows[k], c0, 0 | (nch << 16)};
          tt.push_back(a);
          if (k + 1 < rows.size()) {
            tt.push_back(Item{sl, rows[k + 1], c0, a.c});
          } else {
            Item d = a;
            d.c = (int)((unsigned)d.c | (1u << 29));
            tt.push_back(d);
          }
        }
      }
      ft += get_flop_syrk(0, f.fs, f.ss);
      bt += 8.0 * 0.5 * (double)f.ss * (f.ss + 1) + 2.0 * 2.0 * f.ss * 64.0 * nch;
    }
    if (tt.empty()) return;
    // the last partial round of pairs (one pair per cluster of two SMs) as half-tile pairs
    const int nclu = std::max(1, n_sm / 2), npair = (int)tt.size() / 2, rem = npair % nclu;
    if (npair >= nclu && rem > 0 && 2 * rem <= nclu) {
      std::vector<Item> out(tt.begin(), tt.end() - 2 * rem);
      for (int k = npair - rem; k < npair; ++k)
        for (unsigned h = 1; h <= 2; ++h)
          for (int m = 0; m < 2; ++m) {
            Item x = tt[2 * k + m];
            x.c = (int)((unsigned)x.c | (h << 30));
            out.push_back(x);
          }
      tt.swap(out);
    }
    Op op{OP_TC_CHOL_SCHUR, F32, 0, 0, add_items(tt), (int)tt.size()};
    op.flops = ft;
    op.bytes = bt;
    op.aux = 1;             // paired launch
    ops.push_back(op);
  };
  // one Cholesky step's diagonal block + panel TRSM: fused (every CTA of the
  // TRSM factors the block, the first writes its inverse) or two launches
  auto push_potrf_trsm = [&](int dt, const std::vector<Item>& p_items, const std::vector<Item>& t_items,
                             double fp, double ft) {
    // every fused CTA repeats the latency-bound diagonal factorisation: fuse
    // only while the launch fits fuse_potrf_trsm waves of one CTA per SM
    const size_t n_fused = t_items.size() + p_items.size();
    if (!tune.fuse_potrf_trsm || n_fused > (size_t)tune.fuse_potrf_trsm * n_sm) {
      push(fac_ops, OP_POTRF, dt, NB, 0, p_items, fp);
      push(fac_ops, OP_TRSM, dt, NB, 0, t_items, ft);
      return;
    }
    // consecutive row blocks of a front grouped so that the launch is one wave
    const int per_cta = std::max<int>(1, (int)((t_items.size() + n_sm - 1) / n_sm));
    std::vector<Item> fi;
    for (const Item& d : p_items) {
      std::vector<int> rows;
      for (const Item& t : t_items)
        if (t.front == d.front) rows.push_back(t.b);
      if (rows.empty()) {
        fi.push_back(Item{d.front, d.a, fronts[d.front].n, 1});
        continue;
      }
      for (size_t g0 = 0; g0 < rows.size(); g0 += per_cta) {
        const int cnt = (int)std::min<size_t>(per_cta, rows.size() - g0);
        fi.push_back(Item{d.front, d.a, rows[g0], (g0 == 0 ? 1 : 0) | (cnt << 1)});
      }
    }
    push(fac_ops, OP_POTRF_TRSM, dt, NB, 0, fi, fp + ft);
  };
  // one LU step's 64-column panel: tall panels (many rows below the
  // diagonal) on many CTAs at once (panel-only row swaps, then k_laswp for
  // the other columns), the rest one CTA per front.  nbo > 0 (tensor-core
  // fronts): rows are swapped only in columns below the outer panel's
  // trailing block, whose swaps come after the outer panel
  auto push_lu_panel = [&](int dt, const std::vector<Item>& p_items, double fp, int nbo) {
    const int piv = method == UHM_LU_PIV ? 1 : 0;
    const int rcap = dt == F64 ? GC_RMAX_F64 : GC_RMAX_F32;
    auto col_end = [&](const Item& it) {
      if (nbo <= 0) return 0;
      return std::min((it.a / nbo) * nbo + nbo, fronts[it.front].fs);
    };
    std::vector<Item> one, tall;
    for (const Item& it : p_items) {
      if (fronts[it.front].n - it.a >= tune.gc_min_rows) tall.push_back(it);
      else one.push_back(Item{it.front, it.a, col_end(it), 0});
    }
    push(fac_ops, OP_GETRF, dt, NB, piv, one, tall.empty() ? fp : 0.0);
    size_t i0 = 0;
    while (i0 < tall.size()) {
      // a group whose minimum CTA counts fit one cooperative launch
      size_t i1 = i0;
      int need = 0;
      double rows_sum = 0;
      while (i1 < tall.size()) {
        const int rows = fronts[tall[i1].front].n - tall[i1].a;
        const int mn = (rows + rcap - 1) / rcap;
        if (i1 > i0 && need + mn > n_sm) break;
        need += mn;
        rows_sum += rows;
        ++i1;
      }
      std::vector<Item> g;
      int b = 0, rmax = 1;
      const int spare = std::max(0, n_sm - need);
      for (size_t i = i0; i < i1; ++i) {
        const int rows = fronts[tall[i].front].n - tall[i].a;
        int P = (rows + rcap - 1) / rcap + (int)(spare * (rows / rows_sum));
        P = std::max(1, std::min(P, rows));
        g.push_back(Item{tall[i].front, tall[i].a, b, P});
        rmax = std::max(rmax, (rows + P - 1) / P);
        b += P;
      }
      Op op{OP_GETRF_COOP, dt, NB, piv, add_items(g), (int)g.size()};
      op.q0 = b;
      op.aux = rmax;
      if (i0 == 0) op.flops = fp;
      fac_ops.push_back(op);
      if (piv) {
        std::vector<Item> sw;
        for (const Item& it : g) {
          const int ce = col_end(it), lim = ce > 0 ? ce : fronts[it.front].n;
          for (int c0 = 0; c0 < lim; c0 += 256) sw.push_back(Item{it.front, it.a, c0, ce});
        }
        push(fac_ops, OP_LASWP, dt, NB, 0, sw);
      }
      i0 = i1;
    }
  };
  const int small_max[2] = {tune.small_max_f64, tune.small_max_f32};
  for (auto& lv : levels) {
    for (int dt = 0; dt < 2; ++dt) {
      std::vector<int> fl;
      for (int s : lv)
        if (h_fronts[s].dtype == dt && (!fac_mask || (*fac_mask)[s])) fl.push_back(s);
      if (fl.empty()) continue;
      std::vector<int> tcf, tccf;
      for (int s : fl) {
        if (fronts[s].tcc) tccf.push_back(s);
        else if (fronts[s].tc) tcf.push_back(s);
      }
      std::vector<Item> asm_items, small_items;
      std::vector<int> large;
      int max_small = 1;
      std::vector<Item> asm_big;
      int n_big = 0;
      for (int s : fl) {
        const int n = fronts[s].n;
        if (n >= ASM_SCATTER_MIN && n <= ASM_SCATTER_MAX) {
          for (int J = 0; J < n; ++J) asm_big.push_back(Item{s, J, 0, 0});
          n_big = std::max(n_big, n);
        } else {
          for (int J0 = 0; J0 < n; J0 += ASM_TJ) asm_items.push_back(Item{s, J0, 0, 0});
        }
        if (fronts[s].tc) continue;
        if (n <= small_max[dt]) {
          small_items.push_back(Item{s, 0, 0, 0});
          max_small = std::max(max_small, n);
        } else {
          large.push_back(s);
        }
      }
      // algorithmic bytes of the extend-add: read every source block once,
      // write the parent panel once (lower triangle for Cholesky)
      double asm_bytes = 0, small_flops = 0;
      const double esz = dt == F64 ? 8.0 : 4.0;
      for (int s : fl) {
        const HostFront& f = fronts[s];
        const double tri = chol ? 0.5 : 1.0;
        asm_bytes += tri * (double)f.n * f.n * esz;
        for (int cs : f.children) {
          const HostFront& c = fronts[cs];
          asm_bytes += tri * (double)c.ss * c.ss * (c.prec == PREC_FP64 ? 8.0 : 4.0);
        }
        const int ei = esrc_of_slot[s];
        if (ei >= 0) asm_bytes += (double)esrc[ei].m * esrc[ei].m * 8.0;
        if (f.n <= small_max[dt]) {
          double dec, sol;
          unsigned nz;
          double bf;
          f.e->estimate_cost(method, UHM_REAL, nr, dec, sol, nz, bf);
          small_flops += dec;
        }
      }
      push(fac_ops, OP_ASSEMBLE, dt, 0, chol ? 1 : 0, asm_items, 0, asm_items.empty() ? 0.0 : asm_bytes);
      push(fac_ops, OP_ASSEMBLE_SCATTER, dt, n_big, chol ? 1 : 0, asm_big, 0, asm_items.empty() ? asm_bytes : 0.0);
      push(fac_ops, OP_SMALL_FACTOR, dt, 0, max_small, small_items, small_flops);
      int maxfs = 0;
      for (int s : large) maxfs = std::max(maxfs, fronts[s].fs);
      for (int k0 = 0; k0 < maxfs; k0 += NB) {
        std::vector<Item> p_items, t_items, u_items;
        double fp = 0, ft = 0, fu = 0;
        for (int s : large) {
          const HostFront& f = fronts[s];
          if (f.fs <= k0) continue;
          const int kb = std::min(NB, f.fs - k0);
          const int base = k0 + kb;
          const int mrest = f.n - base;
          if (chol) {
            fp += get_flop_chol(0, kb);
            ft += get_flop_trsm_lower(0, kb, mrest);
            fu += get_flop_syrk(0, kb, mrest);
          } else {
            fp += get_flop_lu(0, f.n - k0, kb);
            ft += get_flop_trsm_lower(0, kb, mrest);
            fu += get_flop_gemm(0, mrest, mrest, kb);
          }
          p_items.push_back(Item{s, k0, 0, 0});
          if (chol) {
            for (int r0 = base; r0 < f.n; r0 += TRSM_RB) t_items.push_back(Item{s, k0, r0, 0});
            const int T = (f.n - base + TILE - 1) / TILE;
            for (int ti = 0; ti < T; ++ti)
              for (int tj = 0; tj <= ti; ++tj) u_items.push_back(Item{s, k0, ti, tj});
          } else {
            for (int c0 = base; c0 < f.n; c0 += LUROW_CB) t_items.push_back(Item{s, k0, c0, 0});
            const int T = (f.n - base + TILE - 1) / TILE;
            for (int ti = 0; ti < T; ++ti)
              for (int tj = 0; tj < T; ++tj) u_items.push_back(Item{s, k0, ti, tj});
          }
        }
        if (chol) {
          push_potrf_trsm(dt, p_items, t_items, fp, ft);
          push(fac_ops, OP_SYRK, dt, NB, 0, u_items, fu);
        } else {
          push_lu_panel(dt, p_items, fp, 0);
          push(fac_ops, OP_LUROW, dt, NB, 0, t_items, ft);
          push(fac_ops, OP_GEMM, dt, NB, 0, u_items, fu);
        }
      }
      // tensor-core fronts: outer panels of tc_nbo columns; inside a panel the
      // SIMT kernels factor 64 columns at a time and update only the panel's
      // columns; the trailing block is then updated once per outer panel on
      // the tensor cores (BF16-split operands, FP32 accumulation)
      int maxfs_tc = 0;
      for (int s : tcf) maxfs_tc = std::max(maxfs_tc, fronts[s].fs);
      const int NBO = tune.tc_nbo;
      const int TB = tc_tile();
      for (int K0 = 0; !chol && K0 < maxfs_tc; K0 += NBO) {
        // LU tensor-core fronts, standard blocked LU with an outer panel of
        // NBO columns: inside it the 64-column steps swap rows and update
        // only columns left of the panel's trailing block (first row /
        // column B); then the panel's swaps for the columns right of it, the
        // panel's rows of U there (row solve + rank-64 updates, block by
        // block), and the trailing block C -= L21 U12 on the tensor cores
        for (int k0 = K0; k0 < K0 + NBO && k0 < maxfs_tc; k0 += NB) {
          std::vector<Item> p_items, t_items, u_items;
          double fp = 0, ft = 0, fu = 0;
          for (int s : tcf) {
            const HostFront& f = fronts[s];
            if (f.fs <= k0) continue;
            const int kb = std::min(NB, f.fs - k0);
            const int base = k0 + kb;
            const int B = std::min(K0 + NBO, f.fs);
            p_items.push_back(Item{s, k0, 0, 0});
            fp += get_flop_lu(0, f.n - k0, kb);
            for (int c0 = base; c0 < B; c0 += LUROW_CB) t_items.push_back(Item{s, k0, c0, B});
            ft += get_flop_trsm_lower(0, kb, std::max(0, B - base));
            const int T = (f.n - base + TILE - 1) / TILE;
            for (int ti = 0; ti < T; ++ti)
              for (int tj = 0; tj < T; ++tj)
                if (base + tj * TILE < B) u_items.push_back(Item{s, k0, ti, tj});
            fu += get_flop_gemm(0, f.n - base, std::max(0, B - base), kb);
          }
          push_lu_panel(dt, p_items, fp, NBO);
          push(fac_ops, OP_LUROW, dt, NB, 0, t_items, ft);
          {
            Op op{OP_GEMM, dt, NB, 0, add_items(u_items), (int)u_items.size()};
            op.q0 = NBO;
            op.aux = 1;     // columns < B
            op.flops = fu;
            if (!u_items.empty()) fac_ops.push_back(op);
          }
        }
        // the outer panel's row swaps on the columns >= B
        if (method == UHM_LU_PIV) {
          std::vector<Item> sw;
          for (int s : tcf) {
            const HostFront& f = fronts[s];
            if (f.fs <= K0) continue;
            const int B = std::min(K0 + NBO, f.fs);
            for (int c0 = B; c0 < f.n; c0 += 256) sw.push_back(Item{s, K0, c0, 0});
          }
          push(fac_ops, OP_LASWP, dt, NBO, 0, sw);
        }
        // the outer panel's rows of U right of it, 64-row block by block
        for (int k0 = K0; k0 < K0 + NBO && k0 < maxfs_tc; k0 += NB) {
          std::vector<Item> t_items, u_items;
          double ft = 0, fu = 0;
          for (int s : tcf) {
            const HostFront& f = fronts[s];
            if (f.fs <= k0) continue;
            const int kb = std::min(NB, f.fs - k0);
            const int base = k0 + kb;
            const int B = std::min(K0 + NBO, f.fs);
            for (int c0 = B; c0 < f.n; c0 += LUROW_CB) t_items.push_back(Item{s, k0, c0, 0});
            ft += get_flop_trsm_lower(0, kb, f.n - B);
            const int T = (f.n - base + TILE - 1) / TILE;
            for (int ti = 0; ti < T; ++ti) {
              if (base + ti * TILE >= B) break;
              for (int tj = 0; tj < T; ++tj)
                if (base + (tj + 1) * TILE > B) u_items.push_back(Item{s, k0, ti, tj});
            }
            fu += get_flop_gemm(0, std::max(0, B - base), f.n - B, kb);
          }
          push(fac_ops, OP_LUROW, dt, NB, 0, t_items, ft);
          Op op{OP_GEMM, dt, NB, 0, add_items(u_items), (int)u_items.size()};
          op.q0 = NBO;
          op.aux = 2;       // rows < B, columns >= B
          op.flops = fu;
          if (!u_items.empty()) fac_ops.push_back(op);
        }
        // trailing block on the tensor cores: L21 (parts 0-1) and U12^T (parts 2-3)
        std::vector<Item> pk, tt;
        double ftc = 0, btc = 0;
        for (int s : tcf) {
          const HostFront& f = fronts[s];
          if (f.fs <= K0) continue;
          const int KB = std::min(NBO, f.fs - K0);
          const int m = f.n - (K0 + KB);
          if (m <= 0) continue;
          for (int rb = 0; rb < (m + 63) / 64; ++rb) pk.push_back(Item{s, K0, rb, 0});
          const int T = (m + TB - 1) / TB;
          for (int ti = 0; ti < T; ++ti)
            for (int tj = 0; tj < T; ++tj) tt.push_back(Item{s, K0, ti, tj});
          ftc += get_flop_gemm(0, m, m, KB);
          btc += 8.0 * (double)m * m + 2.0 * 4 * (double)m * KB;
        }
        if (!pk.empty()) {
          Op pa{OP_TC_PACK, dt, NBO, 2, add_items(pk), (int)pk.size()};
          fac_ops.push_back(pa);
          Op pb = pa;
          pb.q0 = 1;        // transposed: U12^T
          pb.aux = 2;       // into parts 2-3
          fac_ops.push_back(pb);
          push(fac_ops, OP_TC_GEMM, dt, NBO, 2, tt, ftc, btc);
        }
      }
      for (int K0 = 0; chol && K0 < maxfs_tc; K0 += NBO) {
        for (int k0 = K0; k0 < K0 + NBO && k0 < maxfs_tc; k0 += NB) {
          std::vector<Item> p_items, t_items, u_items;
          double fp = 0, ft = 0, fu = 0;
          for (int s : tcf) {
            const HostFront& f = fronts[s];
            if (f.fs <= k0) continue;
            const int kb = std::min(NB, f.fs - k0);
            const int base = k0 + kb;
            const int cmax = std::min(K0 + NBO, f.fs);
            p_items.push_back(Item{s, k0, 0, 0});
            fp += get_flop_chol(0, kb);
            for (int r0 = base; r0 < f.n; r0 += TRSM_RB) t_items.push_back(Item{s, k0, r0, 0});
            ft += get_flop_trsm_lower(0, kb, f.n - base);
            const int T = (f.n - base + TILE - 1) / TILE;
            for (int ti = 0; ti < T; ++ti)
              for (int tj = 0; tj <= ti; ++tj)
                if (base + tj * TILE < cmax) u_items.push_back(Item{s, k0, ti, tj});
            const double w = std::max(0, cmax - base), mr = f.n - base;
            fu += 2.0 * kb * (w * mr - 0.5 * w * (w - 1));
          }
          push_potrf_trsm(dt, p_items, t_items, fp, ft);
          push(fac_ops, OP_SYRK, dt, NB, NBO, u_items, fu);
        }
        std::vector<Item> pk, tt;
        double ftc = 0, btc = 0;
        for (int s : tcf) {
          const HostFront& f = fronts[s];
          if (f.fs <= K0) continue;
          const int KB = std::min(NBO, f.fs - K0);
          const int m = f.n - (K0 + KB);
          if (m <= 0) continue;
          for (int rb = 0; rb < (m + 63) / 64; ++rb) pk.push_back(Item{s, K0, rb, 0});
          const int T = (m + TB - 1) / TB;
          for (int ti = 0; ti < T; ++ti)
            for (int tj = 0; tj <= ti; ++tj) tt.push_back(Item{s, K0, ti, tj});
          ftc += get_flop_syrk(0, KB, m);
          // algorithmic bytes: read and write the FP32 lower triangle of the
          // trailing block once, read the packed panel parts once
          const int np = fronts[s].prec == PREC_BF16X6 ? 3 : 2;
          btc += 8.0 * 0.5 * (double)m * (m + 1) + 2.0 * np * (double)m * KB;
        }
        const int parts = fronts[tcf[0]].prec == PREC_BF16X6 ? 3 : 2;
        push(fac_ops, OP_TC_PACK, dt, NBO, parts, pk);
        push(fac_ops, OP_TC_SYRK, dt, NBO, parts, tt, ftc, btc);
      }
      // BF16X3 Cholesky fronts (k_chol_tc.cu): per outer panel of W1 columns
      // one cooperative panel launch (factor, TRSM, in-panel updates, BF16
      // parts) and one tensor-core launch over the factor block's trailing
      // columns; ABR once at the end with K = fs
      if (!tccf.empty() && tune.tc_panel == CD_PANEL) {
        // panels of 256 columns: diagonal block + its inverse (cooperative,
        // nd CTAs per front), BF16 parts of the rows below, X = A Linv^T on
        // the tensor cores (X and its parts written), trailing update.
        // Lookahead: the trailing update first covers the next panel's
        // diagonal block, then the next panel's diagonal kernel runs on the
        // side stream while the rest of the trailing update (on SMs left
        // free for it) and the next panel's packing run on the main stream.
        const int W1 = CD_PANEL;
        const int TM = TCC_TILE_M, TN = TCC_TILE_N;
        int maxfs_c = 0;
        for (int s : tccf) maxfs_c = std::max(maxfs_c, fronts[s].fs);
        const int n_panels = (maxfs_c + W1 - 1) / W1;
        // the diagonal launch of panel p (items and flags)
        auto diag_op = [&](int K0) {
          std::vector<int> act;
          for (int s : tccf)
            if (fronts[s].fs > K0) act.push_back(s);
          const int64_t tick = pf++;
          // tickets front by front: a front's CTAs wait on one another in
          // both directions (the factorisation on smaller, the inverse's
          // column blocks on larger block rows), so the lowest unfinished
          // front's CTAs are all running once four CTAs fit beside the
          // concurrent update (at least min(items, 16) SMs are left to them).
          // Each front hands its blocks over through its own slot of words.
          std::vector<Item> dit;
          double fp = 0;
          for (size_t q = 0; q < act.size(); ++q) {
            const int sl = act[q];
            const int W = std::min(W1, fronts[sl].fs - K0);
            for (int rel = 0; rel < (W + 63) / 64; ++rel) dit.push_back(Item{sl, K0, rel, (int)q});
          }
          for (int sl : act) fp += get_flop_chol(0, std::min(W1, fronts[sl].fs - K0));
          hand_slots = std::max(hand_slots, (int64_t)act.size());
          if (diag_seq >= CD_MAX_SEQ) fail("factor program holds more diagonal-block launches than tags allow", 6);
          Op op{OP_CHOL_DIAG, F32, W1, (int)tick, add_items(dit), (int)dit.size()};
          op.flops = fp;
          op.aux = (int)dit.size();          // CTAs: the SMs a concurrent update leaves free
          op.q0 = diag_seq++;                // the launch's tag
          return op;
        };
        auto ev_op = [&](int kind, int id, int strm) {
          Op op{kind, 0, 0, id, 0, 0};
          op.strm = strm;
          return op;
        };
        const bool la = tune.lookahead != 0;
        Op d0 = diag_op(0);
        fac_ops.push_back(d0);
        for (int p = 0; p < n_panels; ++p) {
          const int K0 = p * W1;
          std::vector<int> act;
          for (int s : tccf)
            if (fronts[s].fs > K0) act.push_back(s);
          std::vector<Item> pit, xit, tdiag, trest;
          double fx = 0, bx = 0, fd = 0, bd = 0, fr = 0, br = 0, bp = 0;
          bool next = false;
          for (int sl : act) {
            const HostFront& f = fronts[sl];
            const int W = std::min(W1, f.fs - K0), nd = (W + 63) / 64;
            const int base = K0 + W;
            for (int r0 = base; r0 < f.n; r0 += 64)
              for (int cc = 0; cc < nd; ++cc) pit.push_back(Item{sl, K0, r0, cc});
            bp += (double)(f.n - base) * W * (4.0 + 4.0);
            for (int r0 = base; r0 < f.n; r0 += TM) xit.push_back(Item{sl, r0, 0, K0});
            fx += get_flop_trsm_lower(0, W, f.n - base);
            bx += (double)(f.n - base) * 64.0 * nd * (4.0 + 4.0 + 4.0);
            if (base < f.fs) {
              next = true;
              const int kc0 = K0 / 64, kc1 = kc0 + nd;
              const int dnext = base + std::min(W1, f.fs - base);   // end of the next diagonal block
              for (int r0 = base; r0 < f.n; r0 += TM)
                for (int c0 = base; c0 < f.fs && c0 <= r0 + TM - 1; c0 += TN) {
                  const Item t{sl, r0, c0, kc0 | (kc1 << 16)};
                  const bool in_next_diag = la && c0 == base && r0 < dnext;
                  const double rows = std::min(TM, f.n - r0), cols = std::min(TN, f.fs - c0);
                  const double fl = 2.0 * W * rows * cols, by = 8.0 * rows * cols + 2.0 * 2.0 * (rows + cols) * 64.0 * nd;
                  if (in_next_diag) { tdiag.push_back(t); fd += fl; bd += by; }
                  else { trest.push_back(t); fr += fl; br += by; }
                }
            }
          }
          push(fac_ops, OP_CHOL_PACK, F32, 0, 0, pit, 0, bp);
          if (p > 0 && la) fac_ops.push_back(ev_op(OP_EV_WAIT, 2 * p, 0));   // diagonal kernel of panel p done
          push(fac_ops, OP_TC_CHOL_TRSM, F32, 0, 0, xit, fx, bx);
          if (next && la) {
            split_halves(tdiag);
            push(fac_ops, OP_TC_CHOL_TRAIL, F32, 0, 0, tdiag, fd, bd);
            fac_ops.push_back(ev_op(OP_EV_RECORD, 2 * p + 1, 0));
            fac_ops.push_back(ev_op(OP_EV_WAIT, 2 * p + 1, 1));
            Op dn = diag_op(K0 + W1);
            dn.strm = 1;
            const int reserve = std::min(dn.aux, 16);
            fac_ops.push_back(dn);
            fac_ops.push_back(ev_op(OP_EV_RECORD, 2 * (p + 1), 1));
            Op tr{OP_TC_CHOL_TRAIL, F32, 0, 0, add_items(trest), (int)trest.size()};
            tr.flops = fr;
            tr.bytes = br;
            tr.q0 = reserve;
            if (!trest.empty()) fac_ops.push_back(tr);
          } else {
            std::vector<Item> tt = tdiag;
            tt.insert(tt.end(), trest.begin(), trest.end());
            push(fac_ops, OP_TC_CHOL_TRAIL, F32, 0, 0, tt, fd + fr, bd + br);
            if (next) fac_ops.push_back(diag_op(K0 + W1));
          }
        }
        push_schur(fac_ops, tccf);
      } else if (!tccf.empty()) {
        const int W1 = tune.tc_panel;
        const int TM = TCC_TILE_M, TN = TCC_TILE_N;
        int maxfs_c = 0;
        for (int s : tccf) maxfs_c = std::max(maxfs_c, fronts[s].fs);
        for (int K0 = 0; K0 < maxfs_c; K0 += W1) {
          std::vector<int> act;
          for (int s : tccf)
            if (fronts[s].fs > K0) act.push_back(s);
          const int64_t tick = pf++;
          std::vector<int64_t> foff(act.size());
          std::vector<int> nrel(act.size());
          int max_rel = 0;
          double fp = 0, fbytes = 0;
          for (size_t a = 0; a < act.size(); ++a) {
            const HostFront& f = fronts[act[a]];
            const int W = std::min(W1, f.fs - K0), nd = (W + 63) / 64;
            foff[a] = pf;
            pf += CP_FLAGS_PER_FRONT;
            nrel[a] = nd + (f.n - K0 - W + 63) / 64;
            max_rel = std::max(max_rel, nrel[a]);
            fp += get_flop_chol(0, W) + get_flop_trsm_lower(0, W, f.n - K0 - W);
            fbytes += 8.0 * (double)(f.n - K0) * W;
          }
          // tickets by distance from the diagonal, then front: every CTA waits
          // only on CTAs with smaller tickets
          std::vector<Item> pit;
          for (int rel = 0; rel < max_rel; ++rel)
            for (size_t a = 0; a < act.size(); ++a)
              if (rel < nrel[a]) pit.push_back(Item{act[a], K0, rel, (int)foff[a]});
          {
            Op op{OP_CHOL_PANEL, F32, W1, (int)tick, add_items(pit), (int)pit.size()};
            op.flops = fp;
            op.bytes = fbytes;
            fac_ops.push_back(op);
          }
          std::vector<Item> tt;
          double ft = 0, bt = 0;
          for (int sl : act) {
            const HostFront& f = fronts[sl];
            const int W = std::min(W1, f.fs - K0), nd = (W + 63) / 64;
            const int base = K0 + W;
            if (base >= f.fs) continue;
            const int kc0 = K0 / 64, kc1 = kc0 + nd;
            for (int r0 = base; r0 < f.n; r0 += TM)
              for (int c0 = base; c0 < f.fs && c0 <= r0 + TM - 1; c0 += TN)
                tt.push_back(Item{sl, r0, c0, kc0 | (kc1 << 16)});
            const double w = f.fs - base, m = f.n - base;
            const double area = w * m - 0.5 * w * (w - 1);
            ft += 2.0 * W * area;
            bt += 8.0 * area + 2.0 * 2.0 * m * 64.0 * nd;
          }
          push(fac_ops, OP_TC_CHOL_TRAIL, F32, 0, 0, tt, ft, bt);
        }
        push_schur(fac_ops, tccf);
      }
    }
  }
  if (pf > 0) {
    // the panel launches' tickets and flags start at zero in every factorisation
    Op op{OP_CLEAR_FLAGS, 0, 0, 0, 0, 0};
    op.q0 = (int)pf;
    fac_ops.insert(fac_ops.begin(), op);
  }
  if (!fac_mask) {
    pflags_n = pf;
    hand_n = hand_slots;
  } else if (pf > pflags_n || hand_slots > hand_n) {
    fail("partial factor program needs more panel flags than allocated", 6);
  }
  if (fac_mask) return;   // a partial factor program (build_partial) needs no solves
  // solve programs
  const int gm = chol ? M_CHOL : (method == UHM_LU_PIV ? M_LU_PIV : M_LU_NOPIV);
  auto solve_small = [&](const HostFront& f, int dt) {
    return f.n <= small_max[dt] && (int64_t)f.n * nr <= 8192;
  };
  // staged small-front solves (Cholesky): the launch's shared memory holds
  // the largest front's factor panel, its right-hand sides and fs doubles;
  // 0 selects the unstaged kernels (LU, or panels too large)
  auto staged_bytes = [&](const std::vector<Item>& sm, int dt) {
    if (!chol) return 0;
    size_t mx = 0;
    for (const Item& it : sm) {
      const HostFront& f = fronts[it.front];
      const size_t b = (size_t)f.n * nr * 8 + (size_t)f.fs * 8 + (size_t)f.n * f.fs * (dt == F64 ? 8 : 4);
      mx = std::max(mx, b);
    }
    return mx <= 96 * 1024 ? (int)((mx + 15) / 16 * 16) : 0;
  };
  constexpr int GATHER_ROWS = 1024;   // rows per CTA of the forward gather (no pivots)
  constexpr int NR_FLAGS_MAX = 16;    // right-hand sides taken by the flag-driven solves
  for (auto& lv : levels) {
    std::vector<Item> g_items;
    for (int s : lv) {
      if (gm == M_LU_PIV) {
        g_items.push_back(Item{s, 0, 0, 0});
      } else {
        // c = 1: the front takes the flag-driven (or chain) solves, whose
        // forward hand-off words the gather empties
        const int hand = chol && nr <= NR_FLAGS_MAX && !solve_small(fronts[s], h_fronts[s].dtype);
        for (int r0 = 0; r0 < fronts[s].n; r0 += GATHER_ROWS) g_items.push_back(Item{s, r0, GATHER_ROWS, hand});
      }
    }
    push(fwd_ops, OP_FWD_GATHER, 0, 0, gm, g_items);
    for (int dt = 0; dt < 2; ++dt) {
      std::vector<Item> sm;
      std::vector<int> large;
      for (int s : lv) {
        if (h_fronts[s].dtype != dt) continue;
        if (solve_small(fronts[s], dt)) sm.push_back(Item{s, 0, 0, 0});
        else large.push_back(s);
      }
      push(fwd_ops, OP_FWD_SMALL, dt, staged_bytes(sm, dt), gm, sm);
      if (chol && nr <= NR_FLAGS_MAX && !large.empty() && dt == F32 && tune.solve_rows == 64 &&
          tune.solve_chain && (int)large.size() <= CH_MAX_CHAINS) {
        // one chain launch for every large front of this level (per group of
        // FLAG_NR right-hand sides): the chains, the helpers of row blocks
        // b > CH_K in ascending b, then the ABL row blocks
        std::vector<Item> ci;
        int maxb = 0;
        for (int s : large) {
          ci.push_back(Item{s, 0, CH_CHAIN, 0});
          maxb = std::max(maxb, (fronts[s].fs + NB - 1) / NB);
        }
        for (int b = CH_K + 1; b < maxb; ++b)
          for (int s : large)
            if (b < (fronts[s].fs + NB - 1) / NB) ci.push_back(Item{s, b, CH_HELPER, 0});
        for (int s : large) {
          const HostFront& f = fronts[s];
          const int nfb = (f.fs + NB - 1) / NB;
          for (int k = 0; k * NB < f.ss; ++k) ci.push_back(Item{s, nfb + k, CH_ABL, 0});
        }
        const int64_t io = add_items(ci);
        for (int q0 = 0; q0 < nr; q0 += FLAG_NR) {
          Op op{OP_FWD_CHAIN, dt, 0, 0, io, (int)ci.size()};
          op.q0 = q0;
          fwd_ops.push_back(op);
        }
        large.clear();
      }
      if (chol && nr <= NR_FLAGS_MAX && !large.empty()) {
        // one flag-driven launch for every large front of this level (per
        // group of FLAG_NR right-hand sides)
        std::vector<Item> fi, ai;
        const int RB = tune.solve_rows;     // rows per CTA: 64 (k_fwd_flags) or 256 (k_fwd_flags4)
        const int per = RB / NB;
        int maxb = 0;
        for (int s : large) maxb = std::max(maxb, ((fronts[s].fs + NB - 1) / NB + per - 1) / per);
        for (int b = 0; b < maxb; ++b)
          for (int s : large)
            if (b < ((fronts[s].fs + NB - 1) / NB + per - 1) / per) fi.push_back(Item{s, b, 0, 0});
        for (int s : large) {
          const HostFront& f = fronts[s];
          const int nfbr = ((f.fs + NB - 1) / NB + per - 1) / per;
          for (int k = 0; k * RB < f.ss; ++k) ai.push_back(Item{s, nfbr + k, 0, 0});
        }
        fi.insert(fi.end(), ai.begin(), ai.end());
        int f0 = 1 << 30, f1 = 0;
        for (int s : large) {
          f0 = std::min(f0, fronts[s].flag_off);
          f1 = std::max(f1, fronts[s].flag_off + (fronts[s].fs + NB - 1) / NB);
        }
        const int64_t io = add_items(fi);
        for (int q0 = 0; q0 < nr; q0 += FLAG_NR) {
          Op op{OP_FWD_FLAGS, dt, f1 - f0, f0, io, (int)fi.size()};
          op.q0 = q0;
          op.aux = RB;
          fwd_ops.push_back(op);
        }
        large.clear();
      }
      int maxfs = 0;
      for (int s : large) maxfs = std::max(maxfs, fronts[s].fs);
      for (int k0 = 0; k0 < maxfs; k0 += NB) {
        std::vector<Item> fv;
        for (int s : large) {
          const HostFront& f = fronts[s];
          if (f.fs <= k0) continue;
          const int kb = std::min(NB, f.fs - k0);
          const int nch = std::max(1, (f.n - k0 - kb + FWD_RB - 1) / FWD_RB);
          for (int ch = 0; ch < nch; ++ch) fv.push_back(Item{s, k0, ch, 0});
        }
        push(fwd_ops, OP_TRSV_F, dt, NB, gm, fv);
      }
    }
  }
  for (int li = (int)levels.size() - 1; li >= 0; --li) {
    auto& lv = levels[li];
    std::vector<Item> p_items;
    for (int s : lv) p_items.push_back(Item{s, 0, 0, 0});
    push(bwd_ops, OP_BWD_PREP, 0, 0, gm, p_items);
    for (int dt = 0; dt < 2; ++dt) {
      std::vector<Item> sm, st;
      std::vector<int> large;
      for (int s : lv) {
        if (h_fronts[s].dtype != dt) continue;
        if (solve_small(fronts[s], dt)) sm.push_back(Item{s, 0, 0, 0});
        else { large.push_back(s); st.push_back(Item{s, 0, 0, 0}); }
      }
      push(bwd_ops, OP_BWD_SMALL, dt, staged_bytes(sm, dt), gm, sm);
      if (chol && nr <= NR_FLAGS_MAX && !large.empty() && dt == F32 && tune.solve_rows == 64 &&
          tune.solve_chain && (int)large.size() <= CH_MAX_CHAINS) {
        // the chains, then the helpers of the column blocks that have rows
        // outside the chain's window (ABL rows, or factor blocks below
        // b + CH_K) in descending b
        std::vector<Item> ci;
        int maxb = 0;
        for (int s : large) {
          ci.push_back(Item{s, 0, CH_CHAIN, 0});
          maxb = std::max(maxb, (fronts[s].fs + NB - 1) / NB);
        }
        for (int b = maxb - 1; b >= 0; --b)
          for (int s : large) {
            const HostFront& f = fronts[s];
            const int nfb = (f.fs + NB - 1) / NB;
            if (b < nfb && (f.ss > 0 || b + CH_K + 1 <= nfb - 1)) ci.push_back(Item{s, b, CH_HELPER, 0});
          }
        const int64_t io = add_items(ci);
        for (int q0 = 0; q0 < nr; q0 += FLAG_NR) {
          Op op{OP_BWD_CHAIN, dt, 0, 0, io, (int)ci.size()};
          op.q0 = q0;
          bwd_ops.push_back(op);
        }
        large.clear();
      }
      if (chol && nr <= NR_FLAGS_MAX && !large.empty()) {
        std::vector<Item> bi;
        const int per = 1;                       // 64-column blocks per CTA
        int maxb = 0;
        for (int s : large) maxb = std::max(maxb, ((fronts[s].fs + NB - 1) / NB + per - 1) / per);
        for (int b = maxb - 1; b >= 0; --b)
          for (int s : large)
            if (b < ((fronts[s].fs + NB - 1) / NB + per - 1) / per) bi.push_back(Item{s, b, 0, 0});
        int f0 = 1 << 30, f1 = 0;
        for (int s : large) {
          f0 = std::min(f0, fronts[s].flag_off);
          f1 = std::max(f1, fronts[s].flag_off + (fronts[s].fs + NB - 1) / NB);
        }
        const int64_t io = add_items(bi);
        const int qstep = per > 1 ? FLAG_NR : (dt == F64 ? FLAG_NR_BWD_F64 : FLAG_NR);
        for (int q0 = 0; q0 < nr; q0 += qstep) {
          Op op{OP_BWD_FLAGS, dt, f1 - f0, f0, io, (int)bi.size()};
          op.q0 = q0;
          op.aux = NB;
          bwd_ops.push_back(op);
        }
        large.clear();
      }
      int maxfs = 0;
      for (int s : large) maxfs = std::max(maxfs, fronts[s].fs);
      int last = maxfs == 0 ? -1 : ((maxfs - 1) / NB) * NB;
      for (int k0 = last; k0 >= 0; k0 -= NB) {
        std::vector<Item> bv;
        for (int s : large) {
          const HostFront& f = fronts[s];
          if (f.fs <= k0) continue;
          const int kb = std::min(NB, f.fs - k0);
          const int nch = (f.n - k0 - kb + BWD_RB - 1) / BWD_RB;
          for (int ch = 0; ch < std::max(1, nch); ++ch) bv.push_back(Item{s, k0, ch, nch});
        }
        push(bwd_ops, OP_TRSV_B, dt, NB, gm, bv);
      }
      push(bwd_ops, OP_BWD_STORE, dt, 0, gm, st);
    }
  }
  for (auto& f : fronts)
    if (!solve_small(f, h_fronts[f.slot].dtype) && nr > 16)
      fail("more than 16 right-hand sides on a large front is not supported", 8);
}

void Engine::alloc_device(int method) {
  if (dev_ok && (emat_device_only || erhs_device_only)) {
    // element data arrived by direct device copies; keep it across the re-plan
    CK(cudaStreamSynchronize(stream));
    if (emat_device_only)
      CK(cudaMemcpy(h_pinned, ctx.emat, sizeof(double) * (size_t)emat_total, cudaMemcpyDeviceToHost));
    if (erhs_device_only)
      CK(cudaMemcpy(h_pinned + emat_total, d_erhs, sizeof(double) * (size_t)erhs_total, cudaMemcpyDeviceToHost));
    emat_device_only = erhs_device_only = false;
  }
  free_device();
  if (!stream) {
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&stream3, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ev_up, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_anorm, cudaEventDisableTiming));
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev_mid));
    CK(cudaEventCreate(&ev1));
  }
  const int nr = mesh->n_rhs;
  ctx.fronts = (FrontDev*)dmalloc(sizeof(FrontDev) * h_fronts.size());
  ctx.srcs = (SrcDev*)dmalloc(sizeof(SrcDev) * std::max<size_t>(1, h_srcs.size()));
  ctx.inv = (int32_t*)dmalloc(sizeof(int32_t) * std::max<size_t>(1, h_inv.size()));
  ctx.fwd = (int32_t*)dmalloc(sizeof(int32_t) * std::max<size_t>(1, h_fwd.size()));
  ctx.colptr = (int64_t*)dmalloc(sizeof(int64_t) * h_colptr.size());
  ctx.colsrc = (int2*)dmalloc(sizeof(int2) * std::max<size_t>(1, h_colsrc.size()));
  ctx.sgi = (int32_t*)dmalloc(sizeof(int32_t) * std::max<size_t>(1, h_sgi.size()));
  ctx.piv = (int32_t*)dmalloc(sizeof(int32_t) * std::max<int64_t>(1, piv_n));
  ctx.a64 = (double*)dmalloc(sizeof(double) * std::max<int64_t>(1, arena64_n));
  ctx.a32 = (float*)dmalloc(sizeof(float) * std::max<int64_t>(1, arena32_n));
  ctx.emat = (double*)dmalloc(sizeof(double) * std::max<int64_t>(1, emat_total));
  ctx.vec = (double*)dmalloc(sizeof(double) * std::max<int64_t>(1, vec_n));
  ctx.status = (int*)dmalloc(sizeof(int) * fronts.size());
  ctx.dinv64 = dinv64_n ? (double*)dmalloc(sizeof(double) * dinv64_n) : nullptr;
  ctx.dinv32 = dinv32_n ? (float*)dmalloc(sizeof(float) * dinv32_n) : nullptr;
  ctx.flags = (int*)dmalloc(sizeof(int) * std::max<int64_t>(1, flags_n));
  d_ticket = (int*)dmalloc(sizeof(int));
  ctx.n_rhs = nr;
  ctx.symmetric = method == UHM_CHOL ? 1 : 0;
  d_items = (Item*)dmalloc(sizeof(Item) * std::max<size_t>(1, h_items.size()));
  d_err = (int*)dmalloc(sizeof(int));
  CK(cudaMemsetAsync(d_err, 0, sizeof(int), stream));
  if (method != UHM_CHOL) {
    d_gc_xbuf = (double*)dmalloc(sizeof(double) * (size_t)std::max(1, n_sm) * (2 * 66 + 2 * 64));
    d_gc_ctr = (unsigned int*)dmalloc(2 * sizeof(unsigned int));
  }
  if (ws2_rows > 0) {
    // 512 spare rows: tiles that run past the last front's rows stay inside the tensor
    const size_t bytes = 128 * (size_t)(ws2_rows + 512);
    d_ws2 = dmalloc(bytes);
    CK(cudaMemsetAsync(d_ws2, 0, bytes, stream));
    if (!tcc_encode(&ws2_map, d_ws2, ws2_rows + 512)) fail("tensor map encoding failed", 4);
    std::vector<int64_t> r0(fronts.size(), 0), rb(fronts.size(), 0), rl(fronts.size(), 0);
    for (auto& f : fronts)
      if (f.tcc) {
        r0[f.slot] = f.ws2_row0;
        rb[f.slot] = f.ws2b_row0;
        rl[f.slot] = f.linv_row0;
      }
    auto up64 = [&](int64_t*& d, const std::vector<int64_t>& h) {
      d = (int64_t*)dmalloc(sizeof(int64_t) * h.size());
      CK(cudaMemcpyAsync(d, h.data(), sizeof(int64_t) * h.size(), cudaMemcpyHostToDevice, stream));
    };
    up64(d_ws2_row0, r0);
    up64(d_ws2b_row0, rb);
    up64(d_linv_row0, rl);
    CK(cudaStreamSynchronize(stream));
  }
  if (pflags_n > 0) d_pflags = (int*)dmalloc(sizeof(int) * (size_t)pflags_n);
  if (hand_n > 0) {
    // zero: no word carries a tag (every tag has its top bit set)
    const size_t hb = sizeof(uint64_t) * (size_t)(CD_HAND_HEAD + hand_n * CD_HAND_WORDS);
    d_hand = (uint64_t*)dmalloc(hb);
    CK(cudaMemsetAsync(d_hand, 0, hb, stream));
  }
  if (ws_total > 0) {
    // one extra row block so tiles that run past the last part stay inside the tensor
    d_ws = dmalloc(sizeof(uint16_t) * (size_t)(ws_total + 256 * tune.tc_nbo));
    CK(cudaMemsetAsync(d_ws, 0, sizeof(uint16_t) * (size_t)(ws_total + 256 * tune.tc_nbo), stream));
    std::vector<int64_t> wo(fronts.size(), 0), wst(fronts.size(), 0);
    for (auto& f : fronts) {
      if (!f.tc) continue;
      wo[f.slot] = f.ws_off;
      wst[f.slot] = f.ws_stride;
    }
    if (!tc_encode_part(&ws_map, d_ws, ws_total / tune.tc_nbo + 256, tune.tc_nbo))
      fail("tensor map encoding failed", 4);
    d_ws_off = (int64_t*)dmalloc(sizeof(int64_t) * wo.size());
    d_ws_stride = (int64_t*)dmalloc(sizeof(int64_t) * wst.size());
    CK(cudaMemcpyAsync(d_ws_off, wo.data(), sizeof(int64_t) * wo.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_ws_stride, wst.data(), sizeof(int64_t) * wst.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
  }
  {
    std::vector<int64_t> so(fronts.size());
    int64_t tot = 0;
    for (auto& f : fronts) {
      so[f.slot] = tot;
      tot += (int64_t)((f.n + BWD_RB - 1) / BWD_RB + 1) * nr * NB;
    }
    d_scratch = (double*)dmalloc(sizeof(double) * std::max<int64_t>(1, tot));
    d_scr_off = (int64_t*)dmalloc(sizeof(int64_t) * so.size());
    d_counters = (int*)dmalloc(sizeof(int) * fronts.size());
    CK(cudaMemcpyAsync(d_scr_off, so.data(), sizeof(int64_t) * so.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(d_counters, 0, sizeof(int) * fronts.size(), stream));
  }
  const size_t gv = sizeof(double) * (size_t)std::max<int64_t>(1, n_global) * nr;
  d_b = (double*)dmalloc(gv);
  d_x = (double*)dmalloc(gv);
  d_r = (double*)dmalloc(gv);
  d_d = (double*)dmalloc(gv);
  d_erhs = (double*)dmalloc(sizeof(double) * std::max<int64_t>(1, erhs_total));
  d_y = (double*)dmalloc(sizeof(double) * std::max<int64_t>(1, y_total));
  d_red = (double*)dmalloc(sizeof(double) * 2560);
  // the selector's scratch, kept with the plan (a per-call cudaMalloc /
  // cudaFree pair would synchronise the device on every new set of matrices)
  d_sel = (float*)dmalloc(sizeof(float) * (4 * esrc.size() + fronts.size() * (uhm_gpu::SEL_F + uhm_gpu::SEL_C) +
                                           uhm_gpu::SEL_NPARAMS + 4));
  {
    // tree of every global dof (roots numbered in slot order)
    std::vector<int> root_of(fronts.size(), -1);
    n_trees = 0;
    for (int s = (int)fronts.size() - 1; s >= 0; --s)
      root_of[s] = fronts[s].parent < 0 ? n_trees++ : root_of[fronts[s].parent];
    if (n_trees > 1) {
      std::vector<int> dt(std::max<int64_t>(1, n_global), 0);
      for (auto& f : fronts)
        for (int k = 0; k < f.fs; ++k) dt[(size_t)f.g0 + k] = root_of[f.slot];
      d_dof_tree = (int*)dmalloc(sizeof(int) * dt.size());
      d_tree_red = (unsigned long long*)dmalloc(sizeof(unsigned long long) * 4 * n_trees);
      CK(cudaMemcpyAsync(d_dof_tree, dt.data(), sizeof(int) * dt.size(), cudaMemcpyHostToDevice, stream));
    }
    n_trees = std::max(n_trees, 1);
  }
  d_emat_off = (int64_t*)dmalloc(sizeof(int64_t) * std::max<size_t>(1, h_emat_off.size()));
  d_elem_m = (int*)dmalloc(sizeof(int) * std::max<size_t>(1, h_elem_m.size()));
  d_emap_off = (int64_t*)dmalloc(sizeof(int64_t) * std::max<size_t>(1, h_emap_off.size()));
  d_emap = (int32_t*)dmalloc(sizeof(int32_t) * std::max<size_t>(1, h_emap.size()));
  d_y_off = (int64_t*)dmalloc(sizeof(int64_t) * std::max<size_t>(1, h_y_off.size()));
  // dof -> (element, row) CSR for the deterministic residual gather
  std::vector<int64_t> cnt(n_global + 1, 0);
  for (size_t k = 0; k < esrc.size(); ++k)
    if ((int)esrc[k].gdof.size() == esrc[k].m)
      for (int32_t g : esrc[k].gdof) cnt[g + 1]++;
  for (int64_t i = 0; i < n_global; ++i) cnt[i + 1] += cnt[i];
  std::vector<int64_t> idx(cnt[n_global]);
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
  for (size_t k = 0; k < esrc.size(); ++k)
    if ((int)esrc[k].gdof.size() == esrc[k].m)
      for (int r = 0; r < esrc[k].m; ++r) {
        const int64_t v = (h_y_off[k] + r) | ((int64_t)esrc[k].m << 40);
        idx[fill[esrc[k].gdof[r]]++] = v;
      }
  std::vector<int2> del(cnt[n_global]);
  {
    std::vector<int64_t> f2(cnt.begin(), cnt.end() - 1);
    for (size_t k = 0; k < esrc.size(); ++k)
      if ((int)esrc[k].gdof.size() == esrc[k].m)
        for (int r = 0; r < esrc[k].m; ++r) del[f2[esrc[k].gdof[r]]++] = make_int2((int)k, r);
  }
  d_dof_el = (int2*)dmalloc(sizeof(int2) * std::max<size_t>(1, del.size()));
  d_dof_ptr = (int64_t*)dmalloc(sizeof(int64_t) * cnt.size());
  d_dof_idx = (int64_t*)dmalloc(sizeof(int64_t) * std::max<size_t>(1, idx.size()));
  auto up = [&](void* d, const void* h, size_t bytes) {
    if (bytes) CK(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, stream));
  };
  up(ctx.fronts, h_fronts.data(), sizeof(FrontDev) * h_fronts.size());
  up(ctx.srcs, h_srcs.data(), sizeof(SrcDev) * h_srcs.size());
  up(ctx.inv, h_inv.data(), sizeof(int32_t) * h_inv.size());
  up(ctx.fwd, h_fwd.data(), sizeof(int32_t) * h_fwd.size());
  up(ctx.colptr, h_colptr.data(), sizeof(int64_t) * h_colptr.size());
  up(ctx.colsrc, h_colsrc.data(), sizeof(int2) * h_colsrc.size());
  up(ctx.sgi, h_sgi.data(), sizeof(int32_t) * h_sgi.size());
  up(d_items, h_items.data(), sizeof(Item) * h_items.size());
  up(d_emat_off, h_emat_off.data(), sizeof(int64_t) * h_emat_off.size());
  up(d_elem_m, h_elem_m.data(), sizeof(int) * h_elem_m.size());
  up(d_emap_off, h_emap_off.data(), sizeof(int64_t) * h_emap_off.size());
  up(d_emap, h_emap.data(), sizeof(int32_t) * h_emap.size());
  up(d_y_off, h_y_off.data(), sizeof(int64_t) * h_y_off.size());
  up(d_dof_ptr, cnt.data(), sizeof(int64_t) * cnt.size());
  up(d_dof_idx, idx.data(), sizeof(int64_t) * idx.size());
  up(d_dof_el, del.data(), sizeof(int2) * del.size());
  CK(cudaStreamSynchronize(stream));
  dev_ok = true;
  method_built = method;
  prec_dirty = false;
  emat_dirty = erhs_dirty = true;
  anorm_valid = false;
}

void Engine::upload_elements() {
  if (emat_dirty) {
    CK(cudaMemcpyAsync(ctx.emat, h_pinned, sizeof(double) * (size_t)emat_total, cudaMemcpyHostToDevice, stream));
    emat_dirty = false;
  }
}

void Engine::assemble_rhs() {
  if (erhs_dirty) {
    CK(cudaMemcpyAsync(d_erhs, h_pinned + emat_total, sizeof(double) * (size_t)erhs_total,
                       cudaMemcpyHostToDevice, stream));
    erhs_dirty = false;
  }
  launch_dof_gather(d_dof_ptr, d_dof_idx, d_erhs, nullptr, n_global, d_b, n_global, mesh->n_rhs, 0, stream);
}

void Engine::clear_graphs() {
  for (auto& g : graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  graphs.clear();
}

// Replays a program as a CUDA graph: the first call runs it eagerly (kernel
// attributes get set), the second captures and instantiates it, later calls
// launch the instantiated graph (one launch for up to thousands of kernels).
void Engine::run_ops(const std::vector<Op>& ops, double* g_in, double* g_out) {
  if (!use_graphs || profiling || ops.empty()) {
    launch_ops(ops, g_in, g_out);
    return;
  }
  GraphEntry* ge = nullptr;
  for (auto& g : graphs)
    if (g.ops == &ops && g.gin == g_in && g.gout == g_out) ge = &g;
  if (!ge) {
    graphs.push_back(GraphEntry{&ops, g_in, g_out, 0, nullptr});
    ge = &graphs.back();
  }
  if (!ge->exec && ge->eager_runs == 0) {
    ge->eager_runs++;
    launch_ops(ops, g_in, g_out);
    return;
  }
  if (!ge->exec) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    const int64_t before = timing.kernel_launches;
    try {
      launch_ops(ops, g_in, g_out);
    } catch (...) {
      // a launcher refused (bad arguments, a launch the device cannot take):
      // close the capture so that the stream stays usable, then report
      cudaGraph_t broken = nullptr;
      cudaStreamEndCapture(stream, &broken);
      if (broken) cudaGraphDestroy(broken);
      cudaGetLastError();
      throw;
    }
    timing.kernel_launches = before;
    CK(cudaStreamEndCapture(stream, &g));
    CK(cudaGraphInstantiate(&ge->exec, g, 0));
    cudaGraphDestroy(g);
  }
  CK(cudaGraphLaunch(ge->exec, stream));
  for (const Op& op : ops) timing.kernel_launches += is_kernel_op(op.kind) ? 1 : 0;
}

void Engine::launch_ops(const std::vector<Op>& ops, double* g_in, double* g_out, const uhm_gpu::Item* base) {
  std::vector<cudaEvent_t> evs;
  if (profiling) {
    evs.resize(2 * ops.size());
    for (auto& e : evs) CK(cudaEventCreate(&e));
  }
  size_t k = 0;
  for (const Op& op : ops) {
    const Item* it = (base ? base : d_items) + op.item_off;
    if (profiling) CK(cudaEventRecord(evs[2 * k], stream));
    // the side stream only when not profiling (profiled launches are serial)
    const cudaStream_t st = (op.strm && !profiling) ? stream2 : stream;
    if (op.kind == OP_EV_RECORD || op.kind == OP_EV_WAIT) {
      if (!profiling) {
        while ((int)evpool.size() <= op.param) {
          cudaEvent_t e;
          CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
          evpool.push_back(e);
        }
        if (op.kind == OP_EV_RECORD) CK(cudaEventRecord(evpool[op.param], st));
        else CK(cudaStreamWaitEvent(st, evpool[op.param], 0));
      }
      if (profiling) CK(cudaEventRecord(evs[2 * k + 1], stream));
      ++k;
      continue;
    }
    switch (op.kind) {
      case OP_ASSEMBLE: launch_assemble(ctx, it, op.n_items, op.dtype, op.param, st); break;
      case OP_ASSEMBLE_SCATTER:
        launch_assemble_scatter(ctx, it, op.n_items, op.dtype, op.param, op.nb, st);
        break;
      case OP_SMALL_FACTOR:
        launch_small_factor(ctx, it, op.n_items, op.dtype,
                            ctx.symmetric ? M_CHOL : (method_built == UHM_LU_PIV ? M_LU_PIV : M_LU_NOPIV),
                            op.param, st);
        break;
      case OP_POTRF: launch_potrf_diag(ctx, it, op.n_items, op.dtype, op.nb, st); break;
      case OP_TRSM: launch_trsm_panel(ctx, it, op.n_items, op.dtype, op.nb, st); break;
      case OP_POTRF_TRSM: launch_potrf_trsm(ctx, it, op.n_items, op.dtype, st); break;
      case OP_SYRK: launch_syrk_update(ctx, it, op.n_items, op.dtype, op.nb, op.param, st); break;
      case OP_FWD_FLAGS:
        if (op.aux == 256)
          launch_fwd_flags4(ctx, it, op.n_items, op.dtype, d_ticket, d_err, op.q0, st);
        else
          launch_fwd_flags(ctx, it, op.n_items, op.dtype, d_ticket, ctx.flags + op.param, op.nb, d_err, op.q0,
                           st);
        break;
      case OP_FWD_CHAIN: launch_fwd_chain(ctx, it, op.n_items, d_ticket, d_err, op.q0, st); break;
      case OP_BWD_CHAIN: launch_bwd_chain(ctx, it, op.n_items, d_ticket, d_err, op.q0, st); break;
      case OP_BWD_FLAGS:
        launch_bwd_flags(ctx, it, op.n_items, op.dtype, d_ticket, ctx.flags + op.param, op.nb, d_err, op.q0,
                           st);
        break;
      case OP_TC_PACK:
        launch_tc_pack(ctx, it, op.n_items, op.nb, op.param, d_ws, d_ws_off, d_ws_stride, op.q0, op.aux, st);
        break;
      case OP_TC_SYRK:
        launch_tc_syrk(ctx, ws_map, d_ws_off, d_ws_stride, it, op.n_items, op.nb, op.param == 3 ? 6 : 3,
                       op.param == 3 ? TC_TERMS_BF16X6 : TC_TERMS_BF16X3, 1, d_err, st);
        break;
      case OP_GETRF: launch_getrf_panel(ctx, it, op.n_items, op.dtype, op.nb, op.param, st); break;
      case OP_GETRF_COOP:
        launch_getrf_coop(ctx, it, op.n_items, op.q0, op.dtype, op.nb, op.param, op.aux, d_gc_xbuf, d_gc_ctr, d_err,
                          st);
        break;
      case OP_LASWP: launch_laswp(ctx, it, op.n_items, op.dtype, op.nb, st); break;
      case OP_LUROW: launch_lu_row_update(ctx, it, op.n_items, op.dtype, op.nb, 0, st); break;
      case OP_GEMM: launch_gemm_update(ctx, it, op.n_items, op.dtype, op.nb, op.q0, op.aux, st); break;
      case OP_TC_GEMM:
        launch_tc_syrk(ctx, ws_map, d_ws_off, d_ws_stride, it, op.n_items, op.nb, 3, TC_TERMS_LU_BF16X3, 0, d_err,
                       st);
        break;
      case OP_CLEAR_FLAGS:
        launch_clear_flags(d_pflags, op.q0, d_hand ? reinterpret_cast<unsigned*>(d_hand) : nullptr, st);
        break;
      case OP_CHOL_PANEL:
        launch_chol_panel(ctx, it, op.n_items, op.nb, d_pflags + op.param, d_pflags, d_err, d_ws2, d_ws2_row0,
                          st);
        break;
      case OP_TC_CHOL_TRAIL:
      case OP_TC_CHOL_SCHUR:
        launch_tc_chol(ctx, ws2_map, d_ws2_row0, it, op.n_items, d_err, st, 0, nullptr, nullptr, nullptr,
                       profiling ? 0 : op.q0, op.kind == OP_TC_CHOL_SCHUR ? op.aux : 0);
        break;
      case OP_CHOL_DIAG:
        launch_chol_diag(ctx, it, op.n_items, d_pflags + op.param, d_hand + CD_HAND_HEAD,
                         reinterpret_cast<const unsigned*>(d_hand), op.q0, d_err, d_ws2, d_linv_row0, st);
        break;
      case OP_CHOL_PACK: launch_chol_pack(ctx, it, op.n_items, d_ws2, d_ws2b_row0, st); break;
      case OP_TC_CHOL_TRSM:
        launch_tc_chol(ctx, ws2_map, d_ws2_row0, it, op.n_items, d_err, st, 1, d_ws2b_row0, d_linv_row0, d_ws2,
                       profiling ? 0 : op.q0);
        break;
      case OP_FWD_GATHER: launch_fwd_gather(ctx, it, op.n_items, g_in, n_global, op.param, st); break;
      case OP_FWD_SMALL: launch_fwd_small(ctx, it, op.n_items, op.dtype, op.param, op.nb, st); break;
      case OP_TRSV_F: launch_fwd_step(ctx, it, op.n_items, op.dtype, op.param, st); break;
      case OP_BWD_PREP: launch_bwd_prepare(ctx, it, op.n_items, 0, op.param, g_out, n_global, st); break;
      case OP_BWD_SMALL:
        launch_bwd_small(ctx, it, op.n_items, op.dtype, op.param, g_out, n_global, op.nb, st);
        break;
      case OP_TRSV_B:
        launch_bwd_step(ctx, it, op.n_items, op.dtype, op.param, d_scratch, d_scr_off, d_counters, st);
        break;
      case OP_BWD_STORE: launch_bwd_store(ctx, it, op.n_items, g_out, n_global, st); break;
    }
    if (profiling) CK(cudaEventRecord(evs[2 * k + 1], stream));
    ++k;
    if (is_kernel_op(op.kind)) timing.kernel_launches++;
  }
  CK(cudaGetLastError());
  if (profiling) {
    CK(cudaStreamSynchronize(stream));
    for (size_t i = 0; i < ops.size(); ++i) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, evs[2 * i], evs[2 * i + 1]));
      if (ops[i].kind < 0 || ops[i].kind >= N_OP_KINDS) continue;
      op_log.push_back(OpRecord{ops[i].kind, ops[i].n_items, ms});
      profile.ms[ops[i].kind] += ms;
      profile.flops[ops[i].kind] += ops[i].flops;
      profile.bytes[ops[i].kind] += ops[i].bytes;
      profile.launches[ops[i].kind] += 1;
    }
    for (auto& e : evs) cudaEventDestroy(e);
  }
}

// The fronts' status words and the wait error word, copied back behind the
// work just enqueued (one stream sync for both instead of two round trips)
void Engine::enqueue_status_words() {
  const size_t need = fronts.size() + 1;
  if (h_words_n < need) {
    if (h_words) cudaFreeHost(h_words);
    h_words = nullptr;
    h_words_n = 0;
    CK(cudaMallocHost((void**)&h_words, sizeof(int) * need));
    h_words_n = need;
  }
  CK(cudaMemcpyAsync(h_words, ctx.status, sizeof(int) * fronts.size(), cudaMemcpyDeviceToHost, stream));
  CK(cudaMemcpyAsync(h_words + fronts.size(), d_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
}

void Engine::read_status_words(const char* where) {
  for (size_t i = 0; i < fronts.size(); ++i)
    if (h_words[i]) {
      const int st = h_words[i];
      const char* what = st == ST_NOT_SPD ? "front is not positive definite"
                         : st == ST_ZERO_PIVOT ? "zero pivot"
                         : st == ST_WAIT ? "a bounded wait inside a kernel gave up" : "NaN in front";
      status = 10 + st;
      last_error = std::string(where) + ": " + what + " (element " + std::to_string(fronts[i].e->get_id()) + ")";
      break;
    }
  if (h_words[fronts.size()]) {
    CK(cudaMemset(d_err, 0, sizeof(int)));
    const int at = uhm_gpu::solve_wait_where();
    fail(std::string(where) + ": a device wait gave up (bounded wait expired" +
             (at > 0 ? ", solve hand-off " + std::to_string(at) : std::string()) + ")", 14);
  }
}

void Engine::factor(int method) {
  ensure_plan();
  for (auto& es : esrc)
    if (!es.has_lhs) fail("factor: an element matrix has not been copied in", 7);
  if (mode == 1 && default_prec == PREC_LEARNED && !learned_valid) apply_selector(method);
  if (!dev_ok || method_built != method || prec_dirty) {
    build_plan(method);
    build_programs(method);
    alloc_device(method);
  }
  status = 0;
  last_error.clear();
  timing = Timing{};
  CK(cudaEventRecord(ev0, stream));
  upload_elements();
  CK(cudaMemsetAsync(ctx.status, 0, sizeof(int) * fronts.size(), stream));
  CK(cudaEventRecord(ev_mid, stream));
  float ms = 0;
  // factor reuse (operation/element.cxx:202-205 skips the merge and the
  // factorisation of a reusable element): keep a front when its element is
  // flagged, its factor from the last factorisation of this plan is held,
  // its element matrix was not copied in since and all its children are kept
  std::vector<char> act(fronts.size(), 1);
  int n_keep = 0;
  if (front_kept.size() == fronts.size() && leaf_changed.size() == esrc.size())
    for (auto& lv : levels)   // leaves first: children before parents
      for (int s : lv) {
        const HostFront& f = fronts[s];
        bool keep = front_kept[s] && f.e->is_matrix_reusable();
        const int ei = esrc_of_slot[s];
        if (ei >= 0 && leaf_changed[ei]) keep = false;
        for (int c : f.children) keep = keep && !act[c];
        act[s] = keep ? 0 : 1;
        n_keep += keep ? 1 : 0;
      }
  if (n_keep > 0 && act != part_mask) build_partial(method, act);
  n_refactored = (int)fronts.size() - n_keep;
  // until this factorisation succeeds, no front holds a trustworthy factor
  factored = false;
  solved = false;
  front_kept.clear();
  if (!anorm_valid) enqueue_anorm();
  // the diagonal kernels' hand-off words carry 21 bits of the factorisation
  // count in their tag: cleared every 2^20 factorisations (and before the
  // first), no word is left to meet its tag again after the count wraps
  if (d_hand && (hand_factorisations++ & ((int64_t(1) << 20) - 1)) == 0)
    CK(cudaMemsetAsync(d_hand + CD_HAND_HEAD, 0, sizeof(uint64_t) * (size_t)(hand_n * CD_HAND_WORDS), stream));
  if (n_keep > 0) launch_ops(fac_ops_part, nullptr, nullptr, d_items_part);
  else run_ops(fac_ops, nullptr, nullptr);
  CK(cudaEventRecord(ev1, stream));
  enqueue_status_words();
  CK(cudaStreamSynchronize(stream));
  CK(cudaEventElapsedTime(&ms, ev0, ev_mid));
  timing.upload_ms = ms;
  CK(cudaEventElapsedTime(&ms, ev_mid, ev1));
  timing.factor_ms = ms;
  read_status_words("factor");
  if (status && mode == 1) {
    // a low-precision front broke down: escalate the failed fronts to FP64
    std::vector<int> st(fronts.size());
    CK(cudaMemcpy(st.data(), ctx.status, sizeof(int) * st.size(), cudaMemcpyDeviceToHost));
    bool any = false;
    if (front_prec_override.size() != fronts.size()) front_prec_override.assign(fronts.size(), -1);
    for (size_t i = 0; i < st.size(); ++i)
      if (st[i] && fronts[i].prec != PREC_FP64) { front_prec_override[i] = PREC_FP64; any = true; }
    if (any) {
      const double first_ms = timing.factor_ms;
      prec_dirty = true;
      factor(method);
      timing.factor_ms += first_ms;
      return;
    }
  }
  factored = true;
  factored_method = method;
  h_x_valid = false;
  // every front's factor now belongs to the current element matrices
  front_kept.assign(fronts.size(), status == 0 ? 1 : 0);
  if (status == 0) leaf_changed.assign(esrc.size(), 0);
}

// The factor program over the fronts marked in act only: build_programs with
// a mask, its items in their own device array; the full programs (and their
// CUDA graphs) are left as they are.
void Engine::build_partial(int method, const std::vector<char>& act) {
  std::vector<uhm_gpu::Item> items_full = std::move(h_items);
  std::vector<Op> fac_full = std::move(fac_ops), fwd_full = std::move(fwd_ops), bwd_full = std::move(bwd_ops);
  auto restore = [&]() {
    fac_mask = nullptr;
    h_items = std::move(items_full);
    fac_ops = std::move(fac_full);
    fwd_ops = std::move(fwd_full);
    bwd_ops = std::move(bwd_full);
  };
  h_items.clear();
  fac_ops.clear();
  fwd_ops.clear();
  bwd_ops.clear();
  fac_mask = &act;
  std::vector<uhm_gpu::Item> items_part;
  try {
    build_programs(method);
  } catch (...) {
    restore();
    throw;
  }
  fac_ops_part = std::move(fac_ops);
  items_part = std::move(h_items);
  restore();
  part_mask.clear();
  if (items_part.size() > d_items_part_cap) {
    d_items_part = (uhm_gpu::Item*)dmalloc(sizeof(uhm_gpu::Item) * items_part.size());
    d_items_part_cap = items_part.size();
  }
  if (!items_part.empty())
    CK(cudaMemcpyAsync(d_items_part, items_part.data(), sizeof(uhm_gpu::Item) * items_part.size(),
                       cudaMemcpyHostToDevice, stream));
  CK(cudaStreamSynchronize(stream));
  part_mask = act;
}

void Engine::solve_into(int method, double* rhs, double* out, int phase) {
  (void)method;
  if (phase & 1) run_ops(fwd_ops, rhs, out);
  if (phase & 2) run_ops(bwd_ops, rhs, out);
}

// The error word of the bounded device waits: read, and cleared when set so
// that the next call starts clean (the device itself stays usable).
void Engine::check_device_error(const char* where) {
  int derr = 0;
  CK(cudaMemcpy(&derr, d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (derr) {
    CK(cudaMemset(d_err, 0, sizeof(int)));
    const int at = uhm_gpu::solve_wait_where();
    fail(std::string(where) + ": a device wait gave up (bounded wait expired" +
             (at > 0 ? ", solve hand-off " + std::to_string(at) : std::string()) + ")", 14);
  }
}

void Engine::solve(int method, int phase) {
  if (!factored) fail("solve: the mesh has not been factorised", 9);
  if (method != factored_method) fail("solve: method differs from the factorisation", 9);
  float ms = 0;
  clear_solve_status();
  CK(cudaEventRecord(ev0, stream));
  if (phase & 1) assemble_rhs();
  solve_into(method, d_b, d_x, phase);
  h_x_valid = false;
  solved = false;
  if (mode == 1 && phase == 3) {
    // the refinement's first read-back carries this solve's wait error word
    // and time (ev0 .. ev_mid)
    CK(cudaEventRecord(ev_mid, stream));
    refine(method);
    return;
  }
  CK(cudaEventRecord(ev1, stream));
  CK(cudaEventSynchronize(ev1));
  CK(cudaEventElapsedTime(&ms, ev0, ev1));
  timing.solve_ms = ms;
  check_device_error("solve");
  solved = phase == 3;
  // plain path: a NaN or infinity in the right-hand sides (or factors)
  // reaches the solution; report it rather than return it silently
  if (phase & 2) {
    launch_absmax(d_x, n_global * mesh->n_rhs, d_red + 2048, stream);
    const double xn = read_scalar(d_red + 2048);
    if (!std::isfinite(xn)) fail("solve: the solution is not finite (NaN or infinity in the right-hand side or the factors)", 13);
  }
}

// FP64 iterative refinement on the unassembled element matrices:
//   r = b - A x (FP64, element by element), d = M^{-1} r with the
//   low-precision factors, x += d, until the backward error
//   ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= ir_tol.
// A miss after ir_max corrections refactors and solves in plain FP64.
void Engine::refine(int method) {
  float ms = 0;
  const int64_t nv = n_global * mesh->n_rhs;
  if (!h_red) CK(cudaMallocHost((void**)&h_red, sizeof(double) * 8));
  const bool forest = n_trees > 1;
  if (!anorm_valid) enqueue_anorm();
  sync_anorm();
  // ||b||_inf and, on the first pass, ||A||_inf and the solve's wait error
  // word travel with the first residual norms: one stream sync per pass
  launch_absmax(d_b, nv, d_red + 1024, stream);
  double an = anorm_inf, bn = 0.0;
  double berr = 1.0;
  int it = 0;
  if (forest) {
    tree_max_async(d_b, nv, n_global, 2);
    tree_bnorm = read_tree_slot(2);
  }
  for (;; ++it) {
    compute_residual(d_x, d_r);
    if (!forest) {
      launch_absmax(d_r, nv, d_red, stream);
      launch_absmax(d_x, nv, d_red + 512, stream);
      CK(cudaMemcpyAsync(&h_red[0], d_red, sizeof(double), cudaMemcpyDeviceToHost, stream));
      CK(cudaMemcpyAsync(&h_red[1], d_red + 512, sizeof(double), cudaMemcpyDeviceToHost, stream));
    }
    if (it == 0) {
      CK(cudaMemcpyAsync(&h_red[2], d_red + 1024, sizeof(double), cudaMemcpyDeviceToHost, stream));
      CK(cudaMemcpyAsync(&h_red[3], d_red + 1536, sizeof(double), cudaMemcpyDeviceToHost, stream));
      CK(cudaMemcpyAsync(&h_red[4], d_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    }
    CK(cudaStreamSynchronize(stream));
    if (it == 0) {
      int derr = 0;
      std::memcpy(&derr, &h_red[4], sizeof(int));
      if (derr) {
        CK(cudaMemset(d_err, 0, sizeof(int)));
        const int at = uhm_gpu::solve_wait_where();
        fail(std::string("solve: a device wait gave up (bounded wait expired") +
                 (at > 0 ? ", solve hand-off " + std::to_string(at) : std::string()) + ")", 14);
      }
      CK(cudaEventElapsedTime(&ms, ev0, ev_mid));
      timing.solve_ms = ms;
      solved = true;
      bn = h_red[2];
      if (!(an >= 0)) an = anorm_inf = h_red[3];
      if (!std::isfinite(bn) || !std::isfinite(an)) {
        // refinement cannot repair a bad input, and an FP64 redo would not either
        timing.berr = timing.berr_first = NAN;
        fail(std::string("refine: the ") + (std::isfinite(bn) ? "operator" : "right-hand side") +
                 " is not finite (NaN or infinity)", 13);
      }
    }
    if (forest) {
      tree_max_async(d_r, nv, n_global, 0);
      tree_max_async(d_x, nv, n_global, 1);
      const std::vector<double> rn = read_tree_slot(0);
      berr = forest_berr(rn, read_tree_slot(1));
    } else {
      berr = h_red[0] / (an * h_red[1] + bn);
    }
    if (it == 0) timing.berr_first = berr;
    if (berr <= ir_tol || it >= ir_max || !(berr == berr)) break;
    solve_into(method, d_r, d_d, 3);
    launch_axpy(d_x, d_d, nv, 1.0, stream);
  }
  CK(cudaEventRecord(ev1, stream));
  CK(cudaEventSynchronize(ev1));
  CK(cudaEventElapsedTime(&ms, ev_mid, ev1));
  timing.refine_ms = ms;
  timing.ir_iters = it;
  timing.berr = berr;
  if (!(berr <= ir_tol)) {
    // tolerance missed: redo the whole solve in plain FP64
    const Timing keep = timing;
    const int saved = mode;
    mode = 0;
    prec_dirty = true;
    try {
      factor(method);
      solve(method, 3);
    } catch (...) {
      mode = saved;
      prec_dirty = true;
      throw;
    }
    mode = saved;
    prec_dirty = true;
    Timing t2 = timing;
    timing = keep;
    timing.factor_ms += t2.factor_ms;
    timing.solve_ms += t2.solve_ms;
    timing.berr = backward_error();    // of the FP64 solution now in x
    status = 20;
    last_error = "refinement missed its tolerance; solution recomputed in FP64";
  }
}

void Engine::compute_residual(const double* x, double* r) {
  sync_anorm();
  launch_elem_gemv(ctx.emat, d_emat_off, d_elem_m, d_emap_off, d_emap, x, n_global, d_y, d_y_off,
                   (int)esrc.size(), mesh->n_rhs, stream);
  launch_dof_gather(d_dof_ptr, d_dof_idx, d_y, d_b, n_global, r, n_global, mesh->n_rhs, 1, stream);
}

double Engine::residual_norm1() {
  if (!factored) fail("residual: nothing solved", 9);
  compute_residual(d_x, d_r);
  std::vector<double> r((size_t)n_global * mesh->n_rhs);
  CK(cudaMemcpyAsync(r.data(), d_r, sizeof(double) * r.size(), cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  double best = 0;
  for (int q = 0; q < mesh->n_rhs; ++q) {
    double s = 0;
    for (int64_t i = 0; i < n_global; ++i) s += std::fabs(r[i + q * n_global]);
    best = std::max(best, s);
  }
  return best;
}

// ||A||_inf of the assembled operator sum_e P_e^T A_e P_e, exact, on the device
// (k_anorm_partial + deterministic per-dof gather); result in d_red[1536]
void Engine::enqueue_anorm() {
  // on its own stream, after the element matrices' upload on the main
  // stream: it overlaps the factorisation, and the first use joins it
  sync_anorm();
  CK(cudaEventRecord(ev_up, stream));
  CK(cudaStreamWaitEvent(stream3, ev_up, 0));
  launch_anorm_partial(ctx.emat, d_emat_off, d_elem_m, d_emap_off, d_emap, d_dof_ptr, d_dof_el, d_y,
                       d_y_off, (int)esrc.size(), stream3);
  launch_dof_gather(d_dof_ptr, d_dof_idx, d_y, nullptr, n_global, d_r, n_global, 1, 0, stream3);
  launch_absmax(d_r, n_global, d_red + 1536, stream3);
  if (n_trees > 1)
    launch_absmax_tree(d_r, n_global, n_global, d_dof_tree, n_trees, d_tree_red + (size_t)3 * n_trees, stream3);
  CK(cudaEventRecord(ev_anorm, stream3));
  anorm_pending = true;
  anorm_valid = true;
  anorm_inf = -1.0;
  tree_anorm.clear();
}

void Engine::sync_anorm() {
  if (!anorm_pending) return;
  CK(cudaStreamWaitEvent(stream, ev_anorm, 0));
  anorm_pending = false;
}

double Engine::read_scalar(const double* d) {
  double h = 0;
  CK(cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  return h;
}

void Engine::tree_max_async(const double* v, int64_t nv, int64_t ng, int slot) {
  launch_absmax_tree(v, nv, ng, d_dof_tree, n_trees, d_tree_red + (size_t)slot * n_trees, stream);
}

std::vector<double> Engine::read_tree_slot(int slot) {
  std::vector<unsigned long long> bits(n_trees);
  CK(cudaMemcpyAsync(bits.data(), d_tree_red + (size_t)slot * n_trees, sizeof(unsigned long long) * n_trees,
                     cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  std::vector<double> out(n_trees);
  std::memcpy(out.data(), bits.data(), sizeof(double) * n_trees);
  return out;
}

// worst per-tree ||b-Ax|| / (||A|| ||x|| + ||b||); NaN if any tree has a NaN
double Engine::forest_berr(const std::vector<double>& rn, const std::vector<double>& xn) {
  if (tree_anorm.empty()) {
    operator_norm_inf();
    tree_anorm = read_tree_slot(3);
  }
  double worst = 0.0;
  bool nan = false;
  for (int t = 0; t < n_trees; ++t) {
    const double den = tree_anorm[t] * xn[t] + tree_bnorm[t];
    const double b = den > 0 ? rn[t] / den : (rn[t] > 0 ? INFINITY : 0.0);
    if (b != b) nan = true;
    else if (b > worst) worst = b;
  }
  return nan ? NAN : worst;
}

double Engine::operator_norm_inf() {
  if (!anorm_valid) enqueue_anorm();
  sync_anorm();
  if (anorm_inf < 0) anorm_inf = read_scalar(d_red + 1536);
  return anorm_inf;
}

// ---------------------------------------------------------------------------
// learned precision selection
// ---------------------------------------------------------------------------
constexpr double SELECTOR_FP64_CONFIDENCE = 0.9;

void Engine::prepare_device(int method) {
  ensure_plan();
  if (!dev_ok || method_built != method || prec_dirty) {
    build_plan(method);
    build_programs(method);
    alloc_device(method);
  }
}

void Engine::set_selector(const float* params, int n) {
  if (n != uhm_gpu::SEL_NPARAMS) fail("set_selector: wrong parameter count", 7);
  selector_params.assign(params, params + n);
  learned_valid = false;
  prec_dirty = true;
}

// Per front (slot order), SEL_F features from its sizes, its place in the tree
// and statistics of the element matrices of its subtree and of the whole mesh:
//   0 log2(n+1)/14   1 log2(fs+1)/14   2 log2(ss+1)/14   3 depth below the root / 8
//   4 n >= 512 (tensor-core eligible)   5 log10(max/min mean |diagonal|) over the subtree / 6
//   6 mean and 7 min over the subtree of sum(a)/sum|a|
//   8 min column dominance over the subtree (clamped to [-4, 1]) / 4
//   9 min of sum(a)/sum|a| over the mesh   10 log10(max/min mean |diagonal|) over the mesh / 6
//   11 log10(LAWN-41 flops of the front + 1) / 13
void Engine::front_features(std::vector<float>& feat) {
  if (!dev_ok) fail("front features: no device data yet", 7);
  upload_elements();
  const int ne = (int)esrc.size();
  std::vector<float> st((size_t)ne * 4, 0.f);
  if (ne) {
    uhm_gpu::launch_elem_stats(ctx.emat, d_emat_off, d_elem_m, ne, d_sel, stream);
    CK(cudaMemcpyAsync(st.data(), d_sel, sizeof(float) * st.size(), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
  }
  struct Agg {
    double cnt = 0, dmax = 0, dmin = 1e300, rsum = 0, rmin = 1e300, osum = 0, omin = 1e300;
  };
  const int nf = (int)fronts.size();
  std::vector<Agg> agg(nf);
  for (int s = 0; s < nf; ++s) {          // leaf -> root: children come first
    Agg a;
    const int ei = esrc_of_slot[s];
    if (ei >= 0 && esrc[ei].has_lhs) {
      const double dm = st[4 * ei + 0], r = st[4 * ei + 1];
      const double o = std::max(-4.0, std::min(1.0, (double)st[4 * ei + 2]));
      const double om = std::max(-4.0, std::min(1.0, (double)st[4 * ei + 3]));
      a.cnt = 1;
      a.dmax = dm;
      a.dmin = dm;
      a.rsum = r;
      a.rmin = r;
      a.osum = om;
      a.omin = o;
    }
    for (int c : fronts[s].children) {
      const Agg& b = agg[c];
      a.cnt += b.cnt;
      a.dmax = std::max(a.dmax, b.dmax);
      a.dmin = std::min(a.dmin, b.dmin);
      a.rsum += b.rsum;
      a.rmin = std::min(a.rmin, b.rmin);
      a.osum += b.osum;
      a.omin = std::min(a.omin, b.omin);
    }
    agg[s] = a;
  }
  std::vector<int> depth(nf, 0);
  for (int s = nf - 1; s >= 0; --s)
    if (fronts[s].parent >= 0) depth[s] = depth[fronts[s].parent] + 1;
  Agg all;
  for (int s = 0; s < nf; ++s)
    if (fronts[s].parent < 0) {
      const Agg& b = agg[s];
      all.cnt += b.cnt;
      all.dmax = std::max(all.dmax, b.dmax);
      all.dmin = std::min(all.dmin, b.dmin);
      all.rmin = std::min(all.rmin, b.rmin);
    }
  feat.assign((size_t)nf * uhm_gpu::SEL_F, 0.f);
  for (int s = 0; s < nf; ++s) {
    const HostFront& f = fronts[s];
    const Agg& a = agg[s];
    float* x = &feat[(size_t)s * uhm_gpu::SEL_F];
    const double cnt = std::max(1.0, a.cnt);
    const double flops = get_flop_chol(0, f.fs) + get_flop_trsm_lower(0, f.fs, f.ss) + get_flop_syrk(0, f.fs, f.ss);
    x[0] = (float)(std::log2(f.n + 1.0) / 14);
    x[1] = (float)(std::log2(f.fs + 1.0) / 14);
    x[2] = (float)(std::log2(f.ss + 1.0) / 14);
    x[3] = (float)(depth[s] / 8.0);
    x[4] = f.n >= 512 ? 1.f : 0.f;
    x[5] = (float)(a.cnt > 0 && a.dmin > 0 ? std::log10(a.dmax / a.dmin) / 6 : 0.0);
    x[6] = (float)(a.cnt > 0 ? a.rsum / cnt : 0.0);
    x[7] = (float)(a.cnt > 0 ? a.rmin : 0.0);
    x[8] = (float)(a.cnt > 0 ? a.omin / 4 : 0.0);
    x[9] = (float)(all.cnt > 0 ? all.rmin : 0.0);
    x[10] = (float)(all.cnt > 0 && all.dmin > 0 ? std::log10(all.dmax / all.dmin) / 6 : 0.0);
    x[11] = (float)(std::log10(flops + 1.0) / 13);
  }
}

// Runs the selector on the device and records one class per front; the
// device buffers must exist (a provisional plan is built for that on the
// first call), and the plan is rebuilt afterwards with the chosen precisions.
// The per-front class probabilities are decoded per tree level from the mean
// probabilities of its fronts (FP64 only above SELECTOR_FP64_CONFIDENCE), and
// precision may only decrease with depth (class index non-decreasing from the
// root down), which is the shape of the assignments the labels come from.
void Engine::apply_selector(int method) {
  if ((int)selector_params.size() != uhm_gpu::SEL_NPARAMS)
    fail("learned precision requested but no selector parameters were set", 7);
  if (!dev_ok || method_built != method) {
    build_plan(method);
    build_programs(method);
    alloc_device(method);
  }
  std::vector<float> feat;
  front_features(feat);
  const int nf = (int)fronts.size();
  float* d_feat = d_sel + 4 * esrc.size();
  float* d_par = d_feat + (size_t)nf * uhm_gpu::SEL_F;
  float* d_prob = d_par + uhm_gpu::SEL_NPARAMS;
  CK(cudaMemcpyAsync(d_feat, feat.data(), sizeof(float) * feat.size(), cudaMemcpyHostToDevice, stream));
  CK(cudaMemcpyAsync(d_par, selector_params.data(), sizeof(float) * selector_params.size(),
                     cudaMemcpyHostToDevice, stream));
  uhm_gpu::launch_mlp_infer(d_feat, nf, d_par, nullptr, d_prob, stream);
  std::vector<float> prob((size_t)uhm_gpu::SEL_C * nf);
  CK(cudaMemcpyAsync(prob.data(), d_prob, sizeof(float) * prob.size(), cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  std::vector<int> depth(nf, 0);
  int max_depth = 0;
  for (int s = nf - 1; s >= 0; --s) {
    if (fronts[s].parent >= 0) depth[s] = depth[fronts[s].parent] + 1;
    max_depth = std::max(max_depth, depth[s]);
  }
  std::vector<double> lp((size_t)(max_depth + 1) * uhm_gpu::SEL_C, 0.0);
  for (int s = 0; s < nf; ++s)
    for (int c = 0; c < uhm_gpu::SEL_C; ++c) lp[(size_t)depth[s] * uhm_gpu::SEL_C + c] += prob[(size_t)s * uhm_gpu::SEL_C + c];
  std::vector<int> lcls(max_depth + 1, 1);
  for (int d = 0; d <= max_depth; ++d) {
    const double* q = &lp[(size_t)d * uhm_gpu::SEL_C];
    const double tot = q[0] + q[1] + q[2];
    // FP64 costs a large multiple of FP32 on this GPU and a missed target is
    // caught by the FP64 redo anyway: a level goes to FP64 only when the
    // network is confident, otherwise the likelier of FP32 and BF16
    const int best = (tot > 0 && q[0] > SELECTOR_FP64_CONFIDENCE * tot) ? 0 : (q[1] > q[2] ? 1 : 2);
    lcls[d] = d > 0 ? std::max(best, lcls[d - 1]) : best;
  }
  std::vector<int> cls(nf, 1);
  for (int s = 0; s < nf; ++s) cls[s] = lcls[depth[s]];
  // new element matrices often leave the choice unchanged: re-plan only when it moved
  if (cls != learned_class || !dev_ok) prec_dirty = true;
  learned_class.swap(cls);
  learned_valid = true;
}

void Engine::set_tunables(const int* v) {
  Tunables t;
  t.small_max_f64 = v[0];
  t.small_max_f32 = v[1];
  t.tc_min_n = v[2];
  t.gc_min_rows = v[3];
  t.fuse_potrf_trsm = v[4] < 0 ? 0 : v[4];
  t.tc_nbo = v[5];
  t.tc_panel = v[6];
  t.solve_rows = v[7];
  t.lookahead = v[8] ? 1 : 0;
  t.solve_chain = v[9] ? 1 : 0;
  if (t.small_max_f64 < 1 || t.small_max_f64 > SMALL_MAX_F64 || t.small_max_f32 < 1 ||
      t.small_max_f32 > SMALL_MAX_F32 || t.tc_min_n < 256 || t.gc_min_rows < 64 ||
      (t.tc_nbo != 128 && t.tc_nbo != 256 && t.tc_nbo != 512) ||
      (t.tc_panel != 0 && t.tc_panel != 256 && t.tc_panel != 512) || (t.solve_rows != 64 && t.solve_rows != 256))
    fail("set_tunables: value outside the kernels' limits", 7);
  tune = t;
  prec_dirty = true;
  status = 0;          // a valid configuration clears an earlier configuration error
  last_error.clear();
}

void Engine::get_tunables(int* v) const {
  v[0] = tune.small_max_f64;
  v[1] = tune.small_max_f32;
  v[2] = tune.tc_min_n;
  v[3] = tune.gc_min_rows;
  v[4] = tune.fuse_potrf_trsm;
  v[5] = tune.tc_nbo;
  v[6] = tune.tc_panel;
  v[7] = tune.solve_rows;
  v[8] = tune.lookahead;
  v[9] = tune.solve_chain;
}

int Engine::autotune(int method, int reps) {
  if (reps < 1) reps = 1;
  for (auto& es : esrc)
    if (!es.has_lhs) fail("autotune: an element matrix has not been copied in", 7);
  // launch programs as a signature: candidates that produce the same
  // programs need no timing
  auto signature = [&]() {
    build_plan(method);
    build_programs(method);
    std::vector<int64_t> sig;
    for (const auto* ops : {&fac_ops, &fwd_ops, &bwd_ops})
      for (const Op& o : *ops) {
        sig.push_back(o.kind);
        sig.push_back(o.n_items);
        sig.push_back(o.dtype);
      }
    return sig;
  };
  auto time_now = [&]() {
    double best = 1e300;
    for (int r = 0; r < reps + 1; ++r) {        // the first run builds graphs and is not counted
      std::fill(front_kept.begin(), front_kept.end(), 0);   // time whole factorisations
      factor(method);
      solve(method, 3);
      const double t = timing.factor_ms + timing.solve_ms + timing.refine_ms;
      if (r > 0 || reps == 0) best = std::min(best, t);
    }
    return best;
  };
  const bool lu = method != UHM_CHOL;
  struct Knob { int* v; std::vector<int> cand; };
  std::vector<Knob> knobs = {
      {&tune.tc_min_n, {384, 512, 768, 1024, 1536, 1 << 30}},
      {&tune.small_max_f32, {96, 128, 160, 192, 224}},
      {&tune.small_max_f64, {64, 96, 128, 160}},
  };
  if (!lu) knobs.push_back({&tune.fuse_potrf_trsm, {0, 1, 2, 4}});
  if (!lu) knobs.push_back({&tune.tc_panel, {0, 256, 512}});
  if (!lu) knobs.push_back({&tune.solve_rows, {64, 256}});
  if (!lu) knobs.push_back({&tune.lookahead, {0, 1}});
  if (!lu) knobs.push_back({&tune.solve_chain, {0, 1}});
  if (!lu) knobs.push_back({&tune.tc_nbo, {128, 256, 512}});
  if (lu) knobs.push_back({&tune.gc_min_rows, {256, 512, 1024, 2048, 1 << 30}});
  int timed = 0;
  prec_dirty = true;
  double best_t = time_now();
  ++timed;
  for (Knob& k : knobs) {
    const int keep = *k.v;
    std::vector<std::vector<int64_t>> seen;
    seen.push_back(signature());
    int best_v = keep;
    for (int c : k.cand) {
      if (c == keep) continue;
      *k.v = c;
      const std::vector<int64_t> sg = signature();
      bool dup = false;
      for (auto& o : seen) dup = dup || o == sg;
      if (dup) continue;
      seen.push_back(sg);
      prec_dirty = true;
      const double t = time_now();
      ++timed;
      if (t < best_t) { best_t = t; best_v = c; }
    }
    *k.v = best_v;
  }
  prec_dirty = true;
  factor(method);
  solve(method, 3);
  return timed;
}

double Engine::backward_error() {
  if (!factored) fail("backward_error: nothing solved", 9);
  compute_residual(d_x, d_r);
  const int64_t nv = n_global * mesh->n_rhs;
  if (n_trees > 1) {
    operator_norm_inf();
    tree_max_async(d_b, nv, n_global, 2);
    tree_bnorm = read_tree_slot(2);
    tree_max_async(d_r, nv, n_global, 0);
    tree_max_async(d_x, nv, n_global, 1);
    const std::vector<double> rn = read_tree_slot(0);
    return forest_berr(rn, read_tree_slot(1));
  }
  launch_absmax(d_r, nv, d_red, stream);
  launch_absmax(d_x, nv, d_red + 512, stream);
  launch_absmax(d_b, nv, d_red + 1024, stream);
  double h[3];
  CK(cudaMemcpyAsync(&h[0], d_red, sizeof(double), cudaMemcpyDeviceToHost, stream));
  CK(cudaMemcpyAsync(&h[1], d_red + 512, sizeof(double), cudaMemcpyDeviceToHost, stream));
  CK(cudaMemcpyAsync(&h[2], d_red + 1024, sizeof(double), cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  const double an = operator_norm_inf();
  return h[0] / (an * h[1] + h[2]);
}

}  // namespace uhm
