// C ABI of include/uhm_gb300.h: the reference's Fortran interface
// (UHM/src/wrapper/fort.cxx:47-321) plus the uhm_gpu_* additions.
#include "../../include/uhm_gb300.h"

#include <omp.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>

#include <cuda_runtime.h>

#include "engine.hpp"
#include "mesh.hpp"

using uhm::Element;
using uhm::Mesh;
using uhm::Node;

namespace uhm_gpu {
// iteration limits of the bounded device waits, one per kernel unit
int set_wait_limit_factor(long long v);
int set_wait_limit_solve(long long v);
int set_wait_limit_tc(long long v);
int set_wait_limit_noalloc(long long v);
int set_wait_limit_chol_tc(long long v);
}  // namespace uhm_gpu

namespace {
double g_flop = 0.0;
double g_buffer = 0.0, g_buffer_max = 0.0;
thread_local std::string g_err;  // errors raised before a mesh exists

Mesh M(long* h) { return reinterpret_cast<Mesh>(*h); }

void set_err(Mesh m, const std::string& msg, int code) {
  g_err = msg;
  if (m) {
    m->eng().status = code ? code : (m->eng().status ? m->eng().status : 30);
    m->eng().last_error = msg;
  }
  std::fprintf(stderr, "uhm_gb300: %s\n", msg.c_str());
}

template <class F>
int guard(Mesh m, F&& f) {
  try {
    f();
    return m && m->engine ? m->engine->status : 0;
  } catch (const std::exception& e) {
    set_err(m, e.what(), m && m->engine && m->engine->status ? m->engine->status : 30);
    return m && m->engine ? m->engine->status : 30;
  }
}

void account_flops(Mesh m, int method, bool factor) {
  double dec = 0, sol = 0, buf = 0;
  unsigned nnz = 0;
  m->estimate_cost(method, m->datatype, m->n_rhs, dec, sol, nnz, buf);
  g_flop += factor ? dec : sol;
  if (factor) {
    g_buffer = buf;
    g_buffer_max = std::max(g_buffer_max, buf);
  }
}
}  // namespace

extern "C" {

void uhm_initialize_fla_(void) {}
void uhm_finalize_fla_(void) {}
void uhm_set_num_threads_(int* n) { if (n) uhm::set_num_threads(*n); }
void uhm_get_num_threads_(int* n) { *n = uhm::get_num_threads(); }
void uhm_set_hier_block_size_(int* s) { if (s) uhm::set_hier_block_size(*s); }
void uhm_get_hier_block_size_(int* s) { *s = uhm::get_hier_block_size(); }
void uhm_reset_flop_(void) { g_flop = 0.0; }
void uhm_get_flop_(double* f) { *f = g_flop; }
void uhm_get_buffer_used_(double* b) { *b = g_buffer; }
void uhm_get_max_buffer_used_(double* b) { *b = g_buffer_max; }
void uhm_is_multithreading_enable_(int* f) { *f = 1; }
void uhm_is_hier_matrix_enable_(int* f) { *f = 1; }
void uhm_timer_(double* t) { *t = uhm::timer(); }

void uhm_mesh_create_(long* mesh) { *mesh = reinterpret_cast<long>(new uhm::Mesh_()); }
void uhm_mesh_delete_(long* mesh) {
  delete M(mesh);
  *mesh = 0;
}
void uhm_add_element_(long* mesh, long* elt) {
  guard(M(mesh), [&] { *elt = reinterpret_cast<long>(M(mesh)->add_element()); });
}
void uhm_add_node_(long* mesh, int* id, int* phy, int* n_dof, int* p, long* nod) {
  guard(M(mesh), [&] { *nod = reinterpret_cast<long>(M(mesh)->add_node(std::make_pair(*id, *phy), *n_dof, *p)); });
}
void uhm_element_add_node_(long* elt, long* nod) {
  reinterpret_cast<Element>(*elt)->add_node(reinterpret_cast<Node>(*nod));
}
void uhm_copy_in_(long* mesh, long* elt, int* dt, int* mm, int* nn, int* node_disp, int* nods,
                  int* side, double* buffer) {
  guard(M(mesh), [&] {
    M(mesh)->copy_in(reinterpret_cast<Element>(*elt), *dt, *mm, *nn, *node_disp, nods, *side, buffer);
  });
}
void uhm_copy_out_(long* mesh, long* elt, int* dt, int* mm, int* nn, int* node_disp, int* nods,
                   int* side, double* buffer) {
  guard(M(mesh), [&] {
    M(mesh)->copy_out(reinterpret_cast<Element>(*elt), *dt, *mm, *nn, *node_disp, nods, *side, buffer);
  });
}
void uhm_mesh_disp_(long* mesh) {
  Mesh m = M(mesh);
  std::printf("-Mesh-\n  n_nodes [ %d ], n_elements [ %d ], locked [ %d ]\n", m->get_n_nodes(),
              m->get_n_elements(), m->is_locked());
}
void uhm_get_n_dof_(long* mesh, int* n) { *n = (int)M(mesh)->get_n_dof(); }
void uhm_get_n_nonzero_(long* mesh, int* n) { *n = (int)M(mesh)->get_n_nonzero(); }
void uhm_estimate_cost_(long* mesh, int* method, int* dt, int* n_rhs, double* fd, double* fs,
                        unsigned* nnz, double* buf) {
  M(mesh)->estimate_cost(*method, *dt, *n_rhs, *fd, *fs, *nnz, *buf);
}
void uhm_mesh_import_(long* mesh, char* filename) {
  guard(M(mesh), [&] {
    if (!M(mesh)->import_file(filename)) throw std::runtime_error("import_file failed");
  });
}
void uhm_build_tree_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->build_tree(); });
}
void uhm_create_matrix_without_buffer_(long* mesh, int* dt, int* n_rhs) {
  guard(M(mesh), [&] { M(mesh)->create_matrix_without_buffer(*dt, *n_rhs); });
}
void uhm_create_leaf_matrix_buffer_(long* mesh) { M(mesh)->create_leaf_matrix_buffer(); }
void uhm_create_element_matrix_buffer_(long* mesh, int* is_schur) {
  M(mesh)->create_element_matrix_buffer(*is_schur);
}
void uhm_set_rhs_(long* mesh) { M(mesh)->set_rhs(); }
void uhm_lock_(long* mesh) { guard(M(mesh), [&] { M(mesh)->lock(); }); }
void uhm_unlock_(long* mesh) { guard(M(mesh), [&] { M(mesh)->unlock(); }); }

void uhm_chol_with_free_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->chol_with_free(); account_flops(M(mesh), uhm::UHM_CHOL, true); });
}
void uhm_lu_nopiv_with_free_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->lu_nopiv_with_free(); account_flops(M(mesh), uhm::UHM_LU_NOPIV, true); });
}
void uhm_lu_piv_with_free_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->lu_piv_with_free(); account_flops(M(mesh), uhm::UHM_LU_PIV, true); });
}
void uhm_solve_chol_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->solve_chol(); account_flops(M(mesh), uhm::UHM_CHOL, false); });
}
void uhm_solve_lu_nopiv_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->solve_lu_nopiv(); account_flops(M(mesh), uhm::UHM_LU_NOPIV, false); });
}
void uhm_solve_lu_piv_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->solve_lu_piv(); account_flops(M(mesh), uhm::UHM_LU_PIV, false); });
}
void uhm_check_chol_(long* mesh) { M(mesh)->check_chol(); }
void uhm_check_lu_nopiv_(long* mesh) { M(mesh)->check_lu_nopiv(); }
void uhm_check_lu_piv_(long* mesh) { M(mesh)->check_lu_piv(); }
void uhm_lu_incpiv_with_free_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->lu_incpiv_with_free(); account_flops(M(mesh), uhm::UHM_LU_PIV, true); });
}
void uhm_solve_lu_incpiv_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->solve_lu_piv(); account_flops(M(mesh), uhm::UHM_LU_PIV, false); });
}
void uhm_check_lu_incpiv_(long* mesh) { M(mesh)->check_lu_piv(); }
void uhm_random_spd_matrix_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->random_spd_matrix(); });
}
void uhm_random_matrix_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->random_matrix(); });
}
void uhm_triangularize_(long* mesh) { M(mesh)->triangularize(); }
void uhm_svd_with_free_(long* mesh) {
  set_err(M(mesh), "SVD fronts are not provided by this library", 30);
}
void uhm_solve_svd_(long* mesh) { set_err(M(mesh), "SVD fronts are not provided by this library", 30); }
void uhm_check_svd_(long* mesh) { set_err(M(mesh), "SVD fronts are not provided by this library", 30); }
// thresholds of the SVD fronts: kept and returned, used by nothing here
static double g_svd_rel = 0.0, g_svd_abs = 0.0;
static int g_svd_cutoff = 0;
void set_svd_relative_threshold_(double* val) { g_svd_rel = *val; }
void set_svd_absolute_threshold_(double* val) { g_svd_abs = *val; }
void get_svd_relative_threshold_(double* val) { *val = g_svd_rel; }
void get_svd_absolute_threshold_(double* val) { *val = g_svd_abs; }
void set_svd_cutoff_small_(int* flag) { g_svd_cutoff = *flag; }
void get_svd_cutoff_small_(int* flag) { *flag = g_svd_cutoff; }
void uhm_qr_with_free_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->qr_with_free(); });
}
void uhm_solve_qr_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->solve_qr(); });
}
void uhm_check_qr_(long* mesh) {
  guard(M(mesh), [&] { M(mesh)->check_qr(); });
}
void uhm_get_residual_(long* mesh, double* res) {
  guard(M(mesh), [&] { *res = M(mesh)->get_residual(); });
}

// ---- Part 2 ---------------------------------------------------------------
int uhm_gpu_add_element_with_generation(long* mesh, int* gen, long* elt) {
  return guard(M(mesh), [&] { *elt = reinterpret_cast<long>(M(mesh)->add_element(*gen)); });
}
int uhm_gpu_element_set_parent(long* elt, long* parent) {
  try {
    reinterpret_cast<Element>(*elt)->set_parent(reinterpret_cast<Element>(*parent));
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 7;
  }
}
int uhm_gpu_element_add_child(long* elt, long* child) {
  reinterpret_cast<Element>(*elt)->add_child(reinterpret_cast<Element>(*child));
  return 0;
}
int uhm_gpu_element_set_reuse(long* elt, int flag) {
  reinterpret_cast<Element>(*elt)->set_reuse(flag);
  return 0;
}
int uhm_gpu_element_get_reuse(long* elt, int* flag) {
  *flag = reinterpret_cast<Element>(*elt)->is_matrix_reusable() ? 1 : 0;
  return 0;
}
int uhm_gpu_mesh_backup(long* mesh, long* backup) {
  return guard(M(mesh), [&] { M(mesh)->backup(M(backup)); });
}
int uhm_gpu_mesh_check_reuse(long* mesh, long* backup) {
  return guard(M(mesh), [&] { M(mesh)->check_reuse(M(backup)); });
}
int uhm_gpu_export_sparse(long* mesh, int is_sym, int fort, int cs, int compress, int axpy, int* n_dof,
                          int* n_rhs, long* len_ia, long* len_ja, long* n_nz, int* ia, int* ja, double* a,
                          double* b) {
  return guard(M(mesh), [&] {
    uhm::Engine::SparseOut o;
    M(mesh)->eng().export_sparse(is_sym, fort, cs, compress, axpy, o);
    *n_dof = o.n_dof;
    *n_rhs = o.n_rhs;
    *len_ia = (long)o.ia.size();
    *len_ja = (long)o.ja.size();
    *n_nz = (long)o.a.size();
    if (ia) std::memcpy(ia, o.ia.data(), sizeof(int) * o.ia.size());
    if (ja) std::memcpy(ja, o.ja.data(), sizeof(int) * o.ja.size());
    if (a) std::memcpy(a, o.a.data(), sizeof(double) * o.a.size());
    if (b) std::memcpy(b, o.b.data(), sizeof(double) * o.b.size());
  });
}
int uhm_gpu_get_node_offsets(long* mesh, int n, const int* ids, int* offsets) {
  return guard(M(mesh), [&] {
    uhm::Mesh_* m = M(mesh);
    if (!m->is_locked()) throw std::invalid_argument("node offsets: the mesh is not locked");
    for (int i = 0; i < n; ++i) {
      uhm::Node nd = m->find_node(ids[i]);
      if (!nd) throw std::invalid_argument("node offsets: unknown node");
      offsets[i] = nd->get_offset();
    }
  });
}
int uhm_gpu_get_tree(long* mesh, int cap, int* elt_id, int* parent_id, int* generation, int* n) {
  return guard(M(mesh), [&] {
    uhm::Mesh_* m = M(mesh);
    *n = (int)m->elements.size();
    if (cap < *n) return;
    int i = 0;
    for (auto& kv : m->elements) {
      elt_id[i] = kv.first;
      parent_id[i] = kv.second.parent ? kv.second.parent->get_id() : -1;
      generation[i] = kv.second.get_generation();
      ++i;
    }
  });
}
int uhm_gpu_get_children(long* mesh, int elt_id, int cap, int* child_id, int* n) {
  return guard(M(mesh), [&] {
    uhm::Element e = M(mesh)->find_element(elt_id);
    if (!e) throw std::invalid_argument("get_children: unknown element");
    *n = e->get_n_children();
    for (int i = 0; i < *n && i < cap; ++i) child_id[i] = e->get_child(i)->get_id();
  });
}
int uhm_gpu_get_n_refactored(long* mesh, int* n) {
  return guard(M(mesh), [&] { *n = M(mesh)->eng().n_refactored; });
}
int uhm_gpu_get_status(long* mesh) {
  Mesh m = M(mesh);
  return m && m->engine ? m->engine->status : 0;
}
int uhm_gpu_get_last_error(long* mesh, char* buf, int len) {
  Mesh m = M(mesh);
  std::string s = m && m->engine && !m->engine->last_error.empty() ? m->engine->last_error : g_err;
  if (len > 0) {
    std::strncpy(buf, s.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return (int)s.size();
}
int uhm_gpu_set_mode(long* mesh, int mode, int default_prec, double tol, int max_iter) {
  return guard(M(mesh), [&] {
    uhm::Engine& e = M(mesh)->eng();
    if (e.mode != mode || e.default_prec != default_prec) e.invalidate_precision();
    e.mode = mode;
    e.default_prec = default_prec;
    e.ir_tol = tol;
    e.ir_max = max_iter;
  });
}
int uhm_gpu_set_front_precision(long* mesh, int n, const int* prec) {
  return guard(M(mesh), [&] {
    uhm::Mesh_* m = M(mesh);
    uhm::Engine& e = m->eng();
    e.ensure_plan();
    e.front_prec_override.assign(e.fronts.size(), -1);
    for (auto& f : e.fronts) {
      int id = f.e->get_id();
      if (id < n) e.front_prec_override[f.slot] = prec[id];
    }
    e.invalidate_precision();
  });
}
int uhm_gpu_get_op_log(long* mesh, int cap, int* kind, int* n_items, double* ms, int* n_out) {
  return guard(M(mesh), [&] {
    uhm::Engine& e = M(mesh)->eng();
    const int n = (int)e.op_log.size();
    *n_out = n;
    for (int i = 0; i < n && i < cap; ++i) {
      kind[i] = e.op_log[i].kind;
      n_items[i] = e.op_log[i].n_items;
      ms[i] = e.op_log[i].ms;
    }
  });
}
int uhm_gpu_generate_lobatto_elements(long* mesh, int method, int dim, double hh, double cmass, double cconv,
                                      int n_el, const double* ref, const long* ref_off, int n_ref_off,
                                      const int* p_el, const double* kappa, const double* react,
                                      const double* beta, const long* sel_ptr, const int* sel) {
  static_assert(sizeof(long) == sizeof(int64_t), "long is 64-bit");
  return guard(M(mesh), [&] {
    M(mesh)->eng().generate_lobatto_elements(method, dim, hh, cmass, cconv, n_el, ref,
                                             reinterpret_cast<const int64_t*>(ref_off), n_ref_off, p_el, kappa,
                                             react, beta, reinterpret_cast<const int64_t*>(sel_ptr),
                                             reinterpret_cast<const int32_t*>(sel));
  });
}
int uhm_gpu_set_tunables(long* mesh, const int* values) {
  return guard(M(mesh), [&] { M(mesh)->eng().set_tunables(values); });
}
int uhm_gpu_get_tunables(long* mesh, int* values) {
  // a query: it cannot fail and does not report an earlier call's status
  if (!M(mesh)) return 30;
  M(mesh)->eng().get_tunables(values);
  return 0;
}
int uhm_gpu_autotune(long* mesh, int method, int reps, int* n_timed) {
  return guard(M(mesh), [&] { *n_timed = M(mesh)->eng().autotune(method, reps); });
}
int uhm_gpu_set_selector(long* mesh, const float* params, int n) {
  return guard(M(mesh), [&] { M(mesh)->eng().set_selector(params, n); });
}
int uhm_gpu_get_front_features(long* mesh, int method, int n_fronts, float* out) {
  return guard(M(mesh), [&] {
    uhm::Engine& e = M(mesh)->eng();
    e.prepare_device(method);
    std::vector<float> f;
    e.front_features(f);
    if (n_fronts != (int)e.fronts.size()) {
      e.status = 7;
      throw std::invalid_argument("get_front_features: front count mismatch");
    }
    std::copy(f.begin(), f.end(), out);
  });
}
int uhm_gpu_get_front_precision(long* mesh, int n_fronts, int* prec, int* learned_class) {
  return guard(M(mesh), [&] {
    uhm::Engine& e = M(mesh)->eng();
    e.ensure_plan();
    if (n_fronts != (int)e.fronts.size()) {
      e.status = 7;
      throw std::invalid_argument("get_front_precision: front count mismatch");
    }
    for (auto& f : e.fronts) {
      if (prec) prec[f.slot] = f.prec;
      if (learned_class)
        learned_class[f.slot] = (int)e.learned_class.size() > f.slot ? e.learned_class[f.slot] : -1;
    }
  });
}
int uhm_gpu_copy_in_leaves(long* mesh, int side, const int* nods_all, const double* buffer,
                           long n_values) {
  return guard(M(mesh), [&] {
    uhm::Mesh_* m = M(mesh);
    uhm::Engine& e = m->eng();
    e.ensure_plan();
    if (nods_all) e.set_leaf_nodes(nods_all);
    e.copy_in_leaves(side, buffer, n_values);
  });
}
int uhm_gpu_copy_out_leaves(long* mesh, double* buffer, long n_values) {
  return guard(M(mesh), [&] { M(mesh)->eng().copy_out_leaves(buffer, n_values); });
}
int uhm_gpu_get_node_solution(long* mesh, int n_nodes, const int* ids, double* out, long n_values) {
  return guard(M(mesh), [&] { M(mesh)->eng().node_solution(n_nodes, ids, out, n_values); });
}
int uhm_gpu_backward_error(long* mesh, double* berr) {
  return guard(M(mesh), [&] { *berr = M(mesh)->eng().backward_error(); });
}
int uhm_gpu_get_timing(long* mesh, double* out) {
  return guard(M(mesh), [&] {
    const uhm::Timing& t = M(mesh)->eng().timing;
    out[0] = t.upload_ms;
    out[1] = t.factor_ms;
    out[2] = t.solve_ms;
    out[3] = t.refine_ms;
    out[4] = t.total_ms;
    out[5] = t.ir_iters;
    out[6] = t.berr;
    out[7] = (double)t.kernel_launches;
    out[8] = t.berr_first;
  });
}
int uhm_gpu_set_profiling(long* mesh, int on) {
  return guard(M(mesh), [&] {
    uhm::Engine& e = M(mesh)->eng();
    e.profiling = on != 0;
    e.profile = uhm::OpProfile{};
    e.op_log.clear();
  });
}
int uhm_gpu_get_profile(long* mesh, int n_kinds, double* ms, double* flops, double* bytes,
                        long* launches) {
  return guard(M(mesh), [&] {
    const uhm::OpProfile& p = M(mesh)->eng().profile;
    for (int k = 0; k < n_kinds && k < uhm::N_OP_KINDS; ++k) {
      ms[k] = p.ms[k];
      flops[k] = p.flops[k];
      bytes[k] = p.bytes[k];
      launches[k] = (long)p.launches[k];
    }
  });
}
int uhm_gpu_get_n_fronts(long* mesh, int* n) {
  return guard(M(mesh), [&] {
    uhm::Engine& e = M(mesh)->eng();
    e.ensure_plan();
    *n = (int)e.fronts.size();
  });
}
int uhm_gpu_get_fronts(long* mesh, int n, int* eid, int* gen, int* fs, int* ss) {
  return guard(M(mesh), [&] {
    uhm::Engine& e = M(mesh)->eng();
    e.ensure_plan();
    for (int i = 0; i < n && i < (int)e.fronts.size(); ++i) {
      eid[i] = e.fronts[i].e->get_id();
      gen[i] = e.fronts[i].e->get_generation();
      fs[i] = e.fronts[i].fs;
      ss[i] = e.fronts[i].ss;
    }
  });
}
int uhm_gpu_get_front_nodes(long* mesh, int elt_id, int cap, int* ids, int* nf, int* ns) {
  return guard(M(mesh), [&] {
    Element e = M(mesh)->find_element(elt_id);
    if (!e) throw std::invalid_argument("no such element");
    int k = 0;
    for (auto& pr : e->factor)
      if (k < cap) ids[k++] = pr.first->get_id().first;
    for (auto& pr : e->schur)
      if (k < cap) ids[k++] = pr.first->get_id().first;
    *nf = (int)e->factor.size();
    *ns = (int)e->schur.size();
  });
}
int uhm_gpu_get_front_block(long* mesh, int elt_id, int mat, int m, int n, void* out) {
  return guard(M(mesh), [&] {
    Element e = M(mesh)->find_element(elt_id);
    if (!e || !e->get_matrix()) throw std::invalid_argument("get_front_block: no such element or no matrix");
    const int fs = e->hm.fs, ss = e->hm.ss, nr = e->hm.n_rhs;
    int em = 0, en = 0;
    switch (mat) {
      case uhm::UHM_ATL: em = fs; en = fs; break;
      case uhm::UHM_ATR: em = fs; en = ss; break;
      case uhm::UHM_ABL: em = ss; en = fs; break;
      case uhm::UHM_ABR: em = ss; en = ss; break;
      case uhm::UHM_P: em = fs; en = 1; break;
      case uhm::UHM_XT: em = fs; en = nr; break;
      case uhm::UHM_XB: em = ss; en = nr; break;
      default: throw std::invalid_argument("get_front_block: block not held by this engine");
    }
    if (m != em || n != en) throw std::invalid_argument("get_front_block: buffer dimensions do not match the block");
    e->get_matrix()->copy_out(mat, out);
  });
}

void* uhm_gpu_host_alloc(long bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, (size_t)bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}
void uhm_gpu_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int uhm_gpu_set_wait_limit(long long iters) {
  int rc = 0;
  rc |= uhm_gpu::set_wait_limit_factor(iters);
  rc |= uhm_gpu::set_wait_limit_solve(iters);
  rc |= uhm_gpu::set_wait_limit_tc(iters);
  rc |= uhm_gpu::set_wait_limit_noalloc(iters);
  rc |= uhm_gpu::set_wait_limit_chol_tc(iters);
  return rc ? 7 : 0;
}

}  // extern "C"
