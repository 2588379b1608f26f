// Host restatement of UHM's mesh layer and symbolic analysis.
//   Node_      UHM/src/mesh/node.cxx
//   Element_   UHM/src/mesh/element.cxx
//   Mesh_      UHM/src/mesh/mesh.cxx, matrix.cxx, interf.cxx, chol.cxx, lu_piv.cxx
// The numerical methods delegate to the device engine (engine.hpp).
#include "mesh.hpp"

#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cassert>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <set>
#include <stdexcept>

#include "engine.hpp"

namespace uhm {

bool NodeIdLess::operator()(const Node_* a, const Node_* b) const { return a->id < b->id; }
bool ElementIdLess::operator()(const Element_* a, const Element_* b) const { return a->id < b->id; }

// ---------------------------------------------------------------------------
// Node_
// ---------------------------------------------------------------------------
void Node_::clean_connectivity() {
  for (auto it = owner.begin(); it != owner.end();) {
    if (!(*it)->is_leaf()) it = owner.erase(it);
    else ++it;
  }
}

// ---------------------------------------------------------------------------
// Element_
// ---------------------------------------------------------------------------
std::pair<int, int> Element_::get_n_dof() const {
  std::pair<int, int> r(0, 0);
  for (auto& kv : nodes) {
    if (kv.second == UHM_SEPARATED_FACTOR) r.first += kv.first->get_n_dof();
    else if (kv.second == UHM_SEPARATED_SCHUR) r.second += kv.first->get_n_dof();
  }
  return r;
}

int Element_::get_height() const {
  int h = 0;
  const Element_* e = this;
  while (e->parent) { e = e->parent; ++h; }
  return h;
}

void Element_::set_parent(Element p) {
  if (!p) throw std::invalid_argument("set_parent: null element");
  parent = p;
}

void Element_::add_node(Node n, int separated) {
  auto r = nodes.insert(std::make_pair(n, separated));
  r.first->second = separated;
  if (r.second) n->add_owner(this);
}

void Element_::update_generation() {
  if (is_leaf()) return;
  int gen = 0;
  for (Element c : children) gen = std::min(gen, c->get_generation());
  generation = gen - 1;
}

// element.cxx:272-286: a node is eliminated here iff it has one owner and default kind
void Element_::separate_nodes() {
  for (auto& kv : nodes) {
    if (!kv.first->get_n_owner()) throw std::logic_error("node without owner");
    kv.second = (kv.first->get_n_owner() == 1 && kv.first->get_kind() == UHM_NODE_KIND_DEFAULT)
                    ? UHM_SEPARATED_FACTOR : UHM_SEPARATED_SCHUR;
  }
}

// element.cxx:288-334: factor and schur nodes sorted by global offset
void Element_::arrange_nodes() {
  factor.clear();
  schur.clear();
  std::map<int, Node> f, s;
  for (auto& kv : nodes) {
    if (!kv.first->get_n_dof()) continue;
    if (kv.second == UHM_SEPARATED_FACTOR) f.insert({kv.first->get_offset(), kv.first});
    else if (kv.second == UHM_SEPARATED_SCHUR) s.insert({kv.first->get_offset(), kv.first});
  }
  int o = 0;
  for (auto& kv : f) { factor.push_back({kv.second, o}); o += kv.second->get_n_dof(); }
  o = 0;
  for (auto& kv : s) { schur.push_back({kv.second, o}); o += kv.second->get_n_dof(); }
}

// element.cxx:336-360
void Element_::merge_nodes_from_children() {
  if (is_leaf()) return;
  nodes.clear();
  for (Element c : children) merge_nodes(c);
}

void Element_::merge_nodes(Element c) {
  for (auto& kv : c->nodes)
    if (kv.second == UHM_SEPARATED_SCHUR) {
      add_node(kv.first);
      kv.first->remove_owner(c);
    }
}

// element.cxx:362-381
void Element_::restore_connectivity() {
  if (!is_leaf()) return;
  for (auto& kv : nodes) {
    kv.second = UHM_NOT_SEPARATED;
    kv.first->clean_connectivity();
    kv.first->add_owner(this);
  }
  factor.clear();
  schur.clear();
}

// element.cxx:383-392 (node-id order: deterministic)
void Element_::numbering(int64_t& g) {
  for (auto& kv : nodes)
    if (kv.second == UHM_SEPARATED_FACTOR) {
      kv.first->set_offset((int)g);
      g += kv.first->get_n_dof();
    }
}

// ---------------------------------------------------------------------------
// LAWN-41 (LINAL/src/util.cxx:60-116)
// ---------------------------------------------------------------------------
static inline double MUL(int c) { return c ? 6.0 : 1.0; }
static inline double ADD(int c) { return c ? 2.0 : 1.0; }
double get_flop_gemm(int c, int mm, int nn, int kk) {
  double m = mm, n = nn, k = kk;
  return MUL(c) * (m * n * k) + ADD(c) * (m * n * k);
}
double get_flop_syrk(int c, int kk, int nn) {
  double k = kk, n = nn;
  return MUL(c) * (0.5 * k * n * (n + 1.0)) + ADD(c) * (0.5 * k * n * (n + 1.0));
}
double get_flop_trsm_lower(int c, int mm, int nn) {
  double m = mm, n = nn;
  return MUL(c) * (0.5 * n * m * (m + 1.0)) + ADD(c) * (0.5 * n * m * (m - 1.0));
}
double get_flop_trsm_upper(int c, int mm, int nn) {
  double m = mm, n = nn;
  return MUL(c) * (0.5 * m * n * (n + 1.0)) + ADD(c) * (0.5 * m * n * (n - 1.0));
}
double get_flop_lu(int c, int mm, int nn) {
  double m = mm, n = nn;
  if (m > n)
    return MUL(c) * (0.5 * m * n * n - (1.0 / 6.0) * n * n * n + 0.5 * m * n - 0.5 * n * n + (2.0 / 3.0) * n) +
           ADD(c) * (0.5 * m * n * n - (1.0 / 6.0) * n * n * n - 0.5 * m * n + (1.0 / 6.0) * n);
  return MUL(c) * (0.5 * n * m * m - (1.0 / 6.0) * m * m * m + 0.5 * n * m - 0.5 * m * m + (2.0 / 3.0) * m) +
         ADD(c) * (0.5 * n * m * m - (1.0 / 6.0) * m * m * m - 0.5 * n * m + (1.0 / 6.0) * m);
}
double get_flop_chol(int c, int nn) {
  double n = nn;
  return MUL(c) * ((1.0 / 6.0) * n * n * n + 0.5 * n * n + (1.0 / 3.0) * n) +
         ADD(c) * ((1.0 / 6.0) * n * n * n - (1.0 / 6.0) * n);
}

// element.cxx:128-195
void Element_::estimate_cost(int method, int datatype, int n_rhs, double& dec, double& sol,
                             unsigned& nnz, double& buffer) const {
  const int c = datatype == UHM_COMPLEX;
  const std::pair<int, int> d = get_n_dof();
  const int fs = d.first, ss = d.second;
  const double mem = c ? 16.0 : 8.0;
  if (method == UHM_CHOL) {
    dec = get_flop_chol(c, fs) + get_flop_trsm_lower(c, fs, ss) + get_flop_syrk(c, fs, ss);
    buffer = mem * fs * fs + mem * ss * fs;
    nnz = fs * fs + ss * fs;
  } else {
    dec = get_flop_lu(c, fs, fs) + get_flop_trsm_lower(c, fs, ss) + get_flop_trsm_upper(c, ss, fs) +
          get_flop_gemm(c, ss, ss, fs);
    buffer = mem * fs * fs + 2 * mem * ss * fs;
    nnz = (unsigned)(fs * fs + 2.0 * ss * fs);
  }
  sol = get_flop_trsm_lower(c, fs, n_rhs) + get_flop_gemm(c, ss, n_rhs, fs) +
        get_flop_trsm_upper(c, n_rhs, fs) + get_flop_gemm(c, fs, n_rhs, ss);
}

// ---------------------------------------------------------------------------
// Mesh_
// ---------------------------------------------------------------------------
Mesh_::Mesh_() {}
Mesh_::~Mesh_() { delete engine; }

Engine& Mesh_::eng() {
  if (!engine) engine = new Engine(this);
  return *engine;
}

Node Mesh_::add_node(int id, int n_dof) { return add_node(std::make_pair(id, 0), n_dof, n_dof, 0); }
Node Mesh_::add_node(int id, int n_dof, int p) { return add_node(std::make_pair(id, 0), n_dof, p, 0); }
Node Mesh_::add_node(std::pair<int, int> id, int n_dof) { return add_node(id, n_dof, n_dof, 0); }
Node Mesh_::add_node(std::pair<int, int> id, int n_dof, int p) { return add_node(id, n_dof, p, 0); }
Node Mesh_::add_node(std::pair<int, int> id, int n_dof, int p, int kind) {
  auto r = nodes.insert(std::make_pair(id, Node_(id, n_dof, p, kind)));
  if (!r.second) {
    Node_& n = r.first->second;
    if (n.n_dof != n_dof || n.p != p || n.kind != kind)
      throw std::invalid_argument("add_node: node exists with different attributes");
  }
  return &r.first->second;
}

Node Mesh_::find_node(int id) { return find_node(std::make_pair(id, 0)); }
Node Mesh_::find_node(std::pair<int, int> id) {
  auto it = nodes.find(id);
  return it == nodes.end() ? nullptr : &it->second;
}

Element Mesh_::add_element() { return add_element(0); }
Element Mesh_::add_element(int gen) {
  auto r = elements.insert(std::make_pair(id_element, Element_(id_element, gen)));
  ++id_element;
  return &r.first->second;
}

Element Mesh_::find_element(int id) {
  auto it = elements.find(id);
  return it == elements.end() ? nullptr : &it->second;
}

Element Mesh_::get_root() {
  if (elements.empty()) return nullptr;
  Element e = &elements.begin()->second;
  while (e->parent) e = e->parent;
  return e;
}

// mesh.cxx:385-421 (non-binary branch)
Element Mesh_::refine_element(int id, int n_children) {
  Element e = find_element(id);
  if (!e || n_children < 2) throw std::invalid_argument("refine_element");
  for (int i = 0; i < n_children; ++i) {
    Element c = add_element(e->get_generation() + 1);
    c->set_parent(e);
    e->add_child(c);
  }
  return e;
}

void Mesh_::reset() {
  unlock();
  delete engine;
  engine = nullptr;
  elements.clear();
  nodes.clear();
  id_element = 0;
}

// mesh.cxx:113-154: connectivity only, by element id; each factor / schur
// node is kept as (its address in this mesh, n_dof + p + kind)
void Mesh_::backup(Mesh_* b) {
  if (!b || b == this) throw std::invalid_argument("backup: needs another mesh");
  b->reset();
  for (auto& kv : elements) {
    const Element_& a = kv.second;
    Element_& c = b->elements.insert(std::make_pair(a.id, Element_(a.id, a.generation))).first->second;
    for (const auto& pr : a.factor)
      c.factor.emplace_back(pr.first, pr.first->get_n_dof() + pr.first->get_p() + pr.first->get_kind());
    for (const auto& pr : a.schur)
      c.schur.emplace_back(pr.first, pr.first->get_n_dof() + pr.first->get_p() + pr.first->get_kind());
  }
  b->id_element = id_element;
}

// mesh.cxx:156-225, in the same element order (by id): an element keeps its
// factorisation when an element of its id is in the backup with the same
// factor and schur nodes (same node, same n_dof + p + kind, same order);
// one that does not clears the flag on itself and every ancestor
void Mesh_::check_reuse(Mesh_* b) {
  if (!b || b == this) throw std::invalid_argument("check_reuse: needs the backup mesh");
  for (auto& kv : elements) kv.second.set_reuse(1);
  auto same = [](const std::vector<std::pair<Node, int>>& x, const std::vector<std::pair<Node, int>>& y) {
    if (x.size() != y.size()) return false;
    for (size_t i = 0; i < x.size(); ++i) {
      const Node n = x[i].first;
      if (n != y[i].first || n->get_n_dof() + n->get_p() + n->get_kind() != y[i].second) return false;
    }
    return true;
  };
  for (auto& kv : elements) {
    Element a = &kv.second;
    Element bb = b->find_element(a->get_id());
    const bool flag = bb && same(a->factor, bb->factor) && same(a->schur, bb->schur);
    a->set_reuse(flag);
    if (!a->is_matrix_reusable())
      for (Element u = a; u; u = u->get_parent()) u->set_reuse(0);
  }
}

// Heavy-edge matching, level by level (build_tree_var1.cxx:53-181).  Each
// round visits the elements without a parent in order and, through their
// schur nodes, every pair of them that shares a node.  A pair's weight is
// (dofs of the nodes only the two of them own, minus the dofs of every
// other schur node of either); pairs are merged under a new parent from the
// heaviest down (equal weights: the later-listed pair first, as a reverse
// walk of the reference's multimap), each element at most once per round.
// The new parents and the unmerged elements make the next round's list.
// Differences, all deterministic: elements and nodes are ordered by id
// where the reference compares addresses; a round that merges nothing ends
// the build (each connected part of the mesh becomes its own tree, where
// the reference would not stop); and a new element that eliminates no node
// is taken out again, its children moved to its parent in its place (its
// parent merges the same nodes), so every interior front factors something.
int Mesh_::build_tree() {
  unlock();
  // the subtrees already present, children before parents
  std::vector<Element> orphan;
  for (auto& kv : elements)
    if (kv.second.is_orphan()) orphan.push_back(&kv.second);
  std::vector<Element> post;
  std::function<void(Element)> visit = [&](Element e) {
    for (Element c : e->children) visit(c);
    post.push_back(e);
  };
  for (Element e : orphan) visit(e);
  for (Element e : post)
    if (e->is_leaf()) e->restore_connectivity();
  for (Element e : post) {
    e->merge_nodes_from_children();
    e->separate_nodes();
  }
  std::vector<Element> created;
  while (orphan.size() > 1) {
    std::set<std::pair<int, int>> seen;
    struct Cand {
      int w0, w1;
      size_t order;
      Element a, b;
    };
    std::vector<Cand> cand;
    for (Element o : orphan)
      for (auto& kv : o->nodes) {
        if (kv.second != UHM_SEPARATED_SCHUR) continue;
        for (Element nb : kv.first->owner) {
          if (nb == o) continue;
          Element a = o, b = nb;
          if (a->id > b->id) std::swap(a, b);
          if (!seen.insert({a->id, b->id}).second) continue;
          int w0 = 0, w1 = 0;
          const Element pr[2] = {a, b};
          for (int i = 0; i < 2; ++i)
            for (auto& nn : pr[i]->nodes) {
              if (nn.second != UHM_SEPARATED_SCHUR) continue;
              const Node n = nn.first;
              if (n->get_n_owner() == 2 && n->owner.count(pr[1 - i])) {
                if (i == 0) w0 += n->get_n_dof();
              } else {
                w1 -= n->get_n_dof();
              }
            }
          cand.push_back(Cand{w0, w1, cand.size(), a, b});
        }
      }
    std::stable_sort(cand.begin(), cand.end(),
                     [](const Cand& x, const Cand& y) { return x.w0 != y.w0 ? x.w0 < y.w0 : x.w1 < y.w1; });
    std::vector<Element> next;
    for (auto it = cand.rbegin(); it != cand.rend(); ++it) {
      Element a = it->a, b = it->b;
      if (!a->is_orphan() || !b->is_orphan()) continue;
      Element p = add_element(std::min(a->get_generation(), b->get_generation()) - 1);
      p->add_child(a);
      a->set_parent(p);
      p->add_child(b);
      b->set_parent(p);
      p->merge_nodes_from_children();
      p->separate_nodes();
      next.push_back(p);
      created.push_back(p);
    }
    if (next.empty()) break;   // no two parts share a node: one tree per part
    for (Element o : orphan)
      if (o->is_orphan()) next.push_back(o);
    orphan.swap(next);
  }
  // take out new elements that eliminate nothing (their parent merges the
  // same nodes from their children)
  for (Element p : created) {
    if (!p->parent || p->get_n_dof().first > 0) continue;
    Element q = p->parent;
    std::vector<Element> kids;
    for (Element c : q->children) {
      if (c != p) {
        kids.push_back(c);
        continue;
      }
      for (Element g : p->children) {
        g->parent = q;
        kids.push_back(g);
      }
    }
    q->children.swap(kids);
    for (auto& kv : p->nodes) kv.first->remove_owner(p);
    elements.erase(p->id);
  }
  int roots = 0;
  for (auto& kv : elements) roots += kv.second.is_orphan() ? 1 : 0;
  if (engine) engine->invalidate_plan();
  return roots;
}

// ---------------------------------------------------------------------------
// free functions (util.hxx:44-60, matrix.hxx:40-41, operation/mesh.hxx:48)
// ---------------------------------------------------------------------------
static int g_hier_block_size = 256;   // the reference's default (UHM/src/matrix/uhm/matrix.cxx:39-42)

double timer() {
  return std::chrono::duration<double>(std::chrono::system_clock::now().time_since_epoch()).count();
}
bool is_hier_matrix_enable() { return true; }
bool is_multithreading_enable() { return true; }
void set_num_threads(int nt) {
  if (nt > 0) omp_set_num_threads(nt);
}
int get_num_threads() { return omp_get_max_threads(); }
void set_hier_block_size(int size) {
  if (size > 0) g_hier_block_size = size;
}
int get_hier_block_size() { return g_hier_block_size; }
bool build_tree(Mesh m) {
  if (!m) return false;
  m->build_tree();
  return true;
}

// .uhm text format of Mesh_::import_file (UHM/src/mesh/mesh.cxx:511-579)
bool Mesh_::import_file(const char* path) {
  reset();
  FILE* fp = std::fopen(path, "r");
  if (!fp) return false;
  char line[10000];
  auto next = [&](char* buf) -> bool {
    while (std::fgets(buf, sizeof(line), fp)) {
      const char* p = buf;
      while (*p == ' ' || *p == '\t') ++p;
      if (*p == '#' || *p == '\n' || *p == 0) continue;
      return true;
    }
    return false;
  };
  char fmt[32] = {0};
  if (!next(line) || std::sscanf(line, "%31s", fmt) != 1 || std::strcmp(fmt, "UHM")) {
    std::fclose(fp);
    return false;
  }
  int n_nodes = 0, n_elements = 0;
  if (!next(line) || std::sscanf(line, "%d", &n_nodes) != 1) { std::fclose(fp); return false; }
  for (int i = 0; i < n_nodes; ++i) {
    int id, phy, ndof, p, kind;
    if (!next(line) || std::sscanf(line, "%d %d %d %d %d", &id, &phy, &ndof, &p, &kind) != 5) {
      std::fclose(fp);
      return false;
    }
    add_node(std::make_pair(id, phy), ndof, p, kind);
  }
  if (!next(line) || std::sscanf(line, "%d", &n_elements) != 1) { std::fclose(fp); return false; }
  for (int i = 0; i < n_elements; ++i) {
    int nn;
    if (!next(line) || std::sscanf(line, "%d", &nn) != 1) { std::fclose(fp); return false; }
    Element e = add_element();
    for (int j = 0; j < nn; ++j) {
      int id, phy;
      if (!next(line) || std::sscanf(line, "%d %d", &id, &phy) != 2) { std::fclose(fp); return false; }
      Node n = find_node(std::make_pair(id, phy));
      if (!n) { std::fclose(fp); return false; }
      e->add_node(n);
    }
  }
  std::fclose(fp);
  // remove orphan nodes (mesh.cxx:236-241)
  for (auto it = nodes.begin(); it != nodes.end();) {
    if (!it->second.get_n_owner()) it = nodes.erase(it);
    else ++it;
  }
  return true;
}

// mesh.cxx:438-456
void Mesh_::lock() {
  unlock();
  // Scheduler_::load: group by generation (leaf -> root = descending), id order inside
  for (auto& kv : elements) {
    by_generation[kv.second.get_generation()].push_back(&kv.second);
    if (kv.second.is_leaf()) leaves.push_back(&kv.second);
  }
  for (Element e : leaves) e->restore_connectivity();
  for (auto& g : by_generation)
    for (Element e : g.second) {
      e->merge_nodes_from_children();
      e->separate_nodes();
    }
  int64_t goff = 0;
  for (auto& g : by_generation)
    for (Element e : g.second) e->numbering(goff);
  n_dof_total = goff;
  for (auto& g : by_generation)
    for (Element e : g.second) e->arrange_nodes();
  locker = 1;
  if (engine) engine->invalidate_plan();
}

void Mesh_::unlock() {
  by_generation.clear();
  leaves.clear();
  locker = 0;
  if (engine) engine->invalidate_plan();
}

// matrix.cxx:64-90
void Mesh_::create_matrix_without_buffer(int dt, int nrhs) {
  if (dt != UHM_REAL) throw std::invalid_argument("only UHM_REAL (FP64) is supported");
  datatype = dt;
  n_rhs = nrhs;
  for (auto& kv : elements) {
    std::pair<int, int> d = kv.second.get_n_dof();
    Matrix_& h = kv.second.hm;
    h.fs = d.first;
    h.ss = d.second;
    h.n_rhs = nrhs;
    h.datatype = dt;
    h.created = true;
    h.mesh = this;
    h.elt = &kv.second;
  }
  if (engine) engine->invalidate_plan();
}

// buffers live in the device arena, allocated at the first factorisation
void Mesh_::create_matrix_buffer(int) {}
void Mesh_::create_leaf_matrix_buffer() {}
void Mesh_::create_element_matrix_buffer(int) {}
void Mesh_::free_matrix() {
  for (auto& kv : elements) kv.second.hm.created = false;
  delete engine;
  engine = nullptr;
}

void Mesh_::copy_in(Element elt, int dt, int m, int n, int* nods, int side, void* buffer) {
  copy_in(elt, dt, m, n, UHM_PHYSICS_SINGLE, nods, side, buffer);
}
void Mesh_::copy_in(Element elt, int dt, int m, int n, int nod_disp, int* nods, int side, void* buffer) {
  if (dt != UHM_REAL) throw std::invalid_argument("copy_in: only UHM_REAL is supported");
  eng().copy_in(elt, m, n, nod_disp, nods, side, (const double*)buffer);
}
void Mesh_::copy_out(Element elt, int dt, int m, int n, int* nods, int side, void* buffer) {
  copy_out(elt, dt, m, n, UHM_PHYSICS_SINGLE, nods, side, buffer);
}
void Mesh_::copy_out(Element elt, int dt, int m, int n, int nod_disp, int* nods, int side, void* buffer) {
  if (dt != UHM_REAL) throw std::invalid_argument("copy_out: only UHM_REAL is supported");
  eng().copy_out(elt, m, n, nod_disp, nods, side, (double*)buffer);
}

// ---- Matrix_: the front handle ----------------------------------------------
static bool block_dims(const Matrix_& h, int mat, int& m, int& n) {
  switch (mat) {
    case UHM_ATL: m = h.fs; n = h.fs; return true;
    case UHM_ATR: m = h.fs; n = h.ss; return true;
    case UHM_ABL: m = h.ss; n = h.fs; return true;
    case UHM_ABR: m = h.ss; n = h.ss; return true;
    case UHM_P: m = h.fs; n = 1; return true;
    case UHM_XT: m = h.fs; n = h.n_rhs; return true;
    case UHM_XB: m = h.ss; n = h.n_rhs; return true;
    default: m = n = 0; return false;
  }
}
int Matrix_::is_created(int mat) const {
  int m, n;
  return created && block_dims(*this, mat, m, n) ? 1 : 0;
}
int Matrix_::is_buffer(int mat) const {
  int m, n;
  if (!created || !block_dims(*this, mat, m, n) || !mesh || !mesh->engine) return 0;
  return mesh->engine->front_block_ready(elt, mat) ? 1 : 0;
}
void Matrix_::copy_out(int mat, void* buffer) {
  int m, n;
  if (!created || !mesh || !elt) throw std::invalid_argument("Matrix_::copy_out: the front has no matrix");
  if (!block_dims(*this, mat, m, n)) throw std::invalid_argument("Matrix_::copy_out: block not held by this engine");
  if (!mesh->engine || !mesh->engine->front_block_ready(elt, mat))
    throw std::invalid_argument("Matrix_::copy_out: block not computed yet (factor / solve first)");
  mesh->engine->front_block(elt, mat, buffer);
}
void Matrix_::copy_out(int mat, linal::Flat_ B) {
  int m, n;
  if (!block_dims(*this, mat, m, n)) throw std::invalid_argument("Matrix_::copy_out: block not held by this engine");
  if (mat == UHM_P) throw std::invalid_argument("Matrix_::copy_out: pivots go to an int buffer");
  if (B.get_m() != m || B.get_n() != n) throw std::invalid_argument("Matrix_::copy_out: view of the wrong size");
  std::vector<double> buf((size_t)m * n);
  copy_out(mat, buf.data());
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) B(i, j) = buf[(size_t)j * m + i];
}
bool Matrix_::disp(FILE* stream) {
  std::fprintf(stream, "- uhm::Matrix_ (element %d): fs %d, ss %d, n_rhs %d, %s -\n", elt ? elt->get_id() : -1, fs, ss,
               n_rhs, created ? "created" : "not created");
  return true;
}

// The LINAL-view forms: the (id, physics) pairs as a UHM_PHYSICS_MULTI node
// list, the view copied through a contiguous buffer when its leading
// dimension is not its row count.
static std::vector<int> pair_list(const std::vector<std::pair<int, int>>& nods) {
  std::vector<int> v;
  v.reserve(2 * nods.size());
  for (const auto& p : nods) {
    v.push_back(p.first);
    v.push_back(p.second);
  }
  return v;
}

void Mesh_::copy_in(Element elt, std::vector<std::pair<int, int>>& nods, int side, linal::Flat_ A) {
  if (A.get_data_type() != UHM_REAL) throw std::invalid_argument("copy_in: only UHM_REAL views are supported");
  const int m = A.get_m(), n = side == UHM_LHS ? A.get_m() : A.get_n();
  if (side == UHM_LHS && A.get_n() != m) throw std::invalid_argument("copy_in: element matrix view is not square");
  std::vector<int> ids = pair_list(nods);
  std::vector<double> buf((size_t)m * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) buf[(size_t)j * m + i] = A(i, j);
  copy_in(elt, UHM_REAL, m, n, UHM_PHYSICS_MULTI, ids.data(), side, buf.data());
}

void Mesh_::copy_out(Element elt, std::vector<std::pair<int, int>>& nods, int side, linal::Flat_ B) {
  if (B.get_data_type() != UHM_REAL) throw std::invalid_argument("copy_out: only UHM_REAL views are supported");
  const int m = B.get_m(), n = B.get_n();
  std::vector<int> ids = pair_list(nods);
  std::vector<double> buf((size_t)m * n);
  copy_out(elt, UHM_REAL, m, n, UHM_PHYSICS_MULTI, ids.data(), side, buf.data());
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) B(i, j) = buf[(size_t)j * m + i];
}

// matrix.cxx:54-62: the right-hand side is taken from the element rhs at solve time
void Mesh_::set_rhs() {}

void Mesh_::run_factor(int method, int) { eng().factor(method); }
void Mesh_::run_solve(int method, int phase) { eng().solve(method, phase); }

void Mesh_::chol_with_free() { run_factor(UHM_CHOL, 0); }
void Mesh_::chol_without_free() { run_factor(UHM_CHOL, 1); }
void Mesh_::solve_chol_1() { run_solve(UHM_CHOL, 1); }
void Mesh_::solve_chol_2() { run_solve(UHM_CHOL, 2); }
void Mesh_::solve_chol() { run_solve(UHM_CHOL, 3); }
void Mesh_::check_chol() {}
void Mesh_::lu_nopiv_with_free() { run_factor(UHM_LU_NOPIV, 0); }
void Mesh_::lu_nopiv_without_free() { run_factor(UHM_LU_NOPIV, 1); }
void Mesh_::solve_lu_nopiv_1() { run_solve(UHM_LU_NOPIV, 1); }
void Mesh_::solve_lu_nopiv_2() { run_solve(UHM_LU_NOPIV, 2); }
void Mesh_::solve_lu_nopiv() { run_solve(UHM_LU_NOPIV, 3); }
void Mesh_::check_lu_nopiv() {}
void Mesh_::lu_piv_with_free() { run_factor(UHM_LU_PIV, 0); }
void Mesh_::lu_piv_without_free() { run_factor(UHM_LU_PIV, 1); }
void Mesh_::solve_lu_piv_1() { run_solve(UHM_LU_PIV, 1); }
void Mesh_::solve_lu_piv_2() { run_solve(UHM_LU_PIV, 2); }
void Mesh_::solve_lu_piv() { run_solve(UHM_LU_PIV, 3); }
void Mesh_::check_lu_piv() {}
void Mesh_::lu_incpiv_with_free() { run_factor(UHM_LU_PIV, 0); }
void Mesh_::lu_incpiv_without_free() { run_factor(UHM_LU_PIV, 1); }
void Mesh_::random_spd_matrix() { eng().random_elements(1); }
void Mesh_::random_matrix() { eng().random_elements(0); }
void Mesh_::triangularize() {}
static void no_qr() { throw std::invalid_argument("QR fronts are not provided by this library"); }
void Mesh_::qr_with_free() { no_qr(); }
void Mesh_::qr_without_free() { no_qr(); }
void Mesh_::solve_qr_1() { no_qr(); }
void Mesh_::solve_qr_2() { no_qr(); }
void Mesh_::solve_qr() { no_qr(); }
void Mesh_::check_qr() { no_qr(); }
void Mesh_::qr_with_ooc() { no_qr(); }
void Mesh_::check_qr_1() { no_qr(); }
void Mesh_::check_qr_2() { no_qr(); }
void Mesh_::improve_qr() {}
void Mesh_::chol_with_ooc() { run_factor(UHM_CHOL, 0); }
void Mesh_::solve_chol_1_ooc() { run_solve(UHM_CHOL, 1); }
void Mesh_::solve_chol_2_ooc() { run_solve(UHM_CHOL, 2); }
void Mesh_::solve_chol_ooc() { run_solve(UHM_CHOL, 3); }
void Mesh_::check_chol_1() {}
void Mesh_::check_chol_2() {}
void Mesh_::improve_chol() {}
void Mesh_::lu_nopiv_with_ooc() { run_factor(UHM_LU_NOPIV, 0); }
void Mesh_::solve_lu_nopiv_1_ooc() { run_solve(UHM_LU_NOPIV, 1); }
void Mesh_::solve_lu_nopiv_2_ooc() { run_solve(UHM_LU_NOPIV, 2); }
void Mesh_::solve_lu_nopiv_ooc() { run_solve(UHM_LU_NOPIV, 3); }
void Mesh_::check_lu_nopiv_1() {}
void Mesh_::check_lu_nopiv_2() {}
void Mesh_::improve_lu_nopiv() {}
void Mesh_::lu_piv_with_ooc() { run_factor(UHM_LU_PIV, 0); }
void Mesh_::lu_incpiv_with_ooc() { run_factor(UHM_LU_PIV, 0); }
void Mesh_::solve_lu_piv_1_ooc() { run_solve(UHM_LU_PIV, 1); }
void Mesh_::solve_lu_piv_2_ooc() { run_solve(UHM_LU_PIV, 2); }
void Mesh_::solve_lu_piv_ooc() { run_solve(UHM_LU_PIV, 3); }
void Mesh_::check_lu_piv_1() {}
void Mesh_::check_lu_piv_2() {}
void Mesh_::check_lu_piv_1_ooc() {}
void Mesh_::check_lu_piv_2_ooc() {}
void Mesh_::check_lu_piv_ooc() {}
void Mesh_::improve_lu_piv() {}
void Mesh_::improve_lu_piv_ooc() {}

// The reference returns sum over fronts of ||rt||_1 of its factor-based
// check (UHM/src/matrix/uhm/fla/matrix.cxx:222-234); here: ||b - A x||_1 of
// the true residual on the unassembled element matrices.
double Mesh_::get_residual() { return eng().residual_norm1(); }

unsigned Mesh_::get_n_dof() {
  unsigned n = 0;
  for (auto& kv : elements) n += kv.second.get_n_dof().first;
  return n;
}
unsigned Mesh_::get_n_nonzero() {
  unsigned n = 0;
  for (auto& kv : elements)
    if (kv.second.is_leaf()) {
      std::pair<int, int> d = kv.second.get_n_dof();
      n += (d.first + d.second) * (d.first + d.second);
    }
  return n;
}
unsigned Mesh_::get_n_nonzero_factor() {
  unsigned n = 0;
  for (auto& kv : elements) {
    std::pair<int, int> d = kv.second.get_n_dof();
    n += d.first * d.first + d.first * d.second * 2;
  }
  return n;
}
void Mesh_::estimate_cost(int method, int dt, int nrhs, double& dec, double& sol, unsigned& nnz,
                          double& buffer) {
  dec = sol = buffer = 0;
  nnz = 0;
  for (auto& kv : elements) {
    double a, b, c;
    unsigned z;
    kv.second.estimate_cost(method, dt, nrhs, a, b, z, c);
    dec += a;
    sol += b;
    nnz += z;
    buffer += c;
  }
}

}  // namespace uhm
