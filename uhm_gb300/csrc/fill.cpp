// Pseudo-random element matrices for benchmarks and tests without an
// application: the reference's Mesh_::random_spd_matrix / random_matrix
// (UHM/src/mesh/matrix.cxx:155-170,295-310) fill every leaf front's blocks
// through libflame's generator, whose values cannot be reproduced here.
// These give the same use -- a solvable system of the mesh's shape -- with
// their own generator (splitmix64, Steele, Lea and Flood 2014):
//   spd:  A_e = (R + R^T) / 2 + 2 m I   (symmetric, strictly diagonally
//         dominant with a positive diagonal, hence SPD; so is the sum)
//   else: A_e = R + 2 m I               (strictly diagonally dominant)
// R uniform in [-1, 1), m the element's rows; right-hand sides uniform in
// [-1, 1).  Rows follow each element's nodes in node-id order, unless node
// lists were given before (copy_in / uhm_gpu_set_leaf_nodes).
#include "engine.hpp"

#include <cstring>

namespace uhm {

namespace {
struct SplitMix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (2.0 / 9007199254740992.0) - 1.0; }
};
}  // namespace

void Engine::random_elements(int spd) {
  ensure_plan();
  SplitMix64 g{0x5EED0000ULL + random_calls++};
  const int nr = mesh->n_rhs;
  for (auto& es : esrc) {
    if (es.node_order.empty()) {
      std::vector<int> nods;
      for (auto& kv : es.e->nodes) {
        nods.push_back(kv.first->get_id().first);
        nods.push_back(kv.first->get_id().second);
      }
      std::vector<std::pair<int, int>> order;
      std::vector<int> pos;
      std::vector<int32_t> gd;
      element_map(es.e, UHM_PHYSICS_MULTI, nods.data(), order, pos, gd);
      if ((int)pos.size() != es.m) fail("random matrix: element size mismatch", 7);
      es.node_order = order;
      es.pos = pos;
      es.gdof = gd;
      dev_ok = false;   // element maps are part of the device plan
    }
    const int m = es.m;
    double* A = h_pinned + es.mat_off;
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) A[i + (int64_t)j * m] = g.uniform();
    if (spd)
      for (int j = 0; j < m; ++j)
        for (int i = j + 1; i < m; ++i) {
          const double v = 0.5 * (A[i + (int64_t)j * m] + A[j + (int64_t)i * m]);
          A[i + (int64_t)j * m] = v;
          A[j + (int64_t)i * m] = v;
        }
    for (int i = 0; i < m; ++i) A[i + (int64_t)i * m] += 2.0 * m;
    double* B = h_pinned + emat_total + es.rhs_off;
    for (int64_t k = 0; k < (int64_t)m * nr; ++k) B[k] = g.uniform();
    es.has_lhs = es.has_rhs = true;
  }
  std::fill(leaf_changed.begin(), leaf_changed.end(), 1);
  emat_dirty = erhs_dirty = true;
  emat_device_only = erhs_device_only = false;
  anorm_valid = false;
  anorm_inf = -1.0;
  learned_valid = false;
  factored = false;
}

}  // namespace uhm
