// A C++ caller of uhm::Mesh_ through uhm_gb300/csrc/mesh.hpp, written as a
// user of the reference's C++ interface writes it (the free functions and
// the Mesh_ / Element_ calls of UHM/example/cxx/ex1.cxx, in its order): two
// elements of seven nodes sharing three, uhm::build_tree, lock, copy_in of a
// pseudo-random element matrix and right-hand side into both.
//
// usage: two_elements_cxx   prints the mesh's sizes after copy_in (host only)
#include <cstdio>
#include <vector>

#include "mesh.hpp"

int main() {
  uhm::set_num_threads(2);
  uhm::set_hier_block_size(128);
  uhm::Mesh m = new uhm::Mesh_;
  int nods[2][7] = {{3, 4, 5, 7, 9, 8, 1}, {4, 6, 5, 10, 11, 9, 2}};
  const int node_dof[7] = {1, 1, 1, 3, 3, 3, 3};
  uhm::Element e[2];
  for (int j = 0; j < 2; ++j) {
    e[j] = m->add_element();
    for (int i = 0; i < 7; ++i) e[j]->add_node(m->add_node(nods[j][i], node_dof[i]));
  }
  uhm::build_tree(m);
  const int n_elements = m->get_n_elements();
  m->lock();
  const unsigned n_dof = m->get_n_dof();
  m->create_matrix_without_buffer(uhm::UHM_REAL, 1);
  m->create_matrix_buffer(0);
  std::vector<double> A(15 * 15), B(15);
  unsigned long long s = 7;
  for (double& v : A) v = (double)((s = s * 6364136223846793005ULL + 1ULL) >> 11) / 9007199254740992.0;
  for (double& v : B) v = (double)((s = s * 6364136223846793005ULL + 1ULL) >> 11) / 9007199254740992.0;
  for (int j = 0; j < 2; ++j) {
    m->copy_in(e[j], uhm::UHM_REAL, 15, 15, nods[j], uhm::UHM_LHS, A.data());
    m->copy_in(e[j], uhm::UHM_REAL, 15, 1, nods[j], uhm::UHM_RHS, B.data());
  }
  m->set_rhs();
  double fd = 0, fs = 0, buf = 0;
  unsigned nnz = 0;
  m->estimate_cost(uhm::UHM_LU_PIV, uhm::UHM_REAL, 1, fd, fs, nnz, buf);
  std::printf("n_elements %d\nn_dof %u\nthreads %d\nblock %d\nflop_decompose %.17g\n", n_elements, n_dof,
              uhm::get_num_threads(), uhm::get_hier_block_size(), fd);
  m->unlock();
  delete m;
  return 0;
}
