// Element data handed over as LINAL views (the pair-list forms of
// Mesh_::copy_in / copy_out, UHM/include/uhm/mesh/mesh.hxx:181-184,
// 194-197): the element matrix is a 15 x 15 view at (2, 3) of a 20 x 20
// Flat_ (leading dimension 20), the right-hand side a view of one column of
// a 15 x 4 Flat_, and the solution is copied out into another view.  A Hier_
// of 8 x 8 blocks over the big Flat_ checks the block views.  Prints the
// numbers the test compares.
#include "uhm.hxx"

#include <cstdio>
#include <utility>
#include <vector>

int main(int argc, char**) {
  const bool solve = argc > 1;            // without a GPU only the set-up runs
  FLA_Init();
  uhm::Mesh m = new uhm::Mesh_;
  int elt[2][7] = {{3, 4, 5, 7, 9, 8, 1}, {4, 6, 5, 10, 11, 9, 2}};
  int ndof[7] = {1, 1, 1, 3, 3, 3, 3};
  uhm::Element e[2];
  for (int j = 0; j < 2; ++j) {
    e[j] = m->add_element();
    for (int i = 0; i < 7; ++i) e[j]->add_node(m->add_node(elt[j][i], ndof[i]));
  }
  uhm::build_tree(m);
  m->lock();
  m->create_matrix_without_buffer(UHM_REAL, 1);

  linal::Flat_ big, rhs, sol;
  big.create(UHM_REAL, 20, 20);
  rhs.create(UHM_REAL, 15, 4);
  sol.create(UHM_REAL, 15, 3);
  FLA_Random_matrix(~big);
  FLA_Random_matrix(~rhs);
  linal::Flat_ A, b, x;
  big.extract(A, 15, 15, 2, 3);
  rhs.extract(b, 15, 1, 0, 2);
  sol.extract(x, 15, 1, 0, 1);

  linal::Hier_ H;
  H.create(big, 8, 8);
  linal::Flat_ whole = H.flat();
  std::printf("hier %d %d last %d %d whole %d %d same %d\n", H.get_m(), H.get_n(), H(2, 2).m, H(2, 2).n,
              whole.get_m(), whole.get_n(), whole.get_buffer() == big.get_buffer() ? 1 : 0);

  for (int j = 0; j < 2; ++j) {
    std::vector<std::pair<int, int>> nods;
    for (int i = 0; i < 7; ++i) nods.push_back(std::make_pair(elt[j][i], 0));
    m->copy_in(e[j], nods, UHM_LHS, A);
    m->copy_in(e[j], nods, UHM_RHS, b);
  }
  m->set_rhs();
  if (solve) {
    m->lu_piv_with_free();
    m->solve_lu_piv();
    for (int j = 0; j < 2; ++j) {
      std::vector<std::pair<int, int>> nods;
      for (int i = 0; i < 7; ++i) nods.push_back(std::make_pair(elt[j][i], 0));
      m->copy_out(e[j], nods, UHM_RHS, x);
      std::printf("solution %d", j);
      for (int i = 0; i < 15; ++i) std::printf(" %.17g", x(i, 0));
      std::printf("\n");
    }
  }
  big.free();
  rhs.free();
  sol.free();
  delete m;
  FLA_Finalize();
  return 0;
}
