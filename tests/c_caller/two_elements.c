/* A C caller of the Fortran-style interface (include/uhm_gb300.h) making the
 * calls of the reference's two-element example (UHM/example/f90/ex1.f90) in
 * its order: two elements of seven nodes that share three, the tree from
 * uhm_build_tree_, the same pseudo-random element matrix and right-hand side
 * copied into both, LU with partial pivoting, the solution copied out.
 *
 * usage: two_elements [host|full]
 *   host  stop after copy_in (needs no device): print n_dof and the status
 *   full  also factor, solve, residual and copy_out: print the solution
 *
 * The numbers come from a 64-bit linear congruential generator (Knuth's
 * MMIX multiplier and increment, top 53 bits), seed 100. */
#include <stdio.h>
#include <string.h>

#include "uhm_gb300.h"

static unsigned long long lcg = 100ULL;

static double next_uniform(void) {
  lcg = lcg * 6364136223846793005ULL + 1442695040888963407ULL;
  return (double)(lcg >> 11) * (1.0 / 9007199254740992.0);
}

int main(int argc, char** argv) {
  const int full = argc > 1 && strcmp(argv[1], "full") == 0;
  int elt_nodes[2][7] = {{3, 4, 5, 7, 9, 8, 1}, {4, 6, 5, 10, 11, 9, 2}};
  const int node_dof[7] = {1, 1, 1, 3, 3, 3, 3};
  int datatype = UHM_REAL, n_rhs = 1, m = 15, is_schur = 0, disp = UHM_PHYSICS_SINGLE;
  int lhs = UHM_LHS, rhs = UHM_RHS, n_dof = 0, i, j;
  long mesh = 0, elt[2], nod = 0;
  double A[15 * 15], B[15];

  uhm_initialize_fla_();
  uhm_mesh_create_(&mesh);
  for (j = 0; j < 2; ++j) {
    uhm_add_element_(&mesh, &elt[j]);
    for (i = 0; i < 7; ++i) {
      int id = elt_nodes[j][i], phy = 0, nd = node_dof[i], p = node_dof[i];
      uhm_add_node_(&mesh, &id, &phy, &nd, &p, &nod);
      uhm_element_add_node_(&elt[j], &nod);
    }
  }
  uhm_build_tree_(&mesh);
  uhm_lock_(&mesh);
  uhm_get_n_dof_(&mesh, &n_dof);
  uhm_create_matrix_without_buffer_(&mesh, &datatype, &n_rhs);
  uhm_create_element_matrix_buffer_(&mesh, &is_schur);
  for (i = 0; i < 15 * 15; ++i) A[i] = next_uniform();
  for (i = 0; i < 15; ++i) B[i] = next_uniform();
  for (j = 0; j < 2; ++j) {
    uhm_copy_in_(&mesh, &elt[j], &datatype, &m, &m, &disp, elt_nodes[j], &lhs, A);
    uhm_copy_in_(&mesh, &elt[j], &datatype, &m, &n_rhs, &disp, elt_nodes[j], &rhs, B);
  }
  uhm_set_rhs_(&mesh);
  printf("n_dof %d\nstatus %d\n", n_dof, uhm_gpu_get_status(&mesh));
  if (full) {
    double res = -1.0;
    uhm_lu_piv_with_free_(&mesh);
    uhm_solve_lu_piv_(&mesh);
    uhm_check_lu_piv_(&mesh);
    uhm_get_residual_(&mesh, &res);
    printf("solve_status %d\nresidual %.17g\n", uhm_gpu_get_status(&mesh), res);
    for (j = 0; j < 2; ++j) {
      uhm_copy_out_(&mesh, &elt[j], &datatype, &m, &n_rhs, &disp, elt_nodes[j], &rhs, B);
      for (i = 0; i < 15; ++i) printf("x %d %d %.17g\n", j, i, B[i]);
    }
  }
  uhm_unlock_(&mesh);
  uhm_mesh_delete_(&mesh);
  uhm_finalize_fla_();
  return 0;
}
