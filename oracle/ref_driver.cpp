// Runs the reference's CPU multifrontal solver (built by oracle/Makefile) on a
// mesh read from a binary file and writes the solution and the front
// structure.  TEST INFRASTRUCTURE: used only to pin the oracle and to produce
// the golden fixtures (tests/golden/make_golden.py).
//
// The call sequence is the reference's documented workflow
// (UHM/example/cxx/ex1.cxx): add_element / add_node, explicit tree through
// add_element(gen) + add_child + set_parent (as UHM/src/operation/
// build_tree_var1.cxx:158-161 does), lock, create_matrix_without_buffer,
// copy_in of every leaf matrix and right-hand side, set_rhs, factor, solve,
// copy_out of the solution.
//
// usage: uhm_ref_driver IN OUT [n_threads] [sparse | reps]
//
// With a number reps > 1 the factorisation and solve are repeated: before
// each repetition after the first the front matrices are freed and created
// again (free_matrix, create_matrix_without_buffer) and every leaf matrix and
// right-hand side is copied in again, so each repetition does the whole
// numeric work of the first.  The solution written is the last one's; the
// time of every repetition follows the tail (see OUT).
//
// With "sparse" the driver stops after copy_in and instead writes the
// reference's own sparse export of the leaves (DSparse_(fort 0, cs 0,
// n_rhs): import_element of every leaf in input order, then triplet with
// is_sym = 0; UHM/src/interf/sparse.cxx:196-330):
//     "UHMP" int32 version=1, int32 n_nodes; per node (input order) int32
//     its first global dof (Node_::get_offset); int32 n_dof (triplet's),
//     n_rhs, n_nz; int32 ia[n_nz], ja[n_nz]; float64 a[n_nz];
//     int32 n_b; float64 b[n_b]
//
// IN  (little-endian): "UHMS" int32 version=1
//     int32 n_nodes; per node int32 id, n_dof, p, kind
//     int32 n_elements, n_leaves, n_rhs, method (1 chol, 2 lu_nopiv, 3 lu_piv,
//     4 lu_incpiv: factored by lu_incpiv_with_free, solved by solve_lu_piv as
//     the reference's Fortran flow does)
//     int32 generation[n_elements]; int32 child_ptr[n_elements+1];
//     int32 child_idx[child_ptr[n_elements]] (children in add_child order)
//     int32 elem_ptr[n_leaves+1]; int32 elem_node[elem_ptr[n_leaves]]
//     per leaf: float64 A[m*m] (column-major), float64 B[m*n_rhs]
// OUT: "UHMR" int32 version=1
//     int32 n_nodes, n_rhs; per node (input order) float64 x[n_dof*n_rhs]
//     (node-major, rhs-minor); int32 n_elements; per element (input order)
//     int32 n_factor, n_schur; float64 t_factor, t_solve (seconds),
//     flop_decompose, flop_solve, t_lock (seconds, the symbolic phase);
//     int32 reps; per repetition float64 t_factor, t_solve
#include "uhm.hxx"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>
#include <sys/time.h>

static double now() {
  timeval tv;
  gettimeofday(&tv, 0);
  return tv.tv_sec + 1e-6 * tv.tv_usec;
}

static void fail(const char* what) {
  std::fprintf(stderr, "uhm_ref_driver: %s\n", what);
  std::exit(2);
}

struct Reader {
  FILE* f;
  int i32() {
    int v;
    if (std::fread(&v, 4, 1, f) != 1) fail("short read");
    return v;
  }
  void f64(double* p, size_t n) {
    if (n && std::fread(p, 8, n, f) != n) fail("short read");
  }
};

int main(int argc, char** argv) {
  if (argc < 3) fail("usage: uhm_ref_driver IN OUT [n_threads]");
  FILE* fin = std::fopen(argv[1], "rb");
  if (!fin) fail("cannot open input");
  Reader r = {fin};
  char magic[4];
  if (std::fread(magic, 1, 4, fin) != 4 || std::memcmp(magic, "UHMS", 4)) fail("bad magic");
  if (r.i32() != 1) fail("bad version");

  FLA_Init();
  uhm::set_num_threads(argc > 3 ? std::atoi(argv[3]) : 1);
  uhm::Mesh m = new uhm::Mesh_;

  const int n_nodes = r.i32();
  std::vector<int> nid(n_nodes), ndof(n_nodes);
  std::map<int, int> node_index;
  for (int i = 0; i < n_nodes; ++i) {
    nid[i] = r.i32();
    ndof[i] = r.i32();
    const int p = r.i32(), kind = r.i32();
    m->add_node(std::pair<int, int>(nid[i], 0), ndof[i], p, kind);
    node_index[nid[i]] = i;
  }
  const int n_el = r.i32(), n_leaves = r.i32(), n_rhs = r.i32(), method = r.i32();
  std::vector<int> gen(n_el), cptr(n_el + 1), eptr(n_leaves + 1);
  for (int e = 0; e < n_el; ++e) gen[e] = r.i32();
  for (int e = 0; e <= n_el; ++e) cptr[e] = r.i32();
  std::vector<int> cidx(cptr[n_el]);
  for (size_t k = 0; k < cidx.size(); ++k) cidx[k] = r.i32();
  for (int e = 0; e <= n_leaves; ++e) eptr[e] = r.i32();
  std::vector<int> enode(eptr[n_leaves]);
  for (size_t k = 0; k < enode.size(); ++k) enode[k] = r.i32();

  std::vector<uhm::Element> elt(n_el);
  for (int e = 0; e < n_el; ++e) elt[e] = m->add_element(gen[e]);
  for (int e = 0; e < n_leaves; ++e)
    for (int k = eptr[e]; k < eptr[e + 1]; ++k)
      elt[e]->add_node(m->find_node(std::pair<int, int>(enode[k], 0)));
  for (int e = 0; e < n_el; ++e)
    for (int k = cptr[e]; k < cptr[e + 1]; ++k) {
      elt[e]->add_child(elt[cidx[k]]);
      elt[cidx[k]]->set_parent(elt[e]);
    }

  const double tl0 = now();
  m->lock();
  const double t_lock = now() - tl0;
  m->create_matrix_without_buffer(UHM_REAL, n_rhs);

  const bool sparse_mode = argc > 4 && !std::strcmp(argv[4], "sparse");
  const int reps = (argc > 4 && !sparse_mode && std::atoi(argv[4]) > 1) ? std::atoi(argv[4]) : 1;
  std::vector<int> elem_m(n_leaves);
  std::vector<std::vector<double> > As(n_leaves), Bs(n_leaves);
  for (int e = 0; e < n_leaves; ++e) {
    int msz = 0;
    for (int k = eptr[e]; k < eptr[e + 1]; ++k) msz += ndof[node_index[enode[k]]];
    elem_m[e] = msz;
    std::vector<double> A((size_t)msz * msz), B((size_t)msz * n_rhs);
    r.f64(A.data(), A.size());
    r.f64(B.data(), B.size());
    if (msz == 0) continue;
    m->copy_in(elt[e], UHM_REAL, msz, msz, &enode[eptr[e]], UHM_LHS, (void*)A.data());
    m->copy_in(elt[e], UHM_REAL, msz, n_rhs, &enode[eptr[e]], UHM_RHS, (void*)B.data());
    if (reps > 1) {
      As[e].swap(A);
      Bs[e].swap(B);
    }
  }
  std::fclose(fin);
  m->set_rhs();

  if (sparse_mode) {
    uhm::DSparse_ sp(0, 0, n_rhs);
    for (int e = 0; e < n_leaves; ++e)
      if (elem_m[e]) sp.import_element(elt[e]);
    int sd = 0, sr = 0, snz = 0;
    std::vector<int> ia, ja;
    std::vector<double> a, b;
    sp.triplet(0, sd, sr, snz, ia, ja, a, b);
    FILE* fo = std::fopen(argv[2], "wb");
    if (!fo) fail("cannot open output");
    int hdr[2] = {1, n_nodes};
    std::fwrite("UHMP", 1, 4, fo);
    std::fwrite(hdr, 4, 2, fo);
    for (int i = 0; i < n_nodes; ++i) {
      int o = m->find_node(std::pair<int, int>(nid[i], 0))->get_offset();
      std::fwrite(&o, 4, 1, fo);
    }
    int t[3] = {sd, sr, snz};
    std::fwrite(t, 4, 3, fo);
    std::fwrite(ia.data(), 4, ia.size(), fo);
    std::fwrite(ja.data(), 4, ja.size(), fo);
    std::fwrite(a.data(), 8, a.size(), fo);
    int nb = (int)b.size();
    std::fwrite(&nb, 4, 1, fo);
    std::fwrite(b.data(), 8, b.size(), fo);
    std::fclose(fo);
    delete m;
    FLA_Finalize();
    return 0;
  }

  double fd = 0, fs = 0, buf = 0;
  unsigned int nnz = 0;
  m->estimate_cost(method, UHM_REAL, n_rhs, fd, fs, nnz, buf);

  std::vector<double> rep_times;
  double t0 = 0, t1 = 0, t2 = 0;
  for (int rep = 0; rep < reps; ++rep) {
    if (rep > 0) {
      m->free_matrix();
      m->create_matrix_without_buffer(UHM_REAL, n_rhs);
      for (int e = 0; e < n_leaves; ++e) {
        const int msz = elem_m[e];
        if (msz == 0) continue;
        m->copy_in(elt[e], UHM_REAL, msz, msz, &enode[eptr[e]], UHM_LHS, (void*)As[e].data());
        m->copy_in(elt[e], UHM_REAL, msz, n_rhs, &enode[eptr[e]], UHM_RHS, (void*)Bs[e].data());
      }
      m->set_rhs();
    }
    t0 = now();
    if (method == 1) m->chol_with_free();
    else if (method == 2) m->lu_nopiv_with_free();
    else if (method == 3) m->lu_piv_with_free();
    else if (method == 4) m->lu_incpiv_with_free();
    else fail("unknown method");
    t1 = now();
    if (method == 1) m->solve_chol();
    else if (method == 2) m->solve_lu_nopiv();
    else m->solve_lu_piv();
    t2 = now();
    rep_times.push_back(t1 - t0);
    rep_times.push_back(t2 - t1);
  }

  // solution per node, taken from the first leaf element that holds the node
  std::vector<std::vector<double> > x(n_nodes);
  for (int e = 0; e < n_leaves; ++e) {
    const int msz = elem_m[e];
    if (msz == 0) continue;
    std::vector<double> B((size_t)msz * n_rhs);
    m->copy_out(elt[e], UHM_REAL, msz, n_rhs, &enode[eptr[e]], UHM_RHS, (void*)B.data());
    int row = 0;
    for (int k = eptr[e]; k < eptr[e + 1]; ++k) {
      const int i = node_index[enode[k]];
      if (x[i].empty() && ndof[i]) {
        x[i].resize((size_t)ndof[i] * n_rhs);
        for (int d = 0; d < ndof[i]; ++d)
          for (int c = 0; c < n_rhs; ++c) x[i][(size_t)d * n_rhs + c] = B[(row + d) + (size_t)c * msz];
      }
      row += ndof[i];
    }
  }

  FILE* fo = std::fopen(argv[2], "wb");
  if (!fo) fail("cannot open output");
  int hdr[2] = {1, n_nodes};
  std::fwrite("UHMR", 1, 4, fo);
  std::fwrite(hdr, 4, 2, fo);
  std::fwrite(&n_rhs, 4, 1, fo);
  for (int i = 0; i < n_nodes; ++i) {
    if (ndof[i] && x[i].empty()) fail("node without solution");
    if (ndof[i]) std::fwrite(x[i].data(), 8, x[i].size(), fo);
  }
  std::fwrite(&n_el, 4, 1, fo);
  for (int e = 0; e < n_el; ++e) {
    std::pair<int, int> nd = elt[e]->get_n_dof();
    int v[2] = {nd.first, nd.second};
    std::fwrite(v, 4, 2, fo);
  }
  double tail[5] = {t1 - t0, t2 - t1, fd, fs, t_lock};
  std::fwrite(tail, 8, 5, fo);
  std::fwrite(&reps, 4, 1, fo);
  std::fwrite(rep_times.data(), 8, rep_times.size(), fo);
  std::fclose(fo);
  delete m;
  FLA_Finalize();
  return 0;
}
