// Sparse export of the assembled operator (the reference's DSparse_,
// UHM/src/interf/sparse.cxx:188-460), for comparisons with external sparse
// solvers.  Host code: element matrices come from the engine's staging copy
// (fetched from the device first when they only exist there).
//
// The reference adds element matrices into a std::map keyed by (row, col):
// the first contribution inserts, later ones add (axpy) in import order.
// Here every (key, value, leaf) contribution is listed in leaf order, sorted
// by key with a stable sort, and summed front to back: the same sums in the
// same order, so the values are bit-identical to the map's.
#include "engine.hpp"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>

namespace uhm {

static void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void Engine::export_sparse(int is_sym, int fort, int cs, int compress, int axpy, SparseOut& out) {
  ensure_plan();
  // the operator needs every element matrix; the right-hand sides are
  // exported when every leaf has one (the reference takes what is there)
  bool with_rhs = true;
  for (auto& es : esrc) {
    if (!es.has_lhs) fail("export_sparse: an element matrix has not been copied in", 7);
    with_rhs = with_rhs && es.has_rhs;
  }
  if (dev_ok && emat_device_only) {
    ck(cudaStreamSynchronize(stream), "export_sparse: sync");
    ck(cudaMemcpy(h_pinned, ctx.emat, sizeof(double) * (size_t)emat_total, cudaMemcpyDeviceToHost),
       "export_sparse: element matrices");
    emat_device_only = false;
  }
  if (with_rhs && dev_ok && erhs_device_only) {
    ck(cudaStreamSynchronize(stream), "export_sparse: sync");
    ck(cudaMemcpy(h_pinned + emat_total, d_erhs, sizeof(double) * (size_t)erhs_total, cudaMemcpyDeviceToHost),
       "export_sparse: right-hand sides");
    erhs_device_only = false;
  }
  const int nr = mesh->n_rhs;
  const int shift = fort ? 1 : 0;
  // (key, value) of every contribution, leaf order, then column-major within the element
  struct Entry {
    int k0, k1;
    double v;
  };
  auto reduce = [&](std::vector<Entry>& ent) {
    std::vector<size_t> ord(ent.size());
    std::iota(ord.begin(), ord.end(), size_t(0));
    std::stable_sort(ord.begin(), ord.end(), [&](size_t x, size_t y) {
      return ent[x].k0 != ent[y].k0 ? ent[x].k0 < ent[y].k0 : ent[x].k1 < ent[y].k1;
    });
    std::vector<Entry> red;
    red.reserve(ent.size() / 2 + 1);
    for (size_t t : ord) {
      const Entry& e = ent[t];
      if (!red.empty() && red.back().k0 == e.k0 && red.back().k1 == e.k1) {
        if (axpy) red.back().v += e.v;
      } else {
        red.push_back(e);
      }
    }
    return red;
  };
  std::vector<Entry> ea, eb;
  size_t na = 0, nb = 0;
  for (auto& es : esrc) {
    na += (size_t)es.m * es.m;
    nb += (size_t)es.m * nr;
  }
  ea.reserve(na);
  eb.reserve(nb);
  for (auto& es : esrc) {
    const double* A = h_pinned + es.mat_off;
    const double* B = h_pinned + emat_total + es.rhs_off;
    for (int j = 0; j < es.m; ++j)
      for (int i = 0; i < es.m; ++i) {
        const int r = es.gdof[i] + shift, c = es.gdof[j] + shift;
        ea.push_back(cs ? Entry{c, r, A[i + (int64_t)j * es.m]} : Entry{r, c, A[i + (int64_t)j * es.m]});
      }
    // right-hand sides keyed (rhs column, row): a column-major vector
    for (int q = 0; q < (with_rhs ? nr : 0); ++q)
      for (int i = 0; i < es.m; ++i) eb.push_back(Entry{q + shift, es.gdof[i] + shift, B[i + (int64_t)q * es.m]});
  }
  std::vector<Entry> a = reduce(ea), b = reduce(eb);
  ea.clear();
  ea.shrink_to_fit();
  out = SparseOut{};
  out.n_rhs = with_rhs ? nr : 0;
  // sparse.cxx:269-330 (triplet) and 332-460 (compress)
  int prev = a.empty() ? 0 : a.front().k0;
  int cnt = shift;
  std::vector<int>& ptr = cs ? out.ja : out.ia;   // compressed: pointers on the key's major index
  std::vector<int>& idx = cs ? out.ia : out.ja;
  if (compress) ptr.push_back(cnt);
  for (const Entry& e : a) {
    if (is_sym && !(e.k1 >= e.k0)) continue;
    if (compress) {
      if (e.k0 != prev) {
        ptr.push_back(cnt);
        prev = e.k0;
      }
      ++cnt;
      idx.push_back(e.k1);
    } else {
      // rows in ia, columns in ja (the key is (col, row) when cs)
      out.ia.push_back(cs ? e.k1 : e.k0);
      out.ja.push_back(cs ? e.k0 : e.k1);
    }
    out.a.push_back(e.v);
  }
  if (compress) {
    out.n_dof = out.a.empty() ? 0 : (int)ptr.size();
    if (!out.a.empty()) ptr.push_back(cnt);
  } else {
    out.n_dof = (int)n_global;
  }
  out.b.reserve(b.size());
  for (const Entry& e : b) out.b.push_back(e.v);
}

}  // namespace uhm
