// The reference's automatic tree builder (UHM/src/operation/build_tree_var4.cxx)
// needs METIS, which is not available.  The oracle builds every assembly tree
// explicitly through the Mesh API, so the builder is replaced by a stub that
// aborts if anything calls it.  TEST INFRASTRUCTURE.
#include <cstdio>
#include <cstdlib>

namespace uhm {
class Mesh_;
bool build_tree_var_4(Mesh_*) {
  std::fprintf(stderr, "oracle build: automatic tree building (METIS) is not available\n");
  std::abort();
  return false;
}
}  // namespace uhm
