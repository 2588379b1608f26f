// The C++ interface of this library under the reference's umbrella header
// name (UHM/include/uhm.hxx): a program written against the reference's
// uhm::Mesh_ / Element_ / Node_ objects and LINAL's Flat_ / Hier_ views (for
// example the call sequence of the reference's C++ example) compiles against
// this header with only the include path changed, and links
// libuhm_gb300.so.
//
//   uhm::Mesh_, Element_, Node_, build_tree, set_num_threads, ...   mesh.hpp
//   linal::Flat_, Hier_, and the FLAME object subset they use        linal.hpp
#ifndef UHM_GB300_UHM_HXX
#define UHM_GB300_UHM_HXX

#include "../uhm_gb300/csrc/linal.hpp"
#include "../uhm_gb300/csrc/mesh.hpp"

// The reference defines these as global macros (UHM/include/uhm/const.hxx);
// callers name them without the namespace.
using uhm::UHM_REAL;
using uhm::UHM_COMPLEX;
using uhm::UHM_LHS;
using uhm::UHM_RHS;
using uhm::UHM_CHOL;
using uhm::UHM_LU_NOPIV;
using uhm::UHM_LU_PIV;
using uhm::UHM_LU_INCPIV;
using uhm::UHM_QR;
using uhm::UHM_PHYSICS_SINGLE;
using uhm::UHM_PHYSICS_MULTI;
using uhm::UHM_NODE_KIND_DEFAULT;
using uhm::UHM_NODE_KIND_BOUNDARY;
using uhm::UHM_NOT_SEPARATED;
using uhm::UHM_SEPARATED_FACTOR;
using uhm::UHM_SEPARATED_SCHUR;
constexpr int UHM_INT = FLA_INT;
constexpr int UHM_SINGLE_REAL = FLA_FLOAT;
constexpr int UHM_DOUBLE_REAL = FLA_DOUBLE;
constexpr int UHM_SINGLE_COMPLEX = FLA_COMPLEX;
constexpr int UHM_DOUBLE_COMPLEX = FLA_DOUBLE_COMPLEX;

#endif
