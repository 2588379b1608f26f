// Dense-matrix objects for callers of the Mesh_ interface, with the names and
// calling conventions of the reference's LINAL layer:
//   linal::Matrix_  LINAL/include/linal/matrix.hxx:46-180 (a view wrapper)
//   linal::Flat_    LINAL/include/linal/flat.hxx:47-287   (a dense view)
//   linal::Hier_    LINAL/include/linal/hier.hxx:48-401   (one level of blocks)
// and the small part of the FLAME object API those objects and their callers
// use (FLA_Obj views, FLA_Init / FLA_Finalize, FLA_Random_matrix, the
// FLA_Obj_* accessors), so that a program written against the reference's
// uhm.hxx compiles against this library with only an include-path change.
//
// Everything here is host memory and host code: the views hand element
// matrices and right-hand sides to Mesh_::copy_in / copy_out, which copy
// them (the device engine keeps its own arena).  The numerical kernels of the
// reference's LINAL (dense chol / lu / trsm / gemm on these objects) are not
// part of this header: the factorisation they served runs on the GPU behind
// Mesh_::*_with_free.
//
// Differences from libflame, stated for a user:
//  - FLA_Random_matrix fills a view with values uniform in [-1, 1) from a
//    fixed generator (splitmix64 from seed 0x5EED, restarted by FLA_Init): a
//    program gets the same matrices on every run and machine.  Value k of
//    the sequence is 2 * (splitmix64(state += 0x9E3779B97F4A7C15) >> 11) *
//    2^-53 - 1, filled column by column over the view.
//  - Only FLA_DOUBLE data is filled / printed by value; other types keep
//    their bytes (created zeroed).
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

// ---- FLAME object subset ----------------------------------------------------
#ifndef FLA_SUCCESS
#define FLA_SUCCESS (-1)
#define FLA_FAILURE (-2)
#endif
enum : int {
  FLA_FLOAT = 100, FLA_DOUBLE = 101, FLA_COMPLEX = 102, FLA_DOUBLE_COMPLEX = 103, FLA_INT = 104,
  FLA_SCALAR = 150, FLA_MATRIX = 151
};

struct FLA_Base_obj {
  int datatype = FLA_DOUBLE;
  int elemtype = FLA_SCALAR;
  int m = 0, n = 0;          // allocated rows / columns
  int rs = 1, cs = 0;        // row and column stride (elements); column-major: rs = 1, cs = m
  void* buffer = nullptr;
};

struct FLA_Obj {
  int m = 0, n = 0;          // the view
  int offm = 0, offn = 0;    // its first row / column in the base object
  FLA_Base_obj* base = nullptr;
};

namespace linal_detail {
inline uint64_t& rng_state() {
  static uint64_t s = 0x5EEDull;
  return s;
}
inline double next_uniform() {
  uint64_t z = (rng_state() += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return 2.0 * (double)(z >> 11) * (1.0 / 9007199254740992.0) - 1.0;
}
inline size_t elem_size(int datatype, int elemtype) {
  if (elemtype == FLA_MATRIX) return sizeof(FLA_Obj);
  switch (datatype) {
    case FLA_FLOAT: case FLA_INT: return 4;
    case FLA_DOUBLE_COMPLEX: return 16;
    case FLA_COMPLEX: return 8;
    default: return 8;
  }
}
}  // namespace linal_detail

inline int FLA_Init() {
  linal_detail::rng_state() = 0x5EEDull;
  return FLA_SUCCESS;
}
inline int FLA_Finalize() { return FLA_SUCCESS; }

inline int FLA_Obj_length(FLA_Obj A) { return A.m; }
inline int FLA_Obj_width(FLA_Obj A) { return A.n; }
inline int FLA_Obj_datatype(FLA_Obj A) { return A.base ? A.base->datatype : FLA_DOUBLE; }
inline int FLA_Obj_elemtype(FLA_Obj A) { return A.base ? A.base->elemtype : FLA_SCALAR; }
inline int FLA_Obj_col_stride(FLA_Obj A) { return A.base ? A.base->cs : 0; }
inline int FLA_Obj_row_stride(FLA_Obj A) { return A.base ? A.base->rs : 1; }
inline void* FLA_Obj_buffer_at_view(FLA_Obj A) {
  if (!A.base || !A.base->buffer) return nullptr;
  const size_t es = linal_detail::elem_size(A.base->datatype, A.base->elemtype);
  return (char*)A.base->buffer + es * ((size_t)A.offm * A.base->rs + (size_t)A.offn * A.base->cs);
}
inline bool FLA_Obj_buffer_is_null(FLA_Obj A) { return !A.base || !A.base->buffer; }

// elemtype FLA_MATRIX: a buffer of m x n FLA_Obj views (a Hier_)
inline int FLA_Obj_create_ext(int datatype, int elemtype, int m, int n, int, int, int rs, int cs, FLA_Obj* A) {
  FLA_Base_obj* b = new FLA_Base_obj;
  b->datatype = datatype;
  b->elemtype = elemtype;
  b->m = m;
  b->n = n;
  b->rs = rs > 0 ? rs : 1;
  b->cs = cs > 0 ? cs : (m > 0 ? m : 1);
  const size_t es = linal_detail::elem_size(datatype, elemtype);
  if (elemtype == FLA_MATRIX) {
    b->buffer = new FLA_Obj[(size_t)m * n]();
  } else {
    b->buffer = std::calloc((size_t)b->cs * n > 0 ? (size_t)b->cs * n : 1, es);
    if (!b->buffer) {
      delete b;
      throw std::bad_alloc();
    }
  }
  A->m = m;
  A->n = n;
  A->offm = A->offn = 0;
  A->base = b;
  return FLA_SUCCESS;
}
inline int FLA_Obj_create(int datatype, int m, int n, int rs, int cs, FLA_Obj* A) {
  return FLA_Obj_create_ext(datatype, FLA_SCALAR, m, n, m, n, rs, cs, A);
}
inline int FLA_Obj_create_without_buffer(int datatype, int m, int n, FLA_Obj* A) {
  FLA_Base_obj* b = new FLA_Base_obj;
  b->datatype = datatype;
  b->m = m;
  b->n = n;
  b->cs = m > 0 ? m : 1;
  A->m = m;
  A->n = n;
  A->offm = A->offn = 0;
  A->base = b;
  return FLA_SUCCESS;
}
inline int FLA_Obj_free(FLA_Obj* A) {
  if (A->base) {
    if (A->base->elemtype == FLA_MATRIX) delete[] (FLA_Obj*)A->base->buffer;
    else std::free(A->base->buffer);
    delete A->base;
  }
  A->base = nullptr;
  A->m = A->n = 0;
  return FLA_SUCCESS;
}
inline int FLA_Obj_free_without_buffer(FLA_Obj* A) {
  delete A->base;
  A->base = nullptr;
  A->m = A->n = 0;
  return FLA_SUCCESS;
}

// values uniform in [-1, 1), column by column over the view (see the file comment)
inline int FLA_Random_matrix(FLA_Obj A) {
  if (FLA_Obj_datatype(A) != FLA_DOUBLE || FLA_Obj_elemtype(A) != FLA_SCALAR || !A.base || !A.base->buffer)
    return FLA_FAILURE;
  double* p = (double*)FLA_Obj_buffer_at_view(A);
  const int cs = A.base->cs, rs = A.base->rs;
  for (int j = 0; j < A.n; ++j)
    for (int i = 0; i < A.m; ++i) p[(size_t)i * rs + (size_t)j * cs] = linal_detail::next_uniform();
  return FLA_SUCCESS;
}

// title line, one line per row (each entry printed with format and a
// space), then the footer line
inline int FLA_Obj_fshow(FILE* f, const char* title, FLA_Obj A, const char* format, const char* footer) {
  std::fprintf(f, "%s\n", title);
  if (A.base && A.base->buffer && A.base->elemtype == FLA_SCALAR) {
    const char* p = (const char*)FLA_Obj_buffer_at_view(A);
    for (int i = 0; i < A.m; ++i) {
      for (int j = 0; j < A.n; ++j) {
        const size_t k = (size_t)i * A.base->rs + (size_t)j * A.base->cs;
        switch (A.base->datatype) {
          case FLA_INT: std::fprintf(f, format, ((const int*)p)[k]); break;
          case FLA_FLOAT: std::fprintf(f, format, (double)((const float*)p)[k]); break;
          case FLA_DOUBLE_COMPLEX:
            std::fprintf(f, format, ((const double*)p)[2 * k], ((const double*)p)[2 * k + 1]);
            break;
          default: std::fprintf(f, format, ((const double*)p)[k]); break;
        }
        std::fputc(' ', f);
      }
      std::fputc('\n', f);
    }
  }
  std::fprintf(f, "%s\n", footer);
  return FLA_SUCCESS;
}

// ---- LINAL objects ----------------------------------------------------------
namespace linal {

enum { LINAL_INT = FLA_INT, LINAL_REAL = FLA_DOUBLE, LINAL_COMPLEX = FLA_DOUBLE_COMPLEX,
       LINAL_SINGLE_REAL = FLA_FLOAT, LINAL_DOUBLE_REAL = FLA_DOUBLE, LINAL_SINGLE_COMPLEX = FLA_COMPLEX,
       LINAL_DOUBLE_COMPLEX = FLA_DOUBLE_COMPLEX };
enum { LINAL_NO_TRANSPOSE = 400, LINAL_TRANSPOSE = 401 };

inline void linal_check(bool ok, const char* msg) {
  if (!ok) throw std::invalid_argument(std::string("linal: ") + msg);
}

// A view of an FLA_Obj.  A matrix that created its object frees it; copies
// share the object and never free it (the reference's rule, matrix.hxx:
// 58-107), so a Flat_ passed by value to Mesh_::copy_in stays valid.
class Matrix_ {
 protected:
  int created = 0;
  FLA_Obj fla;

 public:
  Matrix_() = default;
  Matrix_(const Matrix_& b) : created(0), fla(b.fla) {}
  Matrix_& operator=(const Matrix_& b) {
    if (this != &b) {
      this->free();
      fla = b.fla;
      created = 0;
    }
    return *this;
  }
  virtual ~Matrix_() { this->free(); }

  void free() {
    if (created) FLA_Obj_free(&fla);
    created = 0;
    fla = FLA_Obj();
  }
  void create_buffer() {
    linal_check(fla.base && !fla.base->buffer, "create_buffer: no object or buffer already present");
    const size_t es = linal_detail::elem_size(fla.base->datatype, fla.base->elemtype);
    fla.base->buffer = std::calloc((size_t)fla.base->cs * fla.base->n > 0 ? (size_t)fla.base->cs * fla.base->n : 1, es);
    if (!fla.base->buffer) throw std::bad_alloc();
  }
  void free_buffer() {
    if (fla.base && fla.base->buffer && fla.base->elemtype == FLA_SCALAR) {
      std::free(fla.base->buffer);
      fla.base->buffer = nullptr;
    }
  }
  bool is_created() const { return created != 0; }
  bool is_buffer_null() const { return FLA_Obj_buffer_is_null(fla); }
  bool is_base_null() const { return fla.base == nullptr; }
  bool is_hier() const { return fla.base && fla.base->elemtype == FLA_MATRIX; }
  bool is_real_datatype() const { return get_data_type() == FLA_DOUBLE || get_data_type() == FLA_FLOAT; }
  bool is_complex_datatype() const {
    return get_data_type() == FLA_DOUBLE_COMPLEX || get_data_type() == FLA_COMPLEX;
  }
  int get_data_type() const { return fla.base ? fla.base->datatype : FLA_DOUBLE; }
  int get_data_size() const {
    return fla.base ? (int)linal_detail::elem_size(fla.base->datatype, fla.base->elemtype) : 0;
  }
  int get_buffer_size() const { return fla.base ? fla.base->cs * fla.base->n * get_data_size() : 0; }
  int get_cs() const { return fla.base ? fla.base->cs : 0; }
  int get_rs() const { return fla.base ? fla.base->rs : 1; }
  void set_m(int m) { fla.m = m; }
  void set_n(int n) { fla.n = n; }
  void set_offm(int o) { fla.offm = o; }
  void set_offn(int o) { fla.offn = o; }
  void set_fla(FLA_Obj obj) { fla = obj; }
  int get_m() const { return fla.m; }
  int get_n() const { return fla.n; }
  int get_offm() const { return fla.offm; }
  int get_offn() const { return fla.offn; }
  FLA_Obj& get_fla() { return fla; }
  FLA_Obj& operator~() { return fla; }
};

// A dense matrix or a view into one (flat.hxx:47-287).
class Flat_ : public Matrix_ {
 public:
  Flat_() = default;
  Flat_(FLA_Obj obj) {
    linal_check(obj.base && obj.base->elemtype == FLA_SCALAR, "Flat_: FLA_Obj is null or of MATRIX type");
    fla = obj;
    created = 0;
  }
  Flat_(const Flat_& b) : Matrix_(b) {}
  Flat_& operator=(const Flat_& b) {
    Matrix_::operator=(b);
    return *this;
  }
  ~Flat_() override { this->free(); }

  // m x n, zeroed; nothing is created when m or n is 0
  void create(int type, int m, int n) {
    if (!m || !n) return;
    linal_check(!is_created(), "create: already created");
    FLA_Obj_create(type, m, n, 0, 0, &fla);
    created = 1;
  }
  void create(int trans, Flat_ b) {
    if (!b.get_m() || !b.get_n()) return;
    linal_check(!is_created(), "create: already created");
    if (trans == LINAL_TRANSPOSE) FLA_Obj_create(b.get_data_type(), b.get_n(), b.get_m(), 0, 0, &fla);
    else FLA_Obj_create(b.get_data_type(), b.get_m(), b.get_n(), 0, 0, &fla);
    created = 1;
  }
  void create_without_buffer(int type, int m, int n) {
    if (!m || !n) return;
    linal_check(!is_created(), "create_without_buffer: already created");
    FLA_Obj_create_without_buffer(type, m, n, &fla);
    created = 1;
  }
  void wrap(FLA_Obj& obj) {
    linal_check(!created, "wrap: already created");
    linal_check(obj.base && obj.base->elemtype == FLA_SCALAR, "wrap: FLA_Obj is null or of MATRIX type");
    fla = obj;
    created = 0;
  }
  // A = the m x n block at (offm, offn) of this view
  void extract(Flat_& A, int m, int n, int offm, int offn) {
    linal_check(offm + m <= get_m() && offn + n <= get_n(), "extract: out of range");
    A.fla.m = m;
    A.fla.n = n;
    A.fla.offm = get_offm() + offm;
    A.fla.offn = get_offn() + offn;
    A.fla.base = fla.base;
  }
  double* get_buffer() { return (double*)FLA_Obj_buffer_at_view(fla); }
  bool operator==(Flat_& b) { return get_m() == b.get_m() && get_n() == b.get_n() && get_data_type() == b.get_data_type(); }
  bool operator!=(Flat_& b) { return !(*this == b); }
  double& operator()(unsigned int row, unsigned int col) {
    linal_check(row < (unsigned)get_m() && col < (unsigned)get_n(), "operator(): out of range");
    return get_buffer()[(size_t)col * get_cs() + row];
  }
  double& operator()(unsigned int row, unsigned int col, unsigned int idx) {
    linal_check(row < (unsigned)get_m() && col < (unsigned)get_n(), "operator(): out of range");
    return get_buffer()[2 * (size_t)col * get_cs() + 2 * row + idx];
  }
  void disp() { disp(stdout, "- Flat -"); }
  void disp(const char* title) { disp(stdout, title); }
  void disp(FILE* stream) { disp(stream, "- Flat -"); }
  void disp(FILE* stream, const char* title) {
    if (!get_m() || !get_n()) return;
    switch (get_data_type()) {
      case LINAL_INT: FLA_Obj_fshow(stream, title, fla, "% d", "----------"); break;
      case LINAL_DOUBLE_COMPLEX:
      case LINAL_SINGLE_COMPLEX: FLA_Obj_fshow(stream, title, fla, "( % E , % E )", "----------"); break;
      default: FLA_Obj_fshow(stream, title, fla, "% E", "----------"); break;
    }
  }
};

// One level of blocks over a dense matrix (hier.hxx:48-401): get_m() x
// get_n() views, block (i, j) = operator()(i, j); the last row / column of
// blocks takes the remainder.
class Hier_ : public Matrix_ {
 public:
  Hier_() = default;
  Hier_(const Hier_& b) : Matrix_(b) {}
  Hier_& operator=(const Hier_& b) {
    Matrix_::operator=(b);
    return *this;
  }
  ~Hier_() override { this->free(); }

  // m x n blocks, each an empty view
  void create(int type, int m, int n) {
    if (!m || !n) return;
    linal_check(!is_created(), "create: already created");
    FLA_Obj_create_ext(type, FLA_MATRIX, m, n, 0, 0, 0, 0, &fla);
    created = 1;
  }
  // blocks of mb x nb over an m x n matrix (views without a base)
  void create(int type, int m, int n, int mb, int nb) {
    if (!m || !n) return;
    linal_check(mb > 0 && nb > 0, "create: block size must be positive");
    linal_check(!is_created(), "create: already created");
    const int mm = (m + mb - 1) / mb, nn = (n + nb - 1) / nb;
    FLA_Obj_create_ext(type, FLA_MATRIX, mm, nn, 0, 0, 0, 0, &fla);
    FLA_Obj* buf = get_buffer();
    for (int j = 0; j < nn; ++j)
      for (int i = 0; i < mm; ++i) {
        FLA_Obj& part = buf[(size_t)j * mm + i];
        part.offm = i * mb;
        part.offn = j * nb;
        part.m = std::min(m, (i + 1) * mb) - i * mb;
        part.n = std::min(n, (j + 1) * nb) - j * nb;
        part.base = nullptr;
      }
    created = 1;
  }
  // blocks of mb x nb over the Flat_ F (views of F's object)
  void create(Flat_ F, int mb, int nb) {
    if (!F.get_m() || !F.get_n()) return;
    create(F.get_data_type(), F.get_m(), F.get_n(), mb, nb);
    for (int j = 0; j < get_n(); ++j)
      for (int i = 0; i < get_m(); ++i) {
        FLA_Obj& part = (*this)(i, j);
        part.offm += F.get_offm();
        part.offn += F.get_offn();
        part.base = (~F).base;
      }
  }
  void wrap(FLA_Obj& obj) {
    linal_check(!created, "wrap: already created");
    linal_check(obj.base && obj.base->elemtype == FLA_MATRIX, "wrap: FLA_Obj is null or not of MATRIX type");
    fla = obj;
    created = 0;
  }
  void extract(Hier_& A, int m, int n, int offm, int offn) {
    linal_check(offm + m <= get_m() && offn + n <= get_n(), "extract: out of range");
    A.fla.m = m;
    A.fla.n = n;
    A.fla.offm = get_offm() + offm;
    A.fla.offn = get_offn() + offn;
    A.fla.base = fla.base;
  }
  // the whole matrix the blocks cover, as one Flat_ view
  Flat_ flat() {
    int m = 0, n = 0;
    if (get_n() > 0)
      for (int i = 0; i < get_m(); ++i) m += (*this)(i, 0).m;
    if (get_m() > 0)
      for (int j = 0; j < get_n(); ++j) n += (*this)(0, j).n;
    FLA_Obj obj;
    if (m && n) obj = (*this)(0, 0);
    obj.m = m;
    obj.n = n;
    if (!obj.base) return Flat_();
    return Flat_(obj);
  }
  FLA_Obj* get_buffer() { return (FLA_Obj*)FLA_Obj_buffer_at_view(fla); }
  void disp() { disp(stdout); }
  void disp(FILE* stream) {
    std::fprintf(stream, " - Hier -\n");
    for (int i = 0; i < get_m(); ++i)
      for (int j = 0; j < get_n(); ++j) {
        const FLA_Obj& p = (*this)(i, j);
        std::fprintf(stream, " (%d, %d): %d x %d at (%d, %d)\n", i, j, p.m, p.n, p.offm, p.offn);
      }
  }
  bool operator==(Hier_& b) { return get_m() == b.get_m() && get_n() == b.get_n() && get_data_type() == b.get_data_type(); }
  bool operator!=(Hier_& b) { return !(*this == b); }
  FLA_Obj& operator()(unsigned int row, unsigned int col) {
    linal_check(row < (unsigned)get_m() && col < (unsigned)get_n(), "operator(): out of range");
    return get_buffer()[(size_t)col * get_cs() + row];
  }
};

typedef Matrix_* Matrix;
typedef Flat_* Flat;
typedef Hier_* Hier;

}  // namespace linal
