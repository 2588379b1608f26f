// FLAME-subset shim implementation (TEST INFRASTRUCTURE for the oracle build).
// See FLAME.h.  Dense numerics call BLAS/LAPACK (the OpenBLAS bundled with
// scipy, linked by oracle/Makefile); objects are column-major views.
#include "FLAME.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <random>

extern "C" {
void scipy_dgemm_(const char*, const char*, const int*, const int*, const int*, const double*,
                  const double*, const int*, const double*, const int*, const double*, double*,
                  const int*);
void scipy_dtrsm_(const char*, const char*, const char*, const char*, const int*, const int*,
                  const double*, const double*, const int*, double*, const int*);
void scipy_dtrmm_(const char*, const char*, const char*, const char*, const int*, const int*,
                  const double*, const double*, const int*, double*, const int*);
void scipy_dsyrk_(const char*, const char*, const int*, const int*, const double*, const double*,
                  const int*, const double*, double*, const int*);
void scipy_dpotrf_(const char*, const int*, double*, const int*, int*);
void scipy_dgetrf_(const int*, const int*, double*, const int*, int*, int*);
}

static double k_one = 1.0, k_zero = 0.0, k_minus_one = -1.0;
static FLA_Base_obj b_one{FLA_DOUBLE, FLA_SCALAR, 1, 1, 1, 1, &k_one, 0};
static FLA_Base_obj b_zero{FLA_DOUBLE, FLA_SCALAR, 1, 1, 1, 1, &k_zero, 0};
static FLA_Base_obj b_minus_one{FLA_DOUBLE, FLA_SCALAR, 1, 1, 1, 1, &k_minus_one, 0};
FLA_Obj FLA_ONE{0, 0, 1, 1, &b_one};
FLA_Obj FLA_ZERO{0, 0, 1, 1, &b_zero};
FLA_Obj FLA_MINUS_ONE{0, 0, 1, 1, &b_minus_one};

static void die(const char* what) {
  std::fprintf(stderr, "FLAME shim: %s\n", what);
  std::abort();
}

FLA_Error FLA_Init(void) { return FLA_SUCCESS; }
FLA_Error FLA_Finalize(void) { return FLA_SUCCESS; }

// ---- objects ---------------------------------------------------------------
dim_t FLA_Obj_datatype_size(FLA_Datatype dt) {
  switch (dt) {
    case FLA_INT: return sizeof(int);
    case FLA_FLOAT: return sizeof(float);
    case FLA_DOUBLE: return sizeof(double);
    case FLA_COMPLEX: return 2 * sizeof(float);
    case FLA_DOUBLE_COMPLEX: return 2 * sizeof(double);
  }
  return sizeof(double);
}

static dim_t elem_size(const FLA_Base_obj* b) {
  return b->elemtype == FLA_MATRIX ? sizeof(FLA_Obj) : FLA_Obj_datatype_size(b->datatype);
}

static FLA_Error make(FLA_Datatype dt, FLA_Elemtype et, dim_t m, dim_t n, FLA_Obj* obj) {
  FLA_Base_obj* b = new FLA_Base_obj;
  b->datatype = dt;
  b->elemtype = et;
  b->m = m;
  b->n = n;
  b->rs = 1;
  b->cs = m ? m : 1;
  b->buffer = nullptr;
  b->buffer_owned = 0;
  obj->offm = obj->offn = 0;
  obj->m = m;
  obj->n = n;
  obj->base = b;
  return FLA_SUCCESS;
}

FLA_Error FLA_Obj_create_without_buffer(FLA_Datatype dt, dim_t m, dim_t n, FLA_Obj* obj) {
  return make(dt, FLA_SCALAR, m, n, obj);
}

FLA_Error FLA_Obj_create_buffer(dim_t rs, dim_t cs, FLA_Obj* obj) {
  FLA_Base_obj* b = obj->base;
  (void)rs;
  (void)cs;
  b->rs = 1;
  b->cs = b->m ? b->m : 1;
  const size_t bytes = std::max<size_t>(1, b->m * b->n) * elem_size(b);
  b->buffer = std::calloc(1, bytes);
  if (!b->buffer) die("allocation failed");
  b->buffer_owned = 1;
  return FLA_SUCCESS;
}

FLA_Error FLA_Obj_create(FLA_Datatype dt, dim_t m, dim_t n, dim_t rs, dim_t cs, FLA_Obj* obj) {
  make(dt, FLA_SCALAR, m, n, obj);
  return FLA_Obj_create_buffer(rs, cs, obj);
}

FLA_Error FLA_Obj_create_ext(FLA_Datatype dt, FLA_Elemtype et, dim_t m, dim_t n, dim_t, dim_t, dim_t rs,
                             dim_t cs, FLA_Obj* obj) {
  make(dt, et, m, n, obj);
  return FLA_Obj_create_buffer(rs, cs, obj);
}

FLA_Error FLA_Obj_attach_buffer(void* buffer, dim_t rs, dim_t cs, FLA_Obj* obj) {
  FLA_Base_obj* b = obj->base;
  b->buffer = buffer;
  b->rs = rs ? rs : 1;
  b->cs = cs ? cs : (b->m ? b->m : 1);
  b->buffer_owned = 0;
  return FLA_SUCCESS;
}

FLA_Error FLA_Obj_free_buffer(FLA_Obj* obj) {
  if (obj->base && obj->base->buffer_owned && obj->base->buffer) std::free(obj->base->buffer);
  if (obj->base) {
    obj->base->buffer = nullptr;
    obj->base->buffer_owned = 0;
  }
  return FLA_SUCCESS;
}

FLA_Error FLA_Obj_free_without_buffer(FLA_Obj* obj) {
  delete obj->base;
  obj->base = nullptr;
  obj->m = obj->n = 0;
  return FLA_SUCCESS;
}

FLA_Error FLA_Obj_free(FLA_Obj* obj) {
  if (!obj->base) return FLA_SUCCESS;
  FLA_Obj_free_buffer(obj);
  return FLA_Obj_free_without_buffer(obj);
}

dim_t FLA_Obj_length(FLA_Obj o) { return o.m; }
dim_t FLA_Obj_width(FLA_Obj o) { return o.n; }
dim_t FLA_Obj_min_dim(FLA_Obj o) { return std::min(o.m, o.n); }
FLA_Datatype FLA_Obj_datatype(FLA_Obj o) { return o.base ? o.base->datatype : FLA_DOUBLE; }
FLA_Elemtype FLA_Obj_elemtype(FLA_Obj o) { return o.base ? o.base->elemtype : FLA_SCALAR; }
dim_t FLA_Obj_col_stride(FLA_Obj o) { return o.base->cs; }
FLA_Bool FLA_Obj_buffer_is_null(FLA_Obj o) { return !o.base || !o.base->buffer; }

void* FLA_Obj_buffer_at_view(FLA_Obj o) {
  if (!o.base || !o.base->buffer) return nullptr;
  const dim_t es = elem_size(o.base);
  return static_cast<char*>(o.base->buffer) + (o.offm * o.base->rs + o.offn * o.base->cs) * es;
}

static inline double* dp(FLA_Obj o) { return static_cast<double*>(FLA_Obj_buffer_at_view(o)); }
static inline int ld(FLA_Obj o) { return (int)o.base->cs; }
static inline double scal(FLA_Obj a) { return *dp(a); }

FLA_Error FLA_Obj_fshow(FILE* f, char* s1, FLA_Obj A, char* format, char* s2) {
  std::fprintf(f, "%s\n", s1);
  for (dim_t i = 0; i < A.m; ++i) {
    for (dim_t j = 0; j < A.n; ++j) {
      if (A.base->datatype == FLA_INT)
        std::fprintf(f, format, static_cast<int*>(FLA_Obj_buffer_at_view(A))[i + j * A.base->cs]);
      else
        std::fprintf(f, format, dp(A)[i + j * A.base->cs]);
      std::fprintf(f, " ");
    }
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "%s\n", s2);
  return FLA_SUCCESS;
}

// ---- partitioning ---------------------------------------------------------------
static FLA_Obj sub(FLA_Obj A, dim_t i, dim_t j, dim_t m, dim_t n) {
  FLA_Obj v;
  v.offm = A.offm + i;
  v.offn = A.offn + j;
  v.m = m;
  v.n = n;
  v.base = A.base;
  return v;
}

FLA_Error FLA_Part_2x2(FLA_Obj A, FLA_Obj* A11, FLA_Obj* A12, FLA_Obj* A21, FLA_Obj* A22, dim_t mb,
                       dim_t nb, FLA_Quadrant q) {
  mb = std::min(mb, A.m);
  nb = std::min(nb, A.n);
  dim_t mt = (q == FLA_TL || q == FLA_TR) ? mb : A.m - mb;   // rows of the top part
  dim_t nl = (q == FLA_TL || q == FLA_BL) ? nb : A.n - nb;   // columns of the left part
  *A11 = sub(A, 0, 0, mt, nl);
  *A12 = sub(A, 0, nl, mt, A.n - nl);
  *A21 = sub(A, mt, 0, A.m - mt, nl);
  *A22 = sub(A, mt, nl, A.m - mt, A.n - nl);
  return FLA_SUCCESS;
}

FLA_Error FLA_Part_2x1(FLA_Obj A, FLA_Obj* A1, FLA_Obj* A2, dim_t mb, FLA_Side side) {
  mb = std::min(mb, A.m);
  const dim_t mt = side == FLA_TOP ? mb : A.m - mb;
  *A1 = sub(A, 0, 0, mt, A.n);
  *A2 = sub(A, mt, 0, A.m - mt, A.n);
  return FLA_SUCCESS;
}

FLA_Error FLA_Part_1x2(FLA_Obj A, FLA_Obj* A1, FLA_Obj* A2, dim_t nb, FLA_Side side) {
  nb = std::min(nb, A.n);
  const dim_t nl = side == FLA_LEFT ? nb : A.n - nb;
  *A1 = sub(A, 0, 0, A.m, nl);
  *A2 = sub(A, 0, nl, A.m, A.n - nl);
  return FLA_SUCCESS;
}

FLA_Error FLA_Repart_2x2_to_3x3(FLA_Obj ATL, FLA_Obj ATR, FLA_Obj* A00, FLA_Obj* A01, FLA_Obj* A02,
                                FLA_Obj* A10, FLA_Obj* A11, FLA_Obj* A12, FLA_Obj ABL, FLA_Obj ABR,
                                FLA_Obj* A20, FLA_Obj* A21, FLA_Obj* A22, dim_t mb, dim_t nb,
                                FLA_Quadrant q) {
  if (q == FLA_BR) {
    mb = std::min(mb, ABR.m);
    nb = std::min(nb, ABR.n);
    *A00 = ATL;
    *A01 = sub(ATR, 0, 0, ATR.m, nb);
    *A02 = sub(ATR, 0, nb, ATR.m, ATR.n - nb);
    *A10 = sub(ABL, 0, 0, mb, ABL.n);
    *A11 = sub(ABR, 0, 0, mb, nb);
    *A12 = sub(ABR, 0, nb, mb, ABR.n - nb);
    *A20 = sub(ABL, mb, 0, ABL.m - mb, ABL.n);
    *A21 = sub(ABR, mb, 0, ABR.m - mb, nb);
    *A22 = sub(ABR, mb, nb, ABR.m - mb, ABR.n - nb);
  } else if (q == FLA_TL) {
    mb = std::min(mb, ATL.m);
    nb = std::min(nb, ATL.n);
    const dim_t mt = ATL.m - mb, nl = ATL.n - nb;
    *A00 = sub(ATL, 0, 0, mt, nl);
    *A01 = sub(ATL, 0, nl, mt, nb);
    *A02 = sub(ATR, 0, 0, mt, ATR.n);
    *A10 = sub(ATL, mt, 0, mb, nl);
    *A11 = sub(ATL, mt, nl, mb, nb);
    *A12 = sub(ATR, mt, 0, mb, ATR.n);
    *A20 = sub(ABL, 0, 0, ABL.m, nl);
    *A21 = sub(ABL, 0, nl, ABL.m, nb);
    *A22 = ABR;
  } else {
    die("Repart_2x2_to_3x3: quadrant not supported");
  }
  return FLA_SUCCESS;
}

FLA_Error FLA_Cont_with_3x3_to_2x2(FLA_Obj* ATL, FLA_Obj* ATR, FLA_Obj A00, FLA_Obj A01, FLA_Obj A02,
                                   FLA_Obj A10, FLA_Obj A11, FLA_Obj A12, FLA_Obj* ABL, FLA_Obj* ABR,
                                   FLA_Obj A20, FLA_Obj A21, FLA_Obj A22, FLA_Quadrant q) {
  (void)A02;
  (void)A20;
  if (q == FLA_TL) {   // A11 joins the top-left part
    *ATL = sub(A00, 0, 0, A00.m + A10.m, A00.n + A01.n);
    *ATR = sub(A02, 0, 0, A02.m + A12.m, A02.n);
    *ABL = sub(A20, 0, 0, A20.m, A20.n + A21.n);
    *ABR = A22;
  } else if (q == FLA_BR) {   // A11 joins the bottom-right part
    *ATL = A00;
    *ATR = sub(A01, 0, 0, A01.m, A01.n + A02.n);
    *ABL = sub(A10, 0, 0, A10.m + A20.m, A10.n);
    *ABR = sub(A11, 0, 0, A11.m + A21.m, A11.n + A12.n);
  } else {
    die("Cont_with_3x3_to_2x2: quadrant not supported");
  }
  return FLA_SUCCESS;
}

FLA_Error FLA_Repart_2x1_to_3x1(FLA_Obj AT, FLA_Obj* A0, FLA_Obj* A1, FLA_Obj AB, FLA_Obj* A2, dim_t mb,
                                FLA_Side side) {
  if (side == FLA_BOTTOM) {
    mb = std::min(mb, AB.m);
    *A0 = AT;
    *A1 = sub(AB, 0, 0, mb, AB.n);
    *A2 = sub(AB, mb, 0, AB.m - mb, AB.n);
  } else {
    mb = std::min(mb, AT.m);
    *A0 = sub(AT, 0, 0, AT.m - mb, AT.n);
    *A1 = sub(AT, AT.m - mb, 0, mb, AT.n);
    *A2 = AB;
  }
  return FLA_SUCCESS;
}

FLA_Error FLA_Cont_with_3x1_to_2x1(FLA_Obj* AT, FLA_Obj A0, FLA_Obj A1, FLA_Obj* AB, FLA_Obj A2,
                                   FLA_Side side) {
  if (side == FLA_TOP) {   // A1 joins the top part
    *AT = sub(A0, 0, 0, A0.m + A1.m, A0.n);
    *AB = A2;
  } else {
    *AT = A0;
    *AB = sub(A1, 0, 0, A1.m + A2.m, A1.n);
  }
  return FLA_SUCCESS;
}

FLA_Error FLA_Repart_1x2_to_1x3(FLA_Obj AL, FLA_Obj AR, FLA_Obj* A0, FLA_Obj* A1, FLA_Obj* A2, dim_t nb,
                                FLA_Side side) {
  if (side == FLA_RIGHT) {
    nb = std::min(nb, AR.n);
    *A0 = AL;
    *A1 = sub(AR, 0, 0, AR.m, nb);
    *A2 = sub(AR, 0, nb, AR.m, AR.n - nb);
  } else {
    nb = std::min(nb, AL.n);
    *A0 = sub(AL, 0, 0, AL.m, AL.n - nb);
    *A1 = sub(AL, 0, AL.n - nb, AL.m, nb);
    *A2 = AR;
  }
  return FLA_SUCCESS;
}

FLA_Error FLA_Cont_with_1x3_to_1x2(FLA_Obj* AL, FLA_Obj* AR, FLA_Obj A0, FLA_Obj A1, FLA_Obj A2,
                                   FLA_Side side) {
  if (side == FLA_LEFT) {   // A1 joins the left part
    *AL = sub(A0, 0, 0, A0.m, A0.n + A1.n);
    *AR = A2;
  } else {
    *AL = A0;
    *AR = sub(A1, 0, 0, A1.m, A1.n + A2.n);
  }
  return FLA_SUCCESS;
}

FLA_Error FLA_Merge_2x1(FLA_Obj AT, FLA_Obj AB, FLA_Obj* A) {
  *A = sub(AT, 0, 0, AT.m + AB.m, AT.n);
  return FLA_SUCCESS;
}

// ---- numerics ------------------------------------------------------------------
static char tr(FLA_Trans t) { return t == FLA_NO_TRANSPOSE || t == FLA_CONJ_NO_TRANSPOSE ? 'N' : 'T'; }
static char up(FLA_Uplo u) { return u == FLA_LOWER_TRIANGULAR ? 'L' : 'U'; }
static char sd(FLA_Side s) { return s == FLA_LEFT ? 'L' : 'R'; }
static char dg(FLA_Diag d) { return d == FLA_UNIT_DIAG ? 'U' : 'N'; }

static void scale_view(double a, FLA_Obj C) {
  if (a == 1.0) return;
  double* c = dp(C);
  for (dim_t j = 0; j < C.n; ++j)
    for (dim_t i = 0; i < C.m; ++i) c[i + j * ld(C)] = a == 0.0 ? 0.0 : a * c[i + j * ld(C)];
}

FLA_Error FLA_Gemm(FLA_Trans ta, FLA_Trans tb, FLA_Obj alpha, FLA_Obj A, FLA_Obj B, FLA_Obj beta, FLA_Obj C) {
  if (!C.m || !C.n) return FLA_SUCCESS;
  const int m = (int)C.m, n = (int)C.n, k = (int)(tr(ta) == 'N' ? A.n : A.m);
  const double a = scal(alpha), b = scal(beta);
  if (k == 0) {
    scale_view(b, C);
    return FLA_SUCCESS;
  }
  const char ca = tr(ta), cb = tr(tb);
  const int lda = ld(A), ldb = ld(B), ldc = ld(C);
  scipy_dgemm_(&ca, &cb, &m, &n, &k, &a, dp(A), &lda, dp(B), &ldb, &b, dp(C), &ldc);
  return FLA_SUCCESS;
}

FLA_Error FLA_Trsm(FLA_Side side, FLA_Uplo uplo, FLA_Trans trans, FLA_Diag diag, FLA_Obj alpha, FLA_Obj A,
                   FLA_Obj B) {
  if (!B.m || !B.n) return FLA_SUCCESS;
  const int m = (int)B.m, n = (int)B.n, lda = ld(A), ldb = ld(B);
  const double a = scal(alpha);
  const char s = sd(side), u = up(uplo), t = tr(trans), d = dg(diag);
  scipy_dtrsm_(&s, &u, &t, &d, &m, &n, &a, dp(A), &lda, dp(B), &ldb);
  return FLA_SUCCESS;
}

FLA_Error FLA_Trmm(FLA_Side side, FLA_Uplo uplo, FLA_Trans trans, FLA_Diag diag, FLA_Obj alpha, FLA_Obj A,
                   FLA_Obj B) {
  if (!B.m || !B.n) return FLA_SUCCESS;
  const int m = (int)B.m, n = (int)B.n, lda = ld(A), ldb = ld(B);
  const double a = scal(alpha);
  const char s = sd(side), u = up(uplo), t = tr(trans), d = dg(diag);
  scipy_dtrmm_(&s, &u, &t, &d, &m, &n, &a, dp(A), &lda, dp(B), &ldb);
  return FLA_SUCCESS;
}

FLA_Error FLA_Syrk(FLA_Uplo uplo, FLA_Trans trans, FLA_Obj alpha, FLA_Obj A, FLA_Obj beta, FLA_Obj C) {
  if (!C.m) return FLA_SUCCESS;
  const int n = (int)C.m, k = (int)(tr(trans) == 'N' ? A.n : A.m);
  const double a = scal(alpha), b = scal(beta);
  if (k == 0) {
    scale_view(b, C);
    return FLA_SUCCESS;
  }
  const char u = up(uplo), t = tr(trans);
  const int lda = ld(A), ldc = ld(C);
  scipy_dsyrk_(&u, &t, &n, &k, &a, dp(A), &lda, &b, dp(C), &ldc);
  return FLA_SUCCESS;
}

FLA_Error FLA_Chol(FLA_Uplo uplo, FLA_Obj A) {
  if (!A.m) return FLA_SUCCESS;
  const int n = (int)A.m, lda = ld(A);
  int info = 0;
  const char u = up(uplo);
  scipy_dpotrf_(&u, &n, dp(A), &lda, &info);
  return info == 0 ? FLA_SUCCESS : info;
}

FLA_Error FLA_LU_nopiv(FLA_Obj A) {
  double* a = dp(A);
  const dim_t m = A.m, n = A.n, l = ld(A);
  const dim_t kmax = std::min(m, n);
  for (dim_t k = 0; k < kmax; ++k) {
    const double p = a[k + k * l];
    for (dim_t i = k + 1; i < m; ++i) a[i + k * l] /= p;
    for (dim_t j = k + 1; j < n; ++j) {
      const double akj = a[k + j * l];
      for (dim_t i = k + 1; i < m; ++i) a[i + j * l] -= a[i + k * l] * akj;
    }
  }
  return FLA_SUCCESS;
}

// pivots: p[i] = offset of the row interchanged with row i, relative to row i
FLA_Error FLA_LU_piv(FLA_Obj A, FLA_Obj p) {
  if (!A.m || !A.n) return FLA_SUCCESS;
  const int m = (int)A.m, n = (int)A.n, lda = ld(A);
  const int kmax = std::min(m, n);
  int* ipiv = static_cast<int*>(std::malloc(sizeof(int) * kmax));
  int info = 0;
  scipy_dgetrf_(&m, &n, dp(A), &lda, ipiv, &info);
  int* pv = static_cast<int*>(FLA_Obj_buffer_at_view(p));
  for (int i = 0; i < kmax; ++i) pv[i * p.base->rs] = ipiv[i] - 1 - i;
  std::free(ipiv);
  return info == 0 ? FLA_SUCCESS : info;
}

FLA_Error FLA_Apply_pivots(FLA_Side side, FLA_Trans trans, FLA_Obj p, FLA_Obj A) {
  if (side != FLA_LEFT) die("Apply_pivots: only FLA_LEFT");
  if (!A.m || !A.n || !p.m) return FLA_SUCCESS;
  const int* pv = static_cast<int*>(FLA_Obj_buffer_at_view(p));
  double* a = dp(A);
  const dim_t l = ld(A);
  const dim_t np = std::min<dim_t>(p.m, A.m);
  auto swap_rows = [&](dim_t i, dim_t k) {
    if (i == k) return;
    for (dim_t j = 0; j < A.n; ++j) std::swap(a[i + j * l], a[k + j * l]);
  };
  if (trans == FLA_NO_TRANSPOSE)
    for (dim_t i = 0; i < np; ++i) swap_rows(i, i + pv[i * p.base->rs]);
  else
    for (dim_t ii = np; ii > 0; --ii) swap_rows(ii - 1, ii - 1 + pv[(ii - 1) * p.base->rs]);
  return FLA_SUCCESS;
}

FLA_Error FLA_Axpyt(FLA_Trans trans, FLA_Obj alpha, FLA_Obj A, FLA_Obj B) {
  const double a = scal(alpha);
  const double* x = dp(A);
  double* y = dp(B);
  const dim_t la = ld(A), lb = ld(B);
  const bool t = tr(trans) == 'T';
  for (dim_t j = 0; j < B.n; ++j)
    for (dim_t i = 0; i < B.m; ++i) y[i + j * lb] += a * (t ? x[j + i * la] : x[i + j * la]);
  return FLA_SUCCESS;
}

FLA_Error FLA_Axpy(FLA_Obj alpha, FLA_Obj A, FLA_Obj B) { return FLA_Axpyt(FLA_NO_TRANSPOSE, alpha, A, B); }

FLA_Error FLA_Copyt(FLA_Trans trans, FLA_Obj A, FLA_Obj B) {
  if (A.base->datatype == FLA_INT) {
    const int* x = static_cast<int*>(FLA_Obj_buffer_at_view(A));
    int* y = static_cast<int*>(FLA_Obj_buffer_at_view(B));
    for (dim_t j = 0; j < B.n; ++j)
      for (dim_t i = 0; i < B.m; ++i) y[i + j * B.base->cs] = x[i + j * A.base->cs];
    return FLA_SUCCESS;
  }
  const double* x = dp(A);
  double* y = dp(B);
  const dim_t la = ld(A), lb = ld(B);
  const bool t = tr(trans) == 'T';
  for (dim_t j = 0; j < B.n; ++j)
    for (dim_t i = 0; i < B.m; ++i) y[i + j * lb] = t ? x[j + i * la] : x[i + j * la];
  return FLA_SUCCESS;
}

FLA_Error FLA_Copy(FLA_Obj A, FLA_Obj B) { return FLA_Copyt(FLA_NO_TRANSPOSE, A, B); }

FLA_Error FLA_Scal(FLA_Obj alpha, FLA_Obj A) {
  if (!A.m || !A.n) return FLA_SUCCESS;
  scale_view(scal(alpha), A);
  return FLA_SUCCESS;
}

FLA_Error FLA_Norm1(FLA_Obj A, FLA_Obj norm) {
  const double* a = dp(A);
  double best = 0.0;
  for (dim_t j = 0; j < A.n; ++j) {
    double s = 0.0;
    for (dim_t i = 0; i < A.m; ++i) s += std::fabs(a[i + j * ld(A)]);
    best = std::max(best, s);
  }
  *dp(norm) = best;
  return FLA_SUCCESS;
}

FLA_Error FLA_Norm_inf(FLA_Obj A, FLA_Obj norm) {
  const double* a = dp(A);
  double best = 0.0;
  for (dim_t i = 0; i < A.m; ++i) {
    double s = 0.0;
    for (dim_t j = 0; j < A.n; ++j) s += std::fabs(a[i + j * ld(A)]);
    best = std::max(best, s);
  }
  *dp(norm) = best;
  return FLA_SUCCESS;
}

FLA_Error FLA_Dot(FLA_Obj x, FLA_Obj y, FLA_Obj rho) {
  const double* a = dp(x);
  const double* b = dp(y);
  const dim_t len = std::max(x.m, x.n);
  const dim_t sa = x.m == 1 ? ld(x) : 1, sb = y.m == 1 ? ld(y) : 1;
  double s = 0.0;
  for (dim_t i = 0; i < len; ++i) s += a[i * sa] * b[i * sb];
  *dp(rho) = s;
  return FLA_SUCCESS;
}

FLA_Error FLA_Triangularize(FLA_Uplo uplo, FLA_Diag diag, FLA_Obj A) {
  double* a = dp(A);
  for (dim_t j = 0; j < A.n; ++j)
    for (dim_t i = 0; i < A.m; ++i) {
      const bool keep = uplo == FLA_LOWER_TRIANGULAR ? i >= j : i <= j;
      if (!keep) a[i + j * ld(A)] = 0.0;
      if (i == j && diag == FLA_UNIT_DIAG) a[i + j * ld(A)] = 1.0;
      if (i == j && diag == FLA_ZERO_DIAG) a[i + j * ld(A)] = 0.0;
    }
  return FLA_SUCCESS;
}

FLA_Error FLA_Obj_set_to_scalar(FLA_Obj alpha, FLA_Obj A) {
  if (!A.m || !A.n || !A.base || !A.base->buffer) return FLA_SUCCESS;
  if (A.base->elemtype == FLA_MATRIX) return FLA_SUCCESS;
  if (A.base->datatype == FLA_INT) {
    int* a = static_cast<int*>(FLA_Obj_buffer_at_view(A));
    for (dim_t j = 0; j < A.n; ++j)
      for (dim_t i = 0; i < A.m; ++i) a[i + j * A.base->cs] = (int)scal(alpha);
    return FLA_SUCCESS;
  }
  double* a = dp(A);
  const double v = scal(alpha);
  for (dim_t j = 0; j < A.n; ++j)
    for (dim_t i = 0; i < A.m; ++i) a[i + j * ld(A)] = v;
  return FLA_SUCCESS;
}

static std::mt19937_64& rng() {
  static std::mt19937_64 g(12345);
  return g;
}

FLA_Error FLA_Random_matrix(FLA_Obj A) {
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  double* a = dp(A);
  for (dim_t j = 0; j < A.n; ++j)
    for (dim_t i = 0; i < A.m; ++i) a[i + j * ld(A)] = u(rng());
  return FLA_SUCCESS;
}

FLA_Error FLA_Random_spd_matrix(FLA_Uplo uplo, FLA_Obj A) {
  (void)uplo;
  FLA_Random_matrix(A);
  double* a = dp(A);
  const dim_t n = A.m;
  for (dim_t j = 0; j < n; ++j)
    for (dim_t i = j; i < n; ++i) {
      const double v = 0.5 * (a[i + j * ld(A)] + a[j + i * ld(A)]) + (i == j ? (double)n : 0.0);
      a[i + j * ld(A)] = a[j + i * ld(A)] = v;
    }
  return FLA_SUCCESS;
}

FLA_Error FLA_QR_UT(FLA_Obj, FLA_Obj) { die("QR is not provided by this shim"); return FLA_FAILURE; }
FLA_Error FLA_QR_UT_blk_var2(FLA_Obj, FLA_Obj, fla_qrut_t*) { die("QR is not provided"); return FLA_FAILURE; }
FLA_Error FLA_QR2_UT_internal(FLA_Obj, FLA_Obj, FLA_Obj, fla_qr2ut_t*) { die("QR is not provided"); return FLA_FAILURE; }
FLA_Error FLA_QR2_UT_inc_blk_var1(FLA_Obj, FLA_Obj, FLA_Obj, fla_qr2ut_t*) { die("QR is not provided"); return FLA_FAILURE; }
FLA_Error FLA_Apply_Q_UT(FLA_Side, FLA_Trans, FLA_Direct, FLA_Store, FLA_Obj, FLA_Obj, FLA_Obj, FLA_Obj) {
  die("QR is not provided");
  return FLA_FAILURE;
}
FLA_Error FLA_Apply_Q2_UT_internal(FLA_Side, FLA_Trans, FLA_Direct, FLA_Store, FLA_Obj, FLA_Obj, FLA_Obj, FLA_Obj,
                                   FLA_Obj, fla_apq2ut_t*) {
  die("QR is not provided");
  return FLA_FAILURE;
}

// control trees declared extern by the reference headers (unused by the shim)
fla_qrutinc_t* flash_qrutinc_cntl = nullptr;
fla_qrut_t* fla_qrut_cntl_leaf = nullptr;
fla_apqut_t* fla_apqut_cntl_leaf = nullptr;
fla_qr2ut_t* fla_qr2ut_cntl_leaf = nullptr;
fla_apq2ut_t* fla_apq2ut_cntl_leaf = nullptr;
fla_axpy_t* flash_axpy_cntl_blas = nullptr;
fla_copy_t* flash_copy_cntl_blas = nullptr;
fla_scal_t* flash_scal_cntl_blas = nullptr;
fla_appiv_t* flash_appiv_cntl = nullptr;
fla_chol_t* flash_chol_cntl_leaf = nullptr;
fla_lu_t* flash_lu_nopiv_cntl_leaf = nullptr;
fla_lu_t* flash_lu_piv_cntl_leaf = nullptr;
fla_qrut_t* flash_qrut_cntl_leaf = nullptr;
fla_apqut_t* flash_apqut_cntl_leaf = nullptr;
fla_qr2ut_t* flash_qr2ut_cntl_leaf = nullptr;
fla_apq2ut_t* flash_apq2ut_cntl_leaf = nullptr;
fla_trsm_t* flash_trsm_cntl_blas = nullptr;
fla_gemm_t* flash_gemm_cntl_blas = nullptr;
fla_trmm_t* flash_trmm_cntl_blas = nullptr;
fla_lu_t* flash_lu_nopiv_cntl = nullptr;
fla_trsm_t* flash_trsm_cntl_mm = nullptr;
fla_gemm_t* flash_gemm_cntl_mm_op = nullptr;
fla_trmm_t* flash_trmm_cntl_mm = nullptr;
