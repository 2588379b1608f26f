/*
 * FLAME-subset shim (TEST INFRASTRUCTURE for the oracle build).
 *
 * Declares the part of libflame's interface that the reference's UHM and
 * LINAL sources call, so that those sources compile unmodified for the
 * oracle (oracle/Makefile).  libflame itself is not available; this is a
 * project-written implementation of the object/view model (FLA_Obj,
 * partitioning) and of the double-precision numerics, on top of BLAS/LAPACK.
 *
 * Enum values that the reference hard-codes are reproduced exactly
 * (LINAL/include/linal/const.hxx:78-100, LINAL/src/dense/gemm.cxx:57-130,
 * LINAL/src/dense/trsm.cxx:50-78, UHM/include/uhm/wrapper/fort.f90:36-37).
 * Everything else is this shim's own choice.  QR-family entry points are
 * stubs that abort: the oracle does not exercise QR.
 */
#ifndef UHM_ORACLE_FLAME_SHIM_H
#define UHM_ORACLE_FLAME_SHIM_H

#include <cstdio>
#include <cstring>
#include <unistd.h>

/* libflame's headers provide min/max and the C string / POSIX headers that
   the reference relies on implicitly. */
template <class T> inline T min(T a, T b) { return a < b ? a : b; }
template <class T> inline T max(T a, T b) { return a > b ? a : b; }

typedef int FLA_Error;
typedef int FLA_Bool;
typedef int FLA_Datatype;
typedef int FLA_Elemtype;
typedef int FLA_Side;
typedef int FLA_Uplo;
typedef int FLA_Trans;
typedef int FLA_Conj;
typedef int FLA_Diag;
typedef int FLA_Quadrant;
typedef int FLA_Direct;
typedef int FLA_Store;
typedef unsigned long dim_t;

#define FLA_SUCCESS (-1)
#define FLA_FAILURE (-2)

/* sides / uplo / trans / conj (values the reference switches on) */
#define FLA_TOP 200
#define FLA_BOTTOM 201
#define FLA_LEFT 210
#define FLA_RIGHT 211
#define FLA_SIDE_MASK 0x1
#define FLA_LOWER_TRIANGULAR 300
#define FLA_UPPER_TRIANGULAR 301
#define FLA_UPLO_MASK 0x1
#define FLA_NO_TRANSPOSE 400
#define FLA_TRANSPOSE 401
#define FLA_CONJ_TRANSPOSE 402
#define FLA_CONJ_NO_TRANSPOSE 403
#define FLA_TRANS_MASK 0x3
#define FLA_NO_CONJUGATE 450
#define FLA_CONJUGATE 451
#define FLA_UNIT_DIAG 500
#define FLA_NONUNIT_DIAG 501
#define FLA_ZERO_DIAG 502
/* quadrants */
#define FLA_TL 11
#define FLA_TR 12
#define FLA_BL 21
#define FLA_BR 22
/* data and element types */
#define FLA_FLOAT 100
#define FLA_DOUBLE 101
#define FLA_COMPLEX 102
#define FLA_DOUBLE_COMPLEX 103
#define FLA_INT 104
#define FLA_SCALAR 150
#define FLA_MATRIX 151
/* QR directions / storage */
#define FLA_FORWARD 600
#define FLA_BACKWARD 601
#define FLA_COLUMNWISE 700
#define FLA_ROWWISE 701

typedef struct FLA_Obj_struct {
  FLA_Datatype datatype;
  FLA_Elemtype elemtype;
  dim_t m, n;           /* base dimensions */
  dim_t rs, cs;         /* row / column strides in elements */
  void* buffer;
  int buffer_owned;
} FLA_Base_obj;

typedef struct FLA_Obj_view {
  dim_t offm, offn, m, n;
  FLA_Base_obj* base;
} FLA_Obj;

/* opaque control-tree types (only pointers are declared by the reference) */
typedef struct fla_cntl_opaque fla_axpy_t;
typedef struct fla_cntl_opaque fla_copy_t;
typedef struct fla_cntl_opaque fla_scal_t;
typedef struct fla_cntl_opaque fla_appiv_t;
typedef struct fla_cntl_opaque fla_chol_t;
typedef struct fla_cntl_opaque fla_lu_t;
typedef struct fla_cntl_opaque fla_qrut_t;
typedef struct fla_cntl_opaque fla_apqut_t;
typedef struct fla_cntl_opaque fla_qr2ut_t;
typedef struct fla_cntl_opaque fla_apq2ut_t;
typedef struct fla_cntl_opaque fla_qrutinc_t;
typedef struct fla_cntl_opaque fla_trsm_t;
typedef struct fla_cntl_opaque fla_gemm_t;
typedef struct fla_cntl_opaque fla_trmm_t;

extern FLA_Obj FLA_ONE, FLA_ZERO, FLA_MINUS_ONE;

/* library */
FLA_Error FLA_Init(void);
FLA_Error FLA_Finalize(void);

/* objects */
FLA_Error FLA_Obj_create(FLA_Datatype dt, dim_t m, dim_t n, dim_t rs, dim_t cs, FLA_Obj* obj);
FLA_Error FLA_Obj_create_ext(FLA_Datatype dt, FLA_Elemtype et, dim_t m, dim_t n, dim_t m_inner,
                             dim_t n_inner, dim_t rs, dim_t cs, FLA_Obj* obj);
FLA_Error FLA_Obj_create_without_buffer(FLA_Datatype dt, dim_t m, dim_t n, FLA_Obj* obj);
FLA_Error FLA_Obj_create_buffer(dim_t rs, dim_t cs, FLA_Obj* obj);
FLA_Error FLA_Obj_attach_buffer(void* buffer, dim_t rs, dim_t cs, FLA_Obj* obj);
FLA_Error FLA_Obj_free(FLA_Obj* obj);
FLA_Error FLA_Obj_free_buffer(FLA_Obj* obj);
FLA_Error FLA_Obj_free_without_buffer(FLA_Obj* obj);
dim_t FLA_Obj_length(FLA_Obj obj);
dim_t FLA_Obj_width(FLA_Obj obj);
dim_t FLA_Obj_min_dim(FLA_Obj obj);
FLA_Datatype FLA_Obj_datatype(FLA_Obj obj);
FLA_Elemtype FLA_Obj_elemtype(FLA_Obj obj);
dim_t FLA_Obj_datatype_size(FLA_Datatype dt);
dim_t FLA_Obj_col_stride(FLA_Obj obj);
void* FLA_Obj_buffer_at_view(FLA_Obj obj);
FLA_Bool FLA_Obj_buffer_is_null(FLA_Obj obj);
FLA_Error FLA_Obj_fshow(FILE* f, char* s1, FLA_Obj A, char* format, char* s2);

/* partitioning */
FLA_Error FLA_Part_2x2(FLA_Obj A, FLA_Obj* A11, FLA_Obj* A12, FLA_Obj* A21, FLA_Obj* A22, dim_t mb,
                       dim_t nb, FLA_Quadrant q);
FLA_Error FLA_Part_2x1(FLA_Obj A, FLA_Obj* A1, FLA_Obj* A2, dim_t mb, FLA_Side side);
FLA_Error FLA_Part_1x2(FLA_Obj A, FLA_Obj* A1, FLA_Obj* A2, dim_t nb, FLA_Side side);
FLA_Error FLA_Repart_2x2_to_3x3(FLA_Obj ATL, FLA_Obj ATR, FLA_Obj* A00, FLA_Obj* A01, FLA_Obj* A02,
                                FLA_Obj* A10, FLA_Obj* A11, FLA_Obj* A12, FLA_Obj ABL, FLA_Obj ABR,
                                FLA_Obj* A20, FLA_Obj* A21, FLA_Obj* A22, dim_t mb, dim_t nb,
                                FLA_Quadrant q);
FLA_Error FLA_Repart_2x1_to_3x1(FLA_Obj AT, FLA_Obj* A0, FLA_Obj* A1, FLA_Obj AB, FLA_Obj* A2, dim_t mb,
                                FLA_Side side);
FLA_Error FLA_Repart_1x2_to_1x3(FLA_Obj AL, FLA_Obj AR, FLA_Obj* A0, FLA_Obj* A1, FLA_Obj* A2, dim_t nb,
                                FLA_Side side);
FLA_Error FLA_Cont_with_3x3_to_2x2(FLA_Obj* ATL, FLA_Obj* ATR, FLA_Obj A00, FLA_Obj A01, FLA_Obj A02,
                                   FLA_Obj A10, FLA_Obj A11, FLA_Obj A12, FLA_Obj* ABL, FLA_Obj* ABR,
                                   FLA_Obj A20, FLA_Obj A21, FLA_Obj A22, FLA_Quadrant q);
FLA_Error FLA_Cont_with_3x1_to_2x1(FLA_Obj* AT, FLA_Obj A0, FLA_Obj A1, FLA_Obj* AB, FLA_Obj A2,
                                   FLA_Side side);
FLA_Error FLA_Cont_with_1x3_to_1x2(FLA_Obj* AL, FLA_Obj* AR, FLA_Obj A0, FLA_Obj A1, FLA_Obj A2,
                                   FLA_Side side);
FLA_Error FLA_Merge_2x1(FLA_Obj AT, FLA_Obj AB, FLA_Obj* A);

/* numerics (FLA_DOUBLE views; pivots FLA_INT) */
FLA_Error FLA_Gemm(FLA_Trans ta, FLA_Trans tb, FLA_Obj alpha, FLA_Obj A, FLA_Obj B, FLA_Obj beta, FLA_Obj C);
FLA_Error FLA_Trsm(FLA_Side side, FLA_Uplo uplo, FLA_Trans trans, FLA_Diag diag, FLA_Obj alpha, FLA_Obj A,
                   FLA_Obj B);
FLA_Error FLA_Trmm(FLA_Side side, FLA_Uplo uplo, FLA_Trans trans, FLA_Diag diag, FLA_Obj alpha, FLA_Obj A,
                   FLA_Obj B);
FLA_Error FLA_Syrk(FLA_Uplo uplo, FLA_Trans trans, FLA_Obj alpha, FLA_Obj A, FLA_Obj beta, FLA_Obj C);
FLA_Error FLA_Chol(FLA_Uplo uplo, FLA_Obj A);
FLA_Error FLA_LU_nopiv(FLA_Obj A);
FLA_Error FLA_LU_piv(FLA_Obj A, FLA_Obj p);
FLA_Error FLA_Apply_pivots(FLA_Side side, FLA_Trans trans, FLA_Obj p, FLA_Obj A);
FLA_Error FLA_Axpy(FLA_Obj alpha, FLA_Obj A, FLA_Obj B);
FLA_Error FLA_Axpyt(FLA_Trans trans, FLA_Obj alpha, FLA_Obj A, FLA_Obj B);
FLA_Error FLA_Copy(FLA_Obj A, FLA_Obj B);
FLA_Error FLA_Copyt(FLA_Trans trans, FLA_Obj A, FLA_Obj B);
FLA_Error FLA_Scal(FLA_Obj alpha, FLA_Obj A);
FLA_Error FLA_Norm1(FLA_Obj A, FLA_Obj norm);
FLA_Error FLA_Norm_inf(FLA_Obj A, FLA_Obj norm);
FLA_Error FLA_Dot(FLA_Obj x, FLA_Obj y, FLA_Obj rho);
FLA_Error FLA_Triangularize(FLA_Uplo uplo, FLA_Diag diag, FLA_Obj A);
FLA_Error FLA_Obj_set_to_scalar(FLA_Obj alpha, FLA_Obj A);
FLA_Error FLA_Random_matrix(FLA_Obj A);
FLA_Error FLA_Random_spd_matrix(FLA_Uplo uplo, FLA_Obj A);

/* QR family: stubs (abort) */
FLA_Error FLA_QR_UT(FLA_Obj A, FLA_Obj T);
FLA_Error FLA_QR_UT_blk_var2(FLA_Obj A, FLA_Obj T, fla_qrut_t* cntl);
FLA_Error FLA_QR2_UT_internal(FLA_Obj U, FLA_Obj D, FLA_Obj T, fla_qr2ut_t* cntl);
FLA_Error FLA_QR2_UT_inc_blk_var1(FLA_Obj U, FLA_Obj D, FLA_Obj T, fla_qr2ut_t* cntl);
FLA_Error FLA_Apply_Q_UT(FLA_Side side, FLA_Trans trans, FLA_Direct direct, FLA_Store storev, FLA_Obj A,
                         FLA_Obj T, FLA_Obj W, FLA_Obj B);
FLA_Error FLA_Apply_Q2_UT_internal(FLA_Side side, FLA_Trans trans, FLA_Direct direct, FLA_Store storev,
                                   FLA_Obj D, FLA_Obj T, FLA_Obj W, FLA_Obj C, FLA_Obj E,
                                   fla_apq2ut_t* cntl);

/* GPU entry points referenced only by LINAL_GPU builds: not provided */

#endif
