// Declarations of the MKL sparse-BLAS names that the reference's
// include/FE/Matrix.h and src/FE/Matrix.C mention, so those files compile
// without MKL for the reference harness (ref_harness.cpp).  TEST
// INFRASTRUCTURE ONLY.  The harness never calls them: TMatrix::SetMklMatrix
// is not linked in, and the harness never destroys a TMatrix.
#ifndef REF_STUB_MKL_SPBLAS_H
#define REF_STUB_MKL_SPBLAS_H
typedef void *sparse_matrix_t;
typedef int sparse_status_t;
enum { SPARSE_STATUS_SUCCESS = 0, SPARSE_STATUS_NOT_SUPPORTED = 6 };
typedef enum { SPARSE_INDEX_BASE_ZERO = 0 } sparse_index_base_t;
typedef enum { SPARSE_MATRIX_TYPE_GENERAL = 20 } sparse_matrix_type_t;
struct matrix_descr {
  sparse_matrix_type_t type;
  int mode;
  int diag;
};
sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *, sparse_index_base_t, int, int, int *,
                                        int *, int *, double *);
sparse_status_t mkl_sparse_order(sparse_matrix_t);
sparse_status_t mkl_sparse_destroy(sparse_matrix_t);
#endif
