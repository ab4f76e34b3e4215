// CBLAS stand-in for the oracle build (test infrastructure only). The
// reference declares cblas_dgemm / cblas_dcopy itself (tensor.cpp:21-22) and
// only needs the layout/transpose enumerations from this header.
#ifndef TJ_ORACLE_CBLAS_H
#define TJ_ORACLE_CBLAS_H
typedef enum CBLAS_LAYOUT { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
#endif
