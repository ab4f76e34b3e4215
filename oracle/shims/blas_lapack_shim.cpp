// BLAS / LAPACK stand-ins for the oracle build (test infrastructure only).
//
// The reference calls, at 3x3 size only:
//   * cblas_dgemm (tensor.cpp:81-115) -- restated here as the textbook triple
//     loop with the k sum innermost and in increasing order, which is the
//     netlib reference BLAS summation order for each element;
//   * cblas_dcopy (tensor.cpp:534-541);
//   * dgesdd_ (tensor.cpp:51-71), reached on the hot path only through
//     matrixSquareRoot (tensor.cpp:452-475) from cleanUpV
//     (boxaccesscellarray.cpp:510-512), always on the symmetric positive
//     definite V V^T. For such input the SVD is the eigendecomposition, which
//     this shim computes with cyclic Jacobi rotations (Golub & Van Loan,
//     "Matrix Computations", sec. 8.5). Singular values are returned in
//     decreasing order with U = Q and VT = Q^T.
//   * dgeev_ is referenced only by find3x3EigenValues, which is never called
//     on the path; it fails loudly.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include "cblas.h"

void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int M, int N, int K, double alpha,
                 const double* A, int lda, const double* B, int ldb, double beta, double* C, int ldc)
{
    if (layout != CblasRowMajor) { std::fprintf(stderr, "oracle cblas_dgemm: row-major only\n"); std::abort(); }
    for (int i = 0; i < M; ++i)
        for (int j = 0; j < N; ++j) {
            double s = 0.0;
            for (int l = 0; l < K; ++l) {
                double a = (ta == CblasNoTrans) ? A[i * lda + l] : A[l * lda + i];
                double b = (tb == CblasNoTrans) ? B[l * ldb + j] : B[j * ldb + l];
                s += a * b;
            }
            double c = alpha * s;
            if (beta != 0.0) c += beta * C[i * ldc + j];
            C[i * ldc + j] = c;
        }
}

void cblas_dcopy(const int N, const double* X, const int incX, double* Y, const int incY)
{
    for (int i = 0; i < N; ++i) Y[i * incY] = X[i * incX];
}

// Symmetric 3x3 eigendecomposition by cyclic Jacobi. a is row-major and
// symmetric; on return w holds the eigenvalues (decreasing) and q the
// eigenvectors as columns (row-major q[r*3+c] = component r of vector c).
static void oracle_sym3_eig(const double* a_in, double* w, double* q)
{
    double a[9];
    for (int i = 0; i < 9; ++i) a[i] = a_in[i];
    for (int i = 0; i < 9; ++i) q[i] = (i % 4 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = std::fabs(a[1]) + std::fabs(a[2]) + std::fabs(a[5]);
        if (off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int r = p + 1; r < 3; ++r) {
                double apr = a[p * 3 + r];
                if (apr == 0.0) continue;
                double app = a[p * 3 + p], arr = a[r * 3 + r];
                double theta = (arr - app) / (2.0 * apr);
                double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0);
                double s = t * c;
                for (int k = 0; k < 3; ++k) {  // A <- A J (columns p, r)
                    double akp = a[k * 3 + p], akr = a[k * 3 + r];
                    a[k * 3 + p] = c * akp - s * akr;
                    a[k * 3 + r] = s * akp + c * akr;
                }
                for (int k = 0; k < 3; ++k) {  // A <- J^T A (rows p, r)
                    double apk = a[p * 3 + k], ark = a[r * 3 + k];
                    a[p * 3 + k] = c * apk - s * ark;
                    a[r * 3 + k] = s * apk + c * ark;
                }
                a[p * 3 + r] = 0.0;
                a[r * 3 + p] = 0.0;
                for (int k = 0; k < 3; ++k) {  // Q <- Q J
                    double qkp = q[k * 3 + p], qkr = q[k * 3 + r];
                    q[k * 3 + p] = c * qkp - s * qkr;
                    q[k * 3 + r] = s * qkp + c * qkr;
                }
            }
    }
    int order[3] = {0, 1, 2};
    double d[3] = {a[0], a[4], a[8]};
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (d[order[j]] > d[order[i]]) { int t = order[i]; order[i] = order[j]; order[j] = t; }
    double qs[9];
    for (int c = 0; c < 3; ++c) {
        w[c] = d[order[c]];
        for (int r = 0; r < 3; ++r) qs[r * 3 + c] = q[r * 3 + order[c]];
    }
    for (int i = 0; i < 9; ++i) q[i] = qs[i];
}

extern "C" {

void dgesdd_(char* jobz, int* m, int* n, double* A, int* lda, double* S, double* U, int* ldu, double* VT, int* ldvt,
             double* work, int* lwork, int* iwork, int* info)
{
    (void)jobz; (void)work; (void)lwork; (void)iwork;
    if (*m != 3 || *n != 3 || *lda != 3 || *ldu != 3 || *ldvt != 3) {
        std::fprintf(stderr, "oracle dgesdd_: 3x3 only\n");
        std::abort();
    }
    // Column-major A: element (r,c) at A[c*3+r]. Symmetric input only.
    double a[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) a[r * 3 + c] = A[c * 3 + r];
    for (int r = 0; r < 3; ++r)
        for (int c = r + 1; c < 3; ++c)
            if (a[r * 3 + c] != a[c * 3 + r]) {
                std::fprintf(stderr, "oracle dgesdd_: symmetric input only\n");
                std::abort();
            }
    double w[3], q[9];
    oracle_sym3_eig(a, w, q);
    for (int i = 0; i < 3; ++i) S[i] = w[i];
    // U = Q (column-major), VT = Q^T (column-major).
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            U[c * 3 + r] = q[r * 3 + c];
            VT[c * 3 + r] = q[c * 3 + r];
        }
    *info = 0;
}

int dgeev_(char*, char*, int*, double*, int*, double*, double*, double*, int*, double*, int*, double*, int*, int*)
{
    std::fprintf(stderr, "oracle dgeev_: not on the path\n");
    std::abort();
    return -1;
}
}
