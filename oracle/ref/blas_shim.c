/*
 * ORACLE / TEST INFRASTRUCTURE ONLY (reference build).
 *
 * The reference links Intel MKL (makefile:21), which is not in this image.  The
 * LP64 BLAS/LAPACK routines it calls (tensor.cpp:11-18, lanczos_su2.cpp:12-15)
 * are forwarded to SciPy's bundled OpenBLAS, whose exports carry a "scipy_"
 * prefix.  OpenBLAS sums in a different order than MKL, so results agree with an
 * MKL build to rounding only (about 1e-16 per GEMM).
 */
void scipy_dgemm_(char*, char*, int*, int*, int*, double*, double*, int*, double*, int*, double*, double*, int*);
void scipy_dsyev_(char*, char*, int*, double*, int*, double*, double*, int*, int*);
void scipy_dsyevx_(char*, char*, char*, int*, double*, int*, double*, double*, int*, int*, double*, int*, double*, double*, int*, double*, int*, int*, int*, int*);
void scipy_dsyrk_(char*, char*, int*, int*, double*, double*, int*, double*, double*, int*);
void scipy_dposv_(char*, int*, int*, double*, int*, double*, int*, int*);
void scipy_dstev_(char*, int*, double*, double*, double*, int*, double*, int*);
void scipy_openblas_set_num_threads(int);

void dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* al, double* a, int* lda, double* b, int* ldb, double* be, double* c, int* ldc) {
  scipy_dgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc);
}
void dsyev_(char* jz, char* ul, int* n, double* a, int* lda, double* w, double* work, int* lwork, int* info) {
  scipy_dsyev_(jz, ul, n, a, lda, w, work, lwork, info);
}
void dsyevx_(char* jz, char* rg, char* ul, int* n, double* a, int* lda, double* vl, double* vu, int* il, int* iu, double* tol, int* m, double* w, double* z, int* ldz, double* work, int* lwork, int* iwork, int* ifail, int* info) {
  scipy_dsyevx_(jz, rg, ul, n, a, lda, vl, vu, il, iu, tol, m, w, z, ldz, work, lwork, iwork, ifail, info);
}
void dsyrk_(char* ul, char* tr, int* n, int* k, double* al, double* a, int* lda, double* be, double* c, int* ldc) {
  scipy_dsyrk_(ul, tr, n, k, al, a, lda, be, c, ldc);
}
void dposv_(char* ul, int* n, int* nrhs, double* a, int* lda, double* b, int* ldb, int* info) {
  scipy_dposv_(ul, n, nrhs, a, lda, b, ldb, info);
}
void dstev_(char* jz, int* n, double* d, double* e, double* z, int* ldz, double* work, int* info) {
  scipy_dstev_(jz, n, d, e, z, ldz, work, info);
}
void mkl_set_num_threads(int n) { scipy_openblas_set_num_threads(n); }
void mkl_set_dynamic(int flag) { (void)flag; }
