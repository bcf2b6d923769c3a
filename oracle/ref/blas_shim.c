/*
 * ORACLE / TEST INFRASTRUCTURE ONLY (reference build).
 *
 * The reference links Intel MKL (makefile:21), which is not in this image.  The
 * LP64 BLAS/LAPACK routines it calls (tensor.cpp:11-18, lanczos_su2.cpp:12-15)
 * are forwarded to SciPy's bundled OpenBLAS, whose exports carry a "scipy_"
 * prefix.  OpenBLAS sums in a different order than MKL, so results agree with an
 * MKL build to rounding only (about 1e-16 per GEMM).
 *
 * The signs of the eigenvectors dsyev and dstev return are LAPACK's free
 * choice (MKL and OpenBLAS need not agree), and the reference fixes none.
 * su2ref_set_sign_convention(1) fixes one, the rule the GPU engine applies to
 * its own eigenvectors: in each column the first entry whose magnitude exceeds
 * 1e-4 of the column's largest is made positive.  Off by default.
 */
void scipy_dgemm_(char*, char*, int*, int*, int*, double*, double*, int*, double*, int*, double*, double*, int*);
void scipy_dsyev_(char*, char*, int*, double*, int*, double*, double*, int*, int*);
void scipy_dsyevx_(char*, char*, char*, int*, double*, int*, double*, double*, int*, int*, double*, int*, double*, double*, int*, double*, int*, int*, int*, int*);
void scipy_dsyrk_(char*, char*, int*, int*, double*, double*, int*, double*, double*, int*);
void scipy_dposv_(char*, int*, int*, double*, int*, double*, int*, int*);
void scipy_dstev_(char*, int*, double*, double*, double*, int*, double*, int*);
void scipy_openblas_set_num_threads(int);

/* Lanczos length of the warm-up (patch_ref.py hooks dmrg_su2.cpp:530 to it) */
int su2ref_idmrg_mlanc = 5;
void su2ref_set_idmrg_mlanc(int m) { su2ref_idmrg_mlanc = m; }

/* The -seed option of the parity runs (patch_ref.py hooks dmrg_su2_omp.cpp:79
 * to it): when set, the warm-up starts each two-site step from
 * random_initialize_tensor instead of initialize_input_vector, the generator
 * seeded once here with initran (the reference seeds it from the clock,
 * main_omp.cpp:39-41).  Off by default. */
int su2ref_seeded = 0;
void initran_(const int* w);
void su2ref_set_seed(int seed) {
  su2ref_seeded = 1;
  initran_(&seed);
}
void su2ref_clear_seed(void) { su2ref_seeded = 0; }

static int sign_convention = 0;
void su2ref_set_sign_convention(int on) { sign_convention = on; }

static void canonical_signs(int rows, int cols, double* z, int ld) {
  for (int c = 0; c < cols; ++c) {
    double* col = z + (long)c * ld;
    double mx = 0;
    for (int i = 0; i < rows; ++i) mx = col[i] > mx ? col[i] : (-col[i] > mx ? -col[i] : mx);
    for (int i = 0; i < rows; ++i)
      if (col[i] > 1e-4 * mx || -col[i] > 1e-4 * mx) {
        if (col[i] < 0)
          for (int k = 0; k < rows; ++k) col[k] = -col[k];
        break;
      }
  }
}

void dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* al, double* a, int* lda, double* b, int* ldb, double* be, double* c, int* ldc) {
  scipy_dgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc);
}
void dsyev_(char* jz, char* ul, int* n, double* a, int* lda, double* w, double* work, int* lwork, int* info) {
  scipy_dsyev_(jz, ul, n, a, lda, w, work, lwork, info);
  if (sign_convention && (*jz == 'V' || *jz == 'v') && *lwork != -1 && *info == 0) canonical_signs(*n, *n, a, *lda);
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
  if (sign_convention && (*jz == 'V' || *jz == 'v') && *info == 0) canonical_signs(*n, *n, z, *ldz);
}
void mkl_set_num_threads(int n) { scipy_openblas_set_num_threads(n); }
void mkl_set_dynamic(int flag) { (void)flag; }
