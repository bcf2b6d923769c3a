/* Stand-in for Intel MKL's header when building the reference here: only the
 * two thread-control calls that main_omp.cpp:153,156 makes are declared.  They
 * are implemented in blas_shim.c on top of SciPy's bundled OpenBLAS. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
void mkl_set_num_threads(int n);
void mkl_set_dynamic(int flag);
#ifdef __cplusplus
}
#endif
