// Build shim for compiling the reference's CPU path against SciPy's bundled OpenBLAS.
// The public CBLAS prototypes (LP64 ints) the reference headers call; every name is
// routed to the "scipy_"-prefixed export of libscipy_openblas. Test infrastructure only.
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
typedef int blasint;
typedef enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_ORDER;
typedef CBLAS_ORDER CBLAS_LAYOUT;
typedef enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113, CblasConjNoTrans = 114 } CBLAS_TRANSPOSE;
#define QLTG_SHIM(n) scipy_##n
#define cblas_sgemm QLTG_SHIM(cblas_sgemm)
#define cblas_dgemm QLTG_SHIM(cblas_dgemm)
#define cblas_cgemm QLTG_SHIM(cblas_cgemm)
#define cblas_zgemm QLTG_SHIM(cblas_zgemm)
#define cblas_saxpy QLTG_SHIM(cblas_saxpy)
#define cblas_daxpy QLTG_SHIM(cblas_daxpy)
#define cblas_caxpy QLTG_SHIM(cblas_caxpy)
#define cblas_zaxpy QLTG_SHIM(cblas_zaxpy)
#define cblas_sscal QLTG_SHIM(cblas_sscal)
#define cblas_dscal QLTG_SHIM(cblas_dscal)
#define cblas_cscal QLTG_SHIM(cblas_cscal)
#define cblas_zscal QLTG_SHIM(cblas_zscal)
#define cblas_scopy QLTG_SHIM(cblas_scopy)
#define cblas_dcopy QLTG_SHIM(cblas_dcopy)
#define cblas_ccopy QLTG_SHIM(cblas_ccopy)
#define cblas_zcopy QLTG_SHIM(cblas_zcopy)
#define cblas_sdot QLTG_SHIM(cblas_sdot)
#define cblas_ddot QLTG_SHIM(cblas_ddot)
#define cblas_snrm2 QLTG_SHIM(cblas_snrm2)
#define cblas_dnrm2 QLTG_SHIM(cblas_dnrm2)
#define cblas_scnrm2 QLTG_SHIM(cblas_scnrm2)
#define cblas_dznrm2 QLTG_SHIM(cblas_dznrm2)
#define cblas_cdotc_sub QLTG_SHIM(cblas_cdotc_sub)
#define cblas_zdotc_sub QLTG_SHIM(cblas_zdotc_sub)
#define cblas_sger QLTG_SHIM(cblas_sger)
#define cblas_dger QLTG_SHIM(cblas_dger)
#define cblas_cgeru QLTG_SHIM(cblas_cgeru)
#define cblas_zgeru QLTG_SHIM(cblas_zgeru)
#define cblas_somatcopy QLTG_SHIM(cblas_somatcopy)
#define cblas_domatcopy QLTG_SHIM(cblas_domatcopy)
#define cblas_comatcopy QLTG_SHIM(cblas_comatcopy)
#define cblas_zomatcopy QLTG_SHIM(cblas_zomatcopy)
#define openblas_set_num_threads QLTG_SHIM(openblas_set_num_threads)
void cblas_sgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, blasint, blasint, blasint, float, const float*, blasint, const float*, blasint, float, float*, blasint);
void cblas_dgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, blasint, blasint, blasint, double, const double*, blasint, const double*, blasint, double, double*, blasint);
void cblas_cgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, blasint, blasint, blasint, const void*, const void*, blasint, const void*, blasint, const void*, void*, blasint);
void cblas_zgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, blasint, blasint, blasint, const void*, const void*, blasint, const void*, blasint, const void*, void*, blasint);
void cblas_saxpy(blasint, float, const float*, blasint, float*, blasint);
void cblas_daxpy(blasint, double, const double*, blasint, double*, blasint);
void cblas_caxpy(blasint, const void*, const void*, blasint, void*, blasint);
void cblas_zaxpy(blasint, const void*, const void*, blasint, void*, blasint);
void cblas_sscal(blasint, float, float*, blasint);
void cblas_dscal(blasint, double, double*, blasint);
void cblas_cscal(blasint, const void*, void*, blasint);
void cblas_zscal(blasint, const void*, void*, blasint);
void cblas_scopy(blasint, const float*, blasint, float*, blasint);
void cblas_dcopy(blasint, const double*, blasint, double*, blasint);
void cblas_ccopy(blasint, const void*, blasint, void*, blasint);
void cblas_zcopy(blasint, const void*, blasint, void*, blasint);
float cblas_sdot(blasint, const float*, blasint, const float*, blasint);
double cblas_ddot(blasint, const double*, blasint, const double*, blasint);
float cblas_snrm2(blasint, const float*, blasint);
double cblas_dnrm2(blasint, const double*, blasint);
float cblas_scnrm2(blasint, const void*, blasint);
double cblas_dznrm2(blasint, const void*, blasint);
void cblas_cdotc_sub(blasint, const void*, blasint, const void*, blasint, void*);
void cblas_zdotc_sub(blasint, const void*, blasint, const void*, blasint, void*);
void cblas_sger(CBLAS_ORDER, blasint, blasint, float, const float*, blasint, const float*, blasint, float*, blasint);
void cblas_dger(CBLAS_ORDER, blasint, blasint, double, const double*, blasint, const double*, blasint, double*, blasint);
void cblas_cgeru(CBLAS_ORDER, blasint, blasint, const void*, const void*, blasint, const void*, blasint, void*, blasint);
void cblas_zgeru(CBLAS_ORDER, blasint, blasint, const void*, const void*, blasint, const void*, blasint, void*, blasint);
void cblas_somatcopy(CBLAS_ORDER, CBLAS_TRANSPOSE, blasint, blasint, float, const float*, blasint, float*, blasint);
void cblas_domatcopy(CBLAS_ORDER, CBLAS_TRANSPOSE, blasint, blasint, double, const double*, blasint, double*, blasint);
void cblas_comatcopy(CBLAS_ORDER, CBLAS_TRANSPOSE, blasint, blasint, const float*, const float*, blasint, float*, blasint);
void cblas_zomatcopy(CBLAS_ORDER, CBLAS_TRANSPOSE, blasint, blasint, const double*, const double*, blasint, double*, blasint);
void openblas_set_num_threads(int);
#ifdef __cplusplus
}
#endif
