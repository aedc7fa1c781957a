// Build shim: public LAPACKE prototypes (LP64) routed to SciPy's bundled OpenBLAS
// ("scipy_" prefix). Test infrastructure only.
#pragma once
#include <complex>
typedef int lapack_int;
#define lapack_complex_float std::complex<float>
#define lapack_complex_double std::complex<double>
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
#define QLTG_LSHIM(n) scipy_##n
extern "C" {
#define LAPACKE_sgesvd QLTG_LSHIM(LAPACKE_sgesvd)
#define LAPACKE_dgesvd QLTG_LSHIM(LAPACKE_dgesvd)
#define LAPACKE_cgesvd QLTG_LSHIM(LAPACKE_cgesvd)
#define LAPACKE_zgesvd QLTG_LSHIM(LAPACKE_zgesvd)
#define LAPACKE_sgesdd QLTG_LSHIM(LAPACKE_sgesdd)
#define LAPACKE_dgesdd QLTG_LSHIM(LAPACKE_dgesdd)
#define LAPACKE_cgesdd QLTG_LSHIM(LAPACKE_cgesdd)
#define LAPACKE_zgesdd QLTG_LSHIM(LAPACKE_zgesdd)
#define LAPACKE_sgeqrf QLTG_LSHIM(LAPACKE_sgeqrf)
#define LAPACKE_dgeqrf QLTG_LSHIM(LAPACKE_dgeqrf)
#define LAPACKE_cgeqrf QLTG_LSHIM(LAPACKE_cgeqrf)
#define LAPACKE_zgeqrf QLTG_LSHIM(LAPACKE_zgeqrf)
#define LAPACKE_sgelqf QLTG_LSHIM(LAPACKE_sgelqf)
#define LAPACKE_dgelqf QLTG_LSHIM(LAPACKE_dgelqf)
#define LAPACKE_cgelqf QLTG_LSHIM(LAPACKE_cgelqf)
#define LAPACKE_zgelqf QLTG_LSHIM(LAPACKE_zgelqf)
#define LAPACKE_sorgqr QLTG_LSHIM(LAPACKE_sorgqr)
#define LAPACKE_dorgqr QLTG_LSHIM(LAPACKE_dorgqr)
#define LAPACKE_cungqr QLTG_LSHIM(LAPACKE_cungqr)
#define LAPACKE_zungqr QLTG_LSHIM(LAPACKE_zungqr)
#define LAPACKE_sorglq QLTG_LSHIM(LAPACKE_sorglq)
#define LAPACKE_dorglq QLTG_LSHIM(LAPACKE_dorglq)
#define LAPACKE_cunglq QLTG_LSHIM(LAPACKE_cunglq)
#define LAPACKE_zunglq QLTG_LSHIM(LAPACKE_zunglq)
#define LAPACKE_ssyev QLTG_LSHIM(LAPACKE_ssyev)
#define LAPACKE_dsyev QLTG_LSHIM(LAPACKE_dsyev)
#define LAPACKE_cheev QLTG_LSHIM(LAPACKE_cheev)
#define LAPACKE_zheev QLTG_LSHIM(LAPACKE_zheev)
lapack_int LAPACKE_sgesvd(int, char, char, lapack_int, lapack_int, float*, lapack_int, float*, float*, lapack_int, float*, lapack_int, float*);
lapack_int LAPACKE_dgesvd(int, char, char, lapack_int, lapack_int, double*, lapack_int, double*, double*, lapack_int, double*, lapack_int, double*);
lapack_int LAPACKE_cgesvd(int, char, char, lapack_int, lapack_int, lapack_complex_float*, lapack_int, float*, lapack_complex_float*, lapack_int, lapack_complex_float*, lapack_int, float*);
lapack_int LAPACKE_zgesvd(int, char, char, lapack_int, lapack_int, lapack_complex_double*, lapack_int, double*, lapack_complex_double*, lapack_int, lapack_complex_double*, lapack_int, double*);
lapack_int LAPACKE_sgesdd(int, char, lapack_int, lapack_int, float*, lapack_int, float*, float*, lapack_int, float*, lapack_int);
lapack_int LAPACKE_dgesdd(int, char, lapack_int, lapack_int, double*, lapack_int, double*, double*, lapack_int, double*, lapack_int);
lapack_int LAPACKE_cgesdd(int, char, lapack_int, lapack_int, lapack_complex_float*, lapack_int, float*, lapack_complex_float*, lapack_int, lapack_complex_float*, lapack_int);
lapack_int LAPACKE_zgesdd(int, char, lapack_int, lapack_int, lapack_complex_double*, lapack_int, double*, lapack_complex_double*, lapack_int, lapack_complex_double*, lapack_int);
lapack_int LAPACKE_sgeqrf(int, lapack_int, lapack_int, float*, lapack_int, float*);
lapack_int LAPACKE_dgeqrf(int, lapack_int, lapack_int, double*, lapack_int, double*);
lapack_int LAPACKE_cgeqrf(int, lapack_int, lapack_int, lapack_complex_float*, lapack_int, lapack_complex_float*);
lapack_int LAPACKE_zgeqrf(int, lapack_int, lapack_int, lapack_complex_double*, lapack_int, lapack_complex_double*);
lapack_int LAPACKE_sgelqf(int, lapack_int, lapack_int, float*, lapack_int, float*);
lapack_int LAPACKE_dgelqf(int, lapack_int, lapack_int, double*, lapack_int, double*);
lapack_int LAPACKE_cgelqf(int, lapack_int, lapack_int, lapack_complex_float*, lapack_int, lapack_complex_float*);
lapack_int LAPACKE_zgelqf(int, lapack_int, lapack_int, lapack_complex_double*, lapack_int, lapack_complex_double*);
lapack_int LAPACKE_sorgqr(int, lapack_int, lapack_int, lapack_int, float*, lapack_int, const float*);
lapack_int LAPACKE_dorgqr(int, lapack_int, lapack_int, lapack_int, double*, lapack_int, const double*);
lapack_int LAPACKE_cungqr(int, lapack_int, lapack_int, lapack_int, lapack_complex_float*, lapack_int, const lapack_complex_float*);
lapack_int LAPACKE_zungqr(int, lapack_int, lapack_int, lapack_int, lapack_complex_double*, lapack_int, const lapack_complex_double*);
lapack_int LAPACKE_sorglq(int, lapack_int, lapack_int, lapack_int, float*, lapack_int, const float*);
lapack_int LAPACKE_dorglq(int, lapack_int, lapack_int, lapack_int, double*, lapack_int, const double*);
lapack_int LAPACKE_cunglq(int, lapack_int, lapack_int, lapack_int, lapack_complex_float*, lapack_int, const lapack_complex_float*);
lapack_int LAPACKE_zunglq(int, lapack_int, lapack_int, lapack_int, lapack_complex_double*, lapack_int, const lapack_complex_double*);
lapack_int LAPACKE_ssyev(int, char, char, lapack_int, float*, lapack_int, float*);
lapack_int LAPACKE_dsyev(int, char, char, lapack_int, double*, lapack_int, double*);
lapack_int LAPACKE_cheev(int, char, char, lapack_int, lapack_complex_float*, lapack_int, float*);
lapack_int LAPACKE_zheev(int, char, char, lapack_int, lapack_complex_double*, lapack_int, double*);
}
