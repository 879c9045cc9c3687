/* CBLAS declarations for building the chemtensor reference as a CPU oracle.
 * The implementation comes from the OpenBLAS build bundled with scipy, whose
 * exported symbols carry a "scipy_" prefix; every name is redirected here.
 * Only the routines the reference sources call are declared. */
#pragma once
#include <stddef.h>

typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_ORDER;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef CBLAS_ORDER CBLAS_LAYOUT;
typedef int blasint;

#define CBLAS_REDIRECT(name) scipy_##name

#define cblas_sgemm  CBLAS_REDIRECT(cblas_sgemm)
#define cblas_dgemm  CBLAS_REDIRECT(cblas_dgemm)
#define cblas_cgemm  CBLAS_REDIRECT(cblas_cgemm)
#define cblas_zgemm  CBLAS_REDIRECT(cblas_zgemm)
#define cblas_sger   CBLAS_REDIRECT(cblas_sger)
#define cblas_dger   CBLAS_REDIRECT(cblas_dger)
#define cblas_cgeru  CBLAS_REDIRECT(cblas_cgeru)
#define cblas_zgeru  CBLAS_REDIRECT(cblas_zgeru)
#define cblas_saxpy  CBLAS_REDIRECT(cblas_saxpy)
#define cblas_daxpy  CBLAS_REDIRECT(cblas_daxpy)
#define cblas_caxpy  CBLAS_REDIRECT(cblas_caxpy)
#define cblas_zaxpy  CBLAS_REDIRECT(cblas_zaxpy)
#define cblas_sscal  CBLAS_REDIRECT(cblas_sscal)
#define cblas_dscal  CBLAS_REDIRECT(cblas_dscal)
#define cblas_cscal  CBLAS_REDIRECT(cblas_cscal)
#define cblas_zscal  CBLAS_REDIRECT(cblas_zscal)
#define cblas_csscal CBLAS_REDIRECT(cblas_csscal)
#define cblas_zdscal CBLAS_REDIRECT(cblas_zdscal)
#define cblas_snrm2  CBLAS_REDIRECT(cblas_snrm2)
#define cblas_dnrm2  CBLAS_REDIRECT(cblas_dnrm2)
#define cblas_scnrm2 CBLAS_REDIRECT(cblas_scnrm2)
#define cblas_dznrm2 CBLAS_REDIRECT(cblas_dznrm2)
#define cblas_ddot   CBLAS_REDIRECT(cblas_ddot)
#define cblas_zdotc_sub CBLAS_REDIRECT(cblas_zdotc_sub)

void cblas_sgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, blasint, blasint, blasint, float, const float*, blasint, const float*, blasint, float, float*, blasint);
void cblas_dgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, blasint, blasint, blasint, double, const double*, blasint, const double*, blasint, double, double*, blasint);
void cblas_cgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, blasint, blasint, blasint, const void*, const void*, blasint, const void*, blasint, const void*, void*, blasint);
void cblas_zgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, blasint, blasint, blasint, const void*, const void*, blasint, const void*, blasint, const void*, void*, blasint);
void cblas_sger(CBLAS_ORDER, blasint, blasint, float, const float*, blasint, const float*, blasint, float*, blasint);
void cblas_dger(CBLAS_ORDER, blasint, blasint, double, const double*, blasint, const double*, blasint, double*, blasint);
void cblas_cgeru(CBLAS_ORDER, blasint, blasint, const void*, const void*, blasint, const void*, blasint, void*, blasint);
void cblas_zgeru(CBLAS_ORDER, blasint, blasint, const void*, const void*, blasint, const void*, blasint, void*, blasint);
void cblas_saxpy(blasint, float, const float*, blasint, float*, blasint);
void cblas_daxpy(blasint, double, const double*, blasint, double*, blasint);
void cblas_caxpy(blasint, const void*, const void*, blasint, void*, blasint);
void cblas_zaxpy(blasint, const void*, const void*, blasint, void*, blasint);
void cblas_sscal(blasint, float, float*, blasint);
void cblas_dscal(blasint, double, double*, blasint);
void cblas_cscal(blasint, const void*, void*, blasint);
void cblas_zscal(blasint, const void*, void*, blasint);
void cblas_csscal(blasint, float, void*, blasint);
void cblas_zdscal(blasint, double, void*, blasint);
float  cblas_snrm2(blasint, const float*, blasint);
double cblas_dnrm2(blasint, const double*, blasint);
float  cblas_scnrm2(blasint, const void*, blasint);
double cblas_dznrm2(blasint, const void*, blasint);
double cblas_ddot(blasint, const double*, blasint, const double*, blasint);
void cblas_zdotc_sub(blasint, const void*, blasint, const void*, blasint, void*);
