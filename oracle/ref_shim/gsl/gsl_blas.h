/* Declarations only, so that the reference's numerical.cu parses in a
 * device-only compile (oracle/ref_build.py).  No GSL code is compiled or
 * linked: the host functions that call these are never built. */
#pragma once
#include <stddef.h>
typedef struct gsl_vector gsl_vector;
typedef struct gsl_matrix gsl_matrix;
typedef struct gsl_eigen_symmv_workspace gsl_eigen_symmv_workspace;
gsl_vector *gsl_vector_alloc(size_t n);
void gsl_vector_set(gsl_vector *v, size_t i, double x);
double gsl_vector_get(const gsl_vector *v, size_t i);
void gsl_vector_free(gsl_vector *v);
gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2);
void gsl_matrix_set(gsl_matrix *m, size_t i, size_t j, double x);
double gsl_matrix_get(const gsl_matrix *m, size_t i, size_t j);
void gsl_matrix_free(gsl_matrix *m);
gsl_eigen_symmv_workspace *gsl_eigen_symmv_alloc(size_t n);
int gsl_eigen_symmv(gsl_matrix *A, gsl_vector *eval, gsl_matrix *evec, gsl_eigen_symmv_workspace *w);
