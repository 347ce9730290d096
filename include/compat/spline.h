/*
 * spline.h -- the reference's cubic-spline interface (spline.h of
 * ren5885a/SCFT_Ver1.01) for the GB300 build: the same four functions with
 * the same arguments, implemented by the library's scft_spline* entry points
 * (../scft_capi.h).  Results are bit-identical to the reference's spline.c.
 */
#ifndef SCFT_GB300_COMPAT_SPLINE_H
#define SCFT_GB300_COMPAT_SPLINE_H

#include "../scft_capi.h"

/* Cubic spline coefficients */
static inline int spline(int n, int e1, int e2, double s1, double s2, double x[], double y[],
                         double b[], double c[], double d[], int *flag) {
  scft_spline(n, e1, e2, s1, s2, x, y, b, c, d, flag);
  return 0;
}
/* spline evaluation */
static inline double seval(int n, double xx, double x[], double y[], double b[], double c[],
                           double d[], int *last) {
  return scft_spline_eval(n, xx, x, y, b, c, d, last);
}
/* derivative evaluation */
static inline double deriv(int n, double xx, double x[], double b[], double c[], double d[],
                           int *last) {
  return scft_spline_deriv(n, xx, x, b, c, d, last);
}
/* integral of spline */
static inline double sinteg(int n, double u, double x[], double y[], double b[], double c[],
                            double d[], int *last) {
  return scft_spline_integral(n, u, x, y, b, c, d, last);
}

#endif
