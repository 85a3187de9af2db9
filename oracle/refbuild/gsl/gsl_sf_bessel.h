/* gsl_sf_bessel.h -- the two GSL functions the reference calls
 * (kernel/bessel_i0.c:375, bessel_i1.c:570), provided by the oracle's power
 * series (TEST INFRASTRUCTURE). */
#ifndef ORACLE_REFBUILD_GSL_SF_BESSEL_H
#define ORACLE_REFBUILD_GSL_SF_BESSEL_H
double gsl_sf_bessel_I0(double x);
double gsl_sf_bessel_I1(double x);
#endif
