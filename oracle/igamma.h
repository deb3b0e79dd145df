/*
 * oracle/igamma.h -- TEST INFRASTRUCTURE ONLY (part of the oracle).
 *
 * Chi-square upper-tail p-value used by the CPU oracle and by the shim that
 * lets the reference's own PC-stable sources compile without their absent
 * third-party math submodules.
 *
 * The reference scores every CI test with
 *     p = 1.0 - stats::pchisq(g2, df, false)
 * (structure_learning/IndependenceTest.cpp:146, :268, :355), where
 * stats::pchisq(x, k) is the chi-square CDF, i.e. the regularised lower
 * incomplete gamma P(k/2, x/2).  That function lives in the un-vendored
 * `lib/stats` + `lib/gcem` submodules (no pinned version, source absent), so
 * it is restated here from the mathematics (Press et al., Numerical Recipes,
 * 3rd ed. section 6.2; DLMF 8.7.1 and 8.9.2):
 *   - x <  a + 1 : P(a,x) = x^a e^-x / Gamma(a) * sum_n x^n / (a (a+1) ... (a+n))
 *   - x >= a + 1 : Q(a,x) by the Legendre continued fraction evaluated with the
 *                  modified Lentz method; P = 1 - Q.
 * Parity for p-values against the reference's library is therefore unpinned
 * at the last-bits level; decisions are pinned through the reference's own
 * golden CPDAG (dataset/alarm/alarm_s5000_struct).
 */
#ifndef FPGM_ORACLE_IGAMMA_H
#define FPGM_ORACLE_IGAMMA_H

#include <math.h>

#define ORACLE_IGAMMA_EPS 1e-16
#define ORACLE_IGAMMA_TINY 1e-300
#define ORACLE_IGAMMA_MAXIT (1 << 22)

static inline double oracle_igamma_lower_series(double a, double x) {
    double ap = a, term = 1.0 / a, sum = term;
    for (int n = 1; n < ORACLE_IGAMMA_MAXIT; ++n) {
        ap += 1.0;
        term *= x / ap;
        sum += term;
        if (fabs(term) < fabs(sum) * ORACLE_IGAMMA_EPS) break;
    }
    return sum * exp(-x + a * log(x) - lgamma(a));
}

static inline double oracle_igamma_upper_cf(double a, double x) {
    double b = x + 1.0 - a;
    double c = 1.0 / ORACLE_IGAMMA_TINY;
    double d = 1.0 / b;
    double h = d;
    for (int i = 1; i < ORACLE_IGAMMA_MAXIT; ++i) {
        double an = -i * (i - a);
        b += 2.0;
        d = an * d + b;
        if (fabs(d) < ORACLE_IGAMMA_TINY) d = ORACLE_IGAMMA_TINY;
        c = b + an / c;
        if (fabs(c) < ORACLE_IGAMMA_TINY) c = ORACLE_IGAMMA_TINY;
        d = 1.0 / d;
        double del = d * c;
        h *= del;
        if (fabs(del - 1.0) < ORACLE_IGAMMA_EPS) break;
    }
    return exp(-x + a * log(x) - lgamma(a)) * h;
}

/* Regularised lower incomplete gamma P(a, x), a > 0. */
static inline double oracle_igamma_p(double a, double x) {
    if (!(x > 0.0)) return 0.0;
    if (x < a + 1.0) return oracle_igamma_lower_series(a, x);
    return 1.0 - oracle_igamma_upper_cf(a, x);
}

/* Chi-square CDF with `dof` degrees of freedom (the quantity stats::pchisq returns). */
static inline double oracle_pchisq(double x, double dof) {
    return oracle_igamma_p(0.5 * dof, 0.5 * x);
}

/* The reference's p-value: 1 - CDF (IndependenceTest.cpp:146). */
static inline double oracle_chisq_pvalue(double g2, int df) {
    return 1.0 - oracle_pchisq(g2, (double)df);
}

#endif
