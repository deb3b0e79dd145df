// oracle/shim/stats.hpp -- TEST INFRASTRUCTURE ONLY.
// Stand-in for the reference's absent `lib/stats` submodule, so that the
// reference's PC-stable sources compile into the oracle binary under
// oracle/_ref.  Only the one function the reference's CI test calls is
// provided (structure_learning/IndependenceTest.cpp:146, :268, :355):
// stats::pchisq(x, dof, log_form) = chi-square CDF, restated in
// oracle/igamma.h from the incomplete-gamma mathematics.
#pragma once
#include <cmath>
#include "../igamma.h"

namespace stats {
inline double pchisq(double x, double dof, bool log_form) {
    double p = oracle_pchisq(x, dof);
    return log_form ? std::log(p) : p;
}
}  // namespace stats
