// oracle/shim/gcem.hpp -- TEST INFRASTRUCTURE ONLY.
// Empty stand-in for the reference's absent lib/gcem submodule; the reference
// includes it (structure_learning/IndependenceTest.h:19) but its PC-stable path
// only needs stats::pchisq, which oracle/shim/stats.hpp provides.
#pragma once
