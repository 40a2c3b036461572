// Correctly rounded acos/cos/sin/pow for the oracle's CCO_CRMATH build
// (test infrastructure only). They are the library's double-double routines,
// which tests/test_crmath_cpu.py checks against high-precision evaluations;
// with them the oracle computes the reference's algorithm as the GPU path
// does, so a step where the two builds of the oracle differ is one where
// glibc's rounding decided the result.
#include "../collision_gb300/csrc/cc_crmath.cuh"

extern "C" {
double cco_cr_acos(double x) { return ccg::cr::acos(x); }
double cco_cr_cos(double x) { return ccg::cr::cos(x); }
double cco_cr_sin(double x) { return ccg::cr::sin(x); }
double cco_cr_pow(double x, double y) { return ccg::cr::pow(x, y); }
}
