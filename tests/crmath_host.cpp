// Host build of the correctly rounded math used by the FP64 kernels, for
// tests/test_crmath_cpu.py (test infrastructure only).
#include "../collision_gb300/csrc/cc_crmath.cuh"

extern "C" {
void cr_eval(int fn, const double* a, const double* b, double* out, int n) {
    for (int i = 0; i < n; ++i) {
        switch (fn) {
            case 0: out[i] = ccg::cr::cos(a[i]); break;
            case 1: out[i] = ccg::cr::sin(a[i]); break;
            case 2: out[i] = ccg::cr::acos(a[i]); break;
            default: out[i] = ccg::cr::pow(a[i], b[i]); break;
        }
    }
}
void libm_eval(int fn, const double* a, const double* b, double* out, int n) {
    for (int i = 0; i < n; ++i) {
        switch (fn) {
            case 0: out[i] = ::cos(a[i]); break;
            case 1: out[i] = ::sin(a[i]); break;
            case 2: out[i] = ::acos(a[i]); break;
            default: out[i] = ::pow(a[i], b[i]); break;
        }
    }
}
}
