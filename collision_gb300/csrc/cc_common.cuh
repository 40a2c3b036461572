// Shared definitions for the GB300 collision kernels.
//
// Every floating-point expression on the plain FP64 path is written in the
// reference's order of evaluation and compiled with --fmad=false, so that
// each a*b+c rounds twice exactly as the reference's x86 build does; the
// only results that can differ from the reference are those that pass
// through acos/cos/pow/sin (CUDA's libdevice versus glibc, an ulp or so).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace ccg {

// Reference constants: collid.h:17-19, AABB.cpp:10-16, dcollid.cpp:433,489,590.
constexpr double kMachEps = 2.220446049250313080847e-16;  // DBL_EPSILON (FronTier MACH_EPS)
constexpr double kRoundEps = 1e-10;
constexpr double kBoxPad = 1e-6;
constexpr double kBig = 1.0e38;
constexpr double kPi = 3.14159265358979323846;
constexpr int kMaxCcdIter = 5;
constexpr double kStrainTol = 0.10;
constexpr int kStrainMaxIter = 10;
constexpr int kTraversalStack = 64;

// Pass kinds, as recorded by the oracle.
enum PassKind { kPassProx = 0, kPassCcd = 1, kPassZone = 2 };

// Status codes of the C ABI (include/collision_gb300.h).
enum Status {
    kOk = 0,
    kBadInput = 1,
    kPairOverflow = 2,
    kStackOverflow = 3,
    kIterCap = 4,
    kNanDetected = 5,
    kCudaError = 6,
    kContactOverflow = 7,
    kNoMemory = 8,
};

// Device error word bits (set by kernels, read by the host after a pass).
enum ErrBits {
    kErrPairOverflow = 1,
    kErrStack = 2,
    kErrNan = 4,
    kErrContribOverflow = 8,
    kErrRecordOverflow = 16,
    kErrMergeOverflow = 32,
};

// One impulse contribution to one point, keyed by the reference's visiting
// order (query leaf rank, found leaf rank, sub-test index).
struct __align__(16) Contrib {
    unsigned long long key;
    int vertex;
    int flags;      // bit0: friction term present
    double imp[3];
    double fric[3];
};

// One narrow-phase visit, in the oracle's record format.
struct VisitRec {
    int pass, kind, a, b, status;
    int dcount[6];
    int rank_b, rank_a;
};

struct Params {
    double dt, thickness, eps, k, m, lambda, cr;
};

struct PassCounters {
    int npairs;       // candidate pairs written by the traversal
    int ncontrib;     // contributions written by the narrow phase
    int nhit_pairs;   // narrow-phase calls that returned true
    int nrec;         // visit records written
    int err;          // ErrBits
    int nvisits;      // narrow-phase calls (pairs not skipped as same-rigid-surface)
    int ncontacts;    // sub-tests that applied an impulse
    int nsub;         // sub-tests evaluated in FP64 (not rejected by a filter)
};

__device__ __forceinline__ double dot3(const double* a, const double* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
__device__ __forceinline__ double mag3(const double* a) { return sqrt(dot3(a, a)); }
__device__ __forceinline__ void cross3(const double* b, const double* c, double* ans) {
    ans[0] = b[1] * c[2] - b[2] * c[1];
    ans[1] = b[2] * c[0] - b[0] * c[2];
    ans[2] = b[0] * c[1] - b[1] * c[0];
}
__device__ __forceinline__ double sqr(double x) { return x * x; }
// std::min / std::max argument conventions (the reference's).
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

__device__ __forceinline__ void load3(const double4_32a* p, int i, double* o) {
    double4_32a v = p[i];
    o[0] = v.x; o[1] = v.y; o[2] = v.z;
}

}  // namespace ccg
