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

#ifdef __CUDACC__
#include <cooperative_groups.h>
#include <cooperative_groups/scan.h>
#endif

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
    kErrUnionOverflow = 64,
    kErrSubOverflow = 128,
    // an index outside its array met in the broad phase (node, leaf,
    // element): the access is skipped and the call fails
    kErrIndexNode = 256,
    kErrIndexLeaf = 512,
    kErrIndexElem = 1024,
    // the pass stopped for the host (a tree to rebuild, buffers to grow):
    // nothing of it is applied, and it runs again afterwards
    kErrHost = 2048,
};
// Errors after which a pass's results are discarded (and the pass retried
// with larger buffers, or the call fails): the impulses are not applied.
constexpr int kErrRetry = kErrPairOverflow | kErrStack | kErrContribOverflow | kErrRecordOverflow |
                          kErrUnionOverflow | kErrSubOverflow | kErrHost;

// Candidate pairs found on swept boxes carry this bit in .y when the two
// elements' static boxes overlap too (the proximity pass's pairs).
constexpr int kPairStatic = (int)0x80000000u;
constexpr int kPairIdMask = 0x7fffffff;

// A sub-test that passed the FP32 filters, queued for the FP64 stage of a
// split narrow pass: its element pair's visiting-order key base, the pair's
// index (for the pair's hit flag), its scene, points and sub-test index.
struct __align__(8) SubRec {
    unsigned long long keybase;
    int pair;
    int scene;
    int p[4];
    int sub;
    int pad;
};

// One createImpZone(pts, 4) call of an impact-zone pass (dcollid.cpp:473-484),
// keyed by the reference's visiting order like a contribution: the host
// replays the calls in key order to rebuild the reference's union-find
// lists, whose member order fixes the summation order of the zone solve.
struct __align__(8) UnionRec {
    unsigned long long key;
    int p[4];
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

// Per-scene description on the device. Scenes are concatenated: points
// [v0, v0+nv), elements [e0, e0+ne), each scene's elements in its own order
// (triangles, then bonds).
// Scenes resolved together: each owns contiguous ranges of points and
// elements (triangles first, then bonds, as in its own mesh) and has its own
// parameters, domain box and strain-sweep schedule.
struct SceneDev {
    Params p;
    double lo[3], hi[3];  // domain box
    int v0, nv, e0, ne;   // point and element ranges
    int strain_hdr0;      // first level of its strain schedule (index into the level headers)
    int strain_levels;
    int strain_slots;     // shared-memory slots of its window sweep
    int wb_final0, wb_final1;  // write-backs after its last level
    int enabled;          // 0: left out of resolve calls (candidates pass through)
    int strain_e0, strain_ne;  // its strain edges
    int nt;               // triangles (its first nt elements)
};

// Per-pass state of a scene (written by the host before a pass, except
// hits, which the narrow phase counts, and root, which the BVH build sets).
enum SceneMode { kSceneIdle = 0, kSceneProx = 1, kSceneCcd = 2, kSceneZone = 3 };
struct SceneRun {
    int mode;   // SceneMode of the current pass
    int hits;   // narrow-phase calls that returned true in the current pass
    int pass;   // the scene's own pass index (for visit records)
    int root;   // the scene's subtree root in the LBVH (-1: fewer than 2 elements)
    int leaf0;  // first sorted leaf of the scene in this pass's LBVH (-1: not in it)
    int pad[3];
};

// Where a scene is in the pass sequence of resolveCollision
// (dcollid.cpp:323-356) during one call.
enum SeqState { kSeqDone = 0, kSeqProx, kSeqCcd, kSeqZone };

// The pass sequence of one scene on the device (the device-resident
// detection loop): state, CCD iteration, CCD and impact-zone passes run this
// step, hasCollision, status (kOk or kIterCap), the scene's first sorted
// leaf in the step's hierarchy, and the tree the host must rebuild
// (0 none, 1 the proximity tree, 2 the collision tree).
struct SceneCtl {
    int state, niter, nccd, nzone;
    int hcol, status, leafbase, rebuild;
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
    int ncr;          // coplanarity cubics whose roots were formed again correctly rounded
    int nunion;       // union records written (impact-zone passes)
    int nsub_pt;      // point-triangle sub-tests queued by a split pass
    int nsub_ee;      // edge-edge sub-tests queued by a split pass
    int npairq;       // pairs with a queued sub-test (split passes)
    int nzones;       // impact zones listed for the zone solve (impact-zone passes)
    int nmembers;     // their members
    int nseg;         // union-record segments, one per zone the pass's unions touch
};

// The device-resident detection loop's own state.
enum LoopHost { kHostRebuild = 1, kHostRetry = 2, kHostFatal = 4 };
enum LoopAcc {
    kAccPasses, kAccCcd, kAccZone, kAccPairs, kAccVisits, kAccHits, kAccContacts, kAccSub, kAccMovingVisits,
    kAccCr, kAccLeaves, kAccBroadPairs, kAccPathBytes, kAccZonePasses, kAccIters, kAccProxPairs, kAccQueries,
    kAccUnions, kNumAcc
};
struct LoopCtl {
    int host;       // LoopHost bits: the loop stopped for the host
    int err;        // the stopping pass's error bits
    int pending;    // the current pass's modes are set: run it again as it is
    int nact;       // scenes in the current pass
    int nact_e;     // their elements
    int nact_p;     // their points
    int nbroad;     // elements the broad phase boxes and walks (0: pairs reused, or stopped)
    int npts;       // points the pass's point kernels cover (0: stopped)
    int any_zone;   // a scene of the pass is in impact-zone mode
    int reuse;      // >= 0: the next pass takes this many pairs of the proximity pass
    int reuse_n;    // pairs the current pass took (-1: none)
    int zone_cap;   // impact-zone passes per scene and step
    unsigned serial;  // the current pass's serial (pass stamps), increasing across steps
    int prune;      // the pass queries only elements with a point the previous pass touched
    int prune_on;   // later passes may prune (CC_TUNE_PRUNE)
    int nq_full;    // queries of the pass's full traversal (0 when it prunes or reuses)
    int nquery;     // queries of the pruned traversal
    unsigned long long acc[kNumAcc];  // counters over the step's passes (LoopAcc)
    PassCounters stopped;  // the counters of the pass that stopped the loop (the sizes to grow to)
};


// One point's entry in the reference's union-find with member lists
// (UF{next_pt, root, tail, num_pts}, collid.h:22-27; makeSet, findSet,
// mergePoint, dcollid.cpp:1015-1059): parent, next member, last member and
// member count (the last two meaningful at a root).
struct __align__(16) UfNode {
    int root, next, tail, w;
};

#ifdef __CUDACC__
// atomicAdd(p, n) for every calling thread, one atomic per group of threads
// that arrive together (warp-aggregated); returns each thread's old value.
__device__ __forceinline__ int aggregated_add(int* p, int n) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    int incl = cg::inclusive_scan(g, n);
    int base = 0;
    if (g.thread_rank() == g.size() - 1) base = atomicAdd(p, incl);
    base = g.shfl(base, g.size() - 1);
    return base + incl - n;
}
#endif

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
