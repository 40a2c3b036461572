// Narrow-phase pass over the candidate pairs: one thread per pair.
//
// The reference visits each overlapping pair once, as (a = the leaf found
// later in its tree's inorder, b = the query leaf), in (b, a) inorder
// (AABB.cpp:254-343), and dispatches it by element type (isProximity /
// isCollision, dcollid.cpp:753-836). Here every pair is oriented by the
// leaf ranks of the reference tree, and each impulse contribution carries the
// key (rank b, rank a, sub-test) so the per-point sums can be formed later in
// exactly the reference's order.
#include "cc_launch.h"
#include "cc_narrow.cuh"

namespace ccg {

namespace {

template <bool MOVING>
__global__ void __launch_bounds__(128) k_narrow(NarrowArgs a, int max_pairs) {
    NarrowCtx c;
    c.xo = a.xo; c.av = a.av; c.fixed = a.fixed; c.ev = a.ev; c.esurf = a.esurf; c.erigid = a.erigid;
    c.vbody = a.vbody; c.body_mass = a.body_mass; c.body_slot0 = a.body_slot0;
    c.rank = a.rank;
    c.contrib = a.contrib; c.contrib_cap = a.contrib_cap; c.ctr = a.ctr; c.urec = a.urec;
    c.urec_cap = a.urec_cap;
    c.rec = a.rec; c.rec_cap = a.rec_cap;
    c.pbox_lo = a.pbox_lo; c.pbox_hi = a.pbox_hi; c.p32 = a.p32; c.v32 = a.v32;
    c.check = a.check;
    c.robust_roots = 0;
    int np = a.ctr->npairs;
    if (np > max_pairs) np = max_pairs;
    // counters summed per thread, added once per warp at the end
    int t_visits = 0, t_sub = 0, t_hits = 0, t_cr = 0, t_contacts = 0;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x) {
        int2 pr = a.pairs[idx];
        if (!MOVING && a.static_only && !(pr.y & kPairStatic)) continue;
        pr.y &= kPairIdMask;
        int sc = a.escene[pr.x];
        const SceneRun run = a.run[sc];
        c.p = a.scenes[sc].p;
        c.zone = run.mode == kSceneZone && !a.check;
        c.pass = run.pass;
        // h of the sub-tests (thickness for proximity, eps for CCD) and the
        // barycentric tolerance eps, rounded up to FP32
        c.hpad = __double2float_ru(MOVING ? c.p.eps : c.p.thickness);
        c.epad = __double2float_ru(c.p.eps);
        c.dt32 = __double2float_ru(c.p.dt);
        int ri = c.rank ? c.rank[pr.x] : pr.x, rj = c.rank ? c.rank[pr.y] : pr.y;
        int ea = ri > rj ? pr.x : pr.y;  // found leaf
        int eb = ri > rj ? pr.y : pr.x;  // query leaf
        int ra = ri > rj ? ri : rj, rb = ri > rj ? rj : ri;
        bool ta = c.ev[3 * ea + 2] >= 0, tb = c.ev[3 * eb + 2] >= 0;
        int kind = (ta && tb) ? 0 : (!ta && !tb) ? 2 : 1;
        if (kind == 0 && c.esurf[ea] == c.esurf[eb] && c.erigid[ea]) continue;  // dcollid.cpp:762-763, 805-806
        // tri-bond pairs are always handed over as (tri, bond)
        int e1 = (kind == 1 && !ta) ? eb : ea;
        int e2 = (kind == 1 && !ta) ? ea : eb;
        const int* P1 = c.ev + 3 * e1;
        const int* P2 = c.ev + 3 * e2;
        CallState st;
        st.keybase = ((unsigned long long)rb << 26) | ((unsigned long long)ra << 4);
        int n1 = (P1[2] >= 0) ? 3 : 2, n2 = (P2[2] >= 0) ? 3 : 2;
        st.np = n1 + n2;
        for (int i = 0; i < 6; ++i) { st.dcount[i] = 0; st.plist[i] = -1; }
        for (int i = 0; i < n1; ++i) st.plist[i] = P1[i];
        for (int i = 0; i < n2; ++i) st.plist[n1 + i] = P2[i];
        st.sub = 0;
        st.nsub = 0;
        st.ncr = 0;
        st.ncontacts = 0;
        int A[3] = {P1[0], P1[1], n1 == 3 ? P1[2] : -1};
        int B[3] = {P2[0], P2[1], n2 == 3 ? P2[2] : -1};
        bool status;
        if (c.pbox_lo && !pair_may_hit<MOVING>(c, A, n1, B, n2))
            status = false;  // no sub-test of the pair can hit
        else if (kind == 0)
            status = tri_to_tri<MOVING>(c, st, A, B);
        else if (kind == 1)
            status = tri_to_bond<MOVING>(c, st, A, B);
        else
            status = bond_to_bond<MOVING>(c, st, A, B);
        t_visits++;
        t_sub += st.nsub;
        t_cr += st.ncr;
        t_contacts += st.ncontacts;
        if (status) {
            t_hits++;
            atomicAdd(&a.run[sc].hits, 1);
            for (int q = 0; q < 3; ++q) {
                if (A[q] >= 0) stamp_point(a.ps, A[q]);
                if (B[q] >= 0) stamp_point(a.ps, B[q]);
            }
        }
        if (c.rec) {
            int slot = atomicAdd(&c.ctr->nrec, 1);
            if (slot < c.rec_cap) {
                VisitRec& r = c.rec[slot];
                r.pass = c.pass; r.kind = kind; r.a = e1; r.b = e2; r.status = status ? 1 : 0;
                for (int i = 0; i < 6; ++i) r.dcount[i] = st.dcount[i];
                r.rank_b = rb; r.rank_a = ra;
            } else {
                atomicOr(&c.ctr->err, kErrRecordOverflow);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        t_visits += __shfl_xor_sync(0xffffffffu, t_visits, o);
        t_sub += __shfl_xor_sync(0xffffffffu, t_sub, o);
        t_hits += __shfl_xor_sync(0xffffffffu, t_hits, o);
        t_cr += __shfl_xor_sync(0xffffffffu, t_cr, o);
        t_contacts += __shfl_xor_sync(0xffffffffu, t_contacts, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (t_visits) atomicAdd(&c.ctr->nvisits, t_visits);
        if (t_sub) atomicAdd(&c.ctr->nsub, t_sub);
        if (t_hits) atomicAdd(&c.ctr->nhit_pairs, t_hits);
        if (t_cr) atomicAdd(&c.ctr->ncr, t_cr);
        if (t_contacts) atomicAdd(&c.ctr->ncontacts, t_contacts);
    }
}

// The sub-tests of an element pair in the order of tri_to_tri /
// tri_to_bond / bond_to_bond (A the found element, B the query element):
// f(sub, pts, ee) for each.
template <bool MOVING, class F>
__device__ __forceinline__ void for_each_subtest(int kind, const int* A, const int* B, F&& f) {
    int pts[4];
    if (kind == 0) {
        int sub = 0;
        for (int k = 0; k < 2; ++k)
            for (int i = 0; i < 3; ++i, ++sub) {
                // proximity tests B's triangle against A's points first; CCD the reverse
                const int* tri = MOVING ? ((k == 0) ? A : B) : ((k == 0) ? B : A);
                const int* pt = MOVING ? ((k == 0) ? B : A) : ((k == 0) ? A : B);
                pts[0] = tri[0]; pts[1] = tri[1]; pts[2] = tri[2]; pts[3] = pt[i];
                f(sub, pts, false);
            }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j, ++sub) {
                pts[0] = A[i]; pts[1] = A[(i + 1) % 3]; pts[2] = B[j]; pts[3] = B[(j + 1) % 3];
                f(sub, pts, true);
            }
    } else if (kind == 1) {
        pts[0] = A[0]; pts[1] = A[1]; pts[2] = A[2];
        pts[3] = B[0];
        f(0, pts, false);
        pts[3] = B[1];
        f(1, pts, false);
        pts[2] = B[0];
        pts[3] = B[1];
        for (int i = 0; i < 3; ++i) {
            pts[0] = A[i];
            pts[1] = A[(i + 1) % 3];
            f(2 + i, pts, true);
        }
    } else {
        pts[0] = A[0]; pts[1] = A[1]; pts[2] = B[0]; pts[3] = B[1];
        f(0, pts, true);
    }
}

// A candidate pair as k_narrow orients it: kind (0 tri-tri, 1 tri-bond,
// 2 bond-bond), the points of the element handed over first (A) and second
// (B), and the visiting-order key base (rank of the query leaf, rank of the
// found leaf). False for a same-rigid-surface pair, which is not visited.
struct OrientedPair {
    int kind, n1, n2;
    int A[3], B[3];
    unsigned long long keybase;
};
__device__ __forceinline__ bool orient_pair(const NarrowArgs& a, int2 pr, OrientedPair& o) {
    int ri = a.rank[pr.x], rj = a.rank[pr.y];
    int ea = ri > rj ? pr.x : pr.y;  // found leaf
    int eb = ri > rj ? pr.y : pr.x;  // query leaf
    int ra = ri > rj ? ri : rj, rb = ri > rj ? rj : ri;
    bool ta = a.ev[3 * ea + 2] >= 0, tb = a.ev[3 * eb + 2] >= 0;
    o.kind = (ta && tb) ? 0 : (!ta && !tb) ? 2 : 1;
    if (o.kind == 0 && a.esurf[ea] == a.esurf[eb] && a.erigid[ea]) return false;  // dcollid.cpp:762-763, 805-806
    int e1 = (o.kind == 1 && !ta) ? eb : ea;  // tri-bond pairs are handed over as (tri, bond)
    int e2 = (o.kind == 1 && !ta) ? ea : eb;
    for (int i = 0; i < 3; ++i) {
        o.A[i] = a.ev[3 * e1 + i];
        o.B[i] = a.ev[3 * e2 + i];
    }
    o.n1 = o.A[2] >= 0 ? 3 : 2;
    o.n2 = o.B[2] >= 0 ? 3 : 2;
    o.keybase = ((unsigned long long)rb << 26) | ((unsigned long long)ra << 4);
    return true;
}

// Stage 1 of a split pass: per candidate pair, the visit bookkeeping of
// k_narrow, the element-pair filter, and the box and separating-axis filter
// of every sub-test, in sub-test order; survivors are queued with their keys,
// and a pair with survivors is queued for stage 3.
template <bool MOVING>
__device__ __forceinline__ void queue_sub(const NarrowArgs& a, const NarrowCtx& c, bool ee, unsigned long long kb,
                                          int pair, int sc, const int* pts, int sub, bool& first) {
    float ext, extb;
    if (!mixed_may_hit(c, pts, ee, &ext, &extb)) return;
    if (ee ? !sat_may_hit<MOVING, true>(c, pts, ext, extb) : !sat_may_hit<MOVING, false>(c, pts, ext, extb)) return;
    int* cnt = ee ? &a.ctr->nsub_ee : &a.ctr->nsub_pt;
    int slot = aggregated_add(cnt, 1);
    if (slot >= a.sub_cap) {
        atomicOr(&a.ctr->err, kErrSubOverflow);
        return;
    }
    if (first) {
        a.pair_hit[pair] = 0;
        int q = aggregated_add(&a.ctr->npairq, 1);
        a.pairq[q] = pair;  // at most one entry per candidate pair: fits the pair buffer
        first = false;
    }
    SubRec r;
    r.keybase = kb;
    r.pair = pair;
    r.scene = sc;
    for (int i = 0; i < 4; ++i) r.p[i] = pts[i];
    r.sub = sub;
    r.pad = 0;
    (ee ? a.sub_ee : a.sub_pt)[slot] = r;
}

template <bool MOVING>
__global__ void __launch_bounds__(512) k_narrow_filter(NarrowArgs a, int max_pairs) {
    NarrowCtx c;
    c.robust_roots = 0;
    c.pbox_lo = a.pbox_lo; c.pbox_hi = a.pbox_hi; c.p32 = a.p32; c.v32 = a.v32;
    int np = a.ctr->npairs;
    if (np > max_pairs) np = max_pairs;
    int t_visits = 0;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x) {
        int2 pr = a.pairs[idx];
        if (!MOVING && a.static_only && !(pr.y & kPairStatic)) continue;
        pr.y &= kPairIdMask;
        OrientedPair o;
        if (!orient_pair(a, pr, o)) continue;
        t_visits++;
        int sc = a.escene[pr.x];
        const double eps = a.scenes[sc].p.eps;
        c.hpad = __double2float_ru(MOVING ? eps : a.scenes[sc].p.thickness);
        c.epad = __double2float_ru(eps);
        c.dt32 = __double2float_ru(a.scenes[sc].p.dt);
        // a shared point makes every test of the pair return false
        bool shared = false;
        for (int i = 0; i < o.n1; ++i)
            for (int j = 0; j < o.n2; ++j) shared |= o.A[i] == o.B[j];
        if (shared || !pair_may_hit<MOVING>(c, o.A, o.n1, o.B, o.n2)) continue;
        bool first = true;
        for_each_subtest<MOVING>(o.kind, o.A, o.B, [&](int sub, const int* pts, bool ee) {
            queue_sub<MOVING>(a, c, ee, o.keybase, idx, sc, pts, sub, first);
        });
    }
    for (int o = 16; o > 0; o >>= 1) t_visits += __shfl_xor_sync(0xffffffffu, t_visits, o);
    if ((threadIdx.x & 31) == 0 && t_visits) atomicAdd(&a.ctr->nvisits, t_visits);
}

// Stage 3 (impact-zone scenes): createImpZone for every sub-test of a pair
// from its first hit on, in sub-test order - the reference's status stays
// true after the first hit (dcollid3d.cpp:300-321), whether or not the
// later sub-tests ran in FP64.
__global__ void __launch_bounds__(128) k_zone_unions(NarrowArgs a) {
    int n = a.ctr->npairq;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int pi = a.pairq[i];
        const int mask = a.pair_hit[pi];
        if (!mask) continue;
        int2 pr = a.pairs[pi];
        pr.y &= kPairIdMask;
        const int sc = a.escene[pr.x];
        if (a.run[sc].mode != kSceneZone) continue;
        OrientedPair o;
        if (!orient_pair(a, pr, o)) continue;
        const int kfirst = __ffs(mask) - 1;
        for_each_subtest<true>(o.kind, o.A, o.B, [&](int sub, const int* pts, bool) {
            if (sub < kfirst) return;
            int slot = aggregated_add(&a.ctr->nunion, 1);
            if (slot >= a.urec_cap) {
                atomicOr(&a.ctr->err, kErrUnionOverflow);
                return;
            }
            UnionRec r;
            r.key = o.keybase | (unsigned long long)sub;
            for (int q = 0; q < 4; ++q) r.p[q] = pts[q];
            a.urec[slot] = r;
        });
    }
}

// Stage 2: the FP64 test of k_narrow for each queued sub-test.
struct SubTally {
    int hits = 0, cr = 0, contacts = 0, sub = 0;
};

__device__ __forceinline__ NarrowCtx subtest_ctx(const NarrowArgs& a) {
    NarrowCtx c;
    c.xo = a.xo; c.av = a.av; c.fixed = a.fixed; c.ev = a.ev; c.esurf = a.esurf; c.erigid = a.erigid;
    c.vbody = a.vbody; c.body_mass = a.body_mass; c.body_slot0 = a.body_slot0;
    c.rank = a.rank;
    c.contrib = a.contrib; c.contrib_cap = a.contrib_cap; c.ctr = a.ctr; c.urec = nullptr; c.urec_cap = 0;
    c.rec = nullptr; c.rec_cap = 0;
    c.pbox_lo = nullptr; c.pbox_hi = nullptr; c.p32 = nullptr; c.v32 = nullptr;
    c.check = 0;
    c.robust_roots = a.robust_roots;
    c.zone = 0;
    return c;
}

// One sub-test: its test, the stamps of its points and its pair's hit flag
// when it hits, the scene's hit count when it is the pair's first.
template <bool MOVING, bool EE>
__device__ __forceinline__ void one_subtest(const NarrowArgs& a, NarrowCtx& c, const SubRec& r, SubTally& t) {
    c.p = a.scenes[r.scene].p;
    c.pass = 0;
    CallState st;
    st.keybase = r.keybase;
    st.np = 0;
    st.sub = r.sub;
    st.nsub = 0;
    st.ncr = 0;
    st.ncontacts = 0;
    bool hit = MOVING ? moving_test<EE>(c, st, r.p) : static_test<EE>(c, st, r.p);
    t.sub++;
    t.cr += st.ncr;
    t.contacts += st.ncontacts;
    if (hit)
        for (int q = 0; q < 4; ++q) stamp_point(a.ps, r.p[q]);
    if (hit && atomicOr(&a.pair_hit[r.pair], 1 << r.sub) == 0) {
        t.hits++;
        atomicAdd(&a.run[r.scene].hits, 1);
    }
}

// The pass's counters from every thread's tally (all lanes take part).
__device__ __forceinline__ void subtest_counts(const NarrowArgs& a, SubTally t) {
    for (int o = 16; o > 0; o >>= 1) {
        t.hits += __shfl_xor_sync(0xffffffffu, t.hits, o);
        t.cr += __shfl_xor_sync(0xffffffffu, t.cr, o);
        t.contacts += __shfl_xor_sync(0xffffffffu, t.contacts, o);
        t.sub += __shfl_xor_sync(0xffffffffu, t.sub, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (t.hits) atomicAdd(&a.ctr->nhit_pairs, t.hits);
        if (t.cr) atomicAdd(&a.ctr->ncr, t.cr);
        if (t.contacts) atomicAdd(&a.ctr->ncontacts, t.contacts);
        if (t.sub) atomicAdd(&a.ctr->nsub, t.sub);
    }
}

// Passes with more sub-tests than this run them as two launches, one per
// kind (k_subtests): measured faster than one launch for both kinds when the
// pass is large, where the FP64 pipes are full either way (each kind's
// kernel keeps a smaller body).
constexpr int kSubMergeMax = 65536;

// One list (point-triangle or edge-edge), one sub-test per thread. merged:
// k_subtests_all takes the passes of at most kSubMergeMax sub-tests.
template <bool MOVING, bool EE>
__global__ void __launch_bounds__(128, 4) k_subtests(NarrowArgs a, int merged) {
    const SubRec* list = EE ? a.sub_ee : a.sub_pt;
    int n = EE ? a.ctr->nsub_ee : a.ctr->nsub_pt;
    if (n > a.sub_cap) n = a.sub_cap;
    if (merged) {
        const int npt = a.ctr->nsub_pt < a.sub_cap ? a.ctr->nsub_pt : a.sub_cap;
        const int nee = a.ctr->nsub_ee < a.sub_cap ? a.ctr->nsub_ee : a.sub_cap;
        if (npt + nee <= kSubMergeMax) return;
    }
    NarrowCtx c = subtest_ctx(a);
    SubTally t;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        one_subtest<MOVING, EE>(a, c, list[i], t);
    subtest_counts(a, t);
}

// Both lists in one launch (passes of at most kSubMergeMax sub-tests),
// point-triangle sub-tests first, so that a small pass's two lists run side
// by side. A warp pays for an FP64 instruction the
// same whatever the number of its lanes that execute it, and the lanes of a
// warp running different sub-tests follow the union of their paths: a pass
// with at most kSubSparse sub-tests (two warps per SM sub-partition) gives
// each its own warp, which then follows one path; larger passes take one
// sub-test per thread, which keeps the FP64 pipe's issue slots full.
// Two blocks per SM: one warp per SM sub-partition already keeps its FP64
// pipe issuing, and the registers then hold both tests without spills.
constexpr int kSubSparse = 1216;
template <bool MOVING>
__global__ void __launch_bounds__(128, 2) k_subtests_all(NarrowArgs a) {
    const int npt = a.ctr->nsub_pt < a.sub_cap ? a.ctr->nsub_pt : a.sub_cap;
    const int nee = a.ctr->nsub_ee < a.sub_cap ? a.ctr->nsub_ee : a.sub_cap;
    const int n = npt + nee;
    if (n > kSubMergeMax) return;  // k_subtests's
    NarrowCtx c = subtest_ctx(a);
    SubTally t;
    const int g = blockIdx.x * blockDim.x + threadIdx.x, threads = gridDim.x * blockDim.x;
    const bool sparse = n <= kSubSparse;
    if (!sparse || (threadIdx.x & 31) == 0) {
        const int first = sparse ? g >> 5 : g, stride = sparse ? threads >> 5 : threads;
        for (int i = first; i < n; i += stride) {
            if (i < npt)
                one_subtest<MOVING, false>(a, c, a.sub_pt[i], t);
            else
                one_subtest<MOVING, true>(a, c, a.sub_ee[i - npt], t);
        }
    }
    subtest_counts(a, t);
}

// FP32 box of every point over the pass's time window, rounded outward:
// [x_old] for proximity, [x_old, x_old + dt*avgVel] for CCD.
template <bool MOVING>
__device__ __forceinline__ void point_box(const double4_32a* __restrict__ xo, const double4_32a* __restrict__ av,
                                          const int* __restrict__ vscene, const SceneDev* __restrict__ scenes, int p,
                                          float4* lo, float4* hi, float4* p32, float4* v32) {
    double dt = MOVING ? scenes[vscene[p]].p.dt : 0.0;
    double4_32a x = xo[p];
    double a[3] = {x.x, x.y, x.z}, b[3] = {x.x, x.y, x.z};
    if (MOVING) {
        double4_32a v = av[p];
        double e[3] = {x.x + v.x * dt, x.y + v.y * dt, x.z + v.z * dt};
        for (int d = 0; d < 3; ++d) {
            a[d] = fmin(a[d], e[d]);
            b[d] = fmax(b[d], e[d]);
        }
    }
    lo[p] = make_float4(__double2float_rd(a[0]), __double2float_rd(a[1]), __double2float_rd(a[2]), 0.f);
    hi[p] = make_float4(__double2float_ru(b[0]), __double2float_ru(b[1]), __double2float_ru(b[2]), 0.f);
    p32[p] = make_float4((float)x.x, (float)x.y, (float)x.z, 0.f);
    if (MOVING) {
        double4_32a v = av[p];
        v32[p] = make_float4((float)v.x, (float)v.y, (float)v.z, 0.f);
    }
}

// dn (may be null): the point count in device memory; the grid strides.
template <bool MOVING>
__global__ void k_point_boxes(const double4_32a* __restrict__ xo, const double4_32a* __restrict__ av,
                              const int* __restrict__ vscene, const SceneDev* __restrict__ scenes,
                              const int* __restrict__ act, int n, const int* __restrict__ dn, float4* lo, float4* hi,
                              float4* p32, float4* v32) {
    if (dn) n = *dn;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        point_box<MOVING>(xo, av, vscene, scenes, act ? act[k] : k, lo, hi, p32, v32);
}

}  // namespace

void point_boxes(const double4_32a* xo, const double4_32a* av, const int* vscene, const SceneDev* scenes,
                 const int* act_pts, int n, int moving, float4* lo, float4* hi, float4* p32, float4* v32,
                 cudaStream_t s, const int* dn) {
    if (n <= 0) return;
    int g = (n + 255) / 256;
    if (dn && g > 152 * 8) g = 152 * 8;
    if (moving)
        count_launch(), k_point_boxes<true><<<g, 256, 0, s>>>(xo, av, vscene, scenes, act_pts, n, dn, lo, hi, p32,
                                                              v32);
    else
        count_launch(), k_point_boxes<false><<<g, 256, 0, s>>>(xo, av, vscene, scenes, act_pts, n, dn, lo, hi, p32,
                                                               v32);
}

void narrow_pass(const NarrowArgs& a, int moving, int max_pairs, cudaStream_t s, int) {
    if (max_pairs <= 0) return;
    int threads = 128;
    int blocks = (max_pairs + threads - 1) / threads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (moving)
        count_launch(), k_narrow<true><<<blocks, threads, 0, s>>>(a, max_pairs);
    else
        count_launch(), k_narrow<false><<<blocks, threads, 0, s>>>(a, max_pairs);
}

void narrow_pass_split(const NarrowArgs& a, int moving, int max_pairs, cudaStream_t s, int block, bool zone,
                       int parts) {
    if (max_pairs <= 0) return;
    if (!a.pbox_lo || !a.p32 || (moving && !a.v32)) {  // the filters need the FP32 point data (mode 1)
        if (parts & kSplitFilter) narrow_pass(a, moving, max_pairs, s, block);
        return;
    }
    const int cap_blocks = 152 * 16 * 128 / block;
    int blocks = (max_pairs + block - 1) / block;
    if (blocks > cap_blocks) blocks = cap_blocks;
    int sblocks = (a.sub_cap + 127) / 128;
    if (sblocks > 152 * 16) sblocks = 152 * 16;
    // both lists of a pass of at most kSubMergeMax in one grid, at least one
    // warp per sub-test of a sparse pass
    long long mb = (2ll * a.sub_cap + 127) / 128;
    if (mb > (kSubMergeMax + 127) / 128) mb = (kSubMergeMax + 127) / 128;
    if (mb < (kSubSparse + 3) / 4) mb = (kSubSparse + 3) / 4;
    const int mblocks = (int)mb;
    if (moving) {
        if (parts & kSplitFilter) count_launch(), k_narrow_filter<true><<<blocks, block, 0, s>>>(a, max_pairs);
        if (parts & kSplitSubtests) {
            if (a.sub_merge) count_launch(), k_subtests_all<true><<<mblocks, 128, 0, s>>>(a);
            count_launch(), k_subtests<true, false><<<sblocks, 128, 0, s>>>(a, a.sub_merge);
            count_launch(), k_subtests<true, true><<<sblocks, 128, 0, s>>>(a, a.sub_merge);
            if (zone) count_launch(), k_zone_unions<<<blocks, 128, 0, s>>>(a);
        }
    } else {
        if (parts & kSplitFilter) count_launch(), k_narrow_filter<false><<<blocks, block, 0, s>>>(a, max_pairs);
        if (parts & kSplitSubtests) {
            if (a.sub_merge) count_launch(), k_subtests_all<false><<<mblocks, 128, 0, s>>>(a);
            count_launch(), k_subtests<false, false><<<sblocks, 128, 0, s>>>(a, a.sub_merge);
            count_launch(), k_subtests<false, true><<<sblocks, 128, 0, s>>>(a, a.sub_merge);
        }
    }
}

}  // namespace ccg
