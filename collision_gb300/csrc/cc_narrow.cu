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
    c.rank = a.rank;
    c.contrib = a.contrib; c.contrib_cap = a.contrib_cap; c.ctr = a.ctr; c.urec = a.urec;
    c.urec_cap = a.urec_cap;
    c.rec = a.rec; c.rec_cap = a.rec_cap;
    c.pbox_lo = a.pbox_lo; c.pbox_hi = a.pbox_hi; c.p32 = a.p32; c.v32 = a.v32;
    c.check = a.check;
    int np = a.ctr->npairs;
    if (np > max_pairs) np = max_pairs;
    // counters summed per thread, added once per warp at the end
    int t_visits = 0, t_sub = 0, t_hits = 0, t_cr = 0, t_contacts = 0;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x) {
        int2 pr = a.pairs[idx];
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

// FP32 box of every point over the pass's time window, rounded outward:
// [x_old] for proximity, [x_old, x_old + dt*avgVel] for CCD.
template <bool MOVING>
__global__ void k_point_boxes(const double4_32a* __restrict__ xo, const double4_32a* __restrict__ av,
                              const int* __restrict__ vscene, const SceneDev* __restrict__ scenes,
                              const int* __restrict__ act, int n, float4* lo, float4* hi, float4* p32, float4* v32) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int p = act ? act[k] : k;
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

}  // namespace

void point_boxes(const double4_32a* xo, const double4_32a* av, const int* vscene, const SceneDev* scenes,
                 const int* act_pts, int n, int moving, float4* lo, float4* hi, float4* p32, float4* v32,
                 cudaStream_t s) {
    if (n <= 0) return;
    if (moving)
        count_launch(), k_point_boxes<true><<<(n + 255) / 256, 256, 0, s>>>(xo, av, vscene, scenes, act_pts, n, lo,
                                                                            hi, p32, v32);
    else
        count_launch(), k_point_boxes<false><<<(n + 255) / 256, 256, 0, s>>>(xo, av, vscene, scenes, act_pts, n, lo,
                                                                             hi, p32, v32);
}

void narrow_pass(const NarrowArgs& a, int moving, int max_pairs, cudaStream_t s) {
    if (max_pairs <= 0) return;
    int threads = 128;
    int blocks = (max_pairs + threads - 1) / threads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (moving)
        count_launch(), k_narrow<true><<<blocks, threads, 0, s>>>(a, max_pairs);
    else
        count_launch(), k_narrow<false><<<blocks, threads, 0, s>>>(a, max_pairs);
}

}  // namespace ccg
