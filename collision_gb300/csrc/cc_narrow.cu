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
    c.rank = a.rank; c.nt = a.nt; c.pass = a.pass; c.zone = a.zone; c.p = a.p;
    c.contrib = a.contrib; c.contrib_cap = a.contrib_cap; c.ctr = a.ctr; c.uf_parent = a.uf_parent;
    c.rec = a.rec; c.rec_cap = a.rec_cap;
    c.pbox_lo = a.pbox_lo; c.pbox_hi = a.pbox_hi; c.hpad = a.hpad; c.epad = a.epad;
    int np = a.ctr->npairs;
    if (np > max_pairs) np = max_pairs;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x) {
        int2 pr = a.pairs[idx];
        int ri = c.rank[pr.x], rj = c.rank[pr.y];
        int ea = ri > rj ? pr.x : pr.y;  // found leaf
        int eb = ri > rj ? pr.y : pr.x;  // query leaf
        int ra = ri > rj ? ri : rj, rb = ri > rj ? rj : ri;
        bool ta = ea < c.nt, tb = eb < c.nt;
        int kind = (ta && tb) ? 0 : (!ta && !tb) ? 2 : 1;
        if (kind == 0 && c.esurf[ea] == c.esurf[eb] && c.erigid[ea]) continue;  // dcollid.cpp:762-763, 805-806
        // tri-bond pairs are always handed over as (tri, bond)
        int e1 = (kind == 1 && !ta) ? eb : ea;
        int e2 = (kind == 1 && !ta) ? ea : eb;
        const int* P1 = c.ev + 3 * e1;
        const int* P2 = c.ev + 3 * e2;
        CallState st;
        st.keybase = ((unsigned long long)rb << 26) | ((unsigned long long)ra << 4);
        int n1 = (e1 < c.nt) ? 3 : 2, n2 = (e2 < c.nt) ? 3 : 2;
        st.np = n1 + n2;
        for (int i = 0; i < 6; ++i) { st.dcount[i] = 0; st.plist[i] = -1; }
        for (int i = 0; i < n1; ++i) st.plist[i] = P1[i];
        for (int i = 0; i < n2; ++i) st.plist[n1 + i] = P2[i];
        st.sub = 0;
        st.nsub = 0;
        int A[3] = {P1[0], P1[1], n1 == 3 ? P1[2] : -1};
        int B[3] = {P2[0], P2[1], n2 == 3 ? P2[2] : -1};
        bool status;
        if (kind == 0)
            status = tri_to_tri<MOVING>(c, st, A, B);
        else if (kind == 1)
            status = tri_to_bond<MOVING>(c, st, A, B);
        else
            status = bond_to_bond<MOVING>(c, st, A, B);
        atomicAdd(&c.ctr->nvisits, 1);
        if (st.nsub) atomicAdd(&c.ctr->nsub, st.nsub);
        if (status) atomicAdd(&c.ctr->nhit_pairs, 1);
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
}

// FP32 box of every point over the pass's time window, rounded outward:
// [x_old] for proximity, [x_old, x_old + dt*avgVel] for CCD.
template <bool MOVING>
__global__ void k_point_boxes(const double4_32a* __restrict__ xo, const double4_32a* __restrict__ av, double dt,
                              int nv, float4* lo, float4* hi) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv) return;
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
}

}  // namespace

void point_boxes(const double4_32a* xo, const double4_32a* av, double dt, int nv, int moving, float4* lo,
                 float4* hi, cudaStream_t s) {
    if (nv <= 0) return;
    if (moving)
        count_launch(), k_point_boxes<true><<<(nv + 255) / 256, 256, 0, s>>>(xo, av, dt, nv, lo, hi);
    else
        count_launch(), k_point_boxes<false><<<(nv + 255) / 256, 256, 0, s>>>(xo, av, dt, nv, lo, hi);
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
