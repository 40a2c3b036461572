// Narrow phase on the GPU: proximity (t = 0) and continuous (CCD) tests of
// one element pair, and the repulsion / inelastic / friction impulses of each
// hit, emitted as keyed per-point contributions instead of the reference's
// in-place accumulation (dcollid3d.cpp:925-1300).
//
// One thread handles one element pair; positions stay in registers (the
// reference writes them into the shared POINT coordinates, dcollid3d.cpp:333-339).
#pragma once

#include "cc_common.cuh"
#include "cc_crmath.cuh"

namespace ccg {

struct NarrowCtx {
    const double4_32a* xo;       // x_old per point
    const double4_32a* av;       // average velocity per point
    const uint8_t* fixed;    // per point: bit 0 is_fixed, bit 1 is_movableRG
    const int* ev;           // 3 point ids per element (bonds: third is -1)
    const int* esurf;        // surface id per element (-1 for bonds)
    const uint8_t* erigid;   // element has a fixed or movable point (isRigidBody(hse))
    const int* vbody;        // movable body of each point, -1 for none
    const double* body_mass; // total_mass of each body
    int body_slot0;          // contribution slot of body 0 (after every point's)
    const int* rank;         // leaf rank of each element in its scene's reference tree
    int pass;                // the scene's pass index
    int zone;                // impact-zone mode (s_detImpZone) of the scene
    Params p;                // the scene's parameters
    Contrib* contrib;
    int contrib_cap;
    PassCounters* ctr;
    UnionRec* urec;          // createImpZone calls of impact-zone passes
    int urec_cap;
    VisitRec* rec;
    int rec_cap;
    // mixed precision: per-point FP32 boxes over the pass's time window
    // (rounded outward), used to reject sub-tests that cannot hit
    const float4* pbox_lo;
    const float4* pbox_hi;
    const float4* p32;    // x_old rounded to FP32
    const float4* v32;    // avgVel rounded to FP32 (moving passes)
    float hpad;   // h of the sub-tests, rounded up
    float epad;   // eps (barycentric tolerance), rounded up
    int check;    // decide hits only: no impulses, contacts or zones
    int robust_roots;  // mixed sub-tests: skip the correctly rounded roots where no decision needs them
    float dt32;   // dt rounded up to FP32
};

struct CallState {
    unsigned long long keybase;
    int plist[6];
    int np;
    int dcount[6];
    int sub;
    int nsub;   // sub-tests evaluated in FP64
    int ncr;    // cubics whose roots were formed again correctly rounded
    int ncontacts;
};

__device__ __forceinline__ bool is_static(const NarrowCtx& c, int p) { return (c.fixed[p] & 1) != 0; }
__device__ __forceinline__ bool is_movable(const NarrowCtx& c, int p) { return (c.fixed[p] & 2) != 0; }
__device__ __forceinline__ bool is_rigid(const NarrowCtx& c, int p) { return c.fixed[p] != 0; }

__device__ __forceinline__ void emit(const NarrowCtx& c, CallState& st, int vertex, const double* imp,
                                     const double* fric, int has_fric) {
    for (int i = 0; i < st.np; ++i)
        if (st.plist[i] == vertex) { st.dcount[i]++; break; }
    int slot = aggregated_add(&c.ctr->ncontrib, 1);
    if (slot >= c.contrib_cap) {
        atomicOr(&c.ctr->err, kErrContribOverflow);
        return;
    }
    Contrib& o = c.contrib[slot];
    o.key = st.keybase | (unsigned long long)st.sub;
    o.vertex = vertex;
    o.flags = has_fric;
    for (int j = 0; j < 3; ++j) { o.imp[j] = imp[j]; o.fric[j] = fric[j]; }
}

// SpreadImpactZoneImpulse (dcollid.cpp:1101-1115) adds impulse*nor to the
// collsnImpulse_RG of every member of p's zone - a movable body's zone is the
// body - and counts one. Every member gets the same additions in the same
// order, so the sum is kept once per body, in a contribution slot of its own.
__device__ __forceinline__ void emit_body(const NarrowCtx& c, CallState& st, int p, double impulse,
                                          const double* nor) {
    int slot = aggregated_add(&c.ctr->ncontrib, 1);
    if (slot >= c.contrib_cap) {
        atomicOr(&c.ctr->err, kErrContribOverflow);
        return;
    }
    Contrib& o = c.contrib[slot];
    o.key = st.keybase | (unsigned long long)st.sub;
    o.vertex = c.body_slot0 + c.vbody[p];
    o.flags = 0;
    for (int j = 0; j < 3; ++j) { o.imp[j] = impulse * nor[j]; o.fric[j] = 0.0; }
}

// ---------------------------------------------------------------- unions
// createImpZone(pts, 4), dcollid.cpp:473-484: the four points join one zone.
// The call is recorded with its visiting-order key; the unions themselves
// are replayed in that order after the pass.
__device__ __forceinline__ void create_imp_zone(const NarrowCtx& c, const CallState& st, const int* pts) {
    int slot = aggregated_add(&c.ctr->nunion, 1);
    if (slot >= c.urec_cap) {
        atomicOr(&c.ctr->err, kErrUnionOverflow);
        return;
    }
    UnionRec r;
    r.key = st.keybase | (unsigned long long)st.sub;
    for (int i = 0; i < 4; ++i) r.p[i] = pts[i];
    c.urec[slot] = r;
}

// -------------------------------------------------------------- impulses
// PointToTriImpulse, dcollid3d.cpp:925-1107.
static __device__ void point_to_tri_impulse(const NarrowCtx& c, CallState& st, const int* pts, const double* nor,
                                     double* w, double dist) {
    double v_rel[3] = {0.0, 0.0, 0.0}, vn, vt;
    double impulse = 0.0, m_impulse, sum_w = 0.0;
    double rigid_impulse[2] = {0.0, 0.0};
    const double k = c.p.k, m = c.p.m, dt = c.p.dt, lambda = c.p.lambda, h = c.p.thickness, cr = c.p.cr;
    double av[4][3];
    for (int q = 0; q < 4; ++q) load3(c.av, pts[q], av[q]);
    bool st0 = is_static(c, pts[0]), st1 = is_static(c, pts[1]), st2 = is_static(c, pts[2]),
         st3 = is_static(c, pts[3]);
    bool mv[4] = {is_movable(c, pts[0]), is_movable(c, pts[1]), is_movable(c, pts[2]), is_movable(c, pts[3])};
    dist = h - dist;
    for (int i = 0; i < 3; ++i) {
        v_rel[i] += av[3][i];
        for (int j = 0; j < 3; ++j) v_rel[i] -= w[j] * av[j][i];
    }
    vn = dot3(v_rel, nor);
    if (dot3(v_rel, v_rel) > sqr(vn))
        vt = sqrt(dot3(v_rel, v_rel) - sqr(vn));
    else
        vt = 0.0;
    bool tri_static[3] = {st0, st1, st2};
    if (vn < 0) {
        if (st3 || (st0 && st1 && st2)) {
            impulse = vn;
            rigid_impulse[0] = vn;
            rigid_impulse[1] = vn;
        } else if (mv[0] && mv[1] && mv[2] && mv[3]) {
            double m1 = c.body_mass[c.vbody[pts[0]]], m2 = c.body_mass[c.vbody[pts[3]]];
            rigid_impulse[0] = vn * m2 / (m1 + m2);
            rigid_impulse[1] = vn * m1 / (m1 + m2);
        } else if (mv[0] && mv[1] && mv[2]) {
            rigid_impulse[0] = 0.5 * vn;
            impulse = 0.5 * vn;
        } else if (mv[3]) {
            impulse = 0.5 * vn;
            rigid_impulse[1] = 0.5 * vn;
        } else {
            impulse = vn * 0.5;
        }
        for (int i = 0; i < 3; ++i) {
            if (tri_static[i]) w[i] = 0.0;
            sum_w += w[i];
        }
        if (fabs(sum_w) > kMachEps) {
            double inv = 1.0 / sum_w;
            for (int i = 0; i < 3; ++i) w[i] = inv * w[i];
        }
    }
    bool all_rigid = is_rigid(c, pts[0]) && is_rigid(c, pts[1]) && is_rigid(c, pts[2]) && is_rigid(c, pts[3]);
    if (vn * dt < 0.1 * dist) {
        if (all_rigid) {
            rigid_impulse[0] *= 1.0 + cr;
            rigid_impulse[1] *= 1.0 + cr;
        } else {
            double tmp = -smin(dt * k * dist / m, (0.1 * dist / dt - vn));
            impulse += tmp;
            rigid_impulse[0] += tmp;
            rigid_impulse[1] += tmp;
        }
    }
    if (fabs(sum_w) < kMachEps)
        m_impulse = impulse;
    else
        m_impulse = 2.0 * impulse / (1.0 + dot3(w, w));
    if (all_rigid) {
        if (mv[0]) emit_body(c, st, pts[0], rigid_impulse[0], nor);
        if (mv[3]) emit_body(c, st, pts[3], -1.0 * rigid_impulse[1], nor);
        return;
    }
    int has_fric = fabs(vt) > kRoundEps;
    double imp[3], fric[3];
    for (int i = 0; i < 3; ++i) {
        if (tri_static[i]) continue;
        double t_impulse = mv[i] ? rigid_impulse[0] : m_impulse;
        for (int j = 0; j < 3; ++j) {
            imp[j] = w[i] * t_impulse * nor[j];
            fric[j] = has_fric ? smax(-fabs(lambda * w[i] * t_impulse / vt), -1.0) * (v_rel[j] - vn * nor[j]) : 0.0;
        }
        emit(c, st, pts[i], imp, fric, has_fric);
    }
    if (!st3) {
        double t_impulse = mv[3] ? rigid_impulse[1] : m_impulse;
        for (int j = 0; j < 3; ++j) {
            imp[j] = -(t_impulse * nor[j]);
            fric[j] = has_fric ? smax(-fabs(lambda * t_impulse / vt), -1.0) * (v_rel[j] - vn * nor[j]) : 0.0;
        }
        emit(c, st, pts[3], imp, fric, has_fric);
    }
}

// EdgeToEdgeImpulse, dcollid3d.cpp:1109-1300.
static __device__ void edge_to_edge_impulse(const NarrowCtx& c, CallState& st, const int* pts, const double* nor,
                                     double a, double b, double dist) {
    double v_rel[3], vn, vt;
    double impulse = 0.0, m_impulse;
    double rigid_impulse[2] = {0.0, 0.0};
    const double k = c.p.k, m = c.p.m, dt = c.p.dt, lambda = c.p.lambda, h = c.p.thickness, cr = c.p.cr;
    double wa[2] = {1.0 - a, a}, wb[2] = {1.0 - b, b};
    double av[4][3];
    for (int q = 0; q < 4; ++q) load3(c.av, pts[q], av[q]);
    bool sq[4] = {is_static(c, pts[0]), is_static(c, pts[1]), is_static(c, pts[2]), is_static(c, pts[3])};
    bool mv[4] = {is_movable(c, pts[0]), is_movable(c, pts[1]), is_movable(c, pts[2]), is_movable(c, pts[3])};
    dist = h - dist;
    for (int j = 0; j < 3; ++j) {
        v_rel[j] = (1.0 - b) * av[2][j] + b * av[3][j];
        v_rel[j] -= (1.0 - a) * av[0][j] + a * av[1][j];
    }
    vn = dot3(v_rel, nor);
    if (dot3(v_rel, v_rel) > sqr(vn))
        vt = sqrt(dot3(v_rel, v_rel) - sqr(vn));
    else
        vt = 0.0;
    if (vn < 0.0) {
        if ((sq[0] && sq[1]) || (sq[2] && sq[3])) {
            impulse = vn;
            rigid_impulse[0] = vn;
            rigid_impulse[1] = vn;
        } else if (mv[0] && mv[1] && mv[2] && mv[3]) {
            double m1 = c.body_mass[c.vbody[pts[0]]], m2 = c.body_mass[c.vbody[pts[2]]];
            rigid_impulse[0] = vn * m2 / (m1 + m2);
            rigid_impulse[1] = vn * m1 / (m1 + m2);
        } else if (mv[0] && mv[1]) {
            rigid_impulse[0] = 0.5 * vn;
            impulse = 0.5 * vn;
        } else if (mv[2] && mv[3]) {
            impulse = 0.5 * vn;
            rigid_impulse[1] = 0.5 * vn;
        } else {
            impulse = vn * 0.5;
        }
        if (sq[0]) wa[0] = 0.0;
        if (sq[1]) wa[1] = 0.0;
        if (sq[2]) wb[0] = 0.0;
        if (sq[3]) wb[1] = 0.0;
    }
    bool all_rigid = is_rigid(c, pts[0]) && is_rigid(c, pts[1]) && is_rigid(c, pts[2]) && is_rigid(c, pts[3]);
    if (vn * dt < 0.1 * dist) {
        if (all_rigid) {
            rigid_impulse[0] *= 1.0 + cr;
            rigid_impulse[1] *= 1.0 + cr;
        } else {
            double tmp = -smin(dt * k * dist / m, (0.1 * dist / dt - vn));
            impulse += tmp;
            rigid_impulse[0] += tmp;
            rigid_impulse[1] += tmp;
        }
    }
    if (wa[0] + wa[1] < kMachEps || wb[0] + wb[1] < kMachEps)
        m_impulse = impulse;
    else
        m_impulse = 2.0 * impulse / (wa[0] * wa[0] + wa[1] * wa[1] + wb[0] * wb[0] + wb[1] * wb[1]);
    if (all_rigid) {
        if (mv[0]) emit_body(c, st, pts[0], rigid_impulse[0], nor);
        if (mv[2]) emit_body(c, st, pts[2], -1.0 * rigid_impulse[1], nor);
        return;
    }
    int has_fric = fabs(vt) > kRoundEps;
    const double wgt[4] = {wa[0], wa[1], wb[0], wb[1]};
    double imp[3], fric[3];
    for (int q = 0; q < 4; ++q) {
        if (sq[q]) continue;
        double t_impulse = mv[q] ? rigid_impulse[q < 2 ? 0 : 1] : m_impulse;
        for (int j = 0; j < 3; ++j) {
            double d = wgt[q] * t_impulse * nor[j];
            imp[j] = (q < 2) ? d : -d;
            fric[j] = has_fric ? smax(-fabs(lambda * wgt[q] * t_impulse / vt), -1.0) * (v_rel[j] - vn * nor[j]) : 0.0;
        }
        emit(c, st, pts[q], imp, fric, has_fric);
    }
}

// ------------------------------------------------------- point / edge tests
// PointToTri, dcollid3d.cpp:778-922. pts[0..2] the triangle, pts[3] the
// point; X holds the four positions the reference keeps in Coords.
static __device__ bool point_to_tri(const NarrowCtx& c, CallState& st, const int* pts, const double (*X)[3], double h) {
    double w[3] = {0.0, 0.0, 0.0};
    double x13[3], x23[3], x43[3];
    double nor[3] = {0.0, 0.0, 0.0}, nor_mag, dist, det;
    for (int i = 0; i < 3; ++i) {
        x13[i] = X[0][i] - X[2][i];
        x23[i] = X[1][i] - X[2][i];
        x43[i] = X[3][i] - X[2][i];
    }
    det = dot3(x13, x13) * dot3(x23, x23) - dot3(x13, x23) * dot3(x13, x23);
    if (fabs(det) < 1000 * kMachEps) return false;
    cross3(x13, x23, nor);
    nor_mag = mag3(nor);
    double xo[4][3];
    for (int q = 0; q < 4; ++q) load3(c.xo, pts[q], xo[q]);
    double x43_old[3];
    for (int i = 0; i < 3; ++i) x43_old[i] = xo[3][i] - xo[2][i];
    dist = dot3(x43_old, nor);
    for (int i = 0; i < 3; ++i) nor[i] /= nor_mag * ((dist >= 0) ? 1.0 : -1.0);
    dist = fabs(dot3(x43, nor));
    w[0] = (dot3(x13, x43) * dot3(x23, x23) - dot3(x23, x43) * dot3(x13, x23)) / det;
    w[1] = (dot3(x13, x13) * dot3(x23, x43) - dot3(x13, x23) * dot3(x13, x43)) / det;
    w[2] = 1 - w[0] - w[1];
    if (fabs(w[0]) < kRoundEps || fabs(w[1]) < kRoundEps || fabs(w[2]) < kRoundEps) {
        double vec[3];
        for (int j = 0; j < 3; ++j) vec[j] = xo[3][j];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) vec[j] -= w[i] * xo[i][j];
        double vec_mag = mag3(vec);
        if (vec_mag > kRoundEps)
            for (int j = 0; j < 3; ++j) nor[j] = vec[j];
    }
    nor_mag = mag3(nor);
    if (nor_mag > kRoundEps) {
        for (int i = 0; i < 3; ++i) nor[i] /= nor_mag;
    } else {
        atomicOr(&c.ctr->err, kErrNan);  // "nan nor vec": the reference exits
        return false;
    }
    if (dist > h) return false;
    for (int i = 0; i < 3; ++i)
        if (w[i] > 1 + c.p.eps || w[i] < -c.p.eps) return false;
    if (c.check) return true;
    st.ncontacts++;
    point_to_tri_impulse(c, st, pts, nor, w, dist);
    return true;
}

// EdgeToEdge, dcollid3d.cpp:643-776. Edges (pts[0],pts[1]) and (pts[2],pts[3]).
static __device__ bool edge_to_edge(const NarrowCtx& c, CallState& st, const int* pts, const double (*X)[3], double h) {
    double x21[3], x43[3], x31[3], tmp[3], v1[3], v2[3], nor[3];
    double a, b, nor_mag, dist;
    for (int i = 0; i < 3; ++i) {
        x21[i] = X[1][i] - X[0][i];
        x43[i] = X[3][i] - X[2][i];
        x31[i] = X[2][i] - X[0][i];
    }
    cross3(x21, x43, tmp);
    if (mag3(tmp) < kRoundEps) return false;
    double d4343 = dot3(x43, x43), d2131 = dot3(x21, x31), d2143 = dot3(x21, x43), d4331 = dot3(x43, x31),
           d2121 = dot3(x21, x21);
    a = (d4343 * d2131 - d2143 * d4331) / (d2121 * d4343 - d2143 * d2143);
    b = (d2143 * d2131 - d2121 * d4331) / (d2121 * d4343 - d2143 * d2143);
    a = smax(smin(a, 1.0), 0.0);
    b = smax(smin(b, 1.0), 0.0);
    for (int i = 0; i < 3; ++i) {
        v1[i] = a * x21[i];
        v2[i] = b * x43[i];
    }
    for (int i = 0; i < 3; ++i) {
        v1[i] = X[0][i] + v1[i];
        v2[i] = X[2][i] + v2[i];
    }
    for (int i = 0; i < 3; ++i) nor[i] = v2[i] - v1[i];
    nor_mag = mag3(nor);
    if (nor_mag < 1000 * kMachEps) {
        double xo[4][3];
        for (int q = 0; q < 4; ++q) load3(c.xo, pts[q], xo[q]);
        for (int j = 0; j < 3; ++j) {
            nor[j] = (1.0 - b) * xo[2][j] + b * xo[3][j];
            nor[j] -= (1.0 - a) * xo[0][j] + a * xo[1][j];
        }
    }
    double s = 0.0;
    for (int i = 0; i < 3; ++i) s += sqr(v1[i] - v2[i]);
    dist = sqrt(s);
    if (dist > h) return false;
    nor_mag = mag3(nor);
    if (nor_mag < kMachEps) {
        atomicOr(&c.ctr->err, kErrNan);  // "Normal vector is nan": the reference exits
        return false;
    }
    for (int i = 0; i < 3; ++i) nor[i] /= nor_mag;
    if (c.check) return true;
    st.ncontacts++;
    edge_to_edge_impulse(c, st, pts, nor, a, b, dist);
    return true;
}

// ------------------------------------------------------------------- CCD
// Whether the static test (h, barycentric tolerance eps) returns false at
// every time within terr of t. Positions at any such time, as the test
// computes them, lie within dp of X = x_old + t * avgVel (the motion in terr
// plus the positions' rounding). A miss is certain when
//  - the points' boxes at t, padded as in mixed_may_hit (which bounds where
//    a hit can lie) and by dp, are apart along an axis; or
//  - point-triangle (dcollid3d.cpp:778-922): a barycentric coordinate at t
//    is outside [-eps, 1+eps] by more than twice a bound on the formulas'
//    rounding error (the same formulas as the test's) plus how far the
//    coordinates can move when the points move by dp; if the test's
//    determinant is below its cut instead, it returns false too; or
//  - edge-edge (dcollid3d.cpp:643-776): the test's distance is between two
//    points on the segments, so it is at least their true distance, which
//    is at least the gap between the segments' projections on any unit
//    vector (here the one between the segments' closest points): a gap
//    above h by 2 dp plus rounding rules a hit out (and near-parallel
//    edges return false anyway).
template <bool EE>
__device__ __forceinline__ bool root_misses(const double (*xo4)[3], const double (*av4)[3], double t, double terr,
                                            double h, double eps) {
    double X[4][3];
    double vmax = 0.0, xmax = 0.0;
    for (int q = 0; q < 4; ++q)
        for (int k = 0; k < 3; ++k) {
            X[q][k] = xo4[q][k] + t * av4[q][k];
            vmax = fmax(vmax, fabs(av4[q][k]));
            xmax = fmax(xmax, fabs(X[q][k]));
        }
    if (!(xmax < 1e30) || !(vmax < 1e30)) return false;  // NaN or huge: no claim
    const double dp = terr * vmax * 1.001 + xmax * 0x1p-48;
    constexpr int na = EE ? 2 : 3;
    double alo[3], ahi[3], blo[3], bhi[3];
    for (int k = 0; k < 3; ++k) {
        alo[k] = ahi[k] = X[0][k];
        for (int q = 1; q < na; ++q) alo[k] = fmin(alo[k], X[q][k]), ahi[k] = fmax(ahi[k], X[q][k]);
        blo[k] = bhi[k] = X[na][k];
        for (int q = na + 1; q < 4; ++q) blo[k] = fmin(blo[k], X[q][k]), bhi[k] = fmax(bhi[k], X[q][k]);
    }
    double ext = 0.0, extb = 0.0;
    for (int k = 0; k < 3; ++k) ext += ahi[k] - alo[k], extb += bhi[k] - blo[k];
    double pad = EE ? h + (ext + extb) * 0x1p-20 : h + ext * (8.0 * eps + 0x1p-10);
    pad = pad * 1.001 + dp;
    for (int k = 0; k < 3; ++k)
        if (alo[k] - pad > bhi[k] || blo[k] - pad > ahi[k]) return true;
    if (!EE) {
        double x13[3], x23[3], x43[3];
        for (int k = 0; k < 3; ++k) {
            x13[k] = X[0][k] - X[2][k];
            x23[k] = X[1][k] - X[2][k];
            x43[k] = X[3][k] - X[2][k];
        }
        const double a11 = dot3(x13, x13), a22 = dot3(x23, x23), a12 = dot3(x13, x23), a44 = dot3(x43, x43);
        const double det = a11 * a22 - a12 * a12;
        if (!(det > 0.0)) return false;
        const double w0 = (dot3(x13, x43) * a22 - dot3(x23, x43) * a12) / det;
        const double w1 = (a11 * dot3(x23, x43) - a12 * dot3(x13, x43)) / det;
        const double w2 = 1 - w0 - w1;
        const double W = 1.0 + 1.01 * fmax(fmax(fabs(w0), fabs(w1)), fabs(w2));
        // the rounding error of w0 or w1 from these formulas (dot products
        // within 3 units of 2^-53 of their magnitude, then two products, a
        // difference and the quotient): below 15 units times S^2 (1 + |w|)
        // over det, bounded here by 2^-48 S^2 W / det; w2 = 1 - w0 - w1
        // carries at most twice that, and the test's own coordinates, at its
        // own positions, as much again
        const double S = a11 + a22 + a44;
        const double E = 0x1p-48 * S * S * W / det;
        // and how far a coordinate moves when the four points move by dp: a
        // coordinate is a ratio of in-plane areas, each changing by at most
        // dp times the lengths (L bounds every distance among the points;
        // sqrt(det) is twice the triangle's area), padded twice
        const double L = sqrt(a11) + sqrt(a22) + sqrt(a44);
        const double D = 6.0 * dp * L * W / sqrt(det);
        const double m = eps + 4.04 * E + D;
        if (!(m < 0.5)) return false;
        return w0 < -m || w1 < -m || w2 < -m || w0 > 1 + m || w1 > 1 + m || w2 > 1 + m;
    }
    // edge-edge: the closest points of the two segments (clamped), then the
    // gap of the projections on the unit vector between them
    double d1[3], d2[3], r[3];
    for (int k = 0; k < 3; ++k) {
        d1[k] = X[1][k] - X[0][k];
        d2[k] = X[3][k] - X[2][k];
        r[k] = X[0][k] - X[2][k];
    }
    const double aa = dot3(d1, d1), ee = dot3(d2, d2), ff = dot3(d2, r);
    if (!(aa > 0.0) || !(ee > 0.0)) return false;
    const double cc = dot3(d1, r), bb = dot3(d1, d2), den = aa * ee - bb * bb;
    double s1 = den > 0.0 ? fmin(fmax((bb * ff - cc * ee) / den, 0.0), 1.0) : 0.0;
    double s2 = (bb * s1 + ff) / ee;
    if (s2 < 0.0) {
        s2 = 0.0;
        s1 = fmin(fmax(-cc / aa, 0.0), 1.0);
    } else if (s2 > 1.0) {
        s2 = 1.0;
        s1 = fmin(fmax((bb - cc) / aa, 0.0), 1.0);
    }
    double n[3];
    for (int k = 0; k < 3; ++k) n[k] = (X[2][k] + s2 * d2[k]) - (X[0][k] + s1 * d1[k]);
    const double nm = sqrt(dot3(n, n));
    if (!(nm > h)) return false;
    for (int k = 0; k < 3; ++k) n[k] /= nm;
    const double p0 = dot3(X[0], n), p1 = dot3(X[1], n), p2 = dot3(X[2], n), p3 = dot3(X[3], n);
    const double gap = fmax(fmin(p2, p3) - fmax(p0, p1), fmin(p0, p1) - fmax(p2, p3));
    // rounding: the projections (3 products and sums of coordinates up to
    // xmax, n within a few ulp of unit) and the test's own distance
    return gap - 2.0 * dp - xmax * 0x1p-44 > h * 1.001;
}

// isCoplanar, dcollid3d.cpp:371-482: roots of the coplanarity cubic in
// [0, dt], shifted by -MACH_EPS and sorted; roots[3] holds dt.
//
// rb (mixed sub-tests): a root the fast functions put well inside the
// window - farther than twice the margin from its ends, so the correctly
// rounded root is inside too and on the same side of MACH_EPS - and at
// which the static test misses whichever root within the margin it is
// (root_misses), needs no correctly rounded value: its test returns false
// either way and nothing else depends on its exact value. When every root
// near the window is such a root, none is formed again; those roots count
// towards the return value and are then dropped, as their tests would
// return false. Any other root near the window (or a branch threshold
// within the margin) makes all of them formed again, as without rb.
template <bool EE>
static __device__ bool is_coplanar(const double (*xo4)[3], const double (*av4)[3], double dt, double* roots,
                                   int* ncr, bool rb = false, double h = 0.0, double eps = 0.0) {
    double v[4][3], x[4][3];
    for (int j = 0; j < 3; ++j) {
        v[0][j] = av4[0][j];
        x[0][j] = xo4[0][j];
    }
    for (int i = 1; i < 4; ++i)
        for (int j = 0; j < 3; ++j) {
            v[i][j] = av4[i][j] - av4[0][j];
            x[i][j] = xo4[i][j] - xo4[0][j];
        }
    double a, b, c, d;
    double vv[3], vx[3], xx[3];
    vv[0] = v[1][1] * v[2][2] - v[1][2] * v[2][1];
    vv[1] = v[1][0] * v[2][2] - v[1][2] * v[2][0];
    vv[2] = v[1][0] * v[2][1] - v[1][1] * v[2][0];
    vx[0] = v[1][1] * x[2][2] - v[1][2] * x[2][1] - v[2][1] * x[1][2] + v[2][2] * x[1][1];
    vx[1] = v[1][0] * x[2][2] - v[1][2] * x[2][0] - v[2][0] * x[1][2] + v[2][2] * x[1][0];
    vx[2] = v[1][0] * x[2][1] - v[1][1] * x[2][0] - v[2][0] * x[1][1] + v[2][1] * x[1][0];
    xx[0] = x[1][1] * x[2][2] - x[1][2] * x[2][1];
    xx[1] = x[1][0] * x[2][2] - x[1][2] * x[2][0];
    xx[2] = x[1][0] * x[2][1] - x[1][1] * x[2][0];
    a = v[3][0] * vv[0] - v[3][1] * vv[1] + v[3][2] * vv[2];
    b = x[3][0] * vv[0] - x[3][1] * vv[1] + x[3][2] * vv[2] + v[3][0] * vx[0] - v[3][1] * vx[1] + v[3][2] * vx[2];
    c = x[3][0] * vx[0] - x[3][1] * vx[1] + x[3][2] * vx[2] + v[3][0] * xx[0] - v[3][1] * xx[1] + v[3][2] * xx[2];
    d = x[3][0] * xx[0] - x[3][1] * xx[1] + x[3][2] * xx[2];
    if (fabs(a) > kMachEps) {
        b /= a; c /= a; d /= a;
        a = b; b = c; c = d;
        double Q = (a * a - 3 * b) / 9;
        double R = (2 * a * a * a - 9 * a * b + 27 * c) / 54;
        double Q3 = Q * Q * Q;
        double R2 = R * R;
        // The roots are first formed with the fast library functions, whose
        // results lie within 2 ulp of the correctly rounded ones (CUDA's
        // documented bound for acos, cos and pow). Carried through the root
        // formulas that moves a root by at most 2.3e-15 times the root scale
        // (2*sqrt(Q) + |a| in the trigonometric case, |A| + |B| + |a| in
        // Cardano's), and `margin` is four times that. A root farther than
        // the margin from the window [MACH_EPS, dt + MACH_EPS] is discarded
        // whichever way it was formed; roots inside or near the window, and
        // branch thresholds within the margin, are formed again with the
        // correctly rounded functions the reference's libm gives.
        if (R2 < Q3) {
            double Qsqrt = sqrt(Q);
            double z = R / sqrt(Q3);
            double theta = acos(z);
            double f[3];
            f[0] = -2 * Qsqrt * cos(theta / 3) - a / 3;
            f[1] = -2 * Qsqrt * cos((theta + 2 * kPi) / 3) - a / 3;
            f[2] = -2 * Qsqrt * cos((theta - 2 * kPi) / 3) - a / 3;
            double margin = 1e-14 * (2 * fabs(Qsqrt) + fabs(a)) + 1e-300;
            double lo = kMachEps - margin, hi = dt + kMachEps + margin;
            bool near_[3];
            bool any = false;
            for (int i = 0; i < 3; ++i) {
                near_[i] = f[i] > lo && f[i] < hi;
                any |= near_[i];
            }
            if (any && rb) {
                bool skip = true;
                for (int i = 0; i < 3 && skip; ++i)
                    if (near_[i]) {
                        const double t = f[i] - kMachEps;
                        skip = t > kMachEps + 2 * margin && t < dt - 2 * margin &&
                               root_misses<EE>(xo4, av4, t, 2 * margin, h, eps);
                    }
                if (skip) {
                    // every root near the window is inside it and misses
                    for (int i = 0; i < 3; ++i) roots[i] = -1;
                    return true;
                }
            }
            if (any) {
                ++*ncr;
                theta = cr::acos(z);
                if (near_[0]) f[0] = -2 * Qsqrt * cr::cos(theta / 3) - a / 3;
                if (near_[1]) f[1] = -2 * Qsqrt * cr::cos((theta + 2 * kPi) / 3) - a / 3;
                if (near_[2]) f[2] = -2 * Qsqrt * cr::cos((theta - 2 * kPi) / 3) - a / 3;
            }
            roots[0] = f[0];
            roots[1] = f[1];
            roots[2] = f[2];
        } else {
            double sgn = (R > 0) ? 1.0 : -1.0;
            double base = fabs(R) + sqrt(R2 - Q3);
            double A = -sgn * pow(base, 1.0 / 3.0);
            double B = (fabs(A) < kRoundEps) ? 0.0 : Q / A;
            double f0 = (A + B) - a / 3.0;
            double f1 = -0.5 * (A + B) - a / 3.0;
            double scale = fabs(A) + fabs(B) + fabs(a);
            double margin = 1e-14 * scale + 1e-300;
            double lo = kMachEps - margin, hi = dt + kMachEps + margin;
            const bool n0 = f0 > lo && f0 < hi, n1 = f1 > lo && f1 < hi;
            const bool thr = fabs(fabs(A) - kRoundEps) <= 1e-14 * fabs(A) + 1e-300 ||
                             fabs(fabs(A - B) - kRoundEps) <= 1e-14 * scale + 1e-300;
            bool near_ = n0 || n1 || thr;
            if (near_ && rb && !thr) {
                // f1 is a root only when |A - B| < ROUND_EPS (no threshold
                // within the margin, so the same holds correctly rounded)
                const bool use1 = fabs(A - B) < kRoundEps;
                bool skip = true;
                if (n0) {
                    const double t = f0 - kMachEps;
                    skip = t > kMachEps + 2 * margin && t < dt - 2 * margin &&
                           root_misses<EE>(xo4, av4, t, 2 * margin, h, eps);
                }
                if (skip && use1 && n1) {
                    const double t = f1 - kMachEps;
                    skip = t > kMachEps + 2 * margin && t < dt - 2 * margin &&
                           root_misses<EE>(xo4, av4, t, 2 * margin, h, eps);
                }
                if (skip && (n0 || (use1 && n1))) {
                    for (int i = 0; i < 3; ++i) roots[i] = -1;
                    return true;
                }
                if (skip) near_ = false;  // f1 near but not a root, f0 far: nothing to form again
            }
            if (near_) {
                ++*ncr;
                A = -sgn * cr::pow(base, 1.0 / 3.0);
                B = (fabs(A) < kRoundEps) ? 0.0 : Q / A;
                f0 = (A + B) - a / 3.0;
                f1 = -0.5 * (A + B) - a / 3.0;
            }
            roots[0] = f0;
            if (fabs(A - B) < kRoundEps) roots[1] = roots[2] = f1;
        }
    } else {
        a = b; b = c; c = d;
        double delta = b * b - 4.0 * a * c;
        if (fabs(a) > kRoundEps && delta > 0) {
            double ds = sqrt(delta);
            roots[0] = (-b + ds) / (2.0 * a);
            roots[1] = (-b - ds) / (2.0 * a);
        } else if (fabs(a) < kRoundEps && fabs(b) > kRoundEps) {
            roots[0] = -c / b;
        }
    }
    for (int i = 0; i < 3; ++i) {
        roots[i] = roots[i] - kMachEps;
        if (roots[i] < 0 || roots[i] > dt) roots[i] = -1;
    }
    double t;
    if (roots[0] > roots[1]) { t = roots[0]; roots[0] = roots[1]; roots[1] = t; }
    if (roots[0] > roots[2]) { t = roots[0]; roots[0] = roots[2]; roots[2] = t; }
    if (roots[1] > roots[2]) { t = roots[1]; roots[1] = roots[2]; roots[2] = t; }
    return roots[0] > kMachEps || roots[1] > kMachEps || roots[2] > kMachEps;
}

// MovingPointToTri / MovingEdgeToEdge, dcollid3d.cpp:327-369: the static
// test with h = eps at each root of the cubic and at dt, first hit wins.
template <bool EE>
static __device__ bool moving_test(const NarrowCtx& c, CallState& st, const int* pts) {
    double xo4[4][3], av4[4][3];
    for (int q = 0; q < 4; ++q) {
        load3(c.xo, pts[q], xo4[q]);
        load3(c.av, pts[q], av4[q]);
    }
    double dt = c.p.dt;
    double roots[4] = {-1, -1, -1, dt};
    if (!is_coplanar<EE>(xo4, av4, dt, roots, &st.ncr, c.robust_roots != 0, c.p.eps, c.p.eps)) return false;
    for (int i = 0; i < 4; ++i) {
        if (roots[i] < 0) continue;
        double X[4][3];
        for (int q = 0; q < 4; ++q)
            for (int k = 0; k < 3; ++k) X[q][k] = xo4[q][k] + roots[i] * av4[q][k];
        bool hit = EE ? edge_to_edge(c, st, pts, X, c.p.eps) : point_to_tri(c, st, pts, X, c.p.eps);
        if (hit) return true;
    }
    return false;
}

template <bool EE>
__device__ __forceinline__ bool static_test(const NarrowCtx& c, CallState& st, const int* pts) {
    double X[4][3];
    for (int q = 0; q < 4; ++q) load3(c.xo, pts[q], X[q]);
    return EE ? edge_to_edge(c, st, pts, X, c.p.thickness) : point_to_tri(c, st, pts, X, c.p.thickness);
}

// Mixed-precision filter. Every position an FP64 test evaluates lies in its
// point's box (x_old and x_old + dt*avgVel, both rounded outward to FP32):
// the roots are in [0, dt] and x_old + t*avgVel rounds monotonically in t.
//  - Edge-edge (dcollid3d.cpp:643-776): the closest points v1, v2 lie on the
//    two segments, so dist >= the segments' distance >= the gap between
//    their boxes; a hit needs dist <= h.
//  - Point-triangle (dcollid3d.cpp:778-922): a hit needs the point within h
//    of the plane and barycentric coordinates in [-eps, 1+eps], so its
//    projection is within 4*eps*diameter of the triangle. The computed
//    coordinates carry a solve error of about 1e-16/sin^2 of the smallest
//    angle, which the reference's determinant cut (|det| >= 1000*MACH_EPS)
//    keeps below 2^-10 for triangles up to unit size: the reach is padded by
//    (8*eps + 2^-10) times the triangle's box extent.
// When the padded boxes do not overlap, the FP64 test returns false and is
// skipped; every other sub-test runs unchanged, so the results are the plain
// FP64 path's.
__device__ __forceinline__ bool mixed_may_hit(const NarrowCtx& c, const int* pts, bool ee, float* ext_out,
                                              float* extb_out) {
    float4 l0 = c.pbox_lo[pts[0]], h0 = c.pbox_hi[pts[0]];
    float4 l1 = c.pbox_lo[pts[1]], h1 = c.pbox_hi[pts[1]];
    float4 l2 = c.pbox_lo[pts[2]], h2 = c.pbox_hi[pts[2]];
    float4 l3 = c.pbox_lo[pts[3]], h3 = c.pbox_hi[pts[3]];
    float alo[3], ahi[3], blo[3], bhi[3];
    if (ee) {
        alo[0] = fminf(l0.x, l1.x); alo[1] = fminf(l0.y, l1.y); alo[2] = fminf(l0.z, l1.z);
        ahi[0] = fmaxf(h0.x, h1.x); ahi[1] = fmaxf(h0.y, h1.y); ahi[2] = fmaxf(h0.z, h1.z);
        blo[0] = fminf(l2.x, l3.x); blo[1] = fminf(l2.y, l3.y); blo[2] = fminf(l2.z, l3.z);
        bhi[0] = fmaxf(h2.x, h3.x); bhi[1] = fmaxf(h2.y, h3.y); bhi[2] = fmaxf(h2.z, h3.z);
    } else {
        alo[0] = fminf(fminf(l0.x, l1.x), l2.x); alo[1] = fminf(fminf(l0.y, l1.y), l2.y);
        alo[2] = fminf(fminf(l0.z, l1.z), l2.z);
        ahi[0] = fmaxf(fmaxf(h0.x, h1.x), h2.x); ahi[1] = fmaxf(fmaxf(h0.y, h1.y), h2.y);
        ahi[2] = fmaxf(fmaxf(h0.z, h1.z), h2.z);
        blo[0] = l3.x; blo[1] = l3.y; blo[2] = l3.z;
        bhi[0] = h3.x; bhi[1] = h3.y; bhi[2] = h3.z;
    }
    float ext = __fadd_ru(__fadd_ru(__fsub_ru(ahi[0], alo[0]), __fsub_ru(ahi[1], alo[1])), __fsub_ru(ahi[2], alo[2]));
    float pad;
    float extb = 0.f;
    if (ee) {
        extb = __fadd_ru(__fadd_ru(__fsub_ru(bhi[0], blo[0]), __fsub_ru(bhi[1], blo[1])), __fsub_ru(bhi[2], blo[2]));
        pad = __fadd_ru(c.hpad, __fmul_ru(__fadd_ru(ext, extb), 0x1p-20f));
    } else {
        pad = __fadd_ru(c.hpad, __fmul_ru(ext, __fadd_ru(__fmul_ru(8.0f, c.epad), 0x1p-10f)));
    }
    *ext_out = ext;
    *extb_out = extb;
    for (int d = 0; d < 3; ++d) {
        if (__fsub_rd(alo[d], pad) > bhi[d]) return false;
        if (__fadd_ru(ahi[d], pad) < blo[d]) return false;
    }
    return true;
}

// Second stage of the mixed-precision filter: a lower bound on the distance
// between the point and the triangle (PT) or between the two segments (EE)
// over the pass's time window, from FP32 copies of the points.
//
// Any direction n gives a lower bound: the gap between the projections of
// the two point sets onto n, divided by |n| (both sets are convex hulls of
// their points, so their projections are spanned by the points'). The
// direction is taken from FP32 closest points (Ericson, Real-Time Collision
// Detection, 2005, 5.1.5 ClosestPtPointTriangle and 5.1.9
// ClosestPtSegmentSegment); how well it is chosen affects only how often
// the bound rejects, never whether the bound holds. The bound is lowered by
//  - the rounding of its own FP32 evaluation, at most 13*u*L for dot
//    products over difference vectors of length <= L (u = 2^-24), and of the
//    points to FP32, at most 2*sqrt(3)*u*M for coordinates of magnitude <= M:
//    together below 32*u*(L + M);
//  - on moving passes, the distance the sets can close within [0, dt]: the
//    distance between two sets changes by at most the largest displacement
//    of a point of each relative to a common reference (a segment's or a
//    triangle's points move by at most the largest displacement of its
//    corners), dt*(D1 + D2) with D the largest |v - v_ref| of each side.
// A hit needs the distance within reach: for PT the plane distance <= h and
// barycentric coordinates >= -eps - dw (dw <= 2^-10, the solve error the
// box stage allows too) put the point within h + 6*(eps + dw)*diam of the
// triangle (padded to 8*(eps + 2^-10)*ext); for EE the clamped closest
// points within h are points of the segments, so the segments are within
// h + 2^-20*ext. Sub-tests whose bound exceeds the reach return false in
// FP64 too and are skipped.
struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float4 a) { return F3{a.x, a.y, a.z}; }
__device__ __forceinline__ F3 fsub(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 fadd(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 fscale(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float fdot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float fnorm(F3 a) { return sqrtf(fdot(a, a)); }
__device__ __forceinline__ float fmaxabs(F3 a) { return fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fabsf(a.z)); }
__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.f), 1.f); }

// Closest point of triangle (a, b, c) to p (Ericson 5.1.5), as an offset
// from a.
__device__ __forceinline__ F3 closest_on_tri(F3 ap, F3 ab, F3 ac) {
    float d1 = fdot(ab, ap), d2 = fdot(ac, ap);
    if (d1 <= 0.f && d2 <= 0.f) return F3{0.f, 0.f, 0.f};
    F3 bp = fsub(ap, ab);
    float d3 = fdot(ab, bp), d4 = fdot(ac, bp);
    if (d3 >= 0.f && d4 <= d3) return ab;
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) return fscale(ab, d1 / (d1 - d3));
    F3 cp = fsub(ap, ac);
    float d5 = fdot(ab, cp), d6 = fdot(ac, cp);
    if (d6 >= 0.f && d5 <= d6) return ac;
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) return fscale(ac, d2 / (d2 - d6));
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return fadd(ab, fscale(fsub(ac, ab), w));
    }
    float den = 1.f / (va + vb + vc);
    return fadd(fscale(ab, vb * den), fscale(ac, vc * den));
}

template <bool MOVING, bool EE>
__device__ __forceinline__ bool sat_may_hit(const NarrowCtx& c, const int* pts, float ext, float extb) {
    F3 X[4];
    for (int q = 0; q < 4; ++q) X[q] = f3(c.p32[pts[q]]);
    float M = fmaxf(fmaxf(fmaxabs(X[0]), fmaxabs(X[1])), fmaxf(fmaxabs(X[2]), fmaxabs(X[3])));
    float lb, L, reach;
    if (!EE) {
        // triangle X0 X1 X2, point X3; origin X0
        F3 ab = fsub(X[1], X[0]), ac = fsub(X[2], X[0]), ap = fsub(X[3], X[0]);
        F3 n = fsub(ap, closest_on_tri(ap, ab, ac));
        float nn = fnorm(n);
        if (!(nn > 0.f)) return true;
        float gap = fdot(n, ap) - fmaxf(0.f, fmaxf(fdot(n, ab), fdot(n, ac)));
        lb = gap / nn;
        L = fmaxf(fmaxf(fnorm(ab), fnorm(ac)), fnorm(ap));
        reach = __fadd_ru(c.hpad, __fmul_ru(ext, __fmul_ru(8.0f, __fadd_ru(c.epad, 0x1p-10f))));
    } else {
        // segments S1 = X0 X1, S2 = X2 X3; origin X2
        F3 d1 = fsub(X[1], X[0]), d2 = fsub(X[3], X[2]), r = fsub(X[0], X[2]);
        float a = fdot(d1, d1), e = fdot(d2, d2), f = fdot(d2, r);
        float s = 0.f, t = 0.f;
        if (a > 0.f && e > 0.f) {
            float cc = fdot(d1, r), b = fdot(d1, d2), den = a * e - b * b;
            s = den > 0.f ? clamp01((b * f - cc * e) / den) : 0.f;
            t = (b * s + f) / e;
            if (t < 0.f) {
                t = 0.f;
                s = clamp01(-cc / a);
            } else if (t > 1.f) {
                t = 1.f;
                s = clamp01((b - cc) / a);
            }
        } else if (a > 0.f) {
            s = clamp01(-fdot(d1, r) / a);
        } else if (e > 0.f) {
            t = clamp01(f / e);
        }
        // n from S2's closest point to S1's
        F3 n = fsub(fadd(r, fscale(d1, s)), fscale(d2, t));
        float nn = fnorm(n);
        if (!(nn > 0.f)) return true;
        F3 q1 = fadd(r, d1);  // X1 - X2
        float gap = fminf(fdot(n, r), fdot(n, q1)) - fmaxf(0.f, fdot(n, d2));
        lb = gap / nn;
        L = fmaxf(fmaxf(fnorm(r), fnorm(q1)), fnorm(d2));
        reach = __fadd_ru(c.hpad, __fmul_ru(__fadd_ru(ext, extb), 0x1p-20f));
    }
    float err = __fmul_ru(32.0f * 0x1p-24f, __fadd_ru(L, M));
    float bound = __fsub_rd(lb, err);
    if (MOVING) {
        F3 V[4];
        for (int q = 0; q < 4; ++q) V[q] = f3(c.v32[pts[q]]);
        // reference velocity: the first point's
        float D1, D2;
        if (!EE) {
            D1 = fmaxf(fmaxf(fnorm(fsub(V[1], V[0])), fnorm(fsub(V[2], V[0]))), 0.f);
            D2 = fnorm(fsub(V[3], V[0]));
        } else {
            D1 = fnorm(fsub(V[1], V[0]));
            D2 = fmaxf(fnorm(fsub(V[2], V[0])), fnorm(fsub(V[3], V[0])));
        }
        float Vm = fmaxf(fmaxf(fmaxabs(V[0]), fmaxabs(V[1])), fmaxf(fmaxabs(V[2]), fmaxabs(V[3])));
        // FP32 rounding of the velocities and of the sums above
        float dv = __fadd_ru(__fmul_ru(__fadd_ru(D1, D2), 1.0f + 0x1p-16f), __fmul_ru(Vm, 32.0f * 0x1p-24f));
        bound = __fsub_rd(bound, __fmul_ru(c.dt32, dv));
    }
    return !(bound > reach);
}

__device__ __forceinline__ F3 fcross(F3 a, F3 b) {
    return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Element-pair stage of the mixed-precision filter: one lower bound on the
// distance between the two elements (as point sets) over the pass's time
// window. Every sub-test of the pair involves a point or an edge of each
// element, so its distance is at least this one, and when the bound exceeds
// the largest reach of the pair's sub-tests none of them can hit. The bound
// is the separating-axis gap (as in sat_may_hit, with the same rounding and
// motion allowances) maximised over a few axes: each triangle's normal and
// its three in-plane edge normals (for two disjoint coplanar triangles one of
// those separates them), for two segments their common normal and the
// in-plane normals of each, and the line between the centroids.
// Gap between the projections of two point sets (3 points each) onto ax,
// divided by |ax|: a lower bound on their distance (-1 for a zero axis).
__device__ __forceinline__ float axis_gap(F3 ax, const F3* R) {
    float an = fnorm(ax);
    if (!(an > 0.f)) return -1.f;
    float amin = fdot(ax, R[0]), amax = amin, bmin = fdot(ax, R[3]), bmax = bmin;
#pragma unroll
    for (int q = 1; q < 3; ++q) {
        float ta = fdot(ax, R[q]), tb = fdot(ax, R[3 + q]);
        amin = fminf(amin, ta);
        amax = fmaxf(amax, ta);
        bmin = fminf(bmin, tb);
        bmax = fmaxf(bmax, tb);
    }
    return fmaxf(bmin - amax, amin - bmax) / an;
}

template <bool MOVING>
__device__ __forceinline__ bool pair_may_hit(const NarrowCtx& c, const int* A, int na, const int* B, int nb) {
    // points relative to A's first; a segment's third point repeats its
    // second (the same convex hull, so the same projections)
    const int ia[3] = {A[0], A[1], na == 3 ? A[2] : A[1]};
    const int ib[3] = {B[0], B[1], nb == 3 ? B[2] : B[1]};
    F3 R[6];
    const F3 X0 = f3(c.p32[ia[0]]);
    float M = fmaxabs(X0), L = 0.f;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        F3 x = q < 3 ? f3(c.p32[ia[q]]) : f3(c.p32[ib[q - 3]]);
        M = fmaxf(M, fmaxabs(x));
        R[q] = fsub(x, X0);
        L = fmaxf(L, fnorm(R[q]));
    }
    float lb = -1.f;
    {
        F3 cA = fscale(fadd(fadd(R[0], R[1]), R[2]), 1.f / 3.f);
        F3 cB = fscale(fadd(fadd(R[3], R[4]), R[5]), 1.f / 3.f);
        lb = fmaxf(lb, axis_gap(fsub(cB, cA), R));
    }
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const F3* P = R + 3 * side;
        F3 e0 = fsub(P[1], P[0]), e1 = fsub(P[2], P[1]), e2 = fsub(P[0], P[2]);
        F3 nrm = fcross(e0, fsub(P[2], P[0]));  // zero for a segment: skipped
        lb = fmaxf(lb, axis_gap(nrm, R));
        lb = fmaxf(lb, axis_gap(fcross(nrm, e0), R));
        lb = fmaxf(lb, axis_gap(fcross(nrm, e1), R));
        lb = fmaxf(lb, axis_gap(fcross(nrm, e2), R));
    }
    {
        F3 d1 = fsub(R[1], R[0]), d2 = fsub(R[4], R[3]);
        F3 nrm = fcross(d1, d2);
        lb = fmaxf(lb, axis_gap(nrm, R));
        lb = fmaxf(lb, axis_gap(fcross(nrm, d1), R));
        lb = fmaxf(lb, axis_gap(fcross(nrm, d2), R));
    }
    // the largest reach of the pair's sub-tests, with the boxes' extents
    float extA, extB;
    {
        float4 l = c.pbox_lo[ia[0]], h = c.pbox_hi[ia[0]];
        float lo[3] = {l.x, l.y, l.z}, hi[3] = {h.x, h.y, h.z};
#pragma unroll
        for (int q = 1; q < 3; ++q) {
            l = c.pbox_lo[ia[q]];
            h = c.pbox_hi[ia[q]];
            lo[0] = fminf(lo[0], l.x); lo[1] = fminf(lo[1], l.y); lo[2] = fminf(lo[2], l.z);
            hi[0] = fmaxf(hi[0], h.x); hi[1] = fmaxf(hi[1], h.y); hi[2] = fmaxf(hi[2], h.z);
        }
        extA = __fadd_ru(__fadd_ru(__fsub_ru(hi[0], lo[0]), __fsub_ru(hi[1], lo[1])), __fsub_ru(hi[2], lo[2]));
        l = c.pbox_lo[ib[0]];
        h = c.pbox_hi[ib[0]];
        float lo2[3] = {l.x, l.y, l.z}, hi2[3] = {h.x, h.y, h.z};
#pragma unroll
        for (int q = 1; q < 3; ++q) {
            l = c.pbox_lo[ib[q]];
            h = c.pbox_hi[ib[q]];
            lo2[0] = fminf(lo2[0], l.x); lo2[1] = fminf(lo2[1], l.y); lo2[2] = fminf(lo2[2], l.z);
            hi2[0] = fmaxf(hi2[0], h.x); hi2[1] = fmaxf(hi2[1], h.y); hi2[2] = fmaxf(hi2[2], h.z);
        }
        extB = __fadd_ru(__fadd_ru(__fsub_ru(hi2[0], lo2[0]), __fsub_ru(hi2[1], lo2[1])), __fsub_ru(hi2[2], lo2[2]));
    }
    float ext_tri = fmaxf(na == 3 ? extA : 0.f, nb == 3 ? extB : 0.f);
    float reach_pt = __fmul_ru(ext_tri, __fmul_ru(8.0f, __fadd_ru(c.epad, 0x1p-10f)));
    float reach_ee = __fmul_ru(__fadd_ru(extA, extB), 0x1p-20f);
    float reach = __fadd_ru(c.hpad, fmaxf(reach_pt, reach_ee));
    float err = __fmul_ru(32.0f * 0x1p-24f, __fadd_ru(L, M));
    float bound = __fsub_rd(lb, err);
    if (MOVING) {
        F3 v0 = f3(c.v32[ia[0]]);
        float DA = 0.f, DB = 0.f, Vm = fmaxabs(v0);
#pragma unroll
        for (int q = 1; q < 3; ++q) {
            F3 v = f3(c.v32[ia[q]]);
            DA = fmaxf(DA, fnorm(fsub(v, v0)));
            Vm = fmaxf(Vm, fmaxabs(v));
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            F3 v = f3(c.v32[ib[q]]);
            DB = fmaxf(DB, fnorm(fsub(v, v0)));
            Vm = fmaxf(Vm, fmaxabs(v));
        }
        float dv = __fadd_ru(__fmul_ru(__fadd_ru(DA, DB), 1.0f + 0x1p-16f), __fmul_ru(Vm, 32.0f * 0x1p-24f));
        bound = __fsub_rd(bound, __fmul_ru(c.dt32, dv));
    }
    return !(bound > reach);
}

template <bool MOVING, bool EE>
__device__ __forceinline__ bool sub_test(const NarrowCtx& c, CallState& st, const int* pts) {
    if (c.pbox_lo) {
        float ext, extb;
        if (!mixed_may_hit(c, pts, EE, &ext, &extb)) return false;
        if (!sat_may_hit<MOVING, EE>(c, pts, ext, extb)) return false;
    }
    st.nsub++;
    if (MOVING) return moving_test<EE>(c, st, pts);
    return static_test<EE>(c, st, pts);
}

// ------------------------------------------------------ element-pair tests
// TriToTri (dcollid3d.cpp:570-627) and MovingTriToTri (dcollid3d.cpp:274-325).
// A = found element, B = query element.
template <bool MOVING>
static __device__ bool tri_to_tri(const NarrowCtx& c, CallState& st, const int* A, const int* B) {
    int pts[4];
    bool status = false;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (A[i] == B[j]) return false;
    int sub = 0;
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < 3; ++i, ++sub) {
            // proximity tests B's triangle against A's points first; CCD the reverse
            const int* tri = MOVING ? ((k == 0) ? A : B) : ((k == 0) ? B : A);
            const int* pt = MOVING ? ((k == 0) ? B : A) : ((k == 0) ? A : B);
            for (int j = 0; j < 3; ++j) pts[j] = tri[j];
            pts[3] = pt[i];
            st.sub = sub;
            if (sub_test<MOVING, false>(c, st, pts)) status = true;
            if (MOVING && status && c.zone) create_imp_zone(c, st, pts);
        }
    for (int i = 0; i < 3; ++i) {
        pts[0] = A[i];
        pts[1] = A[(i + 1) % 3];
        for (int j = 0; j < 3; ++j, ++sub) {
            pts[2] = B[j];
            pts[3] = B[(j + 1) % 3];
            st.sub = sub;
            if (sub_test<MOVING, true>(c, st, pts)) status = true;
            if (MOVING && status && c.zone) create_imp_zone(c, st, pts);
        }
    }
    return status;
}

// TriToBond (dcollid3d.cpp:485-533) and MovingTriToBond (dcollid3d.cpp:203-244).
template <bool MOVING>
static __device__ bool tri_to_bond(const NarrowCtx& c, CallState& st, const int* T, const int* Bd) {
    int pts[4];
    bool status = false;
    for (int i = 0; i < 3; ++i)
        if (T[i] == Bd[0] || T[i] == Bd[1]) return false;
    for (int i = 0; i < 3; ++i) pts[i] = T[i];
    for (int e = 0; e < 2; ++e) {
        pts[3] = Bd[e];
        st.sub = e;
        if (sub_test<MOVING, false>(c, st, pts)) status = true;
        if (MOVING && status && c.zone) create_imp_zone(c, st, pts);
    }
    pts[2] = Bd[0];
    pts[3] = Bd[1];
    for (int i = 0; i < 3; ++i) {
        pts[0] = T[i];
        pts[1] = T[(i + 1) % 3];
        st.sub = 2 + i;
        if (sub_test<MOVING, true>(c, st, pts)) status = true;
        if (MOVING && status && c.zone) create_imp_zone(c, st, pts);
    }
    return status;
}

// BondToBond (dcollid3d.cpp:535-568) and MovingBondToBond (dcollid3d.cpp:246-272).
template <bool MOVING>
static __device__ bool bond_to_bond(const NarrowCtx& c, CallState& st, const int* A, const int* B) {
    int pts[4] = {A[0], A[1], B[0], B[1]};
    for (int i = 0; i < 4; ++i)
        for (int j = i + 1; j < 4; ++j)
            if (pts[i] == pts[j]) return false;
    st.sub = 0;
    bool status = sub_test<MOVING, true>(c, st, pts);
    if (MOVING && status && c.zone) create_imp_zone(c, st, pts);
    return status;
}

}  // namespace ccg
