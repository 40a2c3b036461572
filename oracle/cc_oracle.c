/*
 * CPU restatement of antdvid/Collision's collision-handling step,
 * CollisionSolver3d::resolveCollision() (dcollid.cpp:317-362), in plain C.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle: tests/ compare the GPU
 * library with it, __graft_entry__.smoke() checks one GPU step against it,
 * and bench.py times it as the CPU baseline. The shipped library never links
 * or calls it.
 *
 * It restates the reference operation by operation, in the reference's
 * order of floating-point evaluation, so that with contraction off
 * (-ffp-contract=off) it reproduces the reference's results bit for bit; that
 * is pinned by tests/test_oracle_pin.py against the reference compiled from
 * its own sources (oracle/Makefile.ref) and by the golden fixtures in
 * tests/golden/. Each function names the reference lines it follows. Two
 * deliberate differences, neither reachable by the pinned scenes: the
 * impact-zone loop, unbounded in the reference (dcollid.cpp:236), stops with
 * CCO_ITER_CAP after a configurable cap, and fatal errors return a status
 * instead of exiting (clean_up(ERROR)).
 *
 * Movable rigid bodies follow the reference's is_movableRG branches: each
 * surface whose first point is movable is one impact zone from the start of
 * a step (createImpZoneForRG, dcollid3d.cpp:54-68), impulses between rigid
 * points spread over that zone (SpreadImpactZoneImpulse, dcollid.cpp:
 * 1101-1115), the zone moves rigidly after every pass
 * (updateImpactZoneVelocityForRG, dcollid.cpp:267-288), and its centre of
 * mass is advanced at the end (updateFinalForRG, dcollid.cpp:626-675). Out
 * of scope, as for the GPU library: the 2D solver, debug printing.
 */
#include "cc_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
/* The reference's libm calls (isCoplanar, updateImpactListVelocity). Built
 * with CCO_CRMATH, the correctly rounded versions of cc_oracle_crmath.cpp
 * take their place: the reference's algorithm with correctly rounded
 * transcendental functions, which tells a difference that comes from
 * glibc's rare misroundings apart from any other. */
#ifdef CCO_CRMATH
double cco_cr_acos(double x);
double cco_cr_cos(double x);
double cco_cr_sin(double x);
double cco_cr_pow(double x, double y);
#define LM_ACOS cco_cr_acos
#define LM_COS cco_cr_cos
#define LM_SIN cco_cr_sin
#define LM_POW cco_cr_pow
#else
#define LM_ACOS acos
#define LM_COS cos
#define LM_SIN sin
#define LM_POW pow
#endif
#define MACH_EPS DBL_EPSILON
#define ROUND_EPS 1e-10     /* collid.h:17 */
#define BOX_PAD 1e-6        /* AABB.cpp:10-11, 15-16, 65-71 */
#define BIG 1.0e38          /* the reference's HUGE, a min/max identity */
#define MAX_CCD_ITER 5      /* dcollid.cpp:433 */
#define STRAIN_TOL 0.10     /* dcollid.cpp:489 */
#define STRAIN_MAX_ITER 10  /* dcollid.cpp:590 */

enum { PASS_PROX = 0, PASS_CCD = 1, PASS_ZONE = 2 };
enum { TREE_STATIC = 0, TREE_MOVING = 1 };

typedef struct {
    double lo[3], hi[3];
} box_t;

/* Incremental AABB tree, AABB.h:96-120 / AABB.cpp:129-343. Leaves are nodes
 * 0..E-1 (node e holds element e, the reference's nodeArray order); internal
 * nodes are allocated from E upward and abandoned on a rebuild, as the
 * reference leaks them (AABB.cpp:149-161). */
typedef struct {
    int ne;
    int cap;
    int nnodes;
    int root;
    int built;
    box_t* box;
    int* left;
    int* right;
    unsigned char* queried; /* nodeSet, AABB.h:108 */
    int* stack;
    int* stack2;
    int count;              /* hits in the current pass (AABB.h:110) */
} tree_t;

struct cco_solver {
    int nv, nt, nb, ne;
    int* ev;      /* ne*3 vertex ids (bonds: 2, third -1) */
    int* enp;     /* points per element */
    int* esurf;   /* surface id (tris), -1 for bonds */
    double* erest;/* ne*3 rest lengths (side_length0 / length0) */
    unsigned char* fixed; /* bit 0 is_fixed, bit 1 is_movableRG */
    unsigned char* in_elem;

    /* surfaces in element order, each with its HYPER_SURF body data */
    int nsurf;
    int *surf_id, *surf_t0, *surf_t1;
    int* vsurf;           /* surface of each point (pt->hs), -1 for none */
    double *surf_mass, *surf_com, *surf_comv;
    double* mrg_com;      /* CollisionSolver::mrg_com, collid.h:174 */
    unsigned char* mrg_set;
    double* imp_rg;       /* collsnImpulse_RG: the solver never clears it */
    int* num_rg;          /* collsn_num_RG */

    /* per-point state (STATE, collid.h:20-39) */
    double *coords, *x_old, *vel, *avg, *imp, *fric;
    int* num;
    unsigned char *has_collsn, *sorted;
    int *uf_root, *uf_next, *uf_tail, *uf_w;

    /* parameters (class statics, collid.h:134-140) */
    double dt, thickness, eps, k, m, lambda, cr;
    double L[3], U[3];
    int det_imp_zone; /* s_detImpZone */

    tree_t tree[2];
    double volume;    /* shared by both trees, collid.h:133 */

    int pass;
    int zone_cap;
    int status;
    int record;
    int npass, pass_cap;
    int* pass_kind;
    cco_pair_rec* pairs;
    int npairs, pairs_cap;
    cco_contact_rec* contacts;
    int ncontacts, contacts_cap;
    double* snaps;
    int nsnaps, snaps_cap;

    /* current narrow-phase call being recorded */
    int cur_a, cur_b, cur_kind, cur_sub;
    long long ctr[7];
    int check; /* cco_check_ccd: hit decisions only, no impulses */
};

/* ------------------------------------------------------------ vector ops */
/* FronTier macros as pinned by oracle/stub/inc/FronTier.h. */
static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline double mag3(const double* a) { return sqrt(dot3(a, a)); }
static inline void cross3(const double* b, const double* c, double* ans) {
    ans[0] = b[1] * c[2] - b[2] * c[1];
    ans[1] = b[2] * c[0] - b[0] * c[2];
    ans[2] = b[0] * c[1] - b[1] * c[0];
}
static inline double sqr(double x) { return x * x; }
static inline double dist_pos(const double* p, const double* q) {
    double s = 0.0;
    for (int i = 0; i < 3; ++i) s += sqr(p[i] - q[i]);
    return sqrt(s);
}
/* std::min / std::max argument conventions */
static inline double smin(double a, double b) { return (b < a) ? b : a; }
static inline double smax(double a, double b) { return (a < b) ? b : a; }

#define XO(p) (s->x_old + 3 * (p))
#define CO(p) (s->coords + 3 * (p))
#define AV(p) (s->avg + 3 * (p))

static inline int is_static(const cco_solver* s, int p) { return (s->fixed[p] & 1) != 0; }
static inline int is_movable(const cco_solver* s, int p) { return (s->fixed[p] & 2) != 0; }
static inline int is_rigid(const cco_solver* s, int p) { return s->fixed[p] != 0; }
/* isRigidBody(hse), dcollid.cpp:1097-1099: a point of the element is fixed
 * or movable */
static int elem_rigid(const cco_solver* s, int e) {
    for (int i = 0; i < s->enp[e]; ++i)
        if (is_rigid(s, s->ev[3 * e + i])) return 1;
    return 0;
}

/* ------------------------------------------------------------- recording */
static void* grow(void* p, int* cap, int need, size_t sz) {
    if (need <= *cap) return p;
    int nc = *cap ? *cap : 256;
    while (nc < need) nc *= 2;
    void* q = realloc(p, (size_t)nc * sz);
    if (!q) return NULL;
    *cap = nc;
    return q;
}

static void rec_contact(cco_solver* s, const int* pts) {
    s->ctr[3]++;
    if (!(s->record & 2)) return;
    cco_contact_rec* c = grow(s->contacts, &s->contacts_cap, s->ncontacts + 1, sizeof(*c));
    if (!c) { s->status = CCO_NOMEM; return; }
    s->contacts = c;
    cco_contact_rec* r = &c[s->ncontacts++];
    r->pass = s->pass; r->kind = s->cur_kind; r->a = s->cur_a; r->b = s->cur_b;
    r->subtest = s->cur_sub;
    for (int i = 0; i < 4; ++i) r->v[i] = pts[i];
}

/* ------------------------------------------------------------ union-find */
/* makeSet / findSet / mergePoint / createImpZone, dcollid.cpp:1015-1059, 473-484 */
static int find_set(cco_solver* s, int p) {
    int r = p;
    while (s->uf_root[r] != r) r = s->uf_root[r];
    while (s->uf_root[p] != r) { /* path compression, as the recursion does */
        int n = s->uf_root[p];
        s->uf_root[p] = r;
        p = n;
    }
    return r;
}

static void merge_point(cco_solver* s, int x, int y) {
    int px = find_set(s, x), py = find_set(s, y);
    if (px == py) return;
    if (s->uf_w[px] > s->uf_w[py]) {
        s->uf_w[px] += s->uf_w[py];
        s->uf_root[py] = px;
        s->uf_next[s->uf_tail[px]] = py;
        s->uf_tail[px] = s->uf_tail[py];
    } else {
        s->uf_w[py] += s->uf_w[px];
        s->uf_root[px] = py;
        s->uf_next[s->uf_tail[py]] = px;
        s->uf_tail[py] = s->uf_tail[px];
    }
}

/* createImpZone(pts, num, first): with first = NO, pairs with a movable
 * point are left apart */
static void create_imp_zone(cco_solver* s, const int* pts, int num, int first) {
    for (int i = 0; i < num; ++i)
        for (int j = 0; j < i; ++j) {
            if (!first && (is_movable(s, pts[i]) || is_movable(s, pts[j]))) continue;
            merge_point(s, pts[i], pts[j]);
        }
}

/* SpreadImpactZoneImpulse, dcollid.cpp:1101-1115: every member of p's zone */
static void spread_impact_zone_impulse(cco_solver* s, int p, double impulse, const double* nor) {
    for (int q = find_set(s, p); q >= 0; q = s->uf_next[q]) {
        for (int i = 0; i < 3; ++i) s->imp_rg[3 * q + i] += impulse * nor[i];
        s->num_rg[q] += 1;
    }
}

/* total_mass(p->hs) */
static double body_mass(const cco_solver* s, int p) { return s->vsurf[p] >= 0 ? s->surf_mass[s->vsurf[p]] : 0.0; }

/* -------------------------------------------------------------- impulses */
/* PointToTriImpulse, dcollid3d.cpp:925-1107. */
static void point_to_tri_impulse(cco_solver* s, const int* pts, const double* nor, double* w, double dist) {
    double v_rel[3] = {0.0, 0.0, 0.0}, vn, vt;
    double impulse = 0.0, m_impulse, sum_w = 0.0;
    double rigid_impulse[2] = {0.0, 0.0};
    const double k = s->k, m = s->m, dt = s->dt, lambda = s->lambda, h = s->thickness, cr = s->cr;
    dist = h - dist;
    for (int i = 0; i < 3; ++i) {
        v_rel[i] += AV(pts[3])[i];
        for (int j = 0; j < 3; ++j) v_rel[i] -= w[j] * AV(pts[j])[i];
    }
    vn = dot3(v_rel, nor);
    if (dot3(v_rel, v_rel) > sqr(vn))
        vt = sqrt(dot3(v_rel, v_rel) - sqr(vn));
    else
        vt = 0.0;
    if (vn < 0) {
        if (is_static(s, pts[3]) || (is_static(s, pts[0]) && is_static(s, pts[1]) && is_static(s, pts[2]))) {
            impulse = vn;
            rigid_impulse[0] = vn;
            rigid_impulse[1] = vn;
        } else if (is_movable(s, pts[0]) && is_movable(s, pts[1]) && is_movable(s, pts[2]) &&
                   is_movable(s, pts[3])) {
            double m1 = body_mass(s, pts[0]), m2 = body_mass(s, pts[3]);
            rigid_impulse[0] = vn * m2 / (m1 + m2);
            rigid_impulse[1] = vn * m1 / (m1 + m2);
        } else if (is_movable(s, pts[0]) && is_movable(s, pts[1]) && is_movable(s, pts[2])) {
            rigid_impulse[0] = 0.5 * vn;
            impulse = 0.5 * vn;
        } else if (is_movable(s, pts[3])) {
            impulse = 0.5 * vn;
            rigid_impulse[1] = 0.5 * vn;
        } else {
            impulse = vn * 0.5;
        }
        for (int i = 0; i < 3; ++i) {
            if (is_static(s, pts[i])) w[i] = 0.0;
            sum_w += w[i];
        }
        if (fabs(sum_w) > MACH_EPS) {
            double inv = 1.0 / sum_w;
            for (int i = 0; i < 3; ++i) w[i] = inv * w[i];
        }
    }
    int all_rigid = is_rigid(s, pts[0]) && is_rigid(s, pts[1]) && is_rigid(s, pts[2]) && is_rigid(s, pts[3]);
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
    if (fabs(sum_w) < MACH_EPS)
        m_impulse = impulse;
    else
        m_impulse = 2.0 * impulse / (1.0 + dot3(w, w));
    if (all_rigid) {
        if (is_movable(s, pts[0])) spread_impact_zone_impulse(s, pts[0], rigid_impulse[0], nor);
        if (is_movable(s, pts[3])) spread_impact_zone_impulse(s, pts[3], -1.0 * rigid_impulse[1], nor);
        return;
    }
    for (int i = 0; i < 3; ++i) {
        int p = pts[i];
        if (is_static(s, p)) continue;
        double t_impulse = m_impulse;
        if (is_movable(s, p)) t_impulse = rigid_impulse[0];
        for (int j = 0; j < 3; ++j) {
            s->imp[3 * p + j] += w[i] * t_impulse * nor[j];
            if (fabs(vt) > ROUND_EPS)
                s->fric[3 * p + j] += smax(-fabs(lambda * w[i] * t_impulse / vt), -1.0) * (v_rel[j] - vn * nor[j]);
        }
        s->num[p] += 1;
    }
    if (!is_static(s, pts[3])) {
        int p = pts[3];
        double t_impulse = m_impulse;
        if (is_movable(s, p)) t_impulse = rigid_impulse[1];
        for (int j = 0; j < 3; ++j) {
            s->imp[3 * p + j] -= t_impulse * nor[j];
            if (fabs(vt) > ROUND_EPS)
                s->fric[3 * p + j] += smax(-fabs(lambda * t_impulse / vt), -1.0) * (v_rel[j] - vn * nor[j]);
        }
        s->num[p] += 1;
    }
    for (int j = 0; j < 4; ++j)
        for (int i = 0; i < 3; ++i)
            if (!isfinite(s->imp[3 * pts[j] + i])) s->status = CCO_NAN;
}

/* EdgeToEdgeImpulse, dcollid3d.cpp:1109-1300. */
static void edge_to_edge_impulse(cco_solver* s, const int* pts, const double* nor, double a, double b, double dist) {
    double v_rel[3], vn, vt;
    double impulse = 0.0, m_impulse;
    double rigid_impulse[2] = {0.0, 0.0};
    const double k = s->k, m = s->m, dt = s->dt, lambda = s->lambda, h = s->thickness, cr = s->cr;
    double wa[2] = {1.0 - a, a}, wb[2] = {1.0 - b, b};
    dist = h - dist;
    for (int j = 0; j < 3; ++j) {
        v_rel[j] = (1.0 - b) * AV(pts[2])[j] + b * AV(pts[3])[j];
        v_rel[j] -= (1.0 - a) * AV(pts[0])[j] + a * AV(pts[1])[j];
    }
    vn = dot3(v_rel, nor);
    if (dot3(v_rel, v_rel) > sqr(vn))
        vt = sqrt(dot3(v_rel, v_rel) - sqr(vn));
    else
        vt = 0.0;
    if (vn < 0.0) {
        if ((is_static(s, pts[0]) && is_static(s, pts[1])) || (is_static(s, pts[2]) && is_static(s, pts[3]))) {
            impulse = vn;
            rigid_impulse[0] = vn;
            rigid_impulse[1] = vn;
        } else if (is_movable(s, pts[0]) && is_movable(s, pts[1]) && is_movable(s, pts[2]) &&
                   is_movable(s, pts[3])) {
            double m1 = body_mass(s, pts[0]), m2 = body_mass(s, pts[2]);
            rigid_impulse[0] = vn * m2 / (m1 + m2);
            rigid_impulse[1] = vn * m1 / (m1 + m2);
        } else if (is_movable(s, pts[0]) && is_movable(s, pts[1])) {
            rigid_impulse[0] = 0.5 * vn;
            impulse = 0.5 * vn;
        } else if (is_movable(s, pts[2]) && is_movable(s, pts[3])) {
            impulse = 0.5 * vn;
            rigid_impulse[1] = 0.5 * vn;
        } else {
            impulse = vn * 0.5;
        }
        if (is_static(s, pts[0])) wa[0] = 0.0;
        if (is_static(s, pts[1])) wa[1] = 0.0;
        if (is_static(s, pts[2])) wb[0] = 0.0;
        if (is_static(s, pts[3])) wb[1] = 0.0;
    }
    int all_rigid = is_rigid(s, pts[0]) && is_rigid(s, pts[1]) && is_rigid(s, pts[2]) && is_rigid(s, pts[3]);
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
    if (wa[0] + wa[1] < MACH_EPS || wb[0] + wb[1] < MACH_EPS)
        m_impulse = impulse;
    else
        m_impulse = 2.0 * impulse / (wa[0] * wa[0] + wa[1] * wa[1] + wb[0] * wb[0] + wb[1] * wb[1]);
    if (all_rigid) {
        if (is_movable(s, pts[0])) spread_impact_zone_impulse(s, pts[0], rigid_impulse[0], nor);
        if (is_movable(s, pts[2])) spread_impact_zone_impulse(s, pts[2], -1.0 * rigid_impulse[1], nor);
        return;
    }
    const double wgt[4] = {wa[0], wa[1], wb[0], wb[1]};
    for (int j = 0; j < 3; ++j) {
        for (int q = 0; q < 4; ++q) {
            int p = pts[q];
            if (is_static(s, p)) continue;
            double t_impulse = m_impulse;
            if (is_movable(s, p)) t_impulse = rigid_impulse[q < 2 ? 0 : 1];
            if (q < 2)
                s->imp[3 * p + j] += wgt[q] * t_impulse * nor[j];
            else
                s->imp[3 * p + j] -= wgt[q] * t_impulse * nor[j];
            if (fabs(vt) > ROUND_EPS)
                s->fric[3 * p + j] += smax(-fabs(lambda * wgt[q] * t_impulse / vt), -1.0) * (v_rel[j] - vn * nor[j]);
            if (j == 0) s->num[p] += 1;
        }
    }
    for (int q = 0; q < 4; ++q)
        for (int i = 0; i < 3; ++i)
            if (!isfinite(s->imp[3 * pts[q] + i])) s->status = CCO_NAN;
}

/* ---------------------------------------------------- proximity kernels */
/* PointToTri, dcollid3d.cpp:778-922. pts[0..2] the triangle, pts[3] the point. */
static int point_to_tri(cco_solver* s, const int* pts, double h) {
    double w[3] = {0.0, 0.0, 0.0};
    double x13[3], x23[3], x43[3];
    double nor[3] = {0.0, 0.0, 0.0}, nor_mag, dist, det;
    for (int i = 0; i < 3; ++i) {
        x13[i] = CO(pts[0])[i] - CO(pts[2])[i];
        x23[i] = CO(pts[1])[i] - CO(pts[2])[i];
        x43[i] = CO(pts[3])[i] - CO(pts[2])[i];
    }
    det = dot3(x13, x13) * dot3(x23, x23) - dot3(x13, x23) * dot3(x13, x23);
    if (fabs(det) < 1000 * MACH_EPS) return 0;
    cross3(x13, x23, nor);
    nor_mag = mag3(nor);
    double x43_old[3];
    for (int i = 0; i < 3; ++i) x43_old[i] = XO(pts[3])[i] - XO(pts[2])[i];
    dist = dot3(x43_old, nor);
    for (int i = 0; i < 3; ++i) nor[i] /= nor_mag * ((dist >= 0) ? 1.0 : -1.0);
    dist = fabs(dot3(x43, nor));
    w[0] = (dot3(x13, x43) * dot3(x23, x23) - dot3(x23, x43) * dot3(x13, x23)) / det;
    w[1] = (dot3(x13, x13) * dot3(x23, x43) - dot3(x13, x23) * dot3(x13, x43)) / det;
    w[2] = 1 - w[0] - w[1];
    if (fabs(w[0]) < ROUND_EPS || fabs(w[1]) < ROUND_EPS || fabs(w[2]) < ROUND_EPS) {
        double vec[3];
        for (int j = 0; j < 3; ++j) vec[j] = XO(pts[3])[j];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) vec[j] -= w[i] * XO(pts[i])[j];
        double vec_mag = mag3(vec);
        if (vec_mag > ROUND_EPS)
            for (int j = 0; j < 3; ++j) nor[j] = vec[j];
    }
    nor_mag = mag3(nor);
    if (nor_mag > ROUND_EPS) {
        for (int i = 0; i < 3; ++i) nor[i] /= nor_mag;
    } else {
        s->status = CCO_NAN; /* "nan nor vec", clean_up(ERROR) */
        return 0;
    }
    if (dist > h) return 0;
    for (int i = 0; i < 3; ++i)
        if (w[i] > 1 + s->eps || w[i] < -s->eps) return 0;
    if (s->check) return 1;
    rec_contact(s, pts);
    point_to_tri_impulse(s, pts, nor, w, dist);
    return 1;
}

/* EdgeToEdge, dcollid3d.cpp:643-776. Edges (pts[0],pts[1]) and (pts[2],pts[3]). */
static int edge_to_edge(cco_solver* s, const int* pts, double h) {
    double x21[3], x43[3], x31[3], tmp[3], v1[3], v2[3], nor[3];
    double a, b, nor_mag, dist;
    for (int i = 0; i < 3; ++i) {
        x21[i] = CO(pts[1])[i] - CO(pts[0])[i];
        x43[i] = CO(pts[3])[i] - CO(pts[2])[i];
        x31[i] = CO(pts[2])[i] - CO(pts[0])[i];
    }
    cross3(x21, x43, tmp);
    if (mag3(tmp) < ROUND_EPS) return 0; /* parallel edges are ignored */
    a = (dot3(x43, x43) * dot3(x21, x31) - dot3(x21, x43) * dot3(x43, x31)) /
        (dot3(x21, x21) * dot3(x43, x43) - dot3(x21, x43) * dot3(x21, x43));
    b = (dot3(x21, x43) * dot3(x21, x31) - dot3(x21, x21) * dot3(x43, x31)) /
        (dot3(x21, x21) * dot3(x43, x43) - dot3(x21, x43) * dot3(x21, x43));
    a = smax(smin(a, 1.0), 0.0);
    b = smax(smin(b, 1.0), 0.0);
    for (int i = 0; i < 3; ++i) {
        v1[i] = a * x21[i];
        v2[i] = b * x43[i];
    }
    for (int i = 0; i < 3; ++i) {
        v1[i] = CO(pts[0])[i] + v1[i];
        v2[i] = CO(pts[2])[i] + v2[i];
    }
    for (int i = 0; i < 3; ++i) nor[i] = v2[i] - v1[i];
    nor_mag = mag3(nor);
    if (nor_mag < 1000 * MACH_EPS) {
        for (int j = 0; j < 3; ++j) {
            nor[j] = (1.0 - b) * XO(pts[2])[j] + b * XO(pts[3])[j];
            nor[j] -= (1.0 - a) * XO(pts[0])[j] + a * XO(pts[1])[j];
        }
    }
    dist = dist_pos(v1, v2);
    if (dist > h) return 0;
    nor_mag = mag3(nor);
    if (nor_mag < MACH_EPS) {
        s->status = CCO_NAN; /* "Normal vector is nan", clean_up(ERROR) */
        return 0;
    }
    for (int i = 0; i < 3; ++i) nor[i] /= nor_mag;
    if (s->check) return 1;
    rec_contact(s, pts);
    edge_to_edge_impulse(s, pts, nor, a, b, dist);
    return 1;
}

/* ------------------------------------------------------------------ CCD */
/* isCoplanar, dcollid3d.cpp:371-482. roots[3] must hold dt on entry. */
static int is_coplanar(cco_solver* s, const int* pts, double dt, double* roots) {
    double v[4][3], x[4][3];
    for (int j = 0; j < 3; ++j) {
        v[0][j] = AV(pts[0])[j];
        x[0][j] = XO(pts[0])[j];
    }
    for (int i = 1; i < 4; ++i)
        for (int j = 0; j < 3; ++j) {
            v[i][j] = AV(pts[i])[j] - AV(pts[0])[j];
            x[i][j] = XO(pts[i])[j] - XO(pts[0])[j];
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
    if (fabs(a) > MACH_EPS) {
        b /= a; c /= a; d /= a;
        a = b; b = c; c = d;
        double Q = (a * a - 3 * b) / 9;
        double R = (2 * a * a * a - 9 * a * b + 27 * c) / 54;
        double Q3 = Q * Q * Q;
        double R2 = R * R;
        if (R2 < Q3) {
            double Qsqrt = sqrt(Q);
            double theta = LM_ACOS(R / sqrt(Q3));
            roots[0] = -2 * Qsqrt * LM_COS(theta / 3) - a / 3;
            roots[1] = -2 * Qsqrt * LM_COS((theta + 2 * M_PI) / 3) - a / 3;
            roots[2] = -2 * Qsqrt * LM_COS((theta - 2 * M_PI) / 3) - a / 3;
        } else {
            double sgn = (R > 0) ? 1.0 : -1.0;
            double A = -sgn * LM_POW(fabs(R) + sqrt(R2 - Q3), 1.0 / 3.0);
            double B = (fabs(A) < ROUND_EPS) ? 0.0 : Q / A;
            roots[0] = (A + B) - a / 3.0;
            if (fabs(A - B) < ROUND_EPS) roots[1] = roots[2] = -0.5 * (A + B) - a / 3.0;
        }
    } else {
        a = b; b = c; c = d;
        double delta = b * b - 4.0 * a * c;
        if (fabs(a) > ROUND_EPS && delta > 0) {
            double ds = sqrt(delta);
            roots[0] = (-b + ds) / (2.0 * a);
            roots[1] = (-b - ds) / (2.0 * a);
        } else if (fabs(a) < ROUND_EPS && fabs(b) > ROUND_EPS) {
            roots[0] = -c / b;
        }
    }
    for (int i = 0; i < 3; ++i) {
        roots[i] = roots[i] - MACH_EPS;
        if (roots[i] < 0 || roots[i] > dt) roots[i] = -1;
    }
    double t;
    if (roots[0] > roots[1]) { t = roots[0]; roots[0] = roots[1]; roots[1] = t; }
    if (roots[0] > roots[2]) { t = roots[0]; roots[0] = roots[2]; roots[2] = t; }
    if (roots[1] > roots[2]) { t = roots[1]; roots[1] = roots[2]; roots[2] = t; }
    return roots[0] > MACH_EPS || roots[1] > MACH_EPS || roots[2] > MACH_EPS;
}

/* MovingPointToTri / MovingEdgeToEdge, dcollid3d.cpp:327-369. */
static int moving_test(cco_solver* s, const int* pts, double h, int is_ee) {
    double dt = s->dt;
    double roots[4] = {-1, -1, -1, dt};
    if (!is_coplanar(s, pts, dt, roots)) return 0;
    for (int i = 0; i < 4; ++i) {
        if (roots[i] < 0) continue;
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 3; ++k) CO(pts[j])[k] = XO(pts[j])[k] + roots[i] * AV(pts[j])[k];
        if (is_ee ? edge_to_edge(s, pts, h) : point_to_tri(s, pts, h)) return 1;
    }
    return 0;
}

/* --------------------------------------------------- element-pair tests */
static void set_old(cco_solver* s, int p) {
    for (int k = 0; k < 3; ++k) CO(p)[k] = XO(p)[k];
}

/* TriToTri, dcollid3d.cpp:570-627 */
static int tri_to_tri(cco_solver* s, int ta, int tb, double h) {
    const int* A = s->ev + 3 * ta;
    const int* B = s->ev + 3 * tb;
    int pts[4], status = 0, sub = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (A[i] == B[j]) return 0;
    for (int i = 0; i < 3; ++i) { set_old(s, A[i]); set_old(s, B[i]); }
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < 3; ++i, ++sub) {
            const int* t1 = (k == 0) ? A : B;
            const int* t2 = (k == 0) ? B : A;
            for (int j = 0; j < 3; ++j) pts[j] = t2[j];
            pts[3] = t1[i];
            if (pts[3] == pts[0] || pts[3] == pts[1] || pts[3] == pts[2]) continue;
            s->cur_sub = sub;
            if (point_to_tri(s, pts, h)) status = 1;
        }
    for (int i = 0; i < 3; ++i) {
        pts[0] = A[i];
        pts[1] = A[(i + 1) % 3];
        for (int j = 0; j < 3; ++j, ++sub) {
            pts[2] = B[j];
            pts[3] = B[(j + 1) % 3];
            if (pts[0] == pts[2] || pts[0] == pts[3] || pts[1] == pts[2] || pts[1] == pts[3]) continue;
            s->cur_sub = sub;
            if (edge_to_edge(s, pts, h)) status = 1;
        }
    }
    return status;
}

/* TriToBond, dcollid3d.cpp:485-533 */
static int tri_to_bond(cco_solver* s, int t, int bd, double h) {
    const int* T = s->ev + 3 * t;
    const int* Bd = s->ev + 3 * bd;
    int pts[4], status = 0;
    for (int i = 0; i < 3; ++i)
        if (T[i] == Bd[0] || T[i] == Bd[1]) return 0;
    for (int i = 0; i < 3; ++i) { pts[i] = T[i]; set_old(s, T[i]); }
    pts[3] = Bd[0];
    set_old(s, pts[3]);
    s->cur_sub = 0;
    if (point_to_tri(s, pts, h)) status = 1;
    pts[3] = Bd[1];
    set_old(s, pts[3]);
    s->cur_sub = 1;
    if (point_to_tri(s, pts, h)) status = 1;
    pts[2] = Bd[0];
    pts[3] = Bd[1];
    for (int i = 0; i < 3; ++i) {
        pts[0] = T[i];
        pts[1] = T[(i + 1) % 3];
        s->cur_sub = 2 + i;
        if (edge_to_edge(s, pts, h)) status = 1;
    }
    return status;
}

/* BondToBond, dcollid3d.cpp:535-568 */
static int bond_to_bond(cco_solver* s, int b1, int b2, double h) {
    int pts[4] = {s->ev[3 * b1], s->ev[3 * b1 + 1], s->ev[3 * b2], s->ev[3 * b2 + 1]};
    for (int i = 0; i < 4; ++i)
        for (int j = i + 1; j < 4; ++j)
            if (pts[i] == pts[j]) return 0;
    for (int i = 0; i < 4; ++i) set_old(s, pts[i]);
    s->cur_sub = 0;
    return edge_to_edge(s, pts, h);
}

/* MovingTriToTri, dcollid3d.cpp:274-325 */
static int moving_tri_to_tri(cco_solver* s, int ta, int tb, double h) {
    const int* A = s->ev + 3 * ta;
    const int* B = s->ev + 3 * tb;
    int pts[4], status = 0, sub = 0;
    int zone = s->det_imp_zone;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (A[i] == B[j]) return 0;
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < 3; ++i, ++sub) {
            const int* t1 = (k == 0) ? A : B;
            const int* t2 = (k == 0) ? B : A;
            for (int j = 0; j < 3; ++j) pts[j] = t1[j];
            pts[3] = t2[i];
            if (pts[3] == pts[0] || pts[3] == pts[1] || pts[3] == pts[2]) continue;
            s->cur_sub = sub;
            if (moving_test(s, pts, h, 0)) status = 1;
            if (status && zone) create_imp_zone(s, pts, 4, 0);
        }
    for (int i = 0; i < 3; ++i) {
        pts[0] = A[i];
        pts[1] = A[(i + 1) % 3];
        for (int j = 0; j < 3; ++j, ++sub) {
            pts[2] = B[j];
            pts[3] = B[(j + 1) % 3];
            if (pts[0] == pts[2] || pts[0] == pts[3] || pts[1] == pts[2] || pts[1] == pts[3]) continue;
            s->cur_sub = sub;
            if (moving_test(s, pts, h, 1)) status = 1;
            if (status && zone) create_imp_zone(s, pts, 4, 0);
        }
    }
    return status;
}

/* MovingTriToBond, dcollid3d.cpp:203-244 */
static int moving_tri_to_bond(cco_solver* s, int t, int bd, double h) {
    const int* T = s->ev + 3 * t;
    const int* Bd = s->ev + 3 * bd;
    int pts[4], status = 0;
    int zone = s->det_imp_zone;
    for (int i = 0; i < 3; ++i)
        if (T[i] == Bd[0] || T[i] == Bd[1]) return 0;
    for (int i = 0; i < 3; ++i) pts[i] = T[i];
    pts[3] = Bd[0];
    s->cur_sub = 0;
    if (moving_test(s, pts, h, 0)) status = 1;
    if (status && zone) create_imp_zone(s, pts, 4, 0);
    pts[3] = Bd[1];
    s->cur_sub = 1;
    if (moving_test(s, pts, h, 0)) status = 1;
    if (status && zone) create_imp_zone(s, pts, 4, 0);
    pts[2] = Bd[0];
    pts[3] = Bd[1];
    for (int i = 0; i < 3; ++i) {
        pts[0] = T[i];
        pts[1] = T[(i + 1) % 3];
        s->cur_sub = 2 + i;
        if (moving_test(s, pts, h, 1)) status = 1;
        if (status && zone) create_imp_zone(s, pts, 4, 0);
    }
    return status;
}

/* MovingBondToBond, dcollid3d.cpp:246-272 */
static int moving_bond_to_bond(cco_solver* s, int b1, int b2, double h) {
    int pts[4] = {s->ev[3 * b1], s->ev[3 * b1 + 1], s->ev[3 * b2], s->ev[3 * b2 + 1]};
    int status = 0;
    for (int i = 0; i < 4; ++i)
        for (int j = i + 1; j < 4; ++j)
            if (pts[i] == pts[j]) return 0;
    s->cur_sub = 0;
    if (moving_test(s, pts, h, 1)) status = 1;
    if (status && s->det_imp_zone) create_imp_zone(s, pts, 4, 0);
    return status;
}

/* isProximity / isCollision dispatch, dcollid.cpp:753-836: a = found leaf,
 * b = query leaf. Tri-bond pairs always test (tri, bond). */
static int pair_test(cco_solver* s, int a, int b, int moving) {
    int ta = a < s->nt, tb = b < s->nt;
    int kind = (ta && tb) ? 0 : (!ta && !tb) ? 2 : 1;
    /* the reference hands tri-bond pairs over as (tri, bond) */
    int e1 = (kind == 1 && !ta) ? b : a, e2 = (kind == 1 && !ta) ? a : b;
    int before[6] = {0}, pp[6], n = 0, status;
    if (kind == 0 && s->esurf[a] == s->esurf[b] && elem_rigid(s, a))
        return 0; /* same rigid surface: rejected before any narrow-phase call */
    s->cur_a = e1; s->cur_b = e2; s->cur_kind = kind;
    if (s->record & 1) {
        for (int i = 0; i < s->enp[e1]; ++i) pp[n++] = s->ev[3 * e1 + i];
        for (int i = 0; i < s->enp[e2]; ++i) pp[n++] = s->ev[3 * e2 + i];
        for (int i = 0; i < n; ++i) before[i] = s->num[pp[i]];
    }
    if (kind == 0)
        status = moving ? moving_tri_to_tri(s, e1, e2, s->eps) : tri_to_tri(s, e1, e2, s->thickness);
    else if (kind == 2)
        status = moving ? moving_bond_to_bond(s, e1, e2, s->eps) : bond_to_bond(s, e1, e2, s->thickness);
    else
        status = moving ? moving_tri_to_bond(s, e1, e2, s->eps) : tri_to_bond(s, e1, e2, s->thickness);
    if (s->record & 1) {
        cco_pair_rec* pr = grow(s->pairs, &s->pairs_cap, s->npairs + 1, sizeof(*pr));
        if (!pr) { s->status = CCO_NOMEM; return status; }
        s->pairs = pr;
        cco_pair_rec* r = &pr[s->npairs++];
        r->pass = s->pass; r->kind = kind; r->a = e1; r->b = e2; r->status = status;
        for (int i = 0; i < 6; ++i) r->dcount[i] = i < n ? s->num[pp[i]] - before[i] : 0;
    }
    return status;
}

/* ------------------------------------------------------------ AABB tree */
static double box_volume(const box_t* b) {
    return (b->hi[0] - b->lo[0]) * (b->hi[1] - b->lo[1]) * (b->hi[2] - b->lo[2]);
}
static void box_merge(const box_t* a, const box_t* b, box_t* out) {
    for (int i = 0; i < 3; ++i) {
        out->lo[i] = smin(a->lo[i], b->lo[i]);
        out->hi[i] = smax(a->hi[i], b->hi[i]);
    }
}
static int box_overlap(const box_t* a, const box_t* b) {
    return (a->lo[0] <= b->hi[0] && a->hi[0] >= b->lo[0]) &&
           (a->lo[1] <= b->hi[1] && a->hi[1] >= b->lo[1]) &&
           (a->lo[2] <= b->hi[2] && a->hi[2] >= b->lo[2]);
}

/* Leaf boxes: CD_TRI/CD_BOND::{min,max}_{static,moving}_coord
 * (dcollid.cpp:852-932) padded by 1e-6 (AABB.cpp:6-36, 62-73). Static boxes
 * read x_old for triangles and Coords for bonds; both equal x_old when the
 * proximity tree is built or refit (dcollid.cpp:211-219). */
static void leaf_box(cco_solver* s, int e, int type, box_t* b) {
    int np = s->enp[e];
    const int* P = s->ev + 3 * e;
    for (int d = 0; d < 3; ++d) {
        double mx = -BIG, mn = BIG;
        if (type == TREE_STATIC) {
            for (int i = 0; i < np; ++i) {
                const double* c = (e < s->nt) ? XO(P[i]) : CO(P[i]);
                mx = smax(c[d], mx);
                mn = smin(c[d], mn);
            }
            if (e >= s->nt) { /* std::max(Coords(start), Coords(end)) */
                mx = smax(CO(P[0])[d], CO(P[1])[d]);
                mn = smin(CO(P[0])[d], CO(P[1])[d]);
            }
        } else {
            for (int i = 0; i < np; ++i) {
                mx = smax(mx, XO(P[i])[d]);
                mx = smax(mx, XO(P[i])[d] + AV(P[i])[d] * s->dt);
                mn = smin(mn, XO(P[i])[d]);
                mn = smin(mn, XO(P[i])[d] + AV(P[i])[d] * s->dt);
            }
        }
        b->lo[d] = mn - BOX_PAD;
        b->hi[d] = mx + BOX_PAD;
    }
}

static int tree_alloc(tree_t* t, int ne) {
    t->ne = ne;
    t->cap = 2 * ne + 2;
    t->box = calloc((size_t)t->cap, sizeof(box_t));
    t->left = malloc(sizeof(int) * (size_t)t->cap);
    t->right = malloc(sizeof(int) * (size_t)t->cap);
    t->queried = calloc((size_t)t->cap, 1);
    t->stack = malloc(sizeof(int) * (size_t)t->cap);
    t->stack2 = malloc(sizeof(int) * (size_t)t->cap);
    if (!t->box || !t->left || !t->right || !t->queried || !t->stack || !t->stack2) return -1;
    t->built = 0;
    t->root = -1;
    return 0;
}
static void tree_free(tree_t* t) {
    free(t->box); free(t->left); free(t->right); free(t->queried); free(t->stack); free(t->stack2);
}

/* AABBTree::insertNode, AABB.cpp:163-197: descend to the child whose box
 * grows least (ties go right), pair the new leaf with the leaf found (new
 * leaf on the left), then refresh the boxes on the way back up. */
static void tree_insert(tree_t* t, int n) {
    int* path = t->stack2;
    int depth = 0;
    int p = t->root, *slot = &t->root;
    while (t->left[p] >= 0) {
        box_t m;
        int l = t->left[p], r = t->right[p];
        box_merge(&t->box[l], &t->box[n], &m);
        double vdiff1 = box_volume(&m) - box_volume(&t->box[l]);
        box_merge(&t->box[r], &t->box[n], &m);
        double vdiff2 = box_volume(&m) - box_volume(&t->box[r]);
        path[depth++] = p;
        if (vdiff1 < vdiff2) { slot = &t->left[p]; p = l; }
        else { slot = &t->right[p]; p = r; }
    }
    int np = t->nnodes++;
    t->left[np] = n;
    t->right[np] = p;
    *slot = np;
    box_merge(&t->box[n], &t->box[p], &t->box[np]);
    while (depth > 0) {
        int q = path[--depth];
        box_merge(&t->box[t->left[q]], &t->box[t->right[q]], &t->box[q]);
    }
}

/* Build from scratch (first call: addAABB per element, AABB.cpp:129-146) or
 * rebuild from the current leaf boxes (updateTreeStructure, AABB.cpp:149-161);
 * both insert the leaves in element order. */
static void tree_build(tree_t* t) {
    t->nnodes = t->ne;
    t->root = -1;
    for (int e = 0; e < t->ne; ++e) {
        t->left[e] = t->right[e] = -1;
        if (t->root < 0) t->root = e;
        else tree_insert(t, e);
    }
    t->built = 1;
}

/* Postorder refit (updateAABBTree, AABB.cpp:212-245): new leaf boxes, then
 * every branch is the min/max of its children. */
static void tree_refit_node(tree_t* t, int node) {
    /* iterative postorder with an explicit stack of (node, state) */
    int* st = t->stack;
    int sp = 0;
    st[sp++] = node;
    /* nodes are pushed twice: first visit pushes children, second merges */
    while (sp > 0) {
        int q = st[sp - 1];
        if (q >= 0) {
            st[sp - 1] = -q - 1;
            if (t->left[q] >= 0) {
                st[sp++] = t->right[q];
                st[sp++] = t->left[q];
            }
        } else {
            sp--;
            q = -q - 1;
            if (t->left[q] >= 0) box_merge(&t->box[t->left[q]], &t->box[t->right[q]], &t->box[q]);
        }
    }
}

static int tree_leaf_rank(const tree_t* t, int* rank) {
    if (!t->built) return 0;
    int* st = t->stack;
    int sp = 0, r = 0, cur = t->root;
    while (cur >= 0 || sp > 0) {
        while (cur >= 0) { st[sp++] = cur; cur = t->left[cur]; }
        cur = st[--sp];
        if (t->left[cur] < 0) rank[cur] = r++;
        cur = t->right[cur];
    }
    return 1;
}

/* AABBTree::query + queryProximity/queryCollision, AABB.cpp:254-343: leaves
 * in inorder; for each, a pruned preorder descent reports every overlapping
 * leaf not yet queried, as (found, query). */
static int tree_query(cco_solver* s, tree_t* t, int moving) {
    int* st = t->stack;
    int* st2 = t->stack2;
    int sp = 0, cur = t->root;
    memset(t->queried, 0, (size_t)t->nnodes);
    t->count = 0;
    int is_collsn = 0;
    while (cur >= 0 || sp > 0) {
        while (cur >= 0) { st[sp++] = cur; cur = t->left[cur]; }
        cur = st[--sp];
        if (t->left[cur] < 0) {
            int n = cur;
            int sp2 = 0, c = t->root;
            while (c >= 0 || sp2 > 0) {
                while (c >= 0) {
                    if (box_overlap(&t->box[c], &t->box[n])) {
                        if (t->left[c] < 0 && c != n && !t->queried[c]) {
                            if (moving) s->ctr[2]++; else s->ctr[1]++;
                            if (pair_test(s, c, n, moving)) t->count++;
                            if (s->status) return 0;
                        }
                        st2[sp2++] = c;
                        c = t->left[c];
                    } else {
                        break;
                    }
                }
                if (sp2 == 0) break;
                c = st2[--sp2];
                c = t->right[c];
            }
            if (moving) is_collsn = t->count > 0;
            t->queried[n] = 1;
        }
        cur = t->right[cur];
    }
    return is_collsn;
}

/* aabbProximity / aabbCollision, dcollid.cpp:366-428: build on first use,
 * otherwise refit and rebuild when the root volume has grown by more than
 * 20% over the volume shared by both trees. */
static int detect_pass(cco_solver* s, int which) {
    tree_t* t = &s->tree[which];
    for (int e = 0; e < s->ne; ++e) leaf_box(s, e, which, &t->box[e]);
    if (!t->built) {
        tree_build(t);
        s->volume = box_volume(&t->box[t->root]);
        s->ctr[6]++;
    } else {
        tree_refit_node(t, t->root);
        if ((box_volume(&t->box[t->root]) - s->volume) > 0.2 * s->volume) {
            tree_build(t);
            s->volume = box_volume(&t->box[t->root]);
            s->ctr[6]++;
        }
    }
    return tree_query(s, t, which == TREE_MOVING);
}

/* --------------------------------------------------------- step stages */
static int begin_pass(cco_solver* s, int kind) {
    s->pass++;
    s->ctr[0]++;
    int* pk = grow(s->pass_kind, &s->pass_cap, s->npass + 1, sizeof(int));
    if (!pk) return CCO_NOMEM;
    s->pass_kind = pk;
    s->pass_kind[s->npass++] = kind;
    if (s->record & 4) {
        double* sn = grow(s->snaps, &s->snaps_cap, (s->nsnaps + 1) * 3 * s->nv, sizeof(double));
        if (!sn) return CCO_NOMEM;
        s->snaps = sn;
        memcpy(s->snaps + (size_t)s->nsnaps * 3 * s->nv, s->avg, sizeof(double) * 3 * (size_t)s->nv);
        s->nsnaps++;
    }
    return 0;
}

/* updateImpactListVelocity, dcollid3d.cpp:70-200: rigid motion of one zone,
 * walking the member list from its root. */
static int update_impact_list_velocity(cco_solver* s, int head) {
    double m = s->m;
    double x_cm[3] = {0.0, 0.0, 0.0}, v_cm[3] = {0.0, 0.0, 0.0};
    double L[3] = {0.0, 0.0, 0.0};
    double I[3][3] = {{0.0}}, tmp[3][3];
    int num_pts = 0;
    for (int p = head; p >= 0; p = s->uf_next[p]) {
        num_pts++;
        s->sorted[p] = 1;
        for (int i = 0; i < 3; ++i) {
            x_cm[i] += XO(p)[i];
            v_cm[i] += AV(p)[i];
        }
    }
    for (int i = 0; i < 3; ++i) {
        x_cm[i] /= num_pts;
        v_cm[i] /= num_pts;
    }
    for (int p = head; p >= 0; p = s->uf_next[p]) {
        double dx[3], dv[3], Li[3];
        for (int i = 0; i < 3; ++i) {
            dx[i] = XO(p)[i] - x_cm[i];
            dv[i] = AV(p)[i] - v_cm[i];
        }
        cross3(dx, dv, Li);
        for (int i = 0; i < 3; ++i) Li[i] = m * Li[i];
        for (int i = 0; i < 3; ++i) L[i] = Li[i] + L[i];
    }
    for (int p = head; p >= 0; p = s->uf_next[p]) {
        double dx[3], mag_dx;
        for (int i = 0; i < 3; ++i) dx[i] = XO(p)[i] - x_cm[i];
        mag_dx = mag3(dx);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                tmp[i][j] = -dx[i] * dx[j];
                if (i == j) tmp[i][j] += mag_dx * mag_dx;
                I[i][j] += tmp[i][j] * m;
            }
    }
    double w[3], mag_w;
#define DET3(a) ((a)[0][0] * ((a)[1][1] * (a)[2][2] - (a)[2][1] * (a)[1][2]) - \
                 (a)[0][1] * ((a)[1][0] * (a)[2][2] - (a)[2][0] * (a)[1][2]) + \
                 (a)[0][2] * ((a)[1][0] * (a)[2][1] - (a)[2][0] * (a)[1][1]))
    for (int i = 0; i < 3; ++i) {
        memcpy(tmp, I, sizeof(tmp));
        for (int j = 0; j < 3; ++j) tmp[j][i] = L[j];
        if (DET3(I) < ROUND_EPS)
            w[i] = 0.0;
        else
            w[i] = DET3(tmp) / DET3(I);
    }
#undef DET3
    mag_w = mag3(w);
    double dt = s->dt;
    for (int p = head; p >= 0; p = s->uf_next[p]) {
        if (is_static(s, p)) continue;
        double x_new[3], dx[3], xF[3], xR[3], wxR[3], tmpV[3];
        for (int i = 0; i < 3; ++i) dx[i] = XO(p)[i] - x_cm[i];
        if (mag_w < ROUND_EPS) {
            for (int i = 0; i < 3; ++i) { xF[i] = dx[i]; wxR[i] = 0.0; }
            for (int i = 0; i < 3; ++i) xR[i] = dx[i] - xF[i];
        } else {
            double sc = dot3(dx, w) / dot3(w, w);
            for (int i = 0; i < 3; ++i) xF[i] = sc * w[i];
            for (int i = 0; i < 3; ++i) xR[i] = dx[i] - xF[i];
            double sw = LM_SIN(dt * mag_w) / mag_w;
            for (int i = 0; i < 3; ++i) tmpV[i] = sw * w[i];
            cross3(tmpV, xR, wxR);
        }
        for (int i = 0; i < 3; ++i) {
            x_new[i] = x_cm[i] + dt * v_cm[i] + xF[i] + LM_COS(dt * mag_w) * xR[i] + wxR[i];
            AV(p)[i] = (x_new[i] - XO(p)[i]) / dt;
            if (isnan(AV(p)[i])) return CCO_NAN;
        }
    }
    return 0;
}

/* updateImpactZoneVelocityForRG, dcollid.cpp:267-288: every zone of more
 * than one point reached from a movable point moves rigidly. */
static int update_impact_zone_velocity_for_rg(cco_solver* s) {
    memset(s->sorted, 0, (size_t)s->nv);
    for (int e = 0; e < s->ne; ++e)
        for (int i = 0; i < s->enp[e]; ++i) {
            int p = s->ev[3 * e + i];
            if (s->sorted[p] || s->uf_w[find_set(s, p)] == 1) continue;
            if (!is_movable(s, p)) {
                s->sorted[p] = 1;
                continue;
            }
            int rc = update_impact_list_velocity(s, find_set(s, p));
            if (rc) return rc;
        }
    return 0;
}

/* updateAverageVelocity, dcollid.cpp:677-751 (per point once; static points
 * skipped): the pass's impulses, then the spread rigid-body impulses, then
 * the rigid motion of the movable bodies. */
static int update_average_velocity(cco_solver* s) {
    for (int p = 0; p < s->nv; ++p) {
        if (!s->in_elem[p] || is_static(s, p)) continue;
        if (s->num[p] > 0) {
            s->has_collsn[p] = 1;
            for (int k = 0; k < 3; ++k) {
                s->avg[3 * p + k] += (s->imp[3 * p + k] + s->fric[3 * p + k]) / s->num[p];
                if (!isfinite(s->avg[3 * p + k])) return CCO_NAN;
                s->imp[3 * p + k] = s->fric[3 * p + k] = 0.0;
            }
            s->num[p] = 0;
        }
        if (s->num_rg[p] > 0) {
            s->has_collsn[p] = 1;
            for (int k = 0; k < 3; ++k) s->avg[3 * p + k] += s->imp_rg[3 * p + k] / s->num_rg[p];
            s->num_rg[p] = 0;
        }
    }
    if (s->dt > 0.0) return update_impact_zone_velocity_for_rg(s);
    return 0;
}

/* updateImpactZoneVelocity, dcollid.cpp:290-310: every zone with more than
 * one point, visited from its first member in element order. */
static int update_impact_zone_velocity(cco_solver* s) {
    memset(s->sorted, 0, (size_t)s->nv);
    for (int e = 0; e < s->ne; ++e)
        for (int i = 0; i < s->enp[e]; ++i) {
            int p = s->ev[3 * e + i];
            if (s->sorted[p] || s->uf_w[find_set(s, p)] == 1) continue;
            int rc = update_impact_list_velocity(s, find_set(s, p));
            if (rc) return rc;
        }
    return 0;
}

/* detectDomainBoundaryCollision, dcollid.cpp:116-158, once per point (the
 * reference revisits shared points, which leaves the result unchanged). */
static void detect_domain_boundary(cco_solver* s) {
    double dt = s->dt, mu = s->lambda;
    for (int p = 0; p < s->nv; ++p) {
        if (!s->in_elem[p] || is_movable(s, p)) continue;
        double cand[3], dv = 0;
        for (int j = 0; j < 3; ++j) {
            cand[j] = XO(p)[j] + dt * AV(p)[j];
            if (cand[j] <= s->L[j]) {
                s->has_collsn[p] = 1;
                cand[j] = s->L[j] + s->thickness;
                dv = fabs(AV(p)[j]);
                AV(p)[j] = 0.0;
                CO(p)[j] = cand[j];
            } else if (cand[j] >= s->U[j]) {
                s->has_collsn[p] = 1;
                cand[j] = s->U[j] - s->thickness;
                dv = fabs(AV(p)[j]);
                AV(p)[j] = 0.0;
                CO(p)[j] = cand[j];
            }
        }
        double preVt = mag3(AV(p));
        if (preVt > MACH_EPS)
            for (int j = 0; j < 3; ++j) AV(p)[j] *= smax(1.0 - mu * dv / preVt, 0.0);
    }
}

/* reduceSuperelastOnce, dcollid.cpp:486-560: Gauss-Seidel over the edges of
 * every non-rigid element in element order. */
static int reduce_superelast_once(cco_solver* s) {
    double dt = s->dt;
    int has = 0;
    for (int e = 0; e < s->ne; ++e) {
        int np = s->enp[e];
        if (elem_rigid(s, e)) continue;
        for (int j = 0; j < ((np == 2) ? 1 : np); ++j) {
            int p0 = s->ev[3 * e + j % np], p1 = s->ev[3 * e + (j + 1) % np];
            double xc0[3], xc1[3];
            for (int k = 0; k < 3; ++k) {
                xc0[k] = XO(p0)[k] + dt * AV(p0)[k];
                xc1[k] = XO(p1)[k] + dt * AV(p1)[k];
            }
            double len_new = dist_pos(xc0, xc1);
            double len_old = dist_pos(XO(p0), XO(p1));
            double len0 = s->erest[3 * e + j];
            int flag;
            if (len_old > ROUND_EPS && len_new > ROUND_EPS) {
                double strain_rate = (len_new - len_old) / len_old;
                double strain = (len_new - len0) / len0;
                flag = fabs(strain) > STRAIN_TOL || fabs(strain_rate) > STRAIN_TOL;
            } else {
                flag = 1;
            }
            if (flag) {
                for (int k = 0; k < 3; ++k) {
                    double vt = (AV(p0)[k] + AV(p1)[k]);
                    vt = 0.5 * vt;
                    AV(p0)[k] = vt;
                    AV(p1)[k] = vt;
                }
                has = 1;
            }
        }
    }
    return has;
}

/* ---------------------------------------------------------------- API */
cco_solver* cco_create(int nv, int nt, const int* tris, const int* tri_surf, const double* tri_rest,
                       int nb, const int* bonds, const double* bond_rest, const unsigned char* fixed) {
    if (nv < 0 || nt < 0 || nb < 0) return NULL;
    cco_solver* s = calloc(1, sizeof(*s));
    if (!s) return NULL;
    s->nv = nv; s->nt = nt; s->nb = nb; s->ne = nt + nb;
    size_t V = (size_t)(nv > 0 ? nv : 1), E = (size_t)(s->ne > 0 ? s->ne : 1);
    s->ev = malloc(sizeof(int) * 3 * E);
    s->enp = malloc(sizeof(int) * E);
    s->esurf = malloc(sizeof(int) * E);
    s->erest = malloc(sizeof(double) * 3 * E);
    s->fixed = calloc(V, 1);
    s->in_elem = calloc(V, 1);
    s->coords = calloc(3 * V, sizeof(double));
    s->x_old = calloc(3 * V, sizeof(double));
    s->vel = calloc(3 * V, sizeof(double));
    s->avg = calloc(3 * V, sizeof(double));
    s->imp = calloc(3 * V, sizeof(double));
    s->fric = calloc(3 * V, sizeof(double));
    s->num = calloc(V, sizeof(int));
    s->has_collsn = calloc(V, 1);
    s->sorted = calloc(V, 1);
    s->uf_root = malloc(sizeof(int) * V);
    s->uf_next = malloc(sizeof(int) * V);
    s->uf_tail = malloc(sizeof(int) * V);
    s->uf_w = malloc(sizeof(int) * V);
    s->vsurf = malloc(sizeof(int) * V);
    s->imp_rg = calloc(3 * V, sizeof(double));
    s->num_rg = calloc(V, sizeof(int));
    if (!s->vsurf || !s->imp_rg || !s->num_rg) {
        cco_destroy(s);
        return NULL;
    }
    if (!s->ev || !s->enp || !s->esurf || !s->erest || !s->fixed || !s->in_elem || !s->coords ||
        !s->x_old || !s->vel || !s->avg || !s->imp || !s->fric || !s->num || !s->has_collsn ||
        !s->sorted || !s->uf_root || !s->uf_next || !s->uf_tail || !s->uf_w) {
        cco_destroy(s);
        return NULL;
    }
    for (int t = 0; t < nt; ++t) {
        for (int k = 0; k < 3; ++k) {
            int v = tris[3 * t + k];
            if (v < 0 || v >= nv) { cco_destroy(s); return NULL; }
            s->ev[3 * t + k] = v;
            s->erest[3 * t + k] = tri_rest[3 * t + k];
            s->in_elem[v] = 1;
        }
        s->enp[t] = 3;
        s->esurf[t] = tri_surf ? tri_surf[t] : 0;
    }
    for (int b = 0; b < nb; ++b) {
        int e = nt + b;
        for (int k = 0; k < 2; ++k) {
            int v = bonds[2 * b + k];
            if (v < 0 || v >= nv) { cco_destroy(s); return NULL; }
            s->ev[3 * e + k] = v;
            s->in_elem[v] = 1;
        }
        s->ev[3 * e + 2] = -1;
        s->erest[3 * e] = bond_rest[b];
        s->erest[3 * e + 1] = s->erest[3 * e + 2] = 0.0;
        s->enp[e] = 2;
        s->esurf[e] = -1;
    }
    if (fixed) for (int i = 0; i < nv; ++i) s->fixed[i] = fixed[i] & 3;
    /* surfaces: runs of equal tri_surf; a point's surface is that of the
     * first triangle holding it */
    for (int i = 0; i < nv; ++i) s->vsurf[i] = -1;
    for (int t = 0; t < nt; ++t)
        if (t == 0 || s->esurf[t] != s->esurf[t - 1]) s->nsurf++;
    size_t S = (size_t)(s->nsurf > 0 ? s->nsurf : 1);
    s->surf_id = malloc(sizeof(int) * S);
    s->surf_t0 = malloc(sizeof(int) * S);
    s->surf_t1 = malloc(sizeof(int) * S);
    s->surf_mass = calloc(S, sizeof(double));
    s->surf_com = calloc(3 * S, sizeof(double));
    s->surf_comv = calloc(3 * S, sizeof(double));
    s->mrg_com = calloc(3 * S, sizeof(double));
    s->mrg_set = calloc(S, 1);
    if (!s->surf_id || !s->surf_t0 || !s->surf_t1 || !s->surf_mass || !s->surf_com || !s->surf_comv ||
        !s->mrg_com || !s->mrg_set) {
        cco_destroy(s);
        return NULL;
    }
    for (int t = 0, k = -1; t < nt; ++t) {
        if (t == 0 || s->esurf[t] != s->esurf[t - 1]) {
            ++k;
            s->surf_id[k] = s->esurf[t];
            s->surf_t0[k] = t;
        }
        s->surf_t1[k] = t + 1;
        for (int j = 0; j < 3; ++j)
            if (s->vsurf[s->ev[3 * t + j]] < 0) s->vsurf[s->ev[3 * t + j]] = k;
    }
    if (s->ne > 0 && (tree_alloc(&s->tree[0], s->ne) || tree_alloc(&s->tree[1], s->ne))) {
        cco_destroy(s);
        return NULL;
    }
    s->zone_cap = 100000;
    s->record = 0;
    return s;
}

void cco_destroy(cco_solver* s) {
    if (!s) return;
    free(s->ev); free(s->enp); free(s->esurf); free(s->erest); free(s->fixed); free(s->in_elem);
    free(s->coords); free(s->x_old); free(s->vel); free(s->avg); free(s->imp); free(s->fric);
    free(s->num); free(s->has_collsn); free(s->sorted);
    free(s->uf_root); free(s->uf_next); free(s->uf_tail); free(s->uf_w);
    free(s->vsurf); free(s->imp_rg); free(s->num_rg);
    free(s->surf_id); free(s->surf_t0); free(s->surf_t1); free(s->surf_mass); free(s->surf_com);
    free(s->surf_comv); free(s->mrg_com); free(s->mrg_set);
    if (s->ne > 0) { tree_free(&s->tree[0]); tree_free(&s->tree[1]); }
    free(s->pass_kind); free(s->pairs); free(s->contacts); free(s->snaps);
    free(s);
}

void cco_set_recording(cco_solver* s, int flags) { s->record = flags; }

static int surf_of_id(const cco_solver* s, int id) {
    for (int k = 0; k < s->nsurf; ++k)
        if (s->surf_id[k] == id) return k;
    return -1;
}

/* The HYPER_SURF data of a surface: total_mass, center_of_mass,
 * center_of_mass_velo. The first call also seeds the solver's remembered
 * centre of mass (mrg_com), which the reference would otherwise read before
 * writing when a body's first point collides in the first step. */
int cco_set_body(cco_solver* s, int surf, double mass, const double* com, const double* comv) {
    int k = surf_of_id(s, surf);
    if (k < 0) return CCO_BAD_INPUT;
    s->surf_mass[k] = mass;
    for (int i = 0; i < 3; ++i) {
        s->surf_com[3 * k + i] = com[i];
        s->surf_comv[3 * k + i] = comv[i];
    }
    if (!s->mrg_set[k]) {
        for (int i = 0; i < 3; ++i) s->mrg_com[3 * k + i] = com[i];
        s->mrg_set[k] = 1;
    }
    return 0;
}

int cco_get_body(const cco_solver* s, int surf, double* com, double* comv) {
    int k = surf_of_id(s, surf);
    if (k < 0) return CCO_BAD_INPUT;
    for (int i = 0; i < 3; ++i) {
        com[i] = s->surf_com[3 * k + i];
        comv[i] = s->surf_comv[3 * k + i];
    }
    return 0;
}

/* updateFinalForRG, dcollid.cpp:626-675: per movable body, the first point
 * (in element order) with has_collsn gives the body's velocity and moves its
 * centre of mass from the remembered one. */
static void update_final_for_rg(cco_solver* s) {
    unsigned char* done = calloc((size_t)(s->nsurf > 0 ? s->nsurf : 1), 2);
    if (!done) { s->status = CCO_NOMEM; return; }
    unsigned char* visited = done + (s->nsurf > 0 ? s->nsurf : 1);  /* 0 absent, 1 false, 2 true */
    for (int e = 0; e < s->ne; ++e)
        for (int i = 0; i < s->enp[e]; ++i) {
            int p = s->ev[3 * e + i];
            if (!is_movable(s, p)) continue;
            int k = s->vsurf[p];
            if (k < 0) continue;
            if (s->has_collsn[p] && !done[k]) {
                done[k] = 1;
                for (int j = 0; j < 3; ++j) {
                    s->surf_comv[3 * k + j] = AV(p)[j];
                    s->surf_com[3 * k + j] = AV(p)[j] * s->dt + s->mrg_com[3 * k + j];
                }
                visited[k] = 1;
            }
            if (visited[k] != 2) {
                for (int j = 0; j < 3; ++j) s->mrg_com[3 * k + j] = s->surf_com[3 * k + j];
                s->mrg_set[k] = 1;
                visited[k] = 2;
            }
        }
    free(done);
}
void cco_set_zone_cap(cco_solver* s, int cap) { s->zone_cap = cap; }

/* resolveCollision, dcollid.cpp:317-362, preceded by the host loop's state
 * reset (test.cpp:214-221) and assembleFromInterface (dcollid3d.cpp:12-52). */
int cco_step(cco_solver* s, const double* x_old, const double* x_cand, double* vel,
             unsigned char* has_collsn, const double* params, const double* domain,
             double* x_out, double* avgvel_out, int* has_collision, int* zone_root) {
    int nv = s->nv;
    s->dt = params[0]; s->thickness = params[1]; s->eps = params[2]; s->k = params[3];
    s->m = params[4]; s->lambda = params[5]; s->cr = params[6];
    for (int k = 0; k < 3; ++k) { s->L[k] = domain[k]; s->U[k] = domain[3 + k]; }
    s->pass = -1;
    s->npass = s->npairs = s->ncontacts = s->nsnaps = 0;
    s->status = 0;
    memset(s->ctr, 0, sizeof(s->ctr));
    for (int p = 0; p < nv; ++p) {
        for (int k = 0; k < 3; ++k) {
            s->x_old[3 * p + k] = x_old[3 * p + k];
            s->coords[3 * p + k] = x_cand[3 * p + k];
            s->vel[3 * p + k] = vel[3 * p + k];
            s->imp[3 * p + k] = 0.0;
        }
        s->num[p] = 0;
        s->has_collsn[p] = has_collsn[p] ? 1 : 0;
        /* makeSet */
        s->uf_root[p] = p; s->uf_next[p] = -1; s->uf_tail[p] = p; s->uf_w[p] = 1;
        s->sorted[p] = 0;
    }
    /* createImpZoneForRG, dcollid3d.cpp:54-68 */
    for (int k = 0; k < s->nsurf; ++k) {
        if (!is_movable(s, s->ev[3 * s->surf_t0[k]])) continue;
        for (int t = s->surf_t0[k]; t < s->surf_t1[k]; ++t) create_imp_zone(s, s->ev + 3 * t, 3, 1);
    }
    int rc = 0, hc = 0;
    if (s->ne == 0) goto out; /* the reference dereferences an empty tree here */

    /* computeAverageVelocity, dcollid.cpp:160-220 */
    for (int p = 0; p < nv; ++p) {
        if (!s->in_elem[p]) continue;
        for (int j = 0; j < 3; ++j) {
            if (s->dt > ROUND_EPS)
                s->avg[3 * p + j] = (CO(p)[j] - XO(p)[j]) / s->dt;
            else
                s->avg[3 * p + j] = 0.0;
            if (!isfinite(s->avg[3 * p + j])) { rc = CCO_NAN; goto out; }
        }
    }
    for (int p = 0; p < nv; ++p)
        if (s->in_elem[p])
            for (int j = 0; j < 3; ++j) CO(p)[j] = XO(p)[j];

    /* detectProximity, dcollid.cpp:390-406 */
    if ((rc = begin_pass(s, PASS_PROX))) goto out;
    detect_pass(s, TREE_STATIC);
    if ((rc = s->status)) goto out;
    if ((rc = update_average_velocity(s))) goto out;

    /* detectCollision, dcollid.cpp:430-468 */
    {
        int is_collision = 1, niter = 1, cd_count = 0;
        while (is_collision) {
            if ((rc = begin_pass(s, PASS_CCD))) goto out;
            is_collision = detect_pass(s, TREE_MOVING);
            if ((rc = s->status)) goto out;
            if (cd_count++ == 0 && is_collision) hc = 1;
            if ((rc = update_average_velocity(s))) goto out;
            if (++niter > MAX_CCD_ITER) break;
        }
        /* computeImpactZone, dcollid.cpp:227-265 */
        if (is_collision) {
            s->det_imp_zone = 1;
            int iter = 0;
            while (is_collision) {
                if (iter++ >= s->zone_cap) { rc = CCO_ITER_CAP; s->det_imp_zone = 0; goto out; }
                s->ctr[4]++;
                if ((rc = begin_pass(s, PASS_ZONE))) goto out;
                is_collision = detect_pass(s, TREE_MOVING);
                if ((rc = s->status)) goto out;
                if ((rc = update_average_velocity(s))) goto out;
                if ((rc = update_impact_zone_velocity(s))) goto out;
            }
            s->det_imp_zone = 0;
        }
    }

    detect_domain_boundary(s);

    /* updateFinalPosition, dcollid.cpp:562-584 */
    for (int p = 0; p < nv; ++p)
        if (s->in_elem[p])
            for (int j = 0; j < 3; ++j) CO(p)[j] = XO(p)[j] + AV(p)[j] * s->dt;

    /* reduceSuperelast, dcollid.cpp:586-596 */
    {
        int has = 1, niter = 0;
        while (has && niter++ < STRAIN_MAX_ITER) {
            has = reduce_superelast_once(s);
            s->ctr[5]++;
        }
    }

    /* updateFinalVelocity, dcollid.cpp:598-624 */
    for (int p = 0; p < nv; ++p)
        if (s->in_elem[p] && s->has_collsn[p])
            for (int j = 0; j < 3; ++j) s->vel[3 * p + j] = AV(p)[j];
    update_final_for_rg(s);
    if ((rc = s->status)) goto out;

out:
    s->det_imp_zone = 0;
    for (int p = 0; p < nv; ++p) {
        for (int k = 0; k < 3; ++k) {
            x_out[3 * p + k] = s->coords[3 * p + k];
            vel[3 * p + k] = s->vel[3 * p + k];
            if (avgvel_out) avgvel_out[3 * p + k] = s->avg[3 * p + k];
        }
        has_collsn[p] = s->has_collsn[p];
        if (zone_root) zone_root[p] = find_set(s, p);
    }
    if (has_collision) *has_collision = hc;
    return rc;
}

/* The exact CCD re-check of a finished step (the metric's zero-interpenetration
 * test, not part of the reference): every element pair whose swept boxes over
 * [x_old, x_new] overlap goes through the reference's CCD predicate
 * (isCollision's Moving* tests with h = eps, dcollid.cpp:753-836,
 * dcollid3d.cpp:203-482) with avgVel = (x_new - x_old)/dt, without impulses
 * or impact zones; pairs of one rigid surface are skipped as the reference
 * skips them. Candidate pairs come from a sort and sweep of the boxes on x.
 * Returns the number of pairs that still collide, or a negative status. The
 * solver's step state is left as it was, except its current positions. */
static const box_t* g_sweep_boxes;
static int sweep_cmp(const void* a, const void* b) {
    const double la = g_sweep_boxes[*(const int*)a].lo[0], lb = g_sweep_boxes[*(const int*)b].lo[0];
    if (la < lb) return -1;
    if (la > lb) return 1;
    return *(const int*)a - *(const int*)b;
}

long long cco_check_ccd(cco_solver* s, const double* x_old, const double* x_new, const double* params) {
    const int nv = s->nv, ne = s->ne;
    const double dt = params[0];
    double* keep = malloc(sizeof(double) * 6 * (size_t)(nv > 0 ? nv : 1));
    box_t* box = malloc(sizeof(box_t) * (size_t)(ne > 0 ? ne : 1));
    int* order = malloc(sizeof(int) * (size_t)(ne > 0 ? ne : 1));
    if (!keep || !box || !order) {
        free(keep); free(box); free(order);
        return CCO_NOMEM;
    }
    memcpy(keep, s->x_old, sizeof(double) * 3 * (size_t)nv);
    memcpy(keep + 3 * (size_t)nv, s->avg, sizeof(double) * 3 * (size_t)nv);
    const double sdt = s->dt, seps = s->eps;
    const int zone = s->det_imp_zone, rec = s->record, st0 = s->status;
    s->dt = dt;
    s->eps = params[2];
    s->det_imp_zone = 0;
    s->record = 0;
    s->check = 1;
    s->status = 0;
    for (int p = 0; p < nv; ++p)
        for (int j = 0; j < 3; ++j) {
            s->x_old[3 * p + j] = x_old[3 * p + j];
            s->avg[3 * p + j] = (x_new[3 * p + j] - x_old[3 * p + j]) / dt;
            s->coords[3 * p + j] = x_old[3 * p + j];
        }
    for (int e = 0; e < ne; ++e) {
        leaf_box(s, e, TREE_MOVING, &box[e]);
        order[e] = e;
    }
    g_sweep_boxes = box;
    qsort(order, (size_t)ne, sizeof(int), sweep_cmp);
    long long hits = 0;
    for (int i = 0; i < ne && s->status == 0; ++i) {
        const box_t* a = &box[order[i]];
        for (int j = i + 1; j < ne && box[order[j]].lo[0] <= a->hi[0]; ++j) {
            if (!box_overlap(a, &box[order[j]])) continue;
            int ea = order[i], eb = order[j];
            if (ea < eb) {
                int t = ea;
                ea = eb;
                eb = t;
            }
            hits += pair_test(s, ea, eb, 1);
        }
    }
    const int bad = s->status;
    memcpy(s->x_old, keep, sizeof(double) * 3 * (size_t)nv);
    memcpy(s->avg, keep + 3 * (size_t)nv, sizeof(double) * 3 * (size_t)nv);
    s->dt = sdt;
    s->eps = seps;
    s->det_imp_zone = zone;
    s->record = rec;
    s->check = 0;
    s->status = st0;
    free(keep); free(box); free(order);
    return bad ? bad : hits;
}

int cco_num_passes(const cco_solver* s) { return s->npass; }
void cco_pass_kinds(const cco_solver* s, int* out) { memcpy(out, s->pass_kind, sizeof(int) * (size_t)s->npass); }
int cco_num_pairs(const cco_solver* s) { return s->npairs; }
const cco_pair_rec* cco_pairs(const cco_solver* s) { return s->pairs; }
int cco_num_contacts(const cco_solver* s) { return s->ncontacts; }
const cco_contact_rec* cco_contacts(const cco_solver* s) { return s->contacts; }
int cco_num_vel_snaps(const cco_solver* s) { return s->nsnaps; }
const double* cco_vel_snaps(const cco_solver* s) { return s->snaps; }
int cco_leaf_rank(const cco_solver* s, int which, int* rank_out) {
    if (s->ne == 0) return 0;
    return tree_leaf_rank(&s->tree[which], rank_out);
}
void cco_counters(const cco_solver* s, long long* out7) { memcpy(out7, s->ctr, sizeof(s->ctr)); }
