/*
 * Harness that runs the reference's own CollisionSolver3d (antdvid/Collision
 * AABB.cpp, dcollid.cpp, dcollid3d.cpp, compiled unmodified from the reference
 * tree by oracle/Makefile.ref) on flat mesh arrays.
 *
 * TEST INFRASTRUCTURE ONLY. It exists to pin the C restatement in
 * oracle/cc_oracle.c and to generate the golden fixtures under tests/golden/.
 * It is never linked into the product library and never runs on the GPU machine.
 *
 * What it reproduces from the reference's host loop (test.cpp:96-130,
 * 192-224): per step x_old := current positions, Coords := candidate
 * positions, collsnImpulse := 0, collsn_num := 0 (test.cpp:218-221), then
 * assembleFromInterface (dcollid3d.cpp:12), the static setters
 * (collid.h:180-193) and resolveCollision (dcollid.cpp:317). The per-point
 * STATE persists between steps, as FronTier's state copy does
 * (test.cpp:209).
 *
 * What it records:
 *   - pass boundaries, from the clock hooks the reference calls around each
 *     detection pass (dcollid.cpp:329, 452, 242);
 *   - every narrow-phase call in visiting order with its orientation (a = the
 *     found leaf, b = the query leaf; AABB.cpp:293-296, 323-326), its status,
 *     and the collsn_num increments it caused on the pair's points;
 *   - avgVel of every point at the start of each CCD / zone pass;
 *   - the impact-zone root of every point after the step.
 */
#include <FronTier.h>
#include <functional>
#include <map>
#include <fstream>
#include <stdexcept>
#include <string>
#include <unistd.h>
#include <fcntl.h>

/* Open the solver's private virtuals to the recording subclass below. The
 * standard headers are already included, so only collid.h is affected. */
#define private public
#define protected public
#include "collid.h"
#undef private
#undef protected

namespace {

struct PairRec {
    int pass;
    int kind;     /* 0 tri-tri, 1 tri-bond, 2 bond-bond */
    int a, b;     /* element indices, as passed to isProximity/isCollision */
    int status;
    int dcount[6];/* collsn_num increments: a's points then b's points */
};

struct RefWorld;
RefWorld* g_active = nullptr;

struct RecSolver;

struct RefWorld {
    int nv = 0, nt = 0, nb = 0;
    std::vector<POINT> pts;
    std::vector<STATE> st;
    std::vector<TRI> tris;
    std::vector<BOND> bonds;
    std::vector<SURFACE> surfs;
    std::vector<TRI> sentinels;
    std::vector<CURVE> curves;
    std::vector<SURFACE*> surf_ptrs;
    std::vector<CURVE*> curve_ptrs;
    HYPER_SURF hs_dummy;
    INTFC_TABLE table;
    INTERFACE intfc;
    RecSolver* solver = nullptr;

    /* recording */
    bool record = true;
    bool snap_vel = false;
    int pass = -1;
    std::vector<int> pass_kind;   /* 0 prox, 1 ccd, 2 zone */
    std::vector<PairRec> pairs;
    std::vector<double> pass_vel; /* per recorded pass, nv*3 */

    int tri_index(const TRI* t) const { return (int)(t - tris.data()); }
    int bond_index(const BOND* b) const { return (int)(b - bonds.data()); }
    int vidx(const POINT* p) const { return (int)(p - pts.data()); }
};

struct RecSolver : public CollisionSolver3d {
    RefWorld* w;
    explicit RecSolver(RefWorld* world) : w(world) {}

    template <class F>
    bool rec(int kind, int a, int b, POINT* const* pa, int na, POINT* const* pb, int nbp, F&& call) {
        if (!w->record) return call();
        int before[6] = {0}, n = 0;
        POINT* ps[6];
        for (int i = 0; i < na; ++i) ps[n++] = pa[i];
        for (int i = 0; i < nbp; ++i) ps[n++] = pb[i];
        for (int i = 0; i < n; ++i) before[i] = ((STATE*)left_state(ps[i]))->collsn_num;
        bool s = call();
        PairRec r;
        r.pass = w->pass; r.kind = kind; r.a = a; r.b = b; r.status = s ? 1 : 0;
        for (int i = 0; i < 6; ++i) r.dcount[i] = 0;
        for (int i = 0; i < n; ++i) r.dcount[i] = ((STATE*)left_state(ps[i]))->collsn_num - before[i];
        w->pairs.push_back(r);
        return s;
    }
    /* Element ids: tris are 0..nt-1, bonds nt..nt+nb-1. For the tri-bond
     * calls the reference always passes (tri, bond) whatever the pair order,
     * so the recorded a/b follow the AABB visit (see isProximity,
     * dcollid.cpp:809-829); the caller of rec() gets them from the current
     * visit held in cur_a / cur_b. */
    int cur_a = -1, cur_b = -1;

    bool TriToTri(const TRI* t1, const TRI* t2, double h) override {
        return rec(0, w->tri_index(t1), w->tri_index(t2), t1->__pts, 3, t2->__pts, 3,
                   [&] { return CollisionSolver3d::TriToTri(t1, t2, h); });
    }
    bool MovingTriToTri(const TRI* t1, const TRI* t2, double h) override {
        return rec(0, w->tri_index(t1), w->tri_index(t2), t1->__pts, 3, t2->__pts, 3,
                   [&] { return CollisionSolver3d::MovingTriToTri(t1, t2, h); });
    }
    bool TriToBond(const TRI* t, const BOND* b, double h) override {
        POINT* bp[2] = {b->start, b->end};
        return rec(1, w->tri_index(t), w->nt + w->bond_index(b), t->__pts, 3, bp, 2,
                   [&] { return CollisionSolver3d::TriToBond(t, b, h); });
    }
    bool MovingTriToBond(const TRI* t, const BOND* b, double h) override {
        POINT* bp[2] = {b->start, b->end};
        return rec(1, w->tri_index(t), w->nt + w->bond_index(b), t->__pts, 3, bp, 2,
                   [&] { return CollisionSolver3d::MovingTriToBond(t, b, h); });
    }
    bool BondToBond(const BOND* b1, const BOND* b2, double h) override {
        POINT* p1[2] = {b1->start, b1->end};
        POINT* p2[2] = {b2->start, b2->end};
        return rec(2, w->nt + w->bond_index(b1), w->nt + w->bond_index(b2), p1, 2, p2, 2,
                   [&] { return CollisionSolver3d::BondToBond(b1, b2, h); });
    }
    bool MovingBondToBond(const BOND* b1, const BOND* b2, double h) override {
        POINT* p1[2] = {b1->start, b1->end};
        POINT* p2[2] = {b2->start, b2->end};
        return rec(2, w->nt + w->bond_index(b1), w->nt + w->bond_index(b2), p1, 2, p2, 2,
                   [&] { return CollisionSolver3d::MovingBondToBond(b1, b2, h); });
    }
};

struct CleanUp : std::runtime_error {
    explicit CleanUp(int c) : std::runtime_error("clean_up"), code(c) {}
    int code;
};

void begin_pass(int kind) {
    RefWorld* w = g_active;
    if (!w) return;
    w->pass += 1;
    w->pass_kind.push_back(kind);
    if (w->snap_vel) {
        for (int i = 0; i < w->nv; ++i)
            for (int k = 0; k < 3; ++k) w->pass_vel.push_back(w->st[i].avgVel[k]);
    }
}

}  // namespace

/* FronTier hooks named by the stub header. */
bool debugging(const char*) { return false; }
void clean_up(int code) { throw CleanUp(code); }
void start_clock(const char* name) {
    std::string s(name);
    if (s == "detectProximity") begin_pass(0);
    else if (s == "cgal_collision") begin_pass(1);
    else if (s == "cgal_impactzone") begin_pass(2);
}
void stop_clock(const char*) {}
double cpu_seconds() { return 0.0; }
bool create_directory(const char*, bool) { return false; }

extern "C" {

/*
 * tris: nt*3 vertex indices; tri_surf: surface id per tri (contiguous runs);
 * tri_rest: nt*3 rest lengths of edges (p0,p1),(p1,p2),(p2,p0);
 * bonds: nb*2; bond_curve: curve id per bond (contiguous runs);
 * bond_rest: nb; fixed: nv flags (is_fixed).
 */
void* ref_create(int nv, int nt, const int* tris, const int* tri_surf, const double* tri_rest,
                 int nb, const int* bonds, const int* bond_curve, const double* bond_rest,
                 const unsigned char* fixed) {
    RefWorld* w = new RefWorld;
    w->nv = nv; w->nt = nt; w->nb = nb;
    w->pts.assign(nv, POINT());
    w->st.assign(nv, STATE());
    std::memset(w->pts.data(), 0, sizeof(POINT) * (size_t)nv);
    std::memset(w->st.data(), 0, sizeof(STATE) * (size_t)nv);
    std::memset(&w->hs_dummy, 0, sizeof(w->hs_dummy));
    for (int i = 0; i < nv; ++i) {
        w->pts[i]._left_state = &w->st[i];
        w->pts[i]._right_state = &w->st[i];
        w->pts[i].global_index = i;
        w->pts[i].hs = &w->hs_dummy;
        w->st[i].is_fixed = fixed ? (fixed[i] & 1) != 0 : false;
        w->st[i].is_movableRG = fixed ? (fixed[i] & 2) != 0 : false;
    }
    w->tris.assign(nt, TRI());
    int nsurf = 0;
    for (int t = 0; t < nt; ++t)
        if (t == 0 || tri_surf[t] != tri_surf[t - 1]) ++nsurf;
    w->surfs.assign(nsurf, SURFACE());
    w->sentinels.assign(nsurf, TRI());
    int s = -1;
    for (int t = 0; t < nt; ++t) {
        TRI& tr = w->tris[t];
        for (int k = 0; k < 3; ++k) {
            tr.__pts[k] = &w->pts[tris[3 * t + k]];
            tr.side_length0[k] = tri_rest[3 * t + k];
        }
        if (t == 0 || tri_surf[t] != tri_surf[t - 1]) {
            ++s;
            w->surfs[s].first = &tr;
            w->surfs[s].bdry = 0;
            w->surfs[s].hs.body_index = tri_surf[t];
        }
        tr.surf = &w->surfs[s];
        /* a point belongs to (pt->hs) the surface of its first triangle */
        for (int k = 0; k < 3; ++k)
            if (tr.__pts[k]->hs == &w->hs_dummy) tr.__pts[k]->hs = &w->surfs[s].hs;
        bool last = (t == nt - 1) || tri_surf[t + 1] != tri_surf[t];
        tr.next = last ? &w->sentinels[s] : &w->tris[t + 1];
        if (last) w->surfs[s].tail_sentinel = &w->sentinels[s];
    }
    for (int i = 0; i < nsurf; ++i) w->surf_ptrs.push_back(&w->surfs[i]);
    w->surf_ptrs.push_back(nullptr);

    w->bonds.assign(nb, BOND());
    int ncur = 0;
    for (int b = 0; b < nb; ++b)
        if (b == 0 || bond_curve[b] != bond_curve[b - 1]) ++ncur;
    w->curves.assign(ncur, CURVE());
    int c = -1;
    for (int b = 0; b < nb; ++b) {
        BOND& bd = w->bonds[b];
        bd.start = &w->pts[bonds[2 * b]];
        bd.end = &w->pts[bonds[2 * b + 1]];
        bd.length0 = bond_rest[b];
        if (b == 0 || bond_curve[b] != bond_curve[b - 1]) {
            ++c;
            w->curves[c].first = &bd;
            w->curves[c].hsb_type = STRING_HSBDRY;
        }
        bool last = (b == nb - 1) || bond_curve[b + 1] != bond_curve[b];
        bd.next = last ? nullptr : &w->bonds[b + 1];
        if (last) w->curves[c].last = &bd;
    }
    for (int i = 0; i < ncur; ++i) w->curve_ptrs.push_back(&w->curves[i]);
    w->curve_ptrs.push_back(nullptr);

    w->intfc.surfaces = w->surf_ptrs.data();
    w->intfc.curves = w->curve_ptrs.data();
    w->intfc.table = &w->table;
    w->solver = new RecSolver(w);
    return w;
}

void ref_destroy(void* h) {
    RefWorld* w = (RefWorld*)h;
    delete w->solver;
    delete w;
}

/* HYPER_SURF data of the surface whose tri_surf id is `surf`. The first call
 * also seeds CollisionSolver::mrg_com (collid.h:174), which updateFinalForRG
 * would otherwise read before writing (dcollid.cpp:650) when a body's first
 * point collides in the first step. */
int ref_set_body(void* h, int surf, double mass, const double* com, const double* comv) {
    RefWorld* w = (RefWorld*)h;
    for (auto& sf : w->surfs)
        if (sf.hs.body_index == surf) {
            sf.hs.mass = mass;
            for (int k = 0; k < 3; ++k) {
                sf.hs.com[k] = com[k];
                sf.hs.comv[k] = comv[k];
            }
            if (!w->solver->mrg_com.count(surf)) w->solver->mrg_com[surf] = std::vector<double>(com, com + 3);
            return 0;
        }
    return -4;
}

int ref_get_body(void* h, int surf, double* com, double* comv) {
    RefWorld* w = (RefWorld*)h;
    for (auto& sf : w->surfs)
        if (sf.hs.body_index == surf) {
            for (int k = 0; k < 3; ++k) {
                com[k] = sf.hs.com[k];
                comv[k] = sf.hs.comv[k];
            }
            return 0;
        }
    return -4;
}

void ref_set_recording(void* h, int record, int snap_vel) {
    RefWorld* w = (RefWorld*)h;
    w->record = record != 0;
    w->snap_vel = snap_vel != 0;
}

/*
 * One host step. params = {dt, thickness, eps, k, m, lambda, cr};
 * domain = {L0,L1,L2,U0,U1,U2}. x_old/x_cand/vel are nv*3 (point-major).
 * has_collsn is read on entry and written on exit.
 * Returns 0, or the clean_up() code (the reference's fatal-error exit).
 */
int ref_step(void* h, const double* x_old, const double* x_cand, double* vel,
             unsigned char* has_collsn, const double* params, const double* domain,
             int quiet, double* x_out, double* avgvel_out, int* has_collision,
             int* zone_root) {
    RefWorld* w = (RefWorld*)h;
    for (int i = 0; i < w->nv; ++i) {
        STATE* sl = &w->st[i];
        for (int k = 0; k < 3; ++k) {
            sl->x_old[k] = x_old[3 * i + k];
            w->pts[i]._coords[k] = x_cand[3 * i + k];
            sl->vel[k] = vel[3 * i + k];
            w->pts[i].vel[k] = vel[3 * i + k];
            sl->collsnImpulse[k] = 0.0;
        }
        sl->collsn_num = 0;
        sl->has_collsn = has_collsn[i] != 0;
    }
    for (int k = 0; k < 3; ++k) {
        w->table.rect_grid.L[k] = domain[k];
        w->table.rect_grid.U[k] = domain[3 + k];
    }
    w->pass = -1;
    w->pass_kind.clear();
    w->pairs.clear();
    w->pass_vel.clear();

    int saved = -1;
    if (quiet) {
        fflush(stdout);
        std::cout.flush();
        saved = dup(1);
        int dn = open("/dev/null", O_WRONLY);
        dup2(dn, 1);
        close(dn);
    }
    int rc = 0;
    g_active = w;
    try {
        w->solver->assembleFromInterface(&w->intfc, params[0]);
        CollisionSolver::setFabricThickness(params[1]);
        CollisionSolver::setRoundingTolerance(params[2]);
        CollisionSolver::setSpringConstant(params[3]);
        CollisionSolver::setPointMass(params[4]);
        CollisionSolver::setFrictionConstant(params[5]);
        CollisionSolver::setRestitutionCoef(params[6]);
        w->solver->resolveCollision();
    } catch (const CleanUp& e) {
        rc = e.code == 0 ? -1 : e.code;
    }
    fedisableexcept(FE_ALL_EXCEPT);
    feclearexcept(FE_ALL_EXCEPT);
    g_active = nullptr;
    if (quiet) {
        fflush(stdout);
        std::cout.flush();
        dup2(saved, 1);
        close(saved);
    }
    for (int i = 0; i < w->nv; ++i) {
        STATE* sl = &w->st[i];
        for (int k = 0; k < 3; ++k) {
            x_out[3 * i + k] = w->pts[i]._coords[k];
            vel[3 * i + k] = w->pts[i].vel[k];
            if (avgvel_out) avgvel_out[3 * i + k] = sl->avgVel[k];
        }
        has_collsn[i] = sl->has_collsn ? 1 : 0;
        if (zone_root) {
            POINT* p = &w->pts[i];
            int guard = 0;
            while (((STATE*)left_state(p))->impZone.root != p && guard++ < w->nv)
                p = ((STATE*)left_state(p))->impZone.root;
            zone_root[i] = w->vidx(p);
        }
    }
    if (has_collision) *has_collision = w->solver->hasCollision() ? 1 : 0;
    return rc;
}

int ref_num_passes(void* h) { return (int)((RefWorld*)h)->pass_kind.size(); }
void ref_pass_kinds(void* h, int* out) {
    RefWorld* w = (RefWorld*)h;
    for (size_t i = 0; i < w->pass_kind.size(); ++i) out[i] = w->pass_kind[i];
}
int ref_num_pairs(void* h) { return (int)((RefWorld*)h)->pairs.size(); }
/* out: npairs * 11 ints (pass, kind, a, b, status, dcount[6]) */
void ref_pairs(void* h, int* out) {
    RefWorld* w = (RefWorld*)h;
    for (size_t i = 0; i < w->pairs.size(); ++i) {
        const PairRec& r = w->pairs[i];
        int* o = out + 11 * i;
        o[0] = r.pass; o[1] = r.kind; o[2] = r.a; o[3] = r.b; o[4] = r.status;
        for (int k = 0; k < 6; ++k) o[5 + k] = r.dcount[k];
    }
}
int ref_num_vel_snaps(void* h) {
    RefWorld* w = (RefWorld*)h;
    return w->nv ? (int)(w->pass_vel.size() / (3 * (size_t)w->nv)) : 0;
}
void ref_vel_snaps(void* h, double* out) {
    RefWorld* w = (RefWorld*)h;
    std::memcpy(out, w->pass_vel.data(), sizeof(double) * w->pass_vel.size());
}

}  // extern "C"
