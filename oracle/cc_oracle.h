/*
 * CPU restatement of antdvid/Collision's CollisionSolver3d::resolveCollision()
 * (dcollid.cpp:317-362) in plain C.
 *
 * TEST INFRASTRUCTURE: this is the oracle the GPU library is checked against
 * (tests/, __graft_entry__.smoke()) and the CPU baseline bench.py times. The
 * shipped library never links or calls it.
 */
#ifndef CC_ORACLE_H
#define CC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cco_solver cco_solver;

/* One recorded narrow-phase call, in the format of oracle/ref_harness.cpp. */
typedef struct {
    int pass, kind, a, b, status;
    int dcount[6];
} cco_pair_rec;

/* One sub-test that applied an impulse (a contact). */
typedef struct {
    int pass, kind, a, b, subtest;
    int v[4];
} cco_contact_rec;

enum { CCO_OK = 0, CCO_NAN = -2, CCO_ITER_CAP = -3, CCO_BAD_INPUT = -4, CCO_NOMEM = -5 };

/* fixed: per point, bit 0 is_fixed (static rigid), bit 1 is_movableRG. */
cco_solver* cco_create(int nv, int nt, const int* tris, const int* tri_surf,
                       const double* tri_rest, int nb, const int* bonds,
                       const double* bond_rest, const unsigned char* fixed);
/* Body data of the surface with tri_surf id `surf` (total_mass,
 * center_of_mass, center_of_mass_velo); read back after a step. */
int cco_set_body(cco_solver* s, int surf, double mass, const double* com, const double* comv);
int cco_get_body(const cco_solver* s, int surf, double* com, double* comv);
void cco_destroy(cco_solver* s);
/* record: bit0 pairs, bit1 contacts, bit2 pass-entry avgVel snapshots */
void cco_set_recording(cco_solver* s, int flags);
/* Cap on the impact-zone loop, unbounded in the reference (dcollid.cpp:236). */
void cco_set_zone_cap(cco_solver* s, int cap);

/* params = {dt, thickness, eps, k, m, lambda, cr}; domain = {L[3], U[3]}.
 * vel and has_collsn are in/out. zone_root may be NULL. */
int cco_step(cco_solver* s, const double* x_old, const double* x_cand, double* vel,
             unsigned char* has_collsn, const double* params, const double* domain,
             double* x_out, double* avgvel_out, int* has_collision, int* zone_root);

int cco_num_passes(const cco_solver* s);
void cco_pass_kinds(const cco_solver* s, int* out);
int cco_num_pairs(const cco_solver* s);
const cco_pair_rec* cco_pairs(const cco_solver* s);
int cco_num_contacts(const cco_solver* s);
const cco_contact_rec* cco_contacts(const cco_solver* s);
int cco_num_vel_snaps(const cco_solver* s);
const double* cco_vel_snaps(const cco_solver* s);
/* Leaf order (inorder rank per element) of the proximity (which=0) or
 * collision (which=1) tree as it stands; returns 0 if that tree is unbuilt. */
int cco_leaf_rank(const cco_solver* s, int which, int* rank_out);
/* Counters of the last step: passes, proximity pairs, ccd pairs, contacts,
 * zone iterations, strain passes, tree rebuilds. */
void cco_counters(const cco_solver* s, long long* out7);
/* Exact CCD re-check of a finished step: element pairs that still collide
 * over [x_old, x_new] by the reference's CCD predicate (h = eps, avgVel =
 * (x_new - x_old)/dt, no impulses); negative on error. params as cco_step. */
long long cco_check_ccd(cco_solver* s, const double* x_old, const double* x_new, const double* params);

#ifdef __cplusplus
}
#endif
#endif
