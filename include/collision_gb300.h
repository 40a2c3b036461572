/*
 * collision_gb300 - C ABI of the GB300 collision-handling library.
 *
 * A drop-in for the collision step of antdvid/Collision's CollisionSolver3d:
 * build a solver once per mesh, then once per time step hand it the old and
 * candidate point positions and call cc_resolve(), which runs the reference's
 * resolveCollision() (dcollid.cpp:317-362) on the GPU - proximity repulsion,
 * up to five CCD passes, impact zones, the domain clamp, final positions,
 * strain limiting and final velocities - and writes the results back.
 *
 * Plain pointers and sizes only. Arrays of points are point-major
 * (x0,y0,z0,x1,...) float64. Every call returns a cc_status; on failure
 * cc_last_error() describes it. One solver belongs to one host thread and
 * runs on its own CUDA stream on the device it was created on.
 */
#ifndef COLLISION_GB300_H
#define COLLISION_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cc_solver cc_solver;

typedef enum {
    CC_OK = 0,
    CC_BAD_INPUT = 1,
    CC_PAIR_OVERFLOW = 2,
    CC_STACK_OVERFLOW = 3,
    CC_ITER_CAP = 4,
    CC_NAN_DETECTED = 5,
    CC_CUDA_ERROR = 6,
    CC_CONTACT_OVERFLOW = 7,
    CC_NO_MEMORY = 8
} cc_status;

/* Solver parameters, in this order (the reference's class statics,
 * collid.h:134-140; defaults dcollid.cpp:28-35). */
typedef struct {
    double dt;         /* setTimeStepSize        collid.h:184 */
    double thickness;  /* setFabricThickness     collid.h:182 */
    double eps;        /* setRoundingTolerance   collid.h:180 */
    double k;          /* setSpringConstant      collid.h:186 */
    double m;          /* setPointMass           collid.h:190 */
    double lambda;     /* setFrictionConstant    collid.h:188 */
    double cr;         /* setRestitutionCoef     collid.h:192 */
} cc_params;

/*
 * The element lists the reference assembles from a FronTier interface
 * (assembleFromInterface, dcollid3d.cpp:12-52): triangles of every
 * non-boundary surface, surface by surface, then the bonds of every string
 * curve. Elements are numbered tris first, then bonds, in array order; that
 * order is the reference's hseList order and fixes its tree insertion order.
 *   tris          n_tris*3 point ids
 *   tri_surface   surface id per triangle (a tri pair on one surface with a
 *                 fixed point is skipped, dcollid.cpp:805-806)
 *   tri_rest_len  n_tris*3 rest lengths of edges (p0p1, p1p2, p2p0)
 *                 (TRI::side_length0, dcollid.cpp:513-514)
 *   bonds         n_bonds*2 point ids
 *   bond_rest_len n_bonds rest lengths (BOND::length0, dcollid.cpp:515-516)
 *   fixed         n_points flags: 1 = point of a fixed rigid obstacle
 *                 (STATE::is_fixed, cdinit.cpp:199-202), 2 = point of a
 *                 movable rigid body (STATE::is_movableRG, cdinit.cpp:204;
 *                 see cc_set_body), 0 = free
 */
typedef struct {
    int32_t n_points;
    int32_t n_tris;
    const int32_t* tris;
    const int32_t* tri_surface;
    const double* tri_rest_len;
    int32_t n_bonds;
    const int32_t* bonds;
    const double* bond_rest_len;
    const uint8_t* fixed;
} cc_mesh;

/* new CollisionSolver3d() (collid.h:241, test.cpp:62). device = CUDA ordinal. */
cc_status cc_create(int device, cc_solver** out);

/* delete solver (test.cpp:131). NULL is accepted. */
void cc_destroy(cc_solver* s);

/*
 * assembleFromInterface (collid.h:242, dcollid3d.cpp:12-52) for a mesh whose
 * topology stays fixed across steps - the reference's trees persist and
 * remap leaves by point ids (AABB.cpp:199-245), so it too needs the same
 * elements every step. Copies the mesh to the device. Calling it again
 * replaces the mesh and resets the trees.
 */
cc_status cc_assemble(cc_solver* s, const cc_mesh* mesh);

/* The static setters of collid.h:180-193, all at once. */
cc_status cc_set_params(cc_solver* s, const cc_params* p);

/* setDomainBoundary (collid.h:203, dcollid.cpp:109-114). */
cc_status cc_set_domain_boundary(cc_solver* s, const double lo[3], const double hi[3]);

/*
 * resolveCollision (collid.h:201, dcollid.cpp:317-362) on host buffers.
 *   x_old       n_points*3  positions at the start of the step (STATE::x_old)
 *   x_cand      n_points*3  candidate positions (Coords on entry)
 *   vel         n_points*3  in: velocities; out: avgVel of every point with
 *                           has_collsn, others unchanged (dcollid.cpp:598-624)
 *   has_collsn  n_points    in/out collision flags (STATE::has_collsn)
 *   x_out       n_points*3  out: final positions (Coords on exit)
 *   has_collision  out: hasCollision() (collid.h:205), may be NULL
 * Host-device copies happen inside the call.
 */
cc_status cc_resolve(cc_solver* s, const double* x_old, const double* x_cand, double* vel, uint8_t* has_collsn,
                     double* x_out, int* has_collision);

/* As cc_resolve, with every array already in device memory of the solver's
 * device (no host copies; the call returns when the step is done). */
cc_status cc_resolve_device(cc_solver* s, const double* x_old, const double* x_cand, double* vel,
                            uint8_t* has_collsn, double* x_out, int* has_collision);

/*
 * Batches: several independent scenes resolved together, each with its own
 * mesh, parameters, domain box, trees and pass sequence - as if each were
 * its own CollisionSolver3d and resolveCollision() were called on each.
 * No counterpart in the reference, whose solver state is static
 * (collid.h:134-140) and so holds one scene per process.
 *
 * cc_assemble_batch replaces the solver's mesh by n_scenes meshes. Points
 * and elements of all scenes are numbered scene by scene: the arrays of the
 * resolve calls hold scene 0's points, then scene 1's, and so on;
 * cc_get_scene_offsets gives the first point and first element of each
 * scene (n_scenes + 1 entries each, the last being the totals; either
 * pointer may be NULL). Every scene starts with the solver's current
 * parameters and domain box; cc_set_params and cc_set_domain_boundary set
 * all scenes, the _scene_ forms one. cc_assemble is cc_assemble_batch with
 * one mesh.
 */
cc_status cc_assemble_batch(cc_solver* s, const cc_mesh* meshes, int n_scenes);
int cc_num_scenes(cc_solver* s);
cc_status cc_get_scene_offsets(cc_solver* s, int32_t* point_off, int32_t* elem_off);
cc_status cc_set_scene_params(cc_solver* s, int scene, const cc_params* p);
cc_status cc_set_scene_domain_boundary(cc_solver* s, int scene, const double lo[3], const double hi[3]);

/* resolveCollision on every scene of the batch, as cc_resolve (host
 * buffers) and cc_resolve_device (device buffers), with has_collision
 * holding one flag per scene (may be NULL). cc_resolve and
 * cc_resolve_device on a batch report whether any scene collided. */
cc_status cc_resolve_batch(cc_solver* s, const double* x_old, const double* x_cand, double* vel,
                           uint8_t* has_collsn, double* x_out, int* has_collision);
cc_status cc_resolve_batch_device(cc_solver* s, const double* x_old, const double* x_cand, double* vel,
                                  uint8_t* has_collsn, double* x_out, int* has_collision);

/* Exact FP64 re-check of a finished step (device arrays, all scenes): every
 * element pair whose swept boxes over [x_old, x_new] overlap goes through
 * the reference's CCD predicate (isCoplanar and the point-triangle /
 * edge-edge tests with h = eps, dcollid3d.cpp:203-482, 643-922) with
 * avgVel = (x_new - x_old)/dt, without impulses. *hits receives the number
 * of element pairs that still collide (0 for a fully resolved step),
 * scene_hits (may be NULL) the count per scene. No counterpart in the
 * reference. Replaces the solver's per-step device state (zone roots and
 * recorded visits are kept). */
cc_status cc_check_ccd(cc_solver* s, const double* x_old, const double* x_new, long long* hits, int* scene_hits);

/* Movable rigid bodies. A point whose flag (cc_mesh.fixed) is 2 is movable
 * (is_movableRG). Every triangle surface (a run of equal tri_surface ids)
 * whose first point is movable is one rigid body: createImpZoneForRG
 * (dcollid3d.cpp:54-68) makes it one impact zone at the start of each step,
 * impulses between rigid points spread over it (SpreadImpactZoneImpulse,
 * dcollid.cpp:1101-1115), it moves rigidly after every pass
 * (updateImpactZoneVelocityForRG, dcollid.cpp:267-288) and its centre of
 * mass is advanced at the end of the step (updateFinalForRG,
 * dcollid.cpp:626-675). Its points must all be movable and belong to no
 * other element, and every movable point must lie in such a surface
 * (CC_BAD_INPUT otherwise). cc_set_body gives a body's HYPER_SURF data -
 * total_mass (default 1), center_of_mass and center_of_mass_velo (default
 * 0) - and the first call also seeds the remembered centre of mass that
 * updateFinalForRG reads (dcollid.cpp:650). cc_get_body reads the centre of
 * mass and its velocity after a step. `surface` is the body's tri_surface
 * id in scene `scene`. */
cc_status cc_set_body(cc_solver* s, int scene, int surface, double mass, const double* com, const double* comv);
cc_status cc_get_body(cc_solver* s, int scene, int surface, double* com, double* comv);

/* Impact-zone passes per scene and step before the loop is stopped
 * (default 10000). The reference's loop (dcollid.cpp:346-352) has no bound
 * and does not end for some configurations; a scene that reaches the cap is
 * finished with its current velocities, its status becomes CC_ITER_CAP
 * (cc_get_scene_status, one int per scene) and the call returns CC_ITER_CAP
 * after completing every other scene. */
cc_status cc_set_zone_cap(cc_solver* s, int cap);
cc_status cc_get_scene_status(cc_solver* s, int* out);
/* Leave a scene out of the following resolve calls (on = 0) or take it
 * back: a disabled scene's points get x_out = x_cand and keep their
 * velocities and flags. */
cc_status cc_set_scene_enabled(cc_solver* s, int scene, int on);

/* Tuning knobs (none changes results):
 *   CC_TUNE_SPLIT_NARROW    1 (default): mixed passes without impact zones
 *                           or recording filter per pair, then run the FP64
 *                           sub-tests that pass, one thread each; 0: one
 *                           thread per pair throughout
 *   CC_TUNE_TRAVERSE_BLOCK  threads per block of the BVH traversal (32..1024)
 *   CC_TUNE_NARROW_BLOCK    threads per block of the per-pair filter stage
 *                           of split passes (32..512)
 *   CC_TUNE_STRAIN_BLOCK    threads of each scene's strain-sweep CTA (32..256)
 *   CC_TUNE_TAIL_GRAPH      1 (default): the end of a step (domain clamp and
 *                           final positions, the strain-limiting loop, whose
 *                           end is decided on the device, final velocities)
 *                           runs as one captured CUDA graph, replayed every
 *                           step; 0: launched kernel by kernel
 *   CC_TUNE_COMBINED_BROAD  1 (default): the proximity pass finds its pairs
 *                           on swept boxes, flagged where the static boxes
 *                           overlap, and the first CCD pass reuses them when
 *                           the proximity pass applied no impulse; 0: a
 *                           broad phase per pass
 *   CC_TUNE_STRAIN_WARP     1: each scene's strain sweep runs on one warp
 *                           with its levels staged in shared memory;
 *                           0 (default): on a CTA of CC_TUNE_STRAIN_BLOCK
 *                           threads. Same results; the CTA sweep is faster
 *                           for sheets whose levels hold more than ~32 edges
 *   CC_TUNE_PACKET_TRAVERSE 1: each warp walks the hierarchy as one packet of
 *                           32 Morton-consecutive queries with a shared-memory
 *                           stack; 0 (default): a stack per thread. Same
 *                           pairs; the packets are slower on the cloth
 *                           workloads, whose neighbouring queries diverge
 *   CC_TUNE_TAIL_OVERLAP    1: once half the scenes have finished their
 *                           detection passes, those end their step (final
 *                           positions, strain limiting, final velocities) on
 *                           a second stream while the other scenes' passes
 *                           go on; 0 (default): every scene's end of step
 *                           after the last pass. Same results; no faster on
 *                           the cloth batches, whose strain sweep then
 *                           competes with the passes for the SMs
 *   CC_TUNE_ROPE_TRAVERSE   1 (default): each query walks the hierarchy
 *                           without a stack, from the subtree after its own
 *                           leaf along ropes (the next subtree in depth-first
 *                           order); 0: a stack per thread from the scene's
 *                           root. Same pairs
 *   CC_TUNE_SUBSET_REFIT    1 (default): a detection pass over some of the
 *                           scenes, after the step's first pass built the
 *                           hierarchy over all of them, refits that hierarchy
 *                           over its scenes' leaves; 0: it sorts and builds a
 *                           hierarchy of its own. Same pairs
 *   CC_TUNE_STRAIN_ROLES    1 (default): in the shared-memory strain sweep a
 *                           level's edges, copy-ins and write-backs run on
 *                           separate threads (when they fit in the block);
 *                           0: every thread takes one of each
 *   CC_TUNE_TRAVERSE_REFILL 1..32 (default 8): the stackless traversal runs
 *                           on resident warps whose lanes take new queries
 *                           from a counter once this many of them have
 *                           finished their walks, testing each leaf on a
 *                           32-byte FP32 record before its exact one; 0: one
 *                           thread per query. Same pairs
 *   CC_TUNE_STACK_DEPTH     entries of the per-thread stack of the stack
 *                           traversal: 24, 32, 48 or 64 (default); a pass
 *                           whose walk needs more is run again with 64
 *   CC_TUNE_PAIR_CAPACITY   candidate pairs the pair buffer holds (>= 4096;
 *                           default 8 per element + 4096, grown on overflow
 *                           and by cc_autotune to a timed pass's need plus a
 *                           quarter)
 *   CC_TUNE_DEVICE_LOOP     1 (default): after the proximity pass, every
 *                           detection pass of a step runs in one CUDA graph
 *                           (a WHILE node over one pass, the impact-zone
 *                           stage behind an IF node) with each scene's pass
 *                           sequence on the device; the host steps in only to
 *                           rebuild a reference tree or grow a buffer. Not
 *                           with recording or VTK dumps, which take the host
 *                           loop. 0: the host runs every pass. Same results
 *   CC_TUNE_PRUNE           1 (default): in the device loop, passes after the
 *                           first CCD pass test only the element pairs with a
 *                           point the previous pass touched (the only pairs
 *                           that can hit); 0: every pair. Same results
 *   CC_TUNE_HOST_TREE       0 (default): the reference trees' leaf order is
 *                           built on the GPU (the insertions pipelined, one
 *                           CTA per tree); 1: on host threads, one tree per
 *                           thread. Same ranks and volumes
 *   CC_TUNE_SMALL_SORT      1 (default): an impact-zone pass sorts up to
 *                           8,192 union records in one CTA (in the device
 *                           loop the general radix sort then does not run);
 *                           0: always the general sort. Same results
 *   CC_TUNE_PRUNED_WARP     1 (default): in the device loop's pruned passes
 *                           each query walks its scene with one warp (a
 *                           shared-memory stack, up to 32 nodes per round);
 *                           0: one thread along the ropes. Same results
 *   CC_TUNE_ROBUST_ROOTS    1 (default): the mixed path's FP64 sub-tests
 *                           form a coplanarity root again with correctly
 *                           rounded functions only where a decision can
 *                           depend on it (not for roots well inside the time
 *                           window at which the test misses with a margin
 *                           covering the root's error); 0: every root near
 *                           the window. Same results
 *   CC_TUNE_ZONE_CTA_MIN    members from which an impact zone's rigid
 *                           motion is computed by a CTA of its own (>= 16,
 *                           default 64; smaller zones of 16+ members get a
 *                           warp, the rest a thread). Same results
 *   CC_TUNE_REPLAY_CTA_MIN  union records from which a final impact zone's
 *                           unions are replayed by a CTA in shared memory
 *                           (0, the default: every zone by one thread from
 *                           global memory, measured faster). Same results
 *   CC_TUNE_REFIT_UP        1 (default): the hierarchy refit's walk up takes
 *                           one acquire-release arrival per level, carries
 *                           its box in registers and ends at its scene's
 *                           root; 0: fence, arrival, fence and both children
 *                           loaded per level. Same results
 *   CC_TUNE_ZONE_FEW        impact zones in a pass at or below which every
 *                           zone of two or more members is solved by a warp
 *                           (default 1024; above it, zones under 16 members
 *                           get a thread each). Same results
 *   CC_TUNE_SUBTEST_MERGE   1 (default): the mixed path's point-triangle
 *                           and edge-edge FP64 sub-tests of a pass with at
 *                           most 65,536 of them in one launch, a warp per
 *                           sub-test where there are at most 1,216 (larger
 *                           passes: one launch per kind); 0: one launch per
 *                           kind, a thread per sub-test. Same results
 * cc_get_tuning returns the current value, or -1 for an unknown knob. */
enum {
    CC_TUNE_SPLIT_NARROW = 0,
    CC_TUNE_TRAVERSE_BLOCK = 1,
    CC_TUNE_NARROW_BLOCK = 2,
    CC_TUNE_STRAIN_BLOCK = 3,
    CC_TUNE_TAIL_GRAPH = 4,
    CC_TUNE_COMBINED_BROAD = 5,
    CC_TUNE_STRAIN_WARP = 6,
    CC_TUNE_PACKET_TRAVERSE = 7,
    CC_TUNE_STRAIN_ROLES = 8,
    CC_TUNE_TAIL_OVERLAP = 9,
    CC_TUNE_ROPE_TRAVERSE = 10,
    CC_TUNE_SUBSET_REFIT = 11,
    CC_TUNE_TRAVERSE_REFILL = 12,
    CC_TUNE_STACK_DEPTH = 13,
    CC_TUNE_PAIR_CAPACITY = 14,
    CC_TUNE_DEVICE_LOOP = 15,
    CC_TUNE_PRUNE = 16,
    CC_TUNE_HOST_TREE = 17,
    CC_TUNE_SMALL_SORT = 18,
    CC_TUNE_PRUNED_WARP = 19,
    CC_TUNE_ROBUST_ROOTS = 20,
    CC_TUNE_ZONE_CTA_MIN = 21,
    CC_TUNE_REPLAY_CTA_MIN = 22,
    CC_TUNE_REFIT_UP = 23,
    CC_TUNE_ZONE_FEW = 24,
    CC_TUNE_SUBTEST_MERGE = 25
};
cc_status cc_set_tuning(cc_solver* s, int knob, int value);
int cc_get_tuning(cc_solver* s, int knob);
/* Autotuner: on the state of the last resolve call, times one moving pass
 * of every scene (traversal and narrow phase, no impulses applied) for
 * candidate settings - CC_TUNE_TRAVERSE_REFILL, the stackless traversal's
 * CC_TUNE_TRAVERSE_BLOCK, the stack traversal's block and
 * CC_TUNE_STACK_DEPTH, CC_TUNE_SPLIT_NARROW and CC_TUNE_NARROW_BLOCK -
 * keeps the fastest, and grows the pair and sub-test buffers to at least
 * that pass's needs plus a quarter (CC_TUNE_PAIR_CAPACITY). The solver's
 * state is unchanged. *best_ms (may be NULL) receives the best time. */
cc_status cc_autotune(cc_solver* s, double* best_ms);

/* Debugging dumps, as the reference writes under its "CollisionImpulse"
 * flag (dcollid.cpp:684-693, vtk.cpp:14-93): after every detection pass, one
 * VTK XML PolyData file per scene in dir (created if missing) - surf-NNN.vtp
 * for a single scene, surf-sSSS-NNN.vtp in a batch - with the surface at
 * x_old + dt*avgVel before the pass's impulses, each point's accumulated
 * impulse (CollsnImpulse) and each element red if a point of it was hit in
 * the pass, green otherwise (CollsnRegion). NULL or "" turns dumps off.
 * Call after cc_assemble. Slow (host copies each pass). */
cc_status cc_set_vtk_dump(cc_solver* s, const char* dir);

/* Host threads that emulate the reference's tree insertion order when a
 * scene's tree is (re)built, one scene per thread (0 = one per hardware
 * thread, the default). */
cc_status cc_set_host_threads(cc_solver* s, int n);

/* Arithmetic of the narrow phase:
 *   0  plain FP64 (default): every sub-test evaluated in FP64 as the reference
 *   1  mixed precision: FP32 swept boxes of each sub-test's points, rounded
 *      outward and padded by the test's reach, reject sub-tests that cannot
 *      hit; the others are evaluated in FP64 exactly as in mode 0, so the
 *      results are the same as mode 0's. */
cc_status cc_set_mode(cc_solver* s, int mode);

/* Strain limiting keeps each point's velocity in shared memory while the
 * sweep uses it (default, on); off runs the same sweep on global memory.
 * Both give the same results. */
cc_status cc_set_strain_window(cc_solver* s, int on);

/* Counters of the last step, summed over the scenes of a batch, in this
 * order: detection passes, CCD passes, impact-zone passes, candidate pairs
 * (all passes), narrow-phase visits, pairs that hit, contacts (sub-tests
 * that applied an impulse), strain passes, tree builds, kernel launches,
 * strain edges averaged, strain tests taken the exact way, sub-tests
 * evaluated in FP64, narrow-phase visits of CCD and impact-zone passes,
 * algorithmic bytes of the strain sweeps, coplanarity cubics whose roots
 * were formed again with correctly rounded functions, leaves traversed by
 * the broad phase (summed over its traversals), candidate pairs those
 * traversals wrote, the step's algorithmic bytes (below), the leaves and
 * pairs of the traversals launched from the host (those the "traverse" stage
 * of cc_get_profile times: every traversal in the host loop, the proximity
 * pass's with CC_TUNE_DEVICE_LOOP), the passes the device loop ran, the
 * time spent building the reference trees' leaf order (microseconds, the
 * build on the GPU or its emulation on host threads, with the copies and
 * synchronisation around it), the queries of the device loop's pruned
 * traversals, and the union records of impact-zone passes.
 * Algorithmic bytes: per scene-step 120 per
 * point (x_old, x_cand, v read; x, v written); per scene-pass 72 per point,
 * 12 per triangle, 8 per bond and 48 per hierarchy node (2E-1 nodes of
 * 24-byte FP32 boxes, written by the refit and read by the traversal), plus
 * 48 per point in impact-zone passes; per pass 16 per candidate pair and
 * 416 per contact; per strain pass 48 per point and 24 per element edge.
 * Candidate pairs and
 * visits leave out pairs of elements that share a point (their tests
 * return false at once) unless recording is on. Returns how many were
 * written. */
int cc_get_counters(cc_solver* s, long long* out, int n);

/* Recording for parity checks: when on, every narrow-phase visit of the
 * next steps is kept (13 ints each: pass, kind, a, b, status, dcount[6],
 * rank_b, rank_a; a/b as the reference calls TriToTri/TriToBond/BondToBond). */
cc_status cc_set_recording(cc_solver* s, int on);
int cc_get_visits(cc_solver* s, int* out, int cap);
/* Kinds (0 proximity, 1 CCD, 2 impact zone) of the last step's passes of
 * scene 0, or of the given scene; returns the number of passes. Visit
 * records carry their scene's pass index and batch element ids. */
int cc_get_pass_kinds(cc_solver* s, int* out, int cap);
int cc_get_scene_pass_kinds(cc_solver* s, int scene, int* out, int cap);
/* Impact-zone root of every point after the last step. */
cc_status cc_get_zone_roots(cc_solver* s, int* out);
/* Leaf rank of every element in its scene's proximity (which=0) or
 * collision (which=1) tree; CC_BAD_INPUT while one of them is unbuilt. */
cc_status cc_get_leaf_ranks(cc_solver* s, int which, int* out);
/* Root volume of the scene's last built tree (AABBTree::getVolume,
 * AABB.h:114; the rebuild test of dcollid.cpp:381, 422 compares with it). */
cc_status cc_get_tree_volume(cc_solver* s, int scene, double* out);

/* Candidate pairs of the current state (after cc_resolve: the final x_old
 * and average velocities), by LBVH traversal or by testing all pairs; for
 * cross-checks. Writes up to cap (a,b) pairs, returns the count or -1. */
int cc_debug_candidate_pairs(cc_solver* s, int moving, int brute_force, int* out, int cap);

/* Run the solver on a caller's CUDA stream (cudaStream_t; NULL = a stream
 * of its own). Work is ordered after everything already queued there. */
cc_status cc_set_stream(cc_solver* s, void* stream);

/* Per-stage GPU time of the following steps, measured with CUDA events on
 * the solver's stream: cc_get_profile writes accumulated milliseconds and
 * call counts per stage (names from cc_profile_stage_name) and returns the
 * number of stages. on = 1: stages outside the device loop's graph (that
 * graph counts as one stage, detect_loop); on = 2: also the stages of every
 * pass inside it (loop_*), from boundary kernels that read the global timer
 * (a few launches per pass more); 0: off. */
cc_status cc_set_profiling(cc_solver* s, int on);
int cc_get_profile(cc_solver* s, double* ms, long long* calls, int cap);
const char* cc_profile_stage_name(int i);

/* Self-test of the correctly rounded math the FP64 path uses on the GPU:
 * fn 0 cos(a), 1 sin(a), 2 acos(a), 3 pow(a, b), for n host values; returns
 * n or -1. These functions reproduce the reference's libm (glibc) wherever
 * its result is correctly rounded. */
int cc_selftest_math(int device, int fn, const double* a, const double* b, double* out, int n);

/*
 * Candidate pairs without allocating: no counterpart in the reference.
 *
 * The broad phase of cc_resolve (all pairs of n boxes that overlap, each
 * unordered pair once) for callers that cannot call cudaMalloc - code whose
 * device memory belongs to another allocator (an engine that reserves the
 * GPU at start-up, a framework's caching pool) or a loop that must not
 * stall, since cudaMalloc/cudaFree can synchronise the device and fail under
 * fragmentation. Nothing is allocated: the caller owns the inputs and outputs,
 * and every intermediate array lives in an 8 MiB scratch area compiled into
 * the library (held on every GPU that loads it until exit). Limit: n <= 65536.
 *   boxes   device, n x 6 doubles (lo x,y,z, hi x,y,z), 16-byte aligned;
 *           every coordinate finite and lo <= hi (else CC_BAD_INPUT)
 *   pairs   device, cap x 2 ints (element indices), 8-byte aligned
 *   npairs  host: the number of overlapping pairs (may exceed cap, then only
 *           cap are written and CC_PAIR_OVERFLOW is returned)
 *   stream  cudaStream_t of `device` (else CC_BAD_INPUT) or NULL; the call
 *           waits for its work to finish.
 * The first call on a device looks up the scratch area's address there; make
 * it before any stream capture starts. Calls share the scratch area: calls
 * that overlap on the GPU race. The calling thread's current device is the
 * same after the call as before. A hierarchy index found out of range
 * returns CC_CUDA_ERROR with *npairs = 0. Errors: cc_static_last_error.
 */
cc_status cc_candidate_pairs_static(int device, const double* boxes, int n, int* pairs, int cap, int* npairs,
                                    void* stream);
int cc_static_last_error(char* buf, int len);

/* Last error message of this solver (NUL-terminated, truncated to len). */
int cc_last_error(cc_solver* s, char* buf, int len);

#ifdef __cplusplus
}
#endif

#endif
