// Host-side launch wrappers for the collision kernels. Every wrapper
// enqueues on the given stream and returns without synchronising.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cc_common.cuh"

namespace ccg {

// Kernels launched by this library since load (read by cc_get_counters).
extern long long g_kernel_launches;
inline void count_launch(int n = 1) { g_kernel_launches += n; }

// Launch shapes that do not change results (set through cc_set_tuning).
struct LaunchTuning {
    bool packet_traverse = false;  // warp-cooperative traversal (k_traverse_packet)
    bool rope_traverse = true;     // stackless traversal along ropes (k_traverse_rope)
    int traverse_refill = 8;       // stackless: lanes that refill together (0: one thread per query)
    int stack_depth = kTraversalStack;  // stack traversal: entries per thread
    int traverse_block = 128;     // threads per block of the per-thread traversal
    int narrow_block = 128;
    int strain_block = 256;
};

// ------------------------------------------------------------- primitives
// Scratch bytes needed to sort n (key, value) pairs.
size_t radix_sort_temp_bytes(int n);
// Stable LSD radix sort of (keys, vals) on the low `bits` bits of the keys.
// keys/vals are sorted in place (the temp buffer holds the ping-pong copy).
void radix_sort_pairs(unsigned long long* keys, unsigned int* vals, int n, int bits, void* temp,
                      cudaStream_t s);
// The same for the first min(*dn, cap) pairs, the count in device memory
// (temp sized for cap; the arrays hold cap pairs).
void radix_sort_pairs_dev(unsigned long long* keys, unsigned int* vals, const int* dn, int cap, int bits, void* temp,
                          cudaStream_t s);
// The same with counts of up to 8192 pairs sorted by one CTA in shared
// memory (keys below 2^51); eff: a device int the two stages share. On a
// stream that is being captured, with `nested` (a second stream) given, the
// general sort sits behind a conditional node and runs only for larger
// counts. small = false: always the general sort.
cudaError_t sort_pairs_dev(unsigned long long* keys, unsigned int* vals, const int* dn, int cap, int bits,
                           void* temp, int* eff, cudaStream_t s, cudaStream_t nested, bool small = true);
// Exclusive scan of n ints (out may alias in); total written to *total.
size_t scan_temp_bytes(int n);
void exclusive_scan(const int* in, int* out, int n, int* total, void* temp, cudaStream_t s);

// ------------------------------------------------------------- broad phase
struct __align__(16) Box6 {
    double lo[3];
    double hi[3];
};

// An internal LBVH node as the traversal reads it: both children's boxes in
// FP32, rounded outward (so a test against them never rejects what the
// exact boxes would accept), the children (>= 0 internal, < 0 ~leaf), and
// the last sorted leaf under each child.
struct __align__(16) BvhNode32 {
    float4 b0;  // child 0: lo.x lo.y lo.z hi.x
    float4 b1;  // child 0: hi.y hi.z, child 1: lo.x lo.y
    float4 b2;  // child 1: lo.z hi.x hi.y hi.z
    int4 meta;  // child 0, child 1, last leaf under child 0, under child 1
};

// An internal LBVH node as the stackless traversal reads it: its own box in
// FP32 (rounded outward), its first child (>= 0 internal, < 0 ~leaf) and its
// rope - the subtree that follows it in depth-first order within its scene
// (kRopeEnd: none).
struct __align__(32) RopeNode {
    float lo[3], hi[3];
    int left;
    int rope;
};
constexpr int kRopeEnd = 0x7fffffff;

// A sorted leaf as the traversal's exact test reads it: the element's FP64
// box in the order-preserving integer encoding (lo xyz, hi xyz), its points
// (third -1 for a bond) and its id - one 64-byte record per leaf visit, with
// Morton neighbours next to each other.
struct __align__(64) LeafRec {
    unsigned long long lo[3], hi[3];
    int p[3];
    int e;
};

// A sorted leaf as the stackless traversal tests it first: the element's box
// rounded outward to FP32, the rope after the leaf and the element id - 32
// bytes, so a leaf whose box misses the query costs half a LeafRec load.
struct __align__(32) LeafBox32 {
    float lo[3], hi[3];
    int rope;
    int e;
};

struct BvhBufs {
    int n;                        // leaves of this pass's hierarchy
    const int* act;               // their element ids (null: elements 0..n-1)
    int nscenes;
    const int* elem_scene;        // scene of every element (null: one scene)
    const SceneDev* scenes;       // scene descriptors (null: one scene, root 0)
    SceneRun* run;                // per-pass scene state (null: one scene, root 0)
    int* range_lo;                // n-1: first sorted leaf covered by each internal node
    unsigned long long* keys;     // n Morton keys (sorted)
    unsigned int* order;          // n element ids in Morton order
    int* range_hi;                // n-1: last sorted leaf covered by each internal node
    int* parent;                  // 2n-1: parents of internal nodes [0,n-1) then leaves
    int* flags;                   // n-1 refit arrival counters
    BvhNode32* node;              // n-1 internal nodes
    unsigned long long* bbox_enc; // 6 encoded doubles per scene (scene boxes)
    void* sort_temp;
    // optional: one record per sorted leaf for the traversal's leaf test,
    // filled by bvh_pairs from the boxes and the element points ev
    struct LeafRec* leaf;
    const int* ev;
    int ne_all;  // elements of all scenes (bound of the ids in order)
    // optional: the stackless traversal's nodes and the rope of every leaf
    // boundary (rope[k]: the subtree after sorted leaf k in depth-first
    // order, the right child of the node that splits leaves k and k+1),
    // filled by bvh_build and bvh_refit
    RopeNode* rnode;  // n-1
    int* rope;        // n-1
    // optional: the FP32 leaf boxes of the stackless traversal with dynamic
    // query fetch, written with the leaf records; qnext: its query counter
    LeafBox32* leaf32;
    int* qnext;
    // optional: for a hierarchy over all elements (act null), the sorted
    // leaves of the scenes in this pass; the refit, the leaf records and the
    // traversal then cover only those (walks never leave their scene)
    const int* sub;
    int nsub;
    // optional: the count of sub in device memory (nsub is then its
    // capacity), for passes whose scenes are chosen on the device
    const int* dnsub;
    // optional: the traversal's query count in device memory, when it
    // differs from the leaf count dnsub (the queries are sub's first ones)
    const int* dnq;
    // refit walk: 1 one acquire-release arrival per level, each thread
    // carrying its box and ending at its scene's root; 0 fence, arrival,
    // fence and both children loaded per level, up to the top
    int refit_up = 1;
};

// Leaf boxes of every element (static: x_old; moving: x_old and
// x_old + dt*avgVel with the element's scene's dt), padded by 1e-6, plus
// each scene's union in bbox_enc[6*scene ..].
// Only the n elements listed in act (null: elements 0..n-1) are boxed; box
// is indexed by element id.
// dn (may be null): the element count in device memory, n its capacity; a
// count of 0 leaves the boxes and bbox_enc as they are.
void leaf_boxes(const int* ev, const int* act, int n, const int* elem_scene, const SceneDev* scenes, int nscenes,
                const double4_32a* xo, const double4_32a* av, int moving, Box6* box, unsigned long long* bbox_enc,
                cudaStream_t s, const int* dn = nullptr);
// The elements and points of the given scenes, in scene order:
// elem_off / pt_off are the exclusive prefix sums of their counts.
void expand_scenes(const int* scene_ids, const int* elem_off, const int* pt_off, int nsel, int n_elems, int n_pts,
                   const SceneDev* scenes, int* elems, int* pts, cudaStream_t s);
// Union of n given boxes in bbox_enc (the scene box the Morton keys use).
void boxes_bbox(const Box6* box, int n, unsigned long long* bbox_enc, cudaStream_t s);
// Morton keys (scene id above the 30 Morton bits, each scene normalised to
// its own box), sort, Karras hierarchy, per-scene subtree roots, refit.
void bvh_build(const Box6* box, BvhBufs& b, cudaStream_t s);
// New boxes for the same leaves in the same hierarchy (scene roots and
// refit only): the pairs found are the same, the tree is only less tight.
// roots = false: the scenes' roots set by the build stand (the hierarchy and
// each scene's first leaf are unchanged since).
void bvh_refit(const Box6* box, BvhBufs& b, cudaStream_t s, bool roots = true);
// All leaf pairs of one scene with overlapping boxes, each unordered pair
// once; scenes idle in this pass are skipped. With skip_shared_ev (the
// elements' point ids), pairs of elements sharing a point are left out.
// With box_static, every pair is found on `box` (swept boxes) and carries
// kPairStatic when the elements' static boxes overlap as well. Traversal:
// a stack per thread (default), a warp-cooperative packet, or (rope, with
// the leaf records and rope nodes present) stackless along the ropes.
// refill (rope only, with leaf32 and qnext present): persistent warps whose
// lanes take new queries from a counter once `refill` of them have finished
// their walks (0: one thread per query). stack_depth: entries of the
// per-thread stack of the stack traversal (24, 32, 48 or 64); a walk that
// needs more sets kErrStack.
void bvh_pairs(const Box6* box, const BvhBufs& b, int2* pairs, int cap, PassCounters* ctr, cudaStream_t s,
               const int* skip_shared_ev = nullptr, int block = 128, const Box6* box_static = nullptr,
               bool packet = false, bool rope = false, int refill = 0, int stack_depth = kTraversalStack);
// The same pair set by testing every pair (for cross-checks on small meshes).
void brute_pairs(const Box6* box, int ne, const int* elem_scene, int2* pairs, int cap, PassCounters* ctr,
                 cudaStream_t s);

// Pass stamps (the device loop's pruning of later passes): the kernels that
// change a point's average velocity in a pass, and the narrow phase for the
// points of every sub-test that hits, write the pass's serial into the
// point's stamp. Null: no stamps.
struct PassStamp {
    unsigned* stamp = nullptr;         // per point
    const unsigned* serial = nullptr;  // the current pass's serial, in device memory
};
__device__ __forceinline__ void stamp_point(const PassStamp& ps, int p) {
#ifdef __CUDACC__
    if (ps.stamp) ps.stamp[p] = *ps.serial;
#endif
}

// ------------------------------------------------------------ narrow phase
struct NarrowArgs {
    const double4_32a* xo;
    const double4_32a* av;
    const uint8_t* fixed;
    const int* ev;          // 3 point ids per element (bonds: third is -1)
    const int* esurf;
    const uint8_t* erigid;
    const int* rank;        // leaf rank of each element within its scene's tree (null: element ids)
    const int* escene;      // scene of each element
    const SceneDev* scenes; // parameters per scene
    SceneRun* run;          // mode and pass per scene; hits counted here
    const int2* pairs;
    Contrib* contrib;
    int contrib_cap;
    PassCounters* ctr;
    UnionRec* urec;         // createImpZone records (impact-zone passes)
    int urec_cap;
    VisitRec* rec;
    int rec_cap;
    const float4* pbox_lo;  // null: plain FP64 (no filter)
    const float4* pbox_hi;
    const float4* p32;      // x_old in FP32 (with pbox_lo)
    const float4* v32;      // avgVel in FP32 (with pbox_lo, moving passes)
    int check;              // hit decisions only (no impulses, contacts, zones)
    // split pass (mixed precision, no zones, no recording): the sub-tests
    // that pass the FP32 filters, point-triangle and edge-edge apart, and a
    // hit flag per candidate pair
    SubRec* sub_pt;
    SubRec* sub_ee;
    int sub_cap;
    int* pair_hit;  // per candidate pair: bit s set when sub-test s hit
    int* pairq;     // candidate pairs with a queued sub-test (capacity: the pair buffer's)
    int static_only;  // proximity pass over swept-box pairs: only those with kPairStatic
    PassStamp ps;     // stamps of the points of every sub-test that hits
    // the split sub-tests form a root again with correctly rounded functions
    // only where a decision can depend on it (is_coplanar's rb); 0: always
    int robust_roots = 1;
    // 1: both sub-test lists in one launch, a warp per sub-test in small
    // passes (k_subtests_all); 0: one launch per list, a thread per sub-test
    int sub_merge = 1;
    // movable rigid bodies: the body of each point (-1 none), each body's
    // mass, and the contribution slot of body 0 (the point count)
    const int* vbody;
    const double* body_mass;
    int body_slot0;
};
void narrow_pass(const NarrowArgs& a, int moving, int max_pairs, cudaStream_t s, int block = 128);
// The same pass in stages (mixed precision only, no recording): FP32
// filters per pair, then the FP64 sub-tests that pass them, one thread
// each, then - for scenes in impact-zone mode - the createImpZone calls of
// every pair that hit. parts selects the filters (kSplitFilter), the rest
// (kSplitSubtests) or both, so that the two can be timed apart.
enum { kSplitFilter = 1, kSplitSubtests = 2, kSplitAll = 3 };
void narrow_pass_split(const NarrowArgs& a, int moving, int max_pairs, cudaStream_t s, int block = 128,
                       bool zone = false, int parts = kSplitAll);
// Inputs of the mixed-precision filter: outward-rounded FP32 boxes of every
// point over the pass's time window (with its scene's dt), and x_old and
// (moving passes) avgVel rounded to FP32.
void point_boxes(const double4_32a* xo, const double4_32a* av, const int* vscene, const SceneDev* scenes,
                 const int* act_pts, int n, int moving, float4* lo, float4* hi, float4* p32, float4* v32,
                 cudaStream_t s, const int* dn = nullptr);

// ------------------------------------------------------------- post-pass
// Movable rigid bodies, all scenes' in one list. members / member_body: the
// points of every body in the order of its impact-zone member list (the
// reference's createImpZoneForRG unions) with their body; zone_off: each
// body's range there; visit / visit_off: each body's points in element
// order (updateFinalForRG); acc: the running collsnImpulse_RG per body; num:
// this pass's collsn_num_RG; out: k_final_rg's result per body.
struct BodyBufs {
    int n = 0;
    int nmembers = 0;
    const int* members = nullptr;
    const int* member_body = nullptr;
    const int* zone_off = nullptr;
    const int* visit = nullptr;
    const int* visit_off = nullptr;
    double4_32a* acc = nullptr;
    int* num = nullptr;
    double4_32a* out = nullptr;
    const uint8_t* fixed = nullptr;
};
struct ApplyBufs {
    int* cnt;      // nv + bodies
    int* off;      // nv + bodies
    int* cur;      // nv + bodies
    int* idx;      // contrib_cap
    void* scan_temp;
    PassStamp ps;  // stamps of the points whose velocity the pass changes
};
// Per-point sums of the pass's contributions in visiting order, then
// avgVel += (impulse + friction) / n and has_collsn (updateAverageVelocity).
// dump (may be null): per point, the pass's summed impulse and the number
// of contributions (zero for points without any). With bodies, contribution
// slots nv.. are the bodies' spread impulses, applied to their members after
// each point's own (the buffers in b hold nv + bodies slots).
void apply_contribs(const Contrib* contrib, const PassCounters* ctr, int contrib_cap, int nv, double4_32a* av,
                    uint8_t* has_collsn, ApplyBufs& b, cudaStream_t s, double4_32a* dump = nullptr,
                    const BodyBufs* bodies = nullptr);

// updateImpactZoneVelocity (dcollid.cpp:290-310): rigid motion of every
// zone, one thread per zone over members[zone_off[z] .. zone_off[z+1]) in
// the order of the reference's member list, with its scene's parameters.
// With run set, the zones are movable bodies and move only in scenes that
// are in a pass (updateImpactZoneVelocityForRG).
void zone_solve(const int* members, const int* zone_off, int nzones, const uint8_t* fixed, const double4_32a* xo,
                double4_32a* av, const int* vscene, const SceneDev* scenes, PassCounters* ctr, cudaStream_t s,
                const SceneRun* run = nullptr, PassStamp ps = PassStamp{});
// The same with zone z's members at members[zone_rng[z].x .. .y) and the
// zone count in device memory (*dnz, at most zone_cap).
void zone_solve_dev(const int* members, const int2* zone_rng, const int* dnz, int zone_cap, const uint8_t* fixed,
                    const double4_32a* xo, double4_32a* av, const int* vscene, const SceneDev* scenes,
                    PassCounters* ctr, cudaStream_t s, PassStamp ps = PassStamp{}, int cta_min = 64,
                    int few = 1024);

// Impact zones of a pass on the GPU (cc_zones.cu): buffers of the union
// replay and of the zone lists.
struct ZoneBufs {
    int cap = 0;                         // union records the buffers below hold
    const UnionRec* rec = nullptr;       // the pass's createImpZone records (count: PassCounters::nunion)
    unsigned long long* keys = nullptr;  // cap sort keys
    unsigned int* vals = nullptr;        // cap record indices
    int* seg = nullptr;                  // cap segment starts
    uint8_t* noop = nullptr;             // cap: the record joins nothing new (k_union_noop)
    void* sort_temp = nullptr;           // zone_sort_temp_bytes(cap)
    int* cc = nullptr;                   // per point: parent in the lock-free union-find
    UfNode* uf = nullptr;                // per point: the reference's union-find
    int zone_cap = 0;                    // zones the zone arrays hold
    int2* zone_rng = nullptr;            // per zone: its run of members
    int* zone_root = nullptr;            // per zone: its root
    int* members = nullptr;              // per point (at most one zone each)
    // the previous zone pass's lists (k_zone_members starts from them): a
    // copy of its member array, and per root its run and the epoch it was
    // listed in (prev_epoch == *epoch: the pass just before); n_pts_cap
    // bounds the members and zones of a pass (the points)
    int* prev_members = nullptr;
    int* prev_off = nullptr;
    int* prev_len = nullptr;
    unsigned* prev_epoch = nullptr;
    unsigned* epoch = nullptr;
    int n_pts_cap = 0;
    bool small_sort = true;              // sorts of up to 8192 records in one CTA
    int zone_cta_min = 64;               // zones of this many members are solved by a CTA each
    int zone_few = 1024;                 // passes with at most this many zones: a warp per zone of 2+ members
    int replay_cta_min = 0;              // zones with this many records are replayed in shared memory (0: never)
};
size_t zone_sort_temp_bytes(int cap);
// After a pass's impulses: join the pass's createImpZone records in the
// reference's order (scenes in impact-zone mode only), list every zone of a
// scene in that mode and move it rigidly (updateImpactZoneVelocity,
// dcollid.cpp:290-310). act_pts / n_pts: the points of the pass's scenes
// (null: all n_pts points; dn_pts, if given, holds the count on the device).
// nested: a second stream for conditional sorts while s is being captured
// (null otherwise); marks (may be null): stage boundaries after the sorts,
// the replay, the zone lists and the solve go to slots mark0..mark0+3
// (stage_mark). Returns a launch or capture error.
cudaError_t zone_pass(const ZoneBufs& z, const PassCounters* ctr, const uint8_t* fixed, const int* act_pts, int n_pts,
                      const int* dn_pts, const int* vscene, const SceneRun* run, const SceneDev* scenes,
                      double4_32a* av, const double4_32a* xo, cudaStream_t s, PassStamp ps = PassStamp{},
                      cudaStream_t nested = nullptr, unsigned long long* marks = nullptr, int mark0 = 0);

// ------------------------------------------------ device detection loop
// (cc_loop.cu) One pass of the loop: k_loop_plan picks each scene's mode and
// lists the pass's scenes (sel) with their element and point offsets
// (eoff, poff: nscenes + 1 each); loop_expand writes the pass's elements,
// their sorted leaves in the step's hierarchy and points; tree_check flags
// scenes whose tree `which` must be rebuilt on the host; loop_reset opens
// the pass; pass_end closes it and, in the graph, decides whether the loop
// goes on.
void loop_plan(SceneCtl* ctl, SceneRun* run, const SceneDev* scenes, int nscenes, LoopCtl* L, int* sel, int* eoff,
               int* poff, cudaGraphConditionalHandle h_zone, cudaStream_t s);
void loop_expand(const int* sel, const int* eoff, const int* poff, const SceneDev* scenes, const SceneCtl* ctl,
                 const LoopCtl* L, int cap, int* act_e, int* act_l, int* act_p, cudaStream_t s);
void tree_check(const SceneRun* run, int nscenes, const unsigned long long* bbox_enc, const double* vol,
                const int* built, int which, int* rebuild, LoopCtl* L, cudaStream_t s);
void loop_reset(PassCounters* c, SceneRun* run, int nscenes, LoopCtl* L, cudaStream_t s);
// tree_check then loop_reset as one launch (one block; the two launches
// above 4,096 scenes).
void tree_check_reset(SceneRun* run, int nscenes, const unsigned long long* bbox_enc, const double* vol,
                      const int* built, int which, int* rebuild, LoopCtl* L, PassCounters* c, cudaStream_t s);
// Stage profiling inside the loop graph: acc[0] the last boundary's time,
// then (ns, count) for each of kLoopMarkSlots slots 1.. - the time since the
// previous boundary - then a per-pass log (the row count, then
// kPassLogRows rows of kPassLogCols: each slot's time, and at the slot
// given c the pass's candidate pairs, queued sub-tests (point-triangle,
// edge-edge), union records and pruned queries).
constexpr int kLoopMarkSlots = 16;
constexpr int kPassLogRows = 4096;
constexpr int kPassLogCols = kLoopMarkSlots + 5;
constexpr size_t kMarkWords = 1 + 2 * kLoopMarkSlots + 1 + (size_t)kPassLogRows * kPassLogCols;
void stage_mark(unsigned long long* acc, int slot, cudaStream_t s, const PassCounters* c = nullptr,
                const LoopCtl* L = nullptr);
void pass_end(const PassCounters* c, SceneCtl* ctl, const SceneRun* run, int nscenes, LoopCtl* L, int combined,
              bool in_graph, cudaGraphConditionalHandle h_loop, cudaStream_t s);
// The pruned broad phase of the device loop's later passes (L->prune): the
// pass's elements with a point whose stamp is the previous pass's serial
// walk their whole scene, from its root, and every overlapping pair with
// such an element is written once. act_l: the pass's sorted leaves
// (L->nact_e of them; act_e is unused); edirty, query: ne_cap each.
// warp: one warp per dirty element walking with a shared-memory stack
// (k_traverse_warp_full); otherwise one thread along the ropes.
void pruned_pairs(const BvhBufs& b, const int* act_e, const int* act_l, const unsigned* stamp, LoopCtl* L,
                  uint8_t* edirty, int* query, int ne_cap, int2* pairs, int cap, PassCounters* ctr, const int* ev,
                  cudaStream_t s, bool warp = true);

// updateFinalForRG's device part: per body, the first point in element
// order with has_collsn and its average velocity (into b.out).
void final_rigid(const BodyBufs& b, const uint8_t* has_collsn, const double4_32a* av, cudaStream_t s);

// Step set-up: pack inputs, average velocity (computeAverageVelocity), each
// point with its scene's dt.
void step_init(const double* x_old, const double* x_cand, int nv, const uint8_t* in_elem, const int* vscene,
               const SceneDev* scenes, double4_32a* xo, double4_32a* av, PassCounters* ctr, cudaStream_t s);
// Domain clamp + final position (detectDomainBoundaryCollision,
// updateFinalPosition) with each point's scene's parameters and domain box;
// movable points are not clamped.
void finalize_positions(const uint8_t* in_elem, const double4_32a* xo, double4_32a* av, uint8_t* has_collsn,
                        const double* x_cand, double* x_out, int nv, const int* vscene, const SceneDev* scenes,
                        const uint8_t* fixed, const uint8_t* mask, cudaStream_t s);
// reduceSuperelast: up to 10 Gauss-Seidel passes over each scene's strain
// edges, one CTA per scene.
struct StrainEdge {
    int p0, p1;
    double len0;
    int s0, s1;  // shared-memory slots of p0, p1 in the scene's window sweep
};
// Strain schedule of all scenes: the edges of a scene are contiguous and
// sorted by dependency level; its levels are hdr[2*(hdr0 + l)] =
// (edge begin, end, copy-in begin, end) and hdr[2*(hdr0 + l) + 1] =
// (write-back begin, end, 0, 0) for l < levels, with (point, slot) entries
// in load_list / wb_list; the write-backs after its last level are
// wb_list[wb_final0 .. wb_final1) (SceneDev).
struct StrainPlan {
    bool window;           // sweep in shared memory where the scene's slots fit
    int max_window_slots;  // largest slot count among the scenes that fit
    bool any_global;       // some scene needs more slots than fit
    int block;             // threads per sweep CTA
    bool warp;             // one warp per scene with staged levels (k_strain_warp)
    int ecap, lcap, wcap;  // most edges, copy-ins, write-backs of one level (scenes that fit)
    size_t warp_smem;      // its dynamic shared memory
    const int* order;      // device: scene of each sweep CTA, most levels first
    // window sweep: first thread of the copy-in and the write-back roles (a
    // level's edges on threads [0, cbase)); 0, 0: every thread takes all three
    int cbase, wbase;
};
// Dynamic shared memory of the one-warp sweep for these sizes.
size_t strain_warp_smem(int max_slots, int ecap, int lcap, int wcap);
int strain_window_slot_cap();
// Once per device before any strain_limit (not a stream operation, so it
// stays out of captured graphs).
void strain_configure();
// step_buf holds strain_step_bytes(nedges); passes_out holds 3 ints per
// scene (passes, averaged edges, exact tests).
size_t strain_step_bytes(int nedges);
// chunks: (scene, first edge) of every run of at most 256 edges of one
// scene; flags: 2 ints per scene.
// Per step, before any strain_limit: each edge's records from x_old.
void strain_setup(const StrainEdge* edges, int nedges, const SceneDev* scenes, const StrainPlan& plan,
                  const double4_32a* xo, void* step_buf, const int* vscene, cudaStream_t s);
// The strain loop of the scenes in mask (per scene, nonzero: in; null: all).
void strain_limit(const StrainEdge* edges, int nedges, const int4* hdr, const int2* load_list, const int2* wb_list,
                  const int2* chunks, int nchunks, const SceneDev* scenes, int nscenes, const StrainPlan& plan,
                  const double4_32a* xo, double4_32a* av, void* step_buf, int* flags, int* passes_out,
                  const uint8_t* mask, cudaStream_t s);
// Correctly rounded cos/sin/acos/pow (fn 0..3) on device arrays, for self-tests.
void math_selftest(int fn, const double* a, const double* b, double* out, int n, cudaStream_t s);
// updateFinalVelocity.
void final_velocity(const uint8_t* in_elem, const uint8_t* has_collsn, const double4_32a* av, const int* vscene,
                    const SceneDev* scenes, double* vel, int nv, const uint8_t* mask, cudaStream_t s);

// The reference trees' leaf order on the GPU (cc_tree_gpu.cu). jobs: 3 ints
// per tree (scene, first element, elements); boxes and rank indexed by
// element. Writes each leaf's inorder rank within its tree, each tree's root
// node and root volume. scratch holds tree_scratch_bytes(ne_total), where
// ne_total bounds every tree's first element + elements.
size_t tree_scratch_bytes(long long ne_total);
void tree_order_gpu(const Box6* boxes, const int* jobs, int njobs, int max_ne, void* scratch, long long ne_total,
                    int* rank, int* root_out, double* vol_out, cudaStream_t s);

}  // namespace ccg
