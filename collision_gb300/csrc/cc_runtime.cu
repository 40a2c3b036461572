// Host runtime of the collision library: the solver object, the pass loop of
// resolveCollision (dcollid.cpp:317-362) for a batch of independent scenes,
// and the C ABI of include/collision_gb300.h.
//
// A solver holds one or more scenes. Each scene is one reference
// CollisionSolver3d: its own mesh, parameters (the reference's class
// statics), domain box, pair of trees with their shared volume, and pass
// sequence (proximity, up to five CCD passes, then impact-zone passes until
// nothing hits). All scenes advance together: every detection pass is one
// set of launches over the points and elements of all scenes that still have
// a pass to run, and each scene's state machine steps on the host from its
// own hit count. A single mesh is the one-scene case of the same code.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <queue>
#include <string>
#include <thread>
#include <vector>

#include "../../include/collision_gb300.h"
#include <sys/stat.h>

#include "cc_launch.h"
#include "cc_strain_plan.h"
#include "cc_tree_order.h"
#include "cc_vtk.h"

using namespace ccg;

namespace {

// Stages timed by cc_set_profiling / cc_get_profile.
// In mixed-precision CCD passes of the host loop, narrow_ccd is the
// per-pair FP32 filter stage and ccd_subtests the FP64 sub-tests after it.
// With profiling level 2 the loop graph's passes are split into the loop_*
// stages by boundary kernels reading the global timer (events cannot be
// recorded inside a graph's loop body).
enum Stage { kStInit, kStBoxes, kStBvh, kStTraverse, kStNarrowProx, kStNarrowCcd, kStApply, kStZone,
             kStFinalize, kStStrain, kStLoop, kStSubtests, kStLoopPlan, kStLoopBoxes, kStLoopRefit,
             kStLoopTraverse, kStLoopPruned, kStLoopFilter, kStLoopSubtests, kStLoopApply, kStLoopZoneSort,
             kStLoopZoneReplay, kStLoopZoneList, kStLoopZoneSolve, kStLoopEnd, kNumStages };
const char* kStageNames[kNumStages] = {"init", "leaf_boxes", "bvh_build", "traverse", "narrow_prox",
                                       "narrow_ccd", "apply", "zone", "finalize", "strain", "detect_loop",
                                       "ccd_subtests", "loop_plan", "loop_boxes", "loop_refit", "loop_traverse",
                                       "loop_pruned", "loop_filter", "loop_subtests", "loop_apply",
                                       "loop_zone_sort", "loop_zone_replay", "loop_zone_list", "loop_zone_solve",
                                       "loop_end"};
constexpr int kNumLoopMarks = kNumStages - kStLoopPlan;
static_assert(kNumLoopMarks <= kLoopMarkSlots, "stage mark slots");

constexpr int kMaxSceneElems = (1 << 22) - 1;  // leaf ranks fill 22 bits of a contribution key
constexpr long long kMaxTotal = 1ll << 28;     // points and elements over all scenes
constexpr int kNumCounters = 25;
constexpr int kErrIndex = kErrIndexNode | kErrIndexLeaf | kErrIndexElem;
std::string index_error(int e) {
    std::string m = "broad phase met an index out of range:";
    if (e & kErrIndexNode) m += " node";
    if (e & kErrIndexLeaf) m += " leaf";
    if (e & kErrIndexElem) m += " element";
    return m;
}

template <class T>
cudaError_t dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    return cudaMalloc((void**)p, n * sizeof(T));
}

template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

__global__ void k_reset_counters(PassCounters* c) {
    int keep = c->err & kErrNan;
    c->npairs = 0; c->ncontrib = 0; c->nhit_pairs = 0; c->nrec = 0;
    c->nvisits = 0; c->ncontacts = 0; c->nsub = 0; c->ncr = 0; c->nunion = 0; c->nsub_pt = 0; c->nsub_ee = 0; c->npairq = 0;
    c->nzones = 0; c->nmembers = 0; c->nseg = 0;
    c->err = keep;
}

// Counters and per-scene hit counts of a pass attempt.
// npairs_keep >= 0: the pair buffer holds this many pairs from an earlier
// pass that this one reuses.
__global__ void k_reset_pass(PassCounters* c, SceneRun* run, int nscenes, int npairs_keep = -1) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        int keep = c->err & kErrNan;
        c->npairs = npairs_keep >= 0 ? npairs_keep : 0; c->ncontrib = 0; c->nhit_pairs = 0; c->nrec = 0;
        c->nvisits = 0; c->ncontacts = 0; c->nsub = 0; c->ncr = 0; c->nunion = 0; c->nsub_pt = 0; c->nsub_ee = 0; c->npairq = 0;
        c->nzones = 0; c->nmembers = 0; c->nseg = 0;
        c->err = keep;
    }
    if (i < nscenes) run[i].hits = 0;
}

double dec_host(unsigned long long e) {
    unsigned long long u = (e & 0x8000000000000000ull) ? (e & 0x7fffffffffffffffull) : ~e;
    double x;
    std::memcpy(&x, &u, 8);
    return x;
}

// Runs f(0..n-1) on up to `threads` host threads.
template <class F>
void parallel_for(int n, int threads, F f) {
    if (threads > n) threads = n;
    if (threads <= 1) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    pool.reserve((size_t)threads);
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&] {
            for (int i = next++; i < n; i = next++) f(i);
        });
    for (auto& th : pool) th.join();
}

// Where a scene is in the pass sequence of resolveCollision
// (dcollid.cpp:323-356) during one call.
enum HostState { kHsDone = 0, kHsProx, kHsCcd, kHsZone };

struct SceneHost {
    int v0 = 0, nv = 0, e0 = 0, ne = 0, nt = 0;  // nt: triangles (the first nt elements)
    RefTreeOrder tree[2];  // host emulation (CC_TUNE_HOST_TREE) only
    bool built[2] = {false, false};
    double volume = 0.0;  // shared by both trees (dcollid.cpp:381, 422)
    int strain_edges = 0, strain_points = 0;
    int strain_caps[3] = {0, 0, 0};
    bool enabled = true;
    int status = CC_OK;  // of the last resolve call
    int state = kHsDone;
    int niter = 0, cd_count = 0, zone_it = 0, hcol = 0, npass = 0;
    std::vector<int> pass_kinds;
};


}  // namespace

struct cc_solver {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    // scenes
    int nscenes = 0;
    std::vector<SceneHost> scenes;
    std::vector<SceneDev> h_scenes;
    bool scenes_dirty = false;
    SceneDev* d_scenes = nullptr;
    SceneRun* d_run = nullptr;
    SceneRun* h_run = nullptr;  // pinned, nscenes
    int* d_vscene = nullptr;    // scene of every point
    int* d_escene = nullptr;    // scene of every element

    // topology of all scenes
    int nv = 0, ne = 0;
    int* d_ev = nullptr;
    int* d_esurf = nullptr;
    uint8_t* d_erigid = nullptr;
    uint8_t* d_fixed = nullptr;
    uint8_t* d_in_elem = nullptr;
    StrainEdge* d_edges = nullptr;
    int nedges = 0;
    int4* d_strain_hdr = nullptr;
    int2* d_strain_load = nullptr;
    int2* d_strain_wb = nullptr;
    void* d_strain_step = nullptr;
    int* d_strain_passes = nullptr;  // 3 per scene
    int* d_strain_flags = nullptr;   // 2 per scene
    int2* d_strain_chunks = nullptr; // (scene, first edge) per run of <= 256 edges
    int* d_strain_order = nullptr;   // scenes by strain levels, most first (one sweep CTA each)
    int n_strain_chunks = 0;
    std::vector<int> h_strain_passes;

    // state
    double4_32a* d_xo = nullptr;
    double4_32a* d_av = nullptr;
    // impact zones: the reference's union-find with member lists
    // (dcollid.cpp:1015-1059) on the device (cc_zones.cu), joined by each
    // impact-zone pass's createImpZone records in visiting order. The host
    // arrays compute the state every step starts from (makeSet and the
    // movable bodies' unions) at assembly, and read the zones back on request.
    std::vector<int> uf_root, uf_next, uf_tail, uf_w, uf_touched;
    std::vector<int> h_vscene;
    UnionRec* d_urec = nullptr;
    int urec_cap = 0;
    ZoneBufs zb;
    UfNode* d_uf0 = nullptr;  // the union-find every step starts from
    int* d_cc0 = nullptr;
    bool uf_on_device = false;  // the host arrays are stale: the device holds the last step's zones
    // staging for host-buffer calls
    double* d_xold_in = nullptr;
    double* d_xcand_in = nullptr;
    double* d_vel = nullptr;
    double* d_xout = nullptr;
    uint8_t* d_hc = nullptr;

    // pass buffers
    Box6* d_box = nullptr;
    // The proximity pass finds its pairs on swept boxes, flagging those whose
    // static boxes (d_box_st) overlap too; when it applies no impulse, the
    // first CCD pass over the same scenes reuses the list as it is.
    Box6* d_box_st = nullptr;
    bool combined_broad = true;
    bool reuse_pairs = false;
    int reuse_npairs = 0;
    std::vector<int> reuse_set;
    BvhBufs bvh{};
    int2* d_pairs = nullptr;
    int* d_pair_hit = nullptr;  // hit flag per candidate pair (split passes)
    int* d_pairq = nullptr;     // pairs with queued sub-tests (split passes)
    int pair_cap = 0;
    SubRec* d_sub_pt = nullptr;
    SubRec* d_sub_ee = nullptr;
    int sub_cap = 0;
    Contrib* d_contrib = nullptr;
    int contrib_cap = 0;
    ApplyBufs apply{};

    // movable rigid bodies: one per surface of movable points
    // (createImpZoneForRG, dcollid3d.cpp:54-68), all scenes in one list
    struct BodyHost {
        int scene, surf;
        double mass = 1.0;
        double com[3] = {0.0, 0.0, 0.0}, comv[3] = {0.0, 0.0, 0.0};  // HYPER_SURF
        double mrg_com[3] = {0.0, 0.0, 0.0};                           // CollisionSolver::mrg_com
        bool mrg_set = false;
    };
    std::vector<BodyHost> bodies;
    std::vector<int> body_unions;  // createImpZoneForRG triangles, 3 points each, in order
    std::vector<int> h_body_visit, h_body_visit_off;
    std::vector<double4_32a> h_body_out;
    std::vector<uint8_t> h_fixed;
    int* d_vbody = nullptr;
    double* d_body_mass = nullptr;
    int* d_body_members = nullptr;
    int* d_body_member_body = nullptr;
    int* d_body_zone_off = nullptr;
    int* d_body_visit = nullptr;
    int* d_body_visit_off = nullptr;
    double4_32a* d_body_acc = nullptr;
    int* d_body_num = nullptr;
    double4_32a* d_body_out = nullptr;
    BodyBufs body_bufs;
    int find_body(int scene, int surf) const {
        for (size_t b = 0; b < bodies.size(); ++b)
            if (bodies[b].scene == scene && bodies[b].surf == surf) return (int)b;
        return -1;
    }
    void upload_body_mass() {
        if (bodies.empty()) return;
        std::vector<double> m(bodies.size());
        for (size_t b = 0; b < bodies.size(); ++b) m[b] = bodies[b].mass;
        cudaMemcpy(d_body_mass, m.data(), sizeof(double) * m.size(), cudaMemcpyHostToDevice);
    }
    PassCounters* d_ctr = nullptr;
    PassCounters* h_ctr = nullptr;
    unsigned long long* h_bbox = nullptr;  // pinned, 6 per scene
    int* d_rank[2] = {nullptr, nullptr};
    std::vector<Box6> h_boxes;
    std::vector<int> h_rank;
    float4* d_pbox_lo = nullptr;
    float4* d_pbox_hi = nullptr;
    float4* d_p32 = nullptr;
    float4* d_v32 = nullptr;
    // the scenes of a pass, when not all of them have one: their elements
    // and points (expanded on the device from per-scene ranges)
    int* d_act_e = nullptr;
    int* d_act_p = nullptr;
    int* d_sel = nullptr;        // 3 * nscenes: scene ids, element offsets, point offsets
    int* h_sel = nullptr;        // pinned staging of d_sel
    std::vector<int> sel_prev;   // scene ids of the last expanded selection
    int n_act_e = 0, n_act_p = 0;
    // the LBVH built this step and for which scenes: later passes of the
    // step over the same scenes refit it instead of building anew
    bool bvh_this_step = false;
    std::vector<int> bvh_set, cur_set;
    // the LBVH in bvh was built this step over all elements; with
    // subset_refit, later passes over some of the scenes refit it over those
    // scenes' leaves instead of building their own
    bool full_this_step = false;
    bool subset_refit = true;
    // The hierarchy over all elements, restricted to the scenes of this pass:
    // scene s's sorted leaves there are its element range [e0, e0 + ne), so
    // the pass's element list doubles as its list of leaves.
    BvhBufs full_view() const {
        BvhBufs f = bvh;
        f.n = ne;
        f.act = nullptr;
        f.sub = bvh.act;
        f.nsub = bvh.n;
        return f;
    }

    // The device-resident detection loop (cc_loop.cu): every scene's pass
    // sequence and the loop's state on the device, the passes after the
    // proximity pass in one graph with a WHILE node
    bool device_loop = true;
    bool prune = true;  // the device loop's later passes test only touched pairs
    SceneCtl* d_ctl = nullptr;
    SceneCtl* h_ctl = nullptr;  // pinned, nscenes
    LoopCtl* d_loop = nullptr;
    LoopCtl* h_loop = nullptr;  // pinned
    int* d_lsel = nullptr;      // 3 * (nscenes + 1): the pass's scenes, element and point offsets
    int* d_act_l = nullptr;     // the pass's sorted leaves
    int* d_rebuild = nullptr;   // per scene: tree to rebuild on the host (0 none, 1 proximity, 2 collision)
    int* h_rebuild = nullptr;   // pinned
    unsigned* d_pstamp = nullptr;  // per point: serial of the last pass that touched it
    uint8_t* d_edirty = nullptr;   // per element: a point touched by the previous pass
    int* d_query = nullptr;        // the pruned traversal's queries
    unsigned serial_base = 1;      // the next step's proximity pass serial
    PassStamp loop_stamp() const { return PassStamp{d_pstamp, &d_loop->serial}; }
    double* d_tree_vol = nullptr;  // per scene: the volume both trees share
    int* d_tree_built = nullptr;   // 2 * nscenes: tree built (proximity, then collision)
    // reference tree order built on the GPU (cc_tree_gpu.cu)
    bool host_tree = false;          // CC_TUNE_HOST_TREE: emulate the insertions on host threads instead
    bool pruned_warp = true;         // CC_TUNE_PRUNED_WARP: one warp per pruned query
    bool refit_up = true;            // CC_TUNE_REFIT_UP: the refit walk with one arrival per level
    bool robust_roots = true;        // CC_TUNE_ROBUST_ROOTS: correctly rounded roots only where decisive
    bool sub_merge = true;           // CC_TUNE_SUBTEST_MERGE: both sub-test lists in one launch
    void* d_tree_scratch = nullptr;  // nodes, parent links and leaf counts of the trees being built
    int* d_tree_jobs = nullptr;      // 3 per tree: scene, first element, elements
    int* h_tree_jobs = nullptr;      // pinned
    int* d_tree_root = nullptr;
    double* d_tree_vol_out = nullptr;
    double* h_tree_vol_out = nullptr;  // pinned
    cc_status build_trees(int which, std::vector<int>& ids, const Box6* boxes);
    cudaStream_t cap_stream = nullptr, cap_stream2 = nullptr, cap_stream3 = nullptr;  // graph capture only
    // One graph per arithmetic mode, each valid while the buffers and
    // settings it holds stand (gen) and for the hierarchy size it was built
    // for, so that alternating modes does not rebuild it.
    struct LoopGraph {
        cudaGraphExec_t exec = nullptr;
        unsigned gen = 0;
        int key_n = -1;
        long long body_launches = 0, zone_launches = 0;
    };
    LoopGraph loop_graphs[2];
    unsigned loop_gen = 1;   // bumped whenever a buffer or setting a graph holds changes
    bool loop_dirty = false; // set by the code that changes one; folded into loop_gen
    void clear_loop_graph() {
        for (auto& lg : loop_graphs) {
            if (lg.exec) cudaGraphExecDestroy(lg.exec);
            lg = LoopGraph{};
        }
        ++loop_gen;
        loop_dirty = false;
    }
    LoopGraph* current_loop_graph(int n_hier) {
        if (loop_dirty) {
            ++loop_gen;
            loop_dirty = false;
        }
        LoopGraph& lg = loop_graphs[mode];
        return (lg.exec && lg.gen == loop_gen && lg.key_n == n_hier) ? &lg : nullptr;
    }
    bool use_device_loop() const { return device_loop && !record && vtk_dir.empty() && !overlap_tails; }
    NarrowArgs narrow_args(int moving, bool combined) const {
        NarrowArgs a{};
        a.robust_roots = robust_roots ? 1 : 0;
        a.sub_merge = sub_merge ? 1 : 0;
        a.xo = d_xo; a.av = d_av; a.fixed = d_fixed; a.ev = d_ev; a.esurf = d_esurf; a.erigid = d_erigid;
        a.vbody = d_vbody; a.body_mass = d_body_mass; a.body_slot0 = nv;
        a.rank = d_rank[moving]; a.escene = d_escene; a.scenes = d_scenes; a.run = d_run;
        a.pairs = d_pairs; a.contrib = d_contrib; a.contrib_cap = contrib_cap; a.ctr = d_ctr;
        a.urec = d_urec; a.urec_cap = urec_cap;
        a.rec = nullptr; a.rec_cap = 0;
        a.pbox_lo = mode == 1 ? d_pbox_lo : nullptr;
        a.pbox_hi = mode == 1 ? d_pbox_hi : nullptr;
        a.p32 = d_p32; a.v32 = d_v32;
        a.check = 0;
        a.sub_pt = d_sub_pt; a.sub_ee = d_sub_ee; a.sub_cap = sub_cap;
        a.pair_hit = d_pair_hit; a.pairq = d_pairq;
        a.static_only = combined ? 1 : 0;
        return a;
    }
    void prox_pass_async();
    cc_status build_loop_graph(int n_hier);
    // CC_PASS_LOG with profiling level 2: the loop passes of the last step,
    // one line each (stage times in microseconds, then the pass's counts)
    void print_pass_log() {
        std::vector<unsigned long long> h(kMarkWords);
        cudaMemcpyAsync(h.data(), d_marks, sizeof(unsigned long long) * kMarkWords, cudaMemcpyDeviceToHost, stream);
        if (cudaStreamSynchronize(stream) != cudaSuccess) return;
        const unsigned long long rows = h[1 + 2 * kLoopMarkSlots];
        const unsigned long long* log = h.data() + 2 + 2 * kLoopMarkSlots;
        const unsigned long long n = rows < (unsigned long long)kPassLogRows ? rows : kPassLogRows;
        for (unsigned long long r = 0; r < n; ++r) {
            const unsigned long long* row = log + r * kPassLogCols;
            std::string line = "cc_loop_pass " + std::to_string(r);
            for (int k = 0; k < kNumLoopMarks; ++k)
                line += " " + std::string(kStageNames[kStLoopPlan + k] + 5) + "=" +
                        std::to_string(row[k] / 1000.0).substr(0, 7);
            line += " pairs=" + std::to_string(row[kLoopMarkSlots]) + " sub_pt=" +
                    std::to_string(row[kLoopMarkSlots + 1]) + " sub_ee=" + std::to_string(row[kLoopMarkSlots + 2]) +
                    " unions=" + std::to_string(row[kLoopMarkSlots + 3]) + " queries=" +
                    std::to_string((long long)(int)row[kLoopMarkSlots + 4]);
            std::fprintf(stderr, "%s\n", line.c_str());
        }
    }
    cc_status device_passes(std::string& capped);
    cc_status rebuild_flagged();

    // VTK dumps of every pass (empty: off)
    std::string vtk_dir;
    std::vector<int> vtk_count, h_ev;
    double4_32a* d_dump = nullptr;
    double4_32a* d_av_pre = nullptr;

    // recording
    bool record = false;
    VisitRec* d_rec = nullptr;
    int rec_cap = 0;
    std::vector<VisitRec> visits;

    cc_params prm{1e-3, 1e-4, 1e-6, 1000.0, 0.01, 0.02, 0.0};  // for scenes assembled later
    double lo[3] = {-1e30, -1e30, -1e30}, hi[3] = {1e30, 1e30, 1e30};
    long long counters[kNumCounters] = {0};
    bool own_stream = true;
    long long launches_last = 0;
    int zone_cap = 10000;
    int mode = 0;  // 0 plain FP64, 1 mixed precision
    bool strain_window = true;
    bool split_narrow = true;  // two-stage narrow phase for mixed passes
    bool strain_warp = false;  // one-warp strain sweep with staged levels
    bool strain_roles = true;  // window sweep: edges, copy-ins and write-backs on separate threads
    LaunchTuning tune;
    int host_threads = 0;  // tree emulation threads (0: hardware concurrency)
    const bool pass_log = std::getenv("CC_PASS_LOG") != nullptr;

    // per-stage GPU time, measured with events on the solver's stream
    bool profiling = false;
    bool loop_marks = false;                   // profiling level 2: stage marks inside the loop graph
    unsigned long long* d_marks = nullptr;     // kMarkWords (stage_mark)
    void mark(int slot, cudaStream_t on) {
        if (loop_marks && d_marks) stage_mark(d_marks, slot, on);
    }
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, int>> ev_marks;  // (stage, event index of its start; end = start+1)
    double stage_ms[kNumStages] = {0};
    long long stage_calls[kNumStages] = {0};
    void prof(int stage, bool begin) { prof_on(stage, begin, stream); }
    void prof_on(int stage, bool begin, cudaStream_t on) {
        if (!profiling) return;
        size_t need = ev_marks.size() * 2 + 2;
        while (ev_pool.size() < need) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev_pool.push_back(e);
        }
        if (begin) {
            ev_marks.push_back({stage, (int)(ev_marks.size() * 2)});
            cudaEventRecord(ev_pool[ev_marks.back().second], on);
        } else {
            cudaEventRecord(ev_pool[ev_marks.back().second + 1], on);
        }
    }
    void prof_collect() {
        if (!profiling) return;
        for (auto& m : ev_marks) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ev_pool[m.second], ev_pool[m.second + 1]) == cudaSuccess) {
                stage_ms[m.first] += ms;
                stage_calls[m.first]++;
            }
        }
        ev_marks.clear();
    }

    ~cc_solver() { release(); }

    void release_mesh() {
        clear_tail_graphs();
        dfree(d_ev); dfree(d_esurf); dfree(d_erigid); dfree(d_fixed); dfree(d_in_elem); dfree(d_edges);
        dfree(d_strain_hdr); dfree(d_strain_load); dfree(d_strain_wb); dfree(d_strain_passes);
        dfree(d_strain_flags); dfree(d_strain_chunks); dfree(d_strain_order);
        n_strain_chunks = 0;
        if (d_strain_step) cudaFree(d_strain_step);
        d_strain_step = nullptr;
        dfree(d_scenes); dfree(d_run); dfree(d_vscene); dfree(d_escene); dfree(d_tail_mask);
        if (h_tail_masks) cudaFreeHost(h_tail_masks);
        h_tail_masks = nullptr;
        if (h_run) cudaFreeHost(h_run);
        h_run = nullptr;
        if (h_bbox) cudaFreeHost(h_bbox);
        h_bbox = nullptr;
        dfree(d_xo); dfree(d_av);
        dfree(d_urec);
        urec_cap = 0;
        dfree(zb.keys); dfree(zb.vals); dfree(zb.seg); dfree(zb.noop); dfree(zb.cc); dfree(zb.uf); dfree(zb.zone_rng);
        dfree(zb.zone_root); dfree(zb.members); dfree(d_uf0); dfree(d_cc0);
        dfree(zb.prev_members); dfree(zb.prev_off); dfree(zb.prev_len); dfree(zb.prev_epoch); dfree(zb.epoch);
        if (zb.sort_temp) cudaFree(zb.sort_temp);
        const bool small_sort = zb.small_sort;  // settings, not buffers
        const int zone_cta_min = zb.zone_cta_min, replay_cta_min = zb.replay_cta_min, zone_few = zb.zone_few;
        zb = ZoneBufs{};
        zb.small_sort = small_sort;
        zb.zone_cta_min = zone_cta_min;
        zb.zone_few = zone_few;
        zb.replay_cta_min = replay_cta_min;
        uf_on_device = false;
        dfree(d_xold_in); dfree(d_xcand_in); dfree(d_vel); dfree(d_xout); dfree(d_hc);
        dfree(d_box); dfree(d_box_st); dfree(bvh.keys); dfree(bvh.order); dfree(bvh.range_hi);
        dfree(bvh.range_lo); dfree(bvh.parent); dfree(bvh.flags); dfree(bvh.node); dfree(bvh.bbox_enc); dfree(bvh.leaf);
        dfree(bvh.rnode); dfree(bvh.rope); dfree(bvh.leaf32); dfree(bvh.qnext);
        if (bvh.sort_temp) cudaFree(bvh.sort_temp);
        bvh = BvhBufs{};
        dfree(d_pairs); dfree(d_contrib); dfree(d_pair_hit); dfree(d_pairq); dfree(d_sub_pt); dfree(d_sub_ee);
        sub_cap = 0;
        dfree(apply.cnt); dfree(apply.off); dfree(apply.cur); dfree(apply.idx);
        if (apply.scan_temp) cudaFree(apply.scan_temp);
        apply.scan_temp = nullptr;
        dfree(d_rank[0]); dfree(d_rank[1]);
        dfree(d_rec); dfree(d_pbox_lo); dfree(d_pbox_hi); dfree(d_p32); dfree(d_v32);
        dfree(d_act_e); dfree(d_act_p); dfree(d_sel); dfree(d_dump); dfree(d_av_pre);
        clear_loop_graph();
        dfree(d_pstamp); dfree(d_edirty); dfree(d_query);
        dfree(d_ctl); dfree(d_loop); dfree(d_lsel); dfree(d_act_l); dfree(d_rebuild); dfree(d_tree_vol);
        dfree(d_tree_built);
        if (d_tree_scratch) cudaFree(d_tree_scratch);
        d_tree_scratch = nullptr;
        dfree(d_tree_jobs); dfree(d_tree_root); dfree(d_tree_vol_out);
        if (h_tree_jobs) cudaFreeHost(h_tree_jobs);
        if (h_tree_vol_out) cudaFreeHost(h_tree_vol_out);
        h_tree_jobs = nullptr;
        h_tree_vol_out = nullptr;
        if (h_ctl) cudaFreeHost(h_ctl);
        if (h_loop) cudaFreeHost(h_loop);
        if (h_rebuild) cudaFreeHost(h_rebuild);
        h_ctl = nullptr;
        h_loop = nullptr;
        h_rebuild = nullptr;
        dfree(d_vbody); dfree(d_body_mass); dfree(d_body_members); dfree(d_body_member_body);
        dfree(d_body_zone_off); dfree(d_body_visit); dfree(d_body_visit_off); dfree(d_body_acc);
        dfree(d_body_num); dfree(d_body_out);
        bodies.clear();
        body_unions.clear();
        body_bufs = BodyBufs{};
        if (h_sel) cudaFreeHost(h_sel);
        h_sel = nullptr;
        sel_prev.clear();
        pair_cap = contrib_cap = rec_cap = 0;
        nv = ne = nedges = 0;
        nscenes = 0;
        scenes.clear();
        h_scenes.clear();
    }

    void release() {
        if (device >= 0) cudaSetDevice(device);
        release_mesh();
        dfree(d_ctr);
        dfree(d_marks);
        if (h_ctr) cudaFreeHost(h_ctr);
        h_ctr = nullptr;
        for (auto e : ev_pool) cudaEventDestroy(e);
        ev_pool.clear();
        if (ev_pass) cudaEventDestroy(ev_pass);
        if (ev_tail) cudaEventDestroy(ev_tail);
        ev_pass = ev_tail = nullptr;
        if (tail_stream) cudaStreamDestroy(tail_stream);
        tail_stream = nullptr;
        if (cap_stream) cudaStreamDestroy(cap_stream);
        if (cap_stream2) cudaStreamDestroy(cap_stream2);
        if (cap_stream3) cudaStreamDestroy(cap_stream3);
        cap_stream = cap_stream2 = cap_stream3 = nullptr;
        if (stream && own_stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }

    cc_status fail(cc_status st, const std::string& msg) {
        err = msg;
        return st;
    }
    cc_status cuda_check(const char* where) {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return fail(CC_CUDA_ERROR, std::string(where) + ": " + cudaGetErrorString(e));
        return CC_OK;
    }

    cc_status grow_pairs(int cap) {
        loop_dirty = true;
        dfree(d_pairs);
        dfree(d_pair_hit);
        dfree(d_pairq);
        if (dalloc(&d_pairs, (size_t)cap) != cudaSuccess || dalloc(&d_pair_hit, (size_t)cap) != cudaSuccess ||
            dalloc(&d_pairq, (size_t)cap) != cudaSuccess)
            return fail(CC_NO_MEMORY, "pair buffer");
        pair_cap = cap;
        if (record) {
            dfree(d_rec);
            if (dalloc(&d_rec, (size_t)cap) != cudaSuccess) return fail(CC_NO_MEMORY, "record buffer");
            rec_cap = cap;
        }
        return CC_OK;
    }
    cc_status grow_contrib(int cap) {
        loop_dirty = true;
        dfree(d_contrib);
        dfree(apply.idx);
        if (dalloc(&d_contrib, (size_t)cap) != cudaSuccess || dalloc(&apply.idx, (size_t)cap) != cudaSuccess)
            return fail(CC_NO_MEMORY, "contribution buffer");
        contrib_cap = cap;
        return CC_OK;
    }

    cc_status grow_subs(int cap) {
        loop_dirty = true;
        dfree(d_sub_pt);
        dfree(d_sub_ee);
        if (dalloc(&d_sub_pt, (size_t)cap) != cudaSuccess || dalloc(&d_sub_ee, (size_t)cap) != cudaSuccess)
            return fail(CC_NO_MEMORY, "sub-test queues");
        sub_cap = cap;
        return CC_OK;
    }
    cc_status grow_unions(int cap) {
        loop_dirty = true;
        dfree(d_urec);
        dfree(zb.keys);
        dfree(zb.vals);
        dfree(zb.seg);
        dfree(zb.noop);
        if (zb.sort_temp) cudaFree(zb.sort_temp);
        zb.sort_temp = nullptr;
        if (dalloc(&d_urec, (size_t)cap) != cudaSuccess || dalloc(&zb.keys, (size_t)cap) != cudaSuccess ||
            dalloc(&zb.vals, (size_t)cap) != cudaSuccess || dalloc(&zb.seg, (size_t)cap) != cudaSuccess ||
            dalloc(&zb.noop, (size_t)cap) != cudaSuccess ||
            cudaMalloc(&zb.sort_temp, zone_sort_temp_bytes(cap)) != cudaSuccess)
            return fail(CC_NO_MEMORY, "union record buffer");
        urec_cap = cap;
        zb.cap = cap;
        zb.rec = d_urec;
        return CC_OK;
    }
    // The device union-find as every step starts it.
    void start_zones() {
        if (nv == 0) return;
        cudaMemcpyAsync(zb.uf, d_uf0, sizeof(UfNode) * (size_t)nv, cudaMemcpyDeviceToDevice, stream);
        cudaMemcpyAsync(zb.cc, d_cc0, sizeof(int) * (size_t)nv, cudaMemcpyDeviceToDevice, stream);
        // the lists of the last step's zones no longer hold
        if (zb.prev_epoch) cudaMemsetAsync(zb.prev_epoch, 0xff, sizeof(unsigned) * (size_t)nv, stream);
        uf_on_device = true;
    }
    // The zone root of every point after the last step.
    cc_status zone_roots(int* out) {
        if (!uf_on_device) {
            for (int i = 0; i < nv; ++i) out[i] = find_set(i);
            return CC_OK;
        }
        std::vector<UfNode> u((size_t)nv);
        if (nv && cudaMemcpyAsync(u.data(), zb.uf, sizeof(UfNode) * (size_t)nv, cudaMemcpyDeviceToHost, stream) !=
                      cudaSuccess)
            return cuda_check("zone roots");
        if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("zone roots");
        for (int i = 0; i < nv; ++i) {
            int r = i;
            for (int k = 0; u[r].root != r && k <= nv; ++k) r = u[r].root;
            out[i] = r;
        }
        return CC_OK;
    }

    // makeSet for every point (dcollid.cpp:1015-1022), undoing the last
    // step's unions, then createImpZoneForRG: each movable surface's
    // triangles in order, createImpZone(pts, 3, YES) (dcollid3d.cpp:54-68).
    void reset_zones() {
        for (int p : uf_touched) {
            uf_root[p] = uf_tail[p] = p;
            uf_next[p] = -1;
            uf_w[p] = 1;
        }
        uf_touched.clear();
        for (size_t i = 0; i < body_unions.size(); i += 3) {
            const int* t = &body_unions[i];
            for (int a = 0; a < 3; ++a) uf_touched.push_back(t[a]);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < a; ++b) merge_point(t[a], t[b]);
        }
    }
    // findSet (dcollid.cpp:1024-1031) with path compression.
    int find_set(int p) {
        int r = p;
        while (uf_root[r] != r) r = uf_root[r];
        while (uf_root[p] != r) {
            int n = uf_root[p];
            uf_root[p] = r;
            p = n;
        }
        return r;
    }
    // mergePoint (dcollid.cpp:1033-1059): the lighter set joins the heavier
    // one (the second on equal weights) and its member list is appended.
    void merge_point(int x, int y) {
        int px = find_set(x), py = find_set(y);
        if (px == py) return;
        if (uf_w[px] > uf_w[py]) std::swap(px, py);
        // px joins py
        uf_w[py] += uf_w[px];
        uf_root[px] = py;
        uf_next[uf_tail[py]] = px;
        uf_tail[py] = uf_tail[px];
    }

    // One .vtp per scene of the pass just applied (cc_vtk.cpp).
    cc_status write_vtk_pass() {
        std::vector<double4_32a> xo((size_t)nv), av((size_t)nv), dump((size_t)nv);
        cudaMemcpyAsync(xo.data(), d_xo, sizeof(double4_32a) * (size_t)nv, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(av.data(), d_av_pre, sizeof(double4_32a) * (size_t)nv, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(dump.data(), d_dump, sizeof(double4_32a) * (size_t)nv, cudaMemcpyDeviceToHost, stream);
        if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("vtk dump");
        std::vector<double> pos((size_t)nv * 3), imp((size_t)nv * 3), num((size_t)nv);
        for (int p = 0; p < nv; ++p) {
            double dt = h_scenes[h_vscene[p]].p.dt;  // updateFinalPosition before the impulses
            pos[3 * p] = xo[p].x + dt * av[p].x;
            pos[3 * p + 1] = xo[p].y + dt * av[p].y;
            pos[3 * p + 2] = xo[p].z + dt * av[p].z;
            imp[3 * p] = dump[p].x;
            imp[3 * p + 1] = dump[p].y;
            imp[3 * p + 2] = dump[p].z;
            num[p] = dump[p].w;
        }
        for (int s = 0; s < nscenes; ++s) {
            if (h_run[s].mode == kSceneIdle || scenes[s].ne == 0) continue;
            char name[64];
            if (nscenes == 1)
                std::snprintf(name, sizeof(name), "/surf-%03d.vtp", vtk_count[s]++);
            else
                std::snprintf(name, sizeof(name), "/surf-s%03d-%03d.vtp", s, vtk_count[s]++);
            std::string path = vtk_dir + name;
            if (!write_vtp(path.c_str(), scenes[s].ne, h_ev.data() + 3 * (size_t)scenes[s].e0, pos.data(), imp.data(),
                           num.data()))
                return fail(CC_BAD_INPUT, "cannot write " + path);
        }
        return CC_OK;
    }

    // The end of a step of the scenes in d_tail_mask: final positions,
    // strain limiting and final velocities, on the tail stream.
    void tail(const double* x_cand, double* x_out, double* vel) {
        finalize_positions(d_in_elem, d_xo, d_av, d_hc, x_cand, x_out, nv, d_vscene, d_scenes, d_fixed, d_tail_mask,
                           tail_stream);
        strain_limit(d_edges, nedges, d_strain_hdr, d_strain_load, d_strain_wb, d_strain_chunks, n_strain_chunks,
                     d_scenes, nscenes, strain_plan(), d_xo, d_av, d_strain_step, d_strain_flags, d_strain_passes,
                     d_tail_mask, tail_stream);
        final_velocity(d_in_elem, d_hc, d_av, d_vscene, d_scenes, vel, nv, d_tail_mask, tail_stream);
    }
    // Tail streams: the ends of steps of the scenes that have finished their
    // detection passes run there while the other scenes' passes go on (a
    // scene's end of step reads and writes only its own points).
    cudaStream_t tail_stream = nullptr;
    cudaEvent_t ev_pass = nullptr, ev_tail = nullptr;
    uint8_t* d_tail_mask = nullptr;
    uint8_t* h_tail_masks = nullptr;  // pinned, two masks: a step runs at most two tails
    int tails_this_step = 0;
    std::vector<uint8_t> tail_done;
    bool overlap_tails = false;
    // Ends the step of every finished scene without one yet (all: every
    // scene), after the main stream's work so far.
    cc_status launch_tail(const double* x_cand, double* x_out, double* vel, bool all) {
        std::vector<int> ids;
        for (int s = 0; s < nscenes; ++s)
            if (!tail_done[s] && (all || scenes[s].state == kHsDone)) ids.push_back(s);
        if (ids.empty()) return CC_OK;
        // besides the last, one early end of step, once at least half the
        // scenes have finished (each one runs the whole tail's launches)
        if (!all && (tails_this_step > 0 || 2 * (int)ids.size() < nscenes)) return CC_OK;
        // at most one early tail, then the last: each has its own mask, whose
        // copy may still be in flight when the next is written
        uint8_t* m = h_tail_masks + (size_t)(tails_this_step % 2) * (size_t)nscenes;
        tails_this_step++;
        std::memset(m, 0, (size_t)nscenes);
        for (int s : ids) {
            m[s] = 1;
            tail_done[s] = 1;
        }
        cudaEventRecord(ev_pass, stream);
        cudaStreamWaitEvent(tail_stream, ev_pass, 0);
        cudaMemcpyAsync(d_tail_mask, m, (size_t)nscenes, cudaMemcpyHostToDevice, tail_stream);
        prof_on(kStStrain, true, tail_stream);
        if (tail_graphs_on) {
            cc_status st = run_tail_graph(x_cand, x_out, vel);
            if (st) return st;
        } else {
            tail(x_cand, x_out, vel);
        }
        prof_on(kStStrain, false, tail_stream);
        return CC_OK;
    }
    // The whole end of a step captured once per set of caller pointers and
    // strain settings, then replayed.
    struct TailGraph {
        const void* key[4];
        int block, window, warp, roles;
        cudaGraphExec_t exec;
        long long launches;
    };
    std::vector<TailGraph> tail_graphs;
    bool tail_graphs_on = true;
    void clear_tail_graphs() {
        for (auto& g : tail_graphs) cudaGraphExecDestroy(g.exec);
        tail_graphs.clear();
    }
    cc_status run_tail_graph(const double* x_cand, double* x_out, double* vel) {
        const void* key[4] = {x_cand, x_out, vel, nullptr};
        TailGraph* hit = nullptr;
        for (auto& g : tail_graphs)
            if (std::equal(key, key + 4, g.key) && g.block == tune.strain_block && g.window == (int)strain_window &&
                g.warp == (int)strain_warp && g.roles == (int)strain_roles) {
                hit = &g;
                break;
            }
        if (!hit) {
            if (tail_graphs.size() >= 4) {
                cudaGraphExecDestroy(tail_graphs.front().exec);
                tail_graphs.erase(tail_graphs.begin());
            }
            cudaGraph_t g = nullptr;
            long long l0 = g_kernel_launches;
            if (cudaStreamBeginCapture(tail_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                return cuda_check("tail capture");
            tail(x_cand, x_out, vel);
            cudaError_t e = cudaStreamEndCapture(tail_stream, &g);
            long long n = g_kernel_launches - l0;
            g_kernel_launches = l0;
            if (e != cudaSuccess || !g) return fail(CC_CUDA_ERROR, std::string("tail capture: ") + cudaGetErrorString(e));
            TailGraph tg;
            std::copy(key, key + 4, tg.key);
            tg.block = tune.strain_block;
            tg.window = (int)strain_window;
            tg.warp = (int)strain_warp;
            tg.roles = (int)strain_roles;
            tg.launches = n;
            e = cudaGraphInstantiate(&tg.exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail(CC_CUDA_ERROR, std::string("tail graph: ") + cudaGetErrorString(e));
            tail_graphs.push_back(tg);
            hit = &tail_graphs.back();
        }
        if (cudaGraphLaunch(hit->exec, tail_stream) != cudaSuccess) return cuda_check("tail graph launch");
        count_launch((int)hit->launches);
        return CC_OK;
    }
    // Elements and points of the scenes whose h_run mode is not idle, and
    // each one's first leaf in the pass's hierarchy (sets h_run[].leaf0 and
    // bvh.n / bvh.act; the lists are rebuilt only when the set changes).
    void select_active() {
        std::vector<int>& ids = cur_set;
        ids.clear();
        int with_elems = 0;
        int ae = 0, ap = 0;
        for (int s = 0; s < nscenes; ++s) {
            if (scenes[s].ne > 0) ++with_elems;
            if (h_run[s].mode == kSceneIdle) {
                h_run[s].leaf0 = -1;
                continue;
            }
            h_run[s].leaf0 = ae;
            ids.push_back(s);
            ae += scenes[s].ne;
            ap += scenes[s].nv;
        }
        if ((int)ids.size() == with_elems) {  // every scene: no lists needed
            bvh.act = nullptr;
            bvh.n = ne;
            n_act_e = ne;
            n_act_p = nv;
            return;
        }
        bvh.act = d_act_e;
        bvh.n = ae;
        n_act_e = ae;
        n_act_p = ap;
        if (ids == sel_prev) return;
        int k = (int)ids.size();
        int* eoff = h_sel + k;
        int* poff = h_sel + 2 * k + 1;
        int e = 0, p = 0;
        for (int j = 0; j < k; ++j) {
            h_sel[j] = ids[j];
            eoff[j] = e;
            poff[j] = p;
            e += scenes[ids[j]].ne;
            p += scenes[ids[j]].nv;
        }
        eoff[k] = e;
        poff[k] = p;
        cudaMemcpyAsync(d_sel, h_sel, sizeof(int) * (3 * (size_t)k + 2), cudaMemcpyHostToDevice, stream);
        expand_scenes(d_sel, d_sel + k, d_sel + 2 * k + 1, k, ae, ap, d_scenes, d_act_e, d_act_p, stream);
        sel_prev = ids;
    }

    StrainPlan strain_plan() const {
        StrainPlan pl{strain_window, 0, false, tune.strain_block, false, 0, 0, 0, 0, d_strain_order};
        int cap = strain_window_slot_cap();
        for (int s = 0; s < nscenes; ++s) {
            const SceneDev& sd = h_scenes[s];
            if (strain_window && sd.strain_slots <= cap) {
                pl.max_window_slots = std::max(pl.max_window_slots, sd.strain_slots);
                pl.ecap = std::max(pl.ecap, scenes[s].strain_caps[0]);
                pl.lcap = std::max(pl.lcap, scenes[s].strain_caps[1]);
                pl.wcap = std::max(pl.wcap, scenes[s].strain_caps[2]);
            } else {
                pl.any_global = true;
            }
        }
        pl.warp_smem = strain_warp_smem(pl.max_window_slots, pl.ecap, pl.lcap, pl.wcap);
        // separate threads for a level's edges, copy-ins and write-backs,
        // each role from a warp boundary, where they fit in the block
        pl.cbase = pl.wbase = 0;
        if (strain_roles) {
            const int cb = (pl.ecap + 31) / 32 * 32, wb = cb + (pl.lcap + 31) / 32 * 32;
            if (pl.ecap > 0 && wb + pl.wcap <= pl.block) {
                pl.cbase = cb;
                pl.wbase = wb;
            }
        }
        pl.warp = strain_window && strain_warp && pl.warp_smem <= 200 * 1024;
        return pl;
    }
    void set_scene_params(int i, const cc_params& p) {
        h_scenes[i].p = Params{p.dt, p.thickness, p.eps, p.k, p.m, p.lambda, p.cr};
        scenes_dirty = true;
    }
    void set_scene_domain(int i, const double* l, const double* h) {
        for (int d = 0; d < 3; ++d) {
            h_scenes[i].lo[d] = l[d];
            h_scenes[i].hi[d] = h[d];
        }
        scenes_dirty = true;
    }
    void upload_scenes() {
        if (!scenes_dirty || nscenes == 0) return;
        cudaMemcpyAsync(d_scenes, h_scenes.data(), sizeof(SceneDev) * (size_t)nscenes, cudaMemcpyHostToDevice, stream);
        cudaStreamSynchronize(stream);  // h_scenes is pageable and may change after return
        scenes_dirty = false;
    }

    cc_status assemble(const cc_mesh* meshes, int n);
    cc_status resolve(const double* x_old, const double* x_cand, double* vel, uint8_t* hc, double* x_out,
                      int* has_collision);
    cc_status resolve_impl(const double* x_old, const double* x_cand, double* vel, uint8_t* hc, double* x_out,
                           int* has_collision);
    cc_status detect_pass(int moving, bool any_zone);
    cc_status check_ccd(const double* x_old, const double* x_new, long long* hits, int* scene_hits);
    cc_status autotune(double* best_ms);
    cc_status update_trees(int which, const Box6* boxes);
    void sync_tree_state(const std::vector<int>& ids, int which);
    std::vector<double> h_tree_vol_stage;
};

cc_status cc_solver::assemble(const cc_mesh* meshes, int n) {
    if (!meshes || n <= 0) return fail(CC_BAD_INPUT, "no meshes");
    long long tot_v = 0, tot_e = 0;
    for (int i = 0; i < n; ++i) {
        const cc_mesh* m = &meshes[i];
        if (m->n_points < 0 || m->n_tris < 0 || m->n_bonds < 0) return fail(CC_BAD_INPUT, "bad mesh sizes");
        if ((m->n_tris && (!m->tris || !m->tri_rest_len)) || (m->n_bonds && (!m->bonds || !m->bond_rest_len)))
            return fail(CC_BAD_INPUT, "missing element arrays");
        long long ne_s = (long long)m->n_tris + m->n_bonds;
        if (ne_s > kMaxSceneElems) return fail(CC_BAD_INPUT, "more than 2^22-1 elements in one scene");
        tot_v += m->n_points;
        tot_e += ne_s;
    }
    if (tot_v >= kMaxTotal || tot_e >= kMaxTotal) return fail(CC_BAD_INPUT, "more than 2^28 points or elements");
    cudaSetDevice(device);
    release_mesh();
    nscenes = n;
    nv = (int)tot_v;
    ne = (int)tot_e;
    scenes.resize((size_t)n);
    h_scenes.assign((size_t)n, SceneDev{});
    std::vector<int> ev((size_t)ne * 3, -1), esurf((size_t)ne, -1), vscene((size_t)nv), escene((size_t)ne);
    std::vector<uint8_t> fixed((size_t)nv, 0), in_elem((size_t)nv, 0), erigid((size_t)ne, 0);
    std::vector<StrainEdge> all_edges;
    std::vector<int4> hdr;
    std::vector<int2> load, wb, chunks;
    int v0 = 0, e0 = 0;
    for (int si = 0; si < n; ++si) {
        const cc_mesh* m = &meshes[si];
        const int snv = m->n_points, nt = m->n_tris, nb = m->n_bonds, sne = nt + nb;
        SceneHost& sh = scenes[si];
        sh.v0 = v0; sh.nv = snv; sh.e0 = e0; sh.ne = sne; sh.nt = nt;
        SceneDev& sd = h_scenes[si];
        sd.p = Params{prm.dt, prm.thickness, prm.eps, prm.k, prm.m, prm.lambda, prm.cr};
        for (int d = 0; d < 3; ++d) {
            sd.lo[d] = lo[d];
            sd.hi[d] = hi[d];
        }
        sd.v0 = v0; sd.nv = snv; sd.e0 = e0; sd.ne = sne; sd.nt = nt;
        sd.enabled = 1;
        for (int i = 0; i < snv; ++i) {
            vscene[v0 + i] = si;
            const uint8_t f = m->fixed ? m->fixed[i] : 0;
            if (f > 2) return fail(CC_BAD_INPUT, "point flag must be 0 (free), 1 (fixed) or 2 (movable)");
            fixed[v0 + i] = f;
        }
        for (int t = 0; t < nt; ++t) {
            int* E = &ev[3 * (size_t)(e0 + t)];
            for (int k = 0; k < 3; ++k) {
                int v = m->tris[3 * t + k];
                if (v < 0 || v >= snv) return fail(CC_BAD_INPUT, "triangle point id out of range");
                E[k] = v0 + v;
            }
            if (E[0] == E[1] || E[0] == E[2] || E[1] == E[2])
                return fail(CC_BAD_INPUT, "triangle with a repeated point");
            esurf[e0 + t] = m->tri_surface ? m->tri_surface[t] : 0;
        }
        for (int b = 0; b < nb; ++b) {
            for (int k = 0; k < 2; ++k) {
                int v = m->bonds[2 * b + k];
                if (v < 0 || v >= snv) return fail(CC_BAD_INPUT, "bond point id out of range");
                ev[3 * (size_t)(e0 + nt + b) + k] = v0 + v;
            }
        }
        std::vector<StrainEdge> edges;
        edges.reserve((size_t)3 * nt + nb);
        for (int e = 0; e < sne; ++e) {
            const int* E = &ev[3 * (size_t)(e0 + e)];
            int np = e < nt ? 3 : 2;
            bool rigid = false;
            escene[e0 + e] = si;
            for (int i = 0; i < np; ++i) {
                in_elem[E[i]] = 1;
                if (fixed[E[i]]) rigid = true;
            }
            erigid[e0 + e] = rigid ? 1 : 0;
            if (rigid) continue;  // isRigidBody(hse), dcollid.cpp:495
            if (np == 3) {
                for (int j = 0; j < 3; ++j)
                    edges.push_back(StrainEdge{E[j], E[(j + 1) % 3], m->tri_rest_len[3 * e + j], 0, 0});
            } else {
                edges.push_back(StrainEdge{E[0], E[1], m->bond_rest_len[e - nt], 0, 0});
            }
        }
        size_t nload = load.size();
        sd.strain_e0 = (int)all_edges.size();
        sd.strain_ne = (int)edges.size();
        for (int c = 0; c < sd.strain_ne; c += 256) chunks.push_back(int2{si, sd.strain_e0 + c});
        append_strain_schedule(edges, v0, snv, all_edges, hdr, load, wb, sd, sh.strain_caps);
        sh.strain_edges = (int)edges.size();
        sh.strain_points = (int)(load.size() - nload);
        v0 += snv;
        e0 += sne;
    }
    nedges = (int)all_edges.size();

    // Movable rigid bodies: a surface (run of equal tri_surface) whose first
    // point is movable (dcollid3d.cpp:62). Its points must all be movable and
    // belong to no other element, and every movable point to such a surface,
    // so that each body stays one impact zone for the whole step.
    std::vector<int> vbody((size_t)nv, -1);
    bodies.clear();
    body_unions.clear();
    for (int si = 0; si < n; ++si) {
        const SceneHost& sh = scenes[si];
        const int nt = meshes[si].n_tris;
        for (int t0 = 0; t0 < nt;) {
            int t1 = t0 + 1;
            while (t1 < nt && esurf[sh.e0 + t1] == esurf[sh.e0 + t0]) ++t1;
            if (fixed[ev[3 * (size_t)(sh.e0 + t0)]] & 2) {
                const int b = (int)bodies.size();
                if (find_body(si, esurf[sh.e0 + t0]) >= 0)
                    return fail(CC_BAD_INPUT, "two movable surfaces of one scene share a surface id");
                BodyHost bh;
                bh.scene = si;
                bh.surf = esurf[sh.e0 + t0];
                bodies.push_back(bh);
                for (int t = t0; t < t1; ++t)
                    for (int k = 0; k < 3; ++k) {
                        const int p = ev[3 * (size_t)(sh.e0 + t) + k];
                        if (!(fixed[p] & 2)) return fail(CC_BAD_INPUT, "a movable surface holds a point that is not movable");
                        if (vbody[p] >= 0 && vbody[p] != b) return fail(CC_BAD_INPUT, "a point in two movable surfaces");
                        vbody[p] = b;
                        body_unions.push_back(p);
                    }
            }
            t0 = t1;
        }
    }
    h_body_visit.clear();
    h_body_visit_off.assign(bodies.size() + 1, 0);
    for (int e = 0; e < ne; ++e)
        for (int k = 0; k < 3; ++k) {
            const int p = ev[3 * (size_t)e + k];
            if (p < 0 || !(fixed[p] & 2)) continue;
            if (vbody[p] < 0) return fail(CC_BAD_INPUT, "a movable point outside a movable surface");
            const int ts = escene[e], te = e - scenes[ts].e0;
            if (te >= meshes[ts].n_tris || esurf[e] != bodies[vbody[p]].surf)
                return fail(CC_BAD_INPUT, "a movable point shared with an element outside its body");
        }
    {
        // each body's points in element order (updateFinalForRG's visit)
        std::vector<std::vector<int>> visit(bodies.size());
        std::vector<uint8_t> seen((size_t)nv, 0);
        for (size_t i = 0; i < body_unions.size(); ++i) {
            const int p = body_unions[i];
            if (!seen[p]) {
                seen[p] = 1;
                visit[vbody[p]].push_back(p);
            }
        }
        for (size_t b = 0; b < bodies.size(); ++b) {
            h_body_visit_off[b + 1] = h_body_visit_off[b] + (int)visit[b].size();
            h_body_visit.insert(h_body_visit.end(), visit[b].begin(), visit[b].end());
        }
    }
    const int nbodies = (int)bodies.size();

    bool ok = true;
    ok &= dalloc(&d_scenes, (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_run, (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_tail_mask, (size_t)n) == cudaSuccess;
    ok &= cudaMallocHost(&h_tail_masks, 2 * (size_t)n) == cudaSuccess;
    ok &= cudaMallocHost(&h_run, sizeof(SceneRun) * (size_t)n) == cudaSuccess;
    ok &= cudaMallocHost(&h_bbox, 6 * sizeof(unsigned long long) * (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_vscene, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_escene, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_ev, (size_t)ne * 3) == cudaSuccess;
    ok &= dalloc(&d_esurf, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_erigid, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_fixed, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_in_elem, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_edges, (size_t)nedges) == cudaSuccess;
    ok &= dalloc(&d_strain_hdr, hdr.size()) == cudaSuccess;
    ok &= dalloc(&d_strain_load, load.size()) == cudaSuccess;
    ok &= dalloc(&d_strain_wb, wb.size()) == cudaSuccess;
    ok &= dalloc(&d_strain_passes, 3 * (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_strain_flags, 2 * (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_strain_chunks, chunks.size()) == cudaSuccess;
    ok &= dalloc(&d_strain_order, (size_t)n) == cudaSuccess;
    n_strain_chunks = (int)chunks.size();
    ok &= cudaMalloc(&d_strain_step, strain_step_bytes(nedges)) == cudaSuccess;
    ok &= dalloc(&d_xo, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_av, (size_t)nv) == cudaSuccess;

    ok &= dalloc(&d_xold_in, (size_t)nv * 3) == cudaSuccess;
    ok &= dalloc(&d_xcand_in, (size_t)nv * 3) == cudaSuccess;
    ok &= dalloc(&d_vel, (size_t)nv * 3) == cudaSuccess;
    ok &= dalloc(&d_xout, (size_t)nv * 3) == cudaSuccess;
    ok &= dalloc(&d_hc, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_box, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_box_st, (size_t)ne) == cudaSuccess;
    bvh.n = ne;
    bvh.nscenes = n;
    bvh.elem_scene = nullptr;
    ok &= dalloc(&bvh.keys, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.order, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.range_hi, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.range_lo, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.parent, (size_t)2 * ne) == cudaSuccess;
    ok &= dalloc(&bvh.flags, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.node, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.leaf, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.rnode, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.rope, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.leaf32, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.qnext, 1) == cudaSuccess;
    ok &= dalloc(&bvh.bbox_enc, 6 * (size_t)n) == cudaSuccess;
    ok &= cudaMalloc(&bvh.sort_temp, radix_sort_temp_bytes(ne > 0 ? ne : 1)) == cudaSuccess;
    ok &= dalloc(&apply.cnt, (size_t)nv + nbodies) == cudaSuccess;
    ok &= dalloc(&apply.off, (size_t)nv + nbodies) == cudaSuccess;
    ok &= dalloc(&apply.cur, (size_t)nv + nbodies) == cudaSuccess;
    ok &= cudaMalloc(&apply.scan_temp, scan_temp_bytes(nv + nbodies > 0 ? nv + nbodies : 1)) == cudaSuccess;
    if (nbodies > 0) {
        const size_t nm = (size_t)h_body_visit.size();
        ok &= dalloc(&d_vbody, (size_t)nv) == cudaSuccess;
        ok &= dalloc(&d_body_mass, (size_t)nbodies) == cudaSuccess;
        ok &= dalloc(&d_body_members, nm) == cudaSuccess;
        ok &= dalloc(&d_body_member_body, nm) == cudaSuccess;
        ok &= dalloc(&d_body_zone_off, (size_t)nbodies + 1) == cudaSuccess;
        ok &= dalloc(&d_body_visit, nm) == cudaSuccess;
        ok &= dalloc(&d_body_visit_off, (size_t)nbodies + 1) == cudaSuccess;
        ok &= dalloc(&d_body_acc, (size_t)nbodies) == cudaSuccess;
        ok &= dalloc(&d_body_num, (size_t)nbodies) == cudaSuccess;
        ok &= dalloc(&d_body_out, (size_t)nbodies) == cudaSuccess;
    }
    ok &= dalloc(&d_rank[0], (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_rank[1], (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_pbox_lo, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_pbox_hi, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_p32, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_v32, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_act_e, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_act_p, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_sel, 3 * (size_t)n + 2) == cudaSuccess;
    ok &= cudaMallocHost(&h_sel, sizeof(int) * (3 * (size_t)n + 2)) == cudaSuccess;
    ok &= dalloc(&d_pstamp, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_edirty, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_query, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_ctl, (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_loop, 1) == cudaSuccess;
    ok &= dalloc(&d_lsel, 3 * ((size_t)n + 1)) == cudaSuccess;
    ok &= dalloc(&d_act_l, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_rebuild, (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_tree_vol, (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_tree_built, 2 * (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_tree_jobs, 3 * (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_tree_root, (size_t)n) == cudaSuccess;
    ok &= dalloc(&d_tree_vol_out, (size_t)n) == cudaSuccess;
    ok &= cudaMallocHost(&h_tree_jobs, sizeof(int) * 3 * (size_t)n) == cudaSuccess;
    ok &= cudaMallocHost(&h_tree_vol_out, sizeof(double) * (size_t)n) == cudaSuccess;
    ok &= cudaMallocHost(&h_ctl, sizeof(SceneCtl) * (size_t)n) == cudaSuccess;
    ok &= cudaMallocHost(&h_loop, sizeof(LoopCtl)) == cudaSuccess;
    ok &= cudaMallocHost(&h_rebuild, sizeof(int) * (size_t)n) == cudaSuccess;
    if (!ok) return fail(CC_NO_MEMORY, "device allocation failed");
    bvh.elem_scene = d_escene;
    bvh.ev = d_ev;
    bvh.ne_all = ne;
    bvh.scenes = d_scenes;
    bvh.run = d_run;
    bvh.refit_up = refit_up ? 1 : 0;
    cc_status st = grow_pairs(8 * ne + 4096);
    if (st) return st;
    st = grow_contrib(4 * ne + 4096);
    if (st) return st;
    cudaMemcpyAsync(d_vscene, vscene.data(), sizeof(int) * vscene.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_escene, escene.data(), sizeof(int) * escene.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_ev, ev.data(), sizeof(int) * ev.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_esurf, esurf.data(), sizeof(int) * esurf.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_erigid, erigid.data(), erigid.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_fixed, fixed.data(), fixed.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_in_elem, in_elem.data(), in_elem.size(), cudaMemcpyHostToDevice, stream);
    if (nedges)
        cudaMemcpyAsync(d_edges, all_edges.data(), sizeof(StrainEdge) * all_edges.size(), cudaMemcpyHostToDevice,
                        stream);
    if (!hdr.empty())
        cudaMemcpyAsync(d_strain_hdr, hdr.data(), sizeof(int4) * hdr.size(), cudaMemcpyHostToDevice, stream);
    if (!chunks.empty())
        cudaMemcpyAsync(d_strain_chunks, chunks.data(), sizeof(int2) * chunks.size(), cudaMemcpyHostToDevice, stream);
    {
        // the sweep of a scene is a chain of its levels: the longest chains
        // start first, so none waits for a second wave of CTAs
        std::vector<int> order((size_t)n);
        for (int i = 0; i < n; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return h_scenes[a].strain_levels > h_scenes[b].strain_levels; });
        cudaMemcpy(d_strain_order, order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
    }
    if (!load.empty()) {
        cudaMemcpyAsync(d_strain_load, load.data(), sizeof(int2) * load.size(), cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_strain_wb, wb.data(), sizeof(int2) * wb.size(), cudaMemcpyHostToDevice, stream);
    }
    cudaMemsetAsync(d_av, 0, sizeof(double4_32a) * (size_t)(nv > 0 ? nv : 1), stream);
    cudaMemsetAsync(d_run, 0, sizeof(SceneRun) * (size_t)n, stream);
    cudaMemsetAsync(d_rank[0], 0, sizeof(int) * (size_t)(ne > 0 ? ne : 1), stream);
    cudaMemsetAsync(d_rank[1], 0, sizeof(int) * (size_t)(ne > 0 ? ne : 1), stream);
    cudaMemsetAsync(d_lsel, 0, sizeof(int) * 3 * ((size_t)n + 1), stream);
    cudaMemsetAsync(d_pstamp, 0xff, sizeof(unsigned) * (size_t)(nv > 0 ? nv : 1), stream);
    cudaMemsetAsync(d_edirty, 0, (size_t)(ne > 0 ? ne : 1), stream);
    cudaMemsetAsync(d_rebuild, 0, sizeof(int) * (size_t)n, stream);
    cudaMemsetAsync(d_tree_vol, 0, sizeof(double) * (size_t)n, stream);
    cudaMemsetAsync(d_tree_built, 0, sizeof(int) * 2 * (size_t)n, stream);
    h_boxes.resize((size_t)ne);
    h_rank.resize((size_t)ne);
    h_tree_vol_stage.assign((size_t)n, 0.0);
    h_vscene.swap(vscene);
    h_ev = ev;
    vtk_count.assign((size_t)n, 0);
    uf_root.resize((size_t)nv);
    uf_next.assign((size_t)nv, -1);
    uf_tail.resize((size_t)nv);
    uf_w.assign((size_t)nv, 1);
    for (int p = 0; p < nv; ++p) uf_root[p] = uf_tail[p] = p;
    uf_touched.clear();
    h_fixed = fixed;
    if (nbodies > 0) {
        // each body's zone member list, as the unions leave it
        reset_zones();
        std::vector<int> members, member_body, zone_off(1, 0);
        for (int b = 0; b < nbodies; ++b) {
            const int r = find_set(h_body_visit[h_body_visit_off[b]]);
            for (int q = r; q >= 0; q = uf_next[q]) {
                members.push_back(q);
                member_body.push_back(b);
            }
            zone_off.push_back((int)members.size());
        }
        cudaMemcpy(d_vbody, vbody.data(), sizeof(int) * (size_t)nv, cudaMemcpyHostToDevice);
        cudaMemcpy(d_body_members, members.data(), sizeof(int) * members.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(d_body_member_body, member_body.data(), sizeof(int) * member_body.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(d_body_zone_off, zone_off.data(), sizeof(int) * zone_off.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(d_body_visit, h_body_visit.data(), sizeof(int) * h_body_visit.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(d_body_visit_off, h_body_visit_off.data(), sizeof(int) * h_body_visit_off.size(),
                   cudaMemcpyHostToDevice);
        cudaMemset(d_body_acc, 0, sizeof(double4_32a) * (size_t)nbodies);
        upload_body_mass();
        body_bufs.n = nbodies;
        body_bufs.nmembers = (int)members.size();
        body_bufs.members = d_body_members;
        body_bufs.member_body = d_body_member_body;
        body_bufs.zone_off = d_body_zone_off;
        body_bufs.visit = d_body_visit;
        body_bufs.visit_off = d_body_visit_off;
        body_bufs.acc = d_body_acc;
        body_bufs.num = d_body_num;
        body_bufs.out = d_body_out;
        body_bufs.fixed = d_fixed;
        h_body_out.assign((size_t)nbodies, double4_32a{});
    }
    {
        // the union-find every step starts from: makeSet, then the movable
        // bodies' unions (reset_zones above, when there are bodies)
        const int nz = nv / 2 + 1;
        bool zok = dalloc(&zb.cc, (size_t)nv) == cudaSuccess && dalloc(&zb.uf, (size_t)nv) == cudaSuccess &&
                   dalloc(&d_cc0, (size_t)nv) == cudaSuccess && dalloc(&d_uf0, (size_t)nv) == cudaSuccess &&
                   dalloc(&zb.zone_rng, (size_t)nz) == cudaSuccess && dalloc(&zb.zone_root, (size_t)nz) == cudaSuccess &&
                   dalloc(&zb.members, (size_t)nv) == cudaSuccess &&
                   dalloc(&zb.prev_members, (size_t)nv) == cudaSuccess &&
                   dalloc(&zb.prev_off, (size_t)nv) == cudaSuccess && dalloc(&zb.prev_len, (size_t)nv) == cudaSuccess &&
                   dalloc(&zb.prev_epoch, (size_t)nv) == cudaSuccess && dalloc(&zb.epoch, 1) == cudaSuccess;
        if (!zok) return fail(CC_NO_MEMORY, "zone buffers");
        zb.zone_cap = nz;
        zb.n_pts_cap = nv;
        cudaMemsetAsync(zb.epoch, 0, sizeof(unsigned), stream);
        std::vector<UfNode> u0((size_t)nv);
        std::vector<int> c0((size_t)nv);
        for (int p = 0; p < nv; ++p) {
            u0[p] = UfNode{uf_root[p], uf_next[p], uf_tail[p], uf_w[p]};
            c0[p] = find_set(p);
        }
        if (nv) {
            cudaMemcpy(d_uf0, u0.data(), sizeof(UfNode) * (size_t)nv, cudaMemcpyHostToDevice);
            cudaMemcpy(d_cc0, c0.data(), sizeof(int) * (size_t)nv, cudaMemcpyHostToDevice);
        }
        uf_on_device = false;
    }
    if (grow_unions(1024)) return CC_NO_MEMORY;
    if (grow_subs(2 * ne + 4096)) return CC_NO_MEMORY;
    h_strain_passes.assign(3 * (size_t)n, 0);
    scenes_dirty = true;
    strain_configure();
    upload_scenes();  // synchronises: the host vectors above are pageable
    return cuda_check("assemble");
}

// Tree build / rebuild bookkeeping of aabbProximity / aabbCollision
// (dcollid.cpp:366-428), per scene in this pass: both trees of a scene share
// one volume; a tree is (re)built on first use or when its root volume has
// grown by more than 20%. Rebuilds emulate the reference's insertion order
// on the host, one scene per host thread.
cc_status cc_solver::update_trees(int which, const Box6* boxes) {
    cudaMemcpyAsync(h_bbox, bvh.bbox_enc, 6 * sizeof(unsigned long long) * (size_t)nscenes, cudaMemcpyDeviceToHost,
                    stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("leaf boxes");
    std::vector<int> todo;
    std::vector<double> vol((size_t)nscenes, 0.0);
    for (int s = 0; s < nscenes; ++s) {
        if (h_run[s].mode == kSceneIdle) continue;
        SceneHost& sh = scenes[s];
        double rlo[3], rhi[3];
        for (int d = 0; d < 3; ++d) {
            rlo[d] = dec_host(h_bbox[6 * s + d]);
            rhi[d] = dec_host(h_bbox[6 * s + 3 + d]);
        }
        double v = box_volume(rlo, rhi);
        if (!sh.built[which] || (v - sh.volume) > 0.2 * sh.volume) todo.push_back(s);
    }
    if (todo.empty()) return CC_OK;
    return build_trees(which, todo, boxes);
}

// Build tree `which` of the scenes in `ids` from their leaf boxes (device):
// the ranks go to d_rank[which], the root volumes to the scenes' shared
// volume. By default on the GPU (cc_tree_gpu.cu: the reference's insertions
// pipelined in one CTA per tree); with CC_TUNE_HOST_TREE on host threads,
// one tree per thread (cc_tree_order.cpp). Both give the same ranks and
// volumes.
cc_status cc_solver::build_trees(int which, std::vector<int>& ids, const Box6* boxes) {
    const auto t0 = std::chrono::steady_clock::now();
    if (host_tree) {
        for (int s : ids)
            cudaMemcpyAsync(h_boxes.data() + scenes[s].e0, boxes + scenes[s].e0, sizeof(Box6) * (size_t)scenes[s].ne,
                            cudaMemcpyDeviceToHost, stream);
        if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("leaf boxes to host");
        // largest scenes first: they bound the time of the parallel build
        std::sort(ids.begin(), ids.end(), [&](int a, int b) { return scenes[a].ne > scenes[b].ne; });
        int threads = host_threads > 0 ? host_threads : (int)std::thread::hardware_concurrency();
        if (threads <= 0) threads = 1;
        parallel_for((int)ids.size(), threads, [&](int i) {
            SceneHost& sh = scenes[ids[i]];
            sh.volume = sh.tree[which].build(h_boxes.data() + sh.e0, sh.ne);
            sh.tree[which].ranks(h_rank.data() + sh.e0);
        });
        for (int s : ids)
            cudaMemcpyAsync(d_rank[which] + scenes[s].e0, h_rank.data() + scenes[s].e0,
                            sizeof(int) * (size_t)scenes[s].ne, cudaMemcpyHostToDevice, stream);
    } else {
        if (!d_tree_scratch &&
            cudaMalloc(&d_tree_scratch, tree_scratch_bytes(bvh.ne_all)) != cudaSuccess) {
            d_tree_scratch = nullptr;
            return fail(CC_NO_MEMORY, "tree build scratch allocation failed");
        }
        int max_ne = 0;
        for (size_t i = 0; i < ids.size(); ++i) {
            const SceneHost& sh = scenes[ids[i]];
            h_tree_jobs[3 * i] = ids[i];
            h_tree_jobs[3 * i + 1] = sh.e0;
            h_tree_jobs[3 * i + 2] = sh.ne;
            max_ne = std::max(max_ne, sh.ne);
        }
        const int nj = (int)ids.size();
        cudaMemcpyAsync(d_tree_jobs, h_tree_jobs, sizeof(int) * 3 * (size_t)nj, cudaMemcpyHostToDevice, stream);
        tree_order_gpu(boxes, d_tree_jobs, nj, max_ne, d_tree_scratch, bvh.ne_all, d_rank[which], d_tree_root,
                       d_tree_vol_out, stream);
        cudaMemcpyAsync(h_tree_vol_out, d_tree_vol_out, sizeof(double) * (size_t)nj, cudaMemcpyDeviceToHost, stream);
        if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("tree build");
        for (int i = 0; i < nj; ++i) scenes[ids[i]].volume = h_tree_vol_out[i];
    }
    for (int s : ids) scenes[s].built[which] = scenes[s].ne > 0;
    counters[22] += std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count();
    counters[8] += (long long)ids.size();
    sync_tree_state(ids, which);
    return CC_OK;
}

// The device copy of the trees' shared volume and built flags, for the
// scenes whose tree `which` was just built (the device loop's rebuild test
// reads them).
void cc_solver::sync_tree_state(const std::vector<int>& ids, int which) {
    for (int s : ids) {
        h_tree_vol_stage[s] = scenes[s].volume;
        cudaMemcpyAsync(d_tree_vol + s, &h_tree_vol_stage[s], sizeof(double), cudaMemcpyHostToDevice, stream);
        cudaMemsetAsync(d_tree_built + (size_t)which * nscenes + s, 0x01, 1, stream);
    }
    // the staging values must not change before the copies have run
    cudaStreamSynchronize(stream);
}

// The trees the device loop flagged (d_rebuild, read into h_rebuild): the
// reference's insertion order emulated on host threads for those scenes,
// from the boxes of the pass that flagged them, and the new ranks, volumes
// and built flags uploaded.
cc_status cc_solver::rebuild_flagged() {
    std::vector<int> todo[2];
    for (int s = 0; s < nscenes; ++s)
        if (h_rebuild[s] == 1 || h_rebuild[s] == 2) todo[h_rebuild[s] - 1].push_back(s);
    for (int which = 0; which < 2; ++which) {
        std::vector<int>& ids = todo[which];
        if (ids.empty()) continue;
        const Box6* boxes = (which == 0 && combined_broad) ? d_box_st : d_box;
        const cc_status st = build_trees(which, ids, boxes);
        if (st) return st;
    }
    cudaMemsetAsync(d_rebuild, 0, sizeof(int) * (size_t)nscenes, stream);
    return cuda_check("tree rebuild");
}

// The proximity pass of a step in the device-loop form: the same work as
// detect_pass(0), launched without waiting for any of it. Whether the
// proximity tree must be built or rebuilt is tested on the device
// (tree_check); if so, nothing of the pass is applied and the host finds out
// after the loop.
void cc_solver::prox_pass_async() {
    cudaMemcpyAsync(d_run, h_run, sizeof(SceneRun) * (size_t)nscenes, cudaMemcpyHostToDevice, stream);
    const bool combined = combined_broad;
    prof(kStBoxes, true);
    leaf_boxes(d_ev, bvh.act, bvh.n, d_escene, d_scenes, nscenes, d_xo, d_av, 0, combined ? d_box_st : d_box,
               bvh.bbox_enc, stream);
    tree_check(d_run, nscenes, bvh.bbox_enc, d_tree_vol, d_tree_built, 0, d_rebuild, d_loop, stream);
    if (combined)
        leaf_boxes(d_ev, bvh.act, bvh.n, d_escene, d_scenes, nscenes, d_xo, d_av, 1, d_box, bvh.bbox_enc, stream);
    prof(kStBoxes, false);
    prof(kStBvh, true);
    bvh_build(d_box, bvh, stream);
    bvh_this_step = true;
    bvh_set = cur_set;
    full_this_step = bvh.act == nullptr;
    if (mode == 1)
        point_boxes(d_xo, d_av, d_vscene, d_scenes, bvh.act ? d_act_p : nullptr, n_act_p, 0, d_pbox_lo, d_pbox_hi,
                    d_p32, d_v32, stream);
    prof(kStBvh, false);
    loop_reset(d_ctr, d_run, nscenes, d_loop, stream);
    prof(kStTraverse, true);
    bvh_pairs(d_box, bvh, d_pairs, pair_cap, d_ctr, stream, d_ev, tune.traverse_block, combined ? d_box_st : nullptr,
              tune.packet_traverse, tune.rope_traverse, tune.traverse_refill, tune.stack_depth);
    prof(kStTraverse, false);
    prof(kStNarrowProx, true);
    NarrowArgs a = narrow_args(0, combined);
    a.ps = loop_stamp();
    if (mode == 1 && split_narrow)
        narrow_pass_split(a, 0, pair_cap, stream, tune.narrow_block, false);
    else
        narrow_pass(a, 0, pair_cap, stream, tune.narrow_block);
    prof(kStNarrowProx, false);
    prof(kStApply, true);
    ApplyBufs ab = apply;
    ab.ps = loop_stamp();
    apply_contribs(d_contrib, d_ctr, contrib_cap, nv, d_av, d_hc, ab, stream, nullptr,
                   bodies.empty() ? nullptr : &body_bufs);
    if (!bodies.empty())  // updateImpactZoneVelocityForRG (dcollid.cpp:744-745)
        zone_solve(d_body_members, d_body_zone_off, (int)bodies.size(), d_fixed, d_xo, d_av, d_vscene, d_scenes, d_ctr,
                   stream, d_run, loop_stamp());
    prof(kStApply, false);
    pass_end(d_ctr, d_ctl, d_run, nscenes, d_loop, (combined && bodies.empty()) ? 1 : 0, false, 0, stream);
}

// The graph of the passes after the proximity pass: a WHILE node whose body
// is one detection pass over the scenes that still have one (planned on the
// device), with the impact-zone stage behind an IF node, and the loop's
// condition set by the pass's last kernel. Built for the hierarchy of
// n_hier leaves that the step's proximity pass builds, and again whenever a
// buffer or a setting it holds changes.
cc_status cc_solver::build_loop_graph(int n_hier) {
    LoopGraph& lg = loop_graphs[mode];
    if (lg.exec) cudaGraphExecDestroy(lg.exec);
    lg = LoopGraph{};
    if (!cap_stream && (cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking) != cudaSuccess ||
                        cudaStreamCreateWithFlags(&cap_stream2, cudaStreamNonBlocking) != cudaSuccess ||
                        cudaStreamCreateWithFlags(&cap_stream3, cudaStreamNonBlocking) != cudaSuccess))
        return cuda_check("capture streams");
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) return cuda_check("loop graph");
    cudaGraphConditionalHandle h_loop_c, h_zone;
    cudaGraphNodeParams wp = {};
    cudaGraphNode_t wnode;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h_loop_c, g, 1, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) {
        wp.type = cudaGraphNodeTypeConditional;
        wp.conditional.handle = h_loop_c;
        wp.conditional.type = cudaGraphCondTypeWhile;
        wp.conditional.size = 1;
        e = cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp);
    }
    cudaGraph_t body = e == cudaSuccess ? wp.conditional.phGraph_out[0] : nullptr;
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h_zone, body, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(cap_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return fail(CC_CUDA_ERROR, std::string("loop graph: ") + cudaGetErrorString(e));
    }
    const long long l0 = g_kernel_launches;
    cudaStream_t cs = cap_stream;
    int* sel = d_lsel;
    int* eoff = d_lsel + (nscenes + 1);
    int* poff = d_lsel + 2 * (nscenes + 1);
    BvhBufs lb = bvh;  // the step's hierarchy, over the pass's scenes' leaves
    lb.n = n_hier;
    lb.act = nullptr;
    lb.sub = d_act_l;
    lb.nsub = ne;
    lb.dnsub = &d_loop->nbroad;
    const int m0 = kStLoopPlan - 1;  // mark slot of stage st: st - m0
    mark(0, cs);
    loop_plan(d_ctl, d_run, d_scenes, nscenes, d_loop, sel, eoff, poff, h_zone, cs);
    loop_expand(sel, eoff, poff, d_scenes, d_ctl, d_loop, ne + nv, d_act_e, d_act_l, d_act_p, cs);
    mark(kStLoopPlan - m0, cs);
    leaf_boxes(d_ev, d_act_e, ne, d_escene, d_scenes, nscenes, d_xo, d_av, 1, d_box, bvh.bbox_enc, cs,
               &d_loop->nbroad);
    tree_check_reset(d_run, nscenes, bvh.bbox_enc, d_tree_vol, d_tree_built + nscenes, 1, d_rebuild, d_loop, d_ctr,
                     cs);
    mark(kStLoopBoxes - m0, cs);
    bvh_refit(d_box, lb, cs, false);  // the roots of the proximity pass's build stand
    if (mode == 1)
        point_boxes(d_xo, d_av, d_vscene, d_scenes, d_act_p, nv, 1, d_pbox_lo, d_pbox_hi, d_p32, d_v32, cs,
                    &d_loop->npts);
    mark(kStLoopRefit - m0, cs);
    // the full traversal (first CCD pass) or the pruned one (later passes)
    lb.dnq = &d_loop->nq_full;
    bvh_pairs(d_box, lb, d_pairs, pair_cap, d_ctr, cs, d_ev, tune.traverse_block, nullptr, false, tune.rope_traverse,
              tune.traverse_refill, tune.stack_depth);
    mark(kStLoopTraverse - m0, cs);
    pruned_pairs(lb, d_act_e, d_act_l, d_pstamp, d_loop, d_edirty, d_query, ne, d_pairs, pair_cap, d_ctr, d_ev, cs,
                 pruned_warp);
    mark(kStLoopPruned - m0, cs);
    NarrowArgs a = narrow_args(1, false);
    a.ps = loop_stamp();
    if (mode == 1 && split_narrow) {
        narrow_pass_split(a, 1, pair_cap, cs, tune.narrow_block, true, kSplitFilter);
        mark(kStLoopFilter - m0, cs);
        narrow_pass_split(a, 1, pair_cap, cs, tune.narrow_block, true, kSplitSubtests);
        mark(kStLoopSubtests - m0, cs);
    } else {
        narrow_pass(a, 1, pair_cap, cs, tune.narrow_block);
        mark(kStLoopSubtests - m0, cs);
    }
    ApplyBufs ab = apply;
    ab.ps = loop_stamp();
    apply_contribs(d_contrib, d_ctr, contrib_cap, nv, d_av, d_hc, ab, cs, nullptr,
                   bodies.empty() ? nullptr : &body_bufs);
    if (!bodies.empty())
        zone_solve(d_body_members, d_body_zone_off, (int)bodies.size(), d_fixed, d_xo, d_av, d_vscene, d_scenes, d_ctr,
                   cs, d_run, loop_stamp());
    mark(kStLoopApply - m0, cs);
    const long long l1 = g_kernel_launches;
    // the impact-zone stage, only in passes with a scene in that mode
    cudaStreamCaptureStatus cst;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaGraphNodeParams ip = {};
    cudaGraphNode_t inode;
    e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &ndeps);
    if (e == cudaSuccess) {
        ip.type = cudaGraphNodeTypeConditional;
        ip.conditional.handle = h_zone;
        ip.conditional.type = cudaGraphCondTypeIf;
        ip.conditional.size = 1;
        e = cudaGraphAddNode(&inode, cg, deps, nullptr, ndeps, &ip);
    }
    if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(cs, &inode, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(cap_stream2, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t ez = zone_pass(zb, d_ctr, d_fixed, d_act_p, nv, &d_loop->npts, d_vscene, d_run, d_scenes,
                                         d_av, d_xo, cap_stream2, loop_stamp(), cap_stream3,
                                         loop_marks ? d_marks : nullptr, kStLoopZoneSort - m0);
        cudaGraph_t zg = nullptr;
        e = cudaStreamEndCapture(cap_stream2, &zg);
        if (e == cudaSuccess) e = ez;
    }
    const long long l2 = g_kernel_launches;
    pass_end(d_ctr, d_ctl, d_run, nscenes, d_loop, 0, true, h_loop_c, cs);
    if (loop_marks && d_marks) stage_mark(d_marks, kStLoopEnd - m0, cs, d_ctr, d_loop);
    cudaGraph_t bg = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cs, &bg);
    lg.body_launches = (l1 - l0) + (g_kernel_launches - l2);
    lg.zone_launches = l2 - l1;
    g_kernel_launches = l0;
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&lg.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        lg.exec = nullptr;
        cudaGetLastError();
        return fail(CC_CUDA_ERROR, std::string("loop graph: ") + cudaGetErrorString(e));
    }
    lg.gen = loop_gen;
    lg.key_n = n_hier;
    return CC_OK;
}

// All detection passes of a step in the device-loop form: the proximity
// pass, then the loop graph, then one synchronisation. When the device asks
// for the host (a tree to rebuild, a buffer to grow), the host does that and
// the stopped pass runs again (the proximity pass and the loop, or the loop
// alone). Fills each scene's pass kinds, hasCollision and status.
cc_status cc_solver::device_passes(std::string& capped) {
    int nact = 0;
    for (int s = 0; s < nscenes; ++s) {
        SceneHost& sh = scenes[s];
        const bool on = sh.ne > 0 && sh.enabled;
        h_ctl[s] = SceneCtl{on ? kSeqProx : kSeqDone, 0, 0, 0, 0, 0, -1, 0};
        h_run[s] = SceneRun{on ? kSceneProx : kSceneIdle, 0, 0, -1, -1, {0, 0, 0}};
        if (!on) continue;
        ++nact;
        counters[0]++;
        counters[18] += 72ll * sh.nv + 12ll * sh.nt + 8ll * (sh.ne - sh.nt) + 48ll * (2ll * sh.ne - 1);
    }
    if (nact == 0) return CC_OK;
    select_active();
    for (int s = 0; s < nscenes; ++s) h_ctl[s].leafbase = h_run[s].leaf0;
    const int n_hier = bvh.n;
    std::memset(h_loop, 0, sizeof(LoopCtl));
    h_loop->nact = nact;
    h_loop->nact_e = bvh.n;
    h_loop->nact_p = n_act_p;
    h_loop->nbroad = bvh.n;
    h_loop->npts = n_act_p;
    h_loop->reuse = -1;
    h_loop->reuse_n = -1;
    h_loop->zone_cap = zone_cap;
    h_loop->serial = serial_base;
    h_loop->prune_on = prune ? 1 : 0;
    h_loop->nq_full = bvh.n;
    const LoopCtl loop_init = *h_loop;
    if (pass_log && loop_marks && d_marks)  // this step's rows of the pass log from row 0
        cudaMemsetAsync(d_marks + 1 + 2 * kLoopMarkSlots, 0, sizeof(unsigned long long), stream);
    cudaMemcpyAsync(d_ctl, h_ctl, sizeof(SceneCtl) * (size_t)nscenes, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_loop, h_loop, sizeof(LoopCtl), cudaMemcpyHostToDevice, stream);
    bool need_prox = true;
    long long graph_runs = 0;
    LoopGraph* lgraph = nullptr;
    for (int round = 0;; ++round) {
        if (round >= 64) return fail(CC_PAIR_OVERFLOW, "the detection loop kept stopping for the host");
        if (need_prox) prox_pass_async();
        LoopGraph* lgp = current_loop_graph(n_hier);
        if (!lgp) {
            cc_status st = build_loop_graph(n_hier);
            if (st) return st;
            lgp = &loop_graphs[mode];
        }
        lgraph = lgp;
        prof(kStLoop, true);
        if (cudaGraphLaunch(lgp->exec, stream) != cudaSuccess) return cuda_check("loop graph launch");
        prof(kStLoop, false);
        ++graph_runs;
        cudaMemcpyAsync(h_loop, d_loop, sizeof(LoopCtl), cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(h_ctl, d_ctl, sizeof(SceneCtl) * (size_t)nscenes, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(h_rebuild, d_rebuild, sizeof(int) * (size_t)nscenes, cudaMemcpyDeviceToHost, stream);
        if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("detection loop");
        const int host = h_loop->host;
        if (!host) break;
        // the proximity pass stopped if no pass has completed yet
        const bool in_prox = h_loop->acc[kAccIters] == 0;
        const int err = h_loop->err;
        if (host & kHostFatal) {
            if (err & kErrNan) return fail(CC_NAN_DETECTED, "non-finite velocity or normal (the reference exits here)");
            return fail(CC_CUDA_ERROR, index_error(err));
        }
        if (host & kHostRebuild) {
            cc_status st = rebuild_flagged();
            if (st) return st;
        }
        if (host & kHostRetry) {
            cc_status st = CC_OK;
            if (err & kErrStack) {
                if (tune.stack_depth >= kTraversalStack)
                    return fail(CC_STACK_OVERFLOW, "BVH traversal stack overflow");
                tune.stack_depth = kTraversalStack;  // a tuned shallower stack was too shallow here
                loop_dirty = true;
            }
            const PassCounters& c = h_loop->stopped;  // the stopped pass's counts
            if (!st && (err & kErrPairOverflow)) st = grow_pairs(2 * c.npairs + 1024);
            if (!st && (err & kErrContribOverflow)) st = grow_contrib(2 * c.ncontrib + 1024);
            if (!st && (err & kErrSubOverflow)) st = grow_subs(2 * std::max(c.nsub_pt, c.nsub_ee) + 1024);
            if (!st && (err & kErrUnionOverflow)) st = grow_unions(2 * c.nunion + 1024);
            if (st) return st;
        }
        // the stopped pass runs again: the proximity pass from the start (no
        // pass has counted anything yet), a later pass with its modes as they
        // are (pending)
        if (in_prox) {
            cudaMemcpy(d_loop, &loop_init, sizeof(LoopCtl), cudaMemcpyHostToDevice);
        } else {
            cudaMemsetAsync(&d_loop->host, 0, sizeof(int), stream);
            cudaMemsetAsync(&d_loop->err, 0, sizeof(int), stream);
        }
        need_prox = in_prox;
    }
    serial_base = h_loop->serial + 1u;
    // the passes' counters (the proximity pass's scene-pass counts are above)
    const unsigned long long* a = h_loop->acc;
    counters[0] += (long long)a[kAccPasses];
    counters[1] += (long long)a[kAccCcd];
    counters[2] += (long long)a[kAccZone];
    counters[3] += (long long)a[kAccPairs];
    counters[4] += (long long)a[kAccVisits];
    counters[5] += (long long)a[kAccHits];
    counters[6] += (long long)a[kAccContacts];
    counters[12] += (long long)a[kAccSub];
    counters[13] += (long long)a[kAccMovingVisits];
    counters[15] += (long long)a[kAccCr];
    counters[16] += (long long)a[kAccLeaves];
    counters[17] += (long long)a[kAccBroadPairs];
    counters[18] += (long long)a[kAccPathBytes];
    counters[19] += n_hier;
    counters[20] += (long long)a[kAccProxPairs];
    counters[23] += (long long)a[kAccQueries];
    counters[24] += (long long)a[kAccUnions];
    const long long loop_iters = (long long)a[kAccIters] - 1;
    counters[21] += loop_iters;
    if (pass_log && loop_marks && d_marks) print_pass_log();
    count_launch((int)(lgraph->body_launches * (loop_iters + graph_runs) +
                       lgraph->zone_launches * (long long)a[kAccZonePasses]));
    for (int s = 0; s < nscenes; ++s) {
        SceneHost& sh = scenes[s];
        const SceneCtl& c = h_ctl[s];
        if (!(sh.ne > 0 && sh.enabled)) continue;
        sh.pass_kinds.push_back(kPassProx);
        for (int i = 0; i < c.nccd; ++i) sh.pass_kinds.push_back(kPassCcd);
        for (int i = 0; i < c.nzone; ++i) sh.pass_kinds.push_back(kPassZone);
        sh.npass = (int)sh.pass_kinds.size();
        sh.hcol = c.hcol;
        sh.state = kHsDone;
        if (c.status == kIterCap) {
            sh.status = CC_ITER_CAP;
            capped += (capped.empty() ? "" : " ") + std::to_string(s);
        }
    }
    return CC_OK;
}

// One detection pass of every scene that has one to run: boxes, tree
// bookkeeping, candidate pairs, narrow phase, impulses applied
// (aabbProximity/aabbCollision + updateAverageVelocity, dcollid.cpp:390-406,
// 430-468), and for scenes in impact-zone mode the rigid zone update
// (dcollid.cpp:236-262). Retried with larger buffers on overflow. Leaves
// every scene's hit count in h_run.
cc_status cc_solver::detect_pass(int moving, bool any_zone) {
    select_active();
    // proximity pass: pairs on swept boxes with the static-overlap flag;
    // first CCD pass after a proximity pass without impulses: those pairs
    const bool combined = combined_broad && !moving;
    const bool reuse = moving && reuse_pairs && cur_set == reuse_set;
    reuse_pairs = false;
    // some of the scenes, after this step's hierarchy over all elements: it
    // is refit over their leaves, where each scene starts at its e0
    const bool on_full = subset_refit && !reuse && full_this_step && bvh.act != nullptr;
    if (on_full)
        for (int s : cur_set) h_run[s].leaf0 = scenes[s].e0;
    cudaMemcpyAsync(d_run, h_run, sizeof(SceneRun) * (size_t)nscenes, cudaMemcpyHostToDevice, stream);
    cc_status st = CC_OK;
    prof(kStBoxes, true);
    if (combined) {
        leaf_boxes(d_ev, bvh.act, bvh.n, d_escene, d_scenes, nscenes, d_xo, d_av, 0, d_box_st, bvh.bbox_enc, stream);
        st = update_trees(0, d_box_st);
        if (st) return st;
        leaf_boxes(d_ev, bvh.act, bvh.n, d_escene, d_scenes, nscenes, d_xo, d_av, 1, d_box, bvh.bbox_enc, stream);
    } else if (!reuse) {
        leaf_boxes(d_ev, bvh.act, bvh.n, d_escene, d_scenes, nscenes, d_xo, d_av, moving, d_box, bvh.bbox_enc, stream);
    }
    prof(kStBoxes, false);
    if (!combined) {
        st = update_trees(moving, d_box);
        if (st) return st;
    }
    prof(kStBvh, true);
    if (reuse) {
        // the hierarchy and the pairs of the proximity pass stand
    } else if (on_full) {
        BvhBufs fv = full_view();
        bvh_refit(d_box, fv, stream);
    } else if (bvh_this_step && cur_set == bvh_set) {
        bvh_refit(d_box, bvh, stream);
    } else {
        bvh_build(d_box, bvh, stream);
        bvh_this_step = true;
        bvh_set = cur_set;
        full_this_step = bvh.act == nullptr;
    }
    if (mode == 1)
        point_boxes(d_xo, d_av, d_vscene, d_scenes, bvh.act ? d_act_p : nullptr, n_act_p, moving, d_pbox_lo,
                    d_pbox_hi, d_p32, d_v32, stream);
    prof(kStBvh, false);
    const bool dump = !vtk_dir.empty();
    if (dump)
        cudaMemcpyAsync(d_av_pre, d_av, sizeof(double4_32a) * (size_t)nv, cudaMemcpyDeviceToDevice, stream);
    for (int attempt = 0; attempt < 8; ++attempt) {
        count_launch(), k_reset_pass<<<(nscenes + 255) / 256, 256, 0, stream>>>(d_ctr, d_run, nscenes,
                                                                                reuse ? reuse_npairs : -1);
        if (!reuse) {
            prof(kStTraverse, true);
            bvh_pairs(d_box, on_full ? full_view() : bvh, d_pairs, pair_cap, d_ctr, stream, record ? nullptr : d_ev,
                      tune.traverse_block, combined ? d_box_st : nullptr, tune.packet_traverse, tune.rope_traverse,
                      tune.traverse_refill, tune.stack_depth);
            prof(kStTraverse, false);
            if (attempt == 0) {
                counters[16] += bvh.n;
                counters[19] += bvh.n;
            }
        }
        NarrowArgs a;
        a.robust_roots = robust_roots ? 1 : 0;
        a.sub_merge = sub_merge ? 1 : 0;
        a.xo = d_xo; a.av = d_av; a.fixed = d_fixed; a.ev = d_ev; a.esurf = d_esurf; a.erigid = d_erigid;
        a.vbody = d_vbody; a.body_mass = d_body_mass; a.body_slot0 = nv;
        a.rank = d_rank[moving]; a.escene = d_escene; a.scenes = d_scenes; a.run = d_run;
        a.pairs = d_pairs; a.contrib = d_contrib; a.contrib_cap = contrib_cap; a.ctr = d_ctr;
        a.urec = d_urec; a.urec_cap = urec_cap;
        a.rec = record ? d_rec : nullptr; a.rec_cap = rec_cap;
        a.pbox_lo = mode == 1 ? d_pbox_lo : nullptr;
        a.pbox_hi = mode == 1 ? d_pbox_hi : nullptr;
        a.p32 = d_p32;
        a.v32 = d_v32;
        a.check = 0;
        a.sub_pt = d_sub_pt;
        a.sub_ee = d_sub_ee;
        a.sub_cap = sub_cap;
        a.pair_hit = d_pair_hit;
        a.pairq = d_pairq;
        a.static_only = combined ? 1 : 0;
        // mixed passes without recording run in stages: per-pair FP32
        // filters, the surviving FP64 sub-tests densely, then the zone unions
        const bool split = mode == 1 && !record && split_narrow;
        if (split && moving && profiling) {
            prof(kStNarrowCcd, true);
            narrow_pass_split(a, moving, pair_cap, stream, tune.narrow_block, any_zone, kSplitFilter);
            prof(kStNarrowCcd, false);
            prof(kStSubtests, true);
            narrow_pass_split(a, moving, pair_cap, stream, tune.narrow_block, any_zone, kSplitSubtests);
            prof(kStSubtests, false);
        } else {
            prof(moving ? kStNarrowCcd : kStNarrowProx, true);
            if (split)
                narrow_pass_split(a, moving, pair_cap, stream, tune.narrow_block, any_zone);
            else
                narrow_pass(a, moving, pair_cap, stream, tune.narrow_block);
            prof(moving ? kStNarrowCcd : kStNarrowProx, false);
        }
        prof(kStApply, true);
        apply_contribs(d_contrib, d_ctr, contrib_cap, nv, d_av, d_hc, apply, stream, dump ? d_dump : nullptr,
                       bodies.empty() ? nullptr : &body_bufs);
        if (!bodies.empty())  // updateImpactZoneVelocityForRG (dcollid.cpp:744-745)
            zone_solve(d_body_members, d_body_zone_off, (int)bodies.size(), d_fixed, d_xo, d_av, d_vscene, d_scenes,
                       d_ctr, stream, d_run);
        prof(kStApply, false);
        cudaMemcpyAsync(h_ctr, d_ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(h_run, d_run, sizeof(SceneRun) * (size_t)nscenes, cudaMemcpyDeviceToHost, stream);
        if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("detection pass");
        int e = h_ctr->err;
        if (e & kErrNan) return fail(CC_NAN_DETECTED, "non-finite velocity or normal (the reference exits here)");
        if (e & kErrIndex) return fail(CC_CUDA_ERROR, index_error(e));
        if ((e & kErrStack) && tune.stack_depth < kTraversalStack) {
            tune.stack_depth = kTraversalStack;  // a tuned shallower stack was too shallow here
            continue;
        }
        if (e & kErrStack) return fail(CC_STACK_OVERFLOW, "BVH traversal stack overflow");
        if (e & kErrPairOverflow) {
            st = grow_pairs(2 * h_ctr->npairs + 1024);
            if (st) return st;
            continue;
        }
        if (e & kErrContribOverflow) {
            st = grow_contrib(2 * h_ctr->ncontrib + 1024);
            if (st) return st;
            continue;
        }
        if (e & kErrRecordOverflow) {
            st = grow_pairs(pair_cap);
            if (st) return st;
            continue;
        }
        if (e & kErrSubOverflow) {
            st = grow_subs(2 * std::max(h_ctr->nsub_pt, h_ctr->nsub_ee) + 1024);
            if (st) return st;
            continue;
        }
        if (e & kErrUnionOverflow) {
            st = grow_unions(2 * h_ctr->nunion + 1024);
            if (st) return st;
            continue;
        }
        break;
    }
    if (h_ctr->err) return fail(CC_PAIR_OVERFLOW, "buffers kept overflowing");
    if (combined && h_ctr->ncontrib == 0 && bodies.empty()) {
        // velocities unchanged (no impulse, no rigid-body motion): the swept
        // pairs hold for the next pass
        reuse_pairs = true;
        reuse_npairs = h_ctr->npairs;
        reuse_set = cur_set;
    }
    if (dump) {
        st = write_vtk_pass();
        if (st) return st;
    }
    counters[3] += h_ctr->npairs;
    // path bytes per pass: pairs written and read, per-point impulse,
    // friction and count records written and read for each contact
    if (pass_log)  // CC_PASS_LOG: one line per host-loop pass, for matching profiler launches to passes
        std::fprintf(stderr, "cc_pass moving=%d pairs=%d visits=%d sub_pt=%d sub_ee=%d contacts=%d\n", moving,
                     h_ctr->npairs, h_ctr->nvisits, h_ctr->nsub_pt, h_ctr->nsub_ee, h_ctr->ncontacts);
    counters[18] += 16ll * h_ctr->npairs + 4ll * 2 * 52 * h_ctr->ncontacts;
    counters[4] += h_ctr->nvisits;
    counters[5] += h_ctr->nhit_pairs;
    counters[6] += h_ctr->ncontacts;
    counters[12] += h_ctr->nsub;
    if (moving) counters[13] += h_ctr->nvisits;
    counters[15] += h_ctr->ncr;
    if (!reuse) {
        counters[17] += h_ctr->npairs;
        counters[20] += h_ctr->npairs;
    }
    if (record && h_ctr->nrec > 0) {
        size_t base = visits.size();
        visits.resize(base + (size_t)h_ctr->nrec);
        cudaMemcpyAsync(visits.data() + base, d_rec, sizeof(VisitRec) * (size_t)h_ctr->nrec,
                        cudaMemcpyDeviceToHost, stream);
    }
    if (any_zone) {
        prof(kStZone, true);
        const cudaError_t ez = zone_pass(zb, d_ctr, d_fixed, bvh.act ? d_act_p : nullptr, n_act_p, nullptr, d_vscene,
                                         d_run, d_scenes, d_av, d_xo, stream);
        if (ez != cudaSuccess) return fail(CC_CUDA_ERROR, std::string("zone pass: ") + cudaGetErrorString(ez));
        prof(kStZone, false);
        cudaMemcpyAsync(h_ctr, d_ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, stream);
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("pass tail");
    if (h_ctr->err & kErrNan) return fail(CC_NAN_DETECTED, "non-finite zone velocity (the reference exits here)");
    return CC_OK;
}

cc_status cc_solver::resolve(const double* x_old, const double* x_cand, double* vel, uint8_t* hc, double* x_out,
                             int* has_collision) {
    long long l0 = g_kernel_launches;
    cc_status st0 = resolve_impl(x_old, x_cand, vel, hc, x_out, has_collision);
    launches_last = g_kernel_launches - l0;
    return st0;
}

// resolveCollision (dcollid.cpp:317-362) for every scene: has_collision
// receives one flag per scene.
cc_status cc_solver::resolve_impl(const double* x_old, const double* x_cand, double* vel, uint8_t* hc,
                                  double* x_out, int* has_collision) {
    std::memset(counters, 0, sizeof(counters));
    visits.clear();
    if (has_collision)
        for (int s = 0; s < nscenes; ++s) has_collision[s] = 0;
    for (auto& sh : scenes) {
        sh.pass_kinds.clear();
        sh.state = (sh.ne > 0 && sh.enabled) ? kHsProx : kHsDone;
        // path bytes per scene-step: x_old, x_cand, v read; x, v written
        if (sh.enabled) counters[18] += 120ll * sh.nv;
        sh.niter = sh.cd_count = sh.zone_it = sh.hcol = sh.npass = 0;
        sh.status = CC_OK;
    }
    std::string capped;
    if (ne == 0) {
        // the reference dereferences an empty tree here; nothing collides
        if (nv) cudaMemcpyAsync(x_out, x_cand, sizeof(double) * 3 * (size_t)nv, cudaMemcpyDeviceToDevice, stream);
        start_zones();
        cudaStreamSynchronize(stream);
        return cuda_check("empty mesh");
    }
    upload_scenes();
    // d_hc doubles as the device copy of has_collsn
    if (hc != d_hc) cudaMemcpyAsync(d_hc, hc, (size_t)nv, cudaMemcpyDeviceToDevice, stream);
    count_launch(), k_reset_counters<<<1, 1, 0, stream>>>(d_ctr);
    cudaMemsetAsync(&d_ctr->err, 0, sizeof(int), stream);
    ev_marks.clear();
    prof(kStInit, true);
    step_init(x_old, x_cand, nv, d_in_elem, d_vscene, d_scenes, d_xo, d_av, d_ctr, stream);
    // the strain records depend on x_old only
    strain_setup(d_edges, nedges, d_scenes, strain_plan(), d_xo, d_strain_step, d_vscene, stream);
    tail_done.assign((size_t)nscenes, 0);
    tails_this_step = 0;
    start_zones();
    bvh_this_step = false;
    full_this_step = false;
    reuse_pairs = false;
    prof(kStInit, false);
    if (use_device_loop()) {
        cc_status st = device_passes(capped);
        if (st) return st;
    }
    for (bool first = true; !use_device_loop(); first = false) {
        bool any = false, any_zone = false;
        for (int s = 0; s < nscenes; ++s) {
            SceneHost& sh = scenes[s];
            int m = kSceneIdle;
            if (sh.state == kHsProx) {
                m = kSceneProx;
            } else if (sh.state == kHsCcd) {
                m = kSceneCcd;
            } else if (sh.state == kHsZone) {
                if (sh.zone_it++ >= zone_cap) {
                    // the reference would loop on; this scene stops here and
                    // is finished with its current velocities
                    sh.status = CC_ITER_CAP;
                    sh.state = kHsDone;
                    capped += (capped.empty() ? "" : " ") + std::to_string(s);
                } else {
                    m = kSceneZone;
                }
            }
            h_run[s] = SceneRun{m, 0, sh.npass, -1, -1, {0, 0, 0}};
            if (m == kSceneIdle) continue;
            any = true;
            any_zone |= m == kSceneZone;
            sh.npass++;
            sh.pass_kinds.push_back(m == kSceneProx ? kPassProx : m == kSceneCcd ? kPassCcd : kPassZone);
            counters[0]++;
            if (m == kSceneCcd) counters[1]++;
            if (m == kSceneZone) counters[2]++;
            // path bytes per scene-pass: x_old and avgVel read, connectivity,
            // the FP32 hierarchy written by the refit and read once by the
            // traversal, avgVel updated; a zone pass reads the state again
            counters[18] += 72ll * sh.nv + 12ll * sh.nt + 8ll * (sh.ne - sh.nt) + 48ll * (2ll * sh.ne - 1) +
                            (m == kSceneZone ? 48ll * sh.nv : 0ll);
        }
        if (!any) break;
        // proximity is every scene's first pass, so a pass is all static or all moving
        cc_status st = detect_pass(first ? 0 : 1, any_zone);
        if (st) return st;
        for (int s = 0; s < nscenes; ++s) {
            SceneHost& sh = scenes[s];
            bool is_coll = h_run[s].hits > 0;
            switch (sh.state) {
                case kHsProx:  // is_collision = true; niter = 1 (dcollid.cpp:333-336)
                    sh.state = kHsCcd;
                    sh.niter = 1;
                    sh.cd_count = 0;
                    break;
                case kHsCcd:  // dcollid.cpp:337-344
                    if (sh.cd_count++ == 0 && is_coll) sh.hcol = 1;
                    if (!is_coll)
                        sh.state = kHsDone;
                    else if (++sh.niter > kMaxCcdIter)
                        sh.state = kHsZone;  // dcollid.cpp:346-352
                    break;
                case kHsZone:
                    if (!is_coll) sh.state = kHsDone;
                    break;
                default:
                    break;
            }
        }
        if (overlap_tails) {
            // once half the scenes have finished, they end their step now,
            // beside the passes of the others (finalize, strain limiting,
            // final velocities: one graph, whose strain loop ends on the
            // device)
            cc_status st = launch_tail(x_cand, x_out, vel, false);
            if (st) return st;
        }
    }
    {
        cc_status st = launch_tail(x_cand, x_out, vel, true);
        if (st) return st;
    }
    cudaEventRecord(ev_tail, tail_stream);
    cudaStreamWaitEvent(stream, ev_tail, 0);
    if (hc != d_hc) cudaMemcpyAsync(hc, d_hc, (size_t)nv, cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(h_strain_passes.data(), d_strain_passes, sizeof(int) * h_strain_passes.size(),
                    cudaMemcpyDeviceToHost, stream);
    if (!bodies.empty()) {
        final_rigid(body_bufs, d_hc, d_av, stream);
        cudaMemcpyAsync(h_body_out.data(), d_body_out, sizeof(double4_32a) * bodies.size(), cudaMemcpyDeviceToHost,
                        stream);
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("finalize");
    // updateFinalForRG (dcollid.cpp:626-675): a body with a collided point
    // takes that point's velocity, and its centre of mass moves from the
    // remembered one (if that point is the body's first) or the current one
    for (size_t b = 0; b < bodies.size(); ++b) {
        BodyHost& B = bodies[b];
        if (!scenes[B.scene].enabled) continue;
        if (!B.mrg_set) {
            std::copy(B.com, B.com + 3, B.mrg_com);
            B.mrg_set = true;
        }
        const double4_32a o = h_body_out[b];
        const int p = (int)o.w;
        if (p >= 0) {
            const double dt = h_scenes[B.scene].p.dt;
            const double* base = (p == h_body_visit[h_body_visit_off[b]]) ? B.mrg_com : B.com;
            const double v[3] = {o.x, o.y, o.z};
            double com[3];
            for (int j = 0; j < 3; ++j) com[j] = v[j] * dt + base[j];
            for (int j = 0; j < 3; ++j) {
                B.comv[j] = v[j];
                B.com[j] = com[j];
            }
        }
        std::copy(B.com, B.com + 3, B.mrg_com);
    }
    for (int s = 0; s < nscenes; ++s) {
        // algorithmic bytes of the sweep: per pass, each edge's 48-byte
        // record and one 32-byte read and write of each point it touches
        counters[14] += (long long)h_strain_passes[3 * s] *
                        (48ll * scenes[s].strain_edges + 64ll * scenes[s].strain_points);
        // path bytes per strain pass: points read and written, each
        // element edge (three per triangle, one per bond) read
        counters[18] += (long long)h_strain_passes[3 * s] *
                        (48ll * scenes[s].nv + 24ll * (3ll * scenes[s].nt + (scenes[s].ne - scenes[s].nt)));
        counters[7] += h_strain_passes[3 * s];
        counters[10] += h_strain_passes[3 * s + 1];
        counters[11] += h_strain_passes[3 * s + 2];
    }
    prof_collect();
    if (has_collision)
        for (int s = 0; s < nscenes; ++s) has_collision[s] = scenes[s].hcol;
    cc_status st = cuda_check("resolve");
    if (st) return st;
    if (!capped.empty())
        return fail(CC_ITER_CAP, "impact-zone loop did not converge within the cap in scene(s) " + capped +
                                     "; their step was finished with the last velocities");
    return CC_OK;
}

// Exact FP64 re-check of a finished step: every element pair whose swept
// boxes over [x_old, x_new] overlap goes through the reference's CCD
// predicate (isCoplanar, then the point-triangle / edge-edge tests with
// h = eps at each root and at dt; dcollid3d.cpp:203-482, 643-922) with
// avgVel = (x_new - x_old)/dt, as the next step's first CCD pass would see
// it, without impulses or zones. A pair that still hits is a missed
// collision. Uses the solver's pass buffers; the step's state is replaced.
cc_status cc_solver::check_ccd(const double* x_old, const double* x_new, long long* hits, int* scene_hits) {
    if (hits) *hits = 0;
    if (scene_hits)
        for (int s = 0; s < nscenes; ++s) scene_hits[s] = 0;
    if (ne == 0) return CC_OK;
    upload_scenes();
    count_launch(), k_reset_counters<<<1, 1, 0, stream>>>(d_ctr);
    cudaMemsetAsync(&d_ctr->err, 0, sizeof(int), stream);
    step_init(x_old, x_new, nv, d_in_elem, d_vscene, d_scenes, d_xo, d_av, d_ctr, stream);
    for (int s = 0; s < nscenes; ++s)
        h_run[s] = SceneRun{scenes[s].ne > 0 ? kSceneCcd : kSceneIdle, 0, 0, -1, -1, {0, 0, 0}};
    select_active();
    cudaMemcpyAsync(d_run, h_run, sizeof(SceneRun) * (size_t)nscenes, cudaMemcpyHostToDevice, stream);
    leaf_boxes(d_ev, bvh.act, bvh.n, d_escene, d_scenes, nscenes, d_xo, d_av, 1, d_box, bvh.bbox_enc, stream);
    bvh_this_step = false;  // the pass hierarchy and pairs are replaced
    full_this_step = false;
    reuse_pairs = false;
    bvh_build(d_box, bvh, stream);
    for (int attempt = 0; attempt < 8; ++attempt) {
        count_launch(), k_reset_pass<<<(nscenes + 255) / 256, 256, 0, stream>>>(d_ctr, d_run, nscenes);
        bvh_pairs(d_box, bvh, d_pairs, pair_cap, d_ctr, stream, d_ev, tune.traverse_block, nullptr,
                  tune.packet_traverse, tune.rope_traverse, tune.traverse_refill, kTraversalStack);
        NarrowArgs a{};
        a.robust_roots = robust_roots ? 1 : 0;
        a.sub_merge = sub_merge ? 1 : 0;
        a.xo = d_xo; a.av = d_av; a.fixed = d_fixed; a.ev = d_ev; a.esurf = d_esurf; a.erigid = d_erigid;
        a.vbody = d_vbody; a.body_mass = d_body_mass; a.body_slot0 = nv;
        a.rank = nullptr; a.escene = d_escene; a.scenes = d_scenes; a.run = d_run;
        a.pairs = d_pairs; a.contrib = d_contrib; a.contrib_cap = contrib_cap; a.ctr = d_ctr;
        a.urec = nullptr; a.urec_cap = 0;
        a.rec = nullptr; a.rec_cap = 0; a.pbox_lo = nullptr; a.pbox_hi = nullptr;
        a.check = 1;
        narrow_pass(a, 1, pair_cap, stream);
        cudaMemcpyAsync(h_ctr, d_ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(h_run, d_run, sizeof(SceneRun) * (size_t)nscenes, cudaMemcpyDeviceToHost, stream);
        if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("ccd check");
        if (h_ctr->err & kErrPairOverflow) {
            cc_status st = grow_pairs(2 * h_ctr->npairs + 1024);
            if (st) return st;
            continue;
        }
        break;
    }
    int e = h_ctr->err;
    if (e & kErrNan) return fail(CC_NAN_DETECTED, "non-finite velocity or normal in the CCD check");
    if (e & kErrIndex) return fail(CC_CUDA_ERROR, index_error(e));
    if (e & kErrStack) return fail(CC_STACK_OVERFLOW, "BVH traversal stack overflow");
    if (e) return fail(CC_PAIR_OVERFLOW, "buffers kept overflowing");
    if (hits) *hits = h_ctr->nhit_pairs;
    if (scene_hits)
        for (int s = 0; s < nscenes; ++s) scene_hits[s] = h_run[s].hits;
    return cuda_check("ccd check");
}

// Launch-shape autotuner. On the state of the last step (x_old and the
// final average velocities), one moving pass of every scene - leaf boxes,
// a full LBVH build, then the traversal and the narrow phase - is timed for
// each candidate traversal block size, narrow-phase variant (two-stage or
// one kernel, mixed precision only) and filter block size; impulses are not
// applied, so the state is unchanged. The fastest setting is kept, and the
// pair and sub-test buffers are grown to what the pass needed plus a
// quarter, so that the passes that follow do not overflow and retry.
cc_status cc_solver::autotune(double* best_ms) {
    if (best_ms) *best_ms = 0.0;
    if (ne == 0) return CC_OK;
    upload_scenes();
    for (int s = 0; s < nscenes; ++s)
        h_run[s] = SceneRun{scenes[s].ne > 0 && scenes[s].enabled ? kSceneCcd : kSceneIdle, 0, 0, -1, -1, {0, 0, 0}};
    select_active();
    cudaMemcpyAsync(d_run, h_run, sizeof(SceneRun) * (size_t)nscenes, cudaMemcpyHostToDevice, stream);
    leaf_boxes(d_ev, bvh.act, bvh.n, d_escene, d_scenes, nscenes, d_xo, d_av, 1, d_box, bvh.bbox_enc, stream);
    bvh_this_step = false;
    full_this_step = false;
    reuse_pairs = false;
    bvh_build(d_box, bvh, stream);
    if (mode == 1)
        point_boxes(d_xo, d_av, d_vscene, d_scenes, bvh.act ? d_act_p : nullptr, n_act_p, 1, d_pbox_lo, d_pbox_hi,
                    d_p32, d_v32, stream);
    // ranks only orient pairs here; any tree's will do for timing
    const int* rank = d_rank[1];
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto run_once = [&](const LaunchTuning& t, bool split, float* ms) -> cc_status {
        for (int attempt = 0; attempt < 8; ++attempt) {
            count_launch(), k_reset_pass<<<(nscenes + 255) / 256, 256, 0, stream>>>(d_ctr, d_run, nscenes);
            cudaEventRecord(e0, stream);
            bvh_pairs(d_box, bvh, d_pairs, pair_cap, d_ctr, stream, d_ev, t.traverse_block, nullptr,
                      t.packet_traverse, t.rope_traverse, t.traverse_refill, t.stack_depth);
            NarrowArgs a{};
            a.robust_roots = robust_roots ? 1 : 0;
            a.sub_merge = sub_merge ? 1 : 0;
            a.xo = d_xo; a.av = d_av; a.fixed = d_fixed; a.ev = d_ev; a.esurf = d_esurf; a.erigid = d_erigid;
        a.vbody = d_vbody; a.body_mass = d_body_mass; a.body_slot0 = nv;
            a.rank = rank; a.escene = d_escene; a.scenes = d_scenes; a.run = d_run;
            a.pairs = d_pairs; a.contrib = d_contrib; a.contrib_cap = contrib_cap; a.ctr = d_ctr;
            a.urec = d_urec; a.urec_cap = urec_cap;
            a.pbox_lo = mode == 1 ? d_pbox_lo : nullptr;
            a.pbox_hi = mode == 1 ? d_pbox_hi : nullptr;
            a.p32 = d_p32; a.v32 = d_v32;
            a.sub_pt = d_sub_pt; a.sub_ee = d_sub_ee; a.sub_cap = sub_cap; a.pair_hit = d_pair_hit;
            a.pairq = d_pairq;
            if (split)
                narrow_pass_split(a, 1, pair_cap, stream, t.narrow_block);
            else
                narrow_pass(a, 1, pair_cap, stream, t.narrow_block);
            cudaEventRecord(e1, stream);
            cudaMemcpyAsync(h_ctr, d_ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, stream);
            if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("autotune");
            int e = h_ctr->err;
            if (e & kErrPairOverflow) {
                cc_status st = grow_pairs(h_ctr->npairs + h_ctr->npairs / 4 + 1024);
                if (st) return st;
                continue;
            }
            if (e & kErrContribOverflow) {
                cc_status st = grow_contrib(h_ctr->ncontrib + h_ctr->ncontrib / 4 + 1024);
                if (st) return st;
                continue;
            }
            if (e & kErrSubOverflow) {
                int need = std::max(h_ctr->nsub_pt, h_ctr->nsub_ee);
                cc_status st = grow_subs(need + need / 4 + 1024);
                if (st) return st;
                continue;
            }
            if (e & kErrUnionOverflow) {
                cc_status st = grow_unions(h_ctr->nunion + h_ctr->nunion / 4 + 1024);
                if (st) return st;
                continue;
            }
            if (e & kErrIndex) return fail(CC_CUDA_ERROR, "autotune: " + index_error(e));
            if ((e & kErrStack) && t.stack_depth < kTraversalStack && !t.rope_traverse) {
                *ms = 1e30f;  // too shallow a stack for this state: not a candidate
                return CC_OK;
            }
            if (e & (kErrStack | kErrNan)) return fail(CC_STACK_OVERFLOW, "autotune pass failed");
            cudaEventElapsedTime(ms, e0, e1);
            return CC_OK;
        }
        return fail(CC_PAIR_OVERFLOW, "autotune: buffers kept overflowing");
    };
    auto time_it = [&](const LaunchTuning& t, bool split, float* best) -> cc_status {
        float m = 0.f, b = 1e30f;
        for (int r = 0; r < 3; ++r) {
            cc_status st = run_once(t, split, &m);
            if (st) return st;
            b = std::min(b, m);
        }
        *best = b;
        return CC_OK;
    };
    LaunchTuning best_t = tune;
    bool best_split = split_narrow && mode == 1;  // the staged pass needs the FP32 point data of mode 1
    float best = 1e30f;
    cc_status st = time_it(best_t, best_split, &best);  // the current setting, which also sizes the buffers
    const int tb[] = {64, 128, 256, 512};
    const int nb[] = {64, 128, 256};
    const int refills[] = {4, 8, 16, 32};
    const int depths[] = {24, 32, 48, 64};
    // the stackless traversal with dynamic query fetch (lanes refilling
    // together), and with one thread per query over the block sizes
    for (int r : refills) {
        LaunchTuning t = best_t;
        t.rope_traverse = true;
        t.traverse_refill = r;
        float m;
        if (!st) st = time_it(t, best_split, &m);
        if (!st && m < best) { best = m; best_t = t; }
    }
    for (int a : tb) {
        LaunchTuning t = best_t;
        t.rope_traverse = true;
        t.traverse_refill = 0;
        t.traverse_block = a;
        float m;
        if (!st) st = time_it(t, best_split, &m);
        if (!st && m < best) { best = m; best_t = t; }
    }
    // the traversal with a stack per thread: block size, then stack depth
    // (the warp packets are slower on cloth)
    for (int a : tb) {
        LaunchTuning t = best_t;
        t.rope_traverse = false;
        t.traverse_block = a;
        t.stack_depth = kTraversalStack;
        float m;
        if (!st) st = time_it(t, best_split, &m);
        if (!st && m < best) { best = m; best_t = t; }
    }
    if (!best_t.rope_traverse)
        for (int d : depths) {
            LaunchTuning t = best_t;
            t.stack_depth = d;
            float m;
            if (!st) st = time_it(t, best_split, &m);
            if (!st && m < best) { best = m; best_t = t; }
        }
    for (int split = (mode == 1 ? 0 : 1); split <= (mode == 1 ? 1 : 0) && !st; ++split) {
        for (int b : nb) {
            LaunchTuning t = best_t;
            t.narrow_block = b;
            float m;
            st = time_it(t, split != 0, &m);
            if (st) break;
            if (m < best) { best = m; best_t = t; best_split = split != 0; }
            if (!split) break;  // the one-kernel pass has a fixed block
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    tune = best_t;
    if (mode == 1) split_narrow = best_split;
    if (best_ms) *best_ms = best;
    return cuda_check("autotune");
}

namespace {

cc_status copy_in_and_resolve(cc_solver* s, const double* x_old, const double* x_cand, double* vel,
                              uint8_t* has_collsn, double* x_out, int* has_collision) {
    if (s->nv && (!x_old || !x_cand || !vel || !has_collsn || !x_out)) return s->fail(CC_BAD_INPUT, "null array");
    cudaSetDevice(s->device);
    size_t b3 = sizeof(double) * 3 * (size_t)s->nv;
    if (s->nv) {
        cudaMemcpyAsync(s->d_xold_in, x_old, b3, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->d_xcand_in, x_cand, b3, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->d_vel, vel, b3, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->d_hc, has_collsn, (size_t)s->nv, cudaMemcpyHostToDevice, s->stream);
    }
    cc_status st = s->resolve(s->d_xold_in, s->d_xcand_in, s->d_vel, s->d_hc, s->d_xout, has_collision);
    // a scene stopped at the zone cap still completes the call's outputs
    if (st != CC_OK && st != CC_ITER_CAP) return st;
    if (s->nv) {
        cudaMemcpyAsync(x_out, s->d_xout, b3, cudaMemcpyDeviceToHost, s->stream);
        cudaMemcpyAsync(vel, s->d_vel, b3, cudaMemcpyDeviceToHost, s->stream);
        cudaMemcpyAsync(has_collsn, s->d_hc, (size_t)s->nv, cudaMemcpyDeviceToHost, s->stream);
    }
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return s->cuda_check("read back");
    return st;
}

// has_collision of a whole solver: any scene's.
cc_status resolve_any(cc_solver* s, bool host, const double* x_old, const double* x_cand, double* vel,
                      uint8_t* has_collsn, double* x_out, int* has_collision) {
    std::vector<int> flags((size_t)(s->nscenes > 0 ? s->nscenes : 1), 0);
    cc_status st = host ? copy_in_and_resolve(s, x_old, x_cand, vel, has_collsn, x_out, flags.data())
                        : (cudaSetDevice(s->device), s->resolve(x_old, x_cand, vel, has_collsn, x_out, flags.data()));
    if (has_collision) {
        *has_collision = 0;
        for (int f : flags) *has_collision |= f;
    }
    return st;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

cc_status cc_create(int device, cc_solver** out) {
    if (!out) return CC_BAD_INPUT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return CC_CUDA_ERROR;
    cc_solver* s = new cc_solver;
    s->device = device;
    cudaSetDevice(device);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->tail_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_pass, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_tail, cudaEventDisableTiming) != cudaSuccess ||
        dalloc(&s->d_ctr, 1) != cudaSuccess || cudaMallocHost(&s->h_ctr, sizeof(PassCounters)) != cudaSuccess) {
        delete s;
        return CC_CUDA_ERROR;
    }
    cudaMemset(s->d_ctr, 0, sizeof(PassCounters));
    *out = s;
    return CC_OK;
}

void cc_destroy(cc_solver* s) { delete s; }

cc_status cc_assemble(cc_solver* s, const cc_mesh* mesh) {
    if (!s) return CC_BAD_INPUT;
    if (!mesh) return s->fail(CC_BAD_INPUT, "no mesh");
    return s->assemble(mesh, 1);
}

cc_status cc_assemble_batch(cc_solver* s, const cc_mesh* meshes, int n_scenes) {
    if (!s) return CC_BAD_INPUT;
    return s->assemble(meshes, n_scenes);
}

int cc_num_scenes(cc_solver* s) { return s ? s->nscenes : -1; }

cc_status cc_get_scene_offsets(cc_solver* s, int32_t* point_off, int32_t* elem_off) {
    if (!s) return CC_BAD_INPUT;
    for (int i = 0; i < s->nscenes; ++i) {
        if (point_off) point_off[i] = s->scenes[i].v0;
        if (elem_off) elem_off[i] = s->scenes[i].e0;
    }
    if (point_off) point_off[s->nscenes] = s->nv;
    if (elem_off) elem_off[s->nscenes] = s->ne;
    return CC_OK;
}

cc_status cc_set_params(cc_solver* s, const cc_params* p) {
    if (!s || !p) return CC_BAD_INPUT;
    s->prm = *p;
    for (int i = 0; i < s->nscenes; ++i) s->set_scene_params(i, *p);
    return CC_OK;
}

cc_status cc_set_scene_params(cc_solver* s, int scene, const cc_params* p) {
    if (!s || !p || scene < 0 || scene >= s->nscenes) return CC_BAD_INPUT;
    s->set_scene_params(scene, *p);
    return CC_OK;
}

cc_status cc_set_domain_boundary(cc_solver* s, const double lo[3], const double hi[3]) {
    if (!s || !lo || !hi) return CC_BAD_INPUT;
    for (int d = 0; d < 3; ++d) {
        s->lo[d] = lo[d];
        s->hi[d] = hi[d];
    }
    for (int i = 0; i < s->nscenes; ++i) s->set_scene_domain(i, lo, hi);
    return CC_OK;
}

cc_status cc_set_scene_domain_boundary(cc_solver* s, int scene, const double lo[3], const double hi[3]) {
    if (!s || !lo || !hi || scene < 0 || scene >= s->nscenes) return CC_BAD_INPUT;
    s->set_scene_domain(scene, lo, hi);
    return CC_OK;
}

cc_status cc_resolve(cc_solver* s, const double* x_old, const double* x_cand, double* vel, uint8_t* has_collsn,
                     double* x_out, int* has_collision) {
    if (!s) return CC_BAD_INPUT;
    return resolve_any(s, true, x_old, x_cand, vel, has_collsn, x_out, has_collision);
}

cc_status cc_resolve_device(cc_solver* s, const double* x_old, const double* x_cand, double* vel,
                            uint8_t* has_collsn, double* x_out, int* has_collision) {
    if (!s) return CC_BAD_INPUT;
    return resolve_any(s, false, x_old, x_cand, vel, has_collsn, x_out, has_collision);
}

cc_status cc_resolve_batch(cc_solver* s, const double* x_old, const double* x_cand, double* vel,
                           uint8_t* has_collsn, double* x_out, int* has_collision) {
    if (!s) return CC_BAD_INPUT;
    return copy_in_and_resolve(s, x_old, x_cand, vel, has_collsn, x_out, has_collision);
}

cc_status cc_resolve_batch_device(cc_solver* s, const double* x_old, const double* x_cand, double* vel,
                                  uint8_t* has_collsn, double* x_out, int* has_collision) {
    if (!s) return CC_BAD_INPUT;
    cudaSetDevice(s->device);
    return s->resolve(x_old, x_cand, vel, has_collsn, x_out, has_collision);
}

cc_status cc_check_ccd(cc_solver* s, const double* x_old, const double* x_new, long long* hits, int* scene_hits) {
    if (!s) return CC_BAD_INPUT;
    if (s->nv && (!x_old || !x_new)) return s->fail(CC_BAD_INPUT, "null array");
    cudaSetDevice(s->device);
    return s->check_ccd(x_old, x_new, hits, scene_hits);
}

cc_status cc_autotune(cc_solver* s, double* best_ms) {
    if (!s) return CC_BAD_INPUT;
    cudaSetDevice(s->device);
    return s->autotune(best_ms);
}

cc_status cc_set_tuning(cc_solver* s, int knob, int value) {
    if (!s) return CC_BAD_INPUT;
    s->loop_dirty = true;
    switch (knob) {
        case CC_TUNE_SPLIT_NARROW:
            s->split_narrow = value != 0;
            return CC_OK;
        case CC_TUNE_TAIL_GRAPH:
            s->tail_graphs_on = value != 0;
            return CC_OK;
        case CC_TUNE_COMBINED_BROAD:
            s->combined_broad = value != 0;
            return CC_OK;
        case CC_TUNE_STRAIN_WARP:
            s->strain_warp = value != 0;
            return CC_OK;
        case CC_TUNE_PACKET_TRAVERSE:
            s->tune.packet_traverse = value != 0;
            return CC_OK;
        case CC_TUNE_STRAIN_ROLES:
            s->strain_roles = value != 0;
            return CC_OK;
        case CC_TUNE_TAIL_OVERLAP:
            s->overlap_tails = value != 0;
            return CC_OK;
        case CC_TUNE_ROPE_TRAVERSE:
            s->tune.rope_traverse = value != 0;
            return CC_OK;
        case CC_TUNE_SUBSET_REFIT:
            s->subset_refit = value != 0;
            return CC_OK;
        case CC_TUNE_DEVICE_LOOP:
            s->device_loop = value != 0;
            return CC_OK;
        case CC_TUNE_PRUNE:
            s->prune = value != 0;
            return CC_OK;
        case CC_TUNE_HOST_TREE:
            s->host_tree = value != 0;
            return CC_OK;
        case CC_TUNE_SMALL_SORT:
            s->zb.small_sort = value != 0;
            s->loop_dirty = true;
            return CC_OK;
        case CC_TUNE_PRUNED_WARP:
            s->pruned_warp = value != 0;
            s->loop_dirty = true;
            return CC_OK;
        case CC_TUNE_ROBUST_ROOTS:
            s->robust_roots = value != 0;
            s->loop_dirty = true;
            return CC_OK;
        case CC_TUNE_ZONE_CTA_MIN:
            if (value < 16) return CC_BAD_INPUT;
            s->zb.zone_cta_min = value;
            s->loop_dirty = true;
            return CC_OK;
        case CC_TUNE_REPLAY_CTA_MIN:
            if (value < 0) return CC_BAD_INPUT;
            s->zb.replay_cta_min = value;
            s->loop_dirty = true;
            return CC_OK;
        case CC_TUNE_SUBTEST_MERGE:
            s->sub_merge = value != 0;
            s->loop_dirty = true;
            return CC_OK;
        case CC_TUNE_ZONE_FEW:
            if (value < 0) return CC_BAD_INPUT;
            s->zb.zone_few = value;
            s->loop_dirty = true;
            return CC_OK;
        case CC_TUNE_REFIT_UP:
            s->refit_up = value != 0;
            s->bvh.refit_up = s->refit_up ? 1 : 0;
            s->loop_dirty = true;
            return CC_OK;
        case CC_TUNE_TRAVERSE_REFILL:
            if (value < 0 || value > 32) return CC_BAD_INPUT;
            s->tune.traverse_refill = value;
            return CC_OK;
        case CC_TUNE_STACK_DEPTH:
            if (value != 24 && value != 32 && value != 48 && value != 64) return CC_BAD_INPUT;
            s->tune.stack_depth = value;
            return CC_OK;
        case CC_TUNE_PAIR_CAPACITY:
            if (value < 4096) return CC_BAD_INPUT;
            cudaSetDevice(s->device);
            cudaStreamSynchronize(s->stream);
            return s->grow_pairs(value);
        case CC_TUNE_STRAIN_BLOCK:
            if (value < 32 || value > 256 || value % 32) return CC_BAD_INPUT;
            s->tune.strain_block = value;
            return CC_OK;
        case CC_TUNE_TRAVERSE_BLOCK:
        case CC_TUNE_NARROW_BLOCK:
            if (value < 32 || value > (knob == CC_TUNE_NARROW_BLOCK ? 512 : 1024) || value % 32) return CC_BAD_INPUT;
            (knob == CC_TUNE_TRAVERSE_BLOCK ? s->tune.traverse_block : s->tune.narrow_block) = value;
            return CC_OK;
        default:
            return CC_BAD_INPUT;
    }
}

int cc_get_tuning(cc_solver* s, int knob) {
    if (!s) return -1;
    switch (knob) {
        case CC_TUNE_SPLIT_NARROW: return s->split_narrow ? 1 : 0;
        case CC_TUNE_TRAVERSE_BLOCK: return s->tune.traverse_block;
        case CC_TUNE_NARROW_BLOCK: return s->tune.narrow_block;
        case CC_TUNE_STRAIN_BLOCK: return s->tune.strain_block;
        case CC_TUNE_TAIL_GRAPH: return s->tail_graphs_on ? 1 : 0;
        case CC_TUNE_COMBINED_BROAD: return s->combined_broad ? 1 : 0;
        case CC_TUNE_STRAIN_WARP: return s->strain_warp ? 1 : 0;
        case CC_TUNE_PACKET_TRAVERSE: return s->tune.packet_traverse ? 1 : 0;
        case CC_TUNE_STRAIN_ROLES: return s->strain_roles ? 1 : 0;
        case CC_TUNE_TAIL_OVERLAP: return s->overlap_tails ? 1 : 0;
        case CC_TUNE_ROPE_TRAVERSE: return s->tune.rope_traverse ? 1 : 0;
        case CC_TUNE_SUBSET_REFIT: return s->subset_refit ? 1 : 0;
        case CC_TUNE_TRAVERSE_REFILL: return s->tune.traverse_refill;
        case CC_TUNE_DEVICE_LOOP: return s->device_loop ? 1 : 0;
        case CC_TUNE_PRUNE: return s->prune ? 1 : 0;
        case CC_TUNE_HOST_TREE: return s->host_tree ? 1 : 0;
        case CC_TUNE_SMALL_SORT: return s->zb.small_sort ? 1 : 0;
        case CC_TUNE_PRUNED_WARP: return s->pruned_warp ? 1 : 0;
        case CC_TUNE_ROBUST_ROOTS: return s->robust_roots ? 1 : 0;
        case CC_TUNE_ZONE_CTA_MIN: return s->zb.zone_cta_min;
        case CC_TUNE_REPLAY_CTA_MIN: return s->zb.replay_cta_min;
        case CC_TUNE_REFIT_UP: return s->refit_up ? 1 : 0;
        case CC_TUNE_ZONE_FEW: return s->zb.zone_few;
        case CC_TUNE_SUBTEST_MERGE: return s->sub_merge ? 1 : 0;
        case CC_TUNE_STACK_DEPTH: return s->tune.stack_depth;
        case CC_TUNE_PAIR_CAPACITY: return s->pair_cap;
        default: return -1;
    }
}

cc_status cc_set_vtk_dump(cc_solver* s, const char* dir) {
    if (!s) return CC_BAD_INPUT;
    cudaSetDevice(s->device);
    s->vtk_dir = dir ? dir : "";
    if (s->vtk_dir.empty()) return CC_OK;
    mkdir(s->vtk_dir.c_str(), 0755);  // as create_directory(fname, NO), dcollid.cpp:689
    struct stat sb;
    if (stat(s->vtk_dir.c_str(), &sb) != 0 || !S_ISDIR(sb.st_mode)) {
        s->vtk_dir.clear();
        return s->fail(CC_BAD_INPUT, "cannot create the dump directory");
    }
    bool ok = true;
    if (!s->d_dump) ok &= dalloc(&s->d_dump, (size_t)s->nv) == cudaSuccess;
    if (!s->d_av_pre) ok &= dalloc(&s->d_av_pre, (size_t)s->nv) == cudaSuccess;
    if (!ok) return s->fail(CC_NO_MEMORY, "dump buffers");
    return CC_OK;
}

cc_status cc_set_body(cc_solver* s, int scene, int surface, double mass, const double* com, const double* comv) {
    if (!s || !com || !comv) return CC_BAD_INPUT;
    const int b = s->find_body(scene, surface);
    if (b < 0) return s->fail(CC_BAD_INPUT, "no movable surface with that id in the scene");
    auto& B = s->bodies[(size_t)b];
    B.mass = mass;
    for (int j = 0; j < 3; ++j) {
        B.com[j] = com[j];
        B.comv[j] = comv[j];
    }
    if (!B.mrg_set) {
        std::copy(com, com + 3, B.mrg_com);
        B.mrg_set = true;
    }
    s->upload_body_mass();
    return s->cuda_check("set body");
}

cc_status cc_get_body(cc_solver* s, int scene, int surface, double* com, double* comv) {
    if (!s || !com || !comv) return CC_BAD_INPUT;
    const int b = s->find_body(scene, surface);
    if (b < 0) return s->fail(CC_BAD_INPUT, "no movable surface with that id in the scene");
    const auto& B = s->bodies[(size_t)b];
    for (int j = 0; j < 3; ++j) {
        com[j] = B.com[j];
        comv[j] = B.comv[j];
    }
    return CC_OK;
}

cc_status cc_set_zone_cap(cc_solver* s, int cap) {
    if (!s || cap < 0) return CC_BAD_INPUT;
    s->zone_cap = cap;
    return CC_OK;
}

cc_status cc_set_scene_enabled(cc_solver* s, int scene, int on) {
    if (!s || scene < 0 || scene >= s->nscenes) return CC_BAD_INPUT;
    s->scenes[scene].enabled = on != 0;
    s->h_scenes[scene].enabled = on != 0;
    s->scenes_dirty = true;
    return CC_OK;
}

cc_status cc_get_scene_status(cc_solver* s, int* out) {
    if (!s || !out) return CC_BAD_INPUT;
    for (int i = 0; i < s->nscenes; ++i) out[i] = s->scenes[i].status;
    return CC_OK;
}

cc_status cc_set_host_threads(cc_solver* s, int n) {
    if (!s || n < 0) return CC_BAD_INPUT;
    s->host_threads = n;
    return CC_OK;
}

int cc_get_counters(cc_solver* s, long long* out, int n) {
    if (!s || !out) return 0;
    s->counters[9] = s->launches_last;
    int m = n < kNumCounters ? n : kNumCounters;
    for (int i = 0; i < m; ++i) out[i] = s->counters[i];
    return m;
}

cc_status cc_set_recording(cc_solver* s, int on) {
    if (!s) return CC_BAD_INPUT;
    cudaSetDevice(s->device);
    s->record = on != 0;
    if (s->record && s->pair_cap && s->rec_cap < s->pair_cap) return s->grow_pairs(s->pair_cap);
    return CC_OK;
}

int cc_get_visits(cc_solver* s, int* out, int cap) {
    if (!s) return -1;
    int n = (int)s->visits.size();
    if (out)
        for (int i = 0; i < n && i < cap; ++i) {
            const VisitRec& r = s->visits[i];
            int* o = out + 13 * i;
            o[0] = r.pass; o[1] = r.kind; o[2] = r.a; o[3] = r.b; o[4] = r.status;
            for (int k = 0; k < 6; ++k) o[5 + k] = r.dcount[k];
            o[11] = r.rank_b; o[12] = r.rank_a;
        }
    return n;
}

int cc_get_scene_pass_kinds(cc_solver* s, int scene, int* out, int cap) {
    if (!s || scene < 0 || scene >= s->nscenes) return -1;
    const std::vector<int>& k = s->scenes[scene].pass_kinds;
    int n = (int)k.size();
    if (out)
        for (int i = 0; i < n && i < cap; ++i) out[i] = k[i];
    return n;
}

int cc_get_pass_kinds(cc_solver* s, int* out, int cap) {
    if (!s) return -1;
    if (s->nscenes == 0) return 0;
    return cc_get_scene_pass_kinds(s, 0, out, cap);
}

cc_status cc_get_zone_roots(cc_solver* s, int* out) {
    if (!s || !out) return CC_BAD_INPUT;
    cudaSetDevice(s->device);
    return s->zone_roots(out);
}

cc_status cc_get_leaf_ranks(cc_solver* s, int which, int* out) {
    if (!s || !out || which < 0 || which > 1) return CC_BAD_INPUT;
    for (const SceneHost& sh : s->scenes)
        if (sh.ne > 0 && !sh.built[which]) return CC_BAD_INPUT;
    if (s->ne == 0) return CC_OK;
    cudaSetDevice(s->device);
    cudaMemcpyAsync(out, s->d_rank[which], sizeof(int) * (size_t)s->ne, cudaMemcpyDeviceToHost, s->stream);
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return s->cuda_check("leaf ranks");
    return CC_OK;
}
cc_status cc_get_tree_volume(cc_solver* s, int scene, double* out) {
    if (!s || !out || scene < 0 || scene >= s->nscenes) return CC_BAD_INPUT;
    *out = s->scenes[scene].volume;
    return CC_OK;
}

int cc_debug_candidate_pairs(cc_solver* s, int moving, int brute_force, int* out, int cap) {
    if (!s || s->ne == 0) return 0;
    cudaSetDevice(s->device);
    s->upload_scenes();
    for (int i = 0; i < s->nscenes; ++i)
        s->h_run[i] = SceneRun{s->scenes[i].ne > 0 ? (moving ? kSceneCcd : kSceneProx) : kSceneIdle, 0, 0, -1, -1,
                               {0, 0, 0}};
    s->select_active();
    cudaMemcpyAsync(s->d_run, s->h_run, sizeof(SceneRun) * (size_t)s->nscenes, cudaMemcpyHostToDevice, s->stream);
    leaf_boxes(s->d_ev, s->bvh.act, s->bvh.n, s->d_escene, s->d_scenes, s->nscenes, s->d_xo, s->d_av, moving,
               s->d_box, s->bvh.bbox_enc, s->stream);
    s->bvh_this_step = false;
    s->full_this_step = false;
    s->reuse_pairs = false;
    if (!brute_force) bvh_build(s->d_box, s->bvh, s->stream);
    for (int attempt = 0; attempt < 8; ++attempt) {
        count_launch(), k_reset_counters<<<1, 1, 0, s->stream>>>(s->d_ctr);
        cudaMemsetAsync(&s->d_ctr->err, 0, sizeof(int), s->stream);
        if (brute_force)
            brute_pairs(s->d_box, s->ne, s->d_escene, s->d_pairs, s->pair_cap, s->d_ctr, s->stream);
        else
            bvh_pairs(s->d_box, s->bvh, s->d_pairs, s->pair_cap, s->d_ctr, s->stream, nullptr, s->tune.traverse_block,
                      nullptr, s->tune.packet_traverse, s->tune.rope_traverse, s->tune.traverse_refill,
                      kTraversalStack);
        cudaMemcpyAsync(s->h_ctr, s->d_ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, s->stream);
        if (cudaStreamSynchronize(s->stream) != cudaSuccess) return -1;
        if (s->h_ctr->err & kErrPairOverflow) {
            if (s->grow_pairs(2 * s->h_ctr->npairs + 1024)) return -1;
            continue;
        }
        if (s->h_ctr->err) return -1;
        break;
    }
    int n = s->h_ctr->npairs;
    if (out && n > 0) {
        int m = n < cap ? n : cap;
        cudaMemcpyAsync(out, s->d_pairs, sizeof(int2) * (size_t)m, cudaMemcpyDeviceToHost, s->stream);
        cudaStreamSynchronize(s->stream);
    }
    return n;
}

cc_status cc_set_stream(cc_solver* s, void* stream) {
    if (!s) return CC_BAD_INPUT;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    if (stream) {
        s->stream = (cudaStream_t)stream;
        s->own_stream = false;
    } else {
        if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return CC_CUDA_ERROR;
        s->own_stream = true;
    }
    return CC_OK;
}

cc_status cc_set_strain_window(cc_solver* s, int on) {
    if (!s) return CC_BAD_INPUT;
    s->strain_window = on != 0;
    return CC_OK;
}

cc_status cc_set_mode(cc_solver* s, int mode) {
    if (!s || mode < 0 || mode > 1) return CC_BAD_INPUT;
    s->mode = mode;  // each mode keeps its own loop graph
    return CC_OK;
}

cc_status cc_set_profiling(cc_solver* s, int on) {
    if (!s || on < 0 || on > 2) return CC_BAD_INPUT;
    s->profiling = on != 0;
    const bool marks = on == 2;
    if (marks != s->loop_marks) s->loop_dirty = true;  // the loop graph holds the marks or not
    s->loop_marks = marks;
    if (marks && !s->d_marks) {
        cudaSetDevice(s->device);
        if (cudaMalloc(&s->d_marks, sizeof(unsigned long long) * kMarkWords) != cudaSuccess) {
            s->d_marks = nullptr;
            s->loop_marks = false;
            return s->fail(CC_NO_MEMORY, "stage marks");
        }
    }
    if (s->d_marks) {
        cudaSetDevice(s->device);
        cudaMemsetAsync(s->d_marks, 0, sizeof(unsigned long long) * kMarkWords, s->stream);
    }
    for (int i = 0; i < kNumStages; ++i) {
        s->stage_ms[i] = 0.0;
        s->stage_calls[i] = 0;
    }
    return CC_OK;
}

int cc_get_profile(cc_solver* s, double* ms, long long* calls, int cap) {
    if (!s) return -1;
    if (s->loop_marks && s->d_marks) {
        unsigned long long h[1 + 2 * kNumLoopMarks];
        cudaSetDevice(s->device);
        cudaMemcpyAsync(h, s->d_marks, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
        if (cudaStreamSynchronize(s->stream) == cudaSuccess)
            for (int k = 0; k < kNumLoopMarks; ++k) {
                s->stage_ms[kStLoopPlan + k] = (double)h[1 + 2 * k] * 1e-6;
                s->stage_calls[kStLoopPlan + k] = (long long)h[2 + 2 * k];
            }
    }
    for (int i = 0; i < kNumStages && i < cap; ++i) {
        if (ms) ms[i] = s->stage_ms[i];
        if (calls) calls[i] = s->stage_calls[i];
    }
    return kNumStages;
}

const char* cc_profile_stage_name(int i) { return (i >= 0 && i < kNumStages) ? kStageNames[i] : ""; }

int cc_selftest_math(int device, int fn, const double* a, const double* b, double* out, int n) {
    if (n <= 0) return 0;
    if (cudaSetDevice(device) != cudaSuccess) return -1;
    double *da = nullptr, *db = nullptr, *dout = nullptr;
    size_t bytes = sizeof(double) * (size_t)n;
    if (cudaMalloc(&da, bytes) != cudaSuccess || cudaMalloc(&db, bytes) != cudaSuccess ||
        cudaMalloc(&dout, bytes) != cudaSuccess) {
        cudaFree(da); cudaFree(db); cudaFree(dout);
        return -1;
    }
    cudaMemcpy(da, a, bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(db, b ? b : a, bytes, cudaMemcpyHostToDevice);
    math_selftest(fn, da, db, dout, n, 0);
    cudaError_t e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
    cudaFree(da); cudaFree(db); cudaFree(dout);
    return e == cudaSuccess ? n : -1;
}

int cc_last_error(cc_solver* s, char* buf, int len) {
    if (!s || !buf || len <= 0) return 0;
    std::snprintf(buf, (size_t)len, "%s", s->err.c_str());
    return (int)s->err.size();
}

}  // extern "C"
