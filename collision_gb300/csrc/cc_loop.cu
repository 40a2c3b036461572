// The detection loop of resolveCollision on the device.
//
// resolveCollision (dcollid.cpp:317-362) runs one proximity pass, then CCD
// passes while they find collisions (at most MAX_ITER = 5, dcollid.cpp:433),
// then impact-zone passes until one finds nothing (dcollid.cpp:227-265) -
// per scene, from that scene's own hit counts. Here every scene's place in
// that sequence (SceneCtl) and the loop's own state (LoopCtl) live in device
// memory, so that one CUDA graph can run all detection passes of a step: a
// WHILE node whose body is one pass over the scenes that still have one,
// planned by k_loop_plan and closed by k_pass_end, which also decides whether
// another pass follows. The host is needed only where the reference's tree
// must be rebuilt (the host emulates its insertion order) or a buffer is too
// small: such a pass applies nothing, the loop stops, and after the host has
// done its part the same pass runs again.
#include "cc_launch.h"

namespace ccg {

namespace {

inline int nblk(int n, int t) { return (n + t - 1) / t; }

constexpr int kPlanThreads = 1024;

// Block-wide exclusive scan of three counts (elements, points, scenes) over
// the calling block; returns the block totals in tot.
__device__ __forceinline__ int3 block_scan3(int3 v, int3* tot) {
    __shared__ int3 warp_sums[kPlanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int3 x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(0xffffffffu, x.x, o), b = __shfl_up_sync(0xffffffffu, x.y, o),
                  c = __shfl_up_sync(0xffffffffu, x.z, o);
        if (lane >= o) x.x += a, x.y += b, x.z += c;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int3 w = lane < kPlanThreads / 32 ? warp_sums[lane] : make_int3(0, 0, 0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int a = __shfl_up_sync(0xffffffffu, w.x, o), b = __shfl_up_sync(0xffffffffu, w.y, o),
                      c = __shfl_up_sync(0xffffffffu, w.z, o);
            if (lane >= o) w.x += a, w.y += b, w.z += c;
        }
        if (lane < kPlanThreads / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    const int3 before = warp > 0 ? warp_sums[warp - 1] : make_int3(0, 0, 0);
    *tot = warp_sums[kPlanThreads / 32 - 1];
    __syncthreads();
    return make_int3(before.x + x.x - v.x, before.y + x.y - v.y, before.z + x.z - v.z);
}

// Plans one pass: each scene's mode from its place in the sequence (a
// pending pass keeps the modes it had), the lists of the pass's scenes with
// their element and point offsets, and each scene's SceneRun. Per
// scene-pass counters are added once per pass, not again when it reruns.
__global__ void __launch_bounds__(kPlanThreads) k_loop_plan(SceneCtl* ctl, SceneRun* run,
                                                            const SceneDev* __restrict__ scenes, int nscenes,
                                                            LoopCtl* L, int* sel, int* eoff, int* poff,
                                                            cudaGraphConditionalHandle h_zone) {
    if (L->host) {
        // a pass before this one stopped for the host: nothing runs
        if (threadIdx.x == 0) {
            L->nact = L->nact_e = L->nact_p = 0;
            L->nbroad = L->npts = 0;
            L->nq_full = L->nquery = 0;
            L->any_zone = 0;
            cudaGraphSetConditional(h_zone, 0u);
        }
        return;
    }
    const bool fresh = L->pending == 0;
    int3 carry = make_int3(0, 0, 0);
    int any_zone = 0;
    unsigned long long bytes = 0, passes = 0, nccd = 0, nzone = 0;
    for (int base = 0; base < nscenes; base += kPlanThreads) {
        const int s = base + threadIdx.x;
        int mode = kSceneIdle;
        if (s < nscenes) {
            SceneCtl c = ctl[s];
            if (fresh) {
                if (c.state == kSeqCcd) {
                    mode = kSceneCcd;
                    c.nccd++;
                } else if (c.state == kSeqZone) {
                    mode = kSceneZone;
                    c.nzone++;
                }
                ctl[s] = c;
                if (mode != kSceneIdle) {
                    // path bytes per scene-pass: x_old and avgVel read,
                    // connectivity, the FP32 hierarchy written by the refit
                    // and read once by the traversal, avgVel updated; a zone
                    // pass reads the state again
                    const SceneDev& sd = scenes[s];
                    bytes += 72ull * sd.nv + 12ull * sd.nt + 8ull * (sd.ne - sd.nt) + 48ull * (2ull * sd.ne - 1) +
                             (mode == kSceneZone ? 48ull * sd.nv : 0ull);
                    passes++;
                    nccd += mode == kSceneCcd;
                    nzone += mode == kSceneZone;
                }
            } else {
                mode = run[s].mode;
            }
            SceneRun r = run[s];
            r.mode = mode;
            r.hits = 0;
            r.pass = c.nccd + c.nzone;
            r.leaf0 = mode != kSceneIdle ? c.leafbase : -1;
            run[s] = r;
            any_zone |= mode == kSceneZone;
        }
        const bool on = mode != kSceneIdle;
        int3 tot;
        const int3 off = block_scan3(on ? make_int3(scenes[s].ne, scenes[s].nv, 1) : make_int3(0, 0, 0), &tot);
        if (on) {
            const int k = carry.z + off.z;
            sel[k] = s;
            eoff[k] = carry.x + off.x;
            poff[k] = carry.y + off.y;
        }
        carry.x += tot.x;
        carry.y += tot.y;
        carry.z += tot.z;
    }
    any_zone = __syncthreads_or(any_zone);
    if (fresh) {
        for (int o = 16; o > 0; o >>= 1) {
            bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
            passes += __shfl_xor_sync(0xffffffffu, passes, o);
            nccd += __shfl_xor_sync(0xffffffffu, nccd, o);
            nzone += __shfl_xor_sync(0xffffffffu, nzone, o);
        }
        if ((threadIdx.x & 31) == 0 && passes) {
            atomicAdd(&L->acc[kAccPathBytes], bytes);
            atomicAdd(&L->acc[kAccPasses], passes);
            atomicAdd(&L->acc[kAccCcd], nccd);
            atomicAdd(&L->acc[kAccZone], nzone);
        }
    }
    if (threadIdx.x == 0) {
        eoff[carry.z] = carry.x;
        poff[carry.z] = carry.y;
        L->nact = carry.z;
        L->nact_e = carry.x;
        L->nact_p = carry.y;
        L->any_zone = any_zone;
        if (fresh) {
            L->reuse_n = L->reuse;  // the proximity pass's pairs, for the first CCD pass only
            L->reuse = -1;
            L->serial++;
            // from the second CCD pass on, only pairs with a point the
            // previous pass touched can hit (see k_dirty_queries)
            L->prune = (L->prune_on && L->acc[kAccIters] >= 2) ? 1 : 0;
        }
        L->nbroad = L->reuse_n >= 0 ? 0 : carry.x;
        L->nq_full = L->prune ? 0 : L->nbroad;
        L->nquery = 0;
        L->npts = carry.y;
        L->pending = 0;
        cudaGraphSetConditional(h_zone, any_zone ? 1u : 0u);
    }
}

// The pass's elements (act_e), their sorted leaves in the step's hierarchy
// (act_l) and points (act_p), scene by scene.
__global__ void k_loop_expand(const int* __restrict__ sel, const int* __restrict__ eoff,
                              const int* __restrict__ poff, const SceneDev* __restrict__ scenes,
                              const SceneCtl* __restrict__ ctl, const LoopCtl* __restrict__ L, int* act_e, int* act_l,
                              int* act_p) {
    const int ns = L->nact, ne = L->nact_e, np = L->nact_p;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ne + np; k += gridDim.x * blockDim.x) {
        const bool pt = k >= ne;
        const int kk = pt ? k - ne : k;
        const int* off = pt ? poff : eoff;
        int lo = 0, hi = ns - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= kk) lo = mid; else hi = mid - 1;
        }
        const int s = sel[lo], d = kk - off[lo];
        if (pt) {
            act_p[kk] = scenes[s].v0 + d;
        } else {
            act_e[kk] = scenes[s].e0 + d;
            act_l[kk] = ctl[s].leafbase + d;
        }
    }
}

__device__ __forceinline__ double dec_double(unsigned long long e) {
    unsigned long long u = (e & 0x8000000000000000ull) ? (e & 0x7fffffffffffffffull) : ~e;
    return __longlong_as_double((long long)u);
}

// aabbProximity / aabbCollision's rebuild test (dcollid.cpp:366-428) for
// every scene of the pass: its tree `which` is unbuilt, or the root volume of
// this pass's boxes has grown by more than 20% over the volume both trees
// share. Such a scene is flagged for the host, and the pass stops.
__device__ __forceinline__ void tree_check_one(const SceneRun* __restrict__ run, int s,
                                               const unsigned long long* bbox_enc, const double* __restrict__ vol,
                                               const int* __restrict__ built, int which, int* rebuild, LoopCtl* L) {
    if (run[s].mode == kSceneIdle || run[s].leaf0 < 0) return;
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = dec_double(bbox_enc[6 * s + d]);
        hi[d] = dec_double(bbox_enc[6 * s + 3 + d]);
    }
    const double v = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
    const double sv = vol[s];
    if (!built[s] || (v - sv) > 0.2 * sv) {
        rebuild[s] = which + 1;
        atomicOr(&L->host, kHostRebuild);
    }
}

__global__ void k_tree_check(const SceneRun* __restrict__ run, int nscenes, const unsigned long long* bbox_enc,
                             const double* __restrict__ vol, const int* __restrict__ built, int which, int* rebuild,
                             LoopCtl* L) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (L->nact == 0 || s >= nscenes) return;
    tree_check_one(run, s, bbox_enc, vol, built, which, rebuild, L);
}

// Counters and hit counts of a pass about to run. A pass stopped for the
// host keeps the error bit kErrHost (nothing of it is applied) and covers no
// elements or points.
__device__ __forceinline__ void loop_reset_counters(PassCounters* c, LoopCtl* L) {
    const int keep = c->err & kErrNan;
    const bool stop = L->host != 0;
    c->npairs = (!stop && L->reuse_n >= 0) ? L->reuse_n : 0;
    c->ncontrib = 0; c->nhit_pairs = 0; c->nrec = 0; c->nvisits = 0; c->ncontacts = 0; c->nsub = 0;
    c->ncr = 0; c->nunion = 0; c->nsub_pt = 0; c->nsub_ee = 0; c->npairq = 0; c->nzones = 0; c->nmembers = 0;
    c->nseg = 0;
    c->err = keep | (stop ? kErrHost : 0);
    if (stop) {
        L->nbroad = 0;
        L->npts = 0;
        L->nq_full = 0;
        L->prune = 0;
    }
}

__global__ void k_loop_reset(PassCounters* c, SceneRun* run, int nscenes, LoopCtl* L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) loop_reset_counters(c, L);
    if (i < nscenes) run[i].hits = 0;
}

// k_tree_check then k_loop_reset in one block (one launch less per pass):
// every scene's test, a barrier (the reset reads the stop bit any test may
// set), then the reset.
__global__ void __launch_bounds__(1024) k_tree_check_reset(SceneRun* run, int nscenes,
                                                            const unsigned long long* bbox_enc,
                                                            const double* __restrict__ vol,
                                                            const int* __restrict__ built, int which, int* rebuild,
                                                            LoopCtl* L, PassCounters* c) {
    if (L->nact != 0)
        for (int s = threadIdx.x; s < nscenes; s += blockDim.x)
            tree_check_one(run, s, bbox_enc, vol, built, which, rebuild, L);
    __syncthreads();
    if (threadIdx.x == 0) loop_reset_counters(c, L);
    for (int s = threadIdx.x; s < nscenes; s += blockDim.x) run[s].hits = 0;
}

// Closes a pass. A pass that stopped or failed stops the loop (the host
// reads why); otherwise its counters are added, every scene that ran it
// steps its sequence from its hit count (dcollid.cpp:333-356) - proximity
// to CCD; a CCD pass without a hit ends the scene, the fifth with hits
// starts the impact zones; an impact-zone pass without a hit ends the scene
// - and the loop goes on while a scene has a pass to run. A scene whose
// impact-zone passes reach the cap is finished with its current velocities
// (status kIterCap). With `combined`, a proximity pass without an impulse
// leaves its pairs (found on swept boxes) to the first CCD pass.
__global__ void __launch_bounds__(kPlanThreads) k_pass_end(const PassCounters* __restrict__ c, SceneCtl* ctl,
                                                           const SceneRun* __restrict__ run, int nscenes, LoopCtl* L,
                                                           int combined, int in_graph,
                                                           cudaGraphConditionalHandle h_loop) {
    __shared__ int stop;
    if (threadIdx.x == 0) {
        const int e = c->err;
        stop = 1;
        if (L->host) {
            // flagged for a rebuild before the pass ran
        } else if (e & (kErrNan | kErrIndexNode | kErrIndexLeaf | kErrIndexElem)) {
            L->host |= kHostFatal;
            L->err = e;
            L->stopped = *c;
        } else if (e & kErrRetry) {
            L->host |= kHostRetry;
            L->err = e;
            L->stopped = *c;  // later iterations of the stopped loop reset *c
        } else {
            stop = 0;
            unsigned long long* a = L->acc;
            a[kAccPairs] += (unsigned)c->npairs;
            a[kAccVisits] += (unsigned)c->nvisits;
            a[kAccHits] += (unsigned)c->nhit_pairs;
            a[kAccContacts] += (unsigned)c->ncontacts;
            a[kAccSub] += (unsigned)c->nsub;
            a[kAccCr] += (unsigned)c->ncr;
            a[kAccZonePasses] += L->any_zone ? 1u : 0u;
            a[kAccQueries] += L->prune ? (unsigned)L->nquery : 0u;
            a[kAccUnions] += L->any_zone ? (unsigned)c->nunion : 0u;
            a[kAccIters] += 1;
            if (in_graph) a[kAccMovingVisits] += (unsigned)c->nvisits;
            // path bytes per pass: pairs written and read, per-point impulse,
            // friction and count records written and read for each contact
            a[kAccPathBytes] += 16ull * (unsigned)c->npairs + 416ull * (unsigned)c->ncontacts;
            if (L->reuse_n < 0) {
                a[kAccLeaves] += (unsigned)L->nbroad;
                a[kAccBroadPairs] += (unsigned)c->npairs;
            }
            if (!in_graph) {
                L->reuse = (combined && c->ncontrib == 0) ? c->npairs : -1;
                a[kAccProxPairs] += (unsigned)c->npairs;
            }
        }
    }
    __syncthreads();
    int more = 0;
    if (!stop) {
        const int cap = L->zone_cap;
        for (int s = threadIdx.x; s < nscenes; s += blockDim.x) {
            if (run[s].mode == kSceneIdle) continue;
            SceneCtl x = ctl[s];
            const bool hit = run[s].hits > 0;
            if (x.state == kSeqProx) {  // is_collision = true; niter = 1 (dcollid.cpp:333-336)
                x.state = kSeqCcd;
                x.niter = 1;
            } else if (x.state == kSeqCcd) {  // dcollid.cpp:337-352
                if (x.nccd == 1 && hit) x.hcol = 1;
                if (!hit)
                    x.state = kSeqDone;
                else if (++x.niter > kMaxCcdIter)
                    x.state = kSeqZone;
            } else if (x.state == kSeqZone) {
                if (!hit) x.state = kSeqDone;
            }
            if (x.state == kSeqZone && x.nzone >= cap) {
                // the reference would loop on; this scene stops here
                x.state = kSeqDone;
                x.status = kIterCap;
            }
            more |= x.state == kSeqCcd || x.state == kSeqZone;
            ctl[s] = x;
        }
    }
    more = __syncthreads_or(more);
    if (threadIdx.x == 0) {
        // a scene still in its sequence after the loop stopped needs the
        // pass again: the host reruns it with the same modes
        if (stop) L->pending = 1;
        if (in_graph) cudaGraphSetConditional(h_loop, (!stop && more) ? 1u : 0u);
    }
}

}  // namespace

void loop_plan(SceneCtl* ctl, SceneRun* run, const SceneDev* scenes, int nscenes, LoopCtl* L, int* sel, int* eoff,
               int* poff, cudaGraphConditionalHandle h_zone, cudaStream_t s) {
    count_launch(), k_loop_plan<<<1, kPlanThreads, 0, s>>>(ctl, run, scenes, nscenes, L, sel, eoff, poff, h_zone);
}

void loop_expand(const int* sel, const int* eoff, const int* poff, const SceneDev* scenes, const SceneCtl* ctl,
                 const LoopCtl* L, int cap, int* act_e, int* act_l, int* act_p, cudaStream_t s) {
    int g = nblk(cap, 256);
    if (g > 152 * 8) g = 152 * 8;
    if (g < 1) g = 1;
    count_launch(), k_loop_expand<<<g, 256, 0, s>>>(sel, eoff, poff, scenes, ctl, L, act_e, act_l, act_p);
}

void tree_check(const SceneRun* run, int nscenes, const unsigned long long* bbox_enc, const double* vol,
                const int* built, int which, int* rebuild, LoopCtl* L, cudaStream_t s) {
    count_launch(), k_tree_check<<<nblk(nscenes, 128), 128, 0, s>>>(run, nscenes, bbox_enc, vol, built, which,
                                                                    rebuild, L);
}

void tree_check_reset(SceneRun* run, int nscenes, const unsigned long long* bbox_enc, const double* vol,
                      const int* built, int which, int* rebuild, LoopCtl* L, PassCounters* c, cudaStream_t s) {
    if (nscenes > 4096) {
        tree_check(run, nscenes, bbox_enc, vol, built, which, rebuild, L, s);
        loop_reset(c, run, nscenes, L, s);
        return;
    }
    const int t = nscenes < 32 ? 32 : (nscenes < 1024 ? (nscenes + 31) / 32 * 32 : 1024);
    count_launch(), k_tree_check_reset<<<1, t, 0, s>>>(run, nscenes, bbox_enc, vol, built, which, rebuild, L, c);
}

void loop_reset(PassCounters* c, SceneRun* run, int nscenes, LoopCtl* L, cudaStream_t s) {
    count_launch(), k_loop_reset<<<nblk(nscenes > 0 ? nscenes : 1, 256), 256, 0, s>>>(c, run, nscenes, L);
}

// A stage boundary inside the loop graph (stage profiling): the device time
// since the previous boundary, from the global nanosecond timer, goes to
// `slot` (0 only records the time and starts a pass's row of the pass log).
// Layout of acc: [0] the last boundary's time, then (ns, count) per slot,
// then the pass log's row counter and kPassLogRows rows of kPassLogCols:
// the pass's time per slot, then (with c given, at the pass's last slot)
// its candidate pairs, queued point-triangle and edge-edge sub-tests,
// union records and pruned queries.
__global__ void k_stage_mark(unsigned long long* acc, int slot, const PassCounters* c, const LoopCtl* L) {
    constexpr int nslots = kLoopMarkSlots;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    unsigned long long* rows = acc + 1 + 2 * nslots;
    unsigned long long* log = rows + 1;
    if (slot > 0) {
        const unsigned long long d = t - acc[0];
        acc[2 * slot - 1] += d;
        acc[2 * slot] += 1;
        const unsigned long long r = *rows;
        if (r > 0) {
            unsigned long long* row = log + ((r - 1) % kPassLogRows) * kPassLogCols;
            row[slot - 1] = d;
            if (c) {
                row[nslots + 0] = (unsigned)c->npairs;
                row[nslots + 1] = (unsigned)c->nsub_pt;
                row[nslots + 2] = (unsigned)c->nsub_ee;
                row[nslots + 3] = (unsigned)c->nunion;
                row[nslots + 4] = L ? (unsigned)(L->prune ? L->nquery : -1) : 0u;
            }
        }
    } else {
        const unsigned long long r = *rows;
        unsigned long long* row = log + (r % kPassLogRows) * kPassLogCols;
        for (int k = 0; k < kPassLogCols; ++k) row[k] = 0;
        *rows = r + 1;
    }
    acc[0] = t;
}

void stage_mark(unsigned long long* acc, int slot, cudaStream_t s, const PassCounters* c, const LoopCtl* L) {
    count_launch(), k_stage_mark<<<1, 1, 0, s>>>(acc, slot, c, L);
}

void pass_end(const PassCounters* c, SceneCtl* ctl, const SceneRun* run, int nscenes, LoopCtl* L, int combined,
              bool in_graph, cudaGraphConditionalHandle h_loop, cudaStream_t s) {
    count_launch(), k_pass_end<<<1, kPlanThreads, 0, s>>>(c, ctl, run, nscenes, L, combined, in_graph ? 1 : 0,
                                                          h_loop);
}

}  // namespace ccg
