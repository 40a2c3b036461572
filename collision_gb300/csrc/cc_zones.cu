// Impact zones on the GPU: the reference's union-find with member lists
// (makeSet / findSet / mergePoint / createImpZone, dcollid.cpp:473-484,
// 1015-1059) and the rigid motion of every zone (computeImpactZone,
// dcollid.cpp:236-262).
//
// The member list of a zone fixes the order in which updateImpactListVelocity
// (dcollid3d.cpp:70-200) sums its centre of mass, momentum and inertia, and
// that order comes from the exact sequence of weighted unions with list
// concatenation: the lighter set's list is appended to the heavier one's.
// A concurrent union-find gives the same partition but another order, so the
// unions of a pass are replayed in the reference's visiting order - but only
// where order matters: the unions of different final zones touch disjoint
// points, so every final zone replays its own unions, one thread per zone,
// all zones at once.
//
//   1. A lock-free union-find over the same points (cc: parent links, the
//      smaller index as root) joins the pass's pairs: its roots label the
//      final zone of every createImpZone record.
//   2. The records are sorted by (label, visiting-order key) - two stable
//      radix sorts, key first - and cut into one segment per label.
//   3. One thread per segment replays its records' unions in key order on
//      the exact union-find (UfNode), with path compression.
//   4. Every root of two or more points in a scene in impact-zone mode is a
//      zone: its members are written out by walking its list, and the zone
//      moves rigidly (k_zone_solve).
// Both union-finds start every step from the state makeSet and the movable
// bodies' unions (createImpZoneForRG, dcollid3d.cpp:54-68) leave.
#include "cc_launch.h"

namespace ccg {

namespace {

inline int nblk(int n, int t) { return (n + t - 1) / t; }

__device__ __forceinline__ int count_of(const int* c, int cap) {
    const int n = *c;
    return n < cap ? n : cap;
}

// A pair of a createImpZone(pts, 4) call that mergePoint joins: every pair
// (a, b), b < a, without a movable point (dcollid.cpp:478-480).
__device__ __forceinline__ bool joins(const uint8_t* fixed, int pa, int pb) {
    return !((fixed[pa] | fixed[pb]) & 2);
}

__device__ __forceinline__ int cc_find(int* cc, int p) {
    // path halving: every link written points to an ancestor, so concurrent
    // finds and unions stay correct
    int q = cc[p];
    while (q != p) {
        const int g = cc[q];
        if (g != q) cc[p] = g;
        p = q;
        q = g;
    }
    return p;
}

__device__ __forceinline__ void cc_union(int* cc, int a, int b) {
    for (;;) {
        a = cc_find(cc, a);
        b = cc_find(cc, b);
        if (a == b) return;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        // the larger root is linked under the smaller one, if still a root
        if (atomicCAS(&cc[a], a, b) == a) return;
    }
}

__global__ void k_cc_union(const UnionRec* __restrict__ rec, const PassCounters* ctr, int cap,
                           const uint8_t* __restrict__ fixed, int* cc) {
    if (ctr->err & kErrRetry) return;
    const int n = count_of(&ctr->nunion, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const UnionRec r = rec[i];
        for (int a = 1; a < 4; ++a)
            for (int b = 0; b < a; ++b)
                if (joins(fixed, r.p[a], r.p[b])) cc_union(cc, r.p[a], r.p[b]);
    }
}

// Sort keys, first pass: the visiting-order key of every record.
__global__ void k_union_keys(const UnionRec* __restrict__ rec, const PassCounters* ctr, int cap,
                             unsigned long long* keys, unsigned int* vals) {
    if (ctr->err & kErrRetry) return;
    const int n = count_of(&ctr->nunion, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        keys[i] = rec[i].key;
        vals[i] = (unsigned int)i;
    }
}

constexpr unsigned long long kNoLabel = (1ull << 31) - 1;

// Second pass: the final zone of each record (in key order), or kNoLabel for
// a record that joins nothing.
__global__ void k_union_labels(const UnionRec* __restrict__ rec, const PassCounters* ctr, int cap,
                               const uint8_t* __restrict__ fixed, int* cc, const unsigned int* __restrict__ vals,
                               unsigned long long* keys) {
    if (ctr->err & kErrRetry) return;
    const int n = count_of(&ctr->nunion, cap);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const UnionRec r = rec[vals[j]];
        unsigned long long lab = kNoLabel;
        for (int a = 1; a < 4 && lab == kNoLabel; ++a)
            for (int b = 0; b < a; ++b)
                if (joins(fixed, r.p[a], r.p[b])) {
                    lab = (unsigned long long)cc_find(cc, r.p[a]);
                    break;
                }
        keys[j] = lab;
    }
}

// The first record of every label's run.
__global__ void k_union_segments(const unsigned long long* __restrict__ keys, PassCounters* ctr, int cap, int* seg) {
    if (ctr->err & kErrRetry) return;
    const int n = count_of(&ctr->nunion, cap);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const unsigned long long k = keys[j];
        if (k != kNoLabel && (j == 0 || keys[j - 1] != k)) seg[atomicAdd(&ctr->nseg, 1)] = j;
    }
}

// findSet (dcollid.cpp:1024-1031) with path compression.
__device__ __forceinline__ int uf_find(UfNode* uf, int p) {
    int r = p;
    while (uf[r].root != r) r = uf[r].root;
    while (uf[p].root != r) {
        const int nx = uf[p].root;
        uf[p].root = r;
        p = nx;
    }
    return r;
}

// The root of each of a record's four points: the four parent links are
// loaded together, then their parents' links; a point whose parent is a
// root (path compression keeps almost every point there) needs nothing
// more, any other takes the full find with path compression.
__device__ __forceinline__ void find4(UfNode* uf, const int* p, int* rt) {
    int a[4], b[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) a[q] = uf[p[q]].root;
#pragma unroll
    for (int q = 0; q < 4; ++q) b[q] = uf[a[q]].root;
#pragma unroll
    for (int q = 0; q < 4; ++q) rt[q] = b[q] == a[q] ? a[q] : uf_find(uf, p[q]);
}

// The weight and tail of the root that won the thread's last merge, kept in
// registers: the next records of a zone mostly join sets to that root, and
// only this thread writes the nodes of its zone.
struct RootCache {
    int id = -1, w = 0, tail = 0;
};

__device__ __forceinline__ int2 root_wt(const UfNode* uf, const RootCache& c, int r) {
    if (r == c.id) return make_int2(c.w, c.tail);
    const int4 u = *reinterpret_cast<const int4*>(&uf[r]);  // root, next, tail, w
    return make_int2(u.w, u.z);
}

// One createImpZone(pts, 4) call: mergePoint (dcollid.cpp:1033-1059) on
// every pair of its points in the reference's order - the lighter set joins
// the heavier one (the second on equal weights) and its member list is
// appended. Only roots, weights, tails and next links are observable
// (membership, list order, the next unions' choices); the root links path
// compression shortens are not. So each point's root is found once, kept in
// a register and updated as the call's merges go, instead of two finds per
// pair.
__device__ __forceinline__ void replay_record(UfNode* uf, const uint8_t* __restrict__ fixed, const UnionRec& r,
                                              RootCache& cache) {
    int rt[4];
    find4(uf, r.p, rt);
#pragma unroll
    for (int a = 1; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < a; ++b) {
            if (!joins(fixed, r.p[a], r.p[b])) continue;
            int px = rt[a], py = rt[b];
            if (px == py) continue;
            int2 sx = root_wt(uf, cache, px), sy = root_wt(uf, cache, py);
            if (sx.x > sy.x) {  // the heavier set keeps its root (the second on equal weights)
                const int t = px;
                px = py;
                py = t;
                const int2 ts = sx;
                sx = sy;
                sy = ts;
            }
            const int w = sx.x + sy.x;
            uf[py].w = w;
            uf[px].root = py;
            uf[sy.y].next = px;
            uf[py].tail = sx.y;
            cache.id = py;
            cache.w = w;
            cache.tail = sx.y;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (rt[q] == px) rt[q] = py;
        }
}

// One thread per final zone touched by the pass: its records' unions in
// visiting order, as createImpZone makes them.
// Records that join nothing new: every pair the call joins already shares a
// root in the union-find as the pass starts. Sets only grow, so such a
// record joins nothing at its turn in the replay either, and skipping it
// changes no root, weight, tail or next link.
__device__ __forceinline__ int uf_root_ro(const UfNode* uf, int p) {
    int r = p;
    for (int k = 0; k < 64; ++k) {
        const int nx = uf[r].root;
        if (nx == r) return r;
        r = nx;
    }
    return -1;  // a longer chain: no claim
}

__global__ void k_union_noop(const UnionRec* __restrict__ rec, const PassCounters* ctr, int cap,
                             const uint8_t* __restrict__ fixed, const UfNode* __restrict__ uf, uint8_t* noop) {
    if (ctr->err & kErrRetry) return;
    const int n = count_of(&ctr->nunion, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const UnionRec r = rec[i];
        int rt[4];
        for (int q = 0; q < 4; ++q) rt[q] = uf_root_ro(uf, r.p[q]);
        bool nothing = true;
        for (int a = 1; a < 4 && nothing; ++a)
            for (int b = 0; b < a; ++b)
                if (joins(fixed, r.p[a], r.p[b]) && (rt[a] < 0 || rt[a] != rt[b])) {
                    nothing = false;
                    break;
                }
        noop[i] = nothing ? 1 : 0;
    }
}

// Final zones with at least big records are replayed by k_union_replay_cta.
__device__ __forceinline__ bool big_segment(const unsigned long long* keys, int j0, int n, int big) {
    return j0 + big - 1 < n && keys[j0 + big - 1] == keys[j0];  // keys sorted by label
}

__global__ void k_union_replay(const UnionRec* __restrict__ rec, const PassCounters* ctr, int cap,
                               const unsigned long long* __restrict__ keys, const unsigned int* __restrict__ vals,
                               const int* __restrict__ seg, const uint8_t* __restrict__ fixed, UfNode* uf, int big,
                               const uint8_t* __restrict__ noop) {
    if (ctr->err & kErrRetry) return;
    const int n = count_of(&ctr->nunion, cap);
    const int nseg = ctr->nseg;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += gridDim.x * blockDim.x) {
        const int j0 = seg[s];
        if (big_segment(keys, j0, n, big)) continue;
        const unsigned long long lab = keys[j0];
        RootCache cache;
        for (int j = j0; j < n && keys[j] == lab; ++j) {
            const unsigned v = vals[j];
            if (!noop[v]) replay_record(uf, fixed, rec[v], cache);
        }
    }
}

// A large final zone replayed in shared memory: the union-find nodes its
// records touch (their points, then any ancestor or tail the replay reaches)
// are copied into a hash table in shared memory, one thread replays the
// records there - the same unions in the same order, each access a shared
// memory one instead of an L2 round trip - and the nodes are written back.
// Only this CTA touches the zone's nodes. If the table fills up, the zone is
// replayed from global memory instead (nothing was written back yet).
constexpr int kTabBits = 13;
constexpr int kTabSize = 1 << kTabBits;
constexpr int kTabMax = kTabSize * 3 / 4;
constexpr int kReplayThreads = 256;
constexpr size_t kTabBytes = (size_t)kTabSize * (sizeof(int) + sizeof(UfNode));

struct SmemUf {
    int* key;      // point id per slot, -1 empty
    UfNode* node;  // the point's node
    int* count;
    const UfNode* uf;
    // the slot of point p, inserting it (single thread) if absent; -1: full
    __device__ __forceinline__ int slot(int p) {
        unsigned h = ((unsigned)p * 2654435761u) >> (32 - kTabBits);
        for (int probe = 0; probe < kTabSize; ++probe) {
            const int k = key[h];
            if (k == p) return (int)h;
            if (k < 0) {
                if (*count >= kTabMax) return -1;
                key[h] = p;
                node[h] = uf[p];
                ++*count;
                return (int)h;
            }
            h = (h + 1) & (kTabSize - 1);
        }
        return -1;
    }
    // findSet with path compression; -1: full (or a root chain longer than
    // the table, which a valid union-find does not have)
    __device__ __forceinline__ int find(int p) {
        int r = p, sr = slot(r);
        if (sr < 0) return -1;
        for (int k = 0; node[sr].root != r; ++k) {
            if (k >= kTabSize) return -1;
            r = node[sr].root;
            sr = slot(r);
            if (sr < 0) return -1;
        }
        int x = p, sx = slot(x);  // every node on the path is in the table now
        for (int k = 0; sx >= 0 && node[sx].root != r && k < kTabSize; ++k) {
            const int nx = node[sx].root;
            node[sx].root = r;
            x = nx;
            sx = slot(x);
        }
        return r;
    }
};

__global__ void __launch_bounds__(kReplayThreads) k_union_replay_cta(
    const UnionRec* __restrict__ rec, const PassCounters* ctr, int cap, const unsigned long long* __restrict__ keys,
    const unsigned int* __restrict__ vals, const int* __restrict__ seg, const uint8_t* __restrict__ fixed,
    UfNode* uf, int big) {
    extern __shared__ int s_key[];
    UfNode* s_node = reinterpret_cast<UfNode*>(s_key + kTabSize);
    __shared__ int s_count, s_end, s_bad;
    if (ctr->err & kErrRetry) return;
    const int n = count_of(&ctr->nunion, cap);
    const int nseg = ctr->nseg;
    const int tid = threadIdx.x;
    for (int si = blockIdx.x; si < nseg; si += gridDim.x) {
        const int j0 = seg[si];
        if (!big_segment(keys, j0, n, big)) continue;
        const unsigned long long lab = keys[j0];
        for (int h = tid; h < kTabSize; h += kReplayThreads) s_key[h] = -1;
        if (tid == 0) {
            s_count = 0;
            s_end = n;
            s_bad = 0;
        }
        __syncthreads();
        // the segment's end: the first record of another label
        for (int k = j0 + tid; k < n; k += kReplayThreads)
            if (keys[k] != lab) {
                atomicMin(&s_end, k);
                break;
            }
        __syncthreads();
        const int j1 = s_end;
        // the records' points into the table
        for (int j = j0 + tid; j < j1 && !s_bad; j += kReplayThreads) {
            const UnionRec r = rec[vals[j]];
            for (int q = 0; q < 4; ++q) {
                const int p = r.p[q];
                unsigned h = ((unsigned)p * 2654435761u) >> (32 - kTabBits);
                for (int probe = 0; probe < kTabSize; ++probe) {
                    const int old = atomicCAS(&s_key[h], -1, p);
                    if (old == -1) {
                        s_node[h] = uf[p];
                        if (atomicAdd(&s_count, 1) >= kTabMax) s_bad = 1;
                        break;
                    }
                    if (old == p) break;
                    h = (h + 1) & (kTabSize - 1);
                }
            }
        }
        __syncthreads();
        if (tid == 0 && !s_bad) {
            SmemUf t{s_key, s_node, &s_count, uf};
            for (int j = j0; j < j1 && !s_bad; ++j) {
                const UnionRec r = rec[vals[j]];
                int rt[4];
                for (int q = 0; q < 4 && !s_bad; ++q) {
                    rt[q] = t.find(r.p[q]);
                    if (rt[q] < 0) s_bad = 1;
                }
                for (int a = 1; a < 4 && !s_bad; ++a)
                    for (int b = 0; b < a && !s_bad; ++b) {
                        if (!joins(fixed, r.p[a], r.p[b])) continue;
                        int px = rt[a], py = rt[b];
                        if (px == py) continue;
                        int sx = t.slot(px), sy = t.slot(py);
                        if (sx < 0 || sy < 0) {
                            s_bad = 1;
                            break;
                        }
                        if (s_node[sx].w > s_node[sy].w) {  // the heavier set keeps its root (the second on equal)
                            const int t1 = px;
                            px = py;
                            py = t1;
                            const int t2 = sx;
                            sx = sy;
                            sy = t2;
                        }
                        const int st = t.slot(s_node[sy].tail);
                        if (st < 0) {
                            s_bad = 1;
                            break;
                        }
                        s_node[sy].w += s_node[sx].w;
                        s_node[sx].root = py;
                        s_node[st].next = px;
                        s_node[sy].tail = s_node[sx].tail;
                        for (int q = 0; q < 4; ++q)
                            if (rt[q] == px) rt[q] = py;
                    }
            }
        }
        __syncthreads();
        if (s_bad) {
            // the table filled up: the zone from global memory (untouched so far)
            if (tid == 0) {
                RootCache cache;
                for (int j = j0; j < j1; ++j) replay_record(uf, fixed, rec[vals[j]], cache);
            }
        } else {
            for (int h = tid; h < kTabSize; h += kReplayThreads)
                if (s_key[h] >= 0) uf[s_key[h]] = s_node[h];
        }
        __syncthreads();
    }
}

// Every zone of a scene in impact-zone mode: a root of two or more points.
// Each gets a contiguous run of the member array (zones in any order: each
// one's rigid motion depends on its own members only).
__global__ void k_zone_enum(const int* __restrict__ act_pts, int n, const int* __restrict__ dn,
                            const int* __restrict__ vscene, const SceneRun* __restrict__ run,
                            const UfNode* __restrict__ uf, PassCounters* ctr, int2* zone_rng, int* zone_root) {
    if (ctr->err & kErrRetry) return;
    if (dn) n = *dn;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int p = act_pts ? act_pts[k] : k;
        const UfNode u = uf[p];
        if (u.root != p || u.w < 2 || run[vscene[p]].mode != kSceneZone) continue;
        const int z = atomicAdd(&ctr->nzones, 1);
        const int m = atomicAdd(&ctr->nmembers, u.w);
        zone_rng[z] = make_int2(m, m + u.w);
        zone_root[z] = p;
    }
}

// The member list of every zone, from its root along the next links, one
// warp per zone. A root's list only ever grows at its end while the root
// stays a root (mergePoint appends the lighter set's list to the heavier
// one's), so a zone listed by the previous zone pass (prev_epoch == epoch)
// starts as a copy of that list, which the warp's lanes make together, and
// only the members appended since are walked.
__global__ void k_zone_members(const PassCounters* ctr, const int2* __restrict__ zone_rng,
                               const int* __restrict__ zone_root, const UfNode* __restrict__ uf, int* members,
                               const int* __restrict__ prev_members, const int* __restrict__ prev_off,
                               const int* __restrict__ prev_len, const unsigned* __restrict__ prev_epoch,
                               const unsigned* __restrict__ epoch) {
    if (ctr->err & kErrRetry) return;
    const int nz = ctr->nzones;
    const unsigned e = *epoch;
    const int lane = threadIdx.x & 31;
    for (int z = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; z < nz; z += (gridDim.x * blockDim.x) >> 5) {
        const int2 r = zone_rng[z];
        const int root = zone_root[z];
        int copied = 0;
        if (prev_epoch[root] == e) {
            const int off = prev_off[root];
            const int len = prev_len[root];
            copied = len < r.y - r.x ? len : r.y - r.x;
            for (int k = lane; k < copied; k += 32) members[r.x + k] = prev_members[off + k];
        }
        __syncwarp();
        if (lane == 0) {
            int p = copied > 0 ? uf[members[r.x + copied - 1]].next : root;
            for (int i = r.x + copied; i < r.y && p >= 0; ++i) {
                members[i] = p;
                p = uf[p].next;
            }
        }
    }
}

// This pass's lists as the next zone pass's previous ones.
__global__ void k_zone_save(const PassCounters* ctr, const int2* __restrict__ zone_rng,
                            const int* __restrict__ zone_root, const int* __restrict__ members, int* prev_members,
                            int* prev_off, int* prev_len, unsigned* prev_epoch, const unsigned* __restrict__ epoch) {
    if (ctr->err & kErrRetry) return;
    const int nz = ctr->nzones, nm = ctr->nmembers;
    const unsigned e = *epoch + 1u;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nm || i < nz; i += gridDim.x * blockDim.x) {
        if (i < nm) prev_members[i] = members[i];
        if (i < nz) {
            const int root = zone_root[i];
            const int2 r = zone_rng[i];
            prev_off[root] = r.x;
            prev_len[root] = r.y - r.x;
            prev_epoch[root] = e;
        }
    }
}

__global__ void k_zone_epoch(const PassCounters* ctr, unsigned* epoch) {
    if (ctr->err & kErrRetry) return;
    *epoch += 1u;
}

}  // namespace

// the sort's scratch, then two ints for the sorts' stage counts
size_t zone_sort_temp_bytes(int cap) { return radix_sort_temp_bytes(cap) + 256; }

cudaError_t zone_pass(const ZoneBufs& z, const PassCounters* ctr_c, const uint8_t* fixed, const int* act_pts,
                      int n_pts, const int* dn_pts, const int* vscene, const SceneRun* run, const SceneDev* scenes,
                      double4_32a* av, const double4_32a* xo, cudaStream_t s, PassStamp ps, cudaStream_t nested,
                      unsigned long long* marks, int mark0) {
    PassCounters* ctr = const_cast<PassCounters*>(ctr_c);
    const int cap = z.cap;
    int* eff = reinterpret_cast<int*>(static_cast<char*>(z.sort_temp) + radix_sort_temp_bytes(cap));
    const int blocks = nblk(cap, 256) < 152 * 8 ? nblk(cap, 256) : 152 * 8;
    count_launch(), k_cc_union<<<blocks, 256, 0, s>>>(z.rec, ctr, cap, fixed, z.cc);
    count_launch(), k_union_keys<<<blocks, 256, 0, s>>>(z.rec, ctr, cap, z.keys, z.vals);
    cudaError_t e = sort_pairs_dev(z.keys, z.vals, &ctr->nunion, cap, 48, z.sort_temp, eff, s, nested, z.small_sort);
    if (e != cudaSuccess) return e;
    count_launch(), k_union_labels<<<blocks, 256, 0, s>>>(z.rec, ctr, cap, fixed, z.cc, z.vals, z.keys);
    e = sort_pairs_dev(z.keys, z.vals, &ctr->nunion, cap, 31, z.sort_temp, eff + 1, s, nested, z.small_sort);
    if (e != cudaSuccess) return e;
    if (marks) stage_mark(marks, mark0, s);
    count_launch(), k_union_segments<<<blocks, 256, 0, s>>>(z.keys, ctr, cap, z.seg);
    const int big = z.replay_cta_min > 0 ? z.replay_cta_min : cap + 1;
    count_launch(), k_union_noop<<<blocks, 256, 0, s>>>(z.rec, ctr, cap, fixed, z.uf, z.noop);
    count_launch(), k_union_replay<<<blocks, 128, 0, s>>>(z.rec, ctr, cap, z.keys, z.vals, z.seg, fixed, z.uf, big,
                                                          z.noop);
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_union_replay_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTabBytes) !=
            cudaSuccess)
            return cudaGetLastError();
        attr = true;
    }
    if (z.replay_cta_min > 0)
        count_launch(), k_union_replay_cta<<<152, kReplayThreads, kTabBytes, s>>>(z.rec, ctr, cap, z.keys, z.vals,
                                                                                   z.seg, fixed, z.uf, big);
    if (marks) stage_mark(marks, mark0 + 1, s);
    const int pb = dn_pts ? 152 * 8 : (nblk(n_pts, 256) < 152 * 8 ? nblk(n_pts, 256) : 152 * 8);
    if (pb > 0)
        count_launch(), k_zone_enum<<<pb, 256, 0, s>>>(act_pts, n_pts, dn_pts, vscene, run, z.uf, ctr, z.zone_rng,
                                                       z.zone_root);
    const int zw = nblk(z.zone_cap, 4) < 152 * 8 ? nblk(z.zone_cap, 4) : 152 * 8;
    count_launch(), k_zone_members<<<zw, 128, 0, s>>>(ctr, z.zone_rng, z.zone_root, z.uf, z.members, z.prev_members,
                                                      z.prev_off, z.prev_len, z.prev_epoch, z.epoch);
    const int zs = nblk(z.n_pts_cap, 256) < 152 * 8 ? nblk(z.n_pts_cap, 256) : 152 * 8;
    count_launch(), k_zone_save<<<zs, 256, 0, s>>>(ctr, z.zone_rng, z.zone_root, z.members, z.prev_members,
                                                   z.prev_off, z.prev_len, z.prev_epoch, z.epoch);
    count_launch(), k_zone_epoch<<<1, 1, 0, s>>>(ctr, z.epoch);
    if (marks) stage_mark(marks, mark0 + 2, s);
    zone_solve_dev(z.members, z.zone_rng, &ctr->nzones, z.zone_cap, fixed, xo, av, vscene, scenes, ctr, s, ps,
                   z.zone_cta_min, z.zone_few);
    if (marks) stage_mark(marks, mark0 + 3, s);
    return cudaGetLastError();
}

}  // namespace ccg
