// Broad phase: linear BVH over the element boxes.
//
// Leaf boxes follow the reference exactly (CD_TRI/CD_BOND::min/max_*_coord,
// dcollid.cpp:852-932, padded by 1e-6 as AABB.cpp:6-36 does), and node boxes
// are exact min/max unions, so the overlap tests prune nothing that the
// reference's incremental tree would report: the pair set is the same set of
// all box-overlapping leaf pairs, whatever the tree shape. Morton keys (10 bits
// per axis) are sorted by the hand-written radix sort; the hierarchy is the
// Karras (2012) construction; refit walks up with arrival counters.
#include "cc_launch.h"

namespace ccg {

namespace {

__device__ __forceinline__ unsigned long long enc_double(double x) {
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dec_double(unsigned long long e) {
    unsigned long long u = (e & 0x8000000000000000ull) ? (e & 0x7fffffffffffffffull) : ~e;
    return __longlong_as_double((long long)u);
}

// dn (may be null): the boxes keep their last values when *dn is 0 (a pass
// that computes no new leaf boxes).
__global__ void k_bbox_init(unsigned long long* bb, int n6, const int* dn = nullptr) {
    if (dn && *dn == 0) return;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n6) bb[t] = (t % 6 < 3) ? ~0ull : 0ull;
}

// Per-scene union of boxes into bb[6*scene ..]: reduced across the warp when
// the whole warp lies in one scene (the common case: scenes are contiguous),
// else one atomic per lane.
__device__ __forceinline__ void scene_bbox_accumulate(unsigned long long* bb, int scene, bool valid,
                                                      const double* lo, const double* hi) {
    int s0 = __shfl_sync(0xffffffffu, scene, 0);
    bool uniform = __all_sync(0xffffffffu, scene == s0);
    for (int d = 0; d < 3; ++d) {
        double l = valid ? lo[d] : kBig, h = valid ? hi[d] : -kBig;
        if (uniform) {
            for (int o = 16; o > 0; o >>= 1) {
                l = fmin(l, __shfl_xor_sync(0xffffffffu, l, o));
                h = fmax(h, __shfl_xor_sync(0xffffffffu, h, o));
            }
            if ((threadIdx.x & 31) == 0 && l <= h && s0 >= 0) {
                atomicMin(&bb[6 * s0 + d], enc_double(l));
                atomicMax(&bb[6 * s0 + 3 + d], enc_double(h));
            }
        } else if (valid) {
            atomicMin(&bb[6 * scene + d], enc_double(l));
            atomicMax(&bb[6 * scene + 3 + d], enc_double(h));
        }
    }
}

template <int MOVING>
__device__ __forceinline__ void leaf_box(const int* __restrict__ ev, const int* __restrict__ act, int n, int k,
                                         const int* __restrict__ elem_scene, const SceneDev* __restrict__ scenes,
                                         const double4_32a* __restrict__ xo, const double4_32a* __restrict__ av,
                                         Box6* __restrict__ box, unsigned long long* bb) {
    bool valid = k < n;
    int e = valid ? (act ? act[k] : k) : 0;
    int scene = valid ? elem_scene[e] : -1;
    double lo[3] = {kBig, kBig, kBig}, hi[3] = {-kBig, -kBig, -kBig};
    if (valid) {
        double dt = scenes[scene].p.dt;
        int np = (ev[3 * e + 2] >= 0) ? 3 : 2;
        double mx[3] = {-kBig, -kBig, -kBig}, mn[3] = {kBig, kBig, kBig};
        for (int i = 0; i < np; ++i) {
            int p = ev[3 * e + i];
            double4_32a x = xo[p];
            double xs[3] = {x.x, x.y, x.z};
            if (MOVING) {
                double4_32a v = av[p];
                double vs[3] = {v.x, v.y, v.z};
                for (int d = 0; d < 3; ++d) {
                    mx[d] = smax(mx[d], xs[d]);
                    mx[d] = smax(mx[d], xs[d] + vs[d] * dt);
                    mn[d] = smin(mn[d], xs[d]);
                    mn[d] = smin(mn[d], xs[d] + vs[d] * dt);
                }
            } else {
                for (int d = 0; d < 3; ++d) {
                    mx[d] = smax(xs[d], mx[d]);
                    mn[d] = smin(xs[d], mn[d]);
                }
            }
        }
        Box6 b;
        for (int d = 0; d < 3; ++d) {
            b.lo[d] = mn[d] - kBoxPad;
            b.hi[d] = mx[d] + kBoxPad;
            lo[d] = b.lo[d];
            hi[d] = b.hi[d];
        }
        box[e] = b;
    }
    scene_bbox_accumulate(bb, scene, valid, lo, hi);
}

// dn (may be null): the element count in device memory; the grid strides.
template <int MOVING>
__global__ void k_leaf_boxes(const int* __restrict__ ev, const int* __restrict__ act, int n,
                             const int* __restrict__ dn, const int* __restrict__ elem_scene,
                             const SceneDev* __restrict__ scenes, const double4_32a* __restrict__ xo,
                             const double4_32a* __restrict__ av, Box6* __restrict__ box, unsigned long long* bb) {
    if (dn) n = *dn;
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
        leaf_box<MOVING>(ev, act, n, base + threadIdx.x, elem_scene, scenes, xo, av, box, bb);
}


// Union of n given boxes into bb (encoded as for k_leaf_boxes).
__global__ void k_boxes_bbox(const Box6* __restrict__ box, int n, unsigned long long* bb) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    double lo[3] = {kBig, kBig, kBig}, hi[3] = {-kBig, -kBig, -kBig};
    if (e < n) {
        Box6 b = box[e];
        for (int d = 0; d < 3; ++d) {
            lo[d] = b.lo[d];
            hi[d] = b.hi[d];
        }
    }
    for (int d = 0; d < 3; ++d) {
        double l = lo[d], h = hi[d];
        for (int o = 16; o > 0; o >>= 1) {
            l = fmin(l, __shfl_xor_sync(0xffffffffu, l, o));
            h = fmax(h, __shfl_xor_sync(0xffffffffu, h, o));
        }
        if ((threadIdx.x & 31) == 0 && l <= h) {
            atomicMin(&bb[d], enc_double(l));
            atomicMax(&bb[3 + d], enc_double(h));
        }
    }
}

__device__ __forceinline__ unsigned int expand_bits10(unsigned int v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(const Box6* __restrict__ box, const int* __restrict__ act, int n,
                         const int* __restrict__ elem_scene, const unsigned long long* bb, unsigned long long* keys,
                         unsigned int* order) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int e = act ? act[k] : k;
    Box6 b = box[e];
    int sc = elem_scene ? elem_scene[e] : 0;
    const unsigned long long* sb = bb + 6 * sc;
    unsigned int q[3];
    for (int d = 0; d < 3; ++d) {
        double lo = dec_double(sb[d]), hi = dec_double(sb[3 + d]);
        double c = 0.5 * (b.lo[d] + b.hi[d]);
        double ext = hi - lo;
        double t = ext > 0.0 ? (c - lo) / ext : 0.0;
        t = fmin(fmax(t, 0.0), 1.0);
        unsigned int v = (unsigned int)(t * 1023.0);
        q[d] = v > 1023u ? 1023u : v;
    }
    unsigned long long m = (unsigned long long)((expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) |
                                                expand_bits10(q[2]));
    keys[k] = ((unsigned long long)sc << 30) | m;
    order[k] = (unsigned int)e;
}

__device__ __forceinline__ int delta(const unsigned long long* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned long long a = keys[i], b = keys[j];
    if (a == b) return 64 + __clz((unsigned int)(i ^ j));
    return __clzll(a ^ b);
}

// Karras, "Maximizing parallelism in the construction of BVHs, octrees and
// k-d trees" (HPG 2012), with index tie-breaking for equal keys.
// With rope given, the node that splits sorted leaves gamma and gamma+1
// (every boundary has exactly one) records its right child as the rope of
// that boundary, or kRopeEnd where the two leaves' scenes differ (the scene
// id sits above the 30 Morton bits of the keys).
__global__ void k_karras(const unsigned long long* __restrict__ keys, int n, BvhNode32* node, int* range_hi,
                         int* range_lo, int* parent, int* rope) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(keys, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + (d < 0 ? d : 0);
    int lo = i < j ? i : j, hi = i < j ? j : i;
    int left = (lo == gamma) ? ~gamma : gamma;
    int right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    // children cover [lo, gamma] and [gamma + 1, hi]
    node[i].meta = make_int4(left, right, gamma, hi);
    range_hi[i] = hi;
    range_lo[i] = lo;
    if (left >= 0) parent[left] = i; else parent[n - 1 + ~left] = i;
    if (right >= 0) parent[right] = i; else parent[n - 1 + ~right] = i;
    if (i == 0) parent[0] = -1;
    if (rope) rope[gamma] = ((keys[gamma] ^ keys[gamma + 1]) >> 30) ? kRopeEnd : right;
}

// Each internal node's first child and rope: a node covering sorted leaves
// [lo, hi] is followed in depth-first order by the rope of boundary hi.
__global__ void k_ropes(const BvhNode32* __restrict__ node, const int* __restrict__ rope, int n, RopeNode* rn) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int4 meta = node[i].meta;
    const int hi = meta.w;
    *reinterpret_cast<int2*>(&rn[i].left) = make_int2(meta.x, hi < n - 1 ? rope[hi] : kRopeEnd);
}

struct Box32 {
    float lo[3], hi[3];
};

__device__ __forceinline__ Box32 box32_out(const Box6& b) {
    Box32 r;
    for (int d = 0; d < 3; ++d) {
        r.lo[d] = __double2float_rd(b.lo[d]);
        r.hi[d] = __double2float_ru(b.hi[d]);
    }
    return r;
}

__device__ __forceinline__ void unpack(const float4& b0, const float4& b1, const float4& b2, Box32& c0, Box32& c1) {
    c0.lo[0] = b0.x; c0.lo[1] = b0.y; c0.lo[2] = b0.z; c0.hi[0] = b0.w;
    c0.hi[1] = b1.x; c0.hi[2] = b1.y; c1.lo[0] = b1.z; c1.lo[1] = b1.w;
    c1.lo[2] = b2.x; c1.hi[0] = b2.y; c1.hi[1] = b2.z; c1.hi[2] = b2.w;
}

// Box of an internal node: the union of its record's two child boxes,
// written by another thread of the refit (read through L2).
__device__ __forceinline__ Box32 node_union_cg(const BvhNode32* nd) {
    const float4* q = reinterpret_cast<const float4*>(nd);
    Box32 a, b, m;
    unpack(__ldcg(q), __ldcg(q + 1), __ldcg(q + 2), a, b);
    for (int d = 0; d < 3; ++d) {
        m.lo[d] = fminf(a.lo[d], b.lo[d]);
        m.hi[d] = fmaxf(a.hi[d], b.hi[d]);
    }
    return m;
}

// Bottom-up refit: the second child to arrive at a node writes the node's
// two child boxes (leaf boxes rounded outward to FP32, internal children as
// the union of their own records), and with rn given the node's own box.
// With sub given, only those leaves and the nodes above them up to their
// scenes' roots (a node with one child in an idle scene sees one arrival).
__device__ __forceinline__ void refit_from(const Box6* __restrict__ box, const unsigned int* __restrict__ order,
                                           int n, int i, const int* __restrict__ parent, int* flags, BvhNode32* node,
                                           RopeNode* rn) {
    if (i < 0 || i >= n) return;  // sub lists sorted leaves of scenes of this hierarchy
    int nd = parent[n - 1 + i];
    while (nd >= 0) {
        __threadfence();
        if (atomicAdd(&flags[nd], 1) == 0) return;
        __threadfence();
        int4 meta = node[nd].meta;
        Box32 a = meta.x >= 0 ? node_union_cg(&node[meta.x]) : box32_out(box[order[~meta.x]]);
        Box32 b = meta.y >= 0 ? node_union_cg(&node[meta.y]) : box32_out(box[order[~meta.y]]);
        float4* q = reinterpret_cast<float4*>(&node[nd]);
        q[0] = make_float4(a.lo[0], a.lo[1], a.lo[2], a.hi[0]);
        q[1] = make_float4(a.hi[1], a.hi[2], b.lo[0], b.lo[1]);
        q[2] = make_float4(b.lo[2], b.hi[0], b.hi[1], b.hi[2]);
        if (rn) {
            float* o = rn[nd].lo;
            *reinterpret_cast<float4*>(o) = make_float4(fminf(a.lo[0], b.lo[0]), fminf(a.lo[1], b.lo[1]),
                                                        fminf(a.lo[2], b.lo[2]), fmaxf(a.hi[0], b.hi[0]));
            *reinterpret_cast<float2*>(o + 4) = make_float2(fmaxf(a.hi[1], b.hi[1]), fmaxf(a.hi[2], b.hi[2]));
        }
        nd = parent[nd];
    }
}

// Arrival at a node of the refit: an add with acquire-release semantics at
// GPU scope, so that the box the first child wrote before it is visible to
// the second child after it (one atomic instead of fence, atomic, fence).
__device__ __forceinline__ int arrive_acq_rel(int* p) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

// One child's box in its parent's record (child 0: b0, b1.xy; child 1:
// b1.zw, b2), written by that child's thread and read back through L2.
__device__ __forceinline__ void put_child(BvhNode32* nd, int side, const Box32& b) {
    float* f = reinterpret_cast<float*>(nd);
    if (side == 0) {
        *reinterpret_cast<float4*>(f) = make_float4(b.lo[0], b.lo[1], b.lo[2], b.hi[0]);
        *reinterpret_cast<float2*>(f + 4) = make_float2(b.hi[1], b.hi[2]);
    } else {
        *reinterpret_cast<float2*>(f + 6) = make_float2(b.lo[0], b.lo[1]);
        *reinterpret_cast<float4*>(f + 8) = make_float4(b.lo[2], b.hi[0], b.hi[1], b.hi[2]);
    }
}
__device__ __forceinline__ Box32 get_child_cg(const BvhNode32* nd, int side) {
    const float* f = reinterpret_cast<const float*>(nd);
    Box32 b;
    if (side == 0) {
        const float4 a = __ldcg(reinterpret_cast<const float4*>(f));
        const float2 c = __ldcg(reinterpret_cast<const float2*>(f + 4));
        b.lo[0] = a.x; b.lo[1] = a.y; b.lo[2] = a.z; b.hi[0] = a.w; b.hi[1] = c.x; b.hi[2] = c.y;
    } else {
        const float2 a = __ldcg(reinterpret_cast<const float2*>(f + 6));
        const float4 c = __ldcg(reinterpret_cast<const float4*>(f + 8));
        b.lo[0] = a.x; b.lo[1] = a.y; b.lo[2] = c.x; b.hi[0] = c.y; b.hi[1] = c.z; b.hi[2] = c.w;
    }
    return b;
}

// The same refit with a shorter chain per level. Each thread carries its
// subtree's box in registers and writes it into its side of the parent's
// record before arriving; the second arrival reads only the other side
// (one L2 round trip), and the next node's children and parent are loaded
// while the arrival is in flight. The walk ends at the leaf's scene root
// (run given; the node records above it, which mix scenes, are read by no
// traversal), so passes over many scenes do not climb the levels between
// scenes. The records and rope boxes it writes equal refit_from's.
__device__ __forceinline__ void refit_up(const Box6* __restrict__ box, const unsigned int* __restrict__ order, int n,
                                         int i, const int* __restrict__ parent, int* flags, BvhNode32* node,
                                         RopeNode* rn, const unsigned long long* __restrict__ keys,
                                         const SceneRun* __restrict__ run) {
    if (i < 0 || i >= n) return;
    int root = -1;  // one scene: up to the top
    if (run) {
        root = run[(int)(keys[i] >> 30)].root;
        if (root < 0) return;  // a scene of one element: no pairs, no nodes
    }
    Box32 mine = box32_out(box[order[i]]);
    int child = ~i;
    int nd = parent[n - 1 + i];
    if (nd < 0) return;
    int4 meta = node[nd].meta;
    int up = parent[nd];
    for (;;) {
        const int side = meta.x == child ? 0 : 1;
        put_child(&node[nd], side, mine);
        int4 meta_up = make_int4(0, 0, 0, 0);
        int up2 = -1;
        if (nd != root && up >= 0) {
            meta_up = node[up].meta;
            up2 = parent[up];
        }
        if (arrive_acq_rel(&flags[nd]) == 0) return;
        const Box32 other = get_child_cg(&node[nd], side ^ 1);
        for (int d = 0; d < 3; ++d) {
            mine.lo[d] = fminf(mine.lo[d], other.lo[d]);
            mine.hi[d] = fmaxf(mine.hi[d], other.hi[d]);
        }
        if (rn) {
            float* o = rn[nd].lo;
            *reinterpret_cast<float4*>(o) = make_float4(mine.lo[0], mine.lo[1], mine.lo[2], mine.hi[0]);
            *reinterpret_cast<float2*>(o + 4) = make_float2(mine.hi[1], mine.hi[2]);
        }
        if (nd == root || up < 0) return;
        child = nd;
        nd = up;
        meta = meta_up;
        up = up2;
    }
}

// dnsub (may be null): the count of sub in device memory; the grid strides.
// UP: refit_up (keys and run used), else refit_from.
template <bool UP>
__global__ void k_refit(const Box6* __restrict__ box, const unsigned int* __restrict__ order, int n,
                        const int* __restrict__ sub, int nsub, const int* __restrict__ dnsub,
                        const int* __restrict__ parent, int* flags, BvhNode32* node, RopeNode* rn,
                        const unsigned long long* __restrict__ keys, const SceneRun* __restrict__ run) {
    const int m = sub ? (dnsub ? *dnsub : nsub) : n;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        if (UP)
            refit_up(box, order, n, sub ? sub[k] : k, parent, flags, node, rn, keys, run);
        else
            refit_from(box, order, n, sub ? sub[k] : k, parent, flags, node, rn);
    }
}

// The LBVH node whose leaves are exactly scene s's (keys carry the scene id
// in their high bits, so every scene owns one subtree).
__global__ void k_scene_roots(const SceneDev* __restrict__ scenes, SceneRun* run, int nscenes, int n,
                              const int* __restrict__ parent, const int* __restrict__ range_lo,
                              const int* __restrict__ range_hi) {
    int sc = blockIdx.x * blockDim.x + threadIdx.x;
    if (sc >= nscenes) return;
    int first = run[sc].leaf0, last = first + scenes[sc].ne - 1;
    if (scenes[sc].ne < 2 || first < 0) {
        run[sc].root = -1;
        return;
    }
    int node = parent[n - 1 + first];
    while (node >= 0 && !(range_lo[node] <= first && range_hi[node] >= last)) node = parent[node];
    run[sc].root = node;
}

__device__ __forceinline__ bool overlap32(const Box32& a, const Box32& b) {
    return (a.lo[0] <= b.hi[0] && a.hi[0] >= b.lo[0]) && (a.lo[1] <= b.hi[1] && a.hi[1] >= b.lo[1]) &&
           (a.lo[2] <= b.hi[2] && a.hi[2] >= b.lo[2]);
}

// Doubles as order-preserving unsigned integers (-0 as +0), so that exact
// box comparisons run on the integer pipe.
__device__ __forceinline__ unsigned long long ord_double(unsigned long long u) {
    if (u == 0x8000000000000000ull) u = 0;
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
// The double ord_double encodes (-0.0 comes back as +0.0).
__device__ __forceinline__ double unord_double(unsigned long long o) {
    return __longlong_as_double((long long)((o & 0x8000000000000000ull) ? (o & 0x7fffffffffffffffull) : ~o));
}
struct BoxOrd {
    unsigned long long lo[3], hi[3];
};
__device__ __forceinline__ BoxOrd box_ord(const Box6& b) {
    BoxOrd r;
    for (int d = 0; d < 3; ++d) {
        r.lo[d] = ord_double((unsigned long long)__double_as_longlong(b.lo[d]));
        r.hi[d] = ord_double((unsigned long long)__double_as_longlong(b.hi[d]));
    }
    return r;
}
// Box6 a vs box b in memory, exactly as overlap(a, b).
__device__ __forceinline__ bool overlap_ord(const BoxOrd& a, const Box6* bp) {
    const ulonglong2* q = reinterpret_cast<const ulonglong2*>(bp);
    ulonglong2 u0 = __ldg(q), u1 = __ldg(q + 1), u2 = __ldg(q + 2);
    unsigned long long lo[3] = {u0.x, u0.y, u1.x}, hi[3] = {u1.y, u2.x, u2.y};
    for (int d = 0; d < 3; ++d)
        if (!(a.lo[d] <= ord_double(hi[d]) && a.hi[d] >= ord_double(lo[d]))) return false;
    return true;
}

__device__ __forceinline__ bool overlap(const Box6& a, const Box6& b) {
    return (a.lo[0] <= b.hi[0] && a.hi[0] >= b.lo[0]) && (a.lo[1] <= b.hi[1] && a.hi[1] >= b.lo[1]) &&
           (a.lo[2] <= b.hi[2] && a.hi[2] >= b.lo[2]);
}

__device__ __forceinline__ void emit_pair(int a, int b, int2* pairs, int cap, PassCounters* ctr) {
    int slot = aggregated_add(&ctr->npairs, 1);
    if (slot < cap)
        pairs[slot] = make_int2(a, b);
    else
        atomicOr(&ctr->err, kErrPairOverflow);
}

// One thread per sorted leaf i reports every leaf j > i of its scene whose
// box overlaps, starting from the scene's subtree root; leaves of scenes
// idle in this pass report nothing. With ev given, pairs of elements that
// share a point are dropped: every narrow-phase test of such a pair returns
// false before any arithmetic (dcollid3d.cpp:493-497, 541-546, 578-582).
// The leaf records of one pass (see LeafRec).
__device__ __forceinline__ void leaf_record(const Box6* __restrict__ box, const unsigned int* __restrict__ order,
                                            int n, int j, const int* __restrict__ ev, LeafRec* out, int ne_all,
                                            PassCounters* ctr, const int* __restrict__ rope, LeafBox32* out32) {
    if (j < 0 || j >= n) {
        atomicOr(&ctr->err, kErrIndexLeaf);
        return;
    }
    const int e = (int)order[j];
    if (e < 0 || e >= ne_all) {
        atomicOr(&ctr->err, kErrIndexElem);
        LeafRec r = {};
        r.e = -1;  // tested by nobody: the traversal skips it
        out[j] = r;
        if (out32) {
            LeafBox32 q = {};
            q.rope = j < n - 1 ? rope[j] : kRopeEnd;
            q.e = -1;
            out32[j] = q;
        }
        return;
    }
    const Box6 bx = box[e];
    if (out32) {
        const Box32 f = box32_out(bx);
        float4* q = reinterpret_cast<float4*>(&out32[j]);
        q[0] = make_float4(f.lo[0], f.lo[1], f.lo[2], f.hi[0]);
        q[1] = make_float4(f.hi[1], f.hi[2], __int_as_float(j < n - 1 ? rope[j] : kRopeEnd), __int_as_float(e));
    }
    const BoxOrd o = box_ord(bx);
    LeafRec r;
    for (int d = 0; d < 3; ++d) {
        r.lo[d] = o.lo[d];
        r.hi[d] = o.hi[d];
    }
    r.p[0] = ev[3 * e];
    r.p[1] = ev[3 * e + 1];
    r.p[2] = ev[3 * e + 2];
    r.e = e;
    out[j] = r;
}

// dnsub (may be null): the count of sub in device memory; the grid strides.
__global__ void k_leaf_records(const Box6* __restrict__ box, const unsigned int* __restrict__ order, int n,
                               const int* __restrict__ sub, int nsub, const int* __restrict__ dnsub,
                               const int* __restrict__ ev, LeafRec* out, int ne_all, PassCounters* ctr,
                               const int* __restrict__ rope, LeafBox32* out32) {
    const int m = sub ? (dnsub ? *dnsub : nsub) : n;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x)
        leaf_record(box, order, n, sub ? sub[k] : k, ev, out, ne_all, ctr, rope, out32);
}

// The same pairs from a warp-cooperative traversal. The 32 lanes of a warp
// hold 32 consecutive sorted leaves - neighbours in Morton order, so their
// paths through the tree mostly coincide - and walk the tree as one packet:
// one node record per step, read once for the warp, a stack per warp in
// shared memory, and a child pushed when the ballot of the lanes whose query
// box overlaps it (and that have leaves after theirs below it) is not
// empty. Leaves reached are tested exactly by the lanes that overlap them.
// Lanes of different scenes (different subtree roots) walk in turn.
constexpr int kPacketWarps = 8;
__global__ void __launch_bounds__(kPacketWarps * 32) k_traverse_packet(
    const unsigned int* __restrict__ order, int n, const BvhNode32* __restrict__ node,
    const int* __restrict__ elem_scene, const SceneRun* __restrict__ run, const int* __restrict__ ev, int2* pairs,
    int cap, PassCounters* ctr, const Box6* __restrict__ box_static, const LeafRec* __restrict__ leaves) {
    __shared__ int s_stack[kPacketWarps][kTraversalStack];
    int* stk = s_stack[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool want = i < n - 1;
    int ei = -1, root = -1, pi0 = -1, pi1 = -1, pi2 = -1;
    Box32 q32;
    BoxOrd qo, qs;
    if (want) {
        const LeafRec r = leaves[i];
        ei = r.e;
        if (ei < 0) want = false;
        Box6 q;
        for (int d = 0; d < 3; ++d) {
            qo.lo[d] = r.lo[d];
            qo.hi[d] = r.hi[d];
            q.lo[d] = unord_double(r.lo[d]);
            q.hi[d] = unord_double(r.hi[d]);
        }
        q32 = box32_out(q);
        if (ev) pi0 = r.p[0], pi1 = r.p[1], pi2 = r.p[2];
        root = 0;
        if (want && run) {
            const SceneRun sr = run[elem_scene[ei]];
            if (sr.mode == kSceneIdle || sr.root < 0) want = false;
            root = sr.root;
        }
        if (want && root >= n - 1) {
            atomicOr(&ctr->err, kErrIndexNode);
            want = false;
        }
        if (want && box_static) qs = box_ord(box_static[ei]);
    }
    unsigned todo = __ballot_sync(0xffffffffu, want);
    while (todo) {
        // this round: the lanes that share the first remaining lane's root
        const int r0 = __shfl_sync(0xffffffffu, root, __ffs(todo) - 1);
        const bool mine = want && root == r0;
        const unsigned in_round = __ballot_sync(0xffffffffu, mine);
        todo &= ~in_round;
        int sp = 1;
        if (lane == 0) stk[0] = r0;
        __syncwarp();
        while (sp > 0) {
            const int nd_id = stk[--sp];  // checked when pushed: in [0, n-1)
            const float4* r4 = reinterpret_cast<const float4*>(&node[nd_id]);
            Box32 cb[2];
            unpack(__ldg(r4), __ldg(r4 + 1), __ldg(r4 + 2), cb[0], cb[1]);
            const int4 meta = __ldg(reinterpret_cast<const int4*>(r4 + 3));
            const int cs[2] = {meta.x, meta.y}, last[2] = {meta.z, meta.w};
            __syncwarp();  // every lane has read the top before it is overwritten
            for (int k = 0; k < 2; ++k) {
                const bool hit = mine && last[k] > i && overlap32(q32, cb[k]);
                if (!__any_sync(0xffffffffu, hit)) continue;
                const int c = cs[k];
                if (c < 0) {
                    if (!hit) continue;
                    if (~c >= n) {
                        atomicOr(&ctr->err, kErrIndexLeaf);
                        continue;
                    }
                    const ulonglong2* lr = reinterpret_cast<const ulonglong2*>(&leaves[~c]);
                    const ulonglong2 u0 = __ldg(lr), u1 = __ldg(lr + 1), u2 = __ldg(lr + 2);
                    const int4 pe = __ldg(reinterpret_cast<const int4*>(lr + 3));
                    if (!(qo.lo[0] <= u1.y && qo.hi[0] >= u0.x && qo.lo[1] <= u2.x && qo.hi[1] >= u0.y &&
                          qo.lo[2] <= u2.y && qo.hi[2] >= u1.x))
                        continue;
                    if (ev && (pe.x == pi0 || pe.x == pi1 || pe.x == pi2 || pe.y == pi0 || pe.y == pi1 ||
                               pe.y == pi2 || (pe.z >= 0 && (pe.z == pi0 || pe.z == pi1 || pe.z == pi2))))
                        continue;
                    const int ej = pe.w;
                    if (ej < 0) continue;  // flagged by k_leaf_records
                    emit_pair(ei, (box_static && overlap_ord(qs, &box_static[ej])) ? (ej | kPairStatic) : ej, pairs,
                              cap, ctr);
                } else if (c >= n - 1) {
                    if (lane == 0) atomicOr(&ctr->err, kErrIndexNode);
                } else if (sp < kTraversalStack) {
                    if (lane == 0) stk[sp] = c;
                    ++sp;
                } else {
                    if (lane == 0) atomicOr(&ctr->err, kErrStack);
                }
            }
            __syncwarp();  // pushes are visible before the next pop
        }
    }
}

template <int DEPTH>
__device__ __forceinline__ void traverse_stack(const Box6* __restrict__ box, const unsigned int* __restrict__ order,
                                               int n, const BvhNode32* __restrict__ node,
                                               const int* __restrict__ elem_scene, const SceneRun* __restrict__ run,
                                               const int* __restrict__ ev, int2* pairs, int cap, PassCounters* ctr,
                                               const Box6* __restrict__ box_static,
                                               const LeafRec* __restrict__ leaves, int i) {
    if (i >= n - 1) return;  // the last leaf has no leaf after it
    if (i < 0) {
        atomicOr(&ctr->err, kErrIndexLeaf);
        return;
    }
    int ei, pi0 = -1, pi1 = -1, pi2 = -1;
    Box6 q;
    BoxOrd qo;
    if (leaves) {  // the query's own record: a coalesced load
        const LeafRec r = leaves[i];
        ei = r.e;
        if (ei < 0) return;  // flagged by k_leaf_records
        for (int d = 0; d < 3; ++d) {
            qo.lo[d] = r.lo[d];
            qo.hi[d] = r.hi[d];
            q.lo[d] = unord_double(r.lo[d]);
            q.hi[d] = unord_double(r.hi[d]);
        }
        if (ev) pi0 = r.p[0], pi1 = r.p[1], pi2 = r.p[2];  // -1 for a bond: matches no point
    } else {
        ei = (int)order[i];
        if (ev) {
            pi0 = ev[3 * ei];
            pi1 = ev[3 * ei + 1];
            pi2 = ev[3 * ei + 2];
        }
        q = box[ei];
        qo = box_ord(q);
    }
    int root = 0;
    if (run) {
        SceneRun r = run[elem_scene[ei]];
        if (r.mode == kSceneIdle || r.root < 0) return;
        root = r.root;
        if (root >= n - 1) {
            atomicOr(&ctr->err, kErrIndexNode);
            return;
        }
    }
    const Box32 q32 = box32_out(q);
    BoxOrd qs;
    if (box_static) qs = box_ord(box_static[ei]);
    int stk[DEPTH];
    int sp = 0;
    stk[sp++] = root;
    while (sp > 0) {
        const BvhNode32* nd = &node[stk[--sp]];
        const float4* r4 = reinterpret_cast<const float4*>(nd);
        Box32 cb[2];
        unpack(__ldg(r4), __ldg(r4 + 1), __ldg(r4 + 2), cb[0], cb[1]);
        const int4 meta = __ldg(reinterpret_cast<const int4*>(r4 + 3));
        const int cs[2] = {meta.x, meta.y}, last[2] = {meta.z, meta.w};
        for (int k = 0; k < 2; ++k) {
            // nothing under this child lies after leaf i
            if (last[k] <= i || !overlap32(q32, cb[k])) continue;
            int c = cs[k];
            if (c < 0) {
                int ej, a, b, c3;
                if (~c >= n) {
                    atomicOr(&ctr->err, kErrIndexLeaf);
                    continue;
                }
                if (leaves) {
                    const ulonglong2* lr = reinterpret_cast<const ulonglong2*>(&leaves[~c]);
                    const ulonglong2 u0 = __ldg(lr), u1 = __ldg(lr + 1), u2 = __ldg(lr + 2);
                    const int4 pe = __ldg(reinterpret_cast<const int4*>(lr + 3));
                    // the exact test on the encoded boxes
                    if (!(qo.lo[0] <= u1.y && qo.hi[0] >= u0.x && qo.lo[1] <= u2.x && qo.hi[1] >= u0.y &&
                          qo.lo[2] <= u2.y && qo.hi[2] >= u1.x))
                        continue;
                    ej = pe.w;
                    if (ej < 0) continue;  // flagged by k_leaf_records
                    a = pe.x, b = pe.y, c3 = pe.z;
                } else {
                    ej = (int)order[~c];
                    if (!overlap_ord(qo, &box[ej])) continue;  // the exact test
                    if (ev) a = ev[3 * ej], b = ev[3 * ej + 1], c3 = ev[3 * ej + 2];
                }
                bool shared = false;
                if (ev)
                    shared = a == pi0 || a == pi1 || a == pi2 || b == pi0 || b == pi1 || b == pi2 ||
                             (c3 >= 0 && (c3 == pi0 || c3 == pi1 || c3 == pi2));
                if (!shared)
                    emit_pair(ei, (box_static && overlap_ord(qs, &box_static[ej])) ? (ej | kPairStatic) : ej, pairs,
                              cap, ctr);
            } else if (c >= n - 1) {
                atomicOr(&ctr->err, kErrIndexNode);
            } else if (sp < DEPTH) {
                stk[sp++] = c;
            } else {
                atomicOr(&ctr->err, kErrStack);
            }
        }
    }
}

// One thread per query leaf (sub, or all leaves but the last); dnsub (may be
// null): the count of sub in device memory, the grid striding over it.
template <int DEPTH>
__global__ void k_traverse(const Box6* __restrict__ box, const unsigned int* __restrict__ order, int n,
                           const BvhNode32* __restrict__ node, const int* __restrict__ elem_scene,
                           const SceneRun* __restrict__ run, const int* __restrict__ ev, int2* pairs, int cap,
                           PassCounters* ctr, const Box6* __restrict__ box_static,
                           const LeafRec* __restrict__ leaves, const int* __restrict__ sub, int nsub,
                           const int* __restrict__ dnsub) {
    const int m = sub ? (dnsub ? *dnsub : nsub) : n - 1;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m; t += gridDim.x * blockDim.x)
        traverse_stack<DEPTH>(box, order, n, node, elem_scene, run, ev, pairs, cap, ctr, box_static, leaves,
                              sub ? sub[t] : t);
}

// The same pairs without a stack. Thread i starts at the rope of its own
// leaf - the subtree right after leaf i in depth-first order - so the nodes
// above leaf i are never visited and only leaves after i are reached; an
// overlapping node is entered at its first child, any other node (or leaf)
// is left along its rope, and the walk ends at its scene's end (kRopeEnd).
// Every step moves forward in depth-first order, so a walk takes fewer than
// 2n steps; a longer one, or an index outside its array, sets an error bit
// and ends the thread.
__device__ __forceinline__ void traverse_rope(int n, const RopeNode* __restrict__ rn, const int* __restrict__ rope,
                                              const int* __restrict__ elem_scene, const SceneRun* __restrict__ run,
                                              const int* __restrict__ ev, int2* pairs, int cap, PassCounters* ctr,
                                              const Box6* __restrict__ box_static,
                                              const LeafRec* __restrict__ leaves, int i) {
    if (i >= n - 1) return;  // the last leaf has no leaf after it
    if (i < 0) {
        atomicOr(&ctr->err, kErrIndexLeaf);
        return;
    }
    const LeafRec r = leaves[i];
    const int ei = r.e;
    if (ei < 0) return;  // flagged by k_leaf_records
    if (run) {
        const SceneRun sr = run[elem_scene[ei]];
        if (sr.mode == kSceneIdle || sr.root < 0) return;
    }
    BoxOrd qo;
    Box6 q;
    for (int d = 0; d < 3; ++d) {
        qo.lo[d] = r.lo[d];
        qo.hi[d] = r.hi[d];
        q.lo[d] = unord_double(r.lo[d]);
        q.hi[d] = unord_double(r.hi[d]);
    }
    const int pi0 = ev ? r.p[0] : -1, pi1 = ev ? r.p[1] : -1, pi2 = ev ? r.p[2] : -1;
    const Box32 q32 = box32_out(q);
    BoxOrd qs;
    if (box_static) qs = box_ord(box_static[ei]);
    int x = __ldg(&rope[i]);
    for (int steps = 0; x != kRopeEnd; ++steps) {
        if (steps >= 2 * n) {
            atomicOr(&ctr->err, kErrIndexNode);
            return;
        }
        if (x >= 0) {
            if (x >= n - 1) {
                atomicOr(&ctr->err, kErrIndexNode);
                return;
            }
            const float4* p4 = reinterpret_cast<const float4*>(&rn[x]);
            const float4 a = __ldg(p4), b = __ldg(p4 + 1);  // lo xyz hi.x | hi.y hi.z left rope
            const bool hit = q32.lo[0] <= a.w && q32.hi[0] >= a.x && q32.lo[1] <= b.x && q32.hi[1] >= a.y &&
                             q32.lo[2] <= b.y && q32.hi[2] >= a.z;
            x = __float_as_int(hit ? b.z : b.w);
            continue;
        }
        const int k = ~x;
        if (k >= n) {
            atomicOr(&ctr->err, kErrIndexLeaf);
            return;
        }
        x = k < n - 1 ? __ldg(&rope[k]) : kRopeEnd;
        const ulonglong2* lr = reinterpret_cast<const ulonglong2*>(&leaves[k]);
        const ulonglong2 u0 = __ldg(lr), u1 = __ldg(lr + 1), u2 = __ldg(lr + 2);
        // the exact test on the encoded boxes
        if (!(qo.lo[0] <= u1.y && qo.hi[0] >= u0.x && qo.lo[1] <= u2.x && qo.hi[1] >= u0.y && qo.lo[2] <= u2.y &&
              qo.hi[2] >= u1.x))
            continue;
        const int4 pe = __ldg(reinterpret_cast<const int4*>(lr + 3));
        const int ej = pe.w;
        if (ej < 0) continue;  // flagged by k_leaf_records
        if (ev && (pe.x == pi0 || pe.x == pi1 || pe.x == pi2 || pe.y == pi0 || pe.y == pi1 || pe.y == pi2 ||
                   (pe.z >= 0 && (pe.z == pi0 || pe.z == pi1 || pe.z == pi2))))
            continue;
        emit_pair(ei, (box_static && overlap_ord(qs, &box_static[ej])) ? (ej | kPairStatic) : ej, pairs, cap, ctr);
    }
}

// One thread per query leaf (sub, or all leaves but the last); dnsub (may be
// null): the count of sub in device memory, the grid striding over it.
__global__ void k_traverse_rope(int n, const RopeNode* __restrict__ rn, const int* __restrict__ rope,
                                const int* __restrict__ elem_scene, const SceneRun* __restrict__ run,
                                const int* __restrict__ ev, int2* pairs, int cap, PassCounters* ctr,
                                const Box6* __restrict__ box_static, const LeafRec* __restrict__ leaves,
                                const int* __restrict__ sub, int nsub, const int* __restrict__ dnsub) {
    const int m = sub ? (dnsub ? *dnsub : nsub) : n - 1;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m; t += gridDim.x * blockDim.x)
        traverse_rope(n, rn, rope, elem_scene, run, ev, pairs, cap, ctr, box_static, leaves, sub ? sub[t] : t);
}

// The stackless walk with dynamic query fetch. The walks of neighbouring
// queries differ in length, and with one thread per query a warp runs until
// its longest walk ends while its other lanes idle. Here warps stay resident
// and a lane whose walk has ended takes the next query from a global counter:
// once at least `refill` lanes of a warp are idle, they fetch that many
// consecutive queries with one atomic. A leaf is tested first on its 32-byte
// FP32 record (outward-rounded box, rope, element), and only a leaf that
// passes loads its 64-byte exact record. Same pairs as k_traverse_rope.
__global__ void __launch_bounds__(128) k_traverse_rope_dyn(
    int n, const RopeNode* __restrict__ rn, const int* __restrict__ elem_scene, const SceneRun* __restrict__ run,
    const int* __restrict__ ev, int2* pairs, int cap, PassCounters* ctr, const Box6* __restrict__ box_static,
    const LeafRec* __restrict__ leaves, const LeafBox32* __restrict__ leaf32, const int* __restrict__ sub, int nsub,
    const int* __restrict__ dnsub, int* qnext, int refill) {
    const int nq = sub ? (dnsub ? *dnsub : nsub) : n - 1;
    const unsigned lane_lt = (1u << (threadIdx.x & 31)) - 1u;
    int x = kRopeEnd, ei = -1, steps = 0;
    int pi0 = -1, pi1 = -1, pi2 = -1;
    BoxOrd qo, qs;
    Box32 q32;
    bool more = true;  // queries left to fetch (warp-uniform)
    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, x == kRopeEnd);
        if (more && (__popc(idle) >= refill || idle == 0xffffffffu)) {
            int base = 0;
            const int want = __popc(idle);
            if ((threadIdx.x & 31) == __ffs(idle) - 1) base = atomicAdd(qnext, want);
            base = __shfl_sync(0xffffffffu, base, __ffs(idle) - 1);
            if (base + want >= nq) more = false;
            const int t = base + __popc(idle & lane_lt);
            if (x == kRopeEnd && t < nq) {
                // a new query: its own leaf record, then the rope after it
                const int i = sub ? sub[t] : t;
                if (i < 0) {
                    atomicOr(&ctr->err, kErrIndexLeaf);
                } else if (i < n - 1) {
                    const LeafRec r = leaves[i];
                    ei = r.e;
                    bool on = ei >= 0;  // negative: flagged by k_leaf_records
                    if (on && run) {
                        const SceneRun sr = run[elem_scene[ei]];
                        on = sr.mode != kSceneIdle && sr.root >= 0;
                    }
                    if (on) {
                        Box6 q;
                        for (int d = 0; d < 3; ++d) {
                            qo.lo[d] = r.lo[d];
                            qo.hi[d] = r.hi[d];
                            q.lo[d] = unord_double(r.lo[d]);
                            q.hi[d] = unord_double(r.hi[d]);
                        }
                        q32 = box32_out(q);
                        if (ev) pi0 = r.p[0], pi1 = r.p[1], pi2 = r.p[2];
                        if (box_static) qs = box_ord(box_static[ei]);
                        x = __float_as_int(__ldg(reinterpret_cast<const float*>(&leaf32[i]) + 6));
                        steps = 0;
                    }
                }
            }
        }
        if (!more && __all_sync(0xffffffffu, x == kRopeEnd)) break;
        if (x == kRopeEnd) continue;
        if (++steps > 2 * n) {
            atomicOr(&ctr->err, kErrIndexNode);
            x = kRopeEnd;
            continue;
        }
        if (x >= 0) {
            if (x >= n - 1) {
                atomicOr(&ctr->err, kErrIndexNode);
                x = kRopeEnd;
                continue;
            }
            const float4* p4 = reinterpret_cast<const float4*>(&rn[x]);
            const float4 a = __ldg(p4), b = __ldg(p4 + 1);  // lo xyz hi.x | hi.y hi.z left rope
            const bool hit = q32.lo[0] <= a.w && q32.hi[0] >= a.x && q32.lo[1] <= b.x && q32.hi[1] >= a.y &&
                             q32.lo[2] <= b.y && q32.hi[2] >= a.z;
            x = __float_as_int(hit ? b.z : b.w);
            continue;
        }
        const int k = ~x;
        if (k >= n) {
            atomicOr(&ctr->err, kErrIndexLeaf);
            x = kRopeEnd;
            continue;
        }
        const float4* l4 = reinterpret_cast<const float4*>(&leaf32[k]);
        const float4 a = __ldg(l4), b = __ldg(l4 + 1);  // lo xyz hi.x | hi.y hi.z rope e
        x = __float_as_int(b.z);
        // the FP32 boxes hold the exact ones: a miss here is a miss
        if (!(q32.lo[0] <= a.w && q32.hi[0] >= a.x && q32.lo[1] <= b.x && q32.hi[1] >= a.y && q32.lo[2] <= b.y &&
              q32.hi[2] >= a.z))
            continue;
        const int ej = __float_as_int(b.w);
        if (ej < 0) continue;  // flagged by k_leaf_records
        const ulonglong2* lr = reinterpret_cast<const ulonglong2*>(&leaves[k]);
        const ulonglong2 u0 = __ldg(lr), u1 = __ldg(lr + 1), u2 = __ldg(lr + 2);
        // the exact test on the encoded boxes
        if (!(qo.lo[0] <= u1.y && qo.hi[0] >= u0.x && qo.lo[1] <= u2.x && qo.hi[1] >= u0.y && qo.lo[2] <= u2.y &&
              qo.hi[2] >= u1.x))
            continue;
        if (ev) {
            const int4 pe = __ldg(reinterpret_cast<const int4*>(lr + 3));
            if (pe.x == pi0 || pe.x == pi1 || pe.x == pi2 || pe.y == pi0 || pe.y == pi1 || pe.y == pi2 ||
                (pe.z >= 0 && (pe.z == pi0 || pe.z == pi1 || pe.z == pi2)))
                continue;
        }
        emit_pair(ei, (box_static && overlap_ord(qs, &box_static[ej])) ? (ej | kPairStatic) : ej, pairs, cap, ctr);
    }
}

// The queries of a pruned pass. Its scenes ran the previous pass too (a
// scene runs its passes one after the other until it is done), and an
// element pair none of whose points that pass touched - no impulse, no
// impact-zone or rigid-body motion, no hitting sub-test - has the inputs it
// had when it was last tested: in the pass after the last change of one of
// its points, or in the step's first CCD pass, which tests every pair.
// There it did not hit (a hit stamps the sub-test's points), so it does not
// hit now, and the pass needs only the pairs with an element holding a
// point stamped by the previous pass ("dirty"). Flags the element of every
// sorted leaf of the pass (act_l: the pass's leaves; order: the element of
// each sorted leaf) and lists the dirty ones' leaves.
__global__ void k_dirty_queries(const int* __restrict__ act_l, const unsigned int* __restrict__ order, int n_hier,
                                int ne_all, const int* __restrict__ ev, const unsigned* __restrict__ stamp, LoopCtl* L,
                                uint8_t* edirty, int* query, PassCounters* ctr) {
    if (!L->prune) return;
    const int n = L->nact_e;
    // stamped by the previous pass - or by this pass's own earlier attempt,
    // when it stopped for a larger buffer after its narrow phase had stamped
    // hits and now runs again: those points were dirty before it, or are
    // touched by it now (a superset is safe)
    const unsigned prev = L->serial - 1u, cur = L->serial;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int j = act_l[k];
        const int e = (j >= 0 && j < n_hier) ? (int)order[j] : -1;
        if (e < 0 || e >= ne_all) {
            atomicOr(&ctr->err, kErrIndexLeaf);
            continue;
        }
        const int p2 = ev[3 * e + 2];
        const unsigned s0 = stamp[ev[3 * e]], s1 = stamp[ev[3 * e + 1]], s2 = p2 >= 0 ? stamp[p2] : 0u;
        const bool d = s0 == prev || s0 == cur || s1 == prev || s1 == cur || (p2 >= 0 && (s2 == prev || s2 == cur));
        edirty[e] = d ? 1 : 0;
        if (d) query[aggregated_add(&L->nquery, 1)] = j;
    }
}

// The pruned traversal: each dirty element walks its whole scene along the
// ropes from the scene's root and writes every overlapping leaf that is not
// itself, shares no point with it, and is clean or dirty with a larger
// element id (a pair of two dirty elements is written by the smaller one).
__global__ void k_traverse_rope_full(int n, const RopeNode* __restrict__ rn, const int* __restrict__ rope,
                                     const int* __restrict__ elem_scene, const SceneRun* __restrict__ run,
                                     const int* __restrict__ ev, int2* pairs, int cap, PassCounters* ctr,
                                     const LeafRec* __restrict__ leaves, const int* __restrict__ query,
                                     const LoopCtl* __restrict__ L, const uint8_t* __restrict__ edirty) {
    const int m = L->prune ? L->nquery : 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m; t += gridDim.x * blockDim.x) {
        const int i = query[t];
        if (i < 0 || i >= n) {
            atomicOr(&ctr->err, kErrIndexLeaf);
            continue;
        }
        const LeafRec r = leaves[i];
        const int ei = r.e;
        if (ei < 0) continue;  // flagged by k_leaf_records
        const SceneRun sr = run[elem_scene[ei]];
        if (sr.mode == kSceneIdle || sr.root < 0) continue;
        BoxOrd qo;
        Box6 q;
        for (int d = 0; d < 3; ++d) {
            qo.lo[d] = r.lo[d];
            qo.hi[d] = r.hi[d];
            q.lo[d] = unord_double(r.lo[d]);
            q.hi[d] = unord_double(r.hi[d]);
        }
        const int pi0 = r.p[0], pi1 = r.p[1], pi2 = r.p[2];
        const Box32 q32 = box32_out(q);
        int x = sr.root;
        for (int steps = 0; x != kRopeEnd; ++steps) {
            if (steps >= 2 * n) {
                atomicOr(&ctr->err, kErrIndexNode);
                break;
            }
            if (x >= 0) {
                if (x >= n - 1) {
                    atomicOr(&ctr->err, kErrIndexNode);
                    break;
                }
                const float4* p4 = reinterpret_cast<const float4*>(&rn[x]);
                const float4 a = __ldg(p4), b = __ldg(p4 + 1);  // lo xyz hi.x | hi.y hi.z left rope
                const bool hit = q32.lo[0] <= a.w && q32.hi[0] >= a.x && q32.lo[1] <= b.x && q32.hi[1] >= a.y &&
                                 q32.lo[2] <= b.y && q32.hi[2] >= a.z;
                x = __float_as_int(hit ? b.z : b.w);
                continue;
            }
            const int k = ~x;
            if (k >= n) {
                atomicOr(&ctr->err, kErrIndexLeaf);
                break;
            }
            x = k < n - 1 ? __ldg(&rope[k]) : kRopeEnd;
            if (k == i) continue;
            const ulonglong2* lr = reinterpret_cast<const ulonglong2*>(&leaves[k]);
            const ulonglong2 u0 = __ldg(lr), u1 = __ldg(lr + 1), u2 = __ldg(lr + 2);
            if (!(qo.lo[0] <= u1.y && qo.hi[0] >= u0.x && qo.lo[1] <= u2.x && qo.hi[1] >= u0.y &&
                  qo.lo[2] <= u2.y && qo.hi[2] >= u1.x))
                continue;
            const int4 pe = __ldg(reinterpret_cast<const int4*>(lr + 3));
            const int ej = pe.w;
            if (ej < 0) continue;
            if (ev && (pe.x == pi0 || pe.x == pi1 || pe.x == pi2 || pe.y == pi0 || pe.y == pi1 || pe.y == pi2 ||
                       (pe.z >= 0 && (pe.z == pi0 || pe.z == pi1 || pe.z == pi2))))
                continue;
            if (edirty[ej] && ej < ei) continue;  // written by ej's query
            emit_pair(ei, ej, pairs, cap, ctr);
        }
    }
}

// The pruned traversal with one warp per dirty element: the walk from the
// scene's root keeps its pending nodes in a shared-memory stack, and each
// round the lanes take up to 32 of them at once, test both children of each
// (the node record holds their FP32 boxes), test the overlapping leaves
// exactly and push the overlapping internal children. A walk then takes
// about as many rounds as the tree is deep, instead of one dependent load
// per visited node. Same pairs as k_traverse_rope_full.
constexpr int kPrunedWarps = 4;     // warps per block
constexpr int kWarpStack = 2048;    // pending nodes per warp

__global__ void __launch_bounds__(kPrunedWarps * 32) k_traverse_warp_full(
    int n, const BvhNode32* __restrict__ node, const int* __restrict__ elem_scene, const SceneRun* __restrict__ run,
    const int* __restrict__ ev, int2* pairs, int cap, PassCounters* ctr, const LeafRec* __restrict__ leaves,
    const int* __restrict__ query, const LoopCtl* __restrict__ L, const uint8_t* __restrict__ edirty) {
    __shared__ int s_stk[kPrunedWarps][kWarpStack];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int* stk = s_stk[w];
    const int m = L->prune ? L->nquery : 0;
    for (int t = blockIdx.x * kPrunedWarps + w; t < m; t += gridDim.x * kPrunedWarps) {
        const int i = query[t];
        if (i < 0 || i >= n) {
            if (lane == 0) atomicOr(&ctr->err, kErrIndexLeaf);
            continue;
        }
        const LeafRec r = leaves[i];
        const int ei = r.e;
        if (ei < 0) continue;  // flagged by k_leaf_records
        const SceneRun sr = run[elem_scene[ei]];
        if (sr.mode == kSceneIdle || sr.root < 0) continue;
        if (sr.root >= n - 1) {
            if (lane == 0) atomicOr(&ctr->err, kErrIndexNode);
            continue;
        }
        BoxOrd qo;
        Box6 q;
        for (int d = 0; d < 3; ++d) {
            qo.lo[d] = r.lo[d];
            qo.hi[d] = r.hi[d];
            q.lo[d] = unord_double(r.lo[d]);
            q.hi[d] = unord_double(r.hi[d]);
        }
        const int pi0 = r.p[0], pi1 = r.p[1], pi2 = r.p[2];
        const Box32 q32 = box32_out(q);
        __syncwarp();
        if (lane == 0) stk[0] = sr.root;
        __syncwarp();
        int sp = 1;  // the same in every lane
        for (int rounds = 0; sp > 0; ++rounds) {
            if (rounds >= 2 * n) {  // a valid hierarchy has fewer nodes than that
                if (lane == 0) atomicOr(&ctr->err, kErrIndexNode);
                break;
            }
            const int take = sp < 32 ? sp : 32;
            const int x = lane < take ? stk[sp - take + lane] : -1;
            __syncwarp();
            sp -= take;
            int push[2] = {-1, -1};
            if (x >= 0) {
                const float4* r4 = reinterpret_cast<const float4*>(&node[x]);
                Box32 cb[2];
                unpack(__ldg(r4), __ldg(r4 + 1), __ldg(r4 + 2), cb[0], cb[1]);
                const int4 meta = __ldg(reinterpret_cast<const int4*>(r4 + 3));
                const int cs[2] = {meta.x, meta.y};
                for (int k = 0; k < 2; ++k) {
                    if (!overlap32(q32, cb[k])) continue;
                    const int c = cs[k];
                    if (c >= 0) {
                        if (c >= n - 1) atomicOr(&ctr->err, kErrIndexNode);
                        else push[k] = c;
                        continue;
                    }
                    const int kl = ~c;
                    if (kl >= n) {
                        atomicOr(&ctr->err, kErrIndexLeaf);
                        continue;
                    }
                    if (kl == i) continue;
                    const ulonglong2* lr = reinterpret_cast<const ulonglong2*>(&leaves[kl]);
                    const ulonglong2 u0 = __ldg(lr), u1 = __ldg(lr + 1), u2 = __ldg(lr + 2);
                    if (!(qo.lo[0] <= u1.y && qo.hi[0] >= u0.x && qo.lo[1] <= u2.x && qo.hi[1] >= u0.y &&
                          qo.lo[2] <= u2.y && qo.hi[2] >= u1.x))
                        continue;
                    const int4 pe = __ldg(reinterpret_cast<const int4*>(lr + 3));
                    const int ej = pe.w;
                    if (ej < 0) continue;
                    if (ev && (pe.x == pi0 || pe.x == pi1 || pe.x == pi2 || pe.y == pi0 || pe.y == pi1 ||
                               pe.y == pi2 || (pe.z >= 0 && (pe.z == pi0 || pe.z == pi1 || pe.z == pi2))))
                        continue;
                    if (edirty[ej] && ej < ei) continue;  // written by ej's query
                    emit_pair(ei, ej, pairs, cap, ctr);
                }
            }
            // push the overlapping internal children (exclusive prefix over the lanes)
            const int cnt = (push[0] >= 0) + (push[1] >= 0);
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            if (sp + total > kWarpStack) {  // the same in every lane: the walk stops with an error
                if (lane == 0) atomicOr(&ctr->err, kErrStack);
                break;
            }
            int at = sp + incl - cnt;
            if (push[0] >= 0) stk[at++] = push[0];
            if (push[1] >= 0) stk[at] = push[1];
            sp += total;
            __syncwarp();
        }
    }
}

__global__ void k_brute_pairs(const Box6* __restrict__ box, int n, const int* __restrict__ elem_scene, int2* pairs,
                              int cap, PassCounters* ctr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Box6 q = box[i];
    int si = elem_scene ? elem_scene[i] : 0;
    for (int j = i + 1; j < n; ++j)
        if ((!elem_scene || elem_scene[j] == si) && overlap(q, box[j])) emit_pair(i, j, pairs, cap, ctr);
}

inline int nblk(int n, int t) { return (n + t - 1) / t; }

}  // namespace

// Grid of a kernel over at most n items whose count is in device memory:
// strided, a few waves at most.
inline int dev_grid(int n, int t) {
    const int b = nblk(n, t);
    return b < 152 * 8 ? b : 152 * 8;
}

void leaf_boxes(const int* ev, const int* act, int n, const int* elem_scene, const SceneDev* scenes, int nscenes,
                const double4_32a* xo, const double4_32a* av, int moving, Box6* box, unsigned long long* bbox_enc,
                cudaStream_t s, const int* dn) {
    count_launch(), k_bbox_init<<<nblk(6 * nscenes, 256), 256, 0, s>>>(bbox_enc, 6 * nscenes, dn);
    if (n <= 0) return;
    const int g = dn ? dev_grid(n, 256) : nblk(n, 256);
    if (moving)
        count_launch(), k_leaf_boxes<1><<<g, 256, 0, s>>>(ev, act, n, dn, elem_scene, scenes, xo, av, box, bbox_enc);
    else
        count_launch(), k_leaf_boxes<0><<<g, 256, 0, s>>>(ev, act, n, dn, elem_scene, scenes, xo, av, box, bbox_enc);
}

// Element / point k of the selection: scene j with off[j] <= k < off[j+1].
__global__ void k_expand(const int* __restrict__ scene_ids, const int* __restrict__ off, int nsel, int n,
                         const SceneDev* __restrict__ scenes, int points, int* out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int lo = 0, hi = nsel - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= k) lo = mid; else hi = mid - 1;
    }
    const SceneDev& sd = scenes[scene_ids[lo]];
    out[k] = (points ? sd.v0 : sd.e0) + (k - off[lo]);
}

void expand_scenes(const int* scene_ids, const int* elem_off, const int* pt_off, int nsel, int n_elems, int n_pts,
                   const SceneDev* scenes, int* elems, int* pts, cudaStream_t s) {
    if (nsel <= 0) return;
    if (n_elems > 0)
        count_launch(), k_expand<<<nblk(n_elems, 256), 256, 0, s>>>(scene_ids, elem_off, nsel, n_elems, scenes, 0,
                                                                    elems);
    if (n_pts > 0)
        count_launch(), k_expand<<<nblk(n_pts, 256), 256, 0, s>>>(scene_ids, pt_off, nsel, n_pts, scenes, 1, pts);
}

void boxes_bbox(const Box6* box, int n, unsigned long long* bbox_enc, cudaStream_t s) {
    count_launch(), k_bbox_init<<<1, 32, 0, s>>>(bbox_enc, 6);
    if (n > 0) count_launch(), k_boxes_bbox<<<nblk(n, 256), 256, 0, s>>>(box, n, bbox_enc);
}

static void launch_refit(const Box6* box, const BvhBufs& b, int n, const int* sub, int nsub, const int* dnsub, int grid,
                         RopeNode* rn, cudaStream_t s) {
    if (b.refit_up)
        count_launch(), k_refit<true><<<grid, 256, 0, s>>>(box, b.order, n, sub, nsub, dnsub, b.parent, b.flags, b.node,
                                                           rn, b.keys, b.run);
    else
        count_launch(), k_refit<false><<<grid, 256, 0, s>>>(box, b.order, n, sub, nsub, dnsub, b.parent, b.flags,
                                                            b.node, rn, nullptr, nullptr);
}

void bvh_build(const Box6* box, BvhBufs& b, cudaStream_t s) {
    int n = b.n;
    if (n <= 1) return;
    count_launch(), k_morton<<<nblk(n, 256), 256, 0, s>>>(box, b.act, n, b.elem_scene, b.bbox_enc, b.keys, b.order);
    int bits = 30;
    while (bits < 62 && (b.nscenes - 1) >> (bits - 30)) ++bits;
    radix_sort_pairs(b.keys, b.order, n, bits, b.sort_temp, s);
    const bool ropes = b.rnode && b.rope;
    count_launch(), k_karras<<<nblk(n - 1, 256), 256, 0, s>>>(b.keys, n, b.node, b.range_hi, b.range_lo, b.parent,
                                                              ropes ? b.rope : nullptr);
    if (ropes) count_launch(), k_ropes<<<nblk(n - 1, 256), 256, 0, s>>>(b.node, b.rope, n, b.rnode);
    // the scenes' roots first: the refit's walks end there
    if (b.run)
        count_launch(), k_scene_roots<<<nblk(b.nscenes, 128), 128, 0, s>>>(b.scenes, b.run, b.nscenes, n, b.parent,
                                                                          b.range_lo, b.range_hi);
    cudaMemsetAsync(b.flags, 0, sizeof(int) * (size_t)(n - 1), s);
    launch_refit(box, b, n, nullptr, 0, nullptr, nblk(n, 256), ropes ? b.rnode : nullptr, s);
}

void bvh_refit(const Box6* box, BvhBufs& b, cudaStream_t s, bool roots) {
    int n = b.n;
    if (n <= 1) return;
    if (b.run && roots)
        count_launch(), k_scene_roots<<<nblk(b.nscenes, 128), 128, 0, s>>>(b.scenes, b.run, b.nscenes, n, b.parent,
                                                                          b.range_lo, b.range_hi);
    cudaMemsetAsync(b.flags, 0, sizeof(int) * (size_t)(n - 1), s);
    const int nleaf = b.sub ? b.nsub : n;
    if (nleaf > 0)
        launch_refit(box, b, n, b.sub, b.nsub, b.sub ? b.dnsub : nullptr,
                     b.sub && b.dnsub ? dev_grid(nleaf, 256) : nblk(nleaf, 256), b.rnode && b.rope ? b.rnode : nullptr,
                     s);
}

template <int DEPTH>
void launch_stack_traverse(const Box6* box, const BvhBufs& b, int nq, int block, int2* pairs, int cap,
                           PassCounters* ctr, cudaStream_t s, const int* skip_shared_ev, const Box6* box_static) {
    const int* dq = b.sub ? (b.dnq ? b.dnq : b.dnsub) : nullptr;
    const int g = dq ? dev_grid(nq, block) : nblk(nq, block);
    count_launch(), k_traverse<DEPTH><<<g, block, 0, s>>>(box, b.order, b.n, b.node, b.elem_scene, b.run,
                                                        skip_shared_ev, pairs, cap, ctr, box_static, b.leaf, b.sub,
                                                        b.nsub, dq);
}

// Resident blocks of the dynamic-fetch traversal per SM, looked up once.
int dyn_blocks_per_sm() {
    static int cached = 0;
    if (!cached) {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_traverse_rope_dyn, 128, 0) != cudaSuccess || nb < 1)
            nb = 8;
        cached = nb;
    }
    return cached;
}

void bvh_pairs(const Box6* box, const BvhBufs& b, int2* pairs, int cap, PassCounters* ctr, cudaStream_t s,
               const int* skip_shared_ev, int block, const Box6* box_static, bool packet, bool rope, int refill,
               int stack_depth) {
    int n = b.n;
    if (n <= 1) return;
    const int nleaf = b.sub ? b.nsub : n, nq = b.sub ? b.nsub : n - 1;
    if (nq <= 0) return;
    const bool dyn = b.leaf && rope && b.rnode && b.rope && b.leaf32 && b.qnext && refill > 0;
    const int* dnsub = b.sub ? b.dnsub : nullptr;
    const int* dq = b.sub ? (b.dnq ? b.dnq : b.dnsub) : nullptr;  // queries of the traversal
    if (b.leaf)
        count_launch(), k_leaf_records<<<dnsub ? dev_grid(nleaf, 256) : nblk(nleaf, 256), 256, 0, s>>>(
            box, b.order, n, b.sub, b.nsub, dnsub, b.ev, b.leaf, b.ne_all, ctr, b.rope, dyn ? b.leaf32 : nullptr);
    if (dyn) {
        static int num_sms = 0;
        if (!num_sms) {
            int dev = 0;
            cudaGetDevice(&dev);
            if (cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) num_sms = 152;
        }
        int blocks = num_sms * dyn_blocks_per_sm();
        const int need = nblk(nq, 128);
        if (blocks > need) blocks = need;
        cudaMemsetAsync(b.qnext, 0, sizeof(int), s);
        count_launch(), k_traverse_rope_dyn<<<blocks, 128, 0, s>>>(n, b.rnode, b.elem_scene, b.run, skip_shared_ev,
                                                                   pairs, cap, ctr, box_static, b.leaf, b.leaf32,
                                                                   b.sub, b.nsub, dq, b.qnext,
                                                                   refill > 32 ? 32 : refill);
    } else if (b.leaf && rope && b.rnode && b.rope) {
        count_launch(), k_traverse_rope<<<dq ? dev_grid(nq, block) : nblk(nq, block), block, 0, s>>>(
            n, b.rnode, b.rope, b.elem_scene, b.run, skip_shared_ev, pairs, cap, ctr, box_static, b.leaf, b.sub,
            b.nsub, dq);
    } else if (b.leaf && packet && !b.sub) {
        count_launch(), k_traverse_packet<<<nblk(n - 1, kPacketWarps * 32), kPacketWarps * 32, 0, s>>>(
            b.order, n, b.node, b.elem_scene, b.run, skip_shared_ev, pairs, cap, ctr, box_static, b.leaf);
    } else if (stack_depth <= 24) {
        launch_stack_traverse<24>(box, b, nq, block, pairs, cap, ctr, s, skip_shared_ev, box_static);
    } else if (stack_depth <= 32) {
        launch_stack_traverse<32>(box, b, nq, block, pairs, cap, ctr, s, skip_shared_ev, box_static);
    } else if (stack_depth <= 48) {
        launch_stack_traverse<48>(box, b, nq, block, pairs, cap, ctr, s, skip_shared_ev, box_static);
    } else {
        launch_stack_traverse<64>(box, b, nq, block, pairs, cap, ctr, s, skip_shared_ev, box_static);
    }
}

void pruned_pairs(const BvhBufs& b, const int* act_e, const int* act_l, const unsigned* stamp, LoopCtl* L,
                  uint8_t* edirty, int* query, int ne_cap, int2* pairs, int cap, PassCounters* ctr, const int* ev,
                  cudaStream_t s, bool warp) {
    if (ne_cap <= 1 || b.n <= 1) return;
    count_launch(), k_dirty_queries<<<dev_grid(ne_cap, 256), 256, 0, s>>>(act_l, b.order, b.n, b.ne_all, ev, stamp, L,
                                                                          edirty, query, ctr);
    if (warp && b.node)
        count_launch(), k_traverse_warp_full<<<dev_grid(ne_cap, kPrunedWarps), kPrunedWarps * 32, 0, s>>>(
            b.n, b.node, b.elem_scene, b.run, ev, pairs, cap, ctr, b.leaf, query, L, edirty);
    else
        count_launch(), k_traverse_rope_full<<<dev_grid(ne_cap, 128), 128, 0, s>>>(
            b.n, b.rnode, b.rope, b.elem_scene, b.run, ev, pairs, cap, ctr, b.leaf, query, L, edirty);
}

void brute_pairs(const Box6* box, int ne, const int* elem_scene, int2* pairs, int cap, PassCounters* ctr,
                 cudaStream_t s) {
    if (ne <= 1) return;
    count_launch(), k_brute_pairs<<<nblk(ne, 128), 128, 0, s>>>(box, ne, elem_scene, pairs, cap, ctr);
}

}  // namespace ccg
