// The reference tree's leaf order, built on the GPU.
//
// The reference builds each AABB tree by inserting leaves 0..n-1 one at a
// time, descending from the root into the child whose box grows least
// (ties go right) and splitting the leaf it reaches into a branch (new leaf
// left, old leaf right); every box on the path is then the union of its
// children's (AABB.cpp:129-197). Only the inorder rank of every leaf and the
// root volume are needed (cc_tree_order.h says why).
//
// The insertions are sequential in the reference, but their descents can
// overlap: insertion e reads, at depth d, only boxes at depth d+1 and the
// child pointers at depth d, and every earlier insertion writes those while
// it is at depth d. So one CTA runs up to blockDim.x insertions as a
// pipeline, every active insertion one level per step with a block barrier
// between steps, and at most one insertion starting per step. Insertion e
// then reaches every depth at least one step after insertion e-1 and sees
// exactly the tree the reference's insertion e sees; in one step no two
// insertions touch the same depth. Boxes are widened on the way down (the
// union with the new leaf's box), which gives the same box as the
// reference's bottom-up union of the children: min and max are exact.
//
// Leaves are nodes 0..n-1 and insertion e (e >= 1) creates node n+e-1, so
// whether a node is a leaf needs no load. Each insertion also keeps parent
// links and leaf counts, from which k_tree_ranks gives each leaf its inorder
// rank by walking to the root.
#include "cc_launch.h"

namespace ccg {

namespace {

constexpr int kTreeThreads = 1024;

// Box coordinates are kept as order-preserving integer keys: key(a) <
// key(b) exactly when a < b for doubles that are not NaN, except that -0
// orders below +0. So min and max run on the integer pipe (GB300's FP64
// rate is a small fraction of its integer rate), and containment is six
// integer compares. Where the reference's std::min/std::max would keep +0
// and the key order keeps -0, the difference is only the sign of a zero
// coordinate, which changes no box extent, volume comparison or decision.
struct __align__(16) TreeNode {
    long long lo[3], hi[3];  // keys
    double vol;              // AABB::volume of the box (AABB.cpp:51-54), kept with it
    int left, right;
};

__device__ __forceinline__ long long okey(double d) {
    const long long b = __double_as_longlong(d);
    return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
__device__ __forceinline__ double odec(long long k) {
    return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffll));
}
__device__ __forceinline__ long long kmin(long long a, long long b) { return b < a ? b : a; }
__device__ __forceinline__ long long kmax(long long a, long long b) { return a < b ? b : a; }

// (hi - lo) products in the reference's order, never contracted
__device__ __forceinline__ double volume_k(const long long* lo, const long long* hi) {
    return __dmul_rn(__dmul_rn(__dsub_rn(odec(hi[0]), odec(lo[0])), __dsub_rn(odec(hi[1]), odec(lo[1]))),
                     __dsub_rn(odec(hi[2]), odec(lo[2])));
}
// the volume of the union of two boxes
__device__ __forceinline__ double volume_union(const long long* alo, const long long* ahi, const long long* blo,
                                               const long long* bhi) {
    long long lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        lo[d] = kmin(alo[d], blo[d]);
        hi[d] = kmax(ahi[d], bhi[d]);
    }
    return volume_k(lo, hi);
}
__device__ __forceinline__ bool contains(const long long* olo, const long long* ohi, const long long* ilo,
                                         const long long* ihi) {
    return olo[0] <= ilo[0] && olo[1] <= ilo[1] && olo[2] <= ilo[2] && ihi[0] <= ohi[0] && ihi[1] <= ohi[1] &&
           ihi[2] <= ohi[2];
}

__device__ __forceinline__ void load_node(const TreeNode* t, long long* lo, long long* hi, double& vol) {
    const longlong2* p = reinterpret_cast<const longlong2*>(t);
    const longlong2 a = p[0], b = p[1], c = p[2];
    lo[0] = a.x; lo[1] = a.y; lo[2] = b.x;
    hi[0] = b.y; hi[1] = c.x; hi[2] = c.y;
    vol = reinterpret_cast<const double*>(t)[6];
}

__global__ void __launch_bounds__(kTreeThreads) k_tree_build(const Box6* __restrict__ boxes, const int* __restrict__ jobs,
                                                            TreeNode* nodes_all, int* parent_all, int* count_all,
                                                            int* root_out, double* vol_out) {
    const int e0 = jobs[3 * blockIdx.x + 1], n = jobs[3 * blockIdx.x + 2];
    TreeNode* nd = nodes_all + 2 * (size_t)e0;
    int* parent = parent_all + 2 * (size_t)e0;
    int* count = count_all + 2 * (size_t)e0;
    const int tid = threadIdx.x, T = blockDim.x;
    for (int e = tid; e < n; e += T) {
        const Box6 b = boxes[e0 + e];
        TreeNode& L = nd[e];
        for (int d = 0; d < 3; ++d) {
            L.lo[d] = okey(b.lo[d]);
            L.hi[d] = okey(b.hi[d]);
        }
        L.vol = __dmul_rn(__dmul_rn(__dsub_rn(b.hi[0], b.lo[0]), __dsub_rn(b.hi[1], b.lo[1])),
                          __dsub_rn(b.hi[2], b.lo[2]));
        L.left = L.right = -1;
        parent[e] = -1;
        count[e] = 1;
    }
    __syncthreads();
    if (n < 2) {
        if (tid == 0) {
            root_out[blockIdx.x] = n - 1;
            vol_out[blockIdx.x] = n == 1 ? nd[0].vol : 0.0;
        }
        return;
    }
    const int root = n;  // insertion 1 splits the root leaf 0 into node n
    if (tid == 0) {
        TreeNode& q = nd[n];
        for (int d = 0; d < 3; ++d) {
            q.lo[d] = kmin(nd[1].lo[d], nd[0].lo[d]);
            q.hi[d] = kmax(nd[1].hi[d], nd[0].hi[d]);
        }
        q.vol = volume_k(q.lo, q.hi);
        q.left = 1;
        q.right = 0;
        parent[n] = -1;
        parent[0] = parent[1] = n;
        count[n] = 2;
    }
    __syncthreads();

    int my_e = -1, p = -1;
    long long nlo[3], nhi[3];
    int next = 2;  // the next insertion to start; the same in every thread
    for (;;) {
        const bool start = next < n && my_e < 0 && next % T == tid;
        if (start) {
            // the root's box is widened here; its volume is formed at the end
            my_e = next;
            p = root;
            double v;
            load_node(&nd[my_e], nlo, nhi, v);
            TreeNode& R = nd[root];
            for (int d = 0; d < 3; ++d) {
                R.lo[d] = kmin(R.lo[d], nlo[d]);
                R.hi[d] = kmax(R.hi[d], nhi[d]);
            }
            ++count[root];
        }
        if (my_e >= 0) {
            // one level: p is an internal node on the path, its box already widened
            const int l = nd[p].left, r = nd[p].right;
            long long llo[3], lhi[3], rlo[3], rhi[3];
            double lv, rv;
            load_node(&nd[l], llo, lhi, lv);
            load_node(&nd[r], rlo, rhi, rv);
            // the volume growth of each child's box by the new leaf's
            // (AABB::merge, AABB.cpp:38-49); a box that holds the new leaf's
            // does not grow (the same doubles), and a growth is never below 0
            bool go_left, grows;
            double gc;  // the chosen child's new volume
            if (contains(rlo, rhi, nlo, nhi)) {
                go_left = false;  // vdiff2 = 0 <= vdiff1
                grows = false;
                gc = rv;
            } else {
                const double gr = volume_union(rlo, rhi, nlo, nhi);
                if (contains(llo, lhi, nlo, nhi)) {
                    go_left = 0.0 < __dsub_rn(gr, rv);  // vdiff1 = 0
                    grows = !go_left;
                    gc = go_left ? lv : gr;
                } else {
                    const double gl = volume_union(llo, lhi, nlo, nhi);
                    go_left = __dsub_rn(gl, lv) < __dsub_rn(gr, rv);
                    grows = true;
                    gc = go_left ? gl : gr;
                }
            }
            const int c = go_left ? l : r;
            long long clo[3], chi[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                clo[d] = go_left ? llo[d] : rlo[d];
                chi[d] = go_left ? lhi[d] : rhi[d];
            }
            if (c >= n) {
                if (grows) {
                    TreeNode& C = nd[c];
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        C.lo[d] = kmin(clo[d], nlo[d]);
                        C.hi[d] = kmax(chi[d], nhi[d]);
                    }
                    C.vol = gc;
                }
                ++count[c];
                p = c;
            } else {
                const int q = n + my_e - 1;
                TreeNode& Q = nd[q];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    Q.lo[d] = kmin(nlo[d], clo[d]);
                    Q.hi[d] = kmax(nhi[d], chi[d]);
                }
                Q.vol = gc;  // the union of the leaf's box and the new one's
                Q.left = my_e;
                Q.right = c;
                parent[q] = p;
                parent[my_e] = q;
                parent[c] = q;
                count[q] = 2;
                if (go_left) nd[p].left = q;
                else nd[p].right = q;
                my_e = -1;
            }
        }
        next += __syncthreads_or(start) ? 1 : 0;
        if (next >= n && !__syncthreads_or(my_e >= 0)) break;
    }
    if (tid == 0) {
        root_out[blockIdx.x] = root;
        vol_out[blockIdx.x] = volume_k(nd[root].lo, nd[root].hi);
    }
}

// Inorder rank of each leaf: the leaves of every left sibling on its path.
__global__ void k_tree_ranks(const int* __restrict__ jobs, const TreeNode* __restrict__ nodes_all,
                             const int* __restrict__ parent_all, const int* __restrict__ count_all, int* rank) {
    const int e0 = jobs[3 * blockIdx.y + 1], n = jobs[3 * blockIdx.y + 2];
    const TreeNode* nd = nodes_all + 2 * (size_t)e0;
    const int* parent = parent_all + 2 * (size_t)e0;
    const int* count = count_all + 2 * (size_t)e0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        int r = 0, x = e;
        for (int a = parent[x]; a >= 0; x = a, a = parent[a]) {
            const int lft = nd[a].left;
            if (lft != x) r += count[lft];
        }
        rank[e0 + e] = r;
    }
}

}  // namespace

size_t tree_scratch_bytes(long long ne) {
    return (size_t)(2 * ne + 1) * (sizeof(TreeNode) + 2 * sizeof(int));
}

void tree_order_gpu(const Box6* boxes, const int* jobs, int njobs, int max_ne, void* scratch, long long ne_total,
                    int* rank, int* root_out, double* vol_out, cudaStream_t s) {
    if (njobs <= 0) return;
    TreeNode* nodes = static_cast<TreeNode*>(scratch);
    int* parent = reinterpret_cast<int*>(nodes + 2 * ne_total + 1);
    int* count = parent + 2 * ne_total + 1;
    k_tree_build<<<njobs, kTreeThreads, 0, s>>>(boxes, jobs, nodes, parent, count, root_out, vol_out);
    const int bx = std::max(1, std::min((max_ne + 255) / 256, 1024));
    k_tree_ranks<<<dim3(bx, njobs), 256, 0, s>>>(jobs, nodes, parent, count, rank);
}

}  // namespace ccg
