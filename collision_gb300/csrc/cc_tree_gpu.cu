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
// union with the new leaf's box), which gives the same doubles as the
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

struct __align__(16) TreeNode {
    double lo[3], hi[3];
    double vol;  // AABB::volume of the box (AABB.cpp:51-54), kept with it
    int left, right;
};

__device__ __forceinline__ double mn(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double mx(double a, double b) { return (a < b) ? b : a; }

// (hi - lo) products in the reference's order, never contracted
__device__ __forceinline__ double volume3(const double* lo, const double* hi) {
    return __dmul_rn(__dmul_rn(__dsub_rn(hi[0], lo[0]), __dsub_rn(hi[1], lo[1])), __dsub_rn(hi[2], lo[2]));
}

__device__ __forceinline__ void load_node(const TreeNode* t, double* lo, double* hi, double& vol) {
    const double2* p = reinterpret_cast<const double2*>(t);
    const double2 a = p[0], b = p[1], c = p[2], d = p[3];
    lo[0] = a.x; lo[1] = a.y; lo[2] = b.x;
    hi[0] = b.y; hi[1] = c.x; hi[2] = c.y;
    vol = d.x;
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
            L.lo[d] = b.lo[d];
            L.hi[d] = b.hi[d];
        }
        L.vol = volume3(b.lo, b.hi);
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
            q.lo[d] = mn(nd[1].lo[d], nd[0].lo[d]);
            q.hi[d] = mx(nd[1].hi[d], nd[0].hi[d]);
        }
        q.vol = volume3(q.lo, q.hi);
        q.left = 1;
        q.right = 0;
        parent[n] = -1;
        parent[0] = parent[1] = n;
        count[n] = 2;
    }
    __syncthreads();

    int my_e = -1, p = -1;
    double nlo[3], nhi[3];
    int next = 2;  // the next insertion to start; the same in every thread
    for (;;) {
        const bool start = next < n && my_e < 0 && next % T == tid;
        if (start) {
            my_e = next;
            p = root;
            double v;
            load_node(&nd[my_e], nlo, nhi, v);
            TreeNode& R = nd[root];
            for (int d = 0; d < 3; ++d) {
                R.lo[d] = mn(R.lo[d], nlo[d]);
                R.hi[d] = mx(R.hi[d], nhi[d]);
            }
            R.vol = volume3(R.lo, R.hi);
            ++count[root];
        }
        if (my_e >= 0) {
            // one level: p is an internal node on the path, its box already widened
            const int l = nd[p].left, r = nd[p].right;
            double llo[3], lhi[3], lv, rlo[3], rhi[3], rv;
            load_node(&nd[l], llo, lhi, lv);
            load_node(&nd[r], rlo, rhi, rv);
            // volume growth of each child's box by the new leaf's (AABB::merge, AABB.cpp:38-49)
            double gl = 1.0, gr = 1.0;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                gl = __dmul_rn(gl, __dsub_rn(mx(lhi[d], nhi[d]), mn(llo[d], nlo[d])));
                gr = __dmul_rn(gr, __dsub_rn(mx(rhi[d], nhi[d]), mn(rlo[d], nlo[d])));
            }
            const bool go_left = __dsub_rn(gl, lv) < __dsub_rn(gr, rv);
            const int c = go_left ? l : r;
            double clo[3], chi[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                clo[d] = go_left ? llo[d] : rlo[d];
                chi[d] = go_left ? lhi[d] : rhi[d];
            }
            if (c >= n) {
                TreeNode& C = nd[c];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    C.lo[d] = mn(clo[d], nlo[d]);
                    C.hi[d] = mx(chi[d], nhi[d]);
                }
                C.vol = go_left ? gl : gr;
                ++count[c];
                p = c;
            } else {
                const int q = n + my_e - 1;
                TreeNode& Q = nd[q];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    Q.lo[d] = mn(nlo[d], clo[d]);
                    Q.hi[d] = mx(nhi[d], chi[d]);
                }
                Q.vol = volume3(Q.lo, Q.hi);
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
        vol_out[blockIdx.x] = nd[root].vol;
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
