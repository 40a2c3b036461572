// Host emulation of the reference tree's insertion order; see cc_tree_order.h.
#include "cc_tree_order.h"

namespace ccg {

double box_volume(const double* lo, const double* hi) {
    return (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
}

namespace {
inline double mn(double a, double b) { return (b < a) ? b : a; }
inline double mx(double a, double b) { return (a < b) ? b : a; }
}  // namespace

double RefTreeOrder::build(const Box6* leaf_boxes, int n) {
    n_ = n;
    nodes_.resize(n > 0 ? 2 * (size_t)n - 1 : 0);
    path_.resize(n > 0 ? (size_t)n : 0);
    for (int e = 0; e < n; ++e) {
        Node& L = nodes_[e];
        for (int d = 0; d < 3; ++d) {
            L.lo[d] = leaf_boxes[e].lo[d];
            L.hi[d] = leaf_boxes[e].hi[d];
        }
        L.left = L.right = -1;
        L.vol = box_volume(L.lo, L.hi);
    }
    int next = n;
    root_ = n > 0 ? 0 : -1;
    for (int e = 1; e < n; ++e) {
        const Node& nb = nodes_[e];
        int depth = 0;
        int p = root_;
        int* slot = &root_;
        while (nodes_[p].left >= 0) {
            const Node& l = nodes_[nodes_[p].left];
            const Node& r = nodes_[nodes_[p].right];
            // the next level's nodes, whichever way this one goes
            if (l.left >= 0) {
                __builtin_prefetch(&nodes_[l.left]);
                __builtin_prefetch(&nodes_[l.right]);
            }
            if (r.left >= 0) {
                __builtin_prefetch(&nodes_[r.left]);
                __builtin_prefetch(&nodes_[r.right]);
            }
            double ml[3], Ml[3], mr[3], Mr[3];
            for (int d = 0; d < 3; ++d) {
                ml[d] = mn(l.lo[d], nb.lo[d]);
                Ml[d] = mx(l.hi[d], nb.hi[d]);
                mr[d] = mn(r.lo[d], nb.lo[d]);
                Mr[d] = mx(r.hi[d], nb.hi[d]);
            }
            double vdiff1 = box_volume(ml, Ml) - l.vol;
            double vdiff2 = box_volume(mr, Mr) - r.vol;
            path_[depth++] = p;
            if (vdiff1 < vdiff2) {
                slot = &nodes_[p].left;
                p = nodes_[p].left;
            } else {
                slot = &nodes_[p].right;
                p = nodes_[p].right;
            }
        }
        int q = next++;
        Node& np = nodes_[q];
        np.left = e;
        np.right = p;
        for (int d = 0; d < 3; ++d) {
            np.lo[d] = mn(nodes_[e].lo[d], nodes_[p].lo[d]);
            np.hi[d] = mx(nodes_[e].hi[d], nodes_[p].hi[d]);
        }
        np.vol = box_volume(np.lo, np.hi);
        *slot = q;
        while (depth > 0) {
            Node& a = nodes_[path_[--depth]];
            const Node& l = nodes_[a.left];
            const Node& r = nodes_[a.right];
            for (int d = 0; d < 3; ++d) {
                a.lo[d] = mn(l.lo[d], r.lo[d]);
                a.hi[d] = mx(l.hi[d], r.hi[d]);
            }
            a.vol = box_volume(a.lo, a.hi);
        }
    }
    built_ = n > 0;
    return n > 0 ? box_volume(nodes_[root_].lo, nodes_[root_].hi) : 0.0;
}

void RefTreeOrder::ranks(int* out) const {
    if (!built_) return;
    std::vector<int> st;
    st.reserve(64);
    int r = 0, cur = root_;
    while (cur >= 0 || !st.empty()) {
        while (cur >= 0) {
            st.push_back(cur);
            cur = nodes_[cur].left;
        }
        cur = st.back();
        st.pop_back();
        if (nodes_[cur].left < 0) out[cur] = r++;
        cur = nodes_[cur].right;
    }
}

}  // namespace ccg
