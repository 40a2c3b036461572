// Leaf order of the reference's incremental AABB tree.
//
// The reference (AABB.cpp:129-343) visits each overlapping element pair once,
// as (a, b) with b the leaf queried first in its tree's inorder. Which element
// of a pair is `a` is observable: edge-edge friction is applied with the same
// sign to both edges (dcollid3d.cpp:1242-1282), impact zones merge by sub-test
// order (dcollid3d.cpp:300-321), and per-point impulses are summed in visiting
// order. The inorder position of each leaf (its rank) therefore has to match
// the reference's tree, which is built by inserting leaves one at a time into
// the child whose box grows least (AABB.cpp:163-197) - a sequential process
// with no parallel formulation. It runs on the host only when a tree is built
// (first detection pass of each kind) or rebuilt (root volume grown by more
// than 20%, dcollid.cpp:381, 422); refits keep the structure and the ranks.
#pragma once

#include <vector>

#include "cc_launch.h"

namespace ccg {

class RefTreeOrder {
public:
    // Insert leaves 0..n-1 in order with the given boxes; returns the root
    // box volume (AABB::volume of the root, AABB.cpp:51-54).
    double build(const Box6* leaf_boxes, int n);
    // Inorder rank of every leaf.
    void ranks(int* out) const;
    bool built() const { return built_; }

private:
    struct Node {
        double lo[3], hi[3];
        double vol;  // AABB::volume of the box, kept with it
        int left, right;
    };
    std::vector<Node> nodes_;
    std::vector<int> path_;
    int root_ = -1;
    int n_ = 0;
    bool built_ = false;
};

double box_volume(const double* lo, const double* hi);

}  // namespace ccg
