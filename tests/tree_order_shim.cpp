// Test shim: the host emulation of the reference tree's insertion order
// (collision_gb300/csrc/cc_tree_order.cpp) behind one C function, so that the
// CPU tests can compare its leaf ranks with the oracle's without a GPU.
#include "cc_tree_order.h"

extern "C" double tree_ranks(const double* boxes, int n, int* ranks) {
    ccg::RefTreeOrder t;
    const double vol = t.build(reinterpret_cast<const ccg::Box6*>(boxes), n);
    t.ranks(ranks);
    return vol;
}
