// Strain-limiting schedule of one scene: dependency levels of its edges and
// the shared-memory slots of its points (host side of the window sweep).
#pragma once

#include <vector>

#include "cc_launch.h"

namespace ccg {

// Copy-ins run this many levels before a point's first edge (kWindowAhead of
// the window sweep in cc_post.cu).
constexpr int kStrainAhead = 8;

// Appends one scene's strain schedule to the batch arrays. `edges` are the
// scene's strain edges in the reference's order (elements in order, a
// triangle's three sides p0p1, p1p2, p2p0), with batch point ids; points
// are [v0, v0 + nv).
//
// Level of an edge = 1 + the level of the last earlier edge at either of
// its points: edges of one level share no point, so sweeping level by level
// is the reference's sequential sweep (dcollid.cpp:586-596) reordered only
// where the order cannot matter. For the shared-memory sweep each point gets
// a slot for its live interval - from kAhead levels before its first edge to
// the level after its last one - by interval colouring.
void append_strain_schedule(const std::vector<StrainEdge>& edges, int v0, int nv, std::vector<StrainEdge>& all_edges,
                            std::vector<int4>& hdr, std::vector<int2>& load, std::vector<int2>& wb, SceneDev& sd,
                            int caps[3]);

}  // namespace ccg
