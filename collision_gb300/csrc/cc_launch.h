// Host-side launch wrappers for the collision kernels. Every wrapper
// enqueues on the given stream and returns without synchronising.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cc_common.cuh"

namespace ccg {

// Kernels launched by this library since load (read by cc_get_counters).
extern long long g_kernel_launches;
inline void count_launch(int n = 1) { g_kernel_launches += n; }

// ------------------------------------------------------------- primitives
// Scratch bytes needed to sort n (key, value) pairs.
size_t radix_sort_temp_bytes(int n);
// Stable LSD radix sort of (keys, vals) on the low `bits` bits of the keys.
// keys/vals are sorted in place (the temp buffer holds the ping-pong copy).
void radix_sort_pairs(unsigned long long* keys, unsigned int* vals, int n, int bits, void* temp,
                      cudaStream_t s);
// Exclusive scan of n ints (out may alias in); total written to *total.
size_t scan_temp_bytes(int n);
void exclusive_scan(const int* in, int* out, int n, int* total, void* temp, cudaStream_t s);

// ------------------------------------------------------------- broad phase
struct __align__(16) Box6 {
    double lo[3];
    double hi[3];
};

struct BvhBufs {
    int n;                        // leaves
    unsigned long long* keys;     // n Morton keys (sorted)
    unsigned int* order;          // n element ids in Morton order
    int* child;                   // 2*(n-1): >= 0 internal, < 0 leaf (~sorted index)
    int* range_hi;                // n-1: last sorted leaf covered by each internal node
    int* parent;                  // 2n-1: parents of internal nodes [0,n-1) then leaves
    int* flags;                   // n-1 refit arrival counters
    Box6* node_box;               // n-1 internal boxes
    unsigned long long* bbox_enc; // 6 encoded doubles (scene box)
    void* sort_temp;
};

// Leaf boxes of every element (static: x_old; moving: x_old and
// x_old + dt*avgVel), padded by 1e-6, plus their union in bbox_enc.
void leaf_boxes(const int* ev, int ne, int nt, const double4_32a* xo, const double4_32a* av, double dt, int moving,
                Box6* box, unsigned long long* bbox_enc, cudaStream_t s);
// Union of n given boxes in bbox_enc (the scene box the Morton keys use).
void boxes_bbox(const Box6* box, int n, unsigned long long* bbox_enc, cudaStream_t s);
// Morton keys, sort, Karras hierarchy, refit.
void bvh_build(const Box6* box, BvhBufs& b, cudaStream_t s);
// All leaf pairs with overlapping boxes, each unordered pair once.
void bvh_pairs(const Box6* box, const BvhBufs& b, int2* pairs, int cap, PassCounters* ctr, cudaStream_t s);
// The same pair set by testing every pair (for cross-checks on small meshes).
void brute_pairs(const Box6* box, int ne, int2* pairs, int cap, PassCounters* ctr, cudaStream_t s);

// ------------------------------------------------------------ narrow phase
struct NarrowArgs {
    const double4_32a* xo;
    const double4_32a* av;
    const uint8_t* fixed;
    const int* ev;
    const int* esurf;
    const uint8_t* erigid;
    const int* rank;
    int nt;
    int pass;
    int zone;
    Params p;
    const int2* pairs;
    Contrib* contrib;
    int contrib_cap;
    PassCounters* ctr;
    int* uf_parent;
    VisitRec* rec;
    int rec_cap;
    const float4* pbox_lo;  // null: plain FP64 (no filter)
    const float4* pbox_hi;
    float hpad, epad;
};
void narrow_pass(const NarrowArgs& a, int moving, int max_pairs, cudaStream_t s);
// Outward-rounded FP32 point boxes for the mixed-precision filter.
void point_boxes(const double4_32a* xo, const double4_32a* av, double dt, int nv, int moving, float4* lo,
                 float4* hi, cudaStream_t s);

// ------------------------------------------------------------- post-pass
struct ApplyBufs {
    int* cnt;      // nv
    int* off;      // nv
    int* cur;      // nv
    int* idx;      // contrib_cap
    void* scan_temp;
};
// Per-point sums of the pass's contributions in visiting order, then
// avgVel += (impulse + friction) / n and has_collsn (updateAverageVelocity).
void apply_contribs(const Contrib* contrib, const PassCounters* ctr, int contrib_cap, int nv, double4_32a* av,
                    uint8_t* has_collsn, ApplyBufs& b, cudaStream_t s);

struct ZoneBufs {
    int* root;                  // nv
    int* zcnt;                  // nv
    unsigned long long* keys;   // nv
    unsigned int* vals;         // nv
    int* nmembers;              // 1
    void* sort_temp;
};
void uf_init(int* parent, int nv, cudaStream_t s);
// updateImpactZoneVelocity: rigid motion of every zone with >= 2 points.
void zone_velocity(int* parent, const uint8_t* in_elem, const uint8_t* fixed, const double4_32a* xo, double4_32a* av,
                   int nv, const Params& p, ZoneBufs& z, PassCounters* ctr, cudaStream_t s);

// Step set-up: pack inputs, average velocity (computeAverageVelocity).
void step_init(const double* x_old, const double* x_cand, int nv, const uint8_t* in_elem, double dt, double4_32a* xo,
               double4_32a* av, PassCounters* ctr, cudaStream_t s);
// Domain clamp + final position (detectDomainBoundaryCollision, updateFinalPosition).
void finalize_positions(const uint8_t* in_elem, const double4_32a* xo, double4_32a* av, uint8_t* has_collsn,
                        const double* x_cand, double* x_out, int nv, const Params& p, const double* lo,
                        const double* hi, cudaStream_t s);
// reduceSuperelast: up to 10 Gauss-Seidel passes over the strain edges.
struct StrainEdge {
    int p0, p1;
    double len0;
    int s0, s1;  // shared-memory slots of p0, p1 in the window sweep
};
// Shared-memory window schedule of the strain sweep (see k_strain_window):
// per level l, load_list[load_off[l] .. load_off[l+1]) are (point, slot)
// pairs to copy in and wb_list[wb_off[l] .. wb_off[l+1]) pairs to write back
// (wb level nlevels: after the last level).
struct StrainWindow {
    int nslots;
    const int2* load_list;
    const int* load_off;
    const int2* wb_list;
    const int* wb_off;
    const int4* hdr;  // per level: (edge begin, end, load begin, end), (write-back begin, end, 0, 0)
    int2 wb_final;    // write-backs after the last level
};
// edges sorted by dependency level; level_off has nlevels+1 offsets;
// step_buf holds strain_step_bytes(nedges).
size_t strain_step_bytes(int nedges);
void strain_limit(const StrainEdge* edges, int nedges, const int* level_off, int nlevels, const double4_32a* xo,
                  double4_32a* av, int nv, double dt, void* step_buf, const StrainWindow* win, int* passes_out,
                  cudaStream_t s);
// Correctly rounded cos/sin/acos/pow (fn 0..3) on device arrays, for self-tests.
void math_selftest(int fn, const double* a, const double* b, double* out, int n, cudaStream_t s);
// updateFinalVelocity.
void final_velocity(const uint8_t* in_elem, const uint8_t* has_collsn, const double4_32a* av, double* vel, int nv,
                    cudaStream_t s);

}  // namespace ccg
