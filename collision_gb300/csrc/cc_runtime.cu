// Host runtime of the collision library: the solver object, the pass loop of
// resolveCollision (dcollid.cpp:317-362) and the C ABI of
// include/collision_gb300.h.
#include <cstdio>
#include <algorithm>
#include <queue>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/collision_gb300.h"
#include "cc_launch.h"
#include "cc_tree_order.h"

using namespace ccg;

namespace {

// Stages timed by cc_set_profiling / cc_get_profile.
enum Stage { kStInit, kStBoxes, kStBvh, kStTraverse, kStNarrowProx, kStNarrowCcd, kStApply, kStZone,
             kStFinalize, kStStrain, kNumStages };
const char* kStageNames[kNumStages] = {"init", "leaf_boxes", "bvh_build", "traverse", "narrow_prox",
                                       "narrow_ccd", "apply", "zone", "finalize", "strain"};

template <class T>
cudaError_t dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    return cudaMalloc((void**)p, n * sizeof(T));
}

template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

__global__ void k_reset_counters(PassCounters* c) {
    int keep = c->err & kErrNan;
    c->npairs = 0; c->ncontrib = 0; c->nhit_pairs = 0; c->nrec = 0;
    c->nvisits = 0; c->ncontacts = 0; c->nsub = 0; c->err = keep;
}

unsigned long long enc_host(double x) {
    unsigned long long u;
    std::memcpy(&u, &x, 8);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
double dec_host(unsigned long long e) {
    unsigned long long u = (e & 0x8000000000000000ull) ? (e & 0x7fffffffffffffffull) : ~e;
    double x;
    std::memcpy(&x, &u, 8);
    return x;
}

}  // namespace

struct cc_solver {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    // topology
    int nv = 0, nt = 0, nb = 0, ne = 0;
    int* d_ev = nullptr;
    int* d_esurf = nullptr;
    uint8_t* d_erigid = nullptr;
    uint8_t* d_fixed = nullptr;
    uint8_t* d_in_elem = nullptr;
    StrainEdge* d_edges = nullptr;
    int nedges = 0;

    // state
    double4_32a* d_xo = nullptr;
    double4_32a* d_av = nullptr;
    int* d_uf = nullptr;
    // staging for host-buffer calls
    double* d_xold_in = nullptr;
    double* d_xcand_in = nullptr;
    double* d_vel = nullptr;
    double* d_xout = nullptr;
    uint8_t* d_hc = nullptr;

    // pass buffers
    Box6* d_box = nullptr;
    BvhBufs bvh{};
    int2* d_pairs = nullptr;
    int pair_cap = 0;
    Contrib* d_contrib = nullptr;
    int contrib_cap = 0;
    ApplyBufs apply{};
    ZoneBufs zone{};
    PassCounters* d_ctr = nullptr;
    PassCounters* h_ctr = nullptr;
    unsigned long long* h_bbox = nullptr;
    int* d_rank[2] = {nullptr, nullptr};
    RefTreeOrder tree[2];
    double volume = 0.0;
    int* d_level_off = nullptr;
    int nlevels = 0;
    int win_nslots = 0;
    std::vector<int2> h_win_load, h_win_wb;
    std::vector<int> h_win_load_off, h_win_wb_off;
    std::vector<int4> h_win_hdr;
    int2 h_win_wb_final{0, 0};
    int4* d_win_hdr = nullptr;
    int2* d_win_load = nullptr;
    int* d_win_load_off = nullptr;
    int2* d_win_wb = nullptr;
    int* d_win_wb_off = nullptr;
    void* d_strain_step = nullptr;
    int* d_strain_passes = nullptr;
    std::vector<Box6> h_boxes;
    std::vector<int> h_rank;

    // recording
    bool record = false;
    VisitRec* d_rec = nullptr;
    int rec_cap = 0;
    std::vector<VisitRec> visits;
    std::vector<int> pass_kinds;

    cc_params prm{1e-3, 1e-4, 1e-6, 1000.0, 0.01, 0.02, 0.0};
    double lo[3] = {-1e30, -1e30, -1e30}, hi[3] = {1e30, 1e30, 1e30};
    long long counters[13] = {0};
    int pass_index = 0;
    bool own_stream = true;
    long long launches_last = 0;

    // per-stage GPU time, measured with events on the solver's stream
    bool profiling = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, int>> ev_marks;  // (stage, event index of its start; end = start+1)
    double stage_ms[kNumStages] = {0};
    long long stage_calls[kNumStages] = {0};
    void prof(int stage, bool begin) {
        if (!profiling) return;
        size_t need = ev_marks.size() * 2 + 2;
        while (ev_pool.size() < need) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev_pool.push_back(e);
        }
        if (begin) {
            ev_marks.push_back({stage, (int)(ev_marks.size() * 2)});
            cudaEventRecord(ev_pool[ev_marks.back().second], stream);
        } else {
            cudaEventRecord(ev_pool[ev_marks.back().second + 1], stream);
        }
    }
    void prof_collect() {
        if (!profiling) return;
        for (auto& m : ev_marks) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ev_pool[m.second], ev_pool[m.second + 1]) == cudaSuccess) {
                stage_ms[m.first] += ms;
                stage_calls[m.first]++;
            }
        }
        ev_marks.clear();
    }
    int zone_cap = 10000;
    int mode = 0;  // 0 plain FP64, 1 mixed precision
    bool strain_window = true;
    float4* d_pbox_lo = nullptr;
    float4* d_pbox_hi = nullptr;

    ~cc_solver() { release(); }

    void release_mesh() {
        dfree(d_ev); dfree(d_esurf); dfree(d_erigid); dfree(d_fixed); dfree(d_in_elem); dfree(d_edges);
        dfree(d_xo); dfree(d_av); dfree(d_uf);
        dfree(d_xold_in); dfree(d_xcand_in); dfree(d_vel); dfree(d_xout); dfree(d_hc);
        dfree(d_box); dfree(bvh.keys); dfree(bvh.order); dfree(bvh.child); dfree(bvh.range_hi); dfree(bvh.parent);
        dfree(bvh.flags); dfree(bvh.node_box); dfree(bvh.bbox_enc);
        if (bvh.sort_temp) cudaFree(bvh.sort_temp);
        bvh.sort_temp = nullptr;
        dfree(d_pairs); dfree(d_contrib);
        dfree(apply.cnt); dfree(apply.off); dfree(apply.cur); dfree(apply.idx);
        if (apply.scan_temp) cudaFree(apply.scan_temp);
        apply.scan_temp = nullptr;
        dfree(zone.root); dfree(zone.zcnt); dfree(zone.keys); dfree(zone.vals); dfree(zone.nmembers);
        if (zone.sort_temp) cudaFree(zone.sort_temp);
        zone.sort_temp = nullptr;
        dfree(d_rank[0]); dfree(d_rank[1]);
        dfree(d_level_off); dfree(d_strain_passes); dfree(d_rec); dfree(d_pbox_lo); dfree(d_pbox_hi);
        dfree(d_win_load); dfree(d_win_load_off); dfree(d_win_wb); dfree(d_win_wb_off); dfree(d_win_hdr);
        win_nslots = 0;
        if (d_strain_step) cudaFree(d_strain_step);
        d_strain_step = nullptr;
        pair_cap = contrib_cap = rec_cap = 0;
        nv = nt = nb = ne = nedges = 0;
        tree[0] = RefTreeOrder();
        tree[1] = RefTreeOrder();
    }

    void release() {
        if (device >= 0) cudaSetDevice(device);
        release_mesh();
        dfree(d_ctr);
        if (h_ctr) cudaFreeHost(h_ctr);
        if (h_bbox) cudaFreeHost(h_bbox);
        h_ctr = nullptr;
        h_bbox = nullptr;
        for (auto e : ev_pool) cudaEventDestroy(e);
        ev_pool.clear();
        if (stream && own_stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }

    cc_status fail(cc_status st, const std::string& msg) {
        err = msg;
        return st;
    }
    cc_status cuda_check(const char* where) {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return fail(CC_CUDA_ERROR, std::string(where) + ": " + cudaGetErrorString(e));
        return CC_OK;
    }

    cc_status grow_pairs(int cap) {
        dfree(d_pairs);
        if (dalloc(&d_pairs, (size_t)cap) != cudaSuccess) return fail(CC_NO_MEMORY, "pair buffer");
        pair_cap = cap;
        if (record) {
            dfree(d_rec);
            if (dalloc(&d_rec, (size_t)cap) != cudaSuccess) return fail(CC_NO_MEMORY, "record buffer");
            rec_cap = cap;
        }
        return CC_OK;
    }
    cc_status grow_contrib(int cap) {
        dfree(d_contrib);
        dfree(apply.idx);
        if (dalloc(&d_contrib, (size_t)cap) != cudaSuccess || dalloc(&apply.idx, (size_t)cap) != cudaSuccess)
            return fail(CC_NO_MEMORY, "contribution buffer");
        contrib_cap = cap;
        return CC_OK;
    }

    cc_status assemble(const cc_mesh* m);
    cc_status resolve(const double* x_old, const double* x_cand, double* vel, uint8_t* hc, double* x_out,
                      int* has_collision);
    cc_status resolve_impl(const double* x_old, const double* x_cand, double* vel, uint8_t* hc, double* x_out,
                           int* has_collision);
    cc_status detect_pass(int moving, int zone_mode, bool* is_collision);
    cc_status update_tree(int which);
    Params params() const { return Params{prm.dt, prm.thickness, prm.eps, prm.k, prm.m, prm.lambda, prm.cr}; }
};

cc_status cc_solver::assemble(const cc_mesh* m) {
    if (!m || m->n_points < 0 || m->n_tris < 0 || m->n_bonds < 0) return fail(CC_BAD_INPUT, "bad mesh sizes");
    if ((m->n_tris && (!m->tris || !m->tri_rest_len)) || (m->n_bonds && (!m->bonds || !m->bond_rest_len)))
        return fail(CC_BAD_INPUT, "missing element arrays");
    long long ne_ll = (long long)m->n_tris + m->n_bonds;
    if (ne_ll >= (1ll << 22)) return fail(CC_BAD_INPUT, "more than 2^22-1 elements");
    cudaSetDevice(device);
    release_mesh();
    nv = m->n_points; nt = m->n_tris; nb = m->n_bonds; ne = nt + nb;
    std::vector<int> ev((size_t)ne * 3, -1), esurf((size_t)ne, -1);
    std::vector<uint8_t> fixed((size_t)nv, 0), in_elem((size_t)nv, 0), erigid((size_t)ne, 0);
    if (m->fixed)
        for (int i = 0; i < nv; ++i) fixed[i] = m->fixed[i] ? 1 : 0;
    for (int t = 0; t < nt; ++t) {
        for (int k = 0; k < 3; ++k) {
            int v = m->tris[3 * t + k];
            if (v < 0 || v >= nv) return fail(CC_BAD_INPUT, "triangle point id out of range");
            ev[3 * t + k] = v;
        }
        if (ev[3 * t] == ev[3 * t + 1] || ev[3 * t] == ev[3 * t + 2] || ev[3 * t + 1] == ev[3 * t + 2])
            return fail(CC_BAD_INPUT, "triangle with a repeated point");
        esurf[t] = m->tri_surface ? m->tri_surface[t] : 0;
    }
    for (int b = 0; b < nb; ++b) {
        for (int k = 0; k < 2; ++k) {
            int v = m->bonds[2 * b + k];
            if (v < 0 || v >= nv) return fail(CC_BAD_INPUT, "bond point id out of range");
            ev[3 * (nt + b) + k] = v;
        }
    }
    std::vector<StrainEdge> edges;
    edges.reserve((size_t)3 * nt + nb);
    for (int e = 0; e < ne; ++e) {
        int np = e < nt ? 3 : 2;
        bool rigid = false;
        for (int i = 0; i < np; ++i) {
            in_elem[ev[3 * e + i]] = 1;
            if (fixed[ev[3 * e + i]]) rigid = true;
        }
        erigid[e] = rigid ? 1 : 0;
        if (rigid) continue;  // isRigidBody(hse), dcollid.cpp:495
        if (np == 3) {
            for (int j = 0; j < 3; ++j)
                edges.push_back(StrainEdge{ev[3 * e + j], ev[3 * e + (j + 1) % 3], m->tri_rest_len[3 * e + j], 0, 0});
        } else {
            edges.push_back(StrainEdge{ev[3 * e], ev[3 * e + 1], m->bond_rest_len[e - nt], 0, 0});
        }
    }
    nedges = (int)edges.size();
    // dependency levels of the strain sweep: an edge waits for the last
    // earlier edge at each of its points
    std::vector<int> lvl((size_t)nedges), last((size_t)nv, 0);
    nlevels = 0;
    for (int i = 0; i < nedges; ++i) {
        int l = 1 + std::max(last[edges[i].p0], last[edges[i].p1]);
        lvl[i] = l;
        last[edges[i].p0] = last[edges[i].p1] = l;
        if (l > nlevels) nlevels = l;
    }
    std::vector<int> level_off((size_t)nlevels + 2, 0);
    for (int i = 0; i < nedges; ++i) level_off[lvl[i]]++;  // counts at index level (1-based)
    for (int l = 1; l <= nlevels + 1; ++l) level_off[l] += level_off[l - 1];
    // level_off[l] now = edges with level <= l; shift to start offsets of level l+1 (0-based)
    std::vector<StrainEdge> sorted((size_t)nedges);
    {
        std::vector<int> cur(level_off.begin(), level_off.end());
        for (int i = 0; i < nedges; ++i) sorted[cur[lvl[i] - 1]++] = edges[i];
    }
    edges.swap(sorted);
    // shared-memory window of the sweep: each point lives in a slot from a few
    // levels before its first edge to two levels after its last one
    {
        const int ahead = 8;  // kWindowAhead in cc_post.cu
        std::vector<int> first((size_t)nv, -1), lastl((size_t)nv, -1);
        for (int l = 0; l < nlevels; ++l)
            for (int i = level_off[l]; i < level_off[l + 1]; ++i)
                for (int p : {edges[i].p0, edges[i].p1}) {
                    if (first[p] < 0) first[p] = l;
                    lastl[p] = l;
                }
        std::vector<std::pair<int, int>> order;  // (load level, point)
        for (int p = 0; p < nv; ++p)
            if (first[p] >= 0) order.push_back({std::max(0, first[p] - ahead), p});
        std::sort(order.begin(), order.end());
        std::vector<int> slot((size_t)nv, -1);
        std::priority_queue<std::pair<int, int>, std::vector<std::pair<int, int>>, std::greater<>> busy;  // (end, slot)
        std::priority_queue<int, std::vector<int>, std::greater<>> freeq;
        win_nslots = 0;
        for (auto& lp : order) {
            int start = lp.first, p = lp.second;
            while (!busy.empty() && busy.top().first < start) {
                freeq.push(busy.top().second);
                busy.pop();
            }
            int sl;
            if (!freeq.empty()) {
                sl = freeq.top();
                freeq.pop();
            } else {
                sl = win_nslots++;
            }
            slot[p] = sl;
            busy.push({lastl[p] + 2, sl});
        }
        for (auto& ed : edges) {
            ed.s0 = slot[ed.p0];
            ed.s1 = slot[ed.p1];
        }
        std::vector<int> load_off((size_t)nlevels + 1, 0), wb_off((size_t)nlevels + 2, 0);
        for (auto& lp : order) load_off[lp.first + 1]++;
        for (int p = 0; p < nv; ++p)
            if (first[p] >= 0) wb_off[lastl[p] + 2]++;  // written back at level last + 1
        for (int l = 0; l < nlevels; ++l) load_off[l + 1] += load_off[l];
        for (int l = 0; l <= nlevels; ++l) wb_off[l + 1] += wb_off[l];
        h_win_load.assign(order.size(), int2{0, 0});
        h_win_wb.assign(order.size(), int2{0, 0});
        std::vector<int> lc(load_off.begin(), load_off.end()), wc(wb_off.begin(), wb_off.end());
        for (auto& lp : order) h_win_load[lc[lp.first]++] = int2{lp.second, slot[lp.second]};
        for (int p = 0; p < nv; ++p)
            if (first[p] >= 0) h_win_wb[wc[lastl[p] + 1]++] = int2{p, slot[p]};
        h_win_hdr.assign(2 * (size_t)nlevels, int4{0, 0, 0, 0});
        for (int l = 0; l < nlevels; ++l) {
            h_win_hdr[2 * l] = int4{level_off[l], level_off[l + 1], load_off[l], load_off[l + 1]};
            h_win_hdr[2 * l + 1] = int4{wb_off[l], wb_off[l + 1], 0, 0};
        }
        h_win_wb_final = int2{wb_off[nlevels], wb_off[nlevels + 1]};
        h_win_load_off.swap(load_off);
        h_win_wb_off.swap(wb_off);
    }

    bool ok = true;
    ok &= dalloc(&d_ev, (size_t)ne * 3) == cudaSuccess;
    ok &= dalloc(&d_esurf, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_erigid, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_fixed, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_in_elem, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_edges, (size_t)nedges) == cudaSuccess;
    ok &= dalloc(&d_xo, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_av, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_uf, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_xold_in, (size_t)nv * 3) == cudaSuccess;
    ok &= dalloc(&d_xcand_in, (size_t)nv * 3) == cudaSuccess;
    ok &= dalloc(&d_vel, (size_t)nv * 3) == cudaSuccess;
    ok &= dalloc(&d_xout, (size_t)nv * 3) == cudaSuccess;
    ok &= dalloc(&d_hc, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_box, (size_t)ne) == cudaSuccess;
    bvh.n = ne;
    ok &= dalloc(&bvh.keys, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.order, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.child, (size_t)2 * ne) == cudaSuccess;
    ok &= dalloc(&bvh.range_hi, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.parent, (size_t)2 * ne) == cudaSuccess;
    ok &= dalloc(&bvh.flags, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.node_box, (size_t)ne) == cudaSuccess;
    ok &= dalloc(&bvh.bbox_enc, 6) == cudaSuccess;
    ok &= cudaMalloc(&bvh.sort_temp, radix_sort_temp_bytes(ne > 0 ? ne : 1)) == cudaSuccess;
    ok &= dalloc(&apply.cnt, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&apply.off, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&apply.cur, (size_t)nv) == cudaSuccess;
    ok &= cudaMalloc(&apply.scan_temp, scan_temp_bytes(nv > 0 ? nv : 1)) == cudaSuccess;
    ok &= dalloc(&zone.root, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&zone.zcnt, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&zone.keys, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&zone.vals, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&zone.nmembers, 1) == cudaSuccess;
    ok &= cudaMalloc(&zone.sort_temp, radix_sort_temp_bytes(nv > 0 ? nv : 1)) == cudaSuccess;
    ok &= dalloc(&d_rank[0], (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_rank[1], (size_t)ne) == cudaSuccess;
    ok &= dalloc(&d_level_off, (size_t)nlevels + 1) == cudaSuccess;
    ok &= dalloc(&d_win_load, h_win_load.size()) == cudaSuccess;
    ok &= dalloc(&d_win_load_off, h_win_load_off.size()) == cudaSuccess;
    ok &= dalloc(&d_win_wb, h_win_wb.size()) == cudaSuccess;
    ok &= dalloc(&d_win_wb_off, h_win_wb_off.size()) == cudaSuccess;
    ok &= dalloc(&d_win_hdr, h_win_hdr.size()) == cudaSuccess;
    ok &= dalloc(&d_pbox_lo, (size_t)nv) == cudaSuccess;
    ok &= dalloc(&d_pbox_hi, (size_t)nv) == cudaSuccess;
    ok &= cudaMalloc(&d_strain_step, strain_step_bytes(nedges)) == cudaSuccess;
    ok &= dalloc(&d_strain_passes, 3) == cudaSuccess;
    if (!ok) return fail(CC_NO_MEMORY, "device allocation failed");
    cc_status st = grow_pairs(16 * ne + 4096);
    if (st) return st;
    st = grow_contrib(8 * ne + 4096);
    if (st) return st;
    cudaMemcpyAsync(d_ev, ev.data(), sizeof(int) * ev.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_esurf, esurf.data(), sizeof(int) * esurf.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_erigid, erigid.data(), erigid.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_fixed, fixed.data(), fixed.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d_in_elem, in_elem.data(), in_elem.size(), cudaMemcpyHostToDevice, stream);
    if (nedges) {
        cudaMemcpyAsync(d_edges, edges.data(), sizeof(StrainEdge) * edges.size(), cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_level_off, level_off.data(), sizeof(int) * ((size_t)nlevels + 1), cudaMemcpyHostToDevice,
                        stream);
        cudaMemcpyAsync(d_win_load, h_win_load.data(), sizeof(int2) * h_win_load.size(), cudaMemcpyHostToDevice,
                        stream);
        cudaMemcpyAsync(d_win_load_off, h_win_load_off.data(), sizeof(int) * h_win_load_off.size(),
                        cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_win_wb, h_win_wb.data(), sizeof(int2) * h_win_wb.size(), cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_win_wb_off, h_win_wb_off.data(), sizeof(int) * h_win_wb_off.size(),
                        cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_win_hdr, h_win_hdr.data(), sizeof(int4) * h_win_hdr.size(), cudaMemcpyHostToDevice,
                        stream);
    }
    cudaMemsetAsync(d_av, 0, sizeof(double4_32a) * (size_t)(nv > 0 ? nv : 1), stream);
    h_boxes.resize((size_t)ne);
    h_rank.resize((size_t)ne);
    volume = 0.0;
    cudaStreamSynchronize(stream);
    return cuda_check("assemble");
}

// Tree build / rebuild bookkeeping of aabbProximity / aabbCollision
// (dcollid.cpp:366-428): both trees share one volume; a tree is (re)built
// on first use or when its root volume has grown by more than 20%.
cc_status cc_solver::update_tree(int which) {
    cudaMemcpyAsync(h_bbox, bvh.bbox_enc, 6 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("leaf boxes");
    double rlo[3], rhi[3];
    for (int d = 0; d < 3; ++d) {
        rlo[d] = dec_host(h_bbox[d]);
        rhi[d] = dec_host(h_bbox[3 + d]);
    }
    double v = box_volume(rlo, rhi);
    bool rebuild = !tree[which].built() || (v - volume) > 0.2 * volume;
    if (!rebuild) return CC_OK;
    cudaMemcpyAsync(h_boxes.data(), d_box, sizeof(Box6) * (size_t)ne, cudaMemcpyDeviceToHost, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("leaf boxes to host");
    volume = tree[which].build(h_boxes.data(), ne);
    tree[which].ranks(h_rank.data());
    cudaMemcpyAsync(d_rank[which], h_rank.data(), sizeof(int) * (size_t)ne, cudaMemcpyHostToDevice, stream);
    counters[8]++;
    return CC_OK;
}

// One detection pass: boxes, tree bookkeeping, candidate pairs, narrow
// phase, impulses applied (aabbProximity/aabbCollision + updateAverageVelocity,
// dcollid.cpp:390-406, 430-468), and in zone mode the rigid zone update
// (dcollid.cpp:236-262). Retried with larger buffers on overflow.
cc_status cc_solver::detect_pass(int moving, int zone_mode, bool* is_collision) {
    int pass = pass_index++;
    pass_kinds.push_back(moving ? (zone_mode ? kPassZone : kPassCcd) : kPassProx);
    counters[0]++;
    if (moving) counters[zone_mode ? 2 : 1]++;
    prof(kStBoxes, true);
    leaf_boxes(d_ev, ne, nt, d_xo, d_av, prm.dt, moving, d_box, bvh.bbox_enc, stream);
    prof(kStBoxes, false);
    cc_status st = update_tree(moving);
    if (st) return st;
    prof(kStBvh, true);
    bvh_build(d_box, bvh, stream);
    if (mode == 1) point_boxes(d_xo, d_av, prm.dt, nv, moving, d_pbox_lo, d_pbox_hi, stream);
    prof(kStBvh, false);
    Params p = params();
    for (int attempt = 0; attempt < 8; ++attempt) {
        count_launch(), k_reset_counters<<<1, 1, 0, stream>>>(d_ctr);
        prof(kStTraverse, true);
        bvh_pairs(d_box, bvh, d_pairs, pair_cap, d_ctr, stream);
        prof(kStTraverse, false);
        NarrowArgs a;
        a.xo = d_xo; a.av = d_av; a.fixed = d_fixed; a.ev = d_ev; a.esurf = d_esurf; a.erigid = d_erigid;
        a.rank = d_rank[moving]; a.nt = nt; a.pass = pass; a.zone = zone_mode; a.p = p; a.pairs = d_pairs;
        a.contrib = d_contrib; a.contrib_cap = contrib_cap; a.ctr = d_ctr; a.uf_parent = d_uf;
        a.rec = record ? d_rec : nullptr; a.rec_cap = rec_cap;
        a.pbox_lo = mode == 1 ? d_pbox_lo : nullptr;
        a.pbox_hi = mode == 1 ? d_pbox_hi : nullptr;
        {
            // h of the sub-tests (thickness for proximity, eps for CCD) and
            // the barycentric tolerance eps, rounded up to FP32
            double h = moving ? prm.eps : prm.thickness;
            float hf = (float)h, ef = (float)prm.eps;
            if ((double)hf < h) hf = nextafterf(hf, 1e30f);
            if ((double)ef < prm.eps) ef = nextafterf(ef, 1e30f);
            a.hpad = hf;
            a.epad = ef;
        }
        prof(moving ? kStNarrowCcd : kStNarrowProx, true);
        narrow_pass(a, moving, pair_cap, stream);
        prof(moving ? kStNarrowCcd : kStNarrowProx, false);
        prof(kStApply, true);
        apply_contribs(d_contrib, d_ctr, contrib_cap, nv, d_av, d_hc, apply, stream);
        prof(kStApply, false);
        cudaMemcpyAsync(h_ctr, d_ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, stream);
        if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("detection pass");
        int e = h_ctr->err;
        if (e & kErrNan) return fail(CC_NAN_DETECTED, "non-finite velocity or normal (the reference exits here)");
        if (e & kErrStack) return fail(CC_STACK_OVERFLOW, "BVH traversal stack overflow");
        if (e & kErrPairOverflow) {
            st = grow_pairs(2 * h_ctr->npairs + 1024);
            if (st) return st;
            continue;
        }
        if (e & kErrContribOverflow) {
            st = grow_contrib(2 * h_ctr->ncontrib + 1024);
            if (st) return st;
            continue;
        }
        if (e & kErrRecordOverflow) {
            st = grow_pairs(pair_cap);
            if (st) return st;
            continue;
        }
        break;
    }
    if (h_ctr->err) return fail(CC_PAIR_OVERFLOW, "buffers kept overflowing");
    counters[3] += h_ctr->npairs;
    counters[4] += h_ctr->nvisits;
    counters[5] += h_ctr->nhit_pairs;
    counters[6] += h_ctr->ncontacts;
    counters[12] += h_ctr->nsub;
    if (record && h_ctr->nrec > 0) {
        size_t base = visits.size();
        visits.resize(base + (size_t)h_ctr->nrec);
        cudaMemcpyAsync(visits.data() + base, d_rec, sizeof(VisitRec) * (size_t)h_ctr->nrec,
                        cudaMemcpyDeviceToHost, stream);
    }
    if (zone_mode) {
        prof(kStZone, true);
        zone_velocity(d_uf, d_in_elem, d_fixed, d_xo, d_av, nv, p, zone, d_ctr, stream);
        prof(kStZone, false);
        cudaMemcpyAsync(h_ctr, d_ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, stream);
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("pass tail");
    if (h_ctr->err & kErrNan) return fail(CC_NAN_DETECTED, "non-finite zone velocity (the reference exits here)");
    *is_collision = h_ctr->nhit_pairs > 0;
    return CC_OK;
}

cc_status cc_solver::resolve(const double* x_old, const double* x_cand, double* vel, uint8_t* hc, double* x_out,
                             int* has_collision) {
    long long l0 = g_kernel_launches;
    cc_status st0 = resolve_impl(x_old, x_cand, vel, hc, x_out, has_collision);
    launches_last = g_kernel_launches - l0;
    return st0;
}

cc_status cc_solver::resolve_impl(const double* x_old, const double* x_cand, double* vel, uint8_t* hc,
                                  double* x_out, int* has_collision) {
    std::memset(counters, 0, sizeof(counters));
    pass_index = 0;
    visits.clear();
    pass_kinds.clear();
    if (has_collision) *has_collision = 0;
    if (ne == 0) {
        // the reference dereferences an empty tree here; nothing collides
        if (nv) cudaMemcpyAsync(x_out, x_cand, sizeof(double) * 3 * (size_t)nv, cudaMemcpyDeviceToDevice, stream);
        cudaStreamSynchronize(stream);
        return cuda_check("empty mesh");
    }
    // d_hc doubles as the device copy of has_collsn
    if (hc != d_hc) cudaMemcpyAsync(d_hc, hc, (size_t)nv, cudaMemcpyDeviceToDevice, stream);
    count_launch(), k_reset_counters<<<1, 1, 0, stream>>>(d_ctr);
    cudaMemsetAsync(&d_ctr->err, 0, sizeof(int), stream);
    ev_marks.clear();
    prof(kStInit, true);
    step_init(x_old, x_cand, nv, d_in_elem, prm.dt, d_xo, d_av, d_ctr, stream);
    uf_init(d_uf, nv, stream);
    prof(kStInit, false);
    bool is_coll = false;
    cc_status st = detect_pass(0, 0, &is_coll);
    if (st) return st;
    int hcol = 0;
    is_coll = true;
    int niter = 1, cd_count = 0;
    while (is_coll) {
        st = detect_pass(1, 0, &is_coll);
        if (st) return st;
        if (cd_count++ == 0 && is_coll) hcol = 1;
        if (++niter > kMaxCcdIter) break;
    }
    if (is_coll) {
        int it = 0;
        while (is_coll) {
            if (it++ >= zone_cap) return fail(CC_ITER_CAP, "impact-zone loop did not converge");
            st = detect_pass(1, 1, &is_coll);
            if (st) return st;
        }
    }
    Params p = params();
    prof(kStFinalize, true);
    finalize_positions(d_in_elem, d_xo, d_av, d_hc, x_cand, x_out, nv, p, lo, hi, stream);
    prof(kStFinalize, false);
    prof(kStStrain, true);
    StrainWindow win{win_nslots, d_win_load, d_win_load_off, d_win_wb, d_win_wb_off, d_win_hdr, h_win_wb_final};
    strain_limit(d_edges, nedges, d_level_off, nlevels, d_xo, d_av, nv, prm.dt, d_strain_step,
                 strain_window ? &win : nullptr, d_strain_passes, stream);
    prof(kStStrain, false);
    final_velocity(d_in_elem, d_hc, d_av, vel, nv, stream);
    if (hc != d_hc) cudaMemcpyAsync(hc, d_hc, (size_t)nv, cudaMemcpyDeviceToDevice, stream);
    int sp[3] = {0, 0, 0};
    if (nedges) cudaMemcpyAsync(sp, d_strain_passes, 3 * sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess) return cuda_check("finalize");
    counters[7] = nedges ? sp[0] : 1;
    counters[10] = sp[1];
    counters[11] = sp[2];
    prof_collect();
    if (has_collision) *has_collision = hcol;
    return cuda_check("resolve");
}

// ------------------------------------------------------------------ C ABI
extern "C" {

cc_status cc_create(int device, cc_solver** out) {
    if (!out) return CC_BAD_INPUT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return CC_CUDA_ERROR;
    cc_solver* s = new cc_solver;
    s->device = device;
    cudaSetDevice(device);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        dalloc(&s->d_ctr, 1) != cudaSuccess || cudaMallocHost(&s->h_ctr, sizeof(PassCounters)) != cudaSuccess ||
        cudaMallocHost(&s->h_bbox, 6 * sizeof(unsigned long long)) != cudaSuccess) {
        delete s;
        return CC_CUDA_ERROR;
    }
    cudaMemset(s->d_ctr, 0, sizeof(PassCounters));
    *out = s;
    return CC_OK;
}

void cc_destroy(cc_solver* s) { delete s; }

cc_status cc_assemble(cc_solver* s, const cc_mesh* mesh) {
    if (!s) return CC_BAD_INPUT;
    return s->assemble(mesh);
}

cc_status cc_set_params(cc_solver* s, const cc_params* p) {
    if (!s || !p) return CC_BAD_INPUT;
    s->prm = *p;
    return CC_OK;
}

cc_status cc_set_domain_boundary(cc_solver* s, const double lo[3], const double hi[3]) {
    if (!s || !lo || !hi) return CC_BAD_INPUT;
    for (int d = 0; d < 3; ++d) {
        s->lo[d] = lo[d];
        s->hi[d] = hi[d];
    }
    return CC_OK;
}

cc_status cc_resolve(cc_solver* s, const double* x_old, const double* x_cand, double* vel, uint8_t* has_collsn,
                     double* x_out, int* has_collision) {
    if (!s) return CC_BAD_INPUT;
    if (s->nv && (!x_old || !x_cand || !vel || !has_collsn || !x_out)) return s->fail(CC_BAD_INPUT, "null array");
    cudaSetDevice(s->device);
    size_t b3 = sizeof(double) * 3 * (size_t)s->nv;
    if (s->nv) {
        cudaMemcpyAsync(s->d_xold_in, x_old, b3, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->d_xcand_in, x_cand, b3, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->d_vel, vel, b3, cudaMemcpyHostToDevice, s->stream);
        cudaMemcpyAsync(s->d_hc, has_collsn, (size_t)s->nv, cudaMemcpyHostToDevice, s->stream);
    }
    cc_status st = s->resolve(s->d_xold_in, s->d_xcand_in, s->d_vel, s->d_hc, s->d_xout, has_collision);
    if (st) return st;
    if (s->nv) {
        cudaMemcpyAsync(x_out, s->d_xout, b3, cudaMemcpyDeviceToHost, s->stream);
        cudaMemcpyAsync(vel, s->d_vel, b3, cudaMemcpyDeviceToHost, s->stream);
        cudaMemcpyAsync(has_collsn, s->d_hc, (size_t)s->nv, cudaMemcpyDeviceToHost, s->stream);
    }
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return s->cuda_check("read back");
    return CC_OK;
}

cc_status cc_resolve_device(cc_solver* s, const double* x_old, const double* x_cand, double* vel,
                            uint8_t* has_collsn, double* x_out, int* has_collision) {
    if (!s) return CC_BAD_INPUT;
    cudaSetDevice(s->device);
    return s->resolve(x_old, x_cand, vel, has_collsn, x_out, has_collision);
}

int cc_get_counters(cc_solver* s, long long* out, int n) {
    if (!s || !out) return 0;
    s->counters[9] = s->launches_last;
    int m = n < 13 ? n : 13;
    for (int i = 0; i < m; ++i) out[i] = s->counters[i];
    return m;
}

cc_status cc_set_recording(cc_solver* s, int on) {
    if (!s) return CC_BAD_INPUT;
    cudaSetDevice(s->device);
    s->record = on != 0;
    if (s->record && s->pair_cap && s->rec_cap < s->pair_cap) return s->grow_pairs(s->pair_cap);
    return CC_OK;
}

int cc_get_visits(cc_solver* s, int* out, int cap) {
    if (!s) return -1;
    int n = (int)s->visits.size();
    if (out)
        for (int i = 0; i < n && i < cap; ++i) {
            const VisitRec& r = s->visits[i];
            int* o = out + 13 * i;
            o[0] = r.pass; o[1] = r.kind; o[2] = r.a; o[3] = r.b; o[4] = r.status;
            for (int k = 0; k < 6; ++k) o[5 + k] = r.dcount[k];
            o[11] = r.rank_b; o[12] = r.rank_a;
        }
    return n;
}

int cc_get_pass_kinds(cc_solver* s, int* out, int cap) {
    if (!s) return -1;
    int n = (int)s->pass_kinds.size();
    if (out)
        for (int i = 0; i < n && i < cap; ++i) out[i] = s->pass_kinds[i];
    return n;
}

cc_status cc_get_zone_roots(cc_solver* s, int* out) {
    if (!s || !out) return CC_BAD_INPUT;
    cudaSetDevice(s->device);
    if (s->nv == 0) return CC_OK;
    std::vector<int> parent((size_t)s->nv);
    cudaMemcpyAsync(parent.data(), s->d_uf, sizeof(int) * (size_t)s->nv, cudaMemcpyDeviceToHost, s->stream);
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return s->cuda_check("zone roots");
    for (int i = 0; i < s->nv; ++i) {
        int r = i, guard = 0;
        while (parent[r] != r && guard++ < s->nv) r = parent[r];
        out[i] = r;
    }
    return CC_OK;
}

cc_status cc_get_leaf_ranks(cc_solver* s, int which, int* out) {
    if (!s || !out || which < 0 || which > 1 || !s->tree[which].built()) return CC_BAD_INPUT;
    s->tree[which].ranks(out);
    return CC_OK;
}

int cc_debug_candidate_pairs(cc_solver* s, int moving, int brute_force, int* out, int cap) {
    if (!s || s->ne == 0) return 0;
    cudaSetDevice(s->device);
    leaf_boxes(s->d_ev, s->ne, s->nt, s->d_xo, s->d_av, s->prm.dt, moving, s->d_box, s->bvh.bbox_enc, s->stream);
    if (!brute_force) bvh_build(s->d_box, s->bvh, s->stream);
    for (int attempt = 0; attempt < 8; ++attempt) {
        count_launch(), k_reset_counters<<<1, 1, 0, s->stream>>>(s->d_ctr);
        cudaMemsetAsync(&s->d_ctr->err, 0, sizeof(int), s->stream);
        if (brute_force)
            brute_pairs(s->d_box, s->ne, s->d_pairs, s->pair_cap, s->d_ctr, s->stream);
        else
            bvh_pairs(s->d_box, s->bvh, s->d_pairs, s->pair_cap, s->d_ctr, s->stream);
        cudaMemcpyAsync(s->h_ctr, s->d_ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, s->stream);
        if (cudaStreamSynchronize(s->stream) != cudaSuccess) return -1;
        if (s->h_ctr->err & kErrPairOverflow) {
            if (s->grow_pairs(2 * s->h_ctr->npairs + 1024)) return -1;
            continue;
        }
        if (s->h_ctr->err) return -1;
        break;
    }
    int n = s->h_ctr->npairs;
    if (out && n > 0) {
        int m = n < cap ? n : cap;
        cudaMemcpyAsync(out, s->d_pairs, sizeof(int2) * (size_t)m, cudaMemcpyDeviceToHost, s->stream);
        cudaStreamSynchronize(s->stream);
    }
    return n;
}

cc_status cc_set_stream(cc_solver* s, void* stream) {
    if (!s) return CC_BAD_INPUT;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    if (stream) {
        s->stream = (cudaStream_t)stream;
        s->own_stream = false;
    } else {
        if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return CC_CUDA_ERROR;
        s->own_stream = true;
    }
    return CC_OK;
}

cc_status cc_set_strain_window(cc_solver* s, int on) {
    if (!s) return CC_BAD_INPUT;
    s->strain_window = on != 0;
    return CC_OK;
}

cc_status cc_set_mode(cc_solver* s, int mode) {
    if (!s || mode < 0 || mode > 1) return CC_BAD_INPUT;
    s->mode = mode;
    return CC_OK;
}

cc_status cc_set_profiling(cc_solver* s, int on) {
    if (!s) return CC_BAD_INPUT;
    s->profiling = on != 0;
    for (int i = 0; i < kNumStages; ++i) {
        s->stage_ms[i] = 0.0;
        s->stage_calls[i] = 0;
    }
    return CC_OK;
}

int cc_get_profile(cc_solver* s, double* ms, long long* calls, int cap) {
    if (!s) return -1;
    for (int i = 0; i < kNumStages && i < cap; ++i) {
        if (ms) ms[i] = s->stage_ms[i];
        if (calls) calls[i] = s->stage_calls[i];
    }
    return kNumStages;
}

const char* cc_profile_stage_name(int i) { return (i >= 0 && i < kNumStages) ? kStageNames[i] : ""; }

int cc_selftest_math(int device, int fn, const double* a, const double* b, double* out, int n) {
    if (n <= 0) return 0;
    if (cudaSetDevice(device) != cudaSuccess) return -1;
    double *da = nullptr, *db = nullptr, *dout = nullptr;
    size_t bytes = sizeof(double) * (size_t)n;
    if (cudaMalloc(&da, bytes) != cudaSuccess || cudaMalloc(&db, bytes) != cudaSuccess ||
        cudaMalloc(&dout, bytes) != cudaSuccess) {
        cudaFree(da); cudaFree(db); cudaFree(dout);
        return -1;
    }
    cudaMemcpy(da, a, bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(db, b ? b : a, bytes, cudaMemcpyHostToDevice);
    math_selftest(fn, da, db, dout, n, 0);
    cudaError_t e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
    cudaFree(da); cudaFree(db); cudaFree(dout);
    return e == cudaSuccess ? n : -1;
}

int cc_last_error(cc_solver* s, char* buf, int len) {
    if (!s || !buf || len <= 0) return 0;
    std::snprintf(buf, (size_t)len, "%s", s->err.c_str());
    return (int)s->err.size();
}

}  // extern "C"
