// Per-point stages around the detection passes: average velocity, applying
// a pass's impulses, impact-zone rigid motion, the domain clamp, final
// positions, strain limiting and final velocities (dcollid.cpp:116-220,
// 290-310, 486-624, 677-751; dcollid3d.cpp:70-200).
#include "cc_launch.h"
#include "cc_narrow.cuh"
#include "cc_strain_plan.h"

namespace ccg {

namespace {

inline int nblk(int n, int t) { return (n + t - 1) / t; }

// computeAverageVelocity, dcollid.cpp:160-220: avgVel = (x_cand - x_old)/dt.
__global__ void k_step_init(const double* __restrict__ x_old, const double* __restrict__ x_cand, int nv,
                            const uint8_t* __restrict__ in_elem, const int* __restrict__ vscene,
                            const SceneDev* __restrict__ scenes, double4_32a* xo, double4_32a* av,
                            PassCounters* ctr) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv) return;
    double o[3] = {x_old[3 * p], x_old[3 * p + 1], x_old[3 * p + 2]};
    xo[p] = make_double4_32a(o[0], o[1], o[2], 0.0);
    if (!in_elem[p]) return;
    const double dt = scenes[vscene[p]].p.dt;
    double v[3];
    bool bad = false;
    for (int j = 0; j < 3; ++j) {
        v[j] = (dt > kRoundEps) ? (x_cand[3 * p + j] - o[j]) / dt : 0.0;
        if (!isfinite(v[j])) bad = true;
    }
    if (bad) atomicOr(&ctr->err, kErrNan);
    av[p] = make_double4_32a(v[0], v[1], v[2], 0.0);
}

__global__ void k_contrib_count(const Contrib* __restrict__ c, const PassCounters* ctr, int cap, int* cnt) {
    if (ctr->err & kErrRetry) return;
    int n = ctr->ncontrib < cap ? ctr->ncontrib : cap;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&cnt[c[i].vertex], 1);
}

__global__ void k_contrib_scatter(const Contrib* __restrict__ c, const PassCounters* ctr, int cap,
                                  const int* __restrict__ off, int* cur, int* idx) {
    if (ctr->err & kErrRetry) return;
    int n = ctr->ncontrib < cap ? ctr->ncontrib : cap;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int v = c[i].vertex;
        idx[off[v] + atomicAdd(&cur[v], 1)] = i;
    }
}

// updateAverageVelocity, dcollid.cpp:677-751, for one point: its
// contributions are put in visiting order and summed one by one from zero,
// as the reference accumulates collsnImpulse and friction. Slots nv.. are
// the movable bodies: their spread impulses are added one by one onto the
// body's running collsnImpulse_RG, which the reference never clears, and
// their count is the pass's collsn_num_RG.
__global__ void k_apply(const Contrib* __restrict__ c, PassCounters* ctr, const int* __restrict__ cnt,
                        const int* __restrict__ off, int* idx, int nv, double4_32a* av, uint8_t* has_collsn,
                        double4_32a* dump, int nbodies, double4_32a* body_acc, int* body_num, PassStamp ps) {
    if (ctr->err & kErrRetry) return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv + nbodies) return;
    int n = cnt[p];
    if (n == 0) return;
    int* seg = idx + off[p];
    // insertion sort of the segment by key (segments are short)
    for (int i = 1; i < n; ++i) {
        int x = seg[i];
        unsigned long long kx = c[x].key;
        int j = i - 1;
        while (j >= 0 && c[seg[j]].key > kx) {
            seg[j + 1] = seg[j];
            --j;
        }
        seg[j + 1] = x;
    }
    if (p >= nv) {
        const int b = p - nv;
        double4_32a a = body_acc[b];
        double acc[3] = {a.x, a.y, a.z};
        for (int i = 0; i < n; ++i) {
            const Contrib& q = c[seg[i]];
            for (int k = 0; k < 3; ++k) acc[k] += q.imp[k];
        }
        body_acc[b] = make_double4_32a(acc[0], acc[1], acc[2], 0.0);
        body_num[b] = n;
        return;
    }
    double imp[3] = {0.0, 0.0, 0.0}, fric[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < n; ++i) {
        const Contrib& q = c[seg[i]];
        for (int k = 0; k < 3; ++k) imp[k] += q.imp[k];
        if (q.flags & 1)
            for (int k = 0; k < 3; ++k) fric[k] += q.fric[k];
    }
    double4_32a a = av[p];
    double v[3] = {a.x, a.y, a.z};
    bool bad = false;
    for (int k = 0; k < 3; ++k) {
        v[k] += (imp[k] + fric[k]) / n;
        if (!isfinite(v[k])) bad = true;
    }
    if (bad) atomicOr(&ctr->err, kErrNan);
    av[p] = make_double4_32a(v[0], v[1], v[2], 0.0);
    has_collsn[p] = 1;
    stamp_point(ps, p);
    if (dump) dump[p] = make_double4_32a(imp[0], imp[1], imp[2], (double)n);  // collsnImpulse, collsn_num
}

// The spread part of updateAverageVelocity (dcollid.cpp:726-733), after
// each point's own impulses: avgVel += collsnImpulse_RG / collsn_num_RG for
// every member of a body that received spread impulses this pass.
__global__ void k_apply_rg(const int* __restrict__ members, const int* __restrict__ member_body, int nmembers,
                           const PassCounters* ctr, const double4_32a* __restrict__ body_acc,
                           const int* __restrict__ body_num, const uint8_t* __restrict__ fixed, double4_32a* av,
                           uint8_t* has_collsn, PassStamp ps) {
    if (ctr->err & kErrRetry) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nmembers) return;
    const int b = member_body[i], n = body_num[b];
    const int p = members[i];
    if (n == 0 || (fixed[p] & 1)) return;
    const double4_32a a = body_acc[b];
    double4_32a v = av[p];
    v.x += a.x / n;
    v.y += a.y / n;
    v.z += a.z / n;
    av[p] = v;
    has_collsn[p] = 1;
    stamp_point(ps, p);
}

__device__ __forceinline__ double det3(const double (*a)[3]) {
    return a[0][0] * (a[1][1] * a[2][2] - a[2][1] * a[1][2]) - a[0][1] * (a[1][0] * a[2][2] - a[2][0] * a[1][2]) +
           a[0][2] * (a[1][0] * a[2][1] - a[2][0] * a[1][1]);
}

// updateImpactListVelocity, dcollid3d.cpp:70-200, one thread per zone over
// its members in the order of the reference's member list (which fixes the
// rounding of every sum); sin and cos correctly rounded, as the reference's
// libm gives them.
// The last loop of updateImpactListVelocity (dcollid3d.cpp:160-199) for one
// member p of a zone: its new average velocity from the zone's rigid motion
// (centre x_cm moving at v_cm, angular velocity w of magnitude mag_w, and
// sw = sin(dt mag_w) / mag_w, cw = cos(dt mag_w), which the reference forms
// again for every member with the same result). Static points keep theirs.
// True when a velocity is NaN.
__device__ __forceinline__ bool zone_member_motion(int p, const uint8_t* __restrict__ fixed,
                                                   const double4_32a* __restrict__ xo, double4_32a* av,
                                                   const double* x_cm, const double* v_cm, const double* w,
                                                   double mag_w, double sw, double cw, double dt,
                                                   const PassStamp& ps) {
    if (fixed[p] & 1) return false;
    stamp_point(ps, p);
    double xs[3], dx[3], xF[3], xR[3], wxR[3], tmpV[3], x_new[3], nv_[3];
    load3(xo, p, xs);
    for (int d = 0; d < 3; ++d) dx[d] = xs[d] - x_cm[d];
    if (mag_w < kRoundEps) {
        for (int d = 0; d < 3; ++d) { xF[d] = dx[d]; wxR[d] = 0.0; }
        for (int d = 0; d < 3; ++d) xR[d] = dx[d] - xF[d];
    } else {
        double sc = dot3(dx, w) / dot3(w, w);
        for (int d = 0; d < 3; ++d) xF[d] = sc * w[d];
        for (int d = 0; d < 3; ++d) xR[d] = dx[d] - xF[d];
        for (int d = 0; d < 3; ++d) tmpV[d] = sw * w[d];
        cross3(tmpV, xR, wxR);
    }
    bool bad = false;
    for (int d = 0; d < 3; ++d) {
        x_new[d] = x_cm[d] + dt * v_cm[d] + xF[d] + cw * xR[d] + wxR[d];
        nv_[d] = (x_new[d] - xs[d]) / dt;
        if (isnan(nv_[d])) bad = true;
    }
    av[p] = make_double4_32a(nv_[0], nv_[1], nv_[2], 0.0);
    return bad;
}

// Angular velocity of a zone from its angular momentum L and inertia I
// (Cramer's rule, dcollid3d.cpp:143-153).
__device__ __forceinline__ void zone_omega(const double (*I)[3], const double* L, double* w) {
    double tmp[3][3];
    for (int r = 0; r < 3; ++r) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) tmp[a][b] = I[a][b];
        for (int s = 0; s < 3; ++s) tmp[s][r] = L[s];
        if (det3(I) < kRoundEps)
            w[r] = 0.0;
        else
            w[r] = det3(tmp) / det3(I);
    }
}

// With `run` set, the zones are movable bodies (updateImpactZoneVelocityForRG,
// dcollid.cpp:267-288, called from updateAverageVelocity when dt > 0): only
// those of scenes in a pass, and of more than one point, move.
__device__ void zone_motion(const int* __restrict__ members, int i, int end, const uint8_t* __restrict__ fixed,
                            const double4_32a* __restrict__ xo, double4_32a* av, const int* __restrict__ vscene,
                            const SceneDev* __restrict__ scenes, PassCounters* ctr,
                            const SceneRun* __restrict__ run, const PassStamp& ps) {
    const int zs = vscene[members[i]];
    const Params prm = scenes[zs].p;
    if (run && (run[zs].mode == kSceneIdle || !(prm.dt > 0.0) || end - i < 2 || (ctr->err & kErrRetry))) return;
    const double m = prm.m, dt = prm.dt;
    double x_cm[3] = {0.0, 0.0, 0.0}, v_cm[3] = {0.0, 0.0, 0.0};
    double L[3] = {0.0, 0.0, 0.0}, I[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}}, tmp[3][3];
    int num_pts = end - i;
    for (int q = i; q < end; ++q) {
        int p = members[q];
        double xs[3], vs[3];
        load3(xo, p, xs);
        load3(av, p, vs);
        for (int d = 0; d < 3; ++d) { x_cm[d] += xs[d]; v_cm[d] += vs[d]; }
    }
    for (int d = 0; d < 3; ++d) { x_cm[d] /= num_pts; v_cm[d] /= num_pts; }
    for (int q = i; q < end; ++q) {
        int p = members[q];
        double xs[3], vs[3], dx[3], dv[3], Li[3];
        load3(xo, p, xs);
        load3(av, p, vs);
        for (int d = 0; d < 3; ++d) { dx[d] = xs[d] - x_cm[d]; dv[d] = vs[d] - v_cm[d]; }
        cross3(dx, dv, Li);
        for (int d = 0; d < 3; ++d) Li[d] = m * Li[d];
        for (int d = 0; d < 3; ++d) L[d] = Li[d] + L[d];
    }
    for (int q = i; q < end; ++q) {
        int p = members[q];
        double xs[3], dx[3];
        load3(xo, p, xs);
        for (int d = 0; d < 3; ++d) dx[d] = xs[d] - x_cm[d];
        double mag_dx = mag3(dx);
        for (int r = 0; r < 3; ++r)
            for (int s = 0; s < 3; ++s) {
                tmp[r][s] = -dx[r] * dx[s];
                if (r == s) tmp[r][s] += mag_dx * mag_dx;
                I[r][s] += tmp[r][s] * m;
            }
    }
    double w[3];
    zone_omega(I, L, w);
    double mag_w = mag3(w);
    double sn, cs;
    cr::sincos(dt * mag_w, &sn, &cs);
    const double sw = mag_w < kRoundEps ? 0.0 : sn / mag_w;
    const double cw = cs;
    bool bad = false;
    for (int q = i; q < end; ++q)
        bad |= zone_member_motion(members[q], fixed, xo, av, x_cm, v_cm, w, mag_w, sw, cw, dt, ps);
    if (bad) atomicOr(&ctr->err, kErrNan);
}

// Zones of at least this many members are solved one warp per zone
// (k_zone_solve_warp) where the zone list is built on the device; in a pass
// with at most `few` zones (a knob), every zone of two or more members is:
// one thread per zone keeps the FP64 pipe busiest when zones are many, one
// warp per zone gives the shortest chain when they are few.
constexpr int kZoneWarpMin = 16;
__device__ __forceinline__ int zone_warp_min(int nzones, int few) { return nzones <= few ? 2 : kZoneWarpMin; }
constexpr int kZoneWarpBlock = 128;
constexpr int kZoneCtaThreads = 256;

// Zone z's members are members[zone_off[z] .. zone_off[z+1]), or with
// zone_rng members[zone_rng[z].x .. zone_rng[z].y); dnz (may be null): the
// zone count in device memory, at most nzones.
__global__ void k_zone_solve(const int* __restrict__ members, const int* __restrict__ zone_off,
                             const int2* __restrict__ zone_rng, int nzones, const int* __restrict__ dnz,
                             const uint8_t* __restrict__ fixed, const double4_32a* __restrict__ xo, double4_32a* av,
                             const int* __restrict__ vscene, const SceneDev* __restrict__ scenes,
                             PassCounters* ctr, const SceneRun* __restrict__ run, PassStamp ps, int few) {
    if (dnz) {
        if (ctr->err & kErrRetry) return;
        if (*dnz < nzones) nzones = *dnz;
    }
    const int warp_min = zone_warp_min(nzones, few);
    for (int z = blockIdx.x * blockDim.x + threadIdx.x; z < nzones; z += gridDim.x * blockDim.x) {
        const int i = zone_rng ? zone_rng[z].x : zone_off[z], end = zone_rng ? zone_rng[z].y : zone_off[z + 1];
        if (dnz && end - i >= warp_min) continue;  // k_zone_solve_warp's
        zone_motion(members, i, end, fixed, xo, av, vscene, scenes, ctr, run, ps);
    }
}

// Zones of at least kZoneWarpMin members: one warp per zone. The sums of
// updateImpactListVelocity (centre of mass and velocity, angular momentum,
// inertia) must be formed member by member in list order to round as the
// reference's do, and GB300's FP64 pipe makes such a chain slow on one
// thread: here the lanes load 32 members at a time and form every per-member
// term in parallel (offsets, m * (dx x dv), m * (|dx|^2 delta - dx dx)),
// and lane 0 only adds the staged terms in order - the same additions on
// the same operands as the one-thread form. The final per-member motion is
// spread over the lanes.
__global__ void __launch_bounds__(kZoneWarpBlock) k_zone_solve_warp(
    const int* __restrict__ members, const int2* __restrict__ zone_rng, int nzones, const int* __restrict__ dnz,
    const uint8_t* __restrict__ fixed, const double4_32a* __restrict__ xo, double4_32a* av,
    const int* __restrict__ vscene, const SceneDev* __restrict__ scenes, PassCounters* ctr, PassStamp ps,
    int cta_min, int few) {
    __shared__ double stage[kZoneWarpBlock / 32][32][12];
    if (ctr->err & kErrRetry) return;
    if (*dnz < nzones) nzones = *dnz;
    const int warp_min = zone_warp_min(nzones, few);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    double(*st)[12] = stage[wib];
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    bool bad = false;
    for (int z = gw; z < nzones; z += nw) {
        const int i = zone_rng[z].x, end = zone_rng[z].y;
        if (end - i < warp_min || end - i >= cta_min) continue;
        const Params prm = scenes[vscene[members[i]]].p;
        const double m = prm.m, dt = prm.dt;
        const int num_pts = end - i;
        double x_cm[3], v_cm[3], L[3], I[3][3];
        double acc = 0.0;  // this lane's component of the current sum
        for (int c = i; c < end; c += 32) {
            const int q = c + lane;
            if (q < end) {
                const int p = members[q];
                double xs[3], vs[3];
                load3(xo, p, xs);
                load3(av, p, vs);
                for (int d = 0; d < 3; ++d) st[lane][d] = xs[d], st[lane][3 + d] = vs[d];
            }
            __syncwarp();
            if (lane < 6) {  // lane d sums component d over the members in list order
                const int k1 = end - c < 32 ? end - c : 32;
                for (int k = 0; k < k1; ++k) acc += st[k][lane];
            }
            __syncwarp();
        }
        for (int d = 0; d < 3; ++d) {
            x_cm[d] = __shfl_sync(0xffffffffu, acc / num_pts, d);
            v_cm[d] = __shfl_sync(0xffffffffu, acc / num_pts, 3 + d);
        }
        acc = 0.0;
        for (int c = i; c < end; c += 32) {
            const int q = c + lane;
            if (q < end) {
                const int p = members[q];
                double xs[3], vs[3], dx[3], dv[3], Li[3];
                load3(xo, p, xs);
                load3(av, p, vs);
                for (int d = 0; d < 3; ++d) { dx[d] = xs[d] - x_cm[d]; dv[d] = vs[d] - v_cm[d]; }
                cross3(dx, dv, Li);
                for (int d = 0; d < 3; ++d) st[lane][d] = m * Li[d];
                const double mag_dx = mag3(dx);
                for (int r = 0; r < 3; ++r)
                    for (int s = 0; s < 3; ++s) {
                        double t = -dx[r] * dx[s];
                        if (r == s) t += mag_dx * mag_dx;
                        st[lane][3 + 3 * r + s] = t * m;
                    }
            }
            __syncwarp();
            if (lane < 12) {  // lane c sums component c (L, then I row by row) in list order
                const int k1 = end - c < 32 ? end - c : 32;
                for (int k = 0; k < k1; ++k) acc = st[k][lane] + acc;
            }
            __syncwarp();
        }
        for (int d = 0; d < 3; ++d) L[d] = __shfl_sync(0xffffffffu, acc, d);
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) I[r][q] = __shfl_sync(0xffffffffu, acc, 3 + 3 * r + q);
        // every lane forms the same rotation (sin and cos on two lanes)
        double w[3];
        zone_omega(I, L, w);
        const double mag_w = mag3(w);
        double sn, cs;
        cr::sincos_warp(dt * mag_w, &sn, &cs);
        const double sw = mag_w < kRoundEps ? 0.0 : sn / mag_w;
        const double cw = cs;
        for (int q = i + lane; q < end; q += 32)
            bad |= zone_member_motion(members[q], fixed, xo, av, x_cm, v_cm, w, mag_w, sw, cw, dt, ps);
        __syncwarp();
    }
    if (bad) atomicOr(&ctr->err, kErrNan);
}

// Zones of at least cta_min members: one CTA per zone. The same sums
// as k_zone_solve_warp, in the same order - one thread per summed component
// adding the members in list order - but every member's terms and its
// final motion are computed by all the CTA's threads (a large zone is
// otherwise bound by one warp's share of the SM's FP64 pipe).
__global__ void __launch_bounds__(kZoneCtaThreads) k_zone_solve_cta(
    const int* __restrict__ members, const int2* __restrict__ zone_rng, int nzones, const int* __restrict__ dnz,
    const uint8_t* __restrict__ fixed, const double4_32a* __restrict__ xo, double4_32a* av,
    const int* __restrict__ vscene, const SceneDev* __restrict__ scenes, PassCounters* ctr, PassStamp ps,
    int cta_min) {
    __shared__ double st[kZoneCtaThreads][12];
    __shared__ double s_sum[12];
    __shared__ double s_rot[6];  // w, mag_w, sw, cw
    if (ctr->err & kErrRetry) return;
    if (*dnz < nzones) nzones = *dnz;
    const int tid = threadIdx.x;
    bool bad = false;
    for (int z = blockIdx.x; z < nzones; z += gridDim.x) {
        const int i = zone_rng[z].x, end = zone_rng[z].y;
        if (end - i < cta_min) continue;
        const Params prm = scenes[vscene[members[i]]].p;
        const double m = prm.m, dt = prm.dt;
        const int num_pts = end - i;
        double acc = 0.0;  // this thread's component of the current sum (threads 0..11)
        for (int c = i; c < end; c += kZoneCtaThreads) {
            const int q = c + tid;
            if (q < end) {
                const int p = members[q];
                double xs[3], vs[3];
                load3(xo, p, xs);
                load3(av, p, vs);
                for (int d = 0; d < 3; ++d) st[tid][d] = xs[d], st[tid][3 + d] = vs[d];
            }
            __syncthreads();
            if (tid < 6) {
                const int k1 = end - c < kZoneCtaThreads ? end - c : kZoneCtaThreads;
                for (int k = 0; k < k1; ++k) acc += st[k][tid];
            }
            __syncthreads();
        }
        if (tid < 6) s_sum[tid] = acc / num_pts;
        __syncthreads();
        double x_cm[3], v_cm[3];
        for (int d = 0; d < 3; ++d) x_cm[d] = s_sum[d], v_cm[d] = s_sum[3 + d];
        acc = 0.0;
        for (int c = i; c < end; c += kZoneCtaThreads) {
            const int q = c + tid;
            if (q < end) {
                const int p = members[q];
                double xs[3], vs[3], dx[3], dv[3], Li[3];
                load3(xo, p, xs);
                load3(av, p, vs);
                for (int d = 0; d < 3; ++d) { dx[d] = xs[d] - x_cm[d]; dv[d] = vs[d] - v_cm[d]; }
                cross3(dx, dv, Li);
                for (int d = 0; d < 3; ++d) st[tid][d] = m * Li[d];
                const double mag_dx = mag3(dx);
                for (int r = 0; r < 3; ++r)
                    for (int s2 = 0; s2 < 3; ++s2) {
                        double t = -dx[r] * dx[s2];
                        if (r == s2) t += mag_dx * mag_dx;
                        st[tid][3 + 3 * r + s2] = t * m;
                    }
            }
            __syncthreads();
            if (tid < 12) {
                const int k1 = end - c < kZoneCtaThreads ? end - c : kZoneCtaThreads;
                for (int k = 0; k < k1; ++k) acc = st[k][tid] + acc;
            }
            __syncthreads();
        }
        if (tid < 12) s_sum[tid] = acc;
        __syncthreads();
        if (tid < 32) {  // warp 0: the same rotation in every lane, sin and cos on two lanes
            double L[3], I[3][3], w[3];
            for (int d = 0; d < 3; ++d) L[d] = s_sum[d];
            for (int r = 0; r < 3; ++r)
                for (int q = 0; q < 3; ++q) I[r][q] = s_sum[3 + 3 * r + q];
            zone_omega(I, L, w);
            const double mag_w = mag3(w);
            double sn, cs;
            cr::sincos_warp(dt * mag_w, &sn, &cs);
            if (tid == 0) {
                for (int d = 0; d < 3; ++d) s_rot[d] = w[d];
                s_rot[3] = mag_w;
                s_rot[4] = mag_w < kRoundEps ? 0.0 : sn / mag_w;
                s_rot[5] = cs;
            }
        }
        __syncthreads();
        const double w[3] = {s_rot[0], s_rot[1], s_rot[2]};
        for (int q = i + tid; q < end; q += kZoneCtaThreads)
            bad |= zone_member_motion(members[q], fixed, xo, av, x_cm, v_cm, w, s_rot[3], s_rot[4], s_rot[5], dt, ps);
        __syncthreads();  // the next zone reuses the shared arrays
    }
    if (bad) atomicOr(&ctr->err, kErrNan);
}

// detectDomainBoundaryCollision (dcollid.cpp:116-158) then
// updateFinalPosition (dcollid.cpp:562-584) for one point. The reference
// revisits points shared by several elements; the clamp is idempotent, so
// once per point gives the same result.
__global__ void k_finalize(const uint8_t* __restrict__ in_elem, const double4_32a* __restrict__ xo, double4_32a* av,
                           uint8_t* has_collsn, const double* __restrict__ x_cand, double* x_out, int nv,
                           const int* __restrict__ vscene, const SceneDev* __restrict__ scenes,
                           const uint8_t* __restrict__ fixed, const uint8_t* __restrict__ mask) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv) return;
    if (mask && !mask[vscene[p]]) return;  // another scene set's end of step
    if (!in_elem[p]) {
        for (int j = 0; j < 3; ++j) x_out[3 * p + j] = x_cand[3 * p + j];
        return;
    }
    const SceneDev& sd = scenes[vscene[p]];
    if (!sd.enabled) {
        for (int j = 0; j < 3; ++j) x_out[3 * p + j] = x_cand[3 * p + j];
        return;
    }
    const Params prm = sd.p;
    double L[3] = {sd.lo[0], sd.lo[1], sd.lo[2]}, U[3] = {sd.hi[0], sd.hi[1], sd.hi[2]};
    double xs[3], v[3];
    load3(xo, p, xs);
    load3(av, p, v);
    double dt = prm.dt, mu = prm.lambda, dv = 0;
    if (fixed[p] & 2) {  // movable points skip the clamp (dcollid.cpp:123)
        for (int j = 0; j < 3; ++j) x_out[3 * p + j] = xs[j] + v[j] * dt;
        return;
    }
    for (int j = 0; j < 3; ++j) {
        double cand = xs[j] + dt * v[j];
        if (cand <= L[j]) {
            has_collsn[p] = 1;
            dv = fabs(v[j]);
            v[j] = 0.0;
        } else if (cand >= U[j]) {
            has_collsn[p] = 1;
            dv = fabs(v[j]);
            v[j] = 0.0;
        }
    }
    double preVt = mag3(v);
    if (preVt > kMachEps)
        for (int j = 0; j < 3; ++j) v[j] *= smax(1.0 - mu * dv / preVt, 0.0);
    av[p] = make_double4_32a(v[0], v[1], v[2], 0.0);
    for (int j = 0; j < 3; ++j) x_out[3 * p + j] = xs[j] + v[j] * dt;
}

// One edge's strain test, reduceSuperelastOnce (dcollid.cpp:496-539),
// evaluated as the reference does.
__device__ __forceinline__ bool strain_flag_exact(int p0, int p1, double len0, const double4_32a* xo,
                                                  const double4_32a* av, double dt) {
    double x0[3], x1[3], v0[3], v1[3], c0[3], c1[3];
    load3(xo, p0, x0);
    load3(xo, p1, x1);
    load3(av, p0, v0);
    load3(av, p1, v1);
    for (int k = 0; k < 3; ++k) {
        c0[k] = x0[k] + dt * v0[k];
        c1[k] = x1[k] + dt * v1[k];
    }
    double sn = 0.0, so = 0.0;
    for (int k = 0; k < 3; ++k) sn += sqr(c0[k] - c1[k]);
    for (int k = 0; k < 3; ++k) so += sqr(x0[k] - x1[k]);
    double len_new = sqrt(sn), len_old = sqrt(so);
    if (len_old > kRoundEps && len_new > kRoundEps) {
        double strain_rate = (len_new - len_old) / len_old;
        double strain = (len_new - len0) / len0;
        return fabs(strain) > kStrainTol || fabs(strain_rate) > kStrainTol;
    }
    return true;
}

// Squared-length bounds that decide |(sqrt(s) - L)/L| > 0.1 without the
// square root and the division: outside [lo_no, hi_no] the answer is "over",
// inside [lo_def, hi_def] ... see strain_quick. The bounds sit 1e-9 (relative)
// inside and outside the exact thresholds L*(1 -+ 0.1); the reference's own
// rounding of sqrt, subtraction and division is below 1e-15, so a decision
// taken here equals the reference's.
struct StrainBounds {
    double hi_def, hi_no, lo_no, lo_def;
};
__device__ __forceinline__ StrainBounds strain_bounds(double L) {
    StrainBounds b;
    double a = L * (1.1 * (1.0 + 1e-9)), c = L * (1.1 * (1.0 - 1e-9));
    double d = L * (0.9 * (1.0 + 1e-9)), e = L * (0.9 * (1.0 - 1e-9));
    b.hi_def = a * a;  // s above: over-stretched for sure
    b.hi_no = c * c;   // s below (and above lo_no): not over-stretched
    b.lo_no = d * d;
    b.lo_def = e * e;  // s below: over-compressed for sure
    return b;
}
// The same bounds from the squared length L2 = L*L, without the square root:
// each differs from the one above by a few ulps, far inside the 1e-9 margin.
__device__ __forceinline__ StrainBounds strain_bounds_sq(double L2) {
    const double ka = (1.1 * (1.0 + 1e-9)) * (1.1 * (1.0 + 1e-9)), kc = (1.1 * (1.0 - 1e-9)) * (1.1 * (1.0 - 1e-9));
    const double kd = (0.9 * (1.0 + 1e-9)) * (0.9 * (1.0 + 1e-9)), ke = (0.9 * (1.0 - 1e-9)) * (0.9 * (1.0 - 1e-9));
    StrainBounds b;
    b.hi_def = L2 * ka;
    b.hi_no = L2 * kc;
    b.lo_no = L2 * kd;
    b.lo_def = L2 * ke;
    return b;
}
// 1: over the limit, 0: within it, -1: too close to tell without the exact test.
__device__ __forceinline__ int strain_quick(double s, const StrainBounds& b) {
    if (s > b.hi_def || s < b.lo_def) return 1;
    if (s < b.hi_no && s > b.lo_no) return 0;
    return -1;
}

struct __align__(16) StrainEdgeStep {
    int p0, p1;
    double len0;
    StrainBounds rest;  // from the rest length
    StrainBounds prev;  // from the start-of-step length (strain rate)
    double x0[3], x1[3];  // x_old of both points (constant through the sweep)
    int exact_only;       // degenerate lengths: always take the exact test
    int s0, s1;           // shared-memory slots of both points (window sweep)
    int pad;
    // FP32 view for the window sweep's first decision: x_old(p0) - x_old(p1)
    // and the four squared-length bounds rounded outward (see k_strain_window)
    float dx[3];
    float over_hi, under_hi, under_lo, over_lo;
    float pad2[2];
};

// The part of an edge record the window sweep reads for every edge: the
// slots, x_old(p0) - x_old(p1) and the four bounds in FP32 (48 bytes).
struct __align__(16) StrainEdgeHot {
    int s0, s1;
    float dx[3];
    float over_hi, under_hi, under_lo, over_lo;
    int pad[3];
};

// Per-step set-up of the strain sweep: the start-of-step length of every
// edge (x_old does not change during the sweep) and both sets of bounds.
// An edge's full record for the step, from its endpoints' x_old: the
// exact test's inputs and the FP32 view of the window sweep.
__device__ __forceinline__ StrainEdgeStep strain_step(const StrainEdge& ed, const double4_32a* __restrict__ xo) {
    double x0[3], x1[3];
    load3(xo, ed.p0, x0);
    load3(xo, ed.p1, x1);
    double so = 0.0;
    for (int k = 0; k < 3; ++k) so += sqr(x0[k] - x1[k]);
    StrainEdgeStep r;
    r.p0 = ed.p0;
    r.p1 = ed.p1;
    r.len0 = ed.len0;
    r.rest = strain_bounds(ed.len0);
    r.prev = strain_bounds_sq(so);
    for (int k = 0; k < 3; ++k) {
        r.x0[k] = x0[k];
        r.x1[k] = x1[k];
    }
    // tiny or non-positive lengths: leave every decision to the exact test
    r.exact_only = !(so > 1e-12 && ed.len0 > 1e-6);
    r.s0 = ed.s0;
    r.s1 = ed.s1;
    r.pad = 0;
    for (int k = 0; k < 3; ++k) r.dx[k] = (float)(x0[k] - x1[k]);
    // strain flags when s > hi_def (either bound) or s < lo_def; it is clear
    // when lo_no < s < hi_no for both; FP32 thresholds rounded outward
    double hdef = fmin(r.rest.hi_def, r.prev.hi_def), ldef = fmax(r.rest.lo_def, r.prev.lo_def);
    double hno = fmin(r.rest.hi_no, r.prev.hi_no), lno = fmax(r.rest.lo_no, r.prev.lo_no);
    r.over_hi = __double2float_ru(hdef);
    r.over_lo = __double2float_rd(ldef);
    r.under_hi = __double2float_rd(hno);
    r.under_lo = __double2float_ru(lno);
    r.pad2[0] = r.pad2[1] = 0.f;
    return r;
}

// Per step: every edge's 48-byte hot record; the full record only for the
// edges of scenes swept by k_strain (too many slots for shared memory) - the
// shared-memory sweeps rebuild it for their rare exact tests.
__global__ void k_strain_setup(const StrainEdge* __restrict__ edges, int m, const double4_32a* __restrict__ xo,
                               StrainEdgeStep* out, StrainEdgeHot* hot, const int* __restrict__ vscene,
                               const SceneDev* __restrict__ scenes, int slot_cap) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const StrainEdge ed = edges[e];
    const StrainEdgeStep r = strain_step(ed, xo);
    if (slot_cap < 0 || scenes[vscene[ed.p0]].strain_slots > slot_cap) out[e] = r;
    StrainEdgeHot hh;
    hh.s0 = r.s0;
    hh.s1 = r.s1;
    for (int k = 0; k < 3; ++k) hh.dx[k] = r.dx[k];
    hh.over_hi = r.over_hi;
    hh.under_hi = r.under_hi;
    hh.under_lo = r.under_lo;
    hh.over_lo = r.over_lo;
    hh.pad[0] = hh.pad[1] = hh.pad[2] = 0;
    hot[e] = hh;
}

// The strain decision for given end velocities v0, v1 (bounds first, the
// exact test of dcollid.cpp:525-530 only inside the bounds' margin).
__device__ __forceinline__ bool strain_flag_vals(const StrainEdgeStep& ed, const double* v0, const double* v1,
                                                 double dt, int* n_exact) {
    double c0[3], c1[3];
    for (int k = 0; k < 3; ++k) {
        c0[k] = ed.x0[k] + dt * v0[k];
        c1[k] = ed.x1[k] + dt * v1[k];
    }
    double sn = 0.0;
    for (int k = 0; k < 3; ++k) sn += sqr(c0[k] - c1[k]);
    if (!ed.exact_only && sn > 1e-18) {
        int q0 = strain_quick(sn, ed.rest), q1 = strain_quick(sn, ed.prev);
        if (q0 == 1 || q1 == 1) return true;
        if (q0 == 0 && q1 == 0) return false;
    }
    ++*n_exact;
    double so = 0.0;
    for (int k = 0; k < 3; ++k) so += sqr(ed.x0[k] - ed.x1[k]);
    double len_new = sqrt(sn), len_old = sqrt(so);
    if (len_old > kRoundEps && len_new > kRoundEps) {
        double strain_rate = (len_new - len_old) / len_old;
        double strain = (len_new - ed.len0) / ed.len0;
        return fabs(strain) > kStrainTol || fabs(strain_rate) > kStrainTol;
    }
    return true;
}

// 0.5 * x, the averaging of the strain sweep: one less in the exponent field
// (in the high 32 bits) when that field is 2..2046, where the halving is
// exact; x itself for +-0; the FP64 multiply otherwise. GB300 issues a
// warp's FP64 multiply in ~64 cycles whatever its active lanes, and the
// averaging lies on the sweep's per-level critical path; these are a few
// 32-bit integer instructions with the same result.
__device__ __forceinline__ double half_of(double x) {
    const int hi = __double2hiint(x), lo = __double2loint(x);
    const unsigned e = ((unsigned)hi >> 20) & 0x7ffu;
    if (e - 2u < 0x7fdu) return __hiloint2double(hi - 0x00100000, lo);
    if ((((unsigned)hi << 1) | (unsigned)lo) == 0u) return x;
    return 0.5 * x;
}

// reduceSuperelast, dcollid.cpp:586-596: up to 10 Gauss-Seidel passes over
// the edges in element order, each averaging the two end velocities of an
// over-strained edge before the next edge is tested (one pass per launch). The edges arrive sorted
// by dependency level (an edge's level is one more than the level of the
// last earlier edge at either of its points), so the edges of one level share
// no point and see exactly the values the sequential sweep gives them: the
// level-by-level walk below is the reference's sweep, reordered only where
// the order cannot matter.
// Per scene and step, flags[2s] ("some edge would average": set by
// k_strain_check) and flags[2s+1] (the sweep is over); passes_out[3s ..] the
// sweeps run, edges averaged, exact tests. One launch is one pass: a scene
// whose check found nothing to average is done - its sweep would change
// nothing, which is how the reference's loop ends (dcollid.cpp:588-595) -
// and counts that sweep; otherwise it sweeps once.
__device__ __forceinline__ bool sweep_gate(int pass, int s, int* flags, int* passes_out_all) {
    __shared__ int s_go;
    if (threadIdx.x == 0) {
        int go = 0;
        if (!flags[2 * s + 1]) {
            if (!flags[2 * s]) {
                flags[2 * s + 1] = 1;
                passes_out_all[3 * s] = pass + 1;
            } else {
                flags[2 * s] = 0;
                go = 1;
            }
        }
        s_go = go;
    }
    __syncthreads();
    return s_go != 0;
}

__device__ __forceinline__ void sweep_done(int pass, int s, int n_avg, int n_exact, int* flags, int* passes_out_all) {
    __shared__ int s_avg, s_exact;
    if (threadIdx.x == 0) s_avg = s_exact = 0;
    __syncthreads();
    atomicAdd(&s_avg, n_avg);
    atomicAdd(&s_exact, n_exact);
    __syncthreads();
    if (threadIdx.x == 0) {
        passes_out_all[3 * s] = pass + 1;
        passes_out_all[3 * s + 1] += s_avg;
        passes_out_all[3 * s + 2] += s_exact;
        if (pass + 1 >= kStrainMaxIter) flags[2 * s + 1] = 1;
    }
}

__global__ void __launch_bounds__(256) k_strain(const StrainEdgeStep* __restrict__ edges,
                                                const int4* __restrict__ hdr_all,
                                                const SceneDev* __restrict__ scenes, int slot_cap,
                                                double4_32a* av, int pass, int* flags, int* passes_out_all,
                                                const int* __restrict__ order) {
    const int sc = order[blockIdx.x];
    const SceneDev& sd = scenes[sc];
    if ((slot_cap >= 0 && sd.strain_slots <= slot_cap) || !sd.enabled) return;  // k_strain_window's, or left out
    if (!sweep_gate(pass, sc, flags, passes_out_all)) return;
    const int4* hdr = hdr_all + 2 * sd.strain_hdr0;
    const int nlevels = sd.strain_levels;
    const double dt = sd.p.dt;
    int n_avg = 0, n_exact = 0;
    // the records of the next level are loaded before the barrier that ends
    // the current one: they do not depend on the velocities
    int e = 0, e1 = 0;
    if (nlevels > 0) {
        int4 h = hdr[0];
        e = h.x + threadIdx.x;
        e1 = h.y;
    }
    StrainEdgeStep cur;
    bool have = e < e1;
    if (have) cur = edges[e];
    for (int l = 0; l < nlevels; ++l) {
        int ne = 0, ne1 = 0;
        if (l + 1 < nlevels) {
            int4 h = hdr[2 * (l + 1)];
            ne = h.x + threadIdx.x;
            ne1 = h.y;
        }
        bool nhave = ne < ne1;
        StrainEdgeStep nxt;
        if (nhave) nxt = edges[ne];
        while (have) {
            double4_32a a0 = av[cur.p0], a1 = av[cur.p1];
            double v0[3] = {a0.x, a0.y, a0.z}, v1[3] = {a1.x, a1.y, a1.z};
            if (strain_flag_vals(cur, v0, v1, dt, &n_exact)) {
                ++n_avg;
                double t0 = a0.x + a1.x, t1 = a0.y + a1.y, t2 = a0.z + a1.z;
                t0 = half_of(t0); t1 = half_of(t1); t2 = half_of(t2);
                double4_32a nv4 = make_double4_32a(t0, t1, t2, 0.0);
                av[cur.p0] = nv4;
                av[cur.p1] = nv4;
            }
            e += blockDim.x;
            have = e < e1;
            if (have) cur = edges[e];
        }
        __syncthreads();
        e = ne;
        e1 = ne1;
        have = nhave;
        cur = nxt;
    }
    sweep_done(pass, sc, n_avg, n_exact, flags, passes_out_all);
}

// The same sweep with each point's velocity in shared memory while the
// sweep uses it. Levels advance along the mesh like a wavefront, so a point
// is live for only a few levels: at assembly every point gets a shared-memory
// slot for its live interval (interval colouring; 418 slots for a 129x129
// cloth). Its velocity is copied in with cp.async kWindowAhead levels before
// its first edge and written back the level after its last one.
//
// FP64 runs at a small fraction of the FP32 rate on this GPU and the sweep
// runs on one SM, so each slot also keeps an FP32 copy of the velocity and
// an edge is first decided in FP32: s32 = |dx + dt (v0 - v1)|^2 from the
// FP32 copies carries an error below 32 * 2^-24 * bnd^2 (bnd: sum of the
// magnitudes entering it), and only when s32 +- that error straddles one of
// the outward-rounded bounds does the FP64 decision (bounds, then the exact
// test) run. The averaging itself is FP64, as in the reference.
constexpr int kWindowAhead = 8;
static_assert(kWindowAhead == kStrainAhead, "copy-ins are scheduled for the sweep's look-ahead");
// dynamic shared memory of one sweep CTA at most: with the kernel's 2 KB of
// static shared memory, within the 227 KB a CTA may hold (3,584 slots; a
// 1025x1025 cloth needs 3,330)
constexpr size_t kStrainWindowBytes = 224 * 1024;
constexpr size_t kStrainWarpBytes = 200 * 1024;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}

// slot layout: [x y] [z -] as double2, then [x y z -] as float4
struct WinSlot {
    double2 a, b;
    float4 f;
    float4 pad;
};

__device__ __forceinline__ int strain_decide32(const StrainEdgeHot& ed, float4 f0, float4 f1, float dt32) {
    float u[3], bnd = 0.f;
    float v0[3] = {f0.x, f0.y, f0.z}, v1[3] = {f1.x, f1.y, f1.z};
    float s32 = 0.f;
    for (int k = 0; k < 3; ++k) {
        float dv = __fsub_rn(v0[k], v1[k]);
        u[k] = __fadd_rn(ed.dx[k], __fmul_rn(dt32, dv));
        bnd = __fadd_ru(bnd, __fadd_ru(fabsf(ed.dx[k]), __fmul_ru(dt32, __fadd_ru(fabsf(v0[k]), fabsf(v1[k])))));
        s32 = __fadd_rn(s32, __fmul_rn(u[k], u[k]));
    }
    float err = __fmul_ru(__fmul_ru(bnd, bnd), 32.0f * 5.9604645e-8f);
    float lo = __fsub_rd(s32, err), hi = __fadd_ru(s32, err);
    if (lo > ed.over_hi || hi < ed.over_lo) return 1;
    if (hi < ed.under_hi && lo > ed.under_lo) return 0;
    return -1;
}

__device__ __forceinline__ void strain_window_edge(const StrainEdgeHot& h, int e,
                                                   const StrainEdge* __restrict__ edges,
                                                   const double4_32a* __restrict__ xo, WinSlot* s_win,
                                                   float dt32, double dt, int* n_avg, int* n_exact, bool* has) {
    WinSlot& w0 = s_win[h.s0];
    WinSlot& w1 = s_win[h.s1];
    int q = strain_decide32(h, w0.f, w1.f, dt32);
    if (q == 0) return;
    double2 a0 = w0.a, a1 = w0.b, b0 = w1.a, b1 = w1.b;
    double v0[3] = {a0.x, a0.y, a1.x}, v1[3] = {b0.x, b0.y, b1.x};
    if (q < 0) {
        const StrainEdgeStep full = strain_step(edges[e], xo);
        if (!strain_flag_vals(full, v0, v1, dt, n_exact)) return;
    }
    ++*n_avg;
    double t[3];
    for (int k = 0; k < 3; ++k) {
        t[k] = v0[k] + v1[k];
        t[k] = half_of(t[k]);
    }
    double2 na = make_double2(t[0], t[1]), nb = make_double2(t[2], 0.0);
    float4 nf = make_float4((float)t[0], (float)t[1], (float)t[2], 0.f);
    w0.a = na; w0.b = nb; w0.f = nf;
    w1.a = na; w1.b = nb; w1.f = nf;
    *has = true;
}

// Everything a thread needs for a level arrives kRing levels early in a
// register ring: the level's ranges, and the thread's first edge record,
// copy-in entry and write-back entry. Entries beyond the first per thread
// (levels wider than the block) are read when needed. The level loop is
// unrolled by kWindowAhead (a multiple of kRing) so that every ring slot has
// a fixed register name and nothing is shifted from level to level.
constexpr int kRing = 4;

struct WinRing {
    int4 h0[kRing], h1[kRing];
    StrainEdgeHot hot[kRing];
    int2 ld[kRing], wb[kRing];
    int lslot[kWindowAhead];  // slot this thread copied in, per recent level (-1: none)
};

// The level headers come from a shared-memory ring of kHdrRing levels,
// filled kHdrAhead levels ahead with cp.async, so that the record loads that
// depend on a header are issued without waiting on a global load.
constexpr int kHdrRing = 64;
constexpr int kHdrChunk = 16;                  // levels per refill, issued at levels l = 0 mod kHdrChunk
constexpr int kHdrAhead = kHdrRing - kHdrChunk;  // a refill at level l brings levels [l + kHdrAhead, l + kHdrRing)

// tid: this thread's edge of the level; tc, tw: its copy-in and write-back
// (negative: none first-hand)
__device__ __forceinline__ void win_fetch(WinRing& r, int j, int lk, int nlevels, int tid, int tc, int tw,
                                          const int4* s_hdr, const StrainEdgeHot* __restrict__ hot,
                                          const int2* __restrict__ load_list, const int2* __restrict__ wb_list) {
    if (lk < nlevels) {
        const int q = 2 * (lk % kHdrRing);
        int4 a = s_hdr[q], b = s_hdr[q + 1];
        r.h0[j] = a;
        r.h1[j] = b;
        if (a.x + tid < a.y) r.hot[j] = hot[a.x + tid];
        if (tc >= 0 && a.z + tc < a.w) r.ld[j] = load_list[a.z + tc];
        if (tw >= 0 && b.x + tw < b.y) r.wb[j] = wb_list[b.x + tw];
    }
}

struct WinArgs {
    const StrainEdge* edges;
    const double4_32a* xo;
    const StrainEdgeHot* hot;
    const int4* hdr;
    int4* s_hdr;  // the header ring
    int nlevels;
    const int2* load_list;
    const int2* wb_list;
    double4_32a* av;
    double dt;
    float dt32;
    int multi_ld;  // some level has more copy-ins than the block has threads
    // first thread of the copy-in and write-back roles; both 0 when every
    // thread takes all three roles (edge, copy-in, write-back number tid)
    int cbase, wbase;
};

// A thread's second and third edge records of the next level, for levels
// wider than the block (WIDE sweeps): loaded a level early, so that they do
// not wait on a global load inside their level.
struct WideNext {
    StrainEdgeHot x1, x2;
};
__device__ __forceinline__ void wide_fetch(WideNext& w, const int4& h, const StrainEdgeHot* __restrict__ hot,
                                           int tid) {
    const int e1 = h.x + tid + (int)blockDim.x, e2 = e1 + (int)blockDim.x;
    if (e1 < h.y) w.x1 = hot[e1];
    if (e2 < h.y) w.x2 = hot[e2];
}

// One level of the window sweep; J = level mod kWindowAhead.
template <int J, bool WIDE>
__device__ __forceinline__ void win_level(const WinArgs& A, WinRing& r, WideNext& wn, WinSlot* s_win, int l, int tid,
                                          int* n_avg, int* n_exact, bool* has) {
    constexpr int R = J % kRing;
    const int4 h0 = r.h0[R], h1 = r.h1[R];
    const StrainEdgeHot cur = r.hot[R];
    const int2 ld = r.ld[R], wb = r.wb[R];
    const int tc = tid - A.cbase, tw = tid - A.wbase;
    StrainEdgeHot c1, c2;
    if (WIDE) {
        c1 = wn.x1;
        c2 = wn.x2;
        if (l + 1 < A.nlevels) wide_fetch(wn, r.h0[(J + 1) % kRing], A.hot, tid);
    }
    win_fetch(r, R, l + kRing, A.nlevels, tid, tc, tw, A.s_hdr, A.hot, A.load_list, A.wb_list);
    if (J % kHdrChunk == 0 && l % kHdrChunk == 0 && l > 0) {
        // headers of levels [l + kHdrAhead, l + kHdrRing) into the slots of
        // levels [l - kHdrChunk, l), whose records were fetched kRing levels
        // early and a barrier ago; they land in this level's copy group
        const int m = l + kHdrAhead + (tid >> 1);
        if (tid < 2 * kHdrChunk && m < A.nlevels)
            cp_async16(&A.s_hdr[2 * (m % kHdrRing) + (tid & 1)], &A.hdr[2 * m + (tid & 1)]);
    }
    // copy in the points whose slot opens now
    int my_slot = -1;
    if (tc >= 0 && h0.z + tc < h0.w) {
        my_slot = ld.y;
        cp_async16(&s_win[ld.y].a, &A.av[ld.x]);
        cp_async16(&s_win[ld.y].b, reinterpret_cast<const double2*>(&A.av[ld.x]) + 1);
        for (int i = h0.z + tc + (int)blockDim.x; i < h0.w; i += blockDim.x) {
            int2 ps = A.load_list[i];
            cp_async16(&s_win[ps.y].a, &A.av[ps.x]);
            cp_async16(&s_win[ps.y].b, reinterpret_cast<const double2*>(&A.av[ps.x]) + 1);
        }
    }
    asm volatile("cp.async.commit_group;\n" ::);
    // FP32 copies of the points whose copy has now landed (each by the thread
    // that issued it): all of level 0's at once, then those issued
    // kWindowAhead levels ago, before their first edge
    const int old_slot = r.lslot[J];
    r.lslot[J] = my_slot;
    int cl = -1, cslot = -1;
    if (l == 0) {
        asm volatile("cp.async.wait_group 0;\n" ::);
        cl = 0;
        cslot = my_slot;
    } else if (l < kWindowAhead) {
        asm volatile("cp.async.wait_group 0;\n" ::);
    } else {
        asm volatile("cp.async.wait_group %0;\n" ::"n"(kWindowAhead));
        if (l - kWindowAhead >= 1) {
            cl = l - kWindowAhead;
            cslot = old_slot;
        }
    }
    if (cl >= 0 && cslot >= 0) {
        WinSlot& w = s_win[cslot];
        w.f = make_float4((float)w.a.x, (float)w.a.y, (float)w.b.x, 0.f);
        if (A.multi_ld) {  // the copy-ins past the first per thread (a dependent load: only when needed)
            int4 hc = A.hdr[2 * cl];
            for (int i = hc.z + tc + (int)blockDim.x; i < hc.w; i += blockDim.x) {
                WinSlot& w2 = s_win[A.load_list[i].y];
                w2.f = make_float4((float)w2.a.x, (float)w2.a.y, (float)w2.b.x, 0.f);
            }
        }
    }
    __syncthreads();
    // write back the points last used at the previous level
    if (tw >= 0 && h1.x + tw < h1.y) {
        double2 a = s_win[wb.y].a, b = s_win[wb.y].b;
        A.av[wb.x] = make_double4_32a(a.x, a.y, b.x, 0.0);
        for (int i = h1.x + tw + (int)blockDim.x; i < h1.y; i += blockDim.x) {
            int2 ps = A.wb_list[i];
            double2 a2 = s_win[ps.y].a, b2 = s_win[ps.y].b;
            A.av[ps.x] = make_double4_32a(a2.x, a2.y, b2.x, 0.0);
        }
    }
    const int bd = (int)blockDim.x;
    int e = h0.x + tid;
    if (e < h0.y) {
        strain_window_edge(cur, e, A.edges, A.xo, s_win, A.dt32, A.dt, n_avg, n_exact, has);
        if (WIDE) {
            if (e + bd < h0.y) strain_window_edge(c1, e + bd, A.edges, A.xo, s_win, A.dt32, A.dt, n_avg, n_exact, has);
            if (e + 2 * bd < h0.y)
                strain_window_edge(c2, e + 2 * bd, A.edges, A.xo, s_win, A.dt32, A.dt, n_avg, n_exact, has);
            e += 2 * bd;
        }
        for (e += bd; e < h0.y; e += bd)
            strain_window_edge(A.hot[e], e, A.edges, A.xo, s_win, A.dt32, A.dt, n_avg, n_exact, has);
    }
}

// WIDE: levels up to three times the block's width take their second and
// third edges from registers loaded a level early (WideNext).
template <bool WIDE>
__global__ void __launch_bounds__(256) k_strain_window(const StrainEdge* __restrict__ edges,
                                                       const double4_32a* __restrict__ xo,
                                                       const StrainEdgeHot* __restrict__ hot,
                                                       const int4* __restrict__ hdr_all,
                                                       const SceneDev* __restrict__ scenes, int slot_cap,
                                                       const int2* __restrict__ load_list,
                                                       const int2* __restrict__ wb_list,
                                                       double4_32a* av, int pass, int* flags,
                                                       int* passes_out_all, int multi_ld,
                                                       const int* __restrict__ order, int cbase, int wbase) {
    extern __shared__ WinSlot s_win[];
    const int sc = order[blockIdx.x];
    const SceneDev& sd = scenes[sc];
    if (sd.strain_slots > slot_cap || !sd.enabled) return;  // k_strain's, or left out
    if (!sweep_gate(pass, sc, flags, passes_out_all)) return;
    const int4* hdr = hdr_all + 2 * sd.strain_hdr0;
    const int nlevels = sd.strain_levels;
    const int2 wb_final = make_int2(sd.wb_final0, sd.wb_final1);
    const double dt = sd.p.dt;
    const int tid = threadIdx.x;
    __shared__ int4 s_hdr[2 * kHdrRing];
    for (int i = tid; i < 2 * kHdrRing && i < 2 * nlevels; i += blockDim.x) s_hdr[i] = hdr[i];
    __syncthreads();
    WinArgs A{edges, xo, hot, hdr, s_hdr, nlevels, load_list, wb_list, av, dt, __double2float_ru(dt), multi_ld,
              cbase, wbase};
    int n_avg = 0, n_exact = 0;
    bool has = false;
    WinRing r;
#pragma unroll
    for (int j = 0; j < kWindowAhead; ++j) r.lslot[j] = -1;
#pragma unroll
    for (int j = 0; j < kRing; ++j)
        win_fetch(r, j, j, nlevels, tid, tid - cbase, tid - wbase, s_hdr, hot, load_list, wb_list);
    WideNext wn;
    if (WIDE && nlevels > 0) wide_fetch(wn, r.h0[0], hot, tid);
    for (int lb = 0; lb < nlevels; lb += kWindowAhead) {
        win_level<0, WIDE>(A, r, wn, s_win, lb + 0, tid, &n_avg, &n_exact, &has);
        if (lb + 1 < nlevels) win_level<1, WIDE>(A, r, wn, s_win, lb + 1, tid, &n_avg, &n_exact, &has);
        if (lb + 2 < nlevels) win_level<2, WIDE>(A, r, wn, s_win, lb + 2, tid, &n_avg, &n_exact, &has);
        if (lb + 3 < nlevels) win_level<3, WIDE>(A, r, wn, s_win, lb + 3, tid, &n_avg, &n_exact, &has);
        if (lb + 4 < nlevels) win_level<4, WIDE>(A, r, wn, s_win, lb + 4, tid, &n_avg, &n_exact, &has);
        if (lb + 5 < nlevels) win_level<5, WIDE>(A, r, wn, s_win, lb + 5, tid, &n_avg, &n_exact, &has);
        if (lb + 6 < nlevels) win_level<6, WIDE>(A, r, wn, s_win, lb + 6, tid, &n_avg, &n_exact, &has);
        if (lb + 7 < nlevels) win_level<7, WIDE>(A, r, wn, s_win, lb + 7, tid, &n_avg, &n_exact, &has);
    }
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncthreads();
    for (int i = wb_final.x + tid; i < wb_final.y; i += blockDim.x) {
        int2 ps = wb_list[i];
        double2 a = s_win[ps.y].a, b = s_win[ps.y].b;
        av[ps.x] = make_double4_32a(a.x, a.y, b.x, 0.0);
    }
    sweep_done(pass, sc, n_avg, n_exact, flags, passes_out_all);
}

// The sweep of one scene by a single warp. The block barrier of
// k_strain_window costs most of a level there; here a level needs only
// __syncwarp. Each level's edge records and its copy-in and write-back
// lists are staged into a shared-memory ring kWarpAhead levels ahead with
// cp.async, and velocities are copied into their slots (the same interval
// schedule) kWindowAhead levels before their first edge, so a level touches
// only shared memory. Slots hold the FP64 velocities; the FP32 values of the
// first decision are converted from them as needed.
constexpr int kWarpAhead = kWindowAhead;   // the copy-in distance of the schedule
constexpr int kWarpRing = kWarpAhead + 1;  // level L+K goes where level L-1 was

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem));
}

struct WarpSlot {
    double2 a, b;  // x y | z -
};

__global__ void __launch_bounds__(32) k_strain_warp(const StrainEdge* __restrict__ edges,
                                                    const double4_32a* __restrict__ xo,
                                                    const StrainEdgeHot* __restrict__ hot,
                                                    const int4* __restrict__ hdr_all,
                                                    const SceneDev* __restrict__ scenes, int slot_cap,
                                                    const int2* __restrict__ load_list,
                                                    const int2* __restrict__ wb_list, double4_32a* av, int pass,
                                                    int* flags, int* passes_out_all, int max_slots, int ecap,
                                                    int lcap, int wcap, const int* __restrict__ order) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int sc = order[blockIdx.x];
    const SceneDev& sd = scenes[sc];
    if (sd.strain_slots > slot_cap || !sd.enabled) return;  // k_strain's, or left out
    if (!sweep_gate(pass, sc, flags, passes_out_all)) return;
    WarpSlot* s_win = reinterpret_cast<WarpSlot*>(smem_raw);
    size_t off = (size_t)max_slots * sizeof(WarpSlot);
    StrainEdgeHot* s_hot = reinterpret_cast<StrainEdgeHot*>(smem_raw + off);
    off += (size_t)kWarpRing * ecap * sizeof(StrainEdgeHot);
    int2* s_ld = reinterpret_cast<int2*>(smem_raw + off);
    off += (size_t)kWarpRing * lcap * 8;
    int2* s_wb = reinterpret_cast<int2*>(smem_raw + off);
    off += (size_t)kWarpRing * wcap * 8;
    off = (off + 15) & ~(size_t)15;  // the headers are int4
    int4* s_h = reinterpret_cast<int4*>(smem_raw + off);
    const int lane = threadIdx.x;
    const int4* hdr = hdr_all + 2 * sd.strain_hdr0;
    const int nlevels = sd.strain_levels;
    const double dt = sd.p.dt;
    const float dt32 = __double2float_ru(dt);
    // level L's records and lists into ring slot L % kWarpRing
    auto stage = [&](int L) {
        if (L >= nlevels) return;
        const int r = L % kWarpRing;
        const int4 h0 = hdr[2 * L], h1 = hdr[2 * L + 1];
        if (lane == 0) {
            s_h[2 * r] = h0;
            s_h[2 * r + 1] = h1;
        }
        const float4* src = reinterpret_cast<const float4*>(hot + h0.x);
        float4* dst = reinterpret_cast<float4*>(s_hot + (size_t)r * ecap);
        const int nchunk = 3 * (h0.y - h0.x);  // 48-byte records, three 16-byte chunks each
        for (int c = lane; c < nchunk; c += 32) cp_async16(dst + c, src + c);
        for (int c = lane; c < h0.w - h0.z; c += 32) cp_async8(s_ld + (size_t)r * lcap + c, load_list + h0.z + c);
        for (int c = lane; c < h1.y - h1.x; c += 32) cp_async8(s_wb + (size_t)r * wcap + c, wb_list + h1.x + c);
    };
    for (int L = 0; L < kWarpAhead; ++L) {
        stage(L);
        asm volatile("cp.async.commit_group;\n" ::);
    }
    int n_avg = 0, n_exact = 0;
    for (int L = 0; L < nlevels; ++L) {
        // level L's stage: the (L+1)-th group committed
        if (L < kWarpAhead)
            asm volatile("cp.async.wait_group 0;\n" ::);
        else
            asm volatile("cp.async.wait_group %0;\n" ::"n"(kWarpAhead - 1));
        __syncwarp();
        const int r = L % kWarpRing;
        const int4 h0 = s_h[2 * r], h1 = s_h[2 * r + 1];
        // velocities whose slots open now (first used kWindowAhead levels on)
        for (int c = lane; c < h0.w - h0.z; c += 32) {
            const int2 ps = s_ld[(size_t)r * lcap + c];
            cp_async16(&s_win[ps.y].a, &av[ps.x]);
            cp_async16(&s_win[ps.y].b, reinterpret_cast<const double2*>(&av[ps.x]) + 1);
        }
        stage(L + kWarpAhead);
        asm volatile("cp.async.commit_group;\n" ::);
        if (L < kWarpAhead) asm volatile("cp.async.wait_group 0;\n" ::);  // first levels use them at once
        __syncwarp();
        // write back the points last used at the previous level
        for (int c = lane; c < h1.y - h1.x; c += 32) {
            const int2 ps = s_wb[(size_t)r * wcap + c];
            const double2 a = s_win[ps.y].a, b = s_win[ps.y].b;
            av[ps.x] = make_double4_32a(a.x, a.y, b.x, 0.0);
        }
        for (int i = lane; i < h0.y - h0.x; i += 32) {
            const StrainEdgeHot h = s_hot[(size_t)r * ecap + i];
            WarpSlot& w0 = s_win[h.s0];
            WarpSlot& w1 = s_win[h.s1];
            const double2 a0 = w0.a, a1 = w0.b, b0 = w1.a, b1 = w1.b;
            int q = strain_decide32(h, make_float4((float)a0.x, (float)a0.y, (float)a1.x, 0.f),
                                    make_float4((float)b0.x, (float)b0.y, (float)b1.x, 0.f), dt32);
            if (q == 0) continue;
            double v0[3] = {a0.x, a0.y, a1.x}, v1[3] = {b0.x, b0.y, b1.x};
            if (q < 0 && !strain_flag_vals(strain_step(edges[h0.x + i], xo), v0, v1, dt, &n_exact)) continue;
            ++n_avg;
            double t[3];
            for (int k = 0; k < 3; ++k) {
                t[k] = v0[k] + v1[k];
                t[k] = half_of(t[k]);
            }
            const double2 na = make_double2(t[0], t[1]), nb = make_double2(t[2], 0.0);
            w0.a = na; w0.b = nb;
            w1.a = na; w1.b = nb;
        }
        __syncwarp();
    }
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncwarp();
    for (int i = sd.wb_final0 + lane; i < sd.wb_final1; i += 32) {
        const int2 ps = wb_list[i];
        const double2 a = s_win[ps.y].a, b = s_win[ps.y].b;
        av[ps.x] = make_double4_32a(a.x, a.y, b.x, 0.0);
    }
    sweep_done(pass, sc, n_avg, n_exact, flags, passes_out_all);
}

// Would any edge of the chunk average on the current velocities? (A block
// per chunk of at most 256 edges of one scene, the grid striding over the
// chunks; chunks of finished scenes, or of scenes where an averaging edge is
// already found, are skipped.) If none of a scene's
// edges would, its sweep changes nothing: before the first edge that
// averages every edge sees the start-of-pass velocities.
__global__ void __launch_bounds__(256) k_strain_check(const StrainEdge* __restrict__ edges,
                                                      const double4_32a* __restrict__ xo,
                                                      const StrainEdgeHot* __restrict__ hot,
                                                      const int2* __restrict__ chunks, int nchunks,
                                                      const SceneDev* __restrict__ scenes,
                                                      const double4_32a* __restrict__ av, int* flags) {
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int2 ch = chunks[c];  // (scene, first edge)
        const SceneDev& sd = scenes[ch.x];
        // done scenes, and scenes where an edge that averages is already found
        if (!sd.enabled || flags[2 * ch.x + 1] || *(volatile int*)&flags[2 * ch.x]) continue;
        const int end = sd.strain_e0 + sd.strain_ne;
        const int e = ch.y + threadIdx.x;
        if (e >= end) continue;
        const StrainEdgeHot h = hot[e];
        const int2 pp = *reinterpret_cast<const int2*>(&edges[e]);  // p0, p1
        const double4_32a a0 = av[pp.x], a1 = av[pp.y];
        const float dt32 = __double2float_ru(sd.p.dt);
        int q = strain_decide32(h, make_float4((float)a0.x, (float)a0.y, (float)a0.z, 0.f),
                                make_float4((float)a1.x, (float)a1.y, (float)a1.z, 0.f), dt32);
        if (q < 0) {
            double v0[3] = {a0.x, a0.y, a0.z}, v1[3] = {a1.x, a1.y, a1.z};
            int n_exact = 0;
            q = strain_flag_vals(strain_step(edges[e], xo), v0, v1, sd.p.dt, &n_exact) ? 1 : 0;
        }
        if (q > 0 && !flags[2 * ch.x]) atomicOr(&flags[2 * ch.x], 1);
    }
}

// Start of a strain loop for the scenes in mask (all: mask null): their
// flags and counters cleared; the others marked finished, so that every
// kernel of this loop leaves them and their counters alone.
__global__ void k_strain_init(const uint8_t* __restrict__ mask, int nscenes, int* flags, int* passes_out) {
    int sc = blockIdx.x * blockDim.x + threadIdx.x;
    if (sc >= nscenes) return;
    if (mask && !mask[sc]) {
        flags[2 * sc + 1] = 1;
        return;
    }
    flags[2 * sc] = flags[2 * sc + 1] = 0;
    passes_out[3 * sc] = passes_out[3 * sc + 1] = passes_out[3 * sc + 2] = 0;
}

__global__ void k_final_velocity(const uint8_t* __restrict__ in_elem, const uint8_t* __restrict__ has_collsn,
                                 const double4_32a* __restrict__ av, const int* __restrict__ vscene,
                                 const SceneDev* __restrict__ scenes, double* vel, int nv,
                                 const uint8_t* __restrict__ mask) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv || !in_elem[p] || !has_collsn[p] || !scenes[vscene[p]].enabled) return;
    if (mask && !mask[vscene[p]]) return;
    double4_32a a = av[p];
    vel[3 * p] = a.x;
    vel[3 * p + 1] = a.y;
    vel[3 * p + 2] = a.z;
}

__global__ void k_math_selftest(int fn, const double* a, const double* b, double* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double r;
    switch (fn) {
        case 0: r = cr::cos(a[i]); break;
        case 1: r = cr::sin(a[i]); break;
        case 2: r = cr::acos(a[i]); break;
        default: r = cr::pow(a[i], b[i]); break;
    }
    out[i] = r;
}

// updateFinalForRG, dcollid.cpp:626-675: the first point of each body, in
// element order, that has has_collsn (its index, -1 for none) and its final
// average velocity.
__global__ void k_final_rg(const int* __restrict__ visit, const int* __restrict__ visit_off, int nbodies,
                           const uint8_t* __restrict__ has_collsn, const double4_32a* __restrict__ av,
                           double4_32a* out) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbodies) return;
    double4_32a r = make_double4_32a(0.0, 0.0, 0.0, -1.0);
    for (int i = visit_off[b]; i < visit_off[b + 1]; ++i) {
        const int p = visit[i];
        if (has_collsn[p]) {
            const double4_32a a = av[p];
            r = make_double4_32a(a.x, a.y, a.z, (double)p);
            break;
        }
    }
    out[b] = r;
}

}  // namespace

size_t strain_warp_smem(int max_slots, int ecap, int lcap, int wcap) {
    size_t b = (size_t)max_slots * sizeof(WarpSlot) +
               (size_t)kWarpRing * ((size_t)ecap * sizeof(StrainEdgeHot) + (size_t)lcap * 8 + (size_t)wcap * 8);
    return ((b + 15) & ~(size_t)15) + (size_t)kWarpRing * 32;
}

void math_selftest(int fn, const double* a, const double* b, double* out, int n, cudaStream_t s) {
    if (n > 0) count_launch(), k_math_selftest<<<nblk(n, 128), 128, 0, s>>>(fn, a, b, out, n);
}

void step_init(const double* x_old, const double* x_cand, int nv, const uint8_t* in_elem, const int* vscene,
               const SceneDev* scenes, double4_32a* xo, double4_32a* av, PassCounters* ctr, cudaStream_t s) {
    if (nv > 0)
        count_launch(), k_step_init<<<nblk(nv, 256), 256, 0, s>>>(x_old, x_cand, nv, in_elem, vscene, scenes, xo, av,
                                                                  ctr);
}

void apply_contribs(const Contrib* contrib, const PassCounters* ctr, int contrib_cap, int nv, double4_32a* av,
                    uint8_t* has_collsn, ApplyBufs& b, cudaStream_t s, double4_32a* dump, const BodyBufs* bodies) {
    if (dump && nv > 0) cudaMemsetAsync(dump, 0, sizeof(double4_32a) * (size_t)nv, s);
    if (nv <= 0) return;
    const int nb = bodies ? bodies->n : 0, nslot = nv + nb;
    cudaMemsetAsync(b.cnt, 0, sizeof(int) * (size_t)nslot, s);
    cudaMemsetAsync(b.cur, 0, sizeof(int) * (size_t)nslot, s);
    if (nb > 0) cudaMemsetAsync(bodies->num, 0, sizeof(int) * (size_t)nb, s);
    int blocks = nblk(contrib_cap, 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    count_launch(), k_contrib_count<<<blocks, 256, 0, s>>>(contrib, ctr, contrib_cap, b.cnt);
    exclusive_scan(b.cnt, b.off, nslot, nullptr, b.scan_temp, s);
    count_launch(), k_contrib_scatter<<<blocks, 256, 0, s>>>(contrib, ctr, contrib_cap, b.off, b.cur, b.idx);
    count_launch(), k_apply<<<nblk(nslot, 128), 128, 0, s>>>(contrib, const_cast<PassCounters*>(ctr), b.cnt, b.off,
                                                             b.idx, nv, av, has_collsn, dump, nb,
                                                             nb ? bodies->acc : nullptr, nb ? bodies->num : nullptr,
                                                             b.ps);
    if (nb > 0)
        count_launch(), k_apply_rg<<<nblk(bodies->nmembers, 128), 128, 0, s>>>(
            bodies->members, bodies->member_body, bodies->nmembers, ctr, bodies->acc, bodies->num, bodies->fixed, av,
            has_collsn, b.ps);
}

void zone_solve(const int* members, const int* zone_off, int nzones, const uint8_t* fixed, const double4_32a* xo,
                double4_32a* av, const int* vscene, const SceneDev* scenes, PassCounters* ctr, cudaStream_t s,
                const SceneRun* run, PassStamp ps) {
    if (nzones > 0)
        count_launch(), k_zone_solve<<<nblk(nzones, 128), 128, 0, s>>>(members, zone_off, nullptr, nzones, nullptr,
                                                                       fixed, xo, av, vscene, scenes, ctr, run, ps, 0);
}

void zone_solve_dev(const int* members, const int2* zone_rng, const int* dnz, int zone_cap, const uint8_t* fixed,
                    const double4_32a* xo, double4_32a* av, const int* vscene, const SceneDev* scenes,
                    PassCounters* ctr, cudaStream_t s, PassStamp ps, int cta_min, int few) {
    if (cta_min < kZoneWarpMin) cta_min = kZoneWarpMin;
    int blocks = nblk(zone_cap, 64);
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks > 0)
        count_launch(), k_zone_solve<<<blocks, 64, 0, s>>>(members, nullptr, zone_rng, zone_cap, dnz, fixed, xo, av,
                                                           vscene, scenes, ctr, nullptr, ps, few);
    int wblocks = nblk(zone_cap, kZoneWarpBlock / 32);
    if (wblocks > 152 * 4) wblocks = 152 * 4;
    if (wblocks > 0)
        count_launch(), k_zone_solve_warp<<<wblocks, kZoneWarpBlock, 0, s>>>(members, zone_rng, zone_cap, dnz, fixed,
                                                                            xo, av, vscene, scenes, ctr, ps, cta_min,
                                                                            few);
    const int cblocks = zone_cap < 152 * 2 ? zone_cap : 152 * 2;
    if (cblocks > 0)
        count_launch(), k_zone_solve_cta<<<cblocks, kZoneCtaThreads, 0, s>>>(members, zone_rng, zone_cap, dnz, fixed,
                                                                            xo, av, vscene, scenes, ctr, ps, cta_min);
}

void final_rigid(const BodyBufs& b, const uint8_t* has_collsn, const double4_32a* av, cudaStream_t s) {
    if (b.n > 0)
        count_launch(), k_final_rg<<<nblk(b.n, 128), 128, 0, s>>>(b.visit, b.visit_off, b.n, has_collsn, av, b.out);
}

void finalize_positions(const uint8_t* in_elem, const double4_32a* xo, double4_32a* av, uint8_t* has_collsn,
                        const double* x_cand, double* x_out, int nv, const int* vscene, const SceneDev* scenes,
                        const uint8_t* fixed, const uint8_t* mask, cudaStream_t s) {
    if (nv > 0)
        count_launch(), k_finalize<<<nblk(nv, 256), 256, 0, s>>>(in_elem, xo, av, has_collsn, x_cand, x_out, nv,
                                                                 vscene, scenes, fixed, mask);
}

size_t strain_step_bytes(int nedges) {
    size_t n = (size_t)(nedges > 0 ? nedges : 1);
    return sizeof(StrainEdgeStep) * n + sizeof(StrainEdgeHot) * n;
}

int strain_window_slot_cap() { return (int)(kStrainWindowBytes / sizeof(WinSlot)); }

void strain_configure() {
    cudaFuncSetAttribute(k_strain_window<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStrainWindowBytes);
    cudaFuncSetAttribute(k_strain_window<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStrainWindowBytes);
    cudaFuncSetAttribute(k_strain_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStrainWarpBytes);
}

void strain_setup(const StrainEdge* edges, int nedges, const SceneDev* scenes, const StrainPlan& plan,
                  const double4_32a* xo, void* step_buf, const int* vscene, cudaStream_t s) {
    if (nedges <= 0) return;
    StrainEdgeStep* se = (StrainEdgeStep*)step_buf;
    StrainEdgeHot* hot = (StrainEdgeHot*)(se + nedges);
    const int cap = plan.window ? strain_window_slot_cap() : -1;
    count_launch(), k_strain_setup<<<nblk(nedges, 256), 256, 0, s>>>(edges, nedges, xo, se, hot, vscene, scenes, cap);
}

void strain_limit(const StrainEdge* edges, int nedges, const int4* hdr, const int2* load_list, const int2* wb_list,
                  const int2* chunks, int nchunks, const SceneDev* scenes, int nscenes, const StrainPlan& plan,
                  const double4_32a* xo, double4_32a* av, void* step_buf, int* flags, int* passes_out,
                  const uint8_t* mask, cudaStream_t s) {
    if (nscenes <= 0) return;
    StrainEdgeStep* se = (StrainEdgeStep*)step_buf;
    StrainEdgeHot* hot = (StrainEdgeHot*)(se + (nedges > 0 ? nedges : 1));
    count_launch(), k_strain_init<<<nblk(nscenes, 128), 128, 0, s>>>(mask, nscenes, flags, passes_out);
    // scenes with at most `cap` slots are swept in shared memory (cap -1: none)
    int cap = plan.window ? strain_window_slot_cap() : -1;
    size_t smem = (size_t)plan.max_window_slots * sizeof(WinSlot);
    for (int pass = 0; pass < kStrainMaxIter; ++pass) {
        if (nchunks > 0)
            count_launch(), k_strain_check<<<nchunks < 152 * 8 ? nchunks : 152 * 8, 256, 0, s>>>(
                edges, xo, hot, chunks, nchunks, scenes, av, flags);
        if (plan.window && plan.warp)
            count_launch(), k_strain_warp<<<nscenes, 32, plan.warp_smem, s>>>(
                edges, xo, hot, hdr, scenes, cap, load_list, wb_list, av, pass, flags, passes_out, plan.max_window_slots,
                plan.ecap, plan.lcap, plan.wcap, plan.order);
        else if (plan.window && plan.ecap > plan.block)
            count_launch(), k_strain_window<true><<<nscenes, plan.block, smem, s>>>(
                edges, xo, hot, hdr, scenes, cap, load_list, wb_list, av, pass, flags, passes_out, plan.lcap > plan.block,
                plan.order, plan.cbase, plan.wbase);
        else if (plan.window)
            count_launch(), k_strain_window<false><<<nscenes, plan.block, smem, s>>>(
                edges, xo, hot, hdr, scenes, cap, load_list, wb_list, av, pass, flags, passes_out, plan.lcap > plan.block,
                plan.order, plan.cbase, plan.wbase);
        if (!plan.window || plan.any_global)
            count_launch(), k_strain<<<nscenes, 256, 0, s>>>(se, hdr, scenes, cap, av, pass, flags, passes_out,
                                                             plan.order);
    }
}

void final_velocity(const uint8_t* in_elem, const uint8_t* has_collsn, const double4_32a* av, const int* vscene,
                    const SceneDev* scenes, double* vel, int nv, const uint8_t* mask, cudaStream_t s) {
    if (nv > 0)
        count_launch(), k_final_velocity<<<nblk(nv, 256), 256, 0, s>>>(in_elem, has_collsn, av, vscene, scenes, vel,
                                                                       nv, mask);
}

}  // namespace ccg
