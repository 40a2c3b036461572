// Per-point stages around the detection passes: average velocity, applying
// a pass's impulses, impact-zone rigid motion, the domain clamp, final
// positions, strain limiting and final velocities (dcollid.cpp:116-220,
// 290-310, 486-624, 677-751; dcollid3d.cpp:70-200).
#include "cc_launch.h"
#include "cc_narrow.cuh"

namespace ccg {

namespace {

inline int nblk(int n, int t) { return (n + t - 1) / t; }

// computeAverageVelocity, dcollid.cpp:160-220: avgVel = (x_cand - x_old)/dt.
__global__ void k_step_init(const double* __restrict__ x_old, const double* __restrict__ x_cand, int nv,
                            const uint8_t* __restrict__ in_elem, double dt, double4_32a* xo, double4_32a* av,
                            PassCounters* ctr) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv) return;
    double o[3] = {x_old[3 * p], x_old[3 * p + 1], x_old[3 * p + 2]};
    xo[p] = make_double4_32a(o[0], o[1], o[2], 0.0);
    if (!in_elem[p]) return;
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
    if (ctr->err & (kErrContribOverflow | kErrPairOverflow | kErrStack)) return;
    int n = ctr->ncontrib < cap ? ctr->ncontrib : cap;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&cnt[c[i].vertex], 1);
}

__global__ void k_contrib_scatter(const Contrib* __restrict__ c, const PassCounters* ctr, int cap,
                                  const int* __restrict__ off, int* cur, int* idx) {
    if (ctr->err & (kErrContribOverflow | kErrPairOverflow | kErrStack)) return;
    int n = ctr->ncontrib < cap ? ctr->ncontrib : cap;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int v = c[i].vertex;
        idx[off[v] + atomicAdd(&cur[v], 1)] = i;
    }
}

// updateAverageVelocity, dcollid.cpp:677-751, for one point: its
// contributions are put in visiting order and summed one by one from zero,
// as the reference accumulates collsnImpulse and friction.
__global__ void k_apply(const Contrib* __restrict__ c, PassCounters* ctr, const int* __restrict__ cnt,
                        const int* __restrict__ off, int* idx, int nv, double4_32a* av, uint8_t* has_collsn) {
    if (ctr->err & (kErrContribOverflow | kErrPairOverflow | kErrStack)) return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv) return;
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
}

__global__ void k_uf_init(int* parent, int nv) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < nv) parent[p] = p;
}

__global__ void k_uf_flatten(int* parent, const uint8_t* in_elem, int nv, int* root, int* zcnt) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv) return;
    int r = uf_find(parent, p);
    root[p] = r;
    if (in_elem[p]) atomicAdd(&zcnt[r], 1);
}

__global__ void k_zone_keys(const int* __restrict__ root, const int* __restrict__ zcnt,
                            const uint8_t* __restrict__ in_elem, int nv, unsigned long long* keys,
                            unsigned int* vals, int* nmembers) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv || !in_elem[p]) return;
    int r = root[p];
    if (zcnt[r] < 2) return;
    int slot = atomicAdd(nmembers, 1);
    keys[slot] = ((unsigned long long)r << 32) | (unsigned long long)p;
    vals[slot] = (unsigned int)p;
}

__device__ __forceinline__ double det3(const double (*a)[3]) {
    return a[0][0] * (a[1][1] * a[2][2] - a[2][1] * a[1][2]) - a[0][1] * (a[1][0] * a[2][2] - a[2][0] * a[1][2]) +
           a[0][2] * (a[1][0] * a[2][1] - a[2][0] * a[1][1]);
}

// updateImpactListVelocity, dcollid3d.cpp:70-200, one thread per zone over
// its members in point order.
__global__ void k_zone_solve(const unsigned long long* __restrict__ keys, const unsigned int* __restrict__ vals,
                             const int* nmembers_p, const uint8_t* __restrict__ fixed,
                             const double4_32a* __restrict__ xo, double4_32a* av, Params prm, PassCounters* ctr) {
    int nm = *nmembers_p;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nm) return;
    unsigned int zr = (unsigned int)(keys[i] >> 32);
    if (i > 0 && (unsigned int)(keys[i - 1] >> 32) == zr) return;  // not the zone's first member
    int end = i;
    while (end < nm && (unsigned int)(keys[end] >> 32) == zr) ++end;
    const double m = prm.m, dt = prm.dt;
    double x_cm[3] = {0.0, 0.0, 0.0}, v_cm[3] = {0.0, 0.0, 0.0};
    double L[3] = {0.0, 0.0, 0.0}, I[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}}, tmp[3][3];
    int num_pts = end - i;
    for (int q = i; q < end; ++q) {
        int p = (int)vals[q];
        double xs[3], vs[3];
        load3(xo, p, xs);
        load3(av, p, vs);
        for (int d = 0; d < 3; ++d) { x_cm[d] += xs[d]; v_cm[d] += vs[d]; }
    }
    for (int d = 0; d < 3; ++d) { x_cm[d] /= num_pts; v_cm[d] /= num_pts; }
    for (int q = i; q < end; ++q) {
        int p = (int)vals[q];
        double xs[3], vs[3], dx[3], dv[3], Li[3];
        load3(xo, p, xs);
        load3(av, p, vs);
        for (int d = 0; d < 3; ++d) { dx[d] = xs[d] - x_cm[d]; dv[d] = vs[d] - v_cm[d]; }
        cross3(dx, dv, Li);
        for (int d = 0; d < 3; ++d) Li[d] = m * Li[d];
        for (int d = 0; d < 3; ++d) L[d] = Li[d] + L[d];
    }
    for (int q = i; q < end; ++q) {
        int p = (int)vals[q];
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
    for (int r = 0; r < 3; ++r) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) tmp[a][b] = I[a][b];
        for (int s = 0; s < 3; ++s) tmp[s][r] = L[s];
        if (det3(I) < kRoundEps)
            w[r] = 0.0;
        else
            w[r] = det3(tmp) / det3(I);
    }
    double mag_w = mag3(w);
    bool bad = false;
    for (int q = i; q < end; ++q) {
        int p = (int)vals[q];
        if (fixed[p]) continue;
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
            double sw = sin(dt * mag_w) / mag_w;
            for (int d = 0; d < 3; ++d) tmpV[d] = sw * w[d];
            cross3(tmpV, xR, wxR);
        }
        double cw = cos(dt * mag_w);
        for (int d = 0; d < 3; ++d) {
            x_new[d] = x_cm[d] + dt * v_cm[d] + xF[d] + cw * xR[d] + wxR[d];
            nv_[d] = (x_new[d] - xs[d]) / dt;
            if (isnan(nv_[d])) bad = true;
        }
        av[p] = make_double4_32a(nv_[0], nv_[1], nv_[2], 0.0);
    }
    if (bad) atomicOr(&ctr->err, kErrNan);
}

// detectDomainBoundaryCollision (dcollid.cpp:116-158) then
// updateFinalPosition (dcollid.cpp:562-584) for one point. The reference
// revisits points shared by several elements; the clamp is idempotent, so
// once per point gives the same result.
__global__ void k_finalize(const uint8_t* __restrict__ in_elem, const double4_32a* __restrict__ xo, double4_32a* av,
                           uint8_t* has_collsn, const double* __restrict__ x_cand, double* x_out, int nv,
                           Params prm, double L0, double L1, double L2, double U0, double U1, double U2) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv) return;
    if (!in_elem[p]) {
        for (int j = 0; j < 3; ++j) x_out[3 * p + j] = x_cand[3 * p + j];
        return;
    }
    double L[3] = {L0, L1, L2}, U[3] = {U0, U1, U2};
    double xs[3], v[3];
    load3(xo, p, xs);
    load3(av, p, v);
    double dt = prm.dt, mu = prm.lambda, dv = 0;
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

// One edge's strain test, reduceSuperelastOnce (dcollid.cpp:496-539).
__device__ __forceinline__ bool strain_flag(const StrainEdge& e, const double4_32a* xo, const double4_32a* av, double dt) {
    double x0[3], x1[3], v0[3], v1[3], c0[3], c1[3];
    load3(xo, e.p0, x0);
    load3(xo, e.p1, x1);
    load3(av, e.p0, v0);
    load3(av, e.p1, v1);
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
        double strain = (len_new - e.len0) / e.len0;
        return fabs(strain) > kStrainTol || fabs(strain_rate) > kStrainTol;
    }
    return true;
}

// reduceSuperelast, dcollid.cpp:586-596: up to 10 Gauss-Seidel passes. The
// sweep order matters (each averaged edge changes the points its successors
// read), so one warp walks the edges in element order; every pass first
// evaluates all edges against the pass-start velocities in parallel, and the
// walk re-evaluates only edges whose points were averaged earlier in the pass.
__global__ void __launch_bounds__(1024) k_strain(const StrainEdge* __restrict__ edges, int m,
                                                 const double4_32a* __restrict__ xo, double4_32a* av, uint8_t* flag0,
                                                 uint8_t* dirty, int nv, double dt, int* passes_out) {
    __shared__ int s_has;
    int passes = 0;
    for (int pass = 0; pass < kStrainMaxIter; ++pass) {
        for (int e = threadIdx.x; e < m; e += blockDim.x) flag0[e] = strain_flag(edges[e], xo, av, dt) ? 1 : 0;
        for (int p = threadIdx.x; p < nv; p += blockDim.x) dirty[p] = 0;
        __syncthreads();
        passes++;
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            bool has = false;
            for (int base = 0; base < m; base += 32) {
                int e = base + lane;
                bool valid = e < m;
                StrainEdge ed;
                if (valid) ed = edges[e];
                unsigned pre0 = __ballot_sync(0xffffffffu, valid && flag0[valid ? e : 0]);
                int cursor = 0;
                while (true) {
                    bool f = false;
                    if (valid && lane >= cursor) {
                        volatile uint8_t* dv = dirty;
                        if (dv[ed.p0] || dv[ed.p1])
                            f = strain_flag(ed, xo, av, dt);
                        else
                            f = flag0[e] != 0;
                    }
                    unsigned b = __ballot_sync(0xffffffffu, f);
                    if (b == 0) break;
                    int first = __ffs(b) - 1;
                    if (lane == first) {
                        double4_32a a0 = av[ed.p0], a1 = av[ed.p1];
                        double t0 = a0.x + a1.x, t1 = a0.y + a1.y, t2 = a0.z + a1.z;
                        t0 = 0.5 * t0; t1 = 0.5 * t1; t2 = 0.5 * t2;
                        double4_32a nv4 = make_double4_32a(t0, t1, t2, 0.0);
                        av[ed.p0] = nv4;
                        av[ed.p1] = nv4;
                        dirty[ed.p0] = 1;
                        dirty[ed.p1] = 1;
                    }
                    has = true;
                    __syncwarp();
                    __threadfence_block();
                    cursor = first + 1;
                    if (cursor >= 32) break;
                }
                (void)pre0;
            }
            if (lane == 0) s_has = has ? 1 : 0;
        }
        __syncthreads();
        if (!s_has) break;
        __syncthreads();
    }
    if (threadIdx.x == 0) *passes_out = passes;
}

__global__ void k_final_velocity(const uint8_t* __restrict__ in_elem, const uint8_t* __restrict__ has_collsn,
                                 const double4_32a* __restrict__ av, double* vel, int nv) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nv || !in_elem[p] || !has_collsn[p]) return;
    double4_32a a = av[p];
    vel[3 * p] = a.x;
    vel[3 * p + 1] = a.y;
    vel[3 * p + 2] = a.z;
}

}  // namespace

void step_init(const double* x_old, const double* x_cand, int nv, const uint8_t* in_elem, double dt, double4_32a* xo,
               double4_32a* av, PassCounters* ctr, cudaStream_t s) {
    if (nv > 0) k_step_init<<<nblk(nv, 256), 256, 0, s>>>(x_old, x_cand, nv, in_elem, dt, xo, av, ctr);
}

void apply_contribs(const Contrib* contrib, const PassCounters* ctr, int contrib_cap, int nv, double4_32a* av,
                    uint8_t* has_collsn, ApplyBufs& b, cudaStream_t s) {
    if (nv <= 0) return;
    cudaMemsetAsync(b.cnt, 0, sizeof(int) * (size_t)nv, s);
    cudaMemsetAsync(b.cur, 0, sizeof(int) * (size_t)nv, s);
    int blocks = nblk(contrib_cap, 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_contrib_count<<<blocks, 256, 0, s>>>(contrib, ctr, contrib_cap, b.cnt);
    exclusive_scan(b.cnt, b.off, nv, nullptr, b.scan_temp, s);
    k_contrib_scatter<<<blocks, 256, 0, s>>>(contrib, ctr, contrib_cap, b.off, b.cur, b.idx);
    k_apply<<<nblk(nv, 128), 128, 0, s>>>(contrib, const_cast<PassCounters*>(ctr), b.cnt, b.off, b.idx, nv, av,
                                           has_collsn);
}

void uf_init(int* parent, int nv, cudaStream_t s) {
    if (nv > 0) k_uf_init<<<nblk(nv, 256), 256, 0, s>>>(parent, nv);
}

void zone_velocity(int* parent, const uint8_t* in_elem, const uint8_t* fixed, const double4_32a* xo, double4_32a* av,
                   int nv, const Params& p, ZoneBufs& z, PassCounters* ctr, cudaStream_t s) {
    if (nv <= 0) return;
    cudaMemsetAsync(z.zcnt, 0, sizeof(int) * (size_t)nv, s);
    cudaMemsetAsync(z.nmembers, 0, sizeof(int), s);
    k_uf_flatten<<<nblk(nv, 256), 256, 0, s>>>(parent, in_elem, nv, z.root, z.zcnt);
    k_zone_keys<<<nblk(nv, 256), 256, 0, s>>>(z.root, z.zcnt, in_elem, nv, z.keys, z.vals, z.nmembers);
    int nm = 0;
    cudaMemcpyAsync(&nm, z.nmembers, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (nm <= 0) return;
    int bits = 32;
    while (bits < 64 && ((unsigned long long)(nv - 1) >> (bits - 32)) != 0ull) ++bits;
    radix_sort_pairs(z.keys, z.vals, nm, bits, z.sort_temp, s);
    k_zone_solve<<<nblk(nm, 128), 128, 0, s>>>(z.keys, z.vals, z.nmembers, fixed, xo, av, p, ctr);
}

void finalize_positions(const uint8_t* in_elem, const double4_32a* xo, double4_32a* av, uint8_t* has_collsn,
                        const double* x_cand, double* x_out, int nv, const Params& p, const double* lo,
                        const double* hi, cudaStream_t s) {
    if (nv > 0)
        k_finalize<<<nblk(nv, 256), 256, 0, s>>>(in_elem, xo, av, has_collsn, x_cand, x_out, nv, p, lo[0], lo[1],
                                                 lo[2], hi[0], hi[1], hi[2]);
}

void strain_limit(const StrainEdge* edges, int nedges, const double4_32a* xo, double4_32a* av, uint8_t* flag0,
                  uint8_t* dirty, int nv, double dt, int* passes_out, cudaStream_t s) {
    if (nedges <= 0) {
        cudaMemsetAsync(passes_out, 0, sizeof(int), s);
        return;
    }
    k_strain<<<1, 1024, 0, s>>>(edges, nedges, xo, av, flag0, dirty, nv, dt, passes_out);
}

void final_velocity(const uint8_t* in_elem, const uint8_t* has_collsn, const double4_32a* av, double* vel, int nv,
                    cudaStream_t s) {
    if (nv > 0) k_final_velocity<<<nblk(nv, 256), 256, 0, s>>>(in_elem, has_collsn, av, vel, nv);
}

}  // namespace ccg
