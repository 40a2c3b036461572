// Device primitives: exclusive scan and a stable LSD radix sort of
// (64-bit key, 32-bit value) pairs with 8-bit digits. Hand-written (no CUB):
// the sort ranks keys inside a tile with __match_any_sync and per-warp digit
// counts in shared memory, so equal digits keep their input order.
#include "cc_launch.h"

namespace ccg {

long long g_kernel_launches = 0;

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 2;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int warp_incl_scan(int v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive scan of one tile per block; block totals to sums[blockIdx.x].
__global__ void k_scan_tile(const int* in, int* out, int n, int* sums) {
    __shared__ int wsum[kScanThreads / 32];
    int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int local = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        local += v[k];
    }
    int incl = warp_incl_scan(local);
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int s = (lane < kScanThreads / 32) ? wsum[lane] : 0;
        s = warp_incl_scan(s);
        if (lane < kScanThreads / 32) wsum[lane] = s;
    }
    __syncthreads();
    int run = incl - local + (warp > 0 ? wsum[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == kScanThreads - 1 && sums) sums[blockIdx.x] = run;
}

__global__ void k_scan_add(int* out, int n, const int* block_off) {
    int i = blockIdx.x * kScanTile + threadIdx.x;
    int add = block_off[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int j = i + k * kScanThreads;
        if (j < n) out[j] += add;
    }
}

__global__ void k_scan_total(const int* in, const int* out, int n, int* total) {
    if (n > 0)
        *total = out[n - 1] + in[n - 1];
    else
        *total = 0;
}

inline int ceil_div(int a, int b) { return (a + b - 1) / b; }

// Levels of block sums for an n-element scan.
size_t scan_levels_bytes(int n) {
    size_t bytes = 0;
    while (n > kScanTile) {
        n = ceil_div(n, kScanTile);
        bytes += ((size_t)n * sizeof(int) + 255) & ~(size_t)255;
    }
    return bytes;
}

void scan_rec(const int* in, int* out, int n, char* temp, cudaStream_t s) {
    int nb = ceil_div(n, kScanTile);
    if (nb <= 1) {
        count_launch(), k_scan_tile<<<1, kScanThreads, 0, s>>>(in, out, n, nullptr);
        return;
    }
    int* sums = (int*)temp;
    char* rest = temp + (((size_t)nb * sizeof(int) + 255) & ~(size_t)255);
    count_launch(), k_scan_tile<<<nb, kScanThreads, 0, s>>>(in, out, n, sums);
    scan_rec(sums, sums, nb, rest, s);
    count_launch(), k_scan_add<<<nb, kScanThreads, 0, s>>>(out, n, sums);
}

// ------------------------------------------------------------------ sort
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kRadix = 256;

// dn (may be null): the number of pairs to sort is min(*dn, n).
__device__ __forceinline__ int sort_count(const int* dn, int n) {
    if (!dn) return n;
    const int m = *dn;
    return m < n ? (m > 0 ? m : 0) : n;
}

__global__ void k_radix_hist(const unsigned long long* keys, int n, int shift, int* hist, int nblocks,
                             const int* dn) {
    n = sort_count(dn, n);
    __shared__ int h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    int base = blockIdx.x * kSortTile;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        int i = base + r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xff], 1);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_radix_scatter(const unsigned long long* keys, const unsigned int* vals, unsigned long long* okeys,
                                unsigned int* ovals, int n, int shift, const int* off, int nblocks, const int* dn) {
    n = sort_count(dn, n);
    __shared__ int run[kRadix];
    __shared__ int wcnt[kSortThreads / 32][kRadix];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    run[threadIdx.x] = 0;
    int base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
#pragma unroll
        for (int w = 0; w < kSortThreads / 32; ++w) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        int i = base + r * kSortThreads + threadIdx.x;
        bool valid = i < n;
        unsigned long long k = valid ? keys[i] : 0ull;
        int d = valid ? (int)((k >> shift) & 0xff) : kRadix;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int lrank = __popc(peers & lt_mask);
        if (valid && lrank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            int pre = run[d] + lrank;
            for (int w = 0; w < warp; ++w) pre += wcnt[w][d];
            int pos = off[d * nblocks + blockIdx.x] + pre;
            okeys[pos] = k;
            ovals[pos] = vals[i];
        }
        __syncthreads();
        int tot = 0;
#pragma unroll
        for (int w = 0; w < kSortThreads / 32; ++w) tot += wcnt[w][threadIdx.x];
        run[threadIdx.x] += tot;
    }
}

// Small sorts in one CTA: up to kSmallSort pairs, each key extended by its
// input position (so the keys are distinct and a bitonic network gives the
// stable order), sorted in shared memory.
constexpr int kSmallSort = 8192;
constexpr int kSmallThreads = 1024;
constexpr int kIdxBits = 13;  // 2^13 = kSmallSort
constexpr size_t kSmallBytes = (size_t)kSmallSort * (sizeof(unsigned long long) + sizeof(unsigned int));

// Sorts the first m = min(*dn, n) pairs when m <= small_max (<= kSmallSort) and sets *eff
// to 0; otherwise leaves them and sets *eff = m. In a graph, also sets the
// conditional handle h (if use_h) to whether the general sort must run.
__global__ void __launch_bounds__(kSmallThreads) k_sort_small(unsigned long long* keys, unsigned int* vals,
                                                             const int* dn, int n, int small_max, int* eff,
                                                             cudaGraphConditionalHandle h, int use_h) {
    extern __shared__ unsigned long long s_k[];
    unsigned int* s_v = reinterpret_cast<unsigned int*>(s_k + kSmallSort);
    const int m = sort_count(dn, n);
    if (m > small_max) {
        if (threadIdx.x == 0) {
            *eff = m;
            if (use_h) cudaGraphSetConditional(h, 1u);
        }
        return;
    }
    int P = 1;
    while (P < m) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        if (i < m) {
            s_k[i] = (keys[i] << kIdxBits) | (unsigned long long)i;
            s_v[i] = vals[i];
        } else {
            s_k[i] = ~0ull;
        }
    }
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long a = s_k[i], b = s_k[ixj];
                    if ((a > b) == ((i & k) == 0)) {
                        s_k[i] = b;
                        s_k[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const unsigned long long c = s_k[i];
        keys[i] = c >> kIdxBits;
        vals[i] = s_v[c & (kSmallSort - 1)];
    }
    if (threadIdx.x == 0) {
        *eff = 0;
        if (use_h) cudaGraphSetConditional(h, 0u);
    }
}

}  // namespace

cudaError_t sort_pairs_dev(unsigned long long* keys, unsigned int* vals, const int* dn, int cap, int bits,
                           void* temp, int* eff, cudaStream_t s, cudaStream_t nested, bool small) {
    const int small_max = small ? kSmallSort : -1;
    if (cap <= 1 || bits <= 0) return cudaSuccess;
    if (bits > 64 - kIdxBits) {
        radix_sort_pairs_dev(keys, vals, dn, cap, bits, temp, s);
        return cudaGetLastError();
    }
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_sort_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kSmallBytes);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(s, &cst);
    if (e != cudaSuccess) return e;
    if (cst != cudaStreamCaptureStatusActive || !nested) {
        count_launch(), k_sort_small<<<1, kSmallThreads, kSmallBytes, s>>>(keys, vals, dn, cap, small_max, eff, 0, 0);
        radix_sort_pairs_dev(keys, vals, eff, cap, bits, temp, s);
        return cudaGetLastError();
    }
    // in a graph: the general sort behind an IF node that the small sort sets
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    e = cudaStreamGetCaptureInfo(s, &cst, nullptr, &g, &deps, nullptr, &ndeps);
    cudaGraphConditionalHandle h;
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    count_launch(), k_sort_small<<<1, kSmallThreads, kSmallBytes, s>>>(keys, vals, dn, cap, small_max, eff, h, 1);
    e = cudaStreamGetCaptureInfo(s, &cst, nullptr, &g, &deps, nullptr, &ndeps);
    cudaGraphNodeParams ip = {};
    cudaGraphNode_t node;
    if (e == cudaSuccess) {
        ip.type = cudaGraphNodeTypeConditional;
        ip.conditional.handle = h;
        ip.conditional.type = cudaGraphCondTypeIf;
        ip.conditional.size = 1;
        e = cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &ip);
    }
    if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(nested, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    radix_sort_pairs_dev(keys, vals, eff, cap, bits, temp, nested);
    cudaGraph_t body = nullptr;
    return cudaStreamEndCapture(nested, &body);
}

size_t scan_temp_bytes(int n) { return scan_levels_bytes(n) + 256; }

void exclusive_scan(const int* in, int* out, int n, int* total, void* temp, cudaStream_t s) {
    if (n <= 0) {
        if (total) cudaMemsetAsync(total, 0, sizeof(int), s);
        return;
    }
    // The last input is needed for the total after an in-place scan.
    int* last = (int*)((char*)temp + scan_levels_bytes(n));
    if (total) cudaMemcpyAsync(last, in + (n - 1), sizeof(int), cudaMemcpyDeviceToDevice, s);
    scan_rec(in, out, n, (char*)temp, s);
    if (total) count_launch(), k_scan_total<<<1, 1, 0, s>>>(last, out + (n - 1), 1, total);
}

size_t radix_sort_temp_bytes(int n) {
    int nb = ceil_div(n > 0 ? n : 1, kSortTile);
    size_t hist = (size_t)kRadix * nb;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    return al((size_t)n * sizeof(unsigned long long)) + al((size_t)n * sizeof(unsigned int)) +
           2 * al(hist * sizeof(int)) + al(scan_temp_bytes((int)hist));
}

void radix_sort_pairs(unsigned long long* keys, unsigned int* vals, int n, int bits, void* temp, cudaStream_t s) {
    radix_sort_pairs_dev(keys, vals, nullptr, n, bits, temp, s);
}

void radix_sort_pairs_dev(unsigned long long* keys, unsigned int* vals, const int* dn, int n, int bits, void* temp,
                          cudaStream_t s) {
    if (n <= 1 || bits <= 0) return;
    int nb = ceil_div(n, kSortTile);
    size_t hist_n = (size_t)kRadix * nb;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    char* t = (char*)temp;
    unsigned long long* k2 = (unsigned long long*)t;
    t += al((size_t)n * sizeof(unsigned long long));
    unsigned int* v2 = (unsigned int*)t;
    t += al((size_t)n * sizeof(unsigned int));
    int* hist = (int*)t;
    t += al(hist_n * sizeof(int));
    int* off = (int*)t;
    t += al(hist_n * sizeof(int));
    void* stemp = t;
    unsigned long long* ka = keys;
    unsigned int* va = vals;
    unsigned long long* kb = k2;
    unsigned int* vb = v2;
    int passes = (bits + 7) / 8;
    for (int ps = 0; ps < passes; ++ps) {
        int shift = ps * 8;
        count_launch(), k_radix_hist<<<nb, kSortThreads, 0, s>>>(ka, n, shift, hist, nb, dn);
        exclusive_scan(hist, off, (int)hist_n, nullptr, stemp, s);
        count_launch(), k_radix_scatter<<<nb, kSortThreads, 0, s>>>(ka, va, kb, vb, n, shift, off, nb, dn);
        unsigned long long* tk = ka; ka = kb; kb = tk;
        unsigned int* tv = va; va = vb; vb = tv;
    }
    if (ka != keys) {
        cudaMemcpyAsync(keys, ka, (size_t)n * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, va, (size_t)n * sizeof(unsigned int), cudaMemcpyDeviceToDevice, s);
    }
}

}  // namespace ccg
