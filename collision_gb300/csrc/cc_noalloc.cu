// Candidate-pair search that allocates no device memory.
//
// Some callers cannot call cudaMalloc: an application whose device memory is
// entirely owned by another allocator (an engine that reserves the GPU at
// start-up, a framework's caching pool), or a real-time loop that must not
// stall - cudaMalloc and cudaFree can synchronise the whole device and can
// fail once memory is fragmented. For them, cc_candidate_pairs_static runs
// the broad phase of the solver (Morton keys, radix sort, LBVH build and
// refit, traversal) on boxes and output buffers the caller owns, with every
// intermediate array carved out of one fixed scratch area compiled into the
// library.
//
// That scratch area is a file-scope __device__ array of kScratchBytes (8 MiB);
// every GPU that loads this library holds it until the process exits. It fits
// at most kMaxStaticElems (65,536) boxes. All calls on a device share it and
// it keeps the last call's contents, so each call clears what must start at
// zero (the pair counter and the refit arrival flags) and calls that overlap
// on the GPU - from two host threads, or on two streams - race on it. Host
// code only sees a stand-in for the array's name: its device address comes
// from cudaGetSymbolAddress, taken once per device, with that device current,
// on the first call there (that first call should come before any stream
// capture begins). A call makes its device current while it runs and gives
// the calling thread its previous current device back before it returns.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/collision_gb300.h"
#include "cc_launch.h"

namespace ccg {

namespace {

constexpr size_t kScratchBytes = (size_t)8 << 20;
constexpr int kMaxStaticElems = 65536;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_pair_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};
thread_local char g_static_err[256] = {0};

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Device address of the scratch array on `device`, looked up once.
cudaError_t scratch_address(int device, void** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_pair_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[device] = p;
    }
    *out = g_scratch_ptr[device];
    return cudaSuccess;
}

// Flags boxes that no hierarchy can order: a coordinate that is NaN or
// infinite, or a lower corner above the upper one.
__global__ void k_check_boxes(const Box6* __restrict__ box, int n, PassCounters* c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Box6 b = box[i];
    bool bad = false;
    for (int k = 0; k < 3; ++k)
        bad |= !isfinite(b.lo[k]) || !isfinite(b.hi[k]) || !(b.lo[k] <= b.hi[k]);
    if (bad) atomicOr(&c->err, kErrNan);
}

cc_status static_fail(cc_status st, const char* msg) {
    std::snprintf(g_static_err, sizeof(g_static_err), "%s", msg);
    return st;
}

// Makes `device` current for the lifetime of the guard and gives the calling
// thread its previous current device back on every return path.
struct DeviceGuard {
    int prev = -1;
    bool ok = false;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        ok = cudaSetDevice(device) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace

}  // namespace ccg

using namespace ccg;

extern "C" {

cc_status cc_candidate_pairs_static(int device, const double* boxes, int n, int* pairs, int cap, int* npairs,
                                    void* stream) {
    if (npairs) *npairs = 0;
    if (n > kMaxStaticElems)
        return static_fail(CC_BAD_INPUT, "more boxes than the static scratch area holds (65536)");
    if (n < 0 || cap < 0 || !npairs || (n > 0 && !boxes) || (cap > 0 && !pairs))
        return static_fail(CC_BAD_INPUT, "bad arguments");
    if (((uintptr_t)boxes & 15) != 0 || ((uintptr_t)pairs & 7) != 0)
        return static_fail(CC_BAD_INPUT, "boxes must be 16-byte and pairs 8-byte aligned");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev || device >= kMaxDevices)
        return static_fail(CC_CUDA_ERROR, "no such device");
    DeviceGuard guard(device);
    if (!guard.ok) return static_fail(CC_CUDA_ERROR, "cudaSetDevice failed");
    cudaStream_t s = (cudaStream_t)stream;
    if (s) {
        // a stream of another device would accept the copies below but not
        // the launches
        int sdev = -1;
        if (cudaStreamGetDevice(s, &sdev) != cudaSuccess || sdev != device)
            return static_fail(CC_BAD_INPUT, "the stream does not belong to the given device");
    }
    if (n <= 1) return CC_OK;
    void* base = nullptr;
    if (scratch_address(device, &base) != cudaSuccess)
        return static_fail(CC_CUDA_ERROR, "cudaGetSymbolAddress failed");

    // carve the scratch area
    char* p = (char*)base;
    size_t used = 0;
    auto take = [&](size_t bytes) {
        char* q = p + used;
        used += align256(bytes);
        return (void*)q;
    };
    BvhBufs b{};
    b.n = n;
    b.act = nullptr;
    b.nscenes = 1;  // one scene: no scene ids, traversal from node 0
    b.keys = (unsigned long long*)take(sizeof(unsigned long long) * (size_t)n);
    b.order = (unsigned int*)take(sizeof(unsigned int) * (size_t)n);
    b.range_hi = (int*)take(sizeof(int) * (size_t)n);
    b.range_lo = (int*)take(sizeof(int) * (size_t)n);
    b.parent = (int*)take(sizeof(int) * 2 * (size_t)n);
    b.flags = (int*)take(sizeof(int) * (size_t)n);
    b.node = (BvhNode32*)take(sizeof(BvhNode32) * (size_t)n);
    b.bbox_enc = (unsigned long long*)take(6 * sizeof(unsigned long long));
    PassCounters* ctr = (PassCounters*)take(sizeof(PassCounters));
    b.sort_temp = take(radix_sort_temp_bytes(n));
    if (used > kScratchBytes) return static_fail(CC_NO_MEMORY, "static scratch layout exceeds its size");

    const Box6* box = (const Box6*)boxes;
    PassCounters h{};
    // every counter starts at zero: the scratch area keeps the last call's
    if (cudaMemsetAsync(ctr, 0, sizeof(PassCounters), s) != cudaSuccess)
        return static_fail(CC_CUDA_ERROR, cudaGetErrorString(cudaGetLastError()));
    // boxes a hierarchy cannot order are rejected before any is built
    count_launch(), k_check_boxes<<<(n + 255) / 256, 256, 0, s>>>(box, n, ctr);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return static_fail(CC_CUDA_ERROR, cudaGetErrorString(e));
    if (h.err & kErrNan) return static_fail(CC_BAD_INPUT, "a box is NaN or infinite, or has lo > hi");

    boxes_bbox(box, n, b.bbox_enc, s);
    bvh_build(box, b, s);  // clears the refit arrival flags itself
    bvh_pairs(box, b, (int2*)pairs, cap, ctr, s);
    // a failed launch leaves the counters of an earlier call in place
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return static_fail(CC_CUDA_ERROR, cudaGetErrorString(e));
    *npairs = h.npairs;
    if (h.err & (kErrIndexNode | kErrIndexLeaf | kErrIndexElem)) {
        *npairs = 0;
        return static_fail(CC_CUDA_ERROR, "broad phase met an index out of range; the pairs are incomplete");
    }
    if (h.err & kErrStack) return static_fail(CC_STACK_OVERFLOW, "BVH traversal stack overflow");
    if (h.npairs > cap) return static_fail(CC_PAIR_OVERFLOW, "more pairs than cap; *npairs holds the count");
    return CC_OK;
}

int cc_static_last_error(char* buf, int len) {
    if (!buf || len <= 0) return 0;
    std::snprintf(buf, (size_t)len, "%s", g_static_err);
    return (int)std::strlen(g_static_err);
}

}  // extern "C"
