// bt_noalloc.cu -- global butterfly count that allocates no device memory.
//
// For callers that may not allocate on the device: plugin hosts that own the
// whole device heap and only hand buffers in, and latency-sensitive paths
// where a cudaMalloc / cudaFree (which can synchronise the device) is not
// acceptable.  The caller passes the graph and the output in its own device
// buffers; the wedge counters this count needs live in one file-scope device
// array, so nothing is allocated per call.
//
// Scratch: g_noalloc_scratch, kScratchWords 32-bit words (32 MiB).  Every GPU
// that loads this library holds it until the process exits.  Each resident CTA
// uses 2n words (a wedge counter and a touched list per vertex), so the count
// runs on min(2 per SM, kScratchWords / 2n) CTAs and rejects graphs with more
// than kScratchWords / 2 vertices.  The last 64 words hold the work counter.
//
// All calls share the array: calls that overlap on the GPU (on different
// streams or threads, without ordering between them) race on it and give
// wrong counts.  The array keeps the last call's contents; each call clears
// the parts that must start at zero (its counters and the work counter).
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (the host-side name of a __device__ array is only a
// stand-in); that set-up runs once per device and context, with the device
// current, and that first call should come before any stream capture.  The
// address is cached together with the CUDA context it belongs to: after the
// caller resets the device (cudaDeviceReset) the next call sees a new context
// and looks the address up again, so it never launches on a stale pointer.
//
// The call makes `device` current only for its own work and restores the
// caller's current device before it returns, on every path.
//
// Arithmetic: the vertex-priority count of the reference's bfc_kernel
// (src/bfc/bfc_vpp.cu:33-107) on the reference CSR layout (rows sorted by
// vertex id, priority p(x) = (degree, id) tested per neighbour).
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "bt_internal.h"

namespace {

constexpr uint64_t kScratchWords = 8ull << 20;  // 32 MiB
constexpr uint64_t kCounterWords = 64;          // work counter at the end
constexpr int kMaxDevices = 64;
constexpr int kThreadsNA = 512;

__device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords + kCounterWords];

uint32_t *g_scratch_addr[kMaxDevices];
CUcontext g_scratch_ctx[kMaxDevices];  // context the cached address belongs to
std::mutex g_scratch_mutex;

// The caller's current device, put back when the scope ends.
struct DeviceGuard {
    int saved = -1;
    DeviceGuard() {
        if (cudaGetDevice(&saved) != cudaSuccess) saved = -1;
    }
    ~DeviceGuard() {
        if (saved >= 0) cudaSetDevice(saved);
    }
    DeviceGuard(const DeviceGuard &) = delete;
    DeviceGuard &operator=(const DeviceGuard &) = delete;
};

// The current CUDA context, through the driver entry point the runtime hands
// out (the library does not link the driver library itself).
bt_status current_context(CUcontext *out) {
    using GetCurrent = CUresult (*)(CUcontext *);
    // looked up once; a function-local static is initialised thread-safely
    static const GetCurrent fn = []() -> GetCurrent {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess) return nullptr;
        return reinterpret_cast<GetCurrent>(p);
    }();
    if (!fn) return bt_fail(BT_ERR_CUDA, "cuCtxGetCurrent is not available from the CUDA driver");
    *out = nullptr;
    if (fn(out) != CUDA_SUCCESS || !*out) return bt_fail(BT_ERR_CUDA, "no current CUDA context");
    return BT_OK;
}

__device__ __forceinline__ bool higher(const uint32_t *off, uint32_t a, uint32_t b) {
    const uint32_t da = off[a + 1] - off[a], db = off[b + 1] - off[b];
    return da > db || (da == db && a > b);
}

// scratch: per CTA cnt[n] then touched[n]; counter[0] = next vertex
__global__ void __launch_bounds__(kThreadsNA) k_bfc_noalloc(uint32_t n, const uint32_t *off, const uint32_t *nbr,
                                                            uint32_t *scratch, uint32_t *counter,
                                                            unsigned long long *count) {
    __shared__ uint32_t s_r, s_nt;
    __shared__ unsigned long long s_red[kThreadsNA / 32];
    uint32_t *cnt = scratch + (size_t)blockIdx.x * 2 * n;
    uint32_t *touched = cnt + n;
    for (uint32_t x = threadIdx.x; x < n; x += blockDim.x) cnt[x] = 0;  // left over from the last call
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned long long local = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            s_r = atomicAdd(counter, 1u);
            s_nt = 0;
        }
        __syncthreads();
        const uint32_t u = s_r;
        if (u >= n) break;
        for (uint32_t i = off[u] + warp; i < off[u + 1]; i += nw) {
            const uint32_t v = nbr[i];
            if (!higher(off, u, v)) continue;
            for (uint32_t j = off[v] + lane; j < off[v + 1]; j += 32) {
                const uint32_t w = nbr[j];
                if (!higher(off, u, w)) continue;
                const uint32_t old = atomicAdd(cnt + w, 1u);
                local += old;
                if (old == 0) touched[atomicAdd(&s_nt, 1u)] = w;
            }
        }
        __syncthreads();
        const uint32_t nt = s_nt;
        for (uint32_t k = threadIdx.x; k < nt; k += blockDim.x) cnt[touched[k]] = 0;
        __syncthreads();
    }
    for (int o = 16; o; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if (lane == 0) s_red[warp] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (uint32_t k = 0; k < nw; k++) t += s_red[k];
        if (t) atomicAdd(count, t);
    }
}

// Device address of the scratch array on the current device: looked up once
// per device and context (`device` is current: cudaSetDevice has created or
// bound its primary context).
bt_status scratch_address(int device, uint32_t **out) {
    if (device < 0 || device >= kMaxDevices) return bt_fail(BT_ERR_INVALID, "device index out of range");
    CUcontext cur = nullptr;
    BT_TRY(current_context(&cur));
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_ctx[device] != cur) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return bt_cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
        g_scratch_addr[device] = static_cast<uint32_t *>(p);
        g_scratch_ctx[device] = cur;
    }
    *out = g_scratch_addr[device];
    return BT_OK;
}

}  // namespace

extern "C" bt_status bt_bfc_noalloc(int device, const uint32_t *d_offsets, const uint32_t *d_neighbors,
                                    uint32_t n, uint64_t m, unsigned long long *d_count, void *stream) {
    if (!d_offsets || !d_count || (m && !d_neighbors)) return bt_fail(BT_ERR_INVALID, "null argument");
    if ((uint64_t)n > kScratchWords / 2)
        return bt_fail(BT_ERR_INVALID, "bt_bfc_noalloc: " + std::to_string(n) +
                                           " vertices exceed the scratch limit of " +
                                           std::to_string(kScratchWords / 2) + " vertices");
    if (m > 0x7fffffffull) return bt_fail(BT_ERR_INVALID, "edge count exceeds the 32-bit CSR offsets");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
        return bt_fail(BT_ERR_NO_DEVICE, "gpu device id " + std::to_string(device) + " is not available");
    DeviceGuard restore;  // the caller's current device comes back on every return
    BT_CUDA(cudaSetDevice(device));
    uint32_t *scratch = nullptr;
    BT_TRY(scratch_address(device, &scratch));
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t *counter = scratch + kScratchWords;
    BT_CUDA(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st));
    if (n == 0) return BT_OK;
    BT_CUDA(cudaMemsetAsync(counter, 0, kCounterWords * sizeof(uint32_t), st));
    int sms = 0;
    BT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    uint64_t ctas = (uint64_t)sms * 2;
    const uint64_t fit = kScratchWords / (2ull * n);
    if (ctas > fit) ctas = fit;
    if (ctas > n) ctas = n;
    k_bfc_noalloc<<<(unsigned)ctas, kThreadsNA, 0, st>>>(n, d_offsets, d_neighbors, scratch, counter, d_count); bt_note_launches(1);
    BT_CUDA(cudaGetLastError());
    return BT_OK;
}
