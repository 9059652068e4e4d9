// Count-to-slot scan that allocates nothing.
//
// iss_gpu_scan_counts_noalloc runs the same three scan kernels that
// iss_gpu_generate uses to turn per-(event, species) hadron counts into output
// slots (launch_offsets_scan, kernels_sample.cu).  Inside iss_gpu_generate the
// per-tile partial sums live in a buffer that the handle allocates.  Here they
// live in one fixed array in device global memory, so the call makes no
// cudaMalloc, no cudaFree and no allocation through any library.
//
// Who needs this: code that draws its own counts and only wants the slot
// offsets, and that cannot allocate device memory at that point.  Two common
// cases: (1) a program whose memory pool has already claimed the device's
// memory; (2) a pipeline that keeps other streams busy.  In case (2),
// cudaFree waits for the whole device and stalls those streams.
//
// Limits and contract:
//   * n <= ISS_GPU_NOALLOC_SCAN_MAX_SEGMENTS (16384 tiles of 4096 counts).
//     Larger n returns ISS_ERR_CAPACITY before any device work.
//   * Nothing in the scratch array has to start at zero.  The first kernel
//     writes every tile slot that the later kernels read.
//   * There is one scratch array per device.  Two calls whose kernels can run
//     at the same time on one device race on it: calls on one device must be
//     ordered, for example by issuing them on one stream.
//   * The scratch address is looked up once per device, on the first call
//     made on that device.  Under CUDA's lazy module loading (the default)
//     that first call loads the module holding the array, and loading it
//     takes the array's 128 KiB of device memory then.  So the first call on
//     a device must come before a memory pool claims that device's memory,
//     and before any stream capture on that device.  Later calls allocate
//     nothing.
//   * Counts must be >= 0; negative counts give wrong offsets (not checked).
//   * A CUDA error that earlier work left pending makes the call return
//     ISS_ERR_CUDA before it launches anything; that error stays pending for
//     its owner.  An error of this call's own launches is cleared and
//     reported as ISS_ERR_CUDA.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "iss_gpu.h"
#include "kernels.h"

namespace {

constexpr int kScratchTiles = 16384;
constexpr int kMaxDevices = 64;

// per-tile partial sums, then per-tile offsets (rewritten in place)
static __device__ __align__(256) int64_t g_scan_scratch[kScratchTiles];

std::atomic<int64_t*> g_addr[kMaxDevices];
std::mutex g_addr_mu;

int64_t* scratch_address(int dev) {
    int64_t* p = g_addr[dev].load(std::memory_order_acquire);
    if (p) return p;
    std::lock_guard<std::mutex> lock(g_addr_mu);
    p = g_addr[dev].load(std::memory_order_relaxed);
    if (p) return p;
    void* a = nullptr;
    if (cudaGetSymbolAddress(&a, g_scan_scratch) != cudaSuccess) return nullptr;
    p = static_cast<int64_t*>(a);
    g_addr[dev].store(p, std::memory_order_release);
    return p;
}

}  // namespace

static_assert(static_cast<int64_t>(kScratchTiles) * 4096 == ISS_GPU_NOALLOC_SCAN_MAX_SEGMENTS,
              "scratch size and the documented limit disagree");

extern "C" iss_status iss_gpu_scan_counts_noalloc(const int32_t* d_counts, int64_t n,
                                                  int64_t* d_offsets, void* stream) {
    if (n < 0 || !d_offsets || (n > 0 && !d_counts)) return ISS_ERR_INVALID_ARG;
    if (n > ISS_GPU_NOALLOC_SCAN_MAX_SEGMENTS || iss::offsets_num_tiles(n) > kScratchTiles)
        return ISS_ERR_CAPACITY;
    // an error left pending by the caller's earlier work is not ours to
    // clear, and launching behind it would misreport it as this call's
    if (cudaPeekAtLastError() != cudaSuccess) return ISS_ERR_CUDA;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return ISS_ERR_CUDA;
    }
    int64_t* scratch = scratch_address(dev);
    if (!scratch) {
        cudaGetLastError();
        return ISS_ERR_CUDA;
    }
    const cudaError_t e = iss::launch_offsets_scan(d_counts, n, scratch, d_offsets,
                                                   static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return ISS_ERR_CUDA;
    }
    return ISS_OK;
}
