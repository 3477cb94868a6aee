// noalloc.cu - all-origins shortest-path labels without any allocation.
//
// Some callers cannot let a library allocate device memory: applications
// that hand every byte of HBM to their own pool or arena and pass the library
// only buffers they own, and latency-critical loops in which a cudaMalloc or
// cudaFree (which can synchronise the whole device) is not acceptable.
// tapgpu_sssp_labels_noalloc serves them: the caller passes the graph, the
// weights, the sources and the output in device memory, and the only other
// memory used is the fixed array below, which every GPU that loads the
// library holds until the process exits.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "fw_kernels.cuh"
#include "tap_gpu.h"

namespace {

// 32 MiB: a 256-byte control block (work counter, error word) followed by
// per-CTA label slices of (8 (N+1) + bitmap) bytes each.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
constexpr size_t kControlBytes = 256;
constexpr int kMaxDevices = 64;
constexpr int kBlock = 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch per device; looked up once per device
// (with that device current), because in host code the symbol's name only
// stands for the array and is not a device address.
void* g_scratch_addr[kMaxDevices] = {nullptr};

int scratch_address(int dev, unsigned char** out) {
  if (dev < 0 || dev >= kMaxDevices) return TAPGPU_ERR_UNSUPPORTED;
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return TAPGPU_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_addr[dev]);
  return TAPGPU_OK;
}

// Check device-resident indices through a fixed stack buffer (no allocation):
// every value in [lo, hi], and non-decreasing when `monotone`.
int check_indices(const int32_t* d, int64_t n, int32_t lo, int32_t hi, bool monotone,
                  cudaStream_t s) {
  int32_t buf[1024];
  int32_t prev = lo;
  for (int64_t i0 = 0; i0 < n; i0 += 1024) {
    const int64_t cnt = n - i0 < 1024 ? n - i0 : 1024;
    if (cudaMemcpyAsync(buf, d + i0, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return TAPGPU_ERR_CUDA;
    for (int64_t i = 0; i < cnt; ++i) {
      if (buf[i] < lo || buf[i] > hi || (monotone && buf[i] < prev)) return TAPGPU_ERR_ARG;
      prev = buf[i];
    }
  }
  return TAPGPU_OK;
}

}  // namespace

extern "C" int tapgpu_sssp_labels_noalloc(int32_t num_nodes1, int32_t num_links,
                                          int32_t first_thru_node, const int32_t* d_row_ptr,
                                          const int32_t* d_head, const double* d_weight,
                                          const int32_t* d_sources, int32_t num_sources,
                                          double* d_dist, void* stream) {
  if (num_nodes1 < 1 || num_links < 0 || num_sources < 0 || !d_row_ptr ||
      (num_links > 0 && (!d_head || !d_weight)) || (num_sources > 0 && (!d_sources || !d_dist))) {
    fprintf(stderr, "tapgpu_sssp_labels_noalloc: invalid argument\n");
    return TAPGPU_ERR_ARG;
  }
  if (num_sources == 0) return TAPGPU_OK;
  const size_t slice = tapgpu::sssp_smem_bytes(num_nodes1, true);
  const size_t room = kNoAllocScratchBytes - kControlBytes;
  if (slice > room) {
    fprintf(stderr,
            "tapgpu_sssp_labels_noalloc: %d nodes need %zu bytes of labels per source, more than "
            "the fixed %zu-byte scratch array holds\n",
            num_nodes1, slice, room);
    return TAPGPU_ERR_UNSUPPORTED;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TAPGPU_ERR_NO_DEVICE;
  unsigned char* base = nullptr;
  int rc = scratch_address(dev, &base);
  if (rc != TAPGPU_OK) {
    fprintf(stderr, "tapgpu_sssp_labels_noalloc: cudaGetSymbolAddress failed\n");
    return rc;
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return TAPGPU_ERR_CUDA;
  const int occ = tapgpu::sssp_occupancy(true, kBlock, false, num_nodes1, tapgpu::kSsspRounds);
  int grid = static_cast<int>(room / slice);
  if (occ > 0 && grid > occ * sms) grid = occ * sms;
  if (grid > num_sources) grid = num_sources;
  if (grid < 1) grid = 1;

  int* counter = reinterpret_cast<int*>(base);
  int* err = counter + 1;
  int* err_info = counter + 2;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // indices come from the caller's device memory: check them before any kernel uses them
  if (check_indices(d_row_ptr, int64_t(num_nodes1) + 1, 0, num_links, true, s) != TAPGPU_OK ||
      check_indices(d_head, num_links, 0, num_nodes1 - 1, false, s) != TAPGPU_OK ||
      check_indices(d_sources, num_sources, 0, num_nodes1 - 1, false, s) != TAPGPU_OK) {
    fprintf(stderr,
            "tapgpu_sssp_labels_noalloc: forward star or sources out of range "
            "(row_ptr must run 0..num_links, heads and sources 0..num_nodes1-1)\n");
    return TAPGPU_ERR_ARG;
  }
  // the array keeps the previous call's contents: clear the control block
  if (cudaMemsetAsync(base, 0, kControlBytes, s) != cudaSuccess) return TAPGPU_ERR_CUDA;

  tapgpu::PathArgs a{};
  a.g.n1 = num_nodes1;
  a.g.m = num_links;
  a.g.first_thru = first_thru_node;
  a.g.row_ptr = d_row_ptr;
  a.g.head = d_head;
  a.w64 = d_weight;
  a.sources = d_sources;
  a.num_sources = num_sources;
  a.task_begin = 0;
  a.task_end = num_sources;
  a.dist = d_dist;
  a.counter = counter;
  a.err = err;
  a.err_info = err_info;
  a.max_rounds = num_nodes1 + 2;
  a.scratch = base + kControlBytes;
  a.scratch_stride = static_cast<long long>(slice);
  if (tapgpu::launch_sssp(a, true, grid, kBlock, false, tapgpu::kSsspRounds, s) != cudaSuccess) {
    cudaGetLastError();
    return TAPGPU_ERR_CUDA;
  }
  int e = 0;
  if (cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return TAPGPU_ERR_CUDA;
  return e ? TAPGPU_ERR_NO_CONVERGENCE : TAPGPU_OK;
}
