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
//
// One call = one memset of the control block, one input check kernel, one
// shortest-path launch and one 4-byte status read-back: the caller's stream
// is synchronised once, at the end.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "fw_kernels.cuh"
#include "tap_gpu.h"

namespace {

// 32 MiB: a 256-byte control block (work counter, error word, missing-path
// info) followed by per-CTA label slices of (8 (N+1) + bitmap) bytes each.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
constexpr size_t kControlBytes = 256;
constexpr int kBlock = 256;
constexpr int kCheckBlock = 256;
// error bit of the input check (the path kernels' own bits are below it)
constexpr int kErrBadInput = 1 << 20;
// a work counter this high makes every CTA of the persistent path kernel
// find no task, so it leaves the caller's buffers untouched
constexpr int kNoTasks = 1 << 30;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The array's device address, looked up on every call with the caller's
// device current: in host code the symbol's name stands for the array and is
// not a device address, and a lookup per call stays valid after a device
// reset or under another context.
int scratch_address(unsigned char** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    cudaGetLastError();
    return TAPGPU_ERR_CUDA;
  }
  *out = static_cast<unsigned char*>(p);
  return TAPGPU_OK;
}

// Checks the caller's device-resident indices and weights before the path
// kernel reads them: row_ptr non-decreasing within 0..num_links,
// heads and sources in 0..num_nodes1-1, weights >= 0 (NaN fails).  On a
// failure it sets kErrBadInput and moves the work counter past every task.
__global__ void __launch_bounds__(kCheckBlock)
    k_check_inputs(int n1, int m, const int32_t* row_ptr, const int32_t* head, const double* w,
                   const int32_t* sources, int num_sources, int* counter, int* err) {
  const int64_t n = static_cast<int64_t>(n1) + 1;
  int64_t longest = n > m ? n : m;
  if (num_sources > longest) longest = num_sources;
  bool bad = false;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * kCheckBlock + threadIdx.x; i < longest;
       i += static_cast<int64_t>(gridDim.x) * kCheckBlock) {
    if (i < n) {
      const int32_t r = row_ptr[i];
      bad |= r < 0 || r > m || (i + 1 < n && row_ptr[i + 1] < r);
    }
    if (i < m) {
      const int32_t h = head[i];
      bad |= h < 0 || h >= n1 || !(w[i] >= 0.0);
    }
    if (i < num_sources) {
      const int32_t s = sources[i];
      bad |= s < 0 || s >= n1;
    }
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) {
    atomicOr(err, kErrBadInput);
    atomicExch(counter, kNoTasks);
  }
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
  // the size limit comes first, before any CUDA call
  const size_t slice = tapgpu::sssp_smem_bytes(num_nodes1, true);
  const size_t room = kNoAllocScratchBytes - kControlBytes;
  if (slice > room) {
    fprintf(stderr,
            "tapgpu_sssp_labels_noalloc: %d nodes need %zu bytes of labels per source, more than "
            "the fixed %zu-byte scratch array holds\n",
            num_nodes1, slice, room);
    return TAPGPU_ERR_UNSUPPORTED;
  }
  if (num_sources == 0) return TAPGPU_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TAPGPU_ERR_NO_DEVICE;
  unsigned char* base = nullptr;
  int rc = scratch_address(&base);
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
  // the array keeps the previous call's contents: clear the control block
  if (cudaMemsetAsync(base, 0, kControlBytes, s) != cudaSuccess) return TAPGPU_ERR_CUDA;
  // indices come from the caller's device memory: checked on the device
  // before the path kernel uses them (a failed check leaves it no task)
  {
    int64_t longest = static_cast<int64_t>(num_nodes1) + 1;
    if (num_links > longest) longest = num_links;
    if (num_sources > longest) longest = num_sources;
    int64_t cgrid = (longest + kCheckBlock - 1) / kCheckBlock;
    if (cgrid > 4 * static_cast<int64_t>(sms)) cgrid = 4 * static_cast<int64_t>(sms);
    k_check_inputs<<<static_cast<int>(cgrid), kCheckBlock, 0, s>>>(
        num_nodes1, num_links, d_row_ptr, d_head, d_weight, d_sources, num_sources, counter, err);
    if (cudaGetLastError() != cudaSuccess) return TAPGPU_ERR_CUDA;
  }

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
  if (e & kErrBadInput) {
    fprintf(stderr,
            "tapgpu_sssp_labels_noalloc: forward star, weights or sources out of range "
            "(row_ptr must be non-decreasing within 0..num_links, heads and sources lie in "
            "0..num_nodes1-1, weights >= 0)\n");
    return TAPGPU_ERR_ARG;
  }
  return e ? TAPGPU_ERR_NO_CONVERGENCE : TAPGPU_OK;
}
