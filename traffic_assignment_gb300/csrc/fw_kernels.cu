// fw_kernels.cu - sm_103a kernels of the Frank-Wolfe user-equilibrium loop.
//
//  k_sssp      all-origins shortest paths: one CTA per (scenario, origin) task,
//              persistent over a work counter.  Labels live in shared memory and
//              are corrected in bulk-synchronous rounds over a frontier bitmap;
//              each warp compacts 32 bitmap words with a ballot-free prefix sum
//              and relaxes the out-links of the set bits with shared-memory
//              atomicMin on the label bits (non-negative IEEE values order as
//              unsigned integers).  Replaces tap/sssp_pape.c:284-501 on the CPU
//              and tap/pape_kernels.cu:122-204 on the GPU.
//  k_aon       all-or-nothing loading (tap/tap_frankwolfe_pthread.c:262-310):
//              recovers a deterministic predecessor tree from the labels, walks
//              each OD pair's path accumulating demand per node in shared memory
//              (64-bit fixed point, so the sums are exact and order-free), then
//              scatters node totals onto the predecessor links.
//  k_ls_pass   one pass of the 2^-k line search (tap/tap_functions.c:469-507)
//              fused with the gap, Beckmann objective and VHT reductions
//              (tap/tap_functions.c:83-152, 408-417): every candidate step of
//              the pass is evaluated in the same sweep over the links.
//  k_step      x += lambda*d, BPR cost and derivative update and the
//              shortest-path weights for the next iteration
//              (tap/tap_frankwolfe_pthread.c:737-739, tap/tap_functions.c:55-65).
#include <type_traits>

#include "fw_kernels.cuh"

#include "bpr.cuh"

#include <cfloat>
#include <cstdio>
#include <mutex>
#include <set>
#include <utility>

namespace tapgpu {

namespace {

constexpr unsigned kFull = 0xffffffffu;

template <typename T>
struct DT;
template <>
struct DT<float> {
  using U = unsigned int;
  static constexpr U kInf = 0x7f800000u;
  __device__ static __forceinline__ U bits(float v) { return __float_as_uint(v); }
  __device__ static __forceinline__ float val(U b) { return __uint_as_float(b); }
  __device__ static __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
};
template <>
struct DT<double> {
  using U = unsigned long long;
  static constexpr U kInf = 0x7ff0000000000000ull;
  __device__ static __forceinline__ U bits(double v) {
    return static_cast<U>(__double_as_longlong(v));
  }
  __device__ static __forceinline__ double val(U b) {
    return __longlong_as_double(static_cast<long long>(b));
  }
  __device__ static __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
};

template <typename U>
__device__ __forceinline__ U vload(const U* p) {
  return *reinterpret_cast<const volatile U*>(p);
}

__host__ __device__ __forceinline__ size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

// position of the n-th (0-based) set bit of w; w must have more than n set bits
__device__ __forceinline__ int nth_set_bit(unsigned w, int n) {
  int pos = 0;
  int c = __popc(w & 0xffffu);
  if (n >= c) { n -= c; pos += 16; w >>= 16; }
  c = __popc(w & 0xffu);
  if (n >= c) { n -= c; pos += 8; w >>= 8; }
  c = __popc(w & 0xfu);
  if (n >= c) { n -= c; pos += 4; w >>= 4; }
  c = __popc(w & 0x3u);
  if (n >= c) { n -= c; pos += 2; w >>= 2; }
  c = static_cast<int>(w & 1u);
  if (n >= c) pos += 1;
  return pos;
}

// Edge records of one scenario.  FP32 paths read one packed 8-byte record
// {head, weight bits} per edge; FP64 paths read head and weight separately.
template <typename T>
struct Edges;
template <>
struct Edges<float> {
  const uint2* e;
  __device__ __forceinline__ void load(int i, int& h, float& w) const {
    const uint2 r = __ldg(e + i);
    h = static_cast<int>(r.x);
    w = __uint_as_float(r.y);
  }
  __device__ __forceinline__ float weight(int i) const { return __uint_as_float(__ldg(&e[i].y)); }
};
template <>
struct Edges<double> {
  const int* head;
  const double* w;
  __device__ __forceinline__ void load(int i, int& h, double& x) const {
    h = __ldg(head + i);
    x = __ldg(w + i);
  }
  __device__ __forceinline__ double weight(int i) const { return __ldg(w + i); }
};

template <typename T>
__device__ __forceinline__ Edges<T> edges_of(const PathArgs& a, int scen);
template <>
__device__ __forceinline__ Edges<float> edges_of<float>(const PathArgs& a, int scen) {
  return Edges<float>{a.e32 + static_cast<size_t>(scen) * a.g.m};
}
template <>
__device__ __forceinline__ Edges<double> edges_of<double>(const PathArgs& a, int scen) {
  return Edges<double>{a.g.head, a.w64 + static_cast<size_t>(scen) * a.g.m};
}

// In-links of a node in reverse-star order (link id ascending).  FP32 paths
// read one packed {tail, weight bits} record per in-link; the link id is
// fetched only for the chosen predecessor.
template <typename T>
struct RevEdges;
template <>
struct RevEdges<float> {
  const uint2* r;
  const int* in_link;
  __device__ __forceinline__ void load(int i, int& u, float& w) const {
    const uint2 x = __ldg(r + i);
    u = static_cast<int>(x.x);
    w = __uint_as_float(x.y);
  }
  __device__ __forceinline__ int link(int i) const { return __ldg(in_link + i); }
};
template <>
struct RevEdges<double> {
  const int* in_link;
  const int* tail;
  const double* w;
  __device__ __forceinline__ void load(int i, int& u, double& x) const {
    const int k = __ldg(in_link + i);
    u = __ldg(tail + k);
    x = __ldg(w + k);
  }
  __device__ __forceinline__ int link(int i) const { return __ldg(in_link + i); }
};

template <typename T>
__device__ __forceinline__ RevEdges<T> rev_edges_of(const PathArgs& a, int scen);
template <>
__device__ __forceinline__ RevEdges<float> rev_edges_of<float>(const PathArgs& a, int scen) {
  return RevEdges<float>{a.r32 + static_cast<size_t>(scen) * a.g.m, a.g.in_link};
}
template <>
__device__ __forceinline__ RevEdges<double> rev_edges_of<double>(const PathArgs& a, int scen) {
  return RevEdges<double>{a.g.in_link, a.g.tail, a.w64 + static_cast<size_t>(scen) * a.g.m};
}

constexpr int kEdgeGroup = 4;  // edge records fetched together before relaxing
// predecessor words of k_aon (real ones are below kPredRoot)
constexpr unsigned kPredNone = 0xffffffffu;     // no tight in-link seen yet
constexpr unsigned kPredPending = 0xfffffffeu;  // reached only over zero / absorbed costs
constexpr unsigned kPredRoot = 0xfffffffdu;     // the source, or unreachable

// Relax the out-links of v; returns 1 if any head label dropped.  The edge
// records of a group are all requested before the first atomic so that
// their memory latencies overlap.
template <typename T>
__device__ __forceinline__ int relax_node(int v, int src, const Graph& g, const Edges<T>& ed,
                                          typename DT<T>::U* dist, unsigned* nxt) {
  using U = typename DT<T>::U;
  if (v < g.first_thru && v != src) return 0;  // zones are never passed through
  const int e0 = __ldg(g.row_ptr + v);
  const int e1 = __ldg(g.row_ptr + v + 1);
  const T du = DT<T>::val(vload(dist + v));
  int pushed = 0;
  for (int b = e0; b < e1; b += kEdgeGroup) {
    int hh[kEdgeGroup];
    T ww[kEdgeGroup];
#pragma unroll
    for (int j = 0; j < kEdgeGroup; ++j)
      if (b + j < e1) ed.load(b + j, hh[j], ww[j]);
#pragma unroll
    for (int j = 0; j < kEdgeGroup; ++j) {
      if (b + j >= e1) break;
      const int h = hh[j];
      const U nb = DT<T>::bits(DT<T>::add(du, ww[j]));
      if (nb < vload(dist + h)) {
        const U old = atomicMin(dist + h, nb);
        if (nb < old) {
          const unsigned bit = 1u << (h & 31);
          if (!(vload(nxt + (h >> 5)) & bit)) atomicOr(nxt + (h >> 5), bit);
          pushed = 1;
        }
      }
    }
  }
  return pushed;
}

template <typename T, int BLOCK, bool SMEM>
__global__ void __launch_bounds__(BLOCK) k_sssp(PathArgs a) {
  using U = typename DT<T>::U;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int sh_task;
  const int n1 = a.g.n1;
  const int nwords = (n1 + 31) >> 5;
  unsigned char* base =
      SMEM ? smem_raw
           : static_cast<unsigned char*>(a.scratch) + static_cast<size_t>(blockIdx.x) * a.scratch_stride;
  U* dist = reinterpret_cast<U*>(base);
  unsigned* bm0 = reinterpret_cast<unsigned*>(base + align16(sizeof(U) * n1));
  unsigned* bm1 = bm0 + nwords;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int kWarps = BLOCK / 32;

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) sh_task = atomicAdd(a.counter, 1) + a.task_begin;
    __syncthreads();
    const int task = sh_task;
    if (task >= a.task_end) break;
    const int slot = task / a.num_sources;
    const int scen = a.scen_list ? a.scen_list[slot] : 0;
    if (a.state && a.state[scen].done) continue;
    const int src = a.sources[task - slot * a.num_sources];
    const Edges<T> ed = edges_of<T>(a, scen);
    unsigned expanded = 0;

    for (int v = threadIdx.x; v < n1; v += BLOCK) dist[v] = DT<T>::kInf;
    for (int i = threadIdx.x; i < 2 * nwords; i += BLOCK) bm0[i] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
      dist[src] = DT<T>::bits(T(0));
      bm0[src >> 5] = 1u << (src & 31);
    }
    __syncthreads();

    unsigned* cur = bm0;
    unsigned* nxt = bm1;
    int rounds = 0;
    const int nchunks = (nwords + 31) >> 5;
    for (;;) {
      int pushed = 0;
      for (int c = warp; c < nchunks; c += kWarps) {
        const int wi = (c << 5) + lane;
        unsigned word = 0u;
        if (wi < nwords) {
          word = cur[wi];
          if (word) cur[wi] = 0u;
        }
        const int cnt = __popc(word);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(kFull, incl, o);
          if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        for (int b = 0; b < total; b += 32) {
          const int j = b + lane;
          int owner = 0;  // number of lanes whose inclusive count is <= j
#pragma unroll
          for (int step = 16; step >= 1; step >>= 1) {
            const int probe = __shfl_sync(kFull, incl, owner + step - 1);
            if (probe <= j) owner += step;
          }
          owner &= 31;
          const unsigned ow = __shfl_sync(kFull, word, owner);
          const int oincl = __shfl_sync(kFull, incl, owner);
          if (j < total) {
            const int rank = j - (oincl - __popc(ow));
            const int v = (((c << 5) + owner) << 5) + nth_set_bit(ow, rank);
            pushed |= relax_node<T>(v, src, a.g, ed, dist, nxt);
            ++expanded;
          }
        }
      }
      const int more = __syncthreads_or(pushed);
      if (!more) break;
      unsigned* tmp = cur;
      cur = nxt;
      nxt = tmp;
      if (++rounds > a.max_rounds) {
        if (threadIdx.x == 0) atomicOr(a.err, kErrRounds);
        break;
      }
    }
    T* out = static_cast<T*>(a.dist) + static_cast<size_t>(task - a.task_begin) * n1;
    for (int v = threadIdx.x; v < n1; v += BLOCK) out[v] = DT<T>::val(dist[v]);
    if (a.stats) {  // rounds and node expansions of this task
      for (int o = 16; o >= 1; o >>= 1) expanded += __shfl_down_sync(kFull, expanded, o);
      if (lane == 0) atomicAdd(a.stats + 2, static_cast<unsigned long long>(expanded));
      if (threadIdx.x == 0) {
        atomicAdd(a.stats + 0, static_cast<unsigned long long>(rounds));
        atomicAdd(a.stats + 1, 1ull);
      }
    }
  }
}

// Relax the out-links e0..e1 of v; returns how many frontier bits it turned
// on.  Zones other than the source are never expanded, so their bits are not
// set (their labels still drop).
template <typename T>
__device__ __forceinline__ int relax_range(int src, int e0, int e1, int first_thru,
                                           const Edges<T>& ed, typename DT<T>::U* dist,
                                           unsigned* bm, T du) {
  using U = typename DT<T>::U;
  int pushes = 0;
  for (int b = e0; b < e1; b += kEdgeGroup) {
    int hh[kEdgeGroup];
    T ww[kEdgeGroup];
#pragma unroll
    for (int j = 0; j < kEdgeGroup; ++j)
      if (b + j < e1) ed.load(b + j, hh[j], ww[j]);
#pragma unroll
    for (int j = 0; j < kEdgeGroup; ++j) {
      if (b + j >= e1) break;
      const int h = hh[j];
      const U nb = DT<T>::bits(DT<T>::add(du, ww[j]));
      if (nb < vload(dist + h)) {
        const U old = atomicMin(dist + h, nb);
        if (nb < old && !(h < first_thru && h != src)) {
          const unsigned bit = 1u << (h & 31);
          if (!(vload(bm + (h >> 5)) & bit)) {
            const unsigned prev = atomicOr(bm + (h >> 5), bit);
            if (!(prev & bit)) ++pushes;
          }
        }
      }
    }
  }
  return pushes;
}

// sum over a converged warp, every lane receiving it (one warp-wide reduction
// instruction on this architecture)
__device__ __forceinline__ int warp_sum(int v) { return __reduce_add_sync(kFull, v); }

constexpr long long kMaxIdlePolls = 1ll << 24;  // bound on one warp's idle polling
constexpr int kMaxRestarts = 64;

// All-origins shortest paths without per-round barriers.  Frontier bitmap
// word i belongs to warp i mod W; a warp claims its set bits with atomicExch
// and relaxes those nodes at once, so a label improvement propagates as soon
// as the owner of the head polls (label correction in the style of the
// reference's d'Esopo-Pape queue, made parallel).  `pending` counts frontier
// bits plus claimed-but-unfinished nodes plus reserved pushes: a warp
// reserves deg(v) before relaxing v's links and releases the unused part
// after, so the counter never under-counts and a warp may leave once it reads
// zero.  A final block-wide check that no bit is left makes the result
// independent of the counter (a premature exit costs a restart only).
template <typename T, int BLOCK, bool SMEM>
__global__ void __launch_bounds__(BLOCK) k_sssp_async(PathArgs a) {
  using U = typename DT<T>::U;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int sh_task;
  __shared__ int pending;
  const int n1 = a.g.n1;
  const int nwords = (n1 + 31) >> 5;
  unsigned char* base =
      SMEM ? smem_raw
           : static_cast<unsigned char*>(a.scratch) + static_cast<size_t>(blockIdx.x) * a.scratch_stride;
  U* dist = reinterpret_cast<U*>(base);
  unsigned* bm = reinterpret_cast<unsigned*>(base + align16(sizeof(U) * n1));
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int kWarps = BLOCK / 32;
  const int F = a.g.first_thru;
  const int my_words = warp < nwords ? (nwords - warp + kWarps - 1) / kWarps : 0;

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) sh_task = atomicAdd(a.counter, 1) + a.task_begin;
    __syncthreads();
    const int task = sh_task;
    if (task >= a.task_end) break;
    const int slot = task / a.num_sources;
    const int scen = a.scen_list ? a.scen_list[slot] : 0;
    if (a.state && a.state[scen].done) continue;
    const int src = a.sources[task - slot * a.num_sources];
    const Edges<T> ed = edges_of<T>(a, scen);
    unsigned expanded = 0;
    int passes = 0;

    for (int v = threadIdx.x; v < n1; v += BLOCK) dist[v] = DT<T>::kInf;
    for (int i = threadIdx.x; i < nwords; i += BLOCK) bm[i] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
      dist[src] = DT<T>::bits(T(0));
      bm[src >> 5] = 1u << (src & 31);
      pending = 1;
    }
    __syncthreads();

    for (int restart = 0;; ++restart) {
      long long idle = 0;
      for (;;) {
        int claimed_any = 0;
        for (int j0 = 0; j0 < my_words; j0 += 32) {
          const int j = j0 + lane;
          const int wi = warp + j * kWarps;
          unsigned word = 0u;
          if (j < my_words) {
            word = vload(bm + wi);
            if (word) word = atomicExch(bm + wi, 0u);
          }
          const int cnt = __popc(word);
          int incl = cnt;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += y;
          }
          const int total = __shfl_sync(kFull, incl, 31);
          if (total == 0) continue;
          claimed_any = 1;
          for (int b = 0; b < total; b += 32) {
            const int jj = b + lane;
            int owner = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
              const int probe = __shfl_sync(kFull, incl, owner + step - 1);
              if (probe <= jj) owner += step;
            }
            owner &= 31;
            const unsigned ow = __shfl_sync(kFull, word, owner);
            const int oincl = __shfl_sync(kFull, incl, owner);
            const bool valid = jj < total;
            int v = 0, e0 = 0, e1 = 0;
            if (valid) {
              v = ((warp + (j0 + owner) * kWarps) << 5) + nth_set_bit(ow, jj - (oincl - __popc(ow)));
              if (!(v < F && v != src)) {
                e0 = __ldg(a.g.row_ptr + v);
                e1 = __ldg(a.g.row_ptr + v + 1);
              }
            }
            const int reserve = warp_sum(e1 - e0);
            const int items = warp_sum(valid ? 1 : 0);
            if (lane == 0) {
              atomicAdd(&pending, reserve);
              __threadfence_block();
            }
            __syncwarp();
            int pushes = 0;
            if (e1 > e0) pushes = relax_range<T>(src, e0, e1, F, ed, dist, bm, DT<T>::val(vload(dist + v)));
            expanded += valid ? 1u : 0u;
            const int used = warp_sum(pushes);
            __syncwarp();
            if (lane == 0) {
              __threadfence_block();
              atomicAdd(&pending, -(reserve - used + items));
            }
          }
        }
        if (warp == 0) ++passes;
        if (!claimed_any) {
          if (vload(&pending) <= 0) break;
          if (++idle > kMaxIdlePolls) {
            if (lane == 0) atomicOr(a.err, kErrRounds);
            break;
          }
          __nanosleep(64);
        }
      }
      __syncthreads();
      int left = 0;
      for (int i = threadIdx.x; i < nwords; i += BLOCK) left |= (bm[i] != 0u);
      if (!__syncthreads_or(left)) break;
      if (restart >= kMaxRestarts) {
        if (threadIdx.x == 0) atomicOr(a.err, kErrRounds);
        break;
      }
      // bits remain after every warp left: recount them and resume
      if (threadIdx.x == 0) pending = 0;
      __syncthreads();
      int c = 0;
      for (int i = threadIdx.x; i < nwords; i += BLOCK) c += __popc(bm[i]);
      c = warp_sum(c);
      if (lane == 0) atomicAdd(&pending, c);
      __syncthreads();
    }
    T* out = static_cast<T*>(a.dist) + static_cast<size_t>(task - a.task_begin) * n1;
    for (int v = threadIdx.x; v < n1; v += BLOCK) out[v] = DT<T>::val(dist[v]);
    if (a.stats) {
      for (int o = 16; o >= 1; o >>= 1) expanded += __shfl_down_sync(kFull, expanded, o);
      if (lane == 0) atomicAdd(a.stats + 2, static_cast<unsigned long long>(expanded));
      if (threadIdx.x == 0) {
        atomicAdd(a.stats + 0, static_cast<unsigned long long>(passes));
        atomicAdd(a.stats + 1, 1ull);
      }
    }
  }
}

// Relax the out-links e0..e1 of v for the near-far variant: a head whose new
// label is below the phase threshold goes to the near bitmap (counted in
// the returned pushes), any other head to the far bitmap.
template <typename T>
__device__ __forceinline__ int relax_range_nf(int src, int e0, int e1, int first_thru,
                                              const Edges<T>& ed, typename DT<T>::U* dist,
                                              unsigned* near, unsigned* far, T du,
                                              typename DT<T>::U thr_bits) {
  using U = typename DT<T>::U;
  int pushes = 0;
  for (int b = e0; b < e1; b += kEdgeGroup) {
    int hh[kEdgeGroup];
    T ww[kEdgeGroup];
#pragma unroll
    for (int j = 0; j < kEdgeGroup; ++j)
      if (b + j < e1) ed.load(b + j, hh[j], ww[j]);
#pragma unroll
    for (int j = 0; j < kEdgeGroup; ++j) {
      if (b + j >= e1) break;
      const int h = hh[j];
      const U nb = DT<T>::bits(DT<T>::add(du, ww[j]));
      if (nb < vload(dist + h)) {
        const U old = atomicMin(dist + h, nb);
        if (nb < old && !(h < first_thru && h != src)) {
          const unsigned bit = 1u << (h & 31);
          if (nb < thr_bits) {
            if (!(vload(near + (h >> 5)) & bit)) {
              const unsigned prev = atomicOr(near + (h >> 5), bit);
              if (!(prev & bit)) ++pushes;
            }
          } else if (!(vload(far + (h >> 5)) & bit)) {
            atomicOr(far + (h >> 5), bit);
          }
        }
      }
    }
  }
  return pushes;
}

// All-origins shortest paths, near-far ordering: labels below a threshold T
// are corrected asynchronously (warp-owned near-bitmap words, as in
// k_sssp_async); heads at or above T wait in a far bitmap.  When no near work
// is left, one block-wide step raises T to (smallest far label + delta) and
// promotes the far nodes below it.  Nodes are then expanded close to once
// (the ordering of delta-stepping) instead of once per improvement.  A far
// node may also sit in the near set; expanding it twice is harmless.  The
// result is the same least fixed point as every other variant.
template <typename T, int BLOCK, bool SMEM>
__global__ void __launch_bounds__(BLOCK) k_sssp_nf(PathArgs a) {
  using U = typename DT<T>::U;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int sh_task;
  __shared__ int pending;
  __shared__ U sh_min;
  const int n1 = a.g.n1;
  const int nwords = (n1 + 31) >> 5;
  unsigned char* base =
      SMEM ? smem_raw
           : static_cast<unsigned char*>(a.scratch) + static_cast<size_t>(blockIdx.x) * a.scratch_stride;
  U* dist = reinterpret_cast<U*>(base);
  unsigned* near = reinterpret_cast<unsigned*>(base + align16(sizeof(U) * n1));
  unsigned* far = near + nwords;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int kWarps = BLOCK / 32;
  const int F = a.g.first_thru;
  const int my_words = warp < nwords ? (nwords - warp + kWarps - 1) / kWarps : 0;
  const T delta = static_cast<T>(a.nf_delta);

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) sh_task = atomicAdd(a.counter, 1) + a.task_begin;
    __syncthreads();
    const int task = sh_task;
    if (task >= a.task_end) break;
    const int slot = task / a.num_sources;
    const int scen = a.scen_list ? a.scen_list[slot] : 0;
    if (a.state && a.state[scen].done) continue;
    const int src = a.sources[task - slot * a.num_sources];
    const Edges<T> ed = edges_of<T>(a, scen);
    unsigned expanded = 0;
    unsigned long long polls = 0, batches = 0;
    int phases = 0;

    for (int v = threadIdx.x; v < n1; v += BLOCK) dist[v] = DT<T>::kInf;
    for (int i = threadIdx.x; i < 2 * nwords; i += BLOCK) near[i] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
      dist[src] = DT<T>::bits(T(0));
      near[src >> 5] = 1u << (src & 31);
      pending = 1;
    }
    __syncthreads();
    U thr = DT<T>::bits(delta);

    for (;;) {  // phases
      // -- asynchronous correction of the near set ---------------------------
      long long idle = 0;
      for (;;) {
        int claimed_any = 0;
        for (int j0 = 0; j0 < my_words; j0 += 32) {
          const int j = j0 + lane;
          const int wi = warp + j * kWarps;
          unsigned word = 0u;
          if (j < my_words) {
            word = vload(near + wi);
            if (word) word = atomicExch(near + wi, 0u);
          }
          const int cnt = __popc(word);
          int incl = cnt;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += y;
          }
          const int total = __shfl_sync(kFull, incl, 31);
          if (total == 0) continue;
          claimed_any = 1;
          for (int b = 0; b < total; b += 32) {
            const int jj = b + lane;
            int owner = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
              const int probe = __shfl_sync(kFull, incl, owner + step - 1);
              if (probe <= jj) owner += step;
            }
            owner &= 31;
            const unsigned ow = __shfl_sync(kFull, word, owner);
            const int oincl = __shfl_sync(kFull, incl, owner);
            const bool valid = jj < total;
            int v = 0, e0 = 0, e1 = 0;
            if (valid) {
              v = ((warp + (j0 + owner) * kWarps) << 5) + nth_set_bit(ow, jj - (oincl - __popc(ow)));
              if (!(v < F && v != src)) {
                e0 = __ldg(a.g.row_ptr + v);
                e1 = __ldg(a.g.row_ptr + v + 1);
              }
            }
            const int reserve = warp_sum(e1 - e0);
            const int items = warp_sum(valid ? 1 : 0);
            if (lane == 0) {
              atomicAdd(&pending, reserve);
              __threadfence_block();
            }
            ++batches;
            __syncwarp();
            int pushes = 0;
            if (e1 > e0)
              pushes = relax_range_nf<T>(src, e0, e1, F, ed, dist, near, far,
                                         DT<T>::val(vload(dist + v)), thr);
            expanded += valid ? 1u : 0u;
            const int used = warp_sum(pushes);
            __syncwarp();
            if (lane == 0) {
              __threadfence_block();
              atomicAdd(&pending, -(reserve - used + items));
            }
          }
        }
        if (!claimed_any) {
          if (vload(&pending) <= 0) break;
          ++polls;
          if (++idle > kMaxIdlePolls) {
            if (lane == 0) atomicOr(a.err, kErrRounds);
            break;
          }
          __nanosleep(32);
        }
      }
      __syncthreads();
      // -- phase step: near set empty?  then raise the threshold --------------
      int left = 0;
      for (int i = threadIdx.x; i < nwords; i += BLOCK) left |= (near[i] != 0u);
      if (__syncthreads_or(left)) {  // a warp left early: recount and resume
        if (threadIdx.x == 0) pending = 0;
        __syncthreads();
        int c = 0;
        for (int i = threadIdx.x; i < nwords; i += BLOCK) c += __popc(near[i]);
        c = warp_sum(c);
        if (lane == 0) atomicAdd(&pending, c);
        __syncthreads();
        if (++phases > a.max_rounds) {
          if (threadIdx.x == 0) atomicOr(a.err, kErrRounds);
          break;
        }
        continue;
      }
      // smallest far label (far bits of nodes already settled below it are dropped)
      if (threadIdx.x == 0) sh_min = DT<T>::kInf;
      __syncthreads();
      // A far node whose label is now below the old threshold got that label
      // by a relaxation that also queued it in the near set, so it has been
      // expanded with it: its far bit is stale.
      U mn = DT<T>::kInf;
      for (int i = threadIdx.x; i < nwords; i += BLOCK) {
        const unsigned w = far[i];
        if (!w) continue;
        unsigned keep = 0u, ww = w;
        while (ww) {
          const int bpos = __ffs(ww) - 1;
          ww &= ww - 1;
          const U dv = dist[(i << 5) + bpos];
          if (dv >= thr) {
            keep |= 1u << bpos;
            if (dv < mn) mn = dv;
          }
        }
        if (keep != w) far[i] = keep;
      }
      if (mn != DT<T>::kInf) atomicMin(&sh_min, mn);
      __syncthreads();
      const U fmin = sh_min;
      if (fmin == DT<T>::kInf) break;  // nothing left: labels are final
      thr = DT<T>::bits(DT<T>::add(DT<T>::val(fmin), delta));
      if (thr <= fmin) thr = fmin + 1;  // delta absorbed: still make progress
      // promote far nodes below the new threshold
      int moved = 0;
      for (int i = threadIdx.x; i < nwords; i += BLOCK) {
        const unsigned w = far[i];
        if (!w) continue;
        unsigned take = 0u;
        unsigned ww = w;
        while (ww) {
          const int bpos = __ffs(ww) - 1;
          ww &= ww - 1;
          if (dist[(i << 5) + bpos] < thr) take |= 1u << bpos;
        }
        if (take) {
          far[i] = w & ~take;
          near[i] = take;
          moved += __popc(take);
        }
      }
      if (threadIdx.x == 0) pending = 0;
      __syncthreads();
      moved = warp_sum(moved);
      if (lane == 0 && moved) atomicAdd(&pending, moved);
      __syncthreads();
      if (++phases > a.max_rounds) {
        if (threadIdx.x == 0) atomicOr(a.err, kErrRounds);
        break;
      }
    }
    T* out = static_cast<T*>(a.dist) + static_cast<size_t>(task - a.task_begin) * n1;
    for (int v = threadIdx.x; v < n1; v += BLOCK) out[v] = DT<T>::val(dist[v]);
    if (a.stats) {
      for (int o = 16; o >= 1; o >>= 1) expanded += __shfl_down_sync(kFull, expanded, o);
      if (lane == 0) {
        atomicAdd(a.stats + 2, static_cast<unsigned long long>(expanded));
        atomicAdd(a.stats + 3, polls);
        atomicAdd(a.stats + 4, batches);
      }
      if (threadIdx.x == 0) {
        atomicAdd(a.stats + 0, static_cast<unsigned long long>(phases));
        atomicAdd(a.stats + 1, 1ull);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Near-far with a FIFO of near nodes (k_sssp_nfq)
// ---------------------------------------------------------------------------
// The near bitmap stays the record of which nodes wait for expansion (a set
// bit is a pending node, as in k_sssp_nf); a ring of 16-bit node ids in
// shared memory lists them in push order so that a warp takes 32 at once
// with one compare-and-swap instead of scanning its bitmap words.  A node is
// expanded by whoever clears its bit (atomicAnd / atomicExch), so stale ring
// entries are skipped, and a node that finds the ring full waits in the
// bitmap, where the word scan of k_sssp_nf still finds it.  The ring is an
// accelerator only: losing an entry cannot lose a node.
constexpr int kQCap = kQueueSlots;           // ring slots
// a free ring slot: all ones (16-bit entries serve networks below 65535 nodes)
template <typename R>
struct QEmpty {
  static constexpr R value = static_cast<R>(~static_cast<R>(0));
};
constexpr int kMaxSlotSpins = 1 << 20;       // bound on waiting for one slot

// Append v to the ring unless fewer than BLOCK slots are free (one per
// thread that may be appending at the same time, so no append overruns a
// slot whose previous node has been claimed but not yet read).
template <int BLOCK, typename R>
__device__ __forceinline__ void ring_push(R* ring, unsigned* qhead, unsigned* qtail,
                                          int v, int* err, int* ovf) {
  if constexpr (BLOCK >= kQCap) {
    *reinterpret_cast<volatile int*>(ovf) = 1;  // no room for a margin: the bitmap alone
    return;
  } else {
    if (vload(qtail) - vload(qhead) >= static_cast<unsigned>(kQCap - BLOCK)) {
      *reinterpret_cast<volatile int*>(ovf) = 1;  // v waits in the bitmap only
      return;
    }
    const unsigned pos = atomicAdd(qtail, 1u);
    volatile R* slot = ring + (pos & (kQCap - 1));
    // wait while the previous lap's node is being read; the store is made
    // inside the loop, so that no lane holds its entry back while another
    // lane of its warp is still waiting
    for (int spins = 0;; ++spins) {
      if (*slot == QEmpty<R>::value) {
        *slot = static_cast<R>(v);
        break;
      }
      if (spins >= kMaxSlotSpins) {  // that node may lose its entry: scan the bitmap
        atomicOr(err, kErrRounds);
        *reinterpret_cast<volatile int*>(ovf) = 1;
        *slot = static_cast<R>(v);
        break;
      }
    }
  }
}

template <typename T, int BLOCK, typename R>
__device__ __forceinline__ int relax_range_nfq(int src, int e0, int e1, int first_thru,
                                               const Edges<T>& ed, typename DT<T>::U* dist,
                                               unsigned* near, unsigned* far, T du,
                                               typename DT<T>::U thr_bits, R* ring,
                                               unsigned* qhead, unsigned* qtail, int* err,
                                               int* ovf) {
  using U = typename DT<T>::U;
  int pushes = 0;
  for (int b = e0; b < e1; b += kEdgeGroup) {
    int hh[kEdgeGroup];
    T ww[kEdgeGroup];
#pragma unroll
    for (int j = 0; j < kEdgeGroup; ++j)
      if (b + j < e1) ed.load(b + j, hh[j], ww[j]);
#pragma unroll
    for (int j = 0; j < kEdgeGroup; ++j) {
      if (b + j >= e1) break;
      const int h = hh[j];
      const U nb = DT<T>::bits(DT<T>::add(du, ww[j]));
      if (nb < vload(dist + h)) {
        const U old = atomicMin(dist + h, nb);
        if (nb < old && !(h < first_thru && h != src)) {
          const unsigned bit = 1u << (h & 31);
          if (nb < thr_bits) {
            const unsigned prev = atomicOr(near + (h >> 5), bit);
            if (!(prev & bit)) {
              ++pushes;
              ring_push<BLOCK>(ring, qhead, qtail, h, err, ovf);
            }
          } else {
            atomicOr(far + (h >> 5), bit);
          }
        }
      }
    }
  }
  return pushes;
}

// Expand each lane's claimed node (valid) with the reservation protocol of
// k_sssp_async: `pending` is raised by the out-degree before relaxing, so it
// cannot reach zero while this warp may still push.
template <typename T, int BLOCK, typename R>
__device__ __forceinline__ void nfq_expand(const PathArgs& a, const uint2* e4s, int src, int F,
                                           const Edges<T>& ed,
                                           typename DT<T>::U* dist, unsigned* near,
                                           unsigned* far, typename DT<T>::U thr,
                                           R* ring, unsigned* qhead,
                                           unsigned* qtail, int* pending, int* ovf, int v,
                                           bool valid, unsigned& expanded) {
  const int lane = threadIdx.x & 31;
  const bool expand = valid && !(v < F && v != src);
  // FP32 paths read the padded layout: degree and the first four records in
  // one round trip; FP64 paths read the CSR records
  constexpr bool kPadded = std::is_same<T, float>::value;
  int deg = 0, e0 = 0;
  uint2 r4[4];
  if (expand) {
    if constexpr (kPadded) {
      // with 16-bit ring entries the degree rides in the upper half of the
      // first record's head word (no separate load); else it is read apart
      constexpr bool kDeg16 = std::is_same<R, unsigned short>::value;
      constexpr unsigned kHead = kDeg16 ? 0xffffu : 0xffffffffu;
      const uint4* p = reinterpret_cast<const uint4*>(e4s + static_cast<size_t>(v) * 4);
      const uint4 q0 = __ldg(p), q1 = __ldg(p + 1);
      if constexpr (kDeg16) {
        deg = static_cast<int>(q0.x >> 16);
      } else {
        deg = __ldg(a.g.out_deg + v);
      }
      r4[0] = make_uint2(q0.x & kHead, q0.y);
      r4[1] = make_uint2(q0.z & kHead, q0.w);
      r4[2] = make_uint2(q1.x & kHead, q1.y);
      r4[3] = make_uint2(q1.z & kHead, q1.w);
    } else {
      e0 = __ldg(a.g.row_ptr + v);
      deg = __ldg(a.g.row_ptr + v + 1) - e0;
    }
  }
  // out-degrees and claimed nodes in one sum (degrees < 2^25 per warp)
  const int packed = warp_sum((deg << 6) | (valid ? 1 : 0));
  const int reserve = packed >> 6, items = packed & 63;
  // No fence around the two updates of `pending`: seen out of order they can
  // only make a warp leave the phase early, and the phase step finds any
  // node still in the near bitmap and resumes (fences cost 1 % of the time).
  if (lane == 0) atomicAdd(pending, reserve);
  __syncwarp();
  int pushes = 0;
  if (deg > 0) {
    const T du = DT<T>::val(vload(dist + v));
    if constexpr (kPadded) {
      using U = typename DT<T>::U;
      // groups of four: the padded records first, then (degree > 4, rare on
      // road networks) the node's further CSR records in the same registers
      for (int base = 0;;) {
        // the group's relaxations first, the ring appends of the heads that
        // entered the near set after them: one copy of the append code, and
        // a node enters the ring only once all its group's labels are set
        // (fewer re-expansions)
        unsigned pm = 0u;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (base + j >= deg) break;
          const int h = static_cast<int>(r4[j].x);
          const U nb = DT<T>::bits(DT<T>::add(du, __uint_as_float(r4[j].y)));
          // the atomic alone: its returned value is the check (the kernel is
          // issue-bound: an atomic costs fewer issue slots than a
          // read-before-atomic check that would skip it); likewise below
          const U old = atomicMin(dist + h, nb);
          if (nb < old && !(h < F && h != src)) {
            const unsigned bit = 1u << (h & 31);
            if (nb < thr) {
              const unsigned prev = atomicOr(near + (h >> 5), bit);
              if (!(prev & bit)) pm |= 1u << j;
            } else {
              atomicOr(far + (h >> 5), bit);
            }
          }
        }
        while (pm) {
          const int j = __ffs(pm) - 1;
          pm &= pm - 1;
          ++pushes;
          ring_push<BLOCK>(ring, qhead, qtail, static_cast<int>(r4[j].x), a.err, ovf);
        }
        base += 4;
        if (base >= deg) break;
        const int c0 = __ldg(a.g.row_ptr + v) + base;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (base + j < deg) r4[j] = __ldg(ed.e + c0 + j);
      }
    } else {
      pushes = relax_range_nfq<T, BLOCK>(src, e0, e0 + deg, F, ed, dist, near, far, du, thr,
                                         ring, qhead, qtail, a.err, ovf);
    }
  }
  expanded += valid ? 1u : 0u;
  const int used = warp_sum(pushes);
  __syncwarp();
  if (lane == 0) atomicAdd(pending, -(reserve - used + items));
}

// five 256-thread CTAs per SM fit the shared memory of a 10k-node network:
// keep registers to that occupancy.  SPLIT (labels too large for shared
// memory): the labels live in the CTA's global scratch slice, the near/far
// bitmaps and the ring in shared memory, so that only the label atomics go
// to L2.
template <typename T, int BLOCK, bool SMEM, typename R, bool SPLIT = false>
__global__ void __launch_bounds__(BLOCK, (1280 / BLOCK > 0 ? 1280 / BLOCK : 1)) k_sssp_nfq(PathArgs a) {
  static_assert(!(SMEM && SPLIT), "the split layout keeps the labels in global memory");
  using U = typename DT<T>::U;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int sh_task;
  __shared__ int pending;
  __shared__ U sh_min;
  __shared__ unsigned qhead, qtail;
  __shared__ int ovf;  // some near node of this phase is in the bitmap only
  const int n1 = a.g.n1;
  const int nwords = (n1 + 31) >> 5;
  unsigned char* base =
      SMEM ? smem_raw
           : static_cast<unsigned char*>(a.scratch) + static_cast<size_t>(blockIdx.x) * a.scratch_stride;
  U* dist = reinterpret_cast<U*>(base);
  unsigned* near = reinterpret_cast<unsigned*>(SPLIT ? smem_raw : base + align16(sizeof(U) * n1));
  unsigned* far = near + nwords;
  R* ring = reinterpret_cast<R*>(far + nwords);
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int kWarps = BLOCK / 32;
  const int F = a.g.first_thru;
  const int my_words = warp < nwords ? (nwords - warp + kWarps - 1) / kWarps : 0;
  const T delta = static_cast<T>(a.nf_delta);

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) sh_task = atomicAdd(a.counter, 1) + a.task_begin;
    __syncthreads();
    const int task = sh_task;
    if (task >= a.task_end) break;
    const int slot = task / a.num_sources;
    const int scen = a.scen_list ? a.scen_list[slot] : 0;
    if (a.state && a.state[scen].done) continue;
    const int src = a.sources[task - slot * a.num_sources];
    const Edges<T> ed = edges_of<T>(a, scen);
    // this scenario's padded records (FP32 paths only)
    const uint2* e4s = a.e4 ? a.e4 + static_cast<size_t>(scen) * n1 * 4 : nullptr;
    unsigned expanded = 0;
    unsigned polls = 0, batches = 0, scanned = 0;  // per task: 32 bits suffice
    int phases = 0;

    for (int v = threadIdx.x; v < n1; v += BLOCK) dist[v] = DT<T>::kInf;
    for (int i = threadIdx.x; i < 2 * nwords; i += BLOCK) near[i] = 0u;
    for (int i = threadIdx.x; i < kQCap; i += BLOCK) ring[i] = QEmpty<R>::value;
    __syncthreads();
    if (threadIdx.x == 0) {
      dist[src] = DT<T>::bits(T(0));
      near[src >> 5] = 1u << (src & 31);
      pending = 1;
      ring[0] = static_cast<R>(src);
      qhead = 0u;
      qtail = 1u;
      ovf = 0;
    }
    __syncthreads();
    U thr = DT<T>::bits(delta);

    for (;;) {  // phases
      int idle = 0;
      for (;;) {
        int claimed_any = 0;
        // -- batches of up to 32 nodes from the ring ---------------------------
        for (;;) {
          unsigned h = 0u;
          int n = 0;
          if (lane == 0) {
            for (int tries = 0; tries < 64; ++tries) {
              h = vload(&qhead);
              const int avail = static_cast<int>(vload(&qtail) - h);
              if (avail <= 0) break;
              const int take = avail < 32 ? avail : 32;
              if (atomicCAS(&qhead, h, h + static_cast<unsigned>(take)) == h) {
                n = take;
                break;
              }
            }
          }
          n = __shfl_sync(kFull, n, 0);
          if (n == 0) break;
          h = __shfl_sync(kFull, h, 0);
          claimed_any = 1;
          int v = 0;
          bool valid = false;
          if (lane < n) {
            volatile R* sl = ring + ((h + static_cast<unsigned>(lane)) & (kQCap - 1));
            // wait for the entry and take it out in the same step (no lane
            // keeps a slot full while another lane of its warp waits)
            int e = -1;
            for (int spins = 0; spins <= kMaxSlotSpins; ++spins) {
              const R q = *sl;
              if (q != QEmpty<R>::value) {
                *sl = QEmpty<R>::value;
                e = q;
                break;
              }
            }
            if (e >= 0) {
              v = e;
              const unsigned bit = 1u << (v & 31);
              valid = (atomicAnd(near + (v >> 5), ~bit) & bit) != 0u;
            } else {  // the entry never arrived: its node is found by the scan
              atomicOr(a.err, kErrRounds);
              *reinterpret_cast<volatile int*>(&ovf) = 1;
            }
          }
          ++batches;
          nfq_expand<T, BLOCK>(a, e4s, src, F, ed, dist, near, far, thr, ring, &qhead, &qtail,
                               &pending, &ovf, v, valid, expanded);
        }
        // -- nodes that found the ring full: scan this warp's bitmap words ------
        // decisions on shared flags are made on lane 0's reading, for the whole warp
        const int scan_words = __shfl_sync(kFull, vload(&ovf), 0) ? my_words : 0;
        for (int j0 = 0; j0 < scan_words; j0 += 32) {
          const int j = j0 + lane;
          const int wi = warp + j * kWarps;
          unsigned word = 0u;
          if (j < my_words) {
            word = vload(near + wi);
            if (word) word = atomicExch(near + wi, 0u);
          }
          const int cnt = __popc(word);
          int incl = cnt;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += y;
          }
          const int total = __shfl_sync(kFull, incl, 31);
          if (total == 0) continue;
          claimed_any = 1;
          for (int b = 0; b < total; b += 32) {
            const int jj = b + lane;
            int owner = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
              const int probe = __shfl_sync(kFull, incl, owner + step - 1);
              if (probe <= jj) owner += step;
            }
            owner &= 31;
            const unsigned ow = __shfl_sync(kFull, word, owner);
            const int oincl = __shfl_sync(kFull, incl, owner);
            const bool valid = jj < total;
            int v = 0;
            if (valid)
              v = ((warp + (j0 + owner) * kWarps) << 5) + nth_set_bit(ow, jj - (oincl - __popc(ow)));
            ++batches;
            scanned += valid ? 1u : 0u;
            nfq_expand<T, BLOCK>(a, e4s, src, F, ed, dist, near, far, thr, ring, &qhead, &qtail,
                                 &pending, &ovf, v, valid, expanded);
          }
        }
        if (!claimed_any) {
          if (__shfl_sync(kFull, vload(&pending), 0) <= 0) break;
          ++polls;
          if (++idle > kMaxIdlePolls) {
            if (lane == 0) atomicOr(a.err, kErrRounds);
            break;
          }
          __nanosleep(32);
        }
      }
      __syncthreads();
      // -- phase step (as k_sssp_nf), promoted nodes also go to the ring ---------
      int left = 0;
      for (int i = threadIdx.x; i < nwords; i += BLOCK) left |= (near[i] != 0u);
      if (__syncthreads_or(left)) {  // a warp left early: recount and resume
        if (threadIdx.x == 0) {
          pending = 0;
          ovf = 1;  // the bits left may have no ring entry
        }
        __syncthreads();
        int c = 0;
        for (int i = threadIdx.x; i < nwords; i += BLOCK) c += __popc(near[i]);
        c = warp_sum(c);
        if (lane == 0) atomicAdd(&pending, c);
        __syncthreads();
        if (++phases > a.max_rounds) {
          if (threadIdx.x == 0) atomicOr(a.err, kErrRounds);
          break;
        }
        continue;
      }
      if (threadIdx.x == 0) {
        sh_min = DT<T>::kInf;
        ovf = 0;  // every near node of the finished phase has been expanded
      }
      __syncthreads();
      U mn = DT<T>::kInf;
      for (int i = threadIdx.x; i < nwords; i += BLOCK) {
        const unsigned w = far[i];
        if (!w) continue;
        unsigned keep = 0u, ww = w;
        while (ww) {
          const int bpos = __ffs(ww) - 1;
          ww &= ww - 1;
          const U dv = dist[(i << 5) + bpos];
          if (dv >= thr) {
            keep |= 1u << bpos;
            if (dv < mn) mn = dv;
          }
        }
        if (keep != w) far[i] = keep;
      }
      if (mn != DT<T>::kInf) atomicMin(&sh_min, mn);
      __syncthreads();
      const U fmin = sh_min;
      if (fmin == DT<T>::kInf) break;  // nothing left: labels are final
      thr = DT<T>::bits(DT<T>::add(DT<T>::val(fmin), delta));
      if (thr <= fmin) thr = fmin + 1;
      int moved = 0;
      for (int i = threadIdx.x; i < nwords; i += BLOCK) {
        const unsigned w = far[i];
        if (!w) continue;
        unsigned take = 0u;
        unsigned ww = w;
        while (ww) {
          const int bpos = __ffs(ww) - 1;
          ww &= ww - 1;
          if (dist[(i << 5) + bpos] < thr) take |= 1u << bpos;
        }
        if (take) {
          far[i] = w & ~take;
          near[i] = take;
          moved += __popc(take);
          unsigned tt = take;
          while (tt) {
            const int bpos = __ffs(tt) - 1;
            tt &= tt - 1;
            ring_push<BLOCK>(ring, &qhead, &qtail, (i << 5) + bpos, a.err, &ovf);
          }
        }
      }
      if (threadIdx.x == 0) pending = 0;
      __syncthreads();
      moved = warp_sum(moved);
      if (lane == 0 && moved) atomicAdd(&pending, moved);
      __syncthreads();
      if (++phases > a.max_rounds) {
        if (threadIdx.x == 0) atomicOr(a.err, kErrRounds);
        break;
      }
    }
    T* out = static_cast<T*>(a.dist) + static_cast<size_t>(task - a.task_begin) * n1;
    for (int v = threadIdx.x; v < n1; v += BLOCK) out[v] = DT<T>::val(dist[v]);
    if (a.stats) {
      for (int o = 16; o >= 1; o >>= 1) expanded += __shfl_down_sync(kFull, expanded, o);
      if (lane == 0) {
        atomicAdd(a.stats + 2, static_cast<unsigned long long>(expanded));
        atomicAdd(a.stats + 3, static_cast<unsigned long long>(polls));
        atomicAdd(a.stats + 4, static_cast<unsigned long long>(batches));
        atomicAdd(a.stats + 5, static_cast<unsigned long long>(scanned));
      }
      if (threadIdx.x == 0) {
        atomicAdd(a.stats + 0, static_cast<unsigned long long>(phases));
        atomicAdd(a.stats + 1, 1ull);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// k_sssp_small: Bellman-Ford sweeps over an edge list held in shared memory
// ---------------------------------------------------------------------------
// For small networks, whose tasks are too small to keep a queue busy (a
// 416-node network has a few dozen origins: one task per SM and nothing to
// hide a queue's latency), the CTA copies the edge list {tail, head,
// weight} of its task's scenario into shared memory and relaxes every edge
// in sweeps until one changes no label.  Labels improve in place during a
// sweep (atomicMin), so an improvement travels along later edges of the same
// sweep; a sweep that changes nothing ends the task.  The labels are the
// same least fixed point of the relaxations as every other schedule's.
template <typename T, int BLOCK, bool SMEM>
__global__ void __launch_bounds__(BLOCK) k_sssp_small(PathArgs a) {
  using U = typename DT<T>::U;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int sh_task;
  const int n1 = a.g.n1, m = a.g.m;
  unsigned char* base =
      SMEM ? smem_raw
           : static_cast<unsigned char*>(a.scratch) + static_cast<size_t>(blockIdx.x) * a.scratch_stride;
  U* dist = reinterpret_cast<U*>(base);
  int* et = reinterpret_cast<int*>(base + align16(sizeof(U) * n1));
  int* eh = et + m;
  T* ew = reinterpret_cast<T*>(base + align16(sizeof(U) * n1) + align16(8 * static_cast<size_t>(m)));
  const int F = a.g.first_thru;
  for (int k = threadIdx.x; k < m; k += BLOCK) et[k] = __ldg(a.g.tail + k);
  int staged = -1;  // scenario whose weights are in shared memory

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) sh_task = atomicAdd(a.counter, 1) + a.task_begin;
    __syncthreads();
    const int task = sh_task;
    if (task >= a.task_end) break;
    const int slot = task / a.num_sources;
    const int scen = a.scen_list ? a.scen_list[slot] : 0;
    if (a.state && a.state[scen].done) continue;
    const int src = a.sources[task - slot * a.num_sources];
    if (scen != staged) {  // (uniform)
      const Edges<T> ed = edges_of<T>(a, scen);
      for (int k = threadIdx.x; k < m; k += BLOCK) {
        int h;
        T w;
        ed.load(k, h, w);
        eh[k] = h;
        ew[k] = w;
      }
      staged = scen;
    }
    for (int v = threadIdx.x; v < n1; v += BLOCK) dist[v] = DT<T>::kInf;
    __syncthreads();
    if (threadIdx.x == 0) dist[src] = DT<T>::bits(T(0));
    __syncthreads();
    int sweeps = 0;
    for (;;) {
      int changed = 0;
      for (int k = threadIdx.x; k < m; k += BLOCK) {
        const int u = et[k];
        if (u < F && u != src) continue;  // zones are never passed through
        const U du = vload(dist + u);
        if (du == DT<T>::kInf) continue;
        const U nb = DT<T>::bits(DT<T>::add(DT<T>::val(du), ew[k]));
        const int h = eh[k];
        if (nb < vload(dist + h) && nb < atomicMin(dist + h, nb)) changed = 1;
      }
      ++sweeps;
      if (!__syncthreads_or(changed)) break;
      if (sweeps > n1 + 1) {  // (cannot happen with non-negative weights)
        if (threadIdx.x == 0) atomicOr(a.err, kErrRounds);
        break;
      }
    }
    T* out = static_cast<T*>(a.dist) + static_cast<size_t>(task - a.task_begin) * n1;
    for (int v = threadIdx.x; v < n1; v += BLOCK) out[v] = DT<T>::val(dist[v]);
    if (a.stats && threadIdx.x == 0) {
      atomicAdd(a.stats + 0, static_cast<unsigned long long>(sweeps));
      atomicAdd(a.stats + 1, 1ull);
    }
  }
}

constexpr unsigned short kNoParent16 = 0xffffu;  // node ids are below 65535 in the compact layout

template <bool COMPACT>
__device__ __forceinline__ int parent_of(const int* parent, const unsigned short* par16, int v) {
  if constexpr (COMPACT) {
    const unsigned short p = par16[v];
    return p == kNoParent16 ? -1 : static_cast<int>(p);
  } else {
    return parent[v];
  }
}

// COMPACT (at most 65535 nodes): 10 bytes per node, so that two CTAs share
// an SM up to ~11,500 nodes and one task's longest walks overlap another
// task's work.  FP32 labels: 8 bytes per node hold the labels and the
// predecessor words, the labels' half later the 32-bit node totals; FP64
// labels (with the padded in-link records): 8 bytes per node hold the labels,
// later the 64-bit totals, and the predecessor words go to the task's slot of
// the label buffer, free once its labels are in shared memory (its second
// half serves as scratch); parents are 16-bit.  Otherwise 16 bytes per node:
// totals (labels first), predecessor links, parents (12 bytes with FP32
// labels, whose totals are 32-bit).
template <typename T, int BLOCK, bool SMEM, bool COMPACT>
__global__ void __launch_bounds__(BLOCK, COMPACT ? (sizeof(T) == 4 ? 2048 : 1024) / BLOCK : 1)
    k_aon(PathArgs a) {
  constexpr bool kPredGlobal = COMPACT && sizeof(T) == 8;  // predecessor words in the label slot
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int sh_task;
  __shared__ unsigned long long sh_red[BLOCK / 32];
  const int n1 = a.g.n1;
  unsigned char* base =
      SMEM ? smem_raw
           : static_cast<unsigned char*>(a.scratch) + static_cast<size_t>(blockIdx.x) * a.scratch_stride;
  T* dS = reinterpret_cast<T*>(base);                         // labels, then ...
  long long* thr = reinterpret_cast<long long*>(base);        // ... node throughput
  int* pred = COMPACT
                  ? reinterpret_cast<int*>(base + 4 * static_cast<size_t>(n1))
                  : reinterpret_cast<int*>(base + align16(sizeof(T) * static_cast<size_t>(n1)));
  int* parent = pred + n1;  // (16- or 12-byte layout)
  unsigned short* par16 = reinterpret_cast<unsigned short*>(base + align16(8 * static_cast<size_t>(n1)));
  const int F = a.g.first_thru;

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) sh_task = atomicAdd(a.counter, 1) + a.task_begin;
    __syncthreads();
    const int task = sh_task;
    if (task >= a.task_end) break;
    const int slot = task / a.num_sources;
    const int scen = a.scen_list ? a.scen_list[slot] : 0;
    if (a.state && a.state[scen].done) continue;
    const int sidx = task - slot * a.num_sources;
    const int src = a.sources[sidx];
    const Edges<T> ed = edges_of<T>(a, scen);
    const RevEdges<T> rv = rev_edges_of<T>(a, scen);
    const T* din = static_cast<const T*>(a.dist) + static_cast<size_t>(task - a.task_begin) * n1;
    // COMPACT: the slot's labels are copied below; it then serves as scratch
    // (FP64: its first half holds the predecessor words)
    int* gslot = reinterpret_cast<int*>(const_cast<T*>(din));
    int* scr = COMPACT ? (kPredGlobal ? gslot + n1 : gslot) : parent;
    int* predw = kPredGlobal ? gslot : pred;

    // labels in, several loads in flight per thread; predecessors cleared
    {
      int v = threadIdx.x;
      for (; v + 3 * BLOCK < n1; v += 4 * BLOCK) {
        const T x0 = din[v], x1 = din[v + BLOCK], x2 = din[v + 2 * BLOCK], x3 = din[v + 3 * BLOCK];
        dS[v] = x0;
        dS[v + BLOCK] = x1;
        dS[v + 2 * BLOCK] = x2;
        dS[v + 3 * BLOCK] = x3;
      }
      for (; v < n1; v += BLOCK) dS[v] = din[v];
    }
    // Predecessor words: the link id, or (link << 16 | tail) when links and
    // nodes both fit 16 bits (the compact layout), so that the parents need
    // no lookup of the link's tail; the minimum still orders by link.
    const bool pack = COMPACT && a.g.m <= 0xffff;
    unsigned* up = reinterpret_cast<unsigned*>(predw);
    int pend = 0;
    bool by_node = false;
    if constexpr (COMPACT && sizeof(T) == 4) {
      if (pack && a.r4) {
        // The same predecessors, node by node: each node's first four
        // in-links come from one padded 32-byte block of {link << 16 | tail,
        // weight} records (in link order; the first word is the predecessor
        // word itself), further in-links from the reverse-star records; the
        // first tight one is the lowest-numbered, so each node's word is
        // written once, without atomics, and the settling of roots and
        // pending nodes happens in the same pass.
        by_node = true;
        __syncthreads();  // (labels in)
        const uint4* r4s = reinterpret_cast<const uint4*>(a.r4 + static_cast<size_t>(scen) * n1 * 4);
        // one node's word from its padded block (slots past its in-links
        // have an infinite weight) and, when it has more, its later in-links
        auto node_word = [&](int v, T dv, uint4 q0, uint4 q1) -> unsigned {
          if (v == src || DT<T>::bits(dv) == DT<T>::kInf) return kPredRoot;
          const unsigned wx[4] = {q0.x, q0.z, q1.x, q1.z};
          const unsigned wb[4] = {q0.y, q0.w, q1.y, q1.w};
          unsigned p = kPredNone;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int u = static_cast<int>(wx[j] & 0xffffu);
            if (p == kPredNone && !(u < F && u != src)) {
              const T du = dS[u];
              if (du < dv && DT<T>::add(du, __uint_as_float(wb[j])) == dv) p = wx[j];
            }
          }
          if (p == kPredNone && ((__ldg(a.r4_more + (v >> 5)) >> (v & 31)) & 1u)) {
            const int i1 = __ldg(a.g.in_ptr + v + 1);
            for (int i = __ldg(a.g.in_ptr + v) + 4; p == kPredNone && i < i1; ++i) {
              int u;
              T w;
              rv.load(i, u, w);
              if (u < F && u != src) continue;
              const T du = dS[u];
              if (du < dv && DT<T>::add(du, w) == dv)
                p = (static_cast<unsigned>(rv.link(i)) << 16) | static_cast<unsigned>(u);
            }
          }
          if (p == kPredNone) {
            pend = 1;
            return kPredPending;
          }
          return p;
        };
        for (int v = threadIdx.x; v < n1; v += BLOCK)
          up[v] = node_word(v, dS[v], __ldg(r4s + 2 * v), __ldg(r4s + 2 * v + 1));
      }
    }
    if constexpr (kPredGlobal) {
      if (a.r4d) {
        // FP64 labels, node by node as above: a node's first four in-links
        // are one padded 64-byte block of {link, tail, weight} records; each
        // node's word goes once, without atomics, to the label slot
        by_node = true;
        __syncthreads();  // (labels in: the slot is free from here)
        const uint4* r4s = a.r4d + static_cast<size_t>(scen) * n1 * 4;
        for (int v = threadIdx.x; v < n1; v += BLOCK) {
          const T dv = dS[v];
          unsigned p = kPredRoot;
          if (v != src && DT<T>::bits(dv) != DT<T>::kInf) {
            p = kPredNone;
            uint4 r[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) r[j] = __ldg(r4s + 4 * static_cast<size_t>(v) + j);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int u = static_cast<int>(r[j].y);
              if (p == kPredNone && !(u < F && u != src)) {
                const T du = dS[u];
                const T w = __hiloint2double(static_cast<int>(r[j].w), static_cast<int>(r[j].z));
                if (du < dv && DT<T>::add(du, w) == dv) p = pack ? (r[j].x << 16) | r[j].y : r[j].x;
              }
            }
            if (p == kPredNone && ((__ldg(a.r4_more + (v >> 5)) >> (v & 31)) & 1u)) {
              const int i1 = __ldg(a.g.in_ptr + v + 1);
              for (int i = __ldg(a.g.in_ptr + v) + 4; p == kPredNone && i < i1; ++i) {
                int u;
                T w;
                rv.load(i, u, w);
                if (u < F && u != src) continue;
                const T du = dS[u];
                if (du < dv && DT<T>::add(du, w) == dv) {
                  const unsigned k = static_cast<unsigned>(rv.link(i));
                  p = pack ? (k << 16) | static_cast<unsigned>(u) : k;
                }
              }
            }
            if (p == kPredNone) {
              p = kPredPending;
              pend = 1;
            }
          }
          up[v] = p;
        }
      }
    }
    if (!by_node) {
      if constexpr (kPredGlobal) __syncthreads();  // (the words overwrite the slot's labels)
      for (int v = threadIdx.x; v < n1; v += BLOCK) up[v] = kPredNone;
      __syncthreads();

      // Predecessor = lowest-numbered tight in-link from a strictly closer tail:
      // one sweep over the reverse-star slots (contiguous records, in link order
      // within a node), keeping the smallest tight link of each head.
      {
        const int m = a.g.m;
        for (int i0 = threadIdx.x; i0 < m; i0 += kEdgeGroup * BLOCK) {
          int vv[kEdgeGroup], uu[kEdgeGroup];
          T ww[kEdgeGroup];
  #pragma unroll
          for (int j = 0; j < kEdgeGroup; ++j) {
            const int i = i0 + j * BLOCK;
            vv[j] = -1;
            uu[j] = 0;
            if (i < m) {
              vv[j] = __ldg(a.g.in_head + i);
              rv.load(i, uu[j], ww[j]);
            }
          }
  #pragma unroll
          for (int j = 0; j < kEdgeGroup; ++j) {
            const int v = vv[j], u = uu[j];
            if (v < 0 || v == src || (u < F && u != src)) continue;
            const T dv = dS[v], du = dS[u];
            if (du < dv && DT<T>::add(du, ww[j]) == dv) {
              const unsigned k = static_cast<unsigned>(rv.link(i0 + j * BLOCK));
              atomicMin(up + v, pack ? (k << 16) | static_cast<unsigned>(u) : k);
            }
          }
        }
      }
      __syncthreads();
      {
        auto settle = [&](int v, unsigned p, T d) {
          if (v == src || DT<T>::bits(d) == DT<T>::kInf) {
            p = kPredRoot;
          } else if (p == kPredNone) {
            p = kPredPending;
            pend = 1;
          }
          up[v] = p;
        };
        int v = threadIdx.x;
        if constexpr (!SMEM) {  // global layout: four nodes' words and labels in flight
          for (; v + 3 * BLOCK < n1; v += 4 * BLOCK) {
            unsigned p[4];
            T d[4];
  #pragma unroll
            for (int j = 0; j < 4; ++j) {
              p[j] = up[v + j * BLOCK];
              d[j] = dS[v + j * BLOCK];
            }
  #pragma unroll
            for (int j = 0; j < 4; ++j) settle(v + j * BLOCK, p[j], d[j]);
          }
        }
        for (; v < n1; v += BLOCK) settle(v, up[v], dS[v]);
      }
    }
    pend = __syncthreads_or(pend);
    // Rare: labels reached only over links too short to change them (zero or
    // absorbed costs).  Attach such nodes level by level to already attached
    // nodes of equal label, lowest link first, so the tree stays acyclic.
    int guard = 0;
    while (pend) {
      for (int v = threadIdx.x; v < n1; v += BLOCK) {
        if (up[v] != kPredPending) continue;
        unsigned c = kPredPending;
        const T dv = dS[v];
        const int i1 = __ldg(a.g.in_ptr + v + 1);
        for (int i = __ldg(a.g.in_ptr + v); i < i1; ++i) {
          const int k = __ldg(a.g.in_link + i);
          const int u = __ldg(a.g.tail + k);
          if (u < F && u != src) continue;
          if (!(u == src || up[u] < kPredRoot)) continue;
          if (DT<T>::add(dS[u], ed.weight(k)) == dv) {
            c = pack ? (static_cast<unsigned>(k) << 16) | static_cast<unsigned>(u)
                     : static_cast<unsigned>(k);
            break;
          }
        }
        scr[v] = static_cast<int>(c);
      }
      __syncthreads();
      int progress = 0, still = 0;
      for (int v = threadIdx.x; v < n1; v += BLOCK) {
        if (up[v] != kPredPending) continue;
        const unsigned c = static_cast<unsigned>(scr[v]);
        if (c != kPredPending) {
          up[v] = c;
          progress = 1;
        } else {
          still = 1;
        }
      }
      const int any_progress = __syncthreads_or(progress);
      const int any_still = __syncthreads_or(still);
      if (!any_still) break;
      if (!any_progress || ++guard > n1) {
        if (threadIdx.x == 0) atomicOr(a.err, kErrPending);
        break;
      }
    }
    __syncthreads();  // (COMPACT: the scratch reads of the loop above precede the links' writes)
    {
      int v = threadIdx.x;
      if constexpr (!SMEM && !COMPACT) {  // four nodes' words, then their tails, in flight
        for (; v + 3 * BLOCK < n1; v += 4 * BLOCK) {
          unsigned p[4];
          int u[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) p[j] = up[v + j * BLOCK];
#pragma unroll
          for (int j = 0; j < 4; ++j) u[j] = p[j] < kPredRoot ? __ldg(a.g.tail + p[j]) : -1;
#pragma unroll
          for (int j = 0; j < 4; ++j) parent[v + j * BLOCK] = u[j];
        }
      }
      for (; v < n1; v += BLOCK) {
        const unsigned p = up[v];
        const bool ok = p < kPredRoot;
        if constexpr (COMPACT) {
          par16[v] = ok ? static_cast<unsigned short>(pack ? (p & 0xffffu) : __ldg(a.g.tail + p))
                        : kNoParent16;
        } else {
          parent[v] = ok ? __ldg(a.g.tail + p) : -1;
        }
      }
    }
    if (a.pred_out) {
      int* po = a.pred_out + static_cast<size_t>(task - a.task_begin) * n1;
      for (int v = threadIdx.x; v < n1; v += BLOCK) {
        const unsigned p = up[v];
        po[v] = p < kPredRoot ? static_cast<int>(pack ? p >> 16 : p) : -1;
      }
    }
    __syncthreads();  // labels no longer needed: their space becomes the node totals
    if (!a.do_load) continue;
    const int j0 = __ldg(a.dem.od_ptr + sidx), j1 = __ldg(a.dem.od_ptr + sidx + 1);
    const long long* oq = a.dem.od_q + scen * a.dem.q_stride;
    // FP32 paths: 32-bit node totals in units of 2^kshift of the
    // fixed point, kshift the smallest that keeps this origin's whole demand
    // below 2^31, so that a walk step is one 32-bit add without a return
    // value.  Each OD demand is rounded to the nearest unit (for a 10k-node
    // network about 1e-6 trips; no bias, and the roundings of at most 2^31
    // OD pairs keep every total below 2^32): far inside the FP32-path
    // tolerance, and the sums stay exact integers, independent of order.
    // FP64 paths: 64-bit totals.
    constexpr bool kWalk32 = std::is_same<T, float>::value;
    unsigned* tot32 = reinterpret_cast<unsigned*>(base);
    int kshift = 0;
    if constexpr (kWalk32) {
      unsigned long long tq = 0;
      for (int j = j0 + threadIdx.x; j < j1; j += BLOCK)
        tq += static_cast<unsigned long long>(__ldg(oq + j));
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) tq += __shfl_xor_sync(kFull, tq, o);
      if ((threadIdx.x & 31) == 0) sh_red[threadIdx.x >> 5] = tq;
      for (int v = threadIdx.x; v < n1; v += BLOCK) tot32[v] = 0u;
      __syncthreads();
      unsigned long long total = 0;
#pragma unroll
      for (int w = 0; w < BLOCK / 32; ++w) total += sh_red[w];
      kshift = total ? 64 - __clzll(static_cast<long long>(total)) - 31 : 0;
      if (kshift < 0) kshift = 0;
    } else {
      for (int v = threadIdx.x; v < n1; v += BLOCK) thr[v] = 0;
      __syncthreads();
    }

    for (int j = j0 + threadIdx.x; j < j1; j += BLOCK) {
      const int dest = __ldg(a.dem.od_dest + j);
      if (dest == src || !(__ldg(a.dem.od_dem + j) > 0.0)) continue;
      const unsigned long long q = static_cast<unsigned long long>(__ldg(oq + j));
      if (q == 0 && a.dem.q_stride) continue;  // a demand scenario removed this OD pair
      if (dest < 0 || dest >= n1 || parent_of<COMPACT>(parent, par16, dest) < 0) {
        atomicOr(a.err, kErrNoPath);
        a.err_info[0] = src;
        a.err_info[1] = dest;
        continue;
      }
      if constexpr (kWalk32) {
        const unsigned qk =
            static_cast<unsigned>(kshift ? (q + (1ull << (kshift - 1))) >> kshift : q);
        if (qk == 0) continue;  // below this task's unit
        int v = dest;
        int steps = 0;
        while (v != src) {
          if (v < 0 || ++steps > n1) {
            atomicOr(a.err, kErrWalk);
            break;
          }
          atomicAdd(tot32 + v, qk);
          v = parent_of<COMPACT>(parent, par16, v);
        }
      } else {
        const unsigned q_lo = static_cast<unsigned>(q), q_hi = static_cast<unsigned>(q >> 32);
        int v = dest;
        int steps = 0;
        while (v != src) {
          if (v < 0 || ++steps > n1) {
            atomicOr(a.err, kErrWalk);
            break;
          }
          // 64-bit total as two native 32-bit adds; a wrapped low word carries
          unsigned* t32 = reinterpret_cast<unsigned*>(thr + v);
          const unsigned old_lo = atomicAdd(t32, q_lo);
          const unsigned carry = old_lo + q_lo < old_lo ? 1u : 0u;
          if (q_hi | carry) atomicAdd(t32 + 1, q_hi + carry);
          v = parent_of<COMPACT>(parent, par16, v);
        }
      }
    }
    __syncthreads();
    unsigned long long* y = a.y_fx + static_cast<size_t>(scen) * a.g.m;
    int vf = threadIdx.x;
    if constexpr (!SMEM) {  // global layout: four nodes' totals and links in flight
      for (; vf + 3 * BLOCK < n1; vf += 4 * BLOCK) {
        unsigned long long q[4];
        unsigned k[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int v = vf + j * BLOCK;
          if constexpr (kWalk32) {
            q[j] = static_cast<unsigned long long>(tot32[v]) << kshift;
            k[j] = COMPACT && pack ? up[v] >> 16 : up[v];
          } else {
            q[j] = static_cast<unsigned long long>(thr[v]);
            k[j] = COMPACT && pack ? up[v] >> 16 : up[v];
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (q[j] != 0ull) atomicAdd(y + k[j], q[j]);
      }
    }
    for (int v = vf; v < n1; v += BLOCK) {
      if constexpr (kWalk32) {
        // the 32-bit totals cover the labels only: the predecessor words
        // (the link, packed with the tail in the compact layout) are intact
        const unsigned q = tot32[v];
        if (q != 0u) {
          const unsigned pw = up[v];
          const unsigned k = COMPACT && pack ? pw >> 16 : pw;
          atomicAdd(y + k, static_cast<unsigned long long>(q) << kshift);
        }
      } else {
        const long long q = thr[v];
        if (q != 0) {
          const unsigned pw = up[v];
          const unsigned k = COMPACT && pack ? pw >> 16 : pw;
          atomicAdd(y + k, static_cast<unsigned long long>(q));
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// link kernels
// ---------------------------------------------------------------------------

__device__ __forceinline__ double pow2neg(int e) {
  // 2^-e for 0 <= e <= 1022 (exact)
  return __longlong_as_double(static_cast<long long>(1023 - e) << 52);
}

// tap/tap_functions.c:55-65, 112-126 (see bpr.cuh)
__device__ __forceinline__ double bpr(double fft, double alpha, double beta, unsigned char ip,
                                      double cap, double q) {
  return bprf::cost(fft, alpha, beta, ip, cap, q);
}
__device__ __forceinline__ double bpr_dq(double fft, double alpha, double beta, unsigned char ip,
                                         double cap, double q) {
  return bprf::dcost_dq(fft, alpha, beta, ip, cap, q);
}
__device__ __forceinline__ double integral(double fft, double alpha, double beta, unsigned char ip,
                                           double cap, double q) {
  return bprf::integral(fft, alpha, beta, ip, cap, q);
}

template <int N, int BLOCK>
__device__ __forceinline__ void block_sum(double (&v)[N], double* sh /* [N][BLOCK/32] */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int W = BLOCK / 32;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    double s = v[i];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) s = __dadd_rn(s, __shfl_down_sync(kFull, s, o));
    if (lane == 0) sh[i * W + warp] = s;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      double s = lane < W ? sh[i * W + lane] : 0.0;
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) s = __dadd_rn(s, __shfl_down_sync(kFull, s, o));
      if (lane == 0) v[i] = s;
    }
  }
}

__device__ __forceinline__ int scen_of(const LinkArgs& a) {
  return a.scen_list ? a.scen_list[blockIdx.y] : static_cast<int>(blockIdx.y);
}

// Last block of a scenario to arrive?  Every block must call this after
// publishing its partials.
__device__ __forceinline__ bool last_block(unsigned* arrive) {
  __shared__ unsigned sh_ticket;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) sh_ticket = atomicAdd(arrive, 1u);
  __syncthreads();
  return sh_ticket == gridDim.x - 1;
}

// index of link k's parameters for scenario scen (shared row or per-scenario rows)
__device__ __forceinline__ size_t lpi(const LinkParams& lp, int scen, int k) {
  return static_cast<size_t>(scen) * static_cast<size_t>(lp.stride) + static_cast<size_t>(k);
}

// link k is not part of scenario scen's network (a link another scenario adds)
__device__ __forceinline__ bool is_absent(const LinkArgs& a, int scen, int k) {
  return a.absent &&
         ((__ldg(a.absent + static_cast<size_t>(scen) * a.absent_words + (k >> 5)) >> (k & 31)) & 1u);
}

// shortest-path weight of link k of scenario scen in every record layout; a
// link absent from the scenario's network gets +inf, so it never relaxes a
// label and never enters a predecessor tree
__device__ __forceinline__ void write_weights(const LinkArgs& a, int scen, int k, double t) {
  if (is_absent(a, scen, k)) t = __longlong_as_double(0x7ff0000000000000ll);
  const size_t i = static_cast<size_t>(scen) * a.m + k;
  if (a.e32) {
    const unsigned bits = __float_as_uint(__double2float_rn(t));
    const uint2 rec = make_uint2(static_cast<unsigned>(__ldg(a.head + k)), bits);
    a.e32[i] = rec;
    a.r32[i - k + __ldg(a.rpos + k)] = make_uint2(static_cast<unsigned>(__ldg(a.tail + k)), bits);
    if (a.e4) {
      const int p = __ldg(a.ell_pos + k);
      if (p >= 0) a.e4[static_cast<size_t>(scen) * a.n1 * 4 + p] = make_uint2(__ldg(a.e4x + k), bits);
    }
    if (a.r4) {
      const int p = __ldg(a.r4_pos + k);
      if (p >= 0) a.r4[static_cast<size_t>(scen) * a.n1 * 4 + p] = make_uint2(__ldg(a.r4x + k), bits);
    }
  }
  if (a.w64) {
    a.w64[i] = t;
    if (a.r4d) {
      const int p = __ldg(a.r4_pos + k);
      if (p >= 0)
        a.r4d[static_cast<size_t>(scen) * a.n1 * 4 + p] =
            make_uint4(static_cast<unsigned>(k), static_cast<unsigned>(__ldg(a.tail + k)),
                       static_cast<unsigned>(__double2loint(t)),
                       static_cast<unsigned>(__double2hiint(t)));
    }
  }
}

constexpr int kLinkBlock = 256;

// x = AON volumes (fixed point), t = BPR(x), weights = t; resets the state.
// With from_x set, x is taken as given (warm start).
__global__ void __launch_bounds__(kLinkBlock) k_init_flows(LinkArgs a, int from_x) {
  const int scen = scen_of(a);
  const size_t off = static_cast<size_t>(scen) * a.m;
  const double* cap = a.cap + off;
  for (int k = blockIdx.x * kLinkBlock + threadIdx.x; k < a.m; k += gridDim.x * kLinkBlock) {
    double x;
    if (from_x) {
      x = a.x[off + k];
      if (is_absent(a, scen, k) && x != 0.0) {  // a link the scenario does not have carries nothing
        x = 0.0;
        a.x[off + k] = x;
      }
    } else {
      x = static_cast<double>(static_cast<long long>(a.y_fx[off + k])) * a.inv_scale;
      a.x[off + k] = x;
    }
    a.y_fx[off + k] = 0ull;
    const size_t pk = lpi(a.lp, scen, k);
    const double t = bpr(a.lp.fft[pk], a.lp.alpha[pk], a.lp.beta[pk], a.lp.ipow[pk], cap[k], x);
    a.t[off + k] = t;
    if (a.dtdx)
      a.dtdx[off + k] =
          bpr_dq(a.lp.fft[pk], a.lp.alpha[pk], a.lp.beta[pk], a.lp.ipow[pk], cap[k], x);
    write_weights(a, scen, k, t);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ScenState& st = a.state[scen];
    st.iter = 0;
    st.ls_pending = 0;
    st.ls_next = 1;
    st.relgap = DBL_MAX;
    st.best_lb = -DBL_MAX;
    st.obj = 0.0;
    st.gap = 0.0;
    st.lambda = 0.0;
    st.vht = 0.0;
    st.avg_excess = 0.0;
    st.g0 = 0.0;
    st.vht_end = 0.0;
    st.done = 0;
  }
}

// weights = free-flow times (the first all-or-nothing of tap/tap_frankwolfe_pthread.c:672,706)
__global__ void __launch_bounds__(kLinkBlock) k_set_free_flow(LinkArgs a) {
  const int scen = scen_of(a);
  const size_t off = static_cast<size_t>(scen) * a.m;
  for (int k = blockIdx.x * kLinkBlock + threadIdx.x; k < a.m; k += gridDim.x * kLinkBlock) {
    a.y_fx[off + k] = 0ull;
    write_weights(a, scen, k, a.lp.fft[lpi(a.lp, scen, k)]);
  }
}

// candidate step j of a pass: 2^-(e0+j) (reference rule) or the j-th of 12
// interior points of the current bracket (exact root)
__device__ __forceinline__ double ls_candidate(int mode, int e0, double lo, double hi, int j) {
  if (mode == kLsExact) return lo + (hi - lo) * static_cast<double>(j + 1) / (kLsPerPass + 1);
  return pow2neg(e0 + j);
}

__device__ void ls_decide(ScenState& st, const double* tot, int first_e, int pass, double total_demand,
                          int mode) {
  if (pass == 0) {
    const double g0 = tot[0];
    st.g0 = g0;
    st.gap = -g0;
    st.vht = tot[1];
    st.obj = tot[2];
    const double lb = st.obj - st.gap;
    if (lb > st.best_lb) st.best_lb = lb;
    if (st.best_lb != 0) st.relgap = (st.obj - st.best_lb) / fabs(st.best_lb);
    st.avg_excess = -g0 / total_demand;
    st.ls_pending = 1;
    if (g0 >= 0) {
      st.lambda = 0.0;
      st.ls_pending = 0;
      return;
    }
    if (tot[3] <= 0) {
      st.lambda = 1.0;
      st.ls_pending = 0;
      return;
    }
    st.ls_lo = 0.0;
    st.ls_glo = g0;
    st.ls_hi = 1.0;
    st.ls_ghi = tot[3];
  }
  if (mode == kLsExact) {
    // g rises with lambda (convex objective): keep the sign change bracketed
    const double lo = st.ls_lo, hi = st.ls_hi;
    for (int j = 0; j < kLsPerPass; ++j) {
      const double lam = ls_candidate(mode, 0, lo, hi, j);
      if (tot[4 + j] > 0) {
        st.ls_hi = lam;
        st.ls_ghi = tot[4 + j];
        break;
      }
      st.ls_lo = lam;
      st.ls_glo = tot[4 + j];
    }
    if (pass + 1 >= kLsExactPasses || st.ls_hi - st.ls_lo <= 1e-15 * st.ls_hi) {
      const double den = st.ls_glo - st.ls_ghi;
      st.lambda = den < 0 ? st.ls_lo + (st.ls_hi - st.ls_lo) * (st.ls_glo / den) : st.ls_lo;
      st.ls_pending = 0;
    }
    return;
  }
  for (int j = 0; j < kLsPerPass; ++j) {
    if (tot[4 + j] <= 0) {
      st.lambda = pow2neg(first_e + j);
      st.ls_pending = 0;
      return;
    }
  }
  st.ls_next = first_e + kLsPerPass;
}

// One link's part of a line-search pass: pass 0 forms d = y - x (stored) and
// adds the link's gap, VHT, objective and g(1) terms; every pass adds its
// candidate steps' terms.
__device__ __forceinline__ void ls_link(const LinkArgs& a, int scen, size_t off, const double* cap,
                                        int k, int pass, int e0, double blo, double bhi,
                                        double (&acc)[kNumSums]) {
  const double x = a.x[off + k];
  const size_t pk = lpi(a.lp, scen, k);
  const double fft = a.lp.fft[pk], al = a.lp.alpha[pk], be = a.lp.beta[pk], c = cap[k];
  const unsigned char ip = a.lp.ipow[pk];
  // FP32-path mode, integer power: t(x + lam d) = fft + (fft alpha) (x/c + lam d/c)^beta
  // with one division per link (FP64 mode keeps the reference's forms,
  // tap/tap_functions.c:55-65, 112-126)
  const bool ratio = a.ls_ratio && ip != 255;
  const double ic = ratio ? 1.0 / c : 0.0;
  const double A = fft * al;
  double d;
  if (pass == 0) {
    const double y = static_cast<double>(static_cast<long long>(a.y_fx[off + k])) * a.inv_scale;
    a.y_fx[off + k] = 0ull;
    d = __dsub_rn(y, x);
    a.d[off + k] = d;
    const double t = a.t[off + k];
    acc[0] = __dadd_rn(acc[0], __dmul_rn(t, d));
    acc[1] = __dadd_rn(acc[1], __dmul_rn(x, t));
    if (ratio) {
      // x fft (1 + alpha / (beta + 1) (x/c)^beta) and t(x + d) d
      const double r0 = x * ic;
      acc[2] += x * (fft + A * bprf::int_pow_fast(r0, ip) * bprf::inv_int(ip + 1));
      acc[3] += (fft + A * bprf::int_pow_fast(r0 + d * ic, ip)) * d;
    } else {
      acc[2] = __dadd_rn(acc[2], integral(fft, al, be, ip, c, x));
      acc[3] = __dadd_rn(acc[3], __dmul_rn(bpr(fft, al, be, ip, c, __dadd_rn(x, d)), d));
    }
  } else {
    d = a.d[off + k];
  }
  if (ratio) {
    const double r0 = x * ic, rd = d * ic;
#pragma unroll
    for (int j = 0; j < kLsPerPass; ++j) {
      const double lam = ls_candidate(a.ls_mode, e0, blo, bhi, j);
      acc[4 + j] += (fft + A * bprf::int_pow_fast(r0 + lam * rd, ip)) * d;
    }
  } else {
#pragma unroll
    for (int j = 0; j < kLsPerPass; ++j) {
      const double lam = ls_candidate(a.ls_mode, e0, blo, bhi, j);
      const double q = __dadd_rn(x, __dmul_rn(lam, d));
      acc[4 + j] = __dadd_rn(acc[4 + j], __dmul_rn(bpr(fft, al, be, ip, c, q), d));
    }
  }
}

// One line-search pass; pass 0 also forms d = y - x and the gap / objective /
// VHT sums.  Candidates of this pass: 2^-(e0 .. e0+kLsPerPass-1).  BLOCK 64
// for small networks (their FP64 work spread over more SMs), else 256.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_ls_pass(LinkArgs a) {
  __shared__ double sh[kNumSums * (BLOCK / 32)];
  const int scen = scen_of(a);
  ScenState& st = a.state[scen];
  if (st.done) return;
  if (a.pass > 0 && !st.ls_pending) return;
  const size_t off = static_cast<size_t>(scen) * a.m;
  const int e0 = a.pass == 0 ? 1 : st.ls_next;
  const double blo = a.pass == 0 ? 0.0 : st.ls_lo;
  const double bhi = a.pass == 0 ? 1.0 : st.ls_hi;
  double acc[kNumSums];
#pragma unroll
  for (int i = 0; i < kNumSums; ++i) acc[i] = 0.0;
  const double* cap = a.cap + off;
  for (int k = blockIdx.x * BLOCK + threadIdx.x; k < a.m; k += gridDim.x * BLOCK)
    ls_link(a, scen, off, cap, k, a.pass, e0, blo, bhi, acc);
  block_sum<kNumSums, BLOCK>(acc, sh);
  double* part = a.partials + (static_cast<size_t>(scen) * gridDim.x + blockIdx.x) * kNumSums;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < kNumSums; ++i) part[i] = acc[i];
  }
  if (!last_block(a.arrive + scen)) return;
  if (threadIdx.x == 0) {
    double tot[kNumSums];
    for (int i = 0; i < kNumSums; ++i) tot[i] = 0.0;
    const double* p0 = a.partials + static_cast<size_t>(scen) * gridDim.x * kNumSums;
    for (unsigned b = 0; b < gridDim.x; ++b)
      for (int i = 0; i < kNumSums; ++i)
        tot[i] = __dadd_rn(tot[i], vload(p0 + b * kNumSums + i));
    ls_decide(st, tot, e0, a.pass, a.total_demand_s ? a.total_demand_s[scen] : a.total_demand,
              a.ls_mode);
    a.arrive[scen] = 0u;
  }
}

// Continue the halving sequence one candidate at a time up to the reference's
// cap of 1000 halvings (never reached on valid inputs), by one block (any
// size up to 1024 threads); every thread of the block calls it.
__device__ void ls_fallback_block(const LinkArgs& a, int scen, ScenState& st, double* sh,
                                  int* sh_found) {
  if (st.done || !st.ls_pending) return;
  if (a.ls_mode == kLsExact) {  // bracket already tight: interpolate
    __syncthreads();            // every thread has read the state before it changes
    if (threadIdx.x == 0) {
      const double den = st.ls_glo - st.ls_ghi;
      st.lambda = den < 0 ? st.ls_lo + (st.ls_hi - st.ls_lo) * (st.ls_glo / den) : st.ls_lo;
      st.ls_pending = 0;
    }
    return;
  }
  const size_t off = static_cast<size_t>(scen) * a.m;
  const double* cap = a.cap + off;
  for (int e = st.ls_next; e <= kLsMaxHalvings; ++e) {
    double s = 0.0;
    const double lam = e <= 1022 ? pow2neg(e) : 0.0;
    for (int k = threadIdx.x; k < a.m; k += blockDim.x) {
      const double x = a.x[off + k], d = a.d[off + k];
      const double q = __dadd_rn(x, __dmul_rn(lam, d));
      const size_t pk = lpi(a.lp, scen, k);
      s = __dadd_rn(s, __dmul_rn(bpr(a.lp.fft[pk], a.lp.alpha[pk], a.lp.beta[pk], a.lp.ipow[pk],
                                     cap[k], q), d));
    }
    for (int o = 16; o >= 1; o >>= 1) s += __shfl_down_sync(kFull, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (unsigned w = 0; w < blockDim.x / 32; ++w) t += sh[w];
      *sh_found = t <= 0 ? 1 : 0;
      if (*sh_found) {
        st.lambda = lam;
        st.ls_pending = 0;
      }
    }
    __syncthreads();
    if (*sh_found) return;
  }
  if (threadIdx.x == 0) {
    st.lambda = 0.0;  // tap/tap_functions.c:506 returns lambda_left == 0
    st.ls_pending = 0;
    atomicOr(a.err, kErrLineSearch);
  }
}

__global__ void __launch_bounds__(1024) k_ls_fallback(LinkArgs a) {
  __shared__ double sh[32];
  __shared__ int sh_found;
  const int scen = scen_of(a);
  ls_fallback_block(a, scen, a.state[scen], sh, &sh_found);
}

// Where iteration `it` of a scenario writes its adjoint tape: every
// direction, the flows only every ckpt_every iterations.
struct TapeAt {
  bool tape, ckpt;
  size_t hoff, xoff;
};
__device__ __forceinline__ TapeAt tape_at(const LinkArgs& a, int scen, int it) {
  TapeAt r;
  r.tape = a.d_hist && it < a.hist_cap;
  r.ckpt = r.tape && (it % a.ckpt_every == 0);
  r.hoff = r.tape ? (static_cast<size_t>(scen) * a.hist_cap + it) * a.m : 0;
  const size_t nck = static_cast<size_t>(a.hist_cap / a.ckpt_every + 1);
  r.xoff = r.ckpt ? (static_cast<size_t>(scen) * nck + it / a.ckpt_every) * a.m : 0;
  return r;
}

// x += lambda d on link k, its BPR cost and derivative, the next weights;
// returns the link's x t (VHT term)
__device__ __forceinline__ double step_link(const LinkArgs& a, int scen, size_t off, const double* cap,
                                            int k, double lam, const TapeAt& tp) {
  const double x0 = a.x[off + k];
  const double d = a.d[off + k];
  if (tp.tape) a.d_hist[tp.hoff + k] = d;
  if (tp.ckpt) a.x_hist[tp.xoff + k] = x0;
  const double x = __dadd_rn(x0, __dmul_rn(lam, d));
  a.x[off + k] = x;
  const size_t pk = lpi(a.lp, scen, k);
  const double fft = a.lp.fft[pk], al = a.lp.alpha[pk], be = a.lp.beta[pk], c = cap[k];
  const unsigned char ip = a.lp.ipow[pk];
  const double t = bpr(fft, al, be, ip, c, x);
  a.t[off + k] = t;
  if (a.dtdx) a.dtdx[off + k] = bpr_dq(fft, al, be, ip, c, x);
  write_weights(a, scen, k, t);
  return __dmul_rn(x, t);
}

// the iteration's bookkeeping once the step's VHT is summed (one thread)
__device__ __forceinline__ void step_finish(const LinkArgs& a, int scen, ScenState& st, int it,
                                            double lam, const TapeAt& tp, double vht) {
  st.vht_end = vht;
  if (tp.tape) a.lam_hist[static_cast<size_t>(scen) * a.hist_cap + it] = lam;
  if (a.trace && it < a.trace_cap) {
    double* r = a.trace + (static_cast<size_t>(scen) * a.trace_cap + it) * kTraceCols;
    r[0] = st.obj;
    r[1] = st.relgap;
    r[2] = st.avg_excess;
    r[3] = st.vht;
    r[4] = lam;
    r[5] = st.gap;
    r[6] = it + 1;
    r[7] = st.g0;
  }
  st.iter = it + 1;
  if ((st.max_iters > 0 && st.iter >= st.max_iters) ||
      (st.target_relgap > 0 && !(st.relgap > st.target_relgap)))
    st.done = 1;
}

// x += lambda d; t = BPR(x); next weights; iteration bookkeeping (BLOCK as
// k_ls_pass).
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_step(LinkArgs a) {
  __shared__ double sh[1 * (BLOCK / 32)];
  const int scen = scen_of(a);
  ScenState& st = a.state[scen];
  if (st.done) return;
  const size_t off = static_cast<size_t>(scen) * a.m;
  const double lam = st.lambda;
  const int it = st.iter;
  const TapeAt tp = tape_at(a, scen, it);
  const double* cap = a.cap + off;
  double acc[1] = {0.0};
  for (int k = blockIdx.x * BLOCK + threadIdx.x; k < a.m; k += gridDim.x * BLOCK)
    acc[0] = __dadd_rn(acc[0], step_link(a, scen, off, cap, k, lam, tp));
  block_sum<1, BLOCK>(acc, sh);
  double* part = a.partials + (static_cast<size_t>(scen) * gridDim.x + blockIdx.x) * kNumSums;
  if (threadIdx.x == 0) part[0] = acc[0];
  if (!last_block(a.arrive + scen)) return;
  if (threadIdx.x == 0) {
    double v = 0.0;
    const double* p0 = a.partials + static_cast<size_t>(scen) * gridDim.x * kNumSums;
    for (unsigned b = 0; b < gridDim.x; ++b) v = __dadd_rn(v, vload(p0 + b * kNumSums));
    step_finish(a, scen, st, it, lam, tp, v);
    a.arrive[scen] = 0u;
  }
}

// Small networks: the whole tail of an iteration (every line-search pass,
// the fallback, the step) by one 256-thread block per scenario, one launch
// instead of seven; the same per-link arithmetic as k_ls_pass, k_ls_fallback
// and k_step, with block-wide sums.
constexpr int kTailBlock = 256;
__global__ void __launch_bounds__(kTailBlock) k_fw_tail_small(LinkArgs a) {
  __shared__ double sh[kNumSums * (kTailBlock / 32)];
  __shared__ int sh_found;
  const int scen = scen_of(a);
  ScenState& st = a.state[scen];
  if (st.done) return;  // (read by every thread before any change to it)
  const size_t off = static_cast<size_t>(scen) * a.m;
  const double* cap = a.cap + off;
  const int passes = a.ls_mode == kLsExact ? kLsExactPasses : kLsPasses;
  for (int pass = 0; pass < passes; ++pass) {
    if (pass > 0 && !st.ls_pending) break;  // (uniform: written before the last barrier)
    const int e0 = pass == 0 ? 1 : st.ls_next;
    const double blo = pass == 0 ? 0.0 : st.ls_lo;
    const double bhi = pass == 0 ? 1.0 : st.ls_hi;
    double acc[kNumSums];
#pragma unroll
    for (int i = 0; i < kNumSums; ++i) acc[i] = 0.0;
    for (int k = threadIdx.x; k < a.m; k += kTailBlock) ls_link(a, scen, off, cap, k, pass, e0, blo, bhi, acc);
    block_sum<kNumSums, kTailBlock>(acc, sh);
    if (threadIdx.x == 0)
      ls_decide(st, acc, e0, pass, a.total_demand_s ? a.total_demand_s[scen] : a.total_demand,
                a.ls_mode);
    __syncthreads();
  }
  ls_fallback_block(a, scen, st, sh, &sh_found);
  __syncthreads();
  const double lam = st.lambda;
  const int it = st.iter;
  const TapeAt tp = tape_at(a, scen, it);
  double acc[1] = {0.0};
  for (int k = threadIdx.x; k < a.m; k += kTailBlock)
    acc[0] = __dadd_rn(acc[0], step_link(a, scen, off, cap, k, lam, tp));
  __syncthreads();  // (sh reused)
  block_sum<1, kTailBlock>(acc, sh);
  if (threadIdx.x == 0) step_finish(a, scen, st, it, lam, tp, acc[0]);
}

// Raise a kernel's dynamic shared-memory limit to the device maximum once, so
// that launches inside a stream capture never change function attributes.
template <typename Fn>
cudaError_t allow_max_smem(Fn fn) {
  // one flag per kernel (all path kernels share the same function type)
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done_set;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(reinterpret_cast<const void*>(fn), dev);
  if (done_set.count(key)) return cudaSuccess;
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, fn);
  if (e != cudaSuccess) return e;
  // the opt-in limit covers static and dynamic shared memory together
  const int dyn = max_smem_optin(dev) - static_cast<int>(fa.sharedSizeBytes);
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
  if (e == cudaSuccess)
    done_set.insert(key);
  else
    cudaGetLastError();
  return e;
}

using PathKernel = void (*)(PathArgs);

template <typename T, int BLOCK, bool SMEM>
PathKernel sssp_kernel(int variant) {
  if (variant == kSsspSmall) return k_sssp_small<T, BLOCK, SMEM>;
  if (variant == kSsspRounds) return k_sssp<T, BLOCK, SMEM>;
  if (variant == kSsspAsync) return k_sssp_async<T, BLOCK, SMEM>;
  if (variant == kSsspNearFarQueue) return k_sssp_nfq<T, BLOCK, SMEM, unsigned short>;
  if (variant == kSsspNearFarQueueWide) return k_sssp_nfq<T, BLOCK, SMEM, unsigned>;
  return k_sssp_nf<T, BLOCK, SMEM>;
}

template <typename T, int BLOCK>
PathKernel nfq_split_kernel(int variant) {
  return variant == kSsspNearFarQueue ? k_sssp_nfq<T, BLOCK, false, unsigned short, true>
                                      : k_sssp_nfq<T, BLOCK, false, unsigned, true>;
}

template <typename T, int BLOCK, bool SMEM>
cudaError_t launch_sssp_t(const PathArgs& a, int grid, size_t smem, int variant, cudaStream_t s) {
  if (!SMEM && !a.all_global && nfq_split(a.g.n1, variant)) {
    PathKernel fn = nfq_split_kernel<T, BLOCK>(variant);
    cudaError_t e = allow_max_smem(fn);
    if (e != cudaSuccess) return e;
    fn<<<grid, BLOCK, nfq_split_smem_bytes(a.g.n1, variant), s>>>(a);
    return cudaGetLastError();
  }
  PathKernel fn = sssp_kernel<T, BLOCK, SMEM>(variant);
  if (SMEM) {
    cudaError_t e = allow_max_smem(fn);
    if (e != cudaSuccess) return e;
  }
  fn<<<grid, BLOCK, SMEM ? smem : 0, s>>>(a);
  return cudaGetLastError();
}

template <typename T, int BLOCK, bool SMEM, bool COMPACT>
cudaError_t launch_aon_t(const PathArgs& a, int grid, size_t smem, cudaStream_t s) {
  auto fn = k_aon<T, BLOCK, SMEM, COMPACT>;
  if (SMEM) {
    cudaError_t e = allow_max_smem(fn);
    if (e != cudaSuccess) return e;
  }
  fn<<<grid, BLOCK, SMEM ? smem : 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

size_t sssp_smem_bytes(int n1, bool fp64, int variant, int m) {
  if (variant == kSsspSmall)  // labels, then tails and heads, then weights
    return align16(align16((fp64 ? 8 : 4) * static_cast<size_t>(n1)) +
                   align16(8 * static_cast<size_t>(m)) + (fp64 ? 8 : 4) * static_cast<size_t>(m));
  const size_t words = (static_cast<size_t>(n1) + 31) / 32;
  const size_t ring = variant == kSsspNearFarQueue       ? sizeof(unsigned short) * kQCap
                      : variant == kSsspNearFarQueueWide ? sizeof(unsigned) * kQCap
                                                         : 0;
  return align16(align16((fp64 ? 8 : 4) * static_cast<size_t>(n1)) + 2 * 4 * words + ring);
}

size_t nfq_split_smem_bytes(int n1, int variant) {
  const size_t words = (static_cast<size_t>(n1) + 31) / 32;
  const size_t ring =
      variant == kSsspNearFarQueue ? sizeof(unsigned short) * kQCap : sizeof(unsigned) * kQCap;
  return align16(2 * 4 * words + ring);
}

// (200 KB of bitmaps: networks up to ~6.5 million nodes)
bool nfq_split(int n1, int variant) {
  return (variant == kSsspNearFarQueue || variant == kSsspNearFarQueueWide) &&
         nfq_split_smem_bytes(n1, variant) <= (size_t(200) << 10);
}

// Both sizes are also the stride between CTAs' slices of the global-memory
// scratch, so they are rounded to 16 bytes (8-byte totals and labels).
bool aon_compact(int n1, bool fp64) { return !fp64 && n1 <= 0xffff; }

size_t aon_smem_bytes(int n1, bool fp64, bool c64) {
  const size_t n = static_cast<size_t>(n1);
  if (aon_compact(n1, fp64) || (fp64 && c64)) return align16(align16(8 * n) + align16(2 * n));
  return align16(align16((fp64 ? 8 : 4) * n) + 2 * 4 * n);  // (FP32: 4-byte labels and totals)
}

int max_smem_optin(int device) {
  int v = 0;
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  return v;
}

cudaError_t launch_sssp(const PathArgs& a, bool fp64, int grid, int block, bool smem,
                        int variant, cudaStream_t s) {
  // FP32 paths of the queue variant read the padded records
  if ((variant == kSsspNearFarQueue || variant == kSsspNearFarQueueWide) && !fp64 && !a.e4)
    return cudaErrorInvalidValue;
  const size_t bytes = sssp_smem_bytes(a.g.n1, fp64, variant, a.g.m);
#define TAPGPU_SSSP_CASE(B)                                                              \
  if (block == B) {                                                                      \
    if (fp64) return smem ? launch_sssp_t<double, B, true>(a, grid, bytes, variant, s)   \
                          : launch_sssp_t<double, B, false>(a, grid, bytes, variant, s); \
    return smem ? launch_sssp_t<float, B, true>(a, grid, bytes, variant, s)              \
                : launch_sssp_t<float, B, false>(a, grid, bytes, variant, s);            \
  }
  TAPGPU_SSSP_CASE(128)
  TAPGPU_SSSP_CASE(256)
  TAPGPU_SSSP_CASE(512)
  TAPGPU_SSSP_CASE(1024)
#undef TAPGPU_SSSP_CASE
  return cudaErrorInvalidValue;
}

cudaError_t launch_aon(const PathArgs& a, bool fp64, int grid, int block, bool smem,
                       cudaStream_t s) {
  const bool c64 = fp64 && a.aon_c64;
  const size_t bytes = aon_smem_bytes(a.g.n1, fp64, c64);
  const bool compact = aon_compact(a.g.n1, fp64);
#define TAPGPU_AON_CASE(B)                                                               \
  if (block == B) {                                                                      \
    if (c64) return smem ? launch_aon_t<double, B, true, true>(a, grid, bytes, s)        \
                         : launch_aon_t<double, B, false, true>(a, grid, bytes, s);      \
    if (fp64) return smem ? launch_aon_t<double, B, true, false>(a, grid, bytes, s)      \
                          : launch_aon_t<double, B, false, false>(a, grid, bytes, s);    \
    if (compact) return smem ? launch_aon_t<float, B, true, true>(a, grid, bytes, s)     \
                             : launch_aon_t<float, B, false, true>(a, grid, bytes, s);   \
    return smem ? launch_aon_t<float, B, true, false>(a, grid, bytes, s)                 \
                : launch_aon_t<float, B, false, false>(a, grid, bytes, s);               \
  }
  TAPGPU_AON_CASE(256)
  TAPGPU_AON_CASE(512)
  TAPGPU_AON_CASE(1024)
#undef TAPGPU_AON_CASE
  return cudaErrorInvalidValue;
}

template <typename T, int BLOCK, bool SMEM>
int occ_sssp_t(size_t smem, int variant, int n1, bool all_global) {
  PathKernel fn = sssp_kernel<T, BLOCK, SMEM>(variant);
  if (!SMEM && !all_global && nfq_split(n1, variant)) {
    fn = nfq_split_kernel<T, BLOCK>(variant);
    smem = nfq_split_smem_bytes(n1, variant);
    if (allow_max_smem(fn) != cudaSuccess) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, BLOCK, smem) != cudaSuccess) return 0;
    return n;
  }
  if (SMEM && allow_max_smem(fn) != cudaSuccess) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, BLOCK, SMEM ? smem : 0) != cudaSuccess)
    return 0;
  return n;
}

template <typename T, int BLOCK, bool SMEM, bool COMPACT>
int occ_aon_t(size_t smem) {
  auto fn = k_aon<T, BLOCK, SMEM, COMPACT>;
  if (SMEM && allow_max_smem(fn) != cudaSuccess) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, BLOCK, SMEM ? smem : 0) != cudaSuccess)
    return 0;
  return n;
}

int sssp_occupancy(bool fp64, int block, bool smem, int n1, int variant, int m, bool all_global) {
  const size_t bytes = sssp_smem_bytes(n1, fp64, variant, m);
#define TAPGPU_OCC(B)                                                                       \
  if (block == B) {                                                                         \
    if (fp64) return smem ? occ_sssp_t<double, B, true>(bytes, variant, n1, all_global)     \
                          : occ_sssp_t<double, B, false>(bytes, variant, n1, all_global);   \
    return smem ? occ_sssp_t<float, B, true>(bytes, variant, n1, all_global)                \
                : occ_sssp_t<float, B, false>(bytes, variant, n1, all_global);              \
  }
  TAPGPU_OCC(128)
  TAPGPU_OCC(256)
  TAPGPU_OCC(512)
  TAPGPU_OCC(1024)
#undef TAPGPU_OCC
  return 0;
}

int aon_occupancy(bool fp64, int block, bool smem, int n1, bool c64) {
  const size_t bytes = aon_smem_bytes(n1, fp64, c64);
  const bool compact = aon_compact(n1, fp64);
#define TAPGPU_OCC(B)                                                                     \
  if (block == B) {                                                                       \
    if (fp64 && c64) return smem ? occ_aon_t<double, B, true, true>(bytes)                \
                                 : occ_aon_t<double, B, false, true>(bytes);              \
    if (fp64) return smem ? occ_aon_t<double, B, true, false>(bytes)                      \
                          : occ_aon_t<double, B, false, false>(bytes);                    \
    if (compact) return smem ? occ_aon_t<float, B, true, true>(bytes)                     \
                             : occ_aon_t<float, B, false, true>(bytes);                   \
    return smem ? occ_aon_t<float, B, true, false>(bytes)                                 \
                : occ_aon_t<float, B, false, false>(bytes);                               \
  }
  TAPGPU_OCC(256)
  TAPGPU_OCC(512)
  TAPGPU_OCC(1024)
#undef TAPGPU_OCC
  return 0;
}

cudaError_t launch_init_flows(const LinkArgs& a, int grid, cudaStream_t s) {
  k_init_flows<<<dim3(grid, a.num_scen), kLinkBlock, 0, s>>>(a, a.pass);
  return cudaGetLastError();
}

cudaError_t launch_set_costs(const LinkArgs& a, int grid, cudaStream_t s) {
  k_set_free_flow<<<dim3(grid, a.num_scen), kLinkBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_ls_pass(const LinkArgs& a, int grid, int block, cudaStream_t s) {
  if (block == kSmallLinkBlock)
    k_ls_pass<kSmallLinkBlock><<<dim3(grid, a.num_scen), kSmallLinkBlock, 0, s>>>(a);
  else
    k_ls_pass<kLinkBlock><<<dim3(grid, a.num_scen), kLinkBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_ls_fallback(const LinkArgs& a, cudaStream_t s) {
  k_ls_fallback<<<dim3(1, a.num_scen), 1024, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fw_tail_small(const LinkArgs& a, cudaStream_t s) {
  k_fw_tail_small<<<dim3(1, a.num_scen), kTailBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_step(const LinkArgs& a, int grid, int block, cudaStream_t s) {
  if (block == kSmallLinkBlock)
    k_step<kSmallLinkBlock><<<dim3(grid, a.num_scen), kSmallLinkBlock, 0, s>>>(a);
  else
    k_step<kLinkBlock><<<dim3(grid, a.num_scen), kLinkBlock, 0, s>>>(a);
  return cudaGetLastError();
}

// Scenario capacity rows made on the device: each row starts as the base
// row (already positive), then one thread per scenario applies its edits in
// their order, a non-positive value replaced by the scenario's smallest
// positive capacity (the zero-capacity fix-up of
// tap/tap_frankwolfe_pthread.c:654-669, computed on the host).
__global__ void __launch_bounds__(kLinkBlock) k_scen_base_rows(double* cap, const double* base,
                                                               int m) {
  const size_t row = static_cast<size_t>(blockIdx.y) * m;
  for (int k = blockIdx.x * kLinkBlock + threadIdx.x; k < m; k += gridDim.x * kLinkBlock)
    cap[row + k] = base[k];
}

__global__ void __launch_bounds__(kLinkBlock) k_scen_edits(double* cap, int m, int nscen,
                                                           const int* ptr, const int* link,
                                                           const double* val,
                                                           const double* min_pos) {
  const int s = blockIdx.x * kLinkBlock + threadIdx.x;
  if (s >= nscen) return;
  double* row = cap + static_cast<size_t>(s) * m;
  for (int i = ptr[s]; i < ptr[s + 1]; ++i) row[link[i]] = val[i] > 0 ? val[i] : min_pos[s];
}

// every record of p[n] becomes val
__global__ void __launch_bounds__(kLinkBlock) k_fill_records(uint2* p, size_t n, uint2 val) {
  for (size_t i = static_cast<size_t>(blockIdx.x) * kLinkBlock + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * kLinkBlock)
    p[i] = val;
}

__global__ void __launch_bounds__(kLinkBlock) k_fill_records4(uint4* p, size_t n, uint4 val) {
  for (size_t i = static_cast<size_t>(blockIdx.x) * kLinkBlock + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * kLinkBlock)
    p[i] = val;
}

// rows 1 .. nscen-1 of x [nscen][m] become copies of row 0
__global__ void __launch_bounds__(kLinkBlock) k_replicate_rows(double* x, int m) {
  const size_t row = static_cast<size_t>(blockIdx.y + 1) * m;
  for (int k = blockIdx.x * kLinkBlock + threadIdx.x; k < m; k += gridDim.x * kLinkBlock)
    x[row + k] = x[k];
}

cudaError_t launch_scenario_caps(double* cap, const double* base, int m, int nscen, const int* ptr,
                                 const int* link, const double* val, const double* min_pos,
                                 int grid, cudaStream_t s) {
  k_scen_base_rows<<<dim3(grid, nscen), kLinkBlock, 0, s>>>(cap, base, m);
  k_scen_edits<<<(nscen + kLinkBlock - 1) / kLinkBlock, kLinkBlock, 0, s>>>(cap, m, nscen, ptr, link,
                                                                           val, min_pos);
  return cudaGetLastError();
}

// per-scenario link parameter rows: base row everywhere, then each scenario's edits
template <typename T>
__global__ void __launch_bounds__(kLinkBlock) k_rows_of_base(T* rows, const T* base, int m) {
  const size_t row = static_cast<size_t>(blockIdx.y) * m;
  for (int k = blockIdx.x * kLinkBlock + threadIdx.x; k < m; k += gridDim.x * kLinkBlock)
    rows[row + k] = base[k];
}

template <typename T>
__global__ void __launch_bounds__(kLinkBlock) k_row_edits(T* rows, int m, int nscen, const int* ptr,
                                                          const int* link, const T* val) {
  const int s = blockIdx.x * kLinkBlock + threadIdx.x;
  if (s >= nscen) return;
  T* row = rows + static_cast<size_t>(s) * m;
  for (int i = ptr[s]; i < ptr[s + 1]; ++i) row[link[i]] = val[i];
}

template <typename T>
cudaError_t launch_param_rows_t(T* rows, const T* base, int m, int nscen, const int* ptr,
                                const int* link, const T* val, int grid, cudaStream_t s) {
  k_rows_of_base<T><<<dim3(grid, nscen), kLinkBlock, 0, s>>>(rows, base, m);
  k_row_edits<T><<<(nscen + kLinkBlock - 1) / kLinkBlock, kLinkBlock, 0, s>>>(rows, m, nscen, ptr,
                                                                             link, val);
  return cudaGetLastError();
}

cudaError_t launch_param_rows(double* rows, const double* base, int m, int nscen, const int* ptr,
                              const int* link, const double* val, int grid, cudaStream_t s) {
  return launch_param_rows_t(rows, base, m, nscen, ptr, link, val, grid, s);
}

cudaError_t launch_param_rows(unsigned char* rows, const unsigned char* base, int m, int nscen,
                              const int* ptr, const int* link, const unsigned char* val, int grid,
                              cudaStream_t s) {
  return launch_param_rows_t(rows, base, m, nscen, ptr, link, val, grid, s);
}

cudaError_t launch_fill_records(uint2* p, size_t n, uint2 val, int grid, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_fill_records<<<grid, kLinkBlock, 0, s>>>(p, n, val);
  return cudaGetLastError();
}

cudaError_t launch_fill_records4(uint4* p, size_t n, uint4 val, int grid, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_fill_records4<<<grid, kLinkBlock, 0, s>>>(p, n, val);
  return cudaGetLastError();
}

cudaError_t launch_replicate_rows(double* x, int m, int nscen, int grid, cudaStream_t s) {
  if (nscen < 2) return cudaSuccess;
  k_replicate_rows<<<dim3(grid, nscen - 1), kLinkBlock, 0, s>>>(x, m);
  return cudaGetLastError();
}

}  // namespace tapgpu
