// linkops.cu - GPU link-array numerics behind the drop-in tap_functions.h
// entry points (tap/tap_functions.c:83-97, 143-152, 167-175, 408-417, 469-507):
// BPR costs, Beckmann objective, directional derivative at many step sizes and
// the VHT dot product.  Sums are block-deterministic: a fixed grid-stride
// assignment, a fixed tree per block and a fixed-order final pass.
#include "linkops.cuh"

#include "bpr.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace tapgpu {

namespace {

constexpr int kBlock = 256;
constexpr int kMaxLambdas = 32;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double bpr(const LinkArrays& l, int k, double q) {
  return bprf::cost(l.fft[k], l.alpha[k], l.beta[k], l.ipow[k], l.cap[k], q);
}

__device__ __forceinline__ double integral(const LinkArrays& l, int k, double q) {
  return bprf::integral(l.fft[k], l.alpha[k], l.beta[k], l.ipow[k], l.cap[k], q);
}

__global__ void __launch_bounds__(kBlock) k_costs(LinkArrays l, const double* x, double* t, int m) {
  for (int k = blockIdx.x * kBlock + threadIdx.x; k < m; k += gridDim.x * kBlock)
    t[k] = bpr(l, k, x[k]);
}

// op 0: sum_k t_k(x_k + lam_j d_k) d_k for each lam_j
// op 1: sum_k integral_k(x_k)
// op 2: sum_k x_k * d_k
__global__ void __launch_bounds__(kBlock) k_sums(LinkArrays l, const double* x, const double* d,
                                                 const double* lams, int nl, int op, int m,
                                                 double* part) {
  __shared__ double sh[kMaxLambdas][kBlock / 32];
  double acc[kMaxLambdas];
  for (int j = 0; j < kMaxLambdas; ++j) acc[j] = 0.0;
  for (int k = blockIdx.x * kBlock + threadIdx.x; k < m; k += gridDim.x * kBlock) {
    if (op == 0) {
      const double xv = x[k], dv = d[k];
      for (int j = 0; j < nl; ++j)
        acc[j] = __dadd_rn(acc[j], __dmul_rn(bpr(l, k, __dadd_rn(xv, __dmul_rn(lams[j], dv))), dv));
    } else if (op == 1) {
      acc[0] = __dadd_rn(acc[0], integral(l, k, x[k]));
    } else {
      acc[0] = __dadd_rn(acc[0], __dmul_rn(x[k], d[k]));
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = 0; j < nl; ++j) {
    double s = acc[j];
    for (int o = 16; o >= 1; o >>= 1) s = __dadd_rn(s, __shfl_down_sync(kFull, s, o));
    if (lane == 0) sh[j][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x < nl) {
    double s = 0.0;
    for (int w = 0; w < kBlock / 32; ++w) s = __dadd_rn(s, sh[threadIdx.x][w]);
    part[blockIdx.x * kMaxLambdas + threadIdx.x] = s;
  }
}

}  // namespace

LinkOps::~LinkOps() { release(); }

void LinkOps::release() {
  void* ps[] = {fft, alpha, beta, cap, ipow, x, d, t, lams, part};
  for (void* p : ps)
    if (p) cudaFree(p);
  fft = alpha = beta = cap = x = d = t = lams = part = nullptr;
  ipow = nullptr;
  m = 0;
}

int LinkOps::upload(int nlinks, const double* h_fft, const double* h_alpha, const double* h_beta,
                    const double* h_cap) {
  if (nlinks != m) {
    release();
    m = nlinks;
    size_t b = sizeof(double) * static_cast<size_t>(m);
    if (cudaMalloc(&fft, b) || cudaMalloc(&alpha, b) || cudaMalloc(&beta, b) ||
        cudaMalloc(&cap, b) || cudaMalloc(&x, b) || cudaMalloc(&d, b) || cudaMalloc(&t, b) ||
        cudaMalloc(&ipow, static_cast<size_t>(m)) ||
        cudaMalloc(&lams, sizeof(double) * kMaxLambdas) ||
        cudaMalloc(&part, sizeof(double) * kMaxLambdas * kGrid)) {
      cudaGetLastError();
      release();
      return -1;
    }
  }
  std::vector<unsigned char> ip(m);
  for (int k = 0; k < m; ++k) {
    const double b = h_beta[k];
    ip[k] = (b >= 0 && b <= 15 && std::floor(b) == b) ? static_cast<unsigned char>(b) : 255;
  }
  size_t b = sizeof(double) * static_cast<size_t>(m);
  if (cudaMemcpy(fft, h_fft, b, cudaMemcpyHostToDevice) ||
      cudaMemcpy(alpha, h_alpha, b, cudaMemcpyHostToDevice) ||
      cudaMemcpy(beta, h_beta, b, cudaMemcpyHostToDevice) ||
      cudaMemcpy(cap, h_cap, b, cudaMemcpyHostToDevice) ||
      cudaMemcpy(ipow, ip.data(), static_cast<size_t>(m), cudaMemcpyHostToDevice))
    return -1;
  return 0;
}

LinkArrays LinkOps::arrays() const {
  LinkArrays l;
  l.fft = fft;
  l.alpha = alpha;
  l.beta = beta;
  l.cap = cap;
  l.ipow = ipow;
  return l;
}

int LinkOps::costs(const double* h_x, double* h_t) {
  size_t b = sizeof(double) * static_cast<size_t>(m);
  if (cudaMemcpy(x, h_x, b, cudaMemcpyHostToDevice)) return -1;
  k_costs<<<kGrid, kBlock>>>(arrays(), x, t, m);
  if (cudaGetLastError() || cudaMemcpy(h_t, t, b, cudaMemcpyDeviceToHost)) return -1;
  return 0;
}

int LinkOps::sums(int op, const double* h_lams, int nl, double* out) {
  if (nl < 1 || nl > kMaxLambdas) return -1;
  if (op == 0 && cudaMemcpy(lams, h_lams, sizeof(double) * nl, cudaMemcpyHostToDevice)) return -1;
  k_sums<<<kGrid, kBlock>>>(arrays(), x, d, lams, nl, op, m, part);
  std::vector<double> hp(static_cast<size_t>(kGrid) * kMaxLambdas);
  if (cudaGetLastError() ||
      cudaMemcpy(hp.data(), part, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost))
    return -1;
  for (int j = 0; j < nl; ++j) {
    double s = 0.0;
    for (int bidx = 0; bidx < kGrid; ++bidx) s += hp[static_cast<size_t>(bidx) * kMaxLambdas + j];
    out[j] = s;
  }
  return 0;
}

int LinkOps::set_xd(const double* h_x, const double* h_d) {
  size_t b = sizeof(double) * static_cast<size_t>(m);
  if (h_x && cudaMemcpy(x, h_x, b, cudaMemcpyHostToDevice)) return -1;
  if (h_d && cudaMemcpy(d, h_d, b, cudaMemcpyHostToDevice)) return -1;
  return 0;
}

int LinkOps::max_lambdas() { return kMaxLambdas; }

}  // namespace tapgpu
