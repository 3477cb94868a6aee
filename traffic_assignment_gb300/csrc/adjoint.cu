// adjoint.cu - dVHT/dcapacity through the recorded Frank-Wolfe iterations.
//
// Forward map (as solved, one scenario): x_0 = all-or-nothing at free flow
// (independent of capacity); for k < K: d_k = y_k - x_k with the loads y_k
// held fixed (piecewise constant in the capacities), lambda_k the step,
// x_{k+1} = x_k + lambda_k d_k; output J = VHT = sum_a x_K,a t_a(x_K,a).
// With the exact line search lambda_k is the root of
//   g(lambda) = sum_a t_a(x_k + lambda d_k) d_k,a
// and differentiable by the implicit-function rule
//   dlambda = -(dg/dx dx + dg/dc dc) / (dg/dlambda),  dg/dlambda = sum t'(q) d^2,
// with q = x_k + lambda d_k and dd/dx = -1.  Reverse sweep, k = K-1 .. 0:
//   s = xbar_{k+1} . d_k,  G = sum t'(q) d_k^2,  coef = -s / G (0 at lambda in {0,1})
//   xbar_k = (1 - lambda) xbar_{k+1} + coef (t'(q) (1 - lambda) d_k - t(q))
//   cbar  += coef dt/dcap(q) d_k
// starting from xbar_K = t + x t' and cbar = x dt/dcap at x_K.  The flows x_k
// are kept only every `ckpt_every` iterations; each segment is recomputed
// forward from its checkpoint with the forward's own rounding.  All sums are
// FP64 with a fixed reduction order.
#include <algorithm>
#include <cstring>
#include <vector>

#include "bpr.cuh"
#include "solver.cuh"

namespace tapgpu {

namespace {

constexpr int kAdjBlock = 256;
constexpr unsigned kFullMask = 0xffffffffu;

struct AdjArgs {
  int m;
  LinkParams lp;
  const double* cap;
  const double* x;    // x_k
  const double* d;    // d_k
  const double* lam;  // &lambda_k
  int exact;
  double* xbar;
  double* cbar;
  double* part;       // [grid][2]
  unsigned* arrive;
  double* scal;       // [2]: G, s
};

__global__ void __launch_bounds__(kAdjBlock) k_adj_init(int m, LinkParams lp, const double* cap,
                                                        const double* x, double* xbar,
                                                        double* cbar) {
  for (int k = blockIdx.x * kAdjBlock + threadIdx.x; k < m; k += gridDim.x * kAdjBlock) {
    const double q = x[k];
    const double fft = lp.fft[k], al = lp.alpha[k], be = lp.beta[k], c = cap[k];
    const unsigned char ip = lp.ipow[k];
    xbar[k] = bprf::cost(fft, al, be, ip, c, q) + q * bprf::dcost_dq(fft, al, be, ip, c, q);
    cbar[k] = q * bprf::dcost_dcap(fft, al, be, ip, c, q);
  }
}

// seg[j] = x_{k0+j} for j < len, from the checkpoint x_{k0}
__global__ void __launch_bounds__(kAdjBlock) k_adj_recompute(int m, const double* xck,
                                                             const double* dhist,
                                                             const double* lamhist, int k0,
                                                             int len, double* seg) {
  for (int k = blockIdx.x * kAdjBlock + threadIdx.x; k < m; k += gridDim.x * kAdjBlock) {
    double x = xck[k];
    seg[k] = x;
    for (int j = 1; j < len; ++j) {
      const int it = k0 + j - 1;
      x = __dadd_rn(x, __dmul_rn(lamhist[it], dhist[static_cast<size_t>(it) * m + k]));
      seg[static_cast<size_t>(j) * m + k] = x;
    }
  }
}

__global__ void __launch_bounds__(kAdjBlock) k_adj_reduce(AdjArgs a) {
  __shared__ double sh[2][kAdjBlock / 32];
  __shared__ unsigned ticket;
  const double lam = *a.lam;
  double G = 0.0, s = 0.0;
  for (int k = blockIdx.x * kAdjBlock + threadIdx.x; k < a.m; k += gridDim.x * kAdjBlock) {
    const double d = a.d[k];
    const double q = __dadd_rn(a.x[k], __dmul_rn(lam, d));
    const double tp = bprf::dcost_dq(a.lp.fft[k], a.lp.alpha[k], a.lp.beta[k], a.lp.ipow[k],
                                     a.cap[k], q);
    G += tp * d * d;
    s += a.xbar[k] * d;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o >= 1; o >>= 1) {
    G += __shfl_down_sync(kFullMask, G, o);
    s += __shfl_down_sync(kFullMask, s, o);
  }
  if (lane == 0) {
    sh[0][warp] = G;
    sh[1][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double g2 = 0.0, s2 = 0.0;
    for (int w = 0; w < kAdjBlock / 32; ++w) {
      g2 += sh[0][w];
      s2 += sh[1][w];
    }
    a.part[2 * blockIdx.x] = g2;
    a.part[2 * blockIdx.x + 1] = s2;
    __threadfence();
    ticket = atomicAdd(a.arrive, 1u);
  }
  __syncthreads();
  if (ticket != gridDim.x - 1 || threadIdx.x != 0) return;
  double g3 = 0.0, s3 = 0.0;
  for (unsigned b = 0; b < gridDim.x; ++b) {
    g3 += *reinterpret_cast<volatile double*>(a.part + 2 * b);
    s3 += *reinterpret_cast<volatile double*>(a.part + 2 * b + 1);
  }
  a.scal[0] = g3;
  a.scal[1] = s3;
  *a.arrive = 0u;
}

__global__ void __launch_bounds__(kAdjBlock) k_adj_update(AdjArgs a) {
  const double lam = *a.lam;
  const double G = a.scal[0], s = a.scal[1];
  const bool interior = a.exact && lam > 0.0 && lam < 1.0 && G > 0.0;
  const double coef = interior ? -s / G : 0.0;
  for (int k = blockIdx.x * kAdjBlock + threadIdx.x; k < a.m; k += gridDim.x * kAdjBlock) {
    const double d = a.d[k];
    double xb = (1.0 - lam) * a.xbar[k];
    if (interior) {
      const double q = __dadd_rn(a.x[k], __dmul_rn(lam, d));
      const double fft = a.lp.fft[k], al = a.lp.alpha[k], be = a.lp.beta[k], c = a.cap[k];
      const unsigned char ip = a.lp.ipow[k];
      const double t = bprf::cost(fft, al, be, ip, c, q);
      const double tp = bprf::dcost_dq(fft, al, be, ip, c, q);
      xb += coef * (tp * (1.0 - lam) * d - t);
      a.cbar[k] += coef * bprf::dcost_dcap(fft, al, be, ip, c, q) * d;
    }
    a.xbar[k] = xb;
  }
}

}  // namespace

}  // namespace tapgpu

#define TA_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      ::tapgpu::set_message(std::string(#call) + ": " + cudaGetErrorString(e_));       \
      return TAPGPU_ERR_CUDA;                                                           \
    }                                                                                   \
  } while (0)

extern "C" {

int tapgpu_adjoint_vht(tapgpu_ctx* ctx, int scenario, double* grad, double* vht) {
  using tapgpu::Ctx;
  if (!ctx || !grad) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  if (scenario < 0 || scenario >= c->S_cap) return TAPGPU_ERR_ARG;
  if (!c->d_hist) {
    tapgpu::set_message("the adjoint needs a solve recorded with record_tape");
    return TAPGPU_ERR_ARG;
  }
  TA_CUDA(cudaSetDevice(c->device));
  TA_CUDA(cudaStreamSynchronize(c->stream));
  tapgpu::ScenState st;
  TA_CUDA(cudaMemcpy(&st, c->state + scenario, sizeof(st), cudaMemcpyDeviceToHost));
  const int K = st.iter;
  if (K > c->hist_cap) {
    tapgpu::set_message("more iterations than the tape holds (raise tape_capacity)");
    return TAPGPU_ERR_UNSUPPORTED;
  }
  const int M = c->M, C = c->ckpt_every;
  const int grid = std::max(1, std::min((M + tapgpu::kAdjBlock - 1) / tapgpu::kAdjBlock,
                                        2 * c->num_sms));
  if (!c->adj_xbar) {
    if (c->alloc_n(&c->adj_xbar, M) || c->alloc_n(&c->adj_cbar, M) ||
        c->alloc_n(&c->adj_seg, static_cast<size_t>(C) * M) ||
        c->alloc_n(&c->adj_part, static_cast<size_t>(2) * 4 * c->num_sms) ||
        c->alloc_n(&c->adj_scal, 2) || c->alloc_n(&c->adj_arrive, 1))
      return TAPGPU_ERR_ALLOC;
    TA_CUDA(cudaMemset(c->adj_arrive, 0, sizeof(unsigned)));
  }
  const size_t off = static_cast<size_t>(scenario) * M;
  const size_t nck = static_cast<size_t>(c->hist_cap / C + 1);
  cudaStream_t s = c->stream;
  tapgpu::k_adj_init<<<grid, tapgpu::kAdjBlock, 0, s>>>(M, c->link_params_of(scenario), c->cap + off,
                                                         c->x + off, c->adj_xbar, c->adj_cbar);
  TA_CUDA(cudaGetLastError());
  const double* dh = c->d_hist + static_cast<size_t>(scenario) * c->hist_cap * M;
  const double* lh = c->lam_hist + static_cast<size_t>(scenario) * c->hist_cap;
  const double* xh = c->x_hist + static_cast<size_t>(scenario) * nck * M;
  for (int seg = K > 0 ? (K - 1) / C : -1; seg >= 0; --seg) {
    const int k0 = seg * C;
    const int len = std::min(C, K - k0);
    tapgpu::k_adj_recompute<<<grid, tapgpu::kAdjBlock, 0, s>>>(
        M, xh + static_cast<size_t>(seg) * M, dh, lh, k0, len, c->adj_seg);
    TA_CUDA(cudaGetLastError());
    for (int k = k0 + len - 1; k >= k0; --k) {
      tapgpu::AdjArgs a;
      a.m = M;
      a.lp = c->link_params_of(scenario);
      a.cap = c->cap + off;
      a.x = c->adj_seg + static_cast<size_t>(k - k0) * M;
      a.d = dh + static_cast<size_t>(k) * M;
      a.lam = lh + k;
      a.exact = c->ls_mode == tapgpu::kLsExact ? 1 : 0;
      a.xbar = c->adj_xbar;
      a.cbar = c->adj_cbar;
      a.part = c->adj_part;
      a.arrive = c->adj_arrive;
      a.scal = c->adj_scal;
      tapgpu::k_adj_reduce<<<grid, tapgpu::kAdjBlock, 0, s>>>(a);
      tapgpu::k_adj_update<<<grid, tapgpu::kAdjBlock, 0, s>>>(a);
      TA_CUDA(cudaGetLastError());
    }
  }
  std::vector<double> g(M);
  TA_CUDA(cudaMemcpyAsync(g.data(), c->adj_cbar, sizeof(double) * M, cudaMemcpyDeviceToHost, s));
  TA_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k < M; ++k) grad[c->perm[k]] = g[k];
  if (vht) *vht = st.vht_end;
  return TAPGPU_OK;
}

int tapgpu_get_tape(tapgpu_ctx* ctx, int scenario, int iteration, double* x_checkpoint,
                    double* direction, double* lambda) {
  using tapgpu::Ctx;
  if (!ctx) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  if (!c->d_hist || scenario < 0 || scenario >= c->S_cap || iteration < 0 ||
      iteration >= c->hist_cap)
    return TAPGPU_ERR_ARG;
  TA_CUDA(cudaSetDevice(c->device));
  TA_CUDA(cudaStreamSynchronize(c->stream));
  const int M = c->M;
  std::vector<double> tmp(M);
  if (direction) {
    TA_CUDA(cudaMemcpy(tmp.data(),
                       c->d_hist + (static_cast<size_t>(scenario) * c->hist_cap + iteration) * M,
                       sizeof(double) * M, cudaMemcpyDeviceToHost));
    for (int k = 0; k < M; ++k) direction[c->perm[k]] = tmp[k];
  }
  if (lambda)
    TA_CUDA(cudaMemcpy(lambda, c->lam_hist + static_cast<size_t>(scenario) * c->hist_cap + iteration,
                       sizeof(double), cudaMemcpyDeviceToHost));
  if (x_checkpoint) {
    if (iteration % c->ckpt_every != 0) return TAPGPU_ERR_ARG;
    const size_t nck = static_cast<size_t>(c->hist_cap / c->ckpt_every + 1);
    TA_CUDA(cudaMemcpy(tmp.data(),
                       c->x_hist + (static_cast<size_t>(scenario) * nck +
                                    iteration / c->ckpt_every) * M,
                       sizeof(double) * M, cudaMemcpyDeviceToHost));
    for (int k = 0; k < M; ++k) x_checkpoint[c->perm[k]] = tmp[k];
  }
  return TAPGPU_OK;
}

}  // extern "C"
