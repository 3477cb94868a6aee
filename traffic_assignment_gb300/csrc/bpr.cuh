// bpr.cuh - BPR link cost and its derivatives on the device (FP64, explicit
// rounding so the operation order matches tap/tap_functions.c).
//   t(q)      = fft (1 + alpha (q / cap)^beta)                tap/tap_functions.c:55-65
//   dt/dq     = fft alpha beta q^(beta-1) / cap^beta
//   dt/dcap   = -fft alpha beta q^beta / cap^(beta+1)
//   integral  = q fft (1 + (alpha / cap^beta) / (beta+1) q^beta)  tap/tap_functions.c:112-126
// Integer powers 0..15 (the usual beta = 4) are formed by repeated squaring.
#pragma once
#include <cuda_runtime.h>

namespace tapgpu {
namespace bprf {

__device__ __forceinline__ double int_pow(double r, int n) {
  double acc = 1.0, b = r;
  while (n) {
    if (n & 1) acc = __dmul_rn(acc, b);
    n >>= 1;
    if (n) b = __dmul_rn(b, b);
  }
  return acc;
}

// r^n for the FP32-path forms, where rounding need not follow the reference:
// the usual beta = 4 as two squarings
__device__ __forceinline__ double int_pow_fast(double r, int n) {
  if (n == 4) {
    const double r2 = r * r;
    return r2 * r2;
  }
  return int_pow(r, n);
}

// 1 / n, the integral's 1 / (beta + 1) for integer beta (beta = 4 without a division)
__device__ __forceinline__ double inv_int(int n) {
  return n == 5 ? 0.2 : 1.0 / static_cast<double>(n);
}

// r^beta; ip is beta when beta is an integer 0..15, else 255
__device__ __forceinline__ double pow_p(double r, double beta, unsigned char ip) {
  return ip != 255 ? int_pow(r, ip) : pow(r, beta);
}

__device__ __forceinline__ double cost(double fft, double alpha, double beta, unsigned char ip,
                                       double cap, double q) {
  const double p = pow_p(__ddiv_rn(q, cap), beta, ip);
  return __dmul_rn(fft, __dadd_rn(1.0, __dmul_rn(alpha, p)));
}

__device__ __forceinline__ double dcost_dq(double fft, double alpha, double beta,
                                           unsigned char ip, double cap, double q) {
  if (beta == 0.0) return 0.0;
  const double r = q / cap;
  const double p1 = ip != 255 ? (ip >= 1 ? int_pow(r, ip - 1) : 0.0) : pow(r, beta - 1.0);
  return fft * alpha * beta * p1 / cap;
}

__device__ __forceinline__ double dcost_dcap(double fft, double alpha, double beta,
                                             unsigned char ip, double cap, double q) {
  const double r = q / cap;
  return -fft * alpha * beta * pow_p(r, beta, ip) / cap;
}

__device__ __forceinline__ double integral(double fft, double alpha, double beta,
                                           unsigned char ip, double cap, double q) {
  if (!(beta >= 0)) return 0.0;
  const double a = __ddiv_rn(__ddiv_rn(alpha, pow_p(cap, beta, ip)), __dadd_rn(beta, 1.0));
  return __dmul_rn(__dmul_rn(q, fft), __dadd_rn(1.0, __dmul_rn(a, pow_p(q, beta, ip))));
}

}  // namespace bprf
}  // namespace tapgpu
