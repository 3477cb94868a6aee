// linkops.cuh - device copies of one link table for the array numerics of the
// drop-in tap_functions.h entry points.
#pragma once
#include <cuda_runtime.h>

namespace tapgpu {

struct LinkArrays {
  const double* fft;
  const double* alpha;
  const double* beta;
  const double* cap;
  const unsigned char* ipow;
};

class LinkOps {
 public:
  static constexpr int kGrid = 304;
  ~LinkOps();
  // (re)load the link parameters; returns 0 on success
  int upload(int nlinks, const double* fft, const double* alpha, const double* beta,
             const double* cap);
  int costs(const double* x, double* t);           // t = BPR(x)
  int set_xd(const double* x, const double* d);    // stage x and d (either may be NULL)
  // op 0: g(lam_j) for j < nl; op 1: Beckmann objective of x; op 2: x.d
  int sums(int op, const double* lams, int nl, double* out);
  static int max_lambdas();
  int size() const { return m; }

 private:
  void release();
  LinkArrays arrays() const;
  int m = 0;
  double *fft = nullptr, *alpha = nullptr, *beta = nullptr, *cap = nullptr;
  double *x = nullptr, *d = nullptr, *t = nullptr, *lams = nullptr, *part = nullptr;
  unsigned char* ipow = nullptr;
};

}  // namespace tapgpu
