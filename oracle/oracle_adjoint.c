/*
 * oracle_adjoint.c - FP64 CPU reference for the VHT adjoint (TEST
 * INFRASTRUCTURE ONLY; the reference has no adjoint, so this follows the
 * mathematics stated in traffic_assignment_gb300/csrc/adjoint.cu).
 *
 *   orc_replay_vht   the frozen-decision map: x_0 given, loads y_k given,
 *                    d_k = y_k - x_k, lambda_k the exact root of
 *                    g(l) = sum t(x_k + l d_k) d_k on [0, 1],
 *                    x_{k+1} = x_k + lambda_k d_k, returns VHT(x_K).  Used for
 *                    central finite differences in the capacities.
 *   orc_adjoint_vht  reverse sweep of that map on a recorded tape
 *                    (x_0, d_k, lambda_k) -> dVHT/dcapacity.
 * The BPR cost is tap/tap_functions.c:55-65 (orc_bpr).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_tap.h"

static double dbpr_dq(double fft, double alpha, double beta, double cap, double q)
{
  if (beta == 0.0) return 0.0;
  return fft * alpha * beta * pow(q / cap, beta - 1.0) / cap;
}

static double dbpr_dcap(double fft, double alpha, double beta, double cap, double q)
{
  return -fft * alpha * beta * pow(q / cap, beta) / cap;
}

static double g_at(const orc_problem_t *p, const double *cap, const double *x, const double *d,
                   double lam)
{
  double s = 0;
  for (int64_t k = 0; k < p->num_links; k++)
    s += orc_bpr(p->fft[k], p->alpha[k], p->beta[k], cap[k], x[k] + lam * d[k]) * d[k];
  return s;
}

/* exact root of g on [0, 1]: 0 if g(0) >= 0, 1 if g(1) <= 0, else bisection
 * then linear interpolation inside the final bracket */
static double exact_step(const orc_problem_t *p, const double *cap, const double *x,
                         const double *d)
{
  double glo = g_at(p, cap, x, d, 0.0);
  if (glo >= 0) return 0.0;
  double ghi = g_at(p, cap, x, d, 1.0);
  if (ghi <= 0) return 1.0;
  double lo = 0.0, hi = 1.0;
  for (int it = 0; it < 200 && hi - lo > 1e-16 * hi; it++) {
    double mid = 0.5 * (lo + hi);
    double gm = g_at(p, cap, x, d, mid);
    if (gm > 0) { hi = mid; ghi = gm; } else { lo = mid; glo = gm; }
  }
  double den = glo - ghi;
  return den < 0 ? lo + (hi - lo) * (glo / den) : lo;
}

double orc_replay_vht(const orc_problem_t *p, const double *cap, int K, const double *x0,
                      const double *Y, double *lam_out)
{
  int64_t m = p->num_links;
  double *x = (double *)malloc((size_t)m * sizeof(double));
  double *d = (double *)malloc((size_t)m * sizeof(double));
  if (!x || !d) { free(x); free(d); return NAN; }
  memcpy(x, x0, (size_t)m * sizeof(double));
  for (int k = 0; k < K; k++) {
    const double *y = Y + (size_t)k * m;
    for (int64_t a = 0; a < m; a++) d[a] = y[a] - x[a];
    double lam = exact_step(p, cap, x, d);
    if (lam_out) lam_out[k] = lam;
    for (int64_t a = 0; a < m; a++) x[a] = x[a] + lam * d[a];
  }
  double v = 0;
  for (int64_t a = 0; a < m; a++)
    v += x[a] * orc_bpr(p->fft[a], p->alpha[a], p->beta[a], cap[a], x[a]);
  free(x);
  free(d);
  return v;
}

int orc_adjoint_vht(const orc_problem_t *p, const double *cap, int K, const double *x0,
                    const double *D, const double *lam, double *grad)
{
  int64_t m = p->num_links;
  double *X = (double *)malloc((size_t)(K + 1) * m * sizeof(double));
  double *xb = (double *)malloc((size_t)m * sizeof(double));
  if (!X || !xb) { free(X); free(xb); return ORC_ERR_ALLOC; }
  memcpy(X, x0, (size_t)m * sizeof(double));
  for (int k = 0; k < K; k++)
    for (int64_t a = 0; a < m; a++)
      X[(size_t)(k + 1) * m + a] = X[(size_t)k * m + a] + lam[k] * D[(size_t)k * m + a];
  const double *xK = X + (size_t)K * m;
  for (int64_t a = 0; a < m; a++) {
    double q = xK[a];
    xb[a] = orc_bpr(p->fft[a], p->alpha[a], p->beta[a], cap[a], q) +
            q * dbpr_dq(p->fft[a], p->alpha[a], p->beta[a], cap[a], q);
    grad[a] = q * dbpr_dcap(p->fft[a], p->alpha[a], p->beta[a], cap[a], q);
  }
  for (int k = K - 1; k >= 0; k--) {
    const double *x = X + (size_t)k * m, *d = D + (size_t)k * m;
    double l = lam[k];
    double G = 0, s = 0;
    for (int64_t a = 0; a < m; a++) {
      double q = x[a] + l * d[a];
      G += dbpr_dq(p->fft[a], p->alpha[a], p->beta[a], cap[a], q) * d[a] * d[a];
      s += xb[a] * d[a];
    }
    int interior = l > 0.0 && l < 1.0 && G > 0.0;
    double coef = interior ? -s / G : 0.0;
    for (int64_t a = 0; a < m; a++) {
      double xba = (1.0 - l) * xb[a];
      if (interior) {
        double q = x[a] + l * d[a];
        double t = orc_bpr(p->fft[a], p->alpha[a], p->beta[a], cap[a], q);
        double tp = dbpr_dq(p->fft[a], p->alpha[a], p->beta[a], cap[a], q);
        xba += coef * (tp * (1.0 - l) * d[a] - t);
        grad[a] += coef * dbpr_dcap(p->fft[a], p->alpha[a], p->beta[a], cap[a], q) * d[a];
      }
      xb[a] = xba;
    }
  }
  free(X);
  free(xb);
  return ORC_OK;
}
