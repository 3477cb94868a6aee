/*
 * oracle_tap.c - CPU oracle for the Frank-Wolfe user-equilibrium loop.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle_tap.h).  A restatement, in this
 * project's own code, of the reference's CPU algorithm for the hot path:
 * d'Esopo-Pape shortest paths with the Large-Label-Last rule, all-or-nothing
 * loading by predecessor walks, BPR costs, the Beckmann objective, the 2^-k
 * line search and the Frank-Wolfe driver loop.  Each function cites the
 * reference file:line it follows (paths relative to trunk/).  The operation
 * order of every floating-point sum matches the reference so that a
 * single-threaded run reproduces `tap_frankwolfe_pthread -n 1` bit for bit.
 */
#define _POSIX_C_SOURCE 200809L
#include "oracle_tap.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define Q_NEVER (-1) /* node has never been queued */
#define Q_LEFT (-2)  /* node was queued and has since been removed */

/* ------------------------------------------------------------------------ */
/* shortest paths                                                           */
/* ------------------------------------------------------------------------ */

/* tap/sssp_pape.c:120-220: d'Esopo-Pape.  Labels are corrected in place; a
 * node that re-enters the queue goes to its head, a first-time node to its
 * tail. */
void orc_sssp_pape(const int64_t Va[], const int64_t Ea[], const double Wa[],
                   int64_t num_nodes, int64_t num_edges, int64_t start_node,
                   int64_t first_thru_node, int64_t prevlink[], double dist[],
                   int64_t queue_next[])
{
  (void)num_edges;
  for (int64_t v = 0; v < num_nodes; v++) {
    prevlink[v] = -1;
    queue_next[v] = Q_NEVER;
    dist[v] = (v == start_node) ? 0.0 : DBL_MAX;
  }
  int64_t head = Q_NEVER, tail = Q_NEVER;
  int64_t u = start_node;
  while (u >= 0) {
    if (u >= first_thru_node || u == start_node) {
      for (int64_t e = Va[u]; e < Va[u + 1]; e++) {
        int64_t v = Ea[e];
        double cand = dist[u] + Wa[e];
        if (cand < dist[v]) {
          dist[v] = cand;
          prevlink[v] = e;
          if (queue_next[v] == Q_LEFT) { /* re-entry: front of the queue */
            queue_next[v] = head;
            head = v;
            if (tail == Q_NEVER) tail = v;
          } else if (queue_next[v] == Q_NEVER && v != tail) { /* first entry: back */
            if (tail != Q_NEVER) {
              queue_next[tail] = v;
              tail = v;
            } else {
              head = tail = v;
              queue_next[v] = Q_NEVER;
            }
          }
        }
      }
    }
    u = head;
    if (u < 0) break;
    head = queue_next[u];
    queue_next[u] = Q_LEFT;
    if (tail == u) tail = Q_NEVER;
  }
}

/* tap/sssp_pape.c:284-501: d'Esopo-Pape with Large-Label-Last.  The queue
 * keeps a running label sum (plain summation, USE_KAHAN_SUM is off at
 * :39); before each scan, heads whose label exceeds the queue average are
 * rotated to the tail, at most queue_size-1 of them. */
void orc_sssp_pape_lll(const int64_t Va[], const int64_t Ea[], const double Wa[],
                       int64_t num_nodes, int64_t num_edges, int64_t start_node,
                       int64_t first_thru_node, int64_t prevlink[], double dist[],
                       int64_t queue_next[])
{
  (void)num_edges;
  for (int64_t v = 0; v < num_nodes; v++) {
    prevlink[v] = -1;
    queue_next[v] = Q_NEVER;
    dist[v] = (v == start_node) ? 0.0 : DBL_MAX;
  }
  int64_t head = Q_NEVER, tail = Q_NEVER;
  int64_t qsize = 0;
  double qsum = 0.0;
  int64_t u = start_node;
  while (u >= 0) {
    if (u >= first_thru_node || u == start_node) {
      for (int64_t e = Va[u]; e < Va[u + 1]; e++) {
        int64_t v = Ea[e];
        double cand = dist[u] + Wa[e];
        if (cand < dist[v]) {
          double before = dist[v];
          dist[v] = cand;
          prevlink[v] = e;
          if (queue_next[v] == Q_LEFT) {
            queue_next[v] = head;
            head = v;
            if (tail == Q_NEVER) tail = v;
            ++qsize;
            qsum += dist[v];
          } else if (queue_next[v] == Q_NEVER && v != tail) {
            if (tail != Q_NEVER) {
              queue_next[tail] = v;
              tail = v;
              ++qsize;
              qsum += dist[v];
            } else {
              head = tail = v;
              queue_next[v] = Q_NEVER;
              qsize = 1;
              qsum = dist[v];
            }
          } else { /* already queued: the sum tracks the lowered label */
            qsum += cand;
            qsum += -before;
          }
        }
      }
    }
    double mean = qsum / (double)qsize;
    int64_t seen = 0;
    u = head;
    while (seen < qsize) {
      int64_t after = queue_next[u];
      if (qsize > 1 && dist[u] > mean && seen < qsize - 1) {
        /* large label: rotate the head to the tail */
        head = queue_next[u];
        queue_next[u] = Q_NEVER;
        if (tail != Q_NEVER) {
          queue_next[tail] = u;
          tail = u;
        } else {
          head = tail = u;
        }
      } else {
        /* scan this node next */
        head = queue_next[u];
        queue_next[u] = Q_LEFT;
        if (tail == u) tail = Q_NEVER;
        --qsize;
        qsum += -dist[u];
        break;
      }
      ++seen;
      u = after;
    }
  }
}

typedef struct {
  const int64_t *Va, *Ea;
  const double *Wa;
  int64_t num_nodes, num_edges, first_thru, num_sources;
  const int64_t *sources;
  int use_lll;
  double *dist;
  int64_t *pred;
  int64_t lo, hi;
} many_job_t;

static void *many_worker(void *arg)
{
  many_job_t *j = (many_job_t *)arg;
  int64_t *qn = (int64_t *)malloc((size_t)j->num_nodes * sizeof(int64_t));
  if (!qn) return (void *)1;
  for (int64_t i = j->lo; i < j->hi; i++) {
    double *d = j->dist + i * j->num_nodes;
    int64_t *p = j->pred + i * j->num_nodes;
    if (j->use_lll)
      orc_sssp_pape_lll(j->Va, j->Ea, j->Wa, j->num_nodes, j->num_edges, j->sources[i],
                        j->first_thru, p, d, qn);
    else
      orc_sssp_pape(j->Va, j->Ea, j->Wa, j->num_nodes, j->num_edges, j->sources[i],
                    j->first_thru, p, d, qn);
  }
  free(qn);
  return NULL;
}

int orc_sssp_many(const int64_t Va[], const int64_t Ea[], const double Wa[],
                  int64_t num_nodes, int64_t num_edges, const int64_t *sources,
                  int64_t num_sources, int64_t first_thru_node, int use_lll,
                  int num_threads, double *dist, int64_t *pred)
{
  if (num_threads < 1) num_threads = 1;
  if (num_threads > 512) num_threads = 512;
  pthread_t th[512];
  many_job_t jobs[512];
  int64_t per = (num_sources + num_threads - 1) / num_threads;
  int started = 0, rc = ORC_OK;
  for (int t = 0; t < num_threads; t++) {
    many_job_t *j = &jobs[t];
    j->Va = Va; j->Ea = Ea; j->Wa = Wa;
    j->num_nodes = num_nodes; j->num_edges = num_edges; j->first_thru = first_thru_node;
    j->num_sources = num_sources; j->sources = sources; j->use_lll = use_lll;
    j->dist = dist; j->pred = pred;
    j->lo = (int64_t)t * per;
    j->hi = j->lo + per < num_sources ? j->lo + per : num_sources;
    if (j->lo >= j->hi) break;
    if (pthread_create(&th[t], NULL, many_worker, j) != 0) { rc = ORC_ERR_ALLOC; break; }
    started++;
  }
  for (int t = 0; t < started; t++) {
    void *r = NULL;
    pthread_join(th[t], &r);
    if (r) rc = ORC_ERR_ALLOC;
  }
  return rc;
}

/* ------------------------------------------------------------------------ */
/* link cost numerics                                                       */
/* ------------------------------------------------------------------------ */

/* tap/tap_functions.c:55-65 */
double orc_bpr(double fft, double alpha, double beta, double capacity, double q)
{
  return fft * (1.0 + alpha * pow(q / capacity, beta));
}

/* tap/tap_functions.c:112-126 (note the algebraic form differs from orc_bpr) */
double orc_linkcost_integral(double fft, double alpha, double beta, double capacity,
                             double q)
{
  if (beta >= 0)
    return q * fft * (1 + ((alpha / pow(capacity, beta)) / (beta + 1)) * pow(q, beta));
  return 0;
}

/* tap/tap_functions.c:83-97: g(lambda) = sum_k t_k(x_k + lambda d_k) d_k */
double orc_directional_derivative(const orc_problem_t *p, const double *cap,
                                  const double *x, const double *d, double lambda)
{
  double s = 0;
  for (int64_t k = 0; k < p->num_links; k++) {
    double q = x[k] + lambda * d[k];
    s += orc_bpr(p->fft[k], p->alpha[k], p->beta[k], cap[k], q) * d[k];
  }
  return s;
}

/* tap/tap_functions.c:469-507.  Returns 0 if g(0) >= 0, 1 if g(1) <= 0, else
 * the largest 2^-k (k >= 1) with g(2^-k) <= 0, giving up after 1000 halvings
 * (the loop at :496 stops as soon as lambda_left moves off zero). */
double orc_line_search(const orc_problem_t *p, const double *cap, const double *x,
                       const double *d)
{
  if (orc_directional_derivative(p, cap, x, d, 0.0) >= 0) return 0.0;
  if (orc_directional_derivative(p, cap, x, d, 1.0) <= 0) return 1.0;
  double left = 0.0, right = 1.0, lam = 0.5;
  if (orc_directional_derivative(p, cap, x, d, lam) <= 0) left = lam;
  else right = lam;
  lam = 0.5 * (left + right);
  for (int n = 0; left == 0 && n < 1000; n++) {
    if (orc_directional_derivative(p, cap, x, d, lam) <= 0) left = lam;
    else right = lam;
    lam = 0.5 * (left + right);
  }
  return left;
}

/* tap/tap_functions.c:143-152 */
double orc_objective(const orc_problem_t *p, const double *cap, const double *x)
{
  double s = 0;
  for (int64_t k = 0; k < p->num_links; k++)
    s += orc_linkcost_integral(p->fft[k], p->alpha[k], p->beta[k], cap[k], x[k]);
  return s;
}

/* tap/tap_functions.c:408-417 */
static double vht(int64_t m, const double *x, const double *t)
{
  double s = 0;
  for (int64_t k = 0; k < m; k++) s += x[k] * t[k];
  return s;
}

/* ------------------------------------------------------------------------ */
/* all-or-nothing loading                                                   */
/* ------------------------------------------------------------------------ */

/* tap/tap_frankwolfe_pthread.c:182-200: lock-free add by compare-and-swap */
static void add_double_atomic(double *addr, double val)
{
  uint64_t *w = (uint64_t *)addr;
  uint64_t seen = __atomic_load_n(w, __ATOMIC_RELAXED);
  for (;;) {
    double cur;
    memcpy(&cur, &seen, sizeof cur);
    double nv = cur + val;
    uint64_t want;
    memcpy(&want, &nv, sizeof want);
    if (__atomic_compare_exchange_n(w, &seen, want, 0, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST))
      return;
  }
}

typedef struct {
  const orc_problem_t *p;
  const int64_t *Va, *Ea;
  const double *Wa;
  double *y;
  int64_t first, last; /* origins first..last inclusive */
  int err;
  int64_t bad_orig, bad_dest;
} aon_job_t;

/* tap/tap_frankwolfe_pthread.c:262-310 */
static void *aon_worker(void *arg)
{
  aon_job_t *j = (aon_job_t *)arg;
  const orc_problem_t *p = j->p;
  int64_t n1 = p->num_nodes + 1;
  int64_t *pred = (int64_t *)malloc((size_t)n1 * sizeof(int64_t));
  int64_t *qn = (int64_t *)malloc((size_t)n1 * sizeof(int64_t));
  double *dist = (double *)malloc((size_t)n1 * sizeof(double));
  if (!pred || !qn || !dist) {
    j->err = ORC_ERR_ALLOC;
    free(pred); free(qn); free(dist);
    return NULL;
  }
  for (int64_t o = j->first; o <= j->last && o < p->num_zones + 1; o++) {
    orc_sssp_pape_lll(j->Va, j->Ea, j->Wa, n1, p->num_links, o, p->first_thru_node,
                      pred, dist, qn);
    for (int64_t i = p->od_ptr[o]; i < p->od_ptr[o + 1]; i++) {
      int64_t dest = p->od_dest[i];
      double flow = p->od_demand[i];
      if (dest == o || flow <= 0) continue;
      int64_t v = dest;
      while (v != o) {
        int64_t k = pred[v];
        if (k < 0) {
          j->err = ORC_ERR_NO_PATH;
          j->bad_orig = o;
          j->bad_dest = dest;
          goto done;
        }
        add_double_atomic(&j->y[k], flow);
        v = p->init[k];
      }
    }
  }
done:
  free(pred); free(qn); free(dist);
  return NULL;
}

/* tap/tap_frankwolfe_pthread.c:345-433: origins split into blocks of
 * ceil(Z / threads), one block per thread, shared volumes updated atomically. */
static int aon_impl(const orc_problem_t *p, const int64_t *Va, const int64_t *Ea,
                    const double *Wa, int num_threads, double *y)
{
  if (num_threads < 1) num_threads = 1;
  if (num_threads > 512) num_threads = 512;
  for (int64_t k = 0; k < p->num_links; k++) y[k] = 0;
  int64_t per = (p->num_zones + num_threads - 1) / num_threads;
  pthread_t th[512];
  aon_job_t jobs[512];
  int started = 0;
  int rc = ORC_OK;
  for (int t = 0; t < num_threads; t++) {
    aon_job_t *j = &jobs[t];
    j->p = p; j->Va = Va; j->Ea = Ea; j->Wa = Wa; j->y = y;
    j->first = 1 + (int64_t)t * per;
    j->last = j->first + per - 1;
    j->err = 0;
    if (num_threads == 1) {
      aon_worker(j);
      started = -1;
      break;
    }
    if (pthread_create(&th[t], NULL, aon_worker, j) != 0) { rc = ORC_ERR_ALLOC; break; }
    started++;
  }
  if (started < 0) return jobs[0].err;
  for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
  for (int t = 0; t < started; t++)
    if (jobs[t].err) rc = jobs[t].err;
  return rc;
}

static void build_csr(const orc_problem_t *p, int64_t *Va, int64_t *Ea)
{
  /* tap/tap_functions.c:313-339 over num_nodes+1 rows (row 0 is a dummy) */
  int64_t e = 0;
  int64_t rows = p->num_nodes + 1;
  for (int64_t v = 0; v < rows; v++) {
    Va[v] = e;
    while (e < p->num_links && p->init[e] == v) {
      Ea[e] = p->term[e];
      e++;
    }
  }
  Va[rows] = e;
}

int orc_aon(const orc_problem_t *p, const double *t, int num_threads, double *y)
{
  int64_t *Va = (int64_t *)malloc((size_t)(p->num_nodes + 2) * sizeof(int64_t));
  int64_t *Ea = (int64_t *)malloc((size_t)(p->num_links + 1) * sizeof(int64_t));
  if (!Va || !Ea) { free(Va); free(Ea); return ORC_ERR_ALLOC; }
  build_csr(p, Va, Ea);
  int rc = aon_impl(p, Va, Ea, t, num_threads, y);
  free(Va); free(Ea);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Frank-Wolfe driver                                                       */
/* ------------------------------------------------------------------------ */

static double now_ms(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

/* tap/tap_frankwolfe_pthread.c:488-825 */
int orc_frankwolfe(const orc_problem_t *p, int num_threads, const double *x0,
                   int max_iters, double target_relgap, double *x_out, double *t_out,
                   orc_iter_t *trace, int trace_cap, double *summary)
{
  int64_t m = p->num_links;
  if (m <= 0 || p->num_nodes <= 0) return ORC_ERR_ARG;
  int64_t *Va = (int64_t *)malloc((size_t)(p->num_nodes + 2) * sizeof(int64_t));
  int64_t *Ea = (int64_t *)malloc((size_t)m * sizeof(int64_t));
  double *x = x_out, *t = t_out;
  double *d = (double *)malloc((size_t)m * sizeof(double));
  double *cap = (double *)malloc((size_t)m * sizeof(double));
  if (!Va || !Ea || !d || !cap) {
    free(Va); free(Ea); free(d); free(cap);
    return ORC_ERR_ALLOC;
  }

  /* :654-669 zero capacity -> smallest nonzero capacity */
  double min_cap = DBL_MAX;
  for (int64_t k = 0; k < m; k++)
    if (p->capacity[k] > 0.0 && p->capacity[k] < min_cap) min_cap = p->capacity[k];
  for (int64_t k = 0; k < m; k++)
    cap[k] = p->capacity[k] <= 0.0 ? min_cap : p->capacity[k];

  /* :672 CSR with the free-flow times as the first costs */
  build_csr(p, Va, Ea);
  for (int64_t k = 0; k < m; k++) t[k] = p->fft[k];

  /* tap/tap_functions.c:377-386 over origins 1..Z */
  double total_demand = 0;
  for (int64_t o = 1; o < p->num_zones + 1; o++)
    for (int64_t i = p->od_ptr[o]; i < p->od_ptr[o + 1]; i++)
      total_demand += p->od_demand[i];

  int rc = ORC_OK;
  int iter = 0;
  double relgap = DBL_MAX, best_lb = -DBL_MAX, obj = 0;
  if (x0) {
    /* :677-691 warm start; iteration state is defined here (the reference
     * leaves it uninitialised on this branch) */
    for (int64_t k = 0; k < m; k++) x[k] = x0[k];
    for (int64_t k = 0; k < m; k++)
      t[k] = orc_bpr(p->fft[k], p->alpha[k], p->beta[k], cap[k], x[k]);
  } else {
    /* :702-710 initial all-or-nothing at free-flow costs */
    rc = aon_impl(p, Va, Ea, t, num_threads, x);
    if (rc) goto out;
    for (int64_t k = 0; k < m; k++)
      t[k] = orc_bpr(p->fft[k], p->alpha[k], p->beta[k], cap[k], x[k]);
  }

  /* :712-793 */
  while ((max_iters <= 0 || iter < max_iters) &&
         (target_relgap <= 0 || relgap > target_relgap)) {
    double t0 = now_ms();
    rc = aon_impl(p, Va, Ea, t, num_threads, d);
    if (rc) goto out;
    for (int64_t k = 0; k < m; k++) d[k] = d[k] - x[k];
    double lam = orc_line_search(p, cap, x, d);
    double gap = -orc_directional_derivative(p, cap, x, d, 0.0);
    obj = orc_objective(p, cap, x);
    double lb = obj - gap;
    if (lb > best_lb) best_lb = lb;
    if (best_lb != 0) relgap = (obj - best_lb) / fabs(best_lb);
    double avg_excess = -vht(m, d, t) / total_demand;
    double total_cost = vht(m, x, t);
    for (int64_t k = 0; k < m; k++) x[k] += lam * d[k];
    for (int64_t k = 0; k < m; k++)
      t[k] = orc_bpr(p->fft[k], p->alpha[k], p->beta[k], cap[k], x[k]);
    if (trace && iter < trace_cap) {
      orc_iter_t *r = &trace[iter];
      r->objective = obj;
      r->relgap = relgap;
      r->avg_excess = avg_excess;
      r->total_cost = total_cost;
      r->lambda = lam;
      r->gap = gap;
      r->ms = now_ms() - t0;
    }
    iter++;
  }
  if (summary) {
    summary[0] = iter;
    summary[1] = obj;
    summary[2] = relgap;
    summary[3] = vht(m, x, t); /* :795 */
  }
out:
  free(Va); free(Ea); free(d); free(cap);
  return rc;
}
