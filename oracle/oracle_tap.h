/*
 * oracle_tap.h - CPU oracle for the Frank-Wolfe user-equilibrium loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * solver (stivalaa/traffic_assignment, trunk/tap) used to check the GPU
 * library and to time the CPU baseline.  Nothing in the shipped library links
 * to it; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * load it.
 *
 * Conventions are the reference's: nodes 1..N with a dummy row 0, zones 1..Z,
 * links sorted by (init, term) so that link k is edge k of the forward star,
 * and nodes below first_thru_node are only expanded when they are the source.
 */
#ifndef ORACLE_TAP_H
#define ORACLE_TAP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* network + demand, flattened (see tap/tap_types.h:20-53 for the originals) */
typedef struct orc_problem_s {
  int64_t num_nodes;       /* N (nodes are 1..N) */
  int64_t num_zones;       /* Z (zones are nodes 1..Z) */
  int64_t first_thru_node; /* tap/tap_types.h:40 */
  int64_t num_links;       /* M */
  const int64_t *init;     /* [M] tail node, sorted by (init, term) */
  const int64_t *term;     /* [M] head node */
  const double *capacity;  /* [M] */
  const double *fft;       /* [M] free-flow time */
  const double *alpha;     /* [M] BPR B */
  const double *beta;      /* [M] BPR power */
  const int64_t *od_ptr;   /* [Z+2] origin o owns entries od_ptr[o]..od_ptr[o+1]-1 */
  const int64_t *od_dest;  /* destinations, in trips-file order */
  const double *od_demand; /* demand of each entry */
} orc_problem_t;

/* one row of the per-iteration log (tap/tap_frankwolfe_pthread.c:751-753) */
typedef struct orc_iter_s {
  double objective;   /* Beckmann objective at x before the step */
  double relgap;      /* relative gap after this iteration's bound update */
  double avg_excess;  /* -sum(delta*t)/total_demand */
  double total_cost;  /* VHT sum(x*t) at x before the step */
  double lambda;      /* step size chosen by the line search */
  double gap;         /* -g(0) */
  double ms;          /* wall time of the iteration */
} orc_iter_t;

enum { ORC_OK = 0, ORC_ERR_NO_PATH = 2, ORC_ERR_ALLOC = 3, ORC_ERR_ARG = 4 };

/* tap/sssp_pape.c:120-220 */
void orc_sssp_pape(const int64_t Va[], const int64_t Ea[], const double Wa[],
                   int64_t num_nodes, int64_t num_edges, int64_t start_node,
                   int64_t first_thru_node, int64_t prevlink[], double dist[],
                   int64_t queue_next[]);

/* tap/sssp_pape.c:284-501 */
void orc_sssp_pape_lll(const int64_t Va[], const int64_t Ea[], const double Wa[],
                       int64_t num_nodes, int64_t num_edges, int64_t start_node,
                       int64_t first_thru_node, int64_t prevlink[], double dist[],
                       int64_t queue_next[]);

/* all origins 1..num_sources of a forward star; dist/pred are [num_sources][num_nodes] */
int orc_sssp_many(const int64_t Va[], const int64_t Ea[], const double Wa[],
                  int64_t num_nodes, int64_t num_edges, const int64_t *sources,
                  int64_t num_sources, int64_t first_thru_node, int use_lll,
                  int num_threads, double *dist, int64_t *pred);

/* tap/tap_functions.c:55-65 */
double orc_bpr(double fft, double alpha, double beta, double capacity, double q);
/* tap/tap_functions.c:112-126 */
double orc_linkcost_integral(double fft, double alpha, double beta, double capacity,
                             double q);
/* tap/tap_functions.c:83-97 over a problem's links */
double orc_directional_derivative(const orc_problem_t *p, const double *cap,
                                  const double *x, const double *d, double lambda);
/* tap/tap_functions.c:469-507 */
double orc_line_search(const orc_problem_t *p, const double *cap, const double *x,
                       const double *d);
/* tap/tap_functions.c:143-152 */
double orc_objective(const orc_problem_t *p, const double *cap, const double *x);

/* All-or-nothing loading at costs t (tap/tap_frankwolfe_pthread.c:262-433). */
int orc_aon(const orc_problem_t *p, const double *t, int num_threads, double *y);

/*
 * Full Frank-Wolfe solve (tap/tap_frankwolfe_pthread.c:488-825).
 *   x0             optional warm-start volumes (NULL = cold start)
 *   max_iters      iteration cap (<= 0: none)
 *   target_relgap  stop when relgap <= target (<= 0: none)
 *   x_out, t_out   final volumes and costs [M]
 *   trace          optional per-iteration rows, up to trace_cap
 *   summary        [4]: iterations, objective, relgap, total cost at end
 */
int orc_frankwolfe(const orc_problem_t *p, int num_threads, const double *x0,
                   int max_iters, double target_relgap, double *x_out, double *t_out,
                   orc_iter_t *trace, int trace_cap, double *summary);

/* oracle_adjoint.c: FP64 CPU reference of the VHT adjoint (frozen loads Y [K][M],
 * exact steps): the replay for finite differences and the reverse sweep on a tape */
double orc_replay_vht(const orc_problem_t *p, const double *cap, int K, const double *x0,
                      const double *Y, double *lam_out);
int orc_adjoint_vht(const orc_problem_t *p, const double *cap, int K, const double *x0,
                    const double *D, const double *lam, double *grad);

#ifdef __cplusplus
}
#endif
#endif /* ORACLE_TAP_H */
