/*
 * tap_gpu.h - C ABI of the GB300 Frank-Wolfe traffic-assignment library
 * (libtapgpu.so).
 *
 * Two layers:
 *
 *  1. Drop-in entry points with the reference's names, argument meanings and
 *     error behaviour (stivalaa/traffic_assignment, trunk/tap).  A driver
 *     written against the reference (tap_main.c, tap_mpi_main.c,
 *     tap_cuda_main.cu) links against this library instead of the reference
 *     objects.  Each declaration cites the reference declaration it replaces.
 *
 *  2. A handle API (tapgpu_*) with explicit contexts, status codes instead of
 *     exit(), plain pointers and sizes: single-scenario solves in FP64 or with
 *     FP32 path costs, batched upgrade-scenario solves, all-origins shortest
 *     paths, all-or-nothing loading and the dVHT/dcapacity adjoint.
 *
 * All computation runs on one CUDA device; there is no CPU fallback.  Node
 * and zone numbers are 1-based as in the reference (node 0 is an unused
 * dummy row); link k is the k-th link of the caller's link array.
 */
#ifndef TAP_GPU_H
#define TAP_GPU_H

#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Reference data types: same member order and types as tap/tap_types.h:20-100 */
/* ------------------------------------------------------------------------ */

typedef struct link_data_s {
  long init_node;        /* from node (1-based) */
  long term_node;        /* to node (1-based) */
  double capacity;       /* BPR Q_max */
  double length;
  double free_flow_time; /* BPR T_0 */
  double B;              /* BPR alpha */
  double power;          /* BPR beta */
  double speed_limit;
  double toll;
  short link_type;
} link_data_t;

typedef struct net_data_s {
  long num_zones;
  long num_nodes;
  long first_thru_node;
  long num_links;
  link_data_t *links;
} net_data_t;

typedef struct demand_data_s {
  long dest;     /* destination zone (1-based); 0 terminates a list */
  double demand;
} demand_data_t;

typedef struct link_flow_s {
  long init_node;
  long term_node;
  double volume;
  double cost;
} link_flow_t;

#define MAX_CHANGE_ID_LEN 127

typedef enum net_mod_type_e {
  MOD_TYPE_INVALID_E = 0,
  MOD_TYPE_ADD_E = 1,
  MOD_TYPE_CHANGE_E = 2
} net_mod_type_e;

typedef struct net_mod_s {
  char change_id[MAX_CHANGE_ID_LEN + 1];
  net_mod_type_e modtype;
  link_data_t mod_link;
  double project_cost;
} net_mod_t;

typedef enum trip_mod_type_e {
  TRIP_MOD_TYPE_INVALID_E = 0,
  TRIP_MOD_TYPE_POINT_E = 1,
  TRIP_MOD_TYPE_UNIFORM_E = 2,
  TRIP_MOD_TYPE_ALL_E = 3
} trip_mod_type_e;

typedef struct trip_mod_s {
  char trip_change_id[MAX_CHANGE_ID_LEN + 1];
  trip_mod_type_e trip_modtype;
  long origin;
  long dest;
  double multiplier;
} trip_mod_t;

/* ------------------------------------------------------------------------ */
/* Drop-in entry points                                                      */
/* ------------------------------------------------------------------------ */

/* replaces tap/tap_frankwolfe_pthread.h:23-24 (kept for link compatibility;
 * the GPU solver does not use host worker threads) */
extern unsigned int num_cores;
extern unsigned int num_threads;

/* replaces tap/tap_frankwolfe_pthread.h:30-38.  Same contract: takes
 * ownership of and frees `demands` and each demands[i]; replaces zero
 * capacities in net->links by the smallest nonzero capacity; closes
 * flows_input_fp in warm-start mode; rewinds and writes flow_fp in the
 * reference's flows format; returns 0, or 1 on failure (a missing path for a
 * positive demand prints "ERROR: no path from %ld to %ld" and exits 1, as
 * tap/tap_frankwolfe_pthread.c:291-298 does).  SIGUSR1/SIGUSR2/SIGTERM are
 * handled like the reference: status line, checkpoint, clean finish. */
int tap_frankwolfe(net_data_t *net, demand_data_t **demands, int warm_start_mode,
                   FILE *flows_input_fp, int target_iterations, double target_relgap,
                   FILE *flow_fp, double *total_cost_at_end, double *objvalue_at_end,
                   int *iterations_at_end, double *relgap_at_end, int time_each_iteration);

/* replaces tap/tap_frankwolfe_cuda.h:21 (ignored: there is one GPU generation) */
extern int using_fermi_architecture;

/* replaces tap/tap_frankwolfe_cuda.h:26-29: all-or-nothing volumes at costs
 * Wa for every origin 1..num_zones.  dist and predlink receive the
 * shortest-path labels and predecessor links in the [v*num_zones + s] layout
 * of tap/pape_cuda_host.cu (arrays of (num_nodes+1)*(num_zones+1) entries). */
void fw_assign(net_data_t *net, demand_data_t *demands[], long Va[], long Ea[], double Wa[],
               double link_volumes[], double dist[], long predlink[]);

/* replaces tap/pape_cuda_host.h:15-19: shortest paths from every start node;
 * distances[v*num_start_nodes + s] and predecessors[v*num_start_nodes + s]
 * for start node s (the reference's layout, which assumes s in
 * 1..num_start_nodes).  num_nodes counts the dummy row 0 (N+1). */
void pape_cuda(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges,
               long start_nodes[], long num_start_nodes, long first_thru_node,
               double *distances, long *predecessors);

/* replace tap/sssp_pape.h:36-53: single-source shortest paths over the
 * forward star (Va, Ea, Wa); num_nodes counts row 0.  prev[v] is the link
 * into v on a shortest path (-1 if none), dist[v] its label (DBL_MAX if
 * unreachable).  queue_next is accepted for signature compatibility and not
 * used.  Among equal-cost predecessors the lowest link index from a strictly
 * closer tail is chosen, so predecessors can differ from the reference on
 * ties; labels are identical. */
void sssp_pape(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges,
               long start_node, long first_thru_node, long prev[], double dist[],
               long queue_next[]);
void sssp_slf(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges,
              long start_node, long first_thru_node, long prev[], double dist[],
              long queue_next[]);
void sssp_slf_lll(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges,
                  long start_node, long first_thru_node, long prev[], double dist[],
                  long queue_next[]);
void sssp_pape_lll(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges,
                   long start_node, long first_thru_node, long prev[], double dist[],
                   long queue_next[]);
/* replaces tap/sssp_pape.h:55-56 (host walk of a predecessor array) */
void get_shortest_path(long pred[], long orig, long dest, long path[], long *pathlen);

/* replace tap/tap_functions.h:30-66.  Array operations run on the GPU. */
double bpr_cost_function(const link_data_t *link, double Q);
double linkcost_integral(const link_data_t *link, double Q);
double links_objective_function(const net_data_t *net, double volumes[]);
double link_directional_derivative(const net_data_t *net, double volume[],
                                   double delta_volume[], double lambda);
void adjlist_to_packed_arrays(link_data_t adjlist[], long num_nodes, long num_edges, long Va[],
                              long Ea[], double Wa[]);
int adjlist_entry_compar(const void *ent1, const void *ent2);
void update_link_costs(net_data_t *net, double link_volumes[], double link_costs[]);
double demand_sum(demand_data_t *const demands[], long num_zones);
double total_link_cost(const net_data_t *net, const double link_volumes[],
                       const double link_costs[]);
void print_flow(FILE *fp, const net_data_t *net, const double link_volumes[],
                const double link_costs[]);
double line_search(const net_data_t *net, double link_volumes[], double link_delta_volumes[]);
int apply_trip_modification(demand_data_t *demands[], trip_mod_t *mod, long num_zones);

/* replace tap/parsetapfiles.h:31-46 (TNTP text formats) */
int parse_net_file(FILE *fp, net_data_t *net);
int parse_trips_file(FILE *fp, demand_data_t **demands[], long *num_zones);
int parse_flows_file(FILE *flow_fp, link_flow_t **link_flows, long *num_links);
int parse_net_mod_file(FILE *fp, net_mod_t **mods, int *num_mods);
int link_data_compar(const void *ent1, const void *ent2);
int parse_trip_mod_file(FILE *fp, trip_mod_t **mods, int *num_mods);

/* ------------------------------------------------------------------------ */
/* Handle API                                                                */
/* ------------------------------------------------------------------------ */

/* status codes */
#define TAPGPU_OK 0
#define TAPGPU_ERR_ARG 1             /* invalid argument or input */
#define TAPGPU_ERR_CUDA 2            /* CUDA runtime error */
#define TAPGPU_ERR_NO_PATH 3         /* positive demand between disconnected zones */
#define TAPGPU_ERR_NO_CONVERGENCE 4  /* a bounded device loop hit its cap */
#define TAPGPU_ERR_ALLOC 5           /* device or host allocation failed */
#define TAPGPU_ERR_UNSUPPORTED 6     /* request outside the supported sizes */
#define TAPGPU_ERR_NO_DEVICE 7       /* no usable CUDA device */

/* precision of the shortest-path costs; gap, objective, line search and VHT
 * always accumulate in FP64 */
#define TAPGPU_FP64 0
#define TAPGPU_FP32_PATHS 1

typedef struct tapgpu_ctx tapgpu_ctx;

typedef struct tapgpu_network_s {
  int64_t num_nodes;       /* N: nodes are 1..N */
  int64_t num_zones;       /* Z: zones are nodes 1..Z */
  int64_t first_thru_node; /* nodes below this are only path ends */
  int64_t num_links;       /* M */
  const int64_t *init;     /* [M] tail node */
  const int64_t *term;     /* [M] head node */
  const double *capacity;  /* [M] (values <= 0 become the smallest positive one) */
  const double *fft;       /* [M] free-flow time, >= 0 */
  const double *alpha;     /* [M] BPR alpha (B), >= 0 */
  const double *beta;      /* [M] BPR power */
} tapgpu_network;

typedef struct tapgpu_demand_s {
  int64_t num_origins;     /* origins are zones 1..num_origins */
  const int64_t *od_ptr;   /* [num_origins+2]: origin o owns entries od_ptr[o]..od_ptr[o+1]-1 */
  const int64_t *od_dest;  /* destination zone of each entry */
  const double *od_demand; /* demand of each entry; entries <= 0 and o == dest are skipped */
} tapgpu_demand;

typedef struct tapgpu_options_s {
  int precision;         /* TAPGPU_FP64 or TAPGPU_FP32_PATHS */
  int device;            /* CUDA device ordinal */
  int sssp_block;        /* threads per shortest-path CTA (128..1024); 0 = tuned */
  int aon_block;         /* threads per loading CTA (256..1024); 0 = tuned */
  int iters_per_launch;  /* FW iterations per captured CUDA graph launch; 0 = auto */
  int use_graphs;        /* 1: replay iterations from a CUDA graph */
  int64_t chunk_tasks;   /* max (scenario, origin) shortest-path tasks per chunk; 0 = auto */
  int record_tape;       /* keep per-iteration flows and directions for the adjoint */
  int tape_capacity;     /* iterations kept on the tape */
  int global_scratch;    /* 1: per-CTA labels in global memory even when shared memory fits
                            (the queue kernels keep their bitmaps and ring in shared memory,
                            as they do whenever the labels do not fit); 2: all per-CTA
                            scratch in global memory */
  int sssp_variant;      /* 0 default (6 up to 4096 nodes and links, else 4, or its 32-bit
                            ring form above 65535 nodes); 1 bulk-synchronous
                            rounds; 2 asynchronous warp-owned frontier; 3 asynchronous near
                            set below a rising threshold; 4 as 3 with a FIFO ring of near
                            nodes (networks of at most 65535 nodes); 6 Bellman-Ford
                            sweeps over the edge list held in shared memory (the default
                            for networks of at most 4096 nodes and 4096 links) */
  double nf_delta;       /* threshold step of variants 3 and 4 in cost units; 0 = 16 x mean
                            link cost */
  int line_search;       /* 0: the reference's 2^-k rule; 1: exact root of the directional
                            derivative (differentiable step sizes, for the adjoint) */
  int tape_checkpoint;   /* with record_tape: flows kept every this many iterations and
                            recomputed in between by the adjoint (0 = sqrt(tape_capacity)) */
  int sssp_ctas_per_sm;  /* resident shortest-path CTAs per SM; 0 = as many as fit */
  int aon_ctas_per_sm;   /* resident loading CTAs per SM; 0 = as many as fit */
} tapgpu_options;

typedef struct tapgpu_result_s {
  int iterations;
  int error_bits;        /* device error bits (0 when clean) */
  double objective;      /* Beckmann objective of the last iteration (pre-step x) */
  double relgap;         /* relative gap of the last iteration */
  double total_cost;     /* VHT at the final flows */
  double avg_excess;
  double lambda_last;
} tapgpu_result;

/* per-iteration trace row (tap/tap_frankwolfe_pthread.c:751-753 fields) */
#define TAPGPU_TRACE_COLS 8 /* objective, relgap, avg_excess, vht, lambda, gap, iter, g0 */

void tapgpu_default_options(tapgpu_options *opt);
const char *tapgpu_status_string(int status);
/* message of the last failing call on this thread */
const char *tapgpu_last_message(void);

int tapgpu_create(const tapgpu_network *net, const tapgpu_demand *dem,
                  const tapgpu_options *opt, tapgpu_ctx **out);
void tapgpu_destroy(tapgpu_ctx *ctx);

/* Solve one network to max_iters and/or target_relgap (at least one > 0).
 * x0: optional warm-start volumes [M] (NULL: all-or-nothing at free flow). */
int tapgpu_solve(tapgpu_ctx *ctx, int max_iters, double target_relgap, const double *x0,
                 tapgpu_result *res);
/* The same solve in steps: begin sets up the state and the first
 * all-or-nothing; each advance runs up to max_new_iters more iterations and
 * reports whether the stopping rule holds. */
int tapgpu_solve_begin(tapgpu_ctx *ctx, int max_iters, double target_relgap, const double *x0);
int tapgpu_solve_advance(tapgpu_ctx *ctx, int max_new_iters, int *done, tapgpu_result *res);
/* volume and cost [M] of scenario s (0 for tapgpu_solve) */
int tapgpu_get_link_flows(tapgpu_ctx *ctx, int scenario, double *volume, double *cost);
/* volume and cost [count][M] of scenarios first .. first+count-1 in one call
 * (either may be NULL).  No counterpart in the reference, whose scenario farm
 * writes one flows file per solve; batched scenarios read back here at once. */
int tapgpu_get_link_flows_batch(tapgpu_ctx *ctx, int first, int count, double *volume,
                                double *cost);
/* per-iteration rows of scenario s: rows[i*TAPGPU_TRACE_COLS + c] */
int tapgpu_get_trace(tapgpu_ctx *ctx, int scenario, double *rows, int max_rows, int *nrows);
/* replace the base capacities [M] */
int tapgpu_set_capacity(tapgpu_ctx *ctx, const double *capacity);

/* Batched upgrade scenarios: scenario s replaces the capacity of links
 * scen_links[scen_ptr[s] .. scen_ptr[s+1]-1] by scen_cap[...].  All scenarios
 * share topology and demand and are solved together on the device.
 * x0: optional warm-start volumes [M] applied to every scenario.
 * results: [num_scen]. */
int tapgpu_solve_scenarios(tapgpu_ctx *ctx, int num_scen, const int64_t *scen_ptr,
                           const int64_t *scen_links, const double *scen_cap, int max_iters,
                           double target_relgap, const double *x0, tapgpu_result *results);

/* Shortest paths at link costs `weights` [M] from `sources` (node ids):
 * dist [num_sources][N+1] (DBL_MAX unreachable) and pred [num_sources][N+1]
 * link indices (-1 none).  Either output may be NULL. */
int tapgpu_sssp(tapgpu_ctx *ctx, const double *weights, const int64_t *sources,
                int64_t num_sources, double *dist, int64_t *pred);

/* All-or-nothing volumes [M] at link costs `weights` [M]. */
int tapgpu_aon(tapgpu_ctx *ctx, const double *weights, double *volume);

/* Device stream the context launches on (a cudaStream_t). */
void *tapgpu_stream(tapgpu_ctx *ctx);

/* Time one FW iteration kernel by kernel with CUDA events on the context's
 * stream, averaged over `reps` iterations of the current solve state:
 * ms[0] shortest paths, ms[1] loading, ms[2] line search, ms[3] step,
 * ms[4] whole iteration. */
int tapgpu_profile_iteration(tapgpu_ctx *ctx, int reps, float *ms);

/* Run `iters` further FW iterations of every scenario of the last solve
 * (ignoring the stopping rule), without host synchronisation in between
 * unless kernel timing is on. */
int tapgpu_run_iterations(tapgpu_ctx *ctx, int iters);

/* Kernel timing: with `on`, CUDA events are recorded around every launch of
 * the iteration loop (as event nodes inside the captured graphs) and their
 * durations accumulated; turning it on or off resets the totals.
 * tapgpu_get_timing returns total ms and launch counts per kernel group
 * [shortest paths, loading, line search, step] and the number of kernels
 * the solver launched since the reset. */
int tapgpu_set_timing(tapgpu_ctx *ctx, int on);
int tapgpu_get_timing(tapgpu_ctx *ctx, double *ms, int64_t *counts, int64_t *kernel_launches);
/* Reverse-mode derivative of the final VHT of scenario s with respect to the
 * link capacities, through every iteration of its last solve (no counterpart
 * in the reference).  Needs a context created with record_tape and
 * tape_capacity >= the iterations run.  The all-or-nothing loads are held
 * fixed (they are piecewise constant in the capacities); with
 * line_search = 1 the step sizes are differentiated by the implicit-function
 * rule, with the reference's 2^-k rule they are held fixed.  grad: [M] in the
 * caller's link order; vht (optional): the VHT the gradient belongs to. */
int tapgpu_adjoint_vht(tapgpu_ctx *ctx, int scenario, double *grad, double *vht);
/* One iteration of the recorded tape: direction d_k [M], step lambda_k, and
 * the flows x_k [M] when k is a checkpoint (k % tape_checkpoint == 0). */
int tapgpu_get_tape(tapgpu_ctx *ctx, int scenario, int iteration, double *x_checkpoint,
                    double *direction, double *lambda);

/* Demand scenarios (trip modifications as a batched scenario axis): from the
 * next tapgpu_solve_scenarios call with num_scen scenarios on, scenario s
 * loads demand[s * nnz + i] for OD entry i, where the entries are those of
 * the demand given to tapgpu_create in its order (origins 1..Z, each
 * origin's destinations as listed) and nnz their count.  Only entries with
 * positive base demand may be positive (a multiplier of the base, as
 * tap/tap_functions.c:521-598 applies them); zero removes a pair.  The
 * fixed-point scale of all demand is lowered if a scenario's total needs
 * it.  num_scen 0 or demand NULL returns to the one base demand; single
 * solves (tapgpu_solve) always use the base demand. */
int tapgpu_set_scenario_demand(tapgpu_ctx *ctx, int num_scen, const double *demand);

/* Link-record scenarios: the batched form of the ADD and CHANGE records of a
 * net-mods file, which the reference's scenario farm applies to one network
 * copy per scenario before solving it alone (tap/tap_mpi_main.c:201-240,
 * 678-753).  The context's network is the union of every scenario's links
 * (the base links and each added link once).  From the next
 * tapgpu_solve_scenarios call with num_scen scenarios on, scenario s uses
 * free-flow time edit_fft[i], BPR alpha edit_alpha[i] and power
 * edit_beta[i] on link edit_links[i] for i in edit_ptr[s] .. edit_ptr[s+1]-1
 * (the base values elsewhere; capacities come from that call's capacity
 * edits), and does not have links absent_links[absent_ptr[s] ..
 * absent_ptr[s+1]-1] at all: they carry no flow, are never on a path and are
 * left out of its zero-capacity fix-up.  A warm start gives added links zero
 * flow, as tap/tap_frankwolfe_pthread.c:564-597 inserts them.  num_scen 0
 * returns to the one base network; single solves (tapgpu_solve) always use
 * it. */
int tapgpu_set_scenario_links(tapgpu_ctx *ctx, int num_scen, const int64_t *edit_ptr,
                              const int64_t *edit_links, const double *edit_fft,
                              const double *edit_alpha, const double *edit_beta,
                              const int64_t *absent_ptr, const int64_t *absent_links);

/* Shortest-path work counters gathered while timing is on (out has 6
 * entries): out[0] label correction rounds or near-far phases, out[1]
 * (scenario, origin) tasks, out[2] node expansions, and for the near-far
 * kernels out[3] idle polls of warps that found no near work, out[4] warp
 * batches of up to 32 expansions and out[5] (queue variant) nodes claimed by
 * the bitmap word scan instead of the ring. */
int tapgpu_get_path_stats(tapgpu_ctx *ctx, int64_t *out);

/* No counterpart in the reference.  All-origins FP64 shortest-path labels for
 * callers that cannot let a library allocate device memory (their own pool
 * owns the HBM, or a cudaMalloc/cudaFree and the device synchronisation it
 * can cause is not acceptable in their loop).  Every argument is device
 * memory owned by the caller: the forward star row_ptr[num_nodes1+1] /
 * head[num_links] (num_nodes1 counts node 0), link costs weight[num_links]
 * (>= 0), sources[num_sources], and the output dist[num_sources][num_nodes1]
 * (+inf where unreachable).  Nodes below first_thru_node are only expanded as
 * sources.  The inputs are checked on the device before use (row_ptr
 * non-decreasing within 0..num_links, heads and sources in 0..num_nodes1-1,
 * weights >= 0); a failed check returns TAPGPU_ERR_ARG and leaves dist
 * untouched.  The only other memory used is a fixed 32 MiB array inside the
 * library (a 256-byte control block plus per-CTA label slices of
 * 8*num_nodes1 + num_nodes1/4 bytes, rounded up to 16): num_nodes1 above
 * 4,067,172 is rejected with TAPGPU_ERR_UNSUPPORTED before any CUDA call.
 * Each call looks up the array's device address with the current device;
 * the first call on a device also loads the library's device code there, so
 * make it before any stream capture.  All calls share the array, so calls
 * that overlap on the GPU (other streams, other host threads) race;
 * serialise them.  Runs on `stream` (a cudaStream_t, NULL for the default
 * stream) and returns after it finishes. */
int tapgpu_sssp_labels_noalloc(int32_t num_nodes1, int32_t num_links, int32_t first_thru_node,
                               const int32_t *row_ptr, const int32_t *head, const double *weight,
                               const int32_t *sources, int32_t num_sources, double *dist,
                               void *stream);

#ifdef __cplusplus
}
#endif
#endif /* TAP_GPU_H */
