// capi.cpp - drop-in entry points with the reference's names and contracts
// (stivalaa/traffic_assignment trunk/tap), implemented on the GPU solver:
//   tap_frankwolfe       tap/tap_frankwolfe_pthread.c:488-825
//   fw_assign            tap/tap_frankwolfe_cuda.cu:176-275
//   pape_cuda            tap/pape_cuda_host.cu:51-195
//   sssp_pape[_lll], sssp_slf[_lll]   tap/sssp_pape.c:120, 284, 534, 677
//   link-array numerics  tap/tap_functions.c:83-97, 143-152, 167-175, 408-417, 469-507
#include <pthread.h>
#include <signal.h>
#include <time.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "linkops.cuh"
#include "tap_gpu.h"

unsigned int num_cores = 0;
unsigned int num_threads = 1;
int using_fermi_architecture = 0;

namespace {

// ---------------------------------------------------------------------------
// signals: tap/tap_frankwolfe_pthread.c:154-254 (status / checkpoint / finish)
// ---------------------------------------------------------------------------
enum { kSigNone = 0, kSigWriteMsg = 1, kSigCheckpoint = 2, kSigTerminate = 3 };
volatile sig_atomic_t g_signal_status = kSigNone;
sigset_t g_sigset;
bool g_sig_started = false;

void* signal_thread(void*) {
  for (;;) {
    int sig = 0;
    if (sigwait(&g_sigset, &sig) != 0) {
      perror("ERROR: sigwait() in signal handler thread failed, signals not handled");
      return nullptr;
    }
    fprintf(stderr, "signal %d received...\n", sig);
    switch (sig) {
      case SIGUSR1: g_signal_status = kSigWriteMsg; break;
      case SIGUSR2: g_signal_status = kSigCheckpoint; break;
      case SIGHUP:
      case SIGINT:
      case SIGTERM:
      case SIGXCPU:
#ifdef SIGPWR
      case SIGPWR:
#endif
        g_signal_status = kSigTerminate;
        break;
      default: fprintf(stderr, "ERROR: unhandled signal %d\n", sig); break;
    }
  }
  return nullptr;
}

void start_signal_thread() {
  if (g_sig_started || getenv("TAPGPU_NO_SIGNALS")) return;
  sigemptyset(&g_sigset);
  sigaddset(&g_sigset, SIGUSR1);
  sigaddset(&g_sigset, SIGUSR2);
  sigaddset(&g_sigset, SIGHUP);
  sigaddset(&g_sigset, SIGINT);
  sigaddset(&g_sigset, SIGTERM);
  sigaddset(&g_sigset, SIGXCPU);
#ifdef SIGPWR
  sigaddset(&g_sigset, SIGPWR);
#endif
  if (pthread_sigmask(SIG_BLOCK, &g_sigset, nullptr) != 0) {
    perror("ERROR: pthread_sigmask() failed");
    fprintf(stderr, "WARNING: signals will not be handled");
    return;
  }
  pthread_t th;
  if (pthread_create(&th, nullptr, signal_thread, nullptr) != 0) {
    fprintf(stderr, "WARNING: signals will not be handled");
    return;
  }
  pthread_detach(th);
  g_sig_started = true;
}

[[noreturn]] void die(const char* where, int rc) {
  fprintf(stderr, "%s: %s (%s)\n", where, tapgpu_status_string(rc), tapgpu_last_message());
  exit(1);
}

int precision_from_env() {
  const char* p = getenv("TAPGPU_PRECISION");
  if (p && (strcmp(p, "fp32") == 0 || strcmp(p, "fp32path") == 0)) return TAPGPU_FP32_PATHS;
  return TAPGPU_FP64;
}

struct NetArrays {
  std::vector<int64_t> init, term;
  std::vector<double> cap, fft, alpha, beta;
  tapgpu_network net{};
  void build(const net_data_t* n) {
    const long m = n->num_links;
    init.resize(m);
    term.resize(m);
    cap.resize(m);
    fft.resize(m);
    alpha.resize(m);
    beta.resize(m);
    for (long k = 0; k < m; ++k) {
      const link_data_t& l = n->links[k];
      init[k] = l.init_node;
      term[k] = l.term_node;
      cap[k] = l.capacity;
      fft[k] = l.free_flow_time;
      alpha[k] = l.B;
      beta[k] = l.power;
    }
    net.num_nodes = n->num_nodes;
    net.num_zones = n->num_zones;
    net.first_thru_node = n->first_thru_node;
    net.num_links = m;
    net.init = init.data();
    net.term = term.data();
    net.capacity = cap.data();
    net.fft = fft.data();
    net.alpha = alpha.data();
    net.beta = beta.data();
  }
};

struct DemArrays {
  std::vector<int64_t> ptr, dest;
  std::vector<double> dem;
  tapgpu_demand d{};
  void build(demand_data_t* const* demands, long zones) {
    ptr.assign(zones + 2, 0);
    dest.clear();
    dem.clear();
    for (long o = 1; o <= zones; ++o) {
      if (demands[o])
        for (long i = 0; demands[o][i].dest != 0; ++i) {
          dest.push_back(demands[o][i].dest);
          dem.push_back(demands[o][i].demand);
        }
      ptr[o + 1] = static_cast<int64_t>(dest.size());
    }
    d.num_origins = zones;
    d.od_ptr = ptr.data();
    d.od_dest = dest.data();
    d.od_demand = dem.data();
  }
};

int link_flow_cmp(const void* a, const void* b) {
  const link_flow_t* x = static_cast<const link_flow_t*>(a);
  const link_flow_t* y = static_cast<const link_flow_t*>(b);
  if (x->init_node != y->init_node) return x->init_node < y->init_node ? -1 : 1;
  if (x->term_node != y->term_node) return x->term_node < y->term_node ? -1 : 1;
  return 0;
}

void print_iter_line(FILE* f, int it, const double* r, int ms, bool with_ms) {
  if (with_ms)
    fprintf(f,
            "iter = %d objective value = %.15f relative gap = %.15f average exccess cost = %.15f "
            "total cost = %.15f (%d ms)\n",
            it, r[0], r[1], r[2], r[3], ms);
  else
    fprintf(f,
            "iter = %d objective value = %.15f relative gap = %.15f average exccess cost = %.15f "
            "total cost = %.15f\n",
            it, r[0], r[1], r[2], r[3]);
}

double now_ms() {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

// ---------------------------------------------------------------------------
// cached contexts for the stateless drop-ins
// ---------------------------------------------------------------------------
struct GraphKey {
  const void* a = nullptr;
  const void* b = nullptr;
  long n = 0, m = 0, f = 0;
  uint64_t sum = 0;
  bool operator==(const GraphKey& o) const {
    return a == o.a && b == o.b && n == o.n && m == o.m && f == o.f && sum == o.sum;
  }
};

uint64_t mix(uint64_t h, uint64_t v) { return (h ^ v) * 0x100000001b3ull; }

struct CsrCache {
  GraphKey key;
  tapgpu_ctx* ctx = nullptr;
};
CsrCache g_csr;

// context over a forward star (Va, Ea) with no demand
tapgpu_ctx* csr_context(const long Va[], const long Ea[], long num_nodes, long num_edges,
                        long first_thru) {
  GraphKey k;
  k.a = Va;
  k.b = Ea;
  k.n = num_nodes;
  k.m = num_edges;
  k.f = first_thru;
  uint64_t h = 0xcbf29ce484222325ull;
  for (long v = 0; v <= num_nodes; ++v) h = mix(h, static_cast<uint64_t>(Va[v]));
  for (long e = 0; e < num_edges; ++e) h = mix(h, static_cast<uint64_t>(Ea[e]));
  k.sum = h;
  if (g_csr.ctx && g_csr.key == k) return g_csr.ctx;
  if (g_csr.ctx) tapgpu_destroy(g_csr.ctx);
  g_csr.ctx = nullptr;
  std::vector<int64_t> init(num_edges), term(num_edges);
  for (long v = 0; v < num_nodes; ++v)
    for (long e = Va[v]; e < Va[v + 1]; ++e) init[e] = v;
  for (long e = 0; e < num_edges; ++e) term[e] = Ea[e];
  std::vector<double> ones(num_edges, 1.0), zeros(num_edges, 0.0);
  tapgpu_network net{};
  net.num_nodes = num_nodes - 1;
  net.num_zones = 0;
  net.first_thru_node = first_thru;
  net.num_links = num_edges;
  net.init = init.data();
  net.term = term.data();
  net.capacity = ones.data();
  net.fft = zeros.data();
  net.alpha = zeros.data();
  net.beta = ones.data();
  tapgpu_options opt;
  tapgpu_default_options(&opt);
  opt.precision = TAPGPU_FP64;
  int rc = tapgpu_create(&net, nullptr, &opt, &g_csr.ctx);
  if (rc != TAPGPU_OK) die("pape_cuda", rc);
  g_csr.key = k;
  return g_csr.ctx;
}

void sssp_one(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges,
              long start_node, long first_thru_node, long prev[], double dist[]) {
  tapgpu_ctx* ctx = csr_context(Va, Ea, num_nodes, num_edges, first_thru_node);
  int64_t src = start_node;
  std::vector<double> d(num_nodes);
  std::vector<int64_t> p(num_nodes);
  int rc = tapgpu_sssp(ctx, Wa, &src, 1, d.data(), p.data());
  if (rc != TAPGPU_OK) die("sssp", rc);
  for (long v = 0; v < num_nodes; ++v) {
    dist[v] = d[v];
    prev[v] = static_cast<long>(p[v]);
  }
}

struct NetCache {
  const void* links = nullptr;
  const void* demands = nullptr;
  long m = 0;
  tapgpu_ctx* ctx = nullptr;
};
NetCache g_net;

tapgpu::LinkOps& linkops() {
  static tapgpu::LinkOps ops;
  return ops;
}

void load_linkops(const net_data_t* net) {
  const long m = net->num_links;
  std::vector<double> fft(m), a(m), b(m), c(m);
  for (long k = 0; k < m; ++k) {
    fft[k] = net->links[k].free_flow_time;
    a[k] = net->links[k].B;
    b[k] = net->links[k].power;
    c[k] = net->links[k].capacity;
  }
  if (linkops().upload(static_cast<int>(m), fft.data(), a.data(), b.data(), c.data()) != 0) {
    fprintf(stderr, "tapgpu: link upload failed\n");
    exit(1);
  }
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// tap_frankwolfe (tap/tap_frankwolfe_pthread.h:30-38)
// ---------------------------------------------------------------------------
int tap_frankwolfe(net_data_t* net, demand_data_t** demands, int warm_start_mode,
                   FILE* flows_input_fp, int target_iterations, double target_relgap,
                   FILE* flow_fp, double* total_cost_at_end, double* objvalue_at_end,
                   int* iterations_at_end, double* relgap_at_end, int time_each_iteration) {
  start_signal_thread();
  const long m = net->num_links;
  std::vector<double> x0;
  std::vector<double> file_cost;
  if (warm_start_mode) {
    link_flow_t* lf = nullptr;
    long nf = 0;
    if (!flows_input_fp || parse_flows_file(flows_input_fp, &lf, &nf) != 0) {
      fprintf(stderr, "error parsing flows input file\n");
      return 1;
    }
    fclose(flows_input_fp);
    qsort(lf, nf, sizeof(link_flow_t), link_flow_cmp);
    if (nf > m) {
      fprintf(stderr, "error: %ld links in net file but %ld in flows input file\n", m, nf);
      free(lf);
      return 1;
    }
    // links added since the flows were written start at zero flow
    // (tap/tap_frankwolfe_pthread.c:564-597)
    x0.assign(m, 0.0);
    file_cost.assign(m, 0.0);
    long j = 0;
    for (long k = 0; k < m; ++k) {
      if (j < nf && lf[j].init_node == net->links[k].init_node &&
          lf[j].term_node == net->links[k].term_node) {
        x0[k] = lf[j].volume;
        file_cost[k] = lf[j].cost;
        ++j;
      }
    }
    free(lf);
  }

  // tap/tap_frankwolfe_pthread.c:654-669
  double min_cap = DBL_MAX;
  for (long k = 0; k < m; ++k)
    if (net->links[k].capacity > 0.0 && net->links[k].capacity < min_cap)
      min_cap = net->links[k].capacity;
  for (long k = 0; k < m; ++k)
    if (net->links[k].capacity <= 0.0) {
      fprintf(stderr,
              "warning: zero capacity for link from %ld to %ld, set to min nonzero capacity %f\n",
              net->links[k].init_node, net->links[k].term_node, min_cap);
      net->links[k].capacity = min_cap;
    }

  NetArrays na;
  na.build(net);
  DemArrays da;
  da.build(demands, net->num_zones);
  tapgpu_options opt;
  tapgpu_default_options(&opt);
  opt.precision = precision_from_env();
  tapgpu_ctx* ctx = nullptr;
  int rc = tapgpu_create(&na.net, &da.d, &opt, &ctx);
  if (rc != TAPGPU_OK) {
    fprintf(stderr, "tap_frankwolfe: %s (%s)\n", tapgpu_status_string(rc), tapgpu_last_message());
    return 1;
  }
  if (warm_start_mode) {
    // the costs recomputed from the flows should match the file's
    std::vector<double> t(m);
    load_linkops(net);
    if (linkops().costs(x0.data(), t.data()) == 0)
      for (long k = 0; k < m; ++k)
        if (std::fabs(t[k] - file_cost[k]) > 1e-08)
          fprintf(stderr, "warning: mismatched costs (delta = %g) on link %ld from %ld to %ld\n",
                  std::fabs(t[k] - file_cost[k]), k, net->links[k].init_node,
                  net->links[k].term_node);
  }

  int max_iters = target_iterations > 0 ? target_iterations : 0;
  double target = target_relgap > 0 ? target_relgap : 0.0;
  rc = tapgpu_solve_begin(ctx, max_iters, target, warm_start_mode ? x0.data() : nullptr);
  if (rc == TAPGPU_ERR_NO_PATH) {
    fprintf(stderr, "%s\n", tapgpu_last_message());
    exit(1);
  }
  if (rc != TAPGPU_OK) {
    fprintf(stderr, "tap_frankwolfe: %s (%s)\n", tapgpu_status_string(rc), tapgpu_last_message());
    tapgpu_destroy(ctx);
    return 1;
  }
  const int per = time_each_iteration ? 1 : 8;
  tapgpu_result res{};
  std::vector<double> rows;
  std::vector<double> vol(m), cost(m);
  int printed = 0;
  int done = 0;
  bool finished = false;
  while (!done && !finished) {
    const double t0 = now_ms();
    rc = tapgpu_solve_advance(ctx, per, &done, &res);
    if (rc == TAPGPU_ERR_NO_PATH) {
      fprintf(stderr, "%s\n", tapgpu_last_message());
      exit(1);
    }
    if (rc != TAPGPU_OK) {
      fprintf(stderr, "tap_frankwolfe: %s (%s)\n", tapgpu_status_string(rc), tapgpu_last_message());
      tapgpu_destroy(ctx);
      return 1;
    }
    const double dt = now_ms() - t0;
    rows.resize(static_cast<size_t>(res.iterations) * TAPGPU_TRACE_COLS);
    int n = 0;
    if (res.iterations > 0)
      tapgpu_get_trace(ctx, 0, rows.data(), res.iterations, &n);
    if (time_each_iteration) {
      const int fresh = std::max(1, n - printed);
      for (int i = printed; i < n; ++i)
        print_iter_line(stderr, i + 1, &rows[static_cast<size_t>(i) * TAPGPU_TRACE_COLS],
                        static_cast<int>(dt / fresh), true);
    }
    printed = n;
    const double* last = n > 0 ? &rows[static_cast<size_t>(n - 1) * TAPGPU_TRACE_COLS] : nullptr;
    switch (g_signal_status) {
      case kSigNone: break;
      case kSigWriteMsg:
        if (last) print_iter_line(stderr, n, last, 0, false);
        break;
      case kSigCheckpoint: {
        if (last) print_iter_line(stderr, n, last, 0, false);
        fprintf(stderr, "checkpointing to flows output file...");
        time_t now = time(nullptr);
        tapgpu_get_link_flows(ctx, 0, vol.data(), cost.data());
        rewind(flow_fp);
        fprintf(flow_fp, "~ checkpoint written at %s\n", ctime(&now));
        fprintf(flow_fp, "~ iterations = %d objvalue = %.15f relgap = %.15f\n", n,
                last ? last[0] : 0.0, last ? last[1] : DBL_MAX);
        fprintf(flow_fp, "~ totalcost = %.15f\n", res.total_cost);
        print_flow(flow_fp, net, vol.data(), cost.data());
        fflush(flow_fp);
        fprintf(stderr, "done\n");
        break;
      }
      case kSigTerminate: finished = true; break;
      default: fprintf(stderr, "ERROR: unknown signal status %d\n", (int)g_signal_status); break;
    }
    g_signal_status = kSigNone;
  }
  tapgpu_get_link_flows(ctx, 0, vol.data(), cost.data());
  const double* last =
      printed > 0 ? &rows[static_cast<size_t>(printed - 1) * TAPGPU_TRACE_COLS] : nullptr;
  const double objective = last ? last[0] : 0.0;
  const double relgap = last ? last[1] : DBL_MAX;
  rewind(flow_fp);
  fprintf(flow_fp, "~ iterations = %d objvalue = %.15f relgap = %.15f\n", res.iterations,
          objective, relgap);
  fprintf(flow_fp, "~ totalcost = %.15f\n", res.total_cost);
  print_flow(flow_fp, net, vol.data(), cost.data());
  fflush(flow_fp);
  tapgpu_destroy(ctx);

  for (long i = 0; i < net->num_zones + 1; i++) free(demands[i]);
  free(demands);
  *total_cost_at_end = res.total_cost;
  *objvalue_at_end = objective;
  *iterations_at_end = res.iterations;
  *relgap_at_end = relgap;
  return 0;
}

// ---------------------------------------------------------------------------
// fw_assign (tap/tap_frankwolfe_cuda.h:26-29)
// ---------------------------------------------------------------------------
void fw_assign(net_data_t* net, demand_data_t* demands[], long Va[], long Ea[], double Wa[],
               double link_volumes[], double dist[], long predlink[]) {
  (void)Va;
  (void)Ea;
  if (!g_net.ctx || g_net.links != net->links || g_net.demands != demands ||
      g_net.m != net->num_links) {
    if (g_net.ctx) tapgpu_destroy(g_net.ctx);
    g_net.ctx = nullptr;
    NetArrays na;
    na.build(net);
    DemArrays da;
    da.build(demands, net->num_zones);
    tapgpu_options opt;
    tapgpu_default_options(&opt);
    opt.precision = TAPGPU_FP64;
    int rc = tapgpu_create(&na.net, &da.d, &opt, &g_net.ctx);
    if (rc != TAPGPU_OK) die("fw_assign", rc);
    g_net.links = net->links;
    g_net.demands = demands;
    g_net.m = net->num_links;
  }
  int rc = tapgpu_aon(g_net.ctx, Wa, link_volumes);
  if (rc == TAPGPU_ERR_NO_PATH) {
    fprintf(stderr, "%s\n", tapgpu_last_message());
    exit(1);
  }
  if (rc != TAPGPU_OK) die("fw_assign", rc);
  if (dist || predlink) {
    const long z = net->num_zones, n1 = net->num_nodes + 1;
    std::vector<int64_t> src(z);
    for (long s = 0; s < z; ++s) src[s] = s + 1;
    std::vector<double> d(static_cast<size_t>(z) * n1);
    std::vector<int64_t> p(static_cast<size_t>(z) * n1);
    rc = tapgpu_sssp(g_net.ctx, Wa, src.data(), z, d.data(), p.data());
    if (rc != TAPGPU_OK) die("fw_assign", rc);
    for (long s = 1; s <= z; ++s)
      for (long v = 0; v < n1; ++v) {
        const size_t i = static_cast<size_t>(s - 1) * n1 + v;
        if (dist) dist[v * z + s] = d[i];
        if (predlink) predlink[v * z + s] = static_cast<long>(p[i]);
      }
  }
}

// ---------------------------------------------------------------------------
// pape_cuda (tap/pape_cuda_host.h:15-19)
// ---------------------------------------------------------------------------
void pape_cuda(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges,
               long start_nodes[], long num_start_nodes, long first_thru_node,
               double* distances, long* predecessors) {
  tapgpu_ctx* ctx = csr_context(Va, Ea, num_nodes, num_edges, first_thru_node);
  std::vector<int64_t> src(start_nodes, start_nodes + num_start_nodes);
  std::vector<double> d(static_cast<size_t>(num_start_nodes) * num_nodes);
  std::vector<int64_t> p(static_cast<size_t>(num_start_nodes) * num_nodes);
  int rc = tapgpu_sssp(ctx, Wa, src.data(), num_start_nodes, d.data(), p.data());
  if (rc != TAPGPU_OK) die("pape_cuda", rc);
  for (long i = 0; i < num_start_nodes; ++i) {
    const long s = start_nodes[i];
    for (long v = 0; v < num_nodes; ++v) {
      const size_t j = static_cast<size_t>(i) * num_nodes + v;
      distances[v * num_start_nodes + s] = d[j];
      predecessors[v * num_start_nodes + s] = static_cast<long>(p[j]);
    }
  }
}

// ---------------------------------------------------------------------------
// single-source entry points (tap/sssp_pape.h:36-53)
// ---------------------------------------------------------------------------
void sssp_pape(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges, long start_node,
               long first_thru_node, long prev[], double dist[], long queue_next[]) {
  (void)queue_next;
  sssp_one(Va, Ea, Wa, num_nodes, num_edges, start_node, first_thru_node, prev, dist);
}
void sssp_pape_lll(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges,
                   long start_node, long first_thru_node, long prev[], double dist[],
                   long queue_next[]) {
  (void)queue_next;
  sssp_one(Va, Ea, Wa, num_nodes, num_edges, start_node, first_thru_node, prev, dist);
}
void sssp_slf(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges, long start_node,
              long first_thru_node, long prev[], double dist[], long queue_next[]) {
  (void)queue_next;
  sssp_one(Va, Ea, Wa, num_nodes, num_edges, start_node, first_thru_node, prev, dist);
}
void sssp_slf_lll(long Va[], long Ea[], double Wa[], long num_nodes, long num_edges,
                  long start_node, long first_thru_node, long prev[], double dist[],
                  long queue_next[]) {
  (void)queue_next;
  sssp_one(Va, Ea, Wa, num_nodes, num_edges, start_node, first_thru_node, prev, dist);
}

// ---------------------------------------------------------------------------
// link-array numerics (tap/tap_functions.h:30-66)
// ---------------------------------------------------------------------------
void update_link_costs(net_data_t* net, double link_volumes[], double link_costs[]) {
  load_linkops(net);
  if (linkops().costs(link_volumes, link_costs) != 0) {
    fprintf(stderr, "tapgpu: update_link_costs failed\n");
    exit(1);
  }
}

double links_objective_function(const net_data_t* net, double volumes[]) {
  load_linkops(net);
  double out = 0;
  if (linkops().set_xd(volumes, nullptr) != 0 || linkops().sums(1, nullptr, 1, &out) != 0) {
    fprintf(stderr, "tapgpu: links_objective_function failed\n");
    exit(1);
  }
  return out;
}

double link_directional_derivative(const net_data_t* net, double volume[], double delta_volume[],
                                   double lambda) {
  load_linkops(net);
  double out = 0;
  if (linkops().set_xd(volume, delta_volume) != 0 || linkops().sums(0, &lambda, 1, &out) != 0) {
    fprintf(stderr, "tapgpu: link_directional_derivative failed\n");
    exit(1);
  }
  return out;
}

double total_link_cost(const net_data_t* net, const double link_volumes[],
                       const double link_costs[]) {
  load_linkops(net);
  double out = 0;
  if (linkops().set_xd(link_volumes, link_costs) != 0 || linkops().sums(2, nullptr, 1, &out) != 0) {
    fprintf(stderr, "tapgpu: total_link_cost failed\n");
    exit(1);
  }
  return out;
}

// tap/tap_functions.c:469-507: 0 if g(0) >= 0, 1 if g(1) <= 0, else the
// largest 2^-k (k >= 1) with g(2^-k) <= 0 within 1000 halvings.  The
// candidates are evaluated in batches on the device.
double line_search(const net_data_t* net, double link_volumes[], double link_delta_volumes[]) {
  load_linkops(net);
  tapgpu::LinkOps& ops = linkops();
  if (ops.set_xd(link_volumes, link_delta_volumes) != 0) {
    fprintf(stderr, "tapgpu: line_search failed\n");
    exit(1);
  }
  double ends[2] = {0.0, 1.0}, g[32];
  if (ops.sums(0, ends, 2, g) != 0) {
    fprintf(stderr, "tapgpu: line_search failed\n");
    exit(1);
  }
  if (g[0] >= 0) return 0.0;
  if (g[1] <= 0) return 1.0;
  const int per = tapgpu::LinkOps::max_lambdas();
  double lams[32];
  for (int e0 = 1; e0 <= 1000; e0 += per) {
    const int nl = std::min(per, 1001 - e0);
    for (int j = 0; j < nl; ++j) lams[j] = std::ldexp(1.0, -(e0 + j));
    if (ops.sums(0, lams, nl, g) != 0) {
      fprintf(stderr, "tapgpu: line_search failed\n");
      exit(1);
    }
    for (int j = 0; j < nl; ++j)
      if (g[j] <= 0) return lams[j];
  }
  return 0.0;
}

}  // extern "C"
