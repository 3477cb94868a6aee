// solver.cuh - host-side solver context behind the tapgpu_* C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "fw_kernels.cuh"
#include "tap_gpu.h"

namespace tapgpu {

void set_message(const std::string& m);

// device allocation owned by a context
struct DevMem {
  void* p = nullptr;
  size_t bytes = 0;
};

struct Ctx {
  // sizes (internal link order: sorted by (init, term))
  int N = 0, n1 = 0, M = 0, Z = 0, F = 0;
  bool fp64 = true;
  int device = 0, num_sms = 0;
  tapgpu_options opt{};
  std::vector<int64_t> perm;  // internal link k -> caller's link index
  std::vector<int> h_tail, h_head;
  std::vector<double> h_cap, h_fft, h_alpha, h_beta;
  // base capacities on the device for the scenario rows, and the links in
  // order of increasing base capacity (both redone after tapgpu_set_capacity)
  double* base_cap = nullptr;
  std::vector<int> h_cap_order;
  bool base_dirty = true;
  // per-call scenario edits on the device (grown as needed)
  int* ed_ptr = nullptr;
  int* ed_link = nullptr;
  double* ed_val = nullptr;
  double* ed_min = nullptr;
  int64_t ed_scen_cap = 0, ed_cap = 0;

  // device topology and link parameters
  int *row_ptr = nullptr, *head = nullptr, *tail = nullptr, *in_ptr = nullptr, *in_link = nullptr;
  int* in_head = nullptr;  // head node of each reverse-star slot
  int* out_deg = nullptr;  // out-degree of each node
  int* ell_pos = nullptr;  // slot of each link among its tail's first four (-1: beyond)
  unsigned* e4x = nullptr;  // first word of each link's padded record (head | tail degree << 16)
  std::vector<unsigned> h_e4x;
  bool deg16 = false;       // node ids and out-degrees fit 16 bits (16-bit queue ring)
  std::vector<int> h_ell_pos;
  // padded reverse records of the loading kernel's per-node predecessor scan
  // (FP32 paths, nodes and links fitting 16 bits)
  bool rev4 = false;
  int* r4_pos = nullptr;    // slot of each link among its head's first four in-links (-1: beyond)
  unsigned* r4x = nullptr;  // first word of each link's padded reverse record (link << 16 | tail)
  unsigned* r4_more = nullptr;  // bit v: node v has more than four in-links
  double *fft = nullptr, *alpha = nullptr, *beta = nullptr;
  unsigned char* ipow = nullptr;

  // demand
  int *od_ptr = nullptr, *od_dest = nullptr;
  long long* od_q = nullptr;
  double* od_dem = nullptr;
  int* sources = nullptr;
  double inv_scale = 1.0, total_demand = 0.0;
  int scale_bits = 0;
  // demand scenarios (trip modifications): their own OD demand per scenario
  std::vector<double> h_od_dem;  // base demand in device entry order
  long long nnz = 0;
  long long* sc_od_q = nullptr;  // [dem_scen][nnz] fixed point
  double* sc_total = nullptr;    // [dem_scen] demand totals
  int dem_scen = 0;              // scenarios with their own demand (0: none set)
  bool use_dem_scen = false;     // the current batched solve uses them
  // link-record scenarios (ADD / CHANGE records): per-scenario parameter rows
  // [link_scen][M] and a bitmask [link_scen][absent_words] of the links a
  // scenario's network does not have
  double *sc_fft = nullptr, *sc_alpha = nullptr, *sc_beta = nullptr;
  unsigned char* sc_ipow = nullptr;
  unsigned* sc_absent = nullptr;
  std::vector<unsigned> h_absent;
  int absent_words = 0;
  int link_scen = 0;             // scenarios with their own link records (0: none set)
  bool use_link_scen = false;    // the current batched solve uses them

  // per-scenario state (capacity for S_cap scenarios)
  int S_cap = 0;
  double *cap = nullptr, *x = nullptr, *t = nullptr, *d = nullptr, *dtdx = nullptr;
  unsigned long long* yfx = nullptr;
  uint2* e32 = nullptr;  // packed {head, f32 weight} per scenario and link
  uint2* r32 = nullptr;  // packed {tail, f32 weight} per scenario, reverse-star order
  uint2* e4 = nullptr;   // per scenario, the first four records of each node (padded)
  uint2* r4 = nullptr;   // per scenario, the first four in-link records of each node (padded)
  uint4* r4d = nullptr;  // the same for FP64 paths: {link, tail, f64 weight}
  bool aon_c64 = false;  // FP64 loading in the compact layout (predecessor words in the label slot)
  int* rpos = nullptr;   // reverse-star slot of each link
  std::vector<int> h_rpos;
  double* w64 = nullptr;
  ScenState* state = nullptr;
  double* partials = nullptr;
  unsigned* arrive = nullptr;
  double* trace = nullptr;
  int trace_cap = 0;
  int* scen_list = nullptr;
  std::vector<int> h_scen_list;
  double *x_hist = nullptr, *d_hist = nullptr, *lam_hist = nullptr;
  int hist_cap = 0;
  int ckpt_every = 1;
  int ls_mode = kLsReference;
  // adjoint work buffers (allocated on first use)
  double *adj_xbar = nullptr, *adj_cbar = nullptr, *adj_seg = nullptr, *adj_part = nullptr;
  double* adj_scal = nullptr;
  unsigned* adj_arrive = nullptr;

  // scratch
  void* dist = nullptr;
  int64_t dist_tasks = 0;  // tasks the dist buffer holds
  void* path_scratch = nullptr;
  size_t path_scratch_bytes = 0;
  int* counters = nullptr;  // [2]
  int* err = nullptr;       // [1]
  int* err_info = nullptr;  // [2]
  int* pred_buf = nullptr;  // [dist_tasks][n1] for the shortest-path API
  unsigned long long* path_stats = nullptr;  // [8] rounds, tasks, expansions, idle polls, batches
  // buffers of the one-shot API (weights in both precisions, loaded volumes)
  uint2* api_e32 = nullptr;
  uint2* api_e4 = nullptr;
  uint2* api_r32 = nullptr;
  double* api_w64 = nullptr;
  unsigned long long* api_yfx = nullptr;

  cudaStream_t stream = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int g_iters = 0, g_nscen = -1;
  bool g_dem = false, g_links = false;
  int solve_max_iters = 0;
  int last_nscen = 1;  // scenarios of the last solve (for run_iterations)

  // kernel timing: event pairs recorded around launches (also inside graphs)
  struct Timed {
    int kind;  // 0 shortest paths, 1 loading, 2 line search, 3 step
    cudaEvent_t a, b;
  };
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<Timed> timed;       // launches of the current graph (or direct enqueue)
  double kt_ms[4] = {0, 0, 0, 0};
  long long kt_n[4] = {0, 0, 0, 0};
  long long launches = 0;         // kernels launched by the solver
  long long g_kernels = 0;        // kernels in the current graph
  long long pending_kernels = 0;  // kernels enqueued directly since the last sync
  bool measuring = false;         // marks enabled for the path kernels of an iteration
  cudaEvent_t next_event();
  int mark(int kind, bool begin);
  int collect_timing();
  void count_launches(long long n);

  // launch shapes
  int sssp_block = 256, aon_block = 512, link_grid = 0;
  // line-search passes and step: block size and blocks per scenario
  int ls_block = 256, ls_link_grid = 0;
  int sssp_variant = kSsspAsync;
  double nf_delta = 1.0;      // near-far threshold step for the solver's costs
  double api_nf_delta = 1.0;  // the same for the weights of the one-shot API
  bool sssp_smem = true, aon_smem = true;
  int sssp_grid = 0, aon_grid = 0;
  // line-search blocks per scenario: about 16 blocks per SM over the whole
  // batch, so that a batch's threads each sum many links and the 16-value
  // block reductions stay a small part of the FP64 work
  int ls_grid(int nscen) const {
    const int want = (16 * num_sms + nscen - 1) / (nscen > 0 ? nscen : 1);
    return want < 1 ? 1 : (want > ls_link_grid ? ls_link_grid : want);
  }

  std::vector<DevMem> owned;

  ~Ctx();
  int alloc(void** p, size_t bytes);
  template <class T>
  int alloc_n(T** p, size_t n) {
    return alloc(reinterpret_cast<void**>(p), n * sizeof(T));
  }
  int ensure_scenarios(int S);
  int plan_launches();

  Graph graph() const;
  LinkParams link_params() const;
  // the parameters of one scenario as a single shared row
  LinkParams link_params_of(int scen) const;
  bool absent_in(int scen, int k) const {
    return use_link_scen && !h_absent.empty() &&
           ((h_absent[static_cast<size_t>(scen) * absent_words + (k >> 5)] >> (k & 31)) & 1u);
  }
  Demand demand() const;
  PathArgs path_args(int nscen_slots) const;
  LinkArgs link_args(int nscen) const;

  // enqueue helpers (stream ordered, capturable)
  int enqueue_paths(int nscen, bool load, const uint2* e32p, const uint2* r32p, const double* w64p,
                    unsigned long long* ydst, bool use_state);
  int enqueue_iteration(int nscen);
  int enqueue_initial(int nscen, bool warm);
  int run_graph(int iters, int nscen);
  int sync_check();
  int read_states(int S, std::vector<ScenState>& out);
};

}  // namespace tapgpu

// the opaque handle of the C ABI
struct tapgpu_ctx {
  tapgpu::Ctx* c;
};
