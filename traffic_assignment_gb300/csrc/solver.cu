// solver.cu - host side of the GB300 Frank-Wolfe solver: builds the device
// graph, demand and per-scenario state, enqueues FW iterations (captured into
// CUDA graphs), and implements the tapgpu_* handle API of include/tap_gpu.h.
#include "solver.cuh"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <limits>
#include <numeric>

namespace tapgpu {

namespace {
thread_local std::string g_message;
}

void set_message(const std::string& m) { g_message = m; }

#define TG_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      ::tapgpu::set_message(std::string(#call) + ": " + cudaGetErrorString(e_));       \
      return TAPGPU_ERR_CUDA;                                                           \
    }                                                                                   \
  } while (0)

#define TG_TRY(call)        \
  do {                      \
    int r_ = (call);        \
    if (r_ != TAPGPU_OK) {  \
      return r_;            \
    }                       \
  } while (0)

Ctx::~Ctx() {
  if (gexec) cudaGraphExecDestroy(gexec);
  for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
  if (stream) cudaStreamDestroy(stream);
  for (auto& m : owned) cudaFree(m.p);
}

int Ctx::alloc(void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_message(std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes: " +
                cudaGetErrorString(e));
    return TAPGPU_ERR_ALLOC;
  }
  owned.push_back({q, bytes});
  *p = q;
  return TAPGPU_OK;
}

cudaEvent_t Ctx::next_event() {
  if (ev_used == ev_pool.size()) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    ev_pool.push_back(e);
  }
  return ev_pool[ev_used++];
}

// Record a timing event before (begin) or after a launch; inside a stream
// capture the record becomes an event node of the graph.
int Ctx::mark(int kind, bool begin) {
  if (!timing) return TAPGPU_OK;
  cudaEvent_t e = next_event();
  if (!e) return TAPGPU_ERR_CUDA;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  TG_CUDA(cudaStreamIsCapturing(stream, &cs));
  if (cs == cudaStreamCaptureStatusActive)
    TG_CUDA(cudaEventRecordWithFlags(e, stream, cudaEventRecordExternal));
  else
    TG_CUDA(cudaEventRecord(e, stream));
  if (begin)
    timed.push_back({kind, e, nullptr});
  else if (!timed.empty())
    timed.back().b = e;
  return TAPGPU_OK;
}

// Accumulate the durations of the marked launches (stream already synchronised).
int Ctx::collect_timing() {
  for (const Timed& t : timed) {
    float ms = 0.f;
    if (t.a && t.b && cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess) {
      kt_ms[t.kind] += ms;
      kt_n[t.kind] += 1;
    }
  }
  cudaGetLastError();
  return TAPGPU_OK;
}

static void free_owned(Ctx* c, void* p) {
  if (!p) return;
  for (size_t i = 0; i < c->owned.size(); ++i) {
    if (c->owned[i].p == p) {
      cudaFree(p);
      c->owned.erase(c->owned.begin() + static_cast<long>(i));
      return;
    }
  }
}

Graph Ctx::graph() const {
  Graph g;
  g.n1 = n1;
  g.m = M;
  g.first_thru = F;
  g.row_ptr = row_ptr;
  g.head = head;
  g.tail = tail;
  g.in_ptr = in_ptr;
  g.in_link = in_link;
  g.in_head = in_head;
  g.out_deg = out_deg;
  return g;
}

LinkParams Ctx::link_params() const {
  LinkParams lp;
  if (use_link_scen && sc_fft) {
    lp.fft = sc_fft;
    lp.alpha = sc_alpha;
    lp.beta = sc_beta;
    lp.ipow = sc_ipow;
    lp.stride = M;
    return lp;
  }
  lp.fft = fft;
  lp.alpha = alpha;
  lp.beta = beta;
  lp.ipow = ipow;
  lp.stride = 0;
  return lp;
}

LinkParams Ctx::link_params_of(int scen) const {
  LinkParams lp = link_params();
  const size_t off = static_cast<size_t>(scen) * static_cast<size_t>(lp.stride);
  lp.fft += off;
  lp.alpha += off;
  lp.beta += off;
  lp.ipow += off;
  lp.stride = 0;
  return lp;
}

Demand Ctx::demand() const {
  Demand dm;
  dm.od_ptr = od_ptr;
  dm.od_dest = od_dest;
  dm.od_q = use_dem_scen ? sc_od_q : od_q;
  dm.q_stride = use_dem_scen ? nnz : 0;
  dm.od_dem = od_dem;
  dm.inv_scale = inv_scale;
  dm.total = total_demand;
  return dm;
}

PathArgs Ctx::path_args(int nscen_slots) const {
  PathArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = graph();
  a.sources = sources;
  a.num_sources = Z;
  a.scen_list = scen_list;
  a.state = state;
  a.task_begin = 0;
  a.task_end = nscen_slots * Z;
  a.dist = dist;
  a.counter = counters;
  a.err = err;
  a.err_info = err_info;
  a.max_rounds = n1 + 2;
  a.dem = demand();
  a.y_fx = yfx;
  a.do_load = 1;
  a.scratch = path_scratch;
  a.scratch_stride = 0;
  a.all_global = opt.global_scratch == 2;
  a.stats = timing ? path_stats : nullptr;
  a.nf_delta = nf_delta;
  a.e4 = (!fp64 && (sssp_variant == kSsspNearFarQueue || sssp_variant == kSsspNearFarQueueWide))
             ? e4
             : nullptr;
  a.r4 = rev4 ? r4 : nullptr;
  a.r4d = fp64 ? r4d : nullptr;
  a.aon_c64 = aon_c64 ? 1 : 0;
  a.r4_more = r4_more;
  return a;
}

LinkArgs Ctx::link_args(int nscen) const {
  LinkArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = M;
  a.num_scen = nscen;
  a.scen_list = scen_list;
  a.lp = link_params();
  a.cap = cap;
  a.x = x;
  a.t = t;
  a.d = d;
  a.y_fx = yfx;
  a.e32 = fp64 ? nullptr : e32;
  a.r32 = fp64 ? nullptr : r32;
  a.e4 = fp64 ? nullptr : e4;
  a.ell_pos = ell_pos;
  a.e4x = e4x;
  a.r4 = rev4 && !fp64 ? r4 : nullptr;
  a.r4d = fp64 ? r4d : nullptr;
  a.r4_pos = r4_pos;
  a.r4x = r4x;
  a.n1 = n1;
  a.head = head;
  a.tail = tail;
  a.rpos = rpos;
  a.w64 = fp64 ? w64 : nullptr;
  a.dtdx = dtdx;
  a.partials = partials;
  a.arrive = arrive;
  a.state = state;
  a.trace = trace;
  a.trace_cap = trace_cap;
  a.inv_scale = inv_scale;
  a.total_demand = total_demand;
  a.total_demand_s = use_dem_scen ? sc_total : nullptr;
  a.err = err;
  a.x_hist = x_hist;
  a.d_hist = d_hist;
  a.lam_hist = lam_hist;
  a.hist_cap = hist_cap;
  a.ckpt_every = ckpt_every;
  a.ls_mode = ls_mode;
  a.ls_ratio = fp64 ? 0 : 1;
  a.absent = use_link_scen ? sc_absent : nullptr;
  a.absent_words = absent_words;
  return a;
}

int Ctx::ensure_scenarios(int S) {
  if (S <= S_cap) return TAPGPU_OK;
  // release the old per-scenario arrays
  void* olds[] = {cap, x, t, d, dtdx, yfx, e32, r32, e4, r4, r4d, w64, state, partials, arrive,
                  trace, scen_list, x_hist, d_hist, lam_hist};
  for (void* p : olds) free_owned(this, p);
  cap = x = t = d = dtdx = nullptr;
  yfx = nullptr;
  e32 = nullptr;
  e4 = nullptr;
  r4 = nullptr;
  r4d = nullptr;
  r32 = nullptr;
  w64 = nullptr;
  state = nullptr;
  partials = nullptr;
  arrive = nullptr;
  trace = nullptr;
  scen_list = nullptr;
  x_hist = d_hist = lam_hist = nullptr;
  const size_t sm = static_cast<size_t>(S) * M;
  TG_TRY(alloc_n(&cap, sm));
  TG_TRY(alloc_n(&x, sm));
  TG_TRY(alloc_n(&t, sm));
  TG_TRY(alloc_n(&d, sm));
  TG_TRY(alloc_n(&yfx, sm));
  if (fp64) {
    TG_TRY(alloc_n(&w64, sm));
    // slots beyond a node's in-links keep an infinite weight: never tight
    const size_t s4 = static_cast<size_t>(S) * n1 * 4;
    TG_TRY(alloc_n(&r4d, s4));
    TG_CUDA(launch_fill_records4(r4d, s4, make_uint4(0u, 0u, 0u, 0x7ff00000u), 2 * num_sms, stream));
  } else
  {
    TG_TRY(alloc_n(&e32, sm));
    TG_TRY(alloc_n(&r32, sm));
    const size_t s4 = static_cast<size_t>(S) * n1 * 4;
    TG_TRY(alloc_n(&e4, s4));
    TG_CUDA(cudaMemset(e4, 0, sizeof(uint2) * s4));
    if (rev4) {
      // slots beyond a node's in-links keep an infinite weight: never tight
      TG_TRY(alloc_n(&r4, s4));
      TG_CUDA(launch_fill_records(r4, s4, make_uint2(0u, 0x7f800000u), 2 * num_sms, stream));
    }
  }
  if (opt.record_tape) TG_TRY(alloc_n(&dtdx, sm));
  TG_TRY(alloc_n(&state, static_cast<size_t>(S)));
  TG_TRY(alloc_n(&partials, static_cast<size_t>(S) * std::max(link_grid, ls_link_grid) * kNumSums));
  TG_TRY(alloc_n(&arrive, static_cast<size_t>(S)));
  TG_CUDA(cudaMemset(arrive, 0, sizeof(unsigned) * S));
  trace_cap = S == 1 ? 100000 : 4096;
  TG_TRY(alloc_n(&trace, static_cast<size_t>(S) * trace_cap * kTraceCols));
  TG_TRY(alloc_n(&scen_list, static_cast<size_t>(S)));
  if (opt.record_tape && opt.tape_capacity > 0) {
    hist_cap = opt.tape_capacity;
    ckpt_every = opt.tape_checkpoint > 0
                     ? opt.tape_checkpoint
                     : std::max(1, static_cast<int>(std::ceil(std::sqrt(double(hist_cap)))));
    TG_TRY(alloc_n(&x_hist, sm * (hist_cap / ckpt_every + 1)));
    TG_TRY(alloc_n(&d_hist, sm * hist_cap));
    TG_TRY(alloc_n(&lam_hist, static_cast<size_t>(S) * hist_cap));
  }
  S_cap = S;
  // Unless the caller fixed the chunk, the label buffer grows to hold a whole
  // batch's tasks (up to 16 GiB), so that an iteration runs one shortest-path
  // and one loading launch instead of one per chunk, each with its tail.
  if (opt.chunk_tasks <= 0 && dist) {
    const int64_t tb = static_cast<int64_t>(n1) * (fp64 ? 8 : 4);
    const int64_t want = std::min<int64_t>(std::max<int64_t>(1, (int64_t(16) << 30) / tb),
                                           static_cast<int64_t>(S) * std::max(Z, 1));
    if (want > dist_tasks) {
      free_owned(this, dist);
      dist = nullptr;
      TG_TRY(alloc(&dist, static_cast<size_t>(tb) * static_cast<size_t>(want)));
      dist_tasks = want;
      if (pred_buf) {  // sized by the label buffer: made again on its next use
        free_owned(this, pred_buf);
        pred_buf = nullptr;
      }
    }
  }
  if (gexec) {
    cudaGraphExecDestroy(gexec);
    gexec = nullptr;
  }
  g_nscen = -1;
  return TAPGPU_OK;
}

int Ctx::plan_launches() {
  cudaDeviceProp prop;
  TG_CUDA(cudaGetDeviceProperties(&prop, device));
  num_sms = prop.multiProcessorCount;
  const int optin = max_smem_optin(device);
  ls_mode = opt.line_search == kLsExact ? kLsExact : kLsReference;
  // default: the edge-list sweeps for small networks (tasks too small to
  // keep a queue busy), else the queue kernel
  const bool small = n1 <= kSmallNet && M <= kSmallNet;
  sssp_variant = (opt.sssp_variant >= kSsspRounds && opt.sssp_variant <= kSsspNearFarQueue) ||
                         opt.sssp_variant == kSsspSmall
                     ? opt.sssp_variant
                     : (small ? kSsspSmall : kSsspNearFarQueue);
  // the ring of the queue variant holds 16-bit node ids, and its padded
  // records 16-bit heads and degrees
  if (sssp_variant == kSsspNearFarQueue && !deg16) sssp_variant = kSsspNearFarQueueWide;
  const bool nf = sssp_variant == kSsspNearFar || sssp_variant == kSsspNearFarQueue ||
                  sssp_variant == kSsspNearFarQueueWide;
  sssp_block = opt.sssp_block > 0 ? opt.sssp_block : (nf ? 256 : 512);
  // the ring keeps one free slot per thread
  if ((sssp_variant == kSsspNearFarQueue || sssp_variant == kSsspNearFarQueueWide) &&
      sssp_block >= kQueueSlots)
    sssp_block = 256;
  // FP64 loading in the compact layout (10 bytes per node, two 512-thread
  // CTAs per SM) up to 65535 nodes
  aon_c64 = fp64 && n1 <= 0xffff && !opt.global_scratch;
  aon_block = opt.aon_block > 0 ? opt.aon_block : (aon_c64 ? 512 : 1024);
  // leave room for the kernels' static shared memory (a few words)
  const size_t room = optin > 1024 ? static_cast<size_t>(optin - 1024) : 0;
  sssp_smem = sssp_smem_bytes(n1, fp64, sssp_variant, M) <= room && !opt.global_scratch;
  aon_smem = aon_smem_bytes(n1, fp64, aon_c64) <= room && !opt.global_scratch;
  // near-far kernels whose shared memory leaves at most four 256-thread CTAs
  // per SM (FP64 labels of a 10k-node network: two) take 512 threads, so
  // that each task has more warps in flight (10k nodes, FP64: 77.0 -> 67.5 ms
  // per 64-scenario iteration)
  if (opt.sssp_block <= 0 && nf && sssp_smem &&
      sssp_occupancy(fp64, 256, true, n1, sssp_variant, M) * 256 <= 1024)
    sssp_block = 512;
  int so = sssp_occupancy(fp64, sssp_block, sssp_smem, n1, sssp_variant, M, opt.global_scratch == 2);
  int ao = aon_occupancy(fp64, aon_block, aon_smem, n1, aon_c64);
  if (so <= 0 || ao <= 0) {
    set_message("no resident CTA fits for the shortest-path kernels");
    return TAPGPU_ERR_UNSUPPORTED;
  }
  if (opt.sssp_ctas_per_sm > 0) so = std::min(so, opt.sssp_ctas_per_sm);
  if (opt.aon_ctas_per_sm > 0) ao = std::min(ao, opt.aon_ctas_per_sm);
  sssp_grid = so * num_sms;
  aon_grid = ao * num_sms;
  size_t scratch = 0;
  if (!sssp_smem) scratch = std::max(scratch, sssp_smem_bytes(n1, fp64, sssp_variant, M) * sssp_grid);
  if (!aon_smem) scratch = std::max(scratch, aon_smem_bytes(n1, fp64, aon_c64) * aon_grid);
  if (scratch) {
    TG_TRY(alloc(&path_scratch, scratch));
    path_scratch_bytes = scratch;
  }
  link_grid = std::max(1, std::min((M + 255) / 256, 2 * num_sms));
  // small networks: 64-thread blocks spread the line search's FP64 work
  // over more SMs
  ls_block = M <= kSmallNet ? kSmallLinkBlock : 256;
  ls_link_grid = std::max(1, std::min((M + ls_block - 1) / ls_block, 2 * num_sms * (256 / ls_block)));
  return TAPGPU_OK;
}

int Ctx::enqueue_paths(int nscen, bool load, const uint2* e32p, const uint2* r32p, const double* w64p,
                       unsigned long long* ydst, bool use_state) {
  const int64_t tasks = static_cast<int64_t>(nscen) * Z;
  for (int64_t t0 = 0; t0 < tasks; t0 += dist_tasks) {
    const int64_t t1 = std::min(tasks, t0 + dist_tasks);
    PathArgs a = path_args(nscen);
    if (a.e4) a.e4 = e32p == e32 ? e4 : (e32p == api_e32 ? api_e4 : nullptr);
    a.e32 = e32p;
    a.r32 = r32p;
    if (r32p != r32) a.r4 = nullptr;  // (the padded reverse records follow the context's own)
    if (w64p != w64) a.r4d = nullptr;
    a.w64 = w64p;
    a.y_fx = ydst;
    a.do_load = load ? 1 : 0;
    a.task_begin = static_cast<int>(t0);
    a.task_end = static_cast<int>(t1);
    if (!use_state) {
      a.state = nullptr;
      a.scen_list = nullptr;
      a.dem.od_q = od_q;
      a.dem.q_stride = 0;
    }
    const int ntask = static_cast<int>(t1 - t0);
    a.scratch_stride = static_cast<long long>(sssp_smem_bytes(n1, fp64, sssp_variant, M));
    TG_CUDA(cudaMemsetAsync(counters, 0, 2 * sizeof(int), stream));
    a.counter = counters;
    if (measuring) TG_TRY(mark(0, true));
    TG_CUDA(launch_sssp(a, fp64, std::min(sssp_grid, ntask), sssp_block, sssp_smem, sssp_variant,
                        stream));
    if (measuring) TG_TRY(mark(0, false));
    a.counter = counters + 1;
    a.scratch_stride = static_cast<long long>(aon_smem_bytes(n1, fp64, aon_c64));
    if (measuring) TG_TRY(mark(1, true));
    TG_CUDA(launch_aon(a, fp64, std::min(aon_grid, ntask), aon_block, aon_smem, stream));
    if (measuring) TG_TRY(mark(1, false));
    count_launches(2);
  }
  return TAPGPU_OK;
}

void Ctx::count_launches(long long n) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(stream, &cs);
  if (cs == cudaStreamCaptureStatusActive)
    g_kernels += n;
  else
    launches += n;
}

int Ctx::enqueue_iteration(int nscen) {
  measuring = true;
  int rc = enqueue_paths(nscen, true, e32, r32, w64, yfx, true);
  measuring = false;
  TG_TRY(rc);
  LinkArgs la = link_args(nscen);
  if (M <= kSmallTail) {  // small networks: the line search and the step in one launch
    TG_TRY(mark(2, true));
    TG_CUDA(launch_fw_tail_small(la, stream));
    TG_TRY(mark(2, false));
    count_launches(1);
    return TAPGPU_OK;
  }
  TG_TRY(mark(2, true));
  const int passes = ls_mode == kLsExact ? kLsExactPasses : kLsPasses;
  for (int p = 0; p < passes; ++p) {
    la.pass = p;
    TG_CUDA(launch_ls_pass(la, ls_grid(nscen), ls_block, stream));
  }
  TG_CUDA(launch_ls_fallback(la, stream));
  TG_TRY(mark(2, false));
  TG_TRY(mark(3, true));
  TG_CUDA(launch_step(la, ls_link_grid, ls_block, stream));
  TG_TRY(mark(3, false));
  count_launches(passes + 2);
  return TAPGPU_OK;
}

// State reset, first all-or-nothing at free-flow costs (or warm flows), costs.
int Ctx::enqueue_initial(int nscen, bool warm) {
  LinkArgs la = link_args(nscen);
  if (!warm) {
    TG_CUDA(launch_set_costs(la, link_grid, stream));
    count_launches(1);
    TG_TRY(enqueue_paths(nscen, true, e32, r32, w64, yfx, true));
    la.pass = 0;
  } else {
    la.pass = 1;
  }
  TG_CUDA(launch_init_flows(la, link_grid, stream));
  count_launches(1);
  return TAPGPU_OK;
}

int Ctx::run_graph(int iters, int nscen) {
  if (!opt.use_graphs) {
    timed.clear();
    ev_used = 0;
    for (int i = 0; i < iters; ++i) TG_TRY(enqueue_iteration(nscen));
    if (timing) {
      TG_CUDA(cudaStreamSynchronize(stream));
      collect_timing();
    }
    return TAPGPU_OK;
  }
  if (!gexec || g_iters != iters || g_nscen != nscen || g_dem != use_dem_scen ||
      g_links != use_link_scen) {
    if (gexec) {
      cudaGraphExecDestroy(gexec);
      gexec = nullptr;
    }
    timed.clear();
    ev_used = 0;
    g_kernels = 0;
    cudaGraph_t graph = nullptr;
    TG_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = TAPGPU_OK;
    for (int i = 0; i < iters && rc == TAPGPU_OK; ++i) rc = enqueue_iteration(nscen);
    cudaError_t ec = cudaStreamEndCapture(stream, &graph);
    if (rc != TAPGPU_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (ec != cudaSuccess) {
      set_message(std::string("graph capture: ") + cudaGetErrorString(ec));
      return TAPGPU_ERR_CUDA;
    }
    cudaError_t ei = cudaGraphInstantiate(&gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
      set_message(std::string("graph instantiate: ") + cudaGetErrorString(ei));
      gexec = nullptr;
      return TAPGPU_ERR_CUDA;
    }
    g_iters = iters;
    g_nscen = nscen;
    g_dem = use_dem_scen;
    g_links = use_link_scen;
  }
  TG_CUDA(cudaGraphLaunch(gexec, stream));
  launches += g_kernels;
  if (timing) {
    // the graph's event nodes are re-recorded by every replay: read them now
    TG_CUDA(cudaStreamSynchronize(stream));
    collect_timing();
  }
  return TAPGPU_OK;
}

int Ctx::sync_check() {
  TG_CUDA(cudaStreamSynchronize(stream));
  int e = 0;
  TG_CUDA(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e & kErrNoPath) {
    int info[2] = {0, 0};
    cudaMemcpy(info, err_info, sizeof(info), cudaMemcpyDeviceToHost);
    set_message("ERROR: no path from " + std::to_string(info[0]) + " to " +
                std::to_string(info[1]));
    return TAPGPU_ERR_NO_PATH;
  }
  if (e & (kErrRounds | kErrWalk | kErrPending)) {
    set_message("device loop hit its bound (error bits " + std::to_string(e) + ")");
    return TAPGPU_ERR_NO_CONVERGENCE;
  }
  return TAPGPU_OK;
}

int Ctx::read_states(int S, std::vector<ScenState>& out) {
  out.resize(S);
  TG_CUDA(cudaMemcpyAsync(out.data(), state, sizeof(ScenState) * S, cudaMemcpyDeviceToHost,
                          stream));
  TG_CUDA(cudaStreamSynchronize(stream));
  return TAPGPU_OK;
}

// ---------------------------------------------------------------------------
// construction
// ---------------------------------------------------------------------------

static int validate(const tapgpu_network* net, const tapgpu_demand* dem) {
  if (!net || !net->init || !net->term || !net->capacity || !net->fft || !net->alpha ||
      !net->beta) {
    set_message("network arrays missing");
    return TAPGPU_ERR_ARG;
  }
  if (net->num_nodes < 1 || net->num_links < 1 || net->num_nodes > (1 << 30) ||
      net->num_links > (1ll << 31) - 2) {
    set_message("network size out of range");
    return TAPGPU_ERR_ARG;
  }
  if (net->num_zones < 0 || net->num_zones > net->num_nodes || net->first_thru_node < 0) {
    set_message("zone count or first thru node out of range");
    return TAPGPU_ERR_ARG;
  }
  for (int64_t k = 0; k < net->num_links; ++k) {
    const int64_t a = net->init[k], b = net->term[k];
    // node 0 is the reference's unused row; 0-based graphs (the Python
    // extension's) use it as an ordinary node
    if (a < 0 || a > net->num_nodes || b < 0 || b > net->num_nodes) {
      set_message("link " + std::to_string(k) + " has a node outside 0..N");
      return TAPGPU_ERR_ARG;
    }
    if (!(net->fft[k] >= 0) || !std::isfinite(net->fft[k]) || !(net->alpha[k] >= 0) ||
        !std::isfinite(net->alpha[k]) || !std::isfinite(net->beta[k]) ||
        std::isnan(net->capacity[k])) {
      set_message("link " + std::to_string(k) + " has an invalid cost parameter");
      return TAPGPU_ERR_ARG;
    }
  }
  if (dem) {
    if (dem->num_origins < 0 || dem->num_origins > net->num_nodes ||
        (dem->num_origins > 0 && (!dem->od_ptr || !dem->od_dest || !dem->od_demand))) {
      set_message("demand arrays missing or origin count out of range");
      return TAPGPU_ERR_ARG;
    }
    for (int64_t o = 1; o <= dem->num_origins; ++o)
      if (dem->od_ptr[o + 1] < dem->od_ptr[o]) {
        set_message("demand pointers not monotone");
        return TAPGPU_ERR_ARG;
      }
    const int64_t nnz = dem->num_origins > 0 ? dem->od_ptr[dem->num_origins + 1] : 0;
    for (int64_t i = 0; i < nnz; ++i)
      if (dem->od_dest[i] < 0 || dem->od_dest[i] > net->num_nodes ||
          std::isnan(dem->od_demand[i])) {
        set_message("demand entry " + std::to_string(i) + " invalid");
        return TAPGPU_ERR_ARG;
      }
  }
  return TAPGPU_OK;
}

static int create_impl(const tapgpu_network* net, const tapgpu_demand* dem,
                       const tapgpu_options* opt_in, Ctx** out) {
  TG_TRY(validate(net, dem));
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_message("no CUDA device");
    return TAPGPU_ERR_NO_DEVICE;
  }
  tapgpu_options opt;
  tapgpu_default_options(&opt);
  if (opt_in) opt = *opt_in;
  if (opt.device < 0 || opt.device >= ndev) {
    set_message("device ordinal out of range");
    return TAPGPU_ERR_ARG;
  }
  TG_CUDA(cudaSetDevice(opt.device));
  Ctx* c = new Ctx();
  std::unique_ptr<Ctx> guard(c);
  c->opt = opt;
  c->device = opt.device;
  c->fp64 = opt.precision == TAPGPU_FP64;
  c->N = static_cast<int>(net->num_nodes);
  c->n1 = c->N + 1;
  c->M = static_cast<int>(net->num_links);
  c->Z = static_cast<int>(dem ? dem->num_origins : net->num_zones);
  c->F = static_cast<int>(std::min<int64_t>(net->first_thru_node, c->n1 + 1));
  const int M = c->M, n1 = c->n1;

  // links sorted by (init, term) as tap/parsetapfiles.c:528-540 orders them
  c->perm.resize(M);
  std::iota(c->perm.begin(), c->perm.end(), 0);
  std::stable_sort(c->perm.begin(), c->perm.end(), [&](int64_t a, int64_t b) {
    if (net->init[a] != net->init[b]) return net->init[a] < net->init[b];
    return net->term[a] < net->term[b];
  });
  c->h_tail.resize(M);
  c->h_head.resize(M);
  c->h_cap.resize(M);
  c->h_fft.resize(M);
  c->h_alpha.resize(M);
  c->h_beta.resize(M);
  std::vector<unsigned char> ip(M);
  double min_cap = DBL_MAX;
  for (int k = 0; k < M; ++k) {
    const int64_t e = c->perm[k];
    c->h_tail[k] = static_cast<int>(net->init[e]);
    c->h_head[k] = static_cast<int>(net->term[e]);
    c->h_cap[k] = net->capacity[e];
    c->h_fft[k] = net->fft[e];
    c->h_alpha[k] = net->alpha[e];
    c->h_beta[k] = net->beta[e];
    const double b = net->beta[e];
    ip[k] = (b >= 0 && b <= 15 && std::floor(b) == b) ? static_cast<unsigned char>(b) : 255;
    if (c->h_cap[k] > 0.0 && c->h_cap[k] < min_cap) min_cap = c->h_cap[k];
  }
  // tap/tap_frankwolfe_pthread.c:654-669 zero capacity -> smallest nonzero capacity
  for (int k = 0; k < M; ++k)
    if (!(c->h_cap[k] > 0.0)) c->h_cap[k] = min_cap;
  {
    double s = 0.0;
    for (int k = 0; k < M; ++k) s += c->h_fft[k];
    const double mean = s / M;
    c->nf_delta = opt.nf_delta > 0 ? opt.nf_delta : (mean > 0 ? 16.0 * mean : 1.0);
  }

  std::vector<int> rp(n1 + 1, 0), ip_in(n1 + 1, 0), inl(M);
  for (int k = 0; k < M; ++k) {
    rp[c->h_tail[k] + 1]++;
    ip_in[c->h_head[k] + 1]++;
  }
  for (int v = 0; v < n1; ++v) {
    rp[v + 1] += rp[v];
    ip_in[v + 1] += ip_in[v];
  }
  c->h_rpos.resize(M);
  {
    std::vector<int> fill(ip_in.begin(), ip_in.end() - 1);
    for (int k = 0; k < M; ++k) {
      c->h_rpos[k] = fill[c->h_head[k]];
      inl[fill[c->h_head[k]]++] = k;
    }
  }

  TG_TRY(c->alloc_n(&c->row_ptr, n1 + 1));
  TG_TRY(c->alloc_n(&c->head, M));
  TG_TRY(c->alloc_n(&c->tail, M));
  TG_TRY(c->alloc_n(&c->in_ptr, n1 + 1));
  TG_TRY(c->alloc_n(&c->in_link, M));
  TG_TRY(c->alloc_n(&c->in_head, M));
  TG_TRY(c->alloc_n(&c->out_deg, n1));
  TG_TRY(c->alloc_n(&c->ell_pos, M));
  TG_TRY(c->alloc_n(&c->e4x, M));
  TG_TRY(c->alloc_n(&c->rpos, M));
  TG_TRY(c->alloc_n(&c->fft, M));
  TG_TRY(c->alloc_n(&c->alpha, M));
  TG_TRY(c->alloc_n(&c->beta, M));
  TG_TRY(c->alloc_n(&c->ipow, M));
  TG_CUDA(cudaMemcpy(c->row_ptr, rp.data(), sizeof(int) * (n1 + 1), cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c->head, c->h_head.data(), sizeof(int) * M, cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c->tail, c->h_tail.data(), sizeof(int) * M, cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c->in_ptr, ip_in.data(), sizeof(int) * (n1 + 1), cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c->in_link, inl.data(), sizeof(int) * M, cudaMemcpyHostToDevice));
  {
    std::vector<int> ih(M);
    for (int i = 0; i < M; ++i) ih[i] = c->h_head[inl[i]];
    TG_CUDA(cudaMemcpy(c->in_head, ih.data(), sizeof(int) * M, cudaMemcpyHostToDevice));
    std::vector<int> deg(n1), pos(M);
    for (int v = 0; v < n1; ++v) deg[v] = rp[v + 1] - rp[v];
    for (int k = 0; k < M; ++k) {
      const int v = c->h_tail[k], j = k - rp[v];
      pos[k] = j < 4 ? v * 4 + j : -1;
    }
    c->h_ell_pos = pos;
    int maxdeg = 0;
    for (int v = 0; v < n1; ++v) maxdeg = std::max(maxdeg, deg[v]);
    c->deg16 = n1 <= 0xffff && maxdeg <= 0xffff;
    c->h_e4x.resize(M);
    for (int k = 0; k < M; ++k) {
      const unsigned h = static_cast<unsigned>(c->h_head[k]);
      c->h_e4x[k] = c->deg16 ? h | (static_cast<unsigned>(deg[c->h_tail[k]]) << 16) : h;
    }
    TG_CUDA(cudaMemcpy(c->out_deg, deg.data(), sizeof(int) * n1, cudaMemcpyHostToDevice));
    TG_CUDA(cudaMemcpy(c->ell_pos, pos.data(), sizeof(int) * M, cudaMemcpyHostToDevice));
    // padded reverse records: FP64 paths always ({link, tail, weight}),
    // FP32 paths when nodes and links fit 16 bits ({link << 16 | tail, weight})
    c->rev4 = !c->fp64 && n1 <= 0xffff && M <= 0xffff;
    if (c->rev4 || c->fp64) {
      std::vector<int> rpos4(M);
      for (int k = 0; k < M; ++k) {
        const int v = c->h_head[k], j = c->h_rpos[k] - ip_in[v];
        rpos4[k] = j < 4 ? v * 4 + j : -1;
      }
      std::vector<unsigned> more((n1 + 31) / 32, 0u);
      for (int v = 0; v < n1; ++v)
        if (ip_in[v + 1] - ip_in[v] > 4) more[v >> 5] |= 1u << (v & 31);
      TG_TRY(c->alloc_n(&c->r4_pos, M));
      TG_TRY(c->alloc_n(&c->r4_more, more.size()));
      TG_CUDA(cudaMemcpy(c->r4_pos, rpos4.data(), sizeof(int) * M, cudaMemcpyHostToDevice));
      TG_CUDA(cudaMemcpy(c->r4_more, more.data(), sizeof(unsigned) * more.size(),
                         cudaMemcpyHostToDevice));
    }
    if (c->rev4) {
      std::vector<unsigned> rx(M);
      for (int k = 0; k < M; ++k)
        rx[k] = (static_cast<unsigned>(k) << 16) | static_cast<unsigned>(c->h_tail[k]);
      TG_TRY(c->alloc_n(&c->r4x, M));
      TG_CUDA(cudaMemcpy(c->r4x, rx.data(), sizeof(unsigned) * M, cudaMemcpyHostToDevice));
    }
    TG_CUDA(cudaMemcpy(c->e4x, c->h_e4x.data(), sizeof(unsigned) * M, cudaMemcpyHostToDevice));
  }
  TG_CUDA(cudaMemcpy(c->rpos, c->h_rpos.data(), sizeof(int) * M, cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c->fft, c->h_fft.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c->alpha, c->h_alpha.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c->beta, c->h_beta.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c->ipow, ip.data(), M, cudaMemcpyHostToDevice));

  // demand as a CSR over origin slots 0..Z-1 (origin node = slot + 1)
  const int Z = c->Z;
  std::vector<int> optr(Z + 1, 0), odest;
  std::vector<long long> oq;
  std::vector<double> odem;
  double total = 0.0, pos = 0.0;
  if (dem && Z > 0) {
    for (int o = 1; o <= Z; ++o)
      for (int64_t i = dem->od_ptr[o]; i < dem->od_ptr[o + 1]; ++i) {
        total += dem->od_demand[i];  // tap/tap_functions.c:377-386 sums every entry
        if (dem->od_demand[i] > 0) pos += dem->od_demand[i];
      }
    // fixed point with headroom: every node/link total stays below 2^61
    int bits = 40;
    if (pos > 1.0) bits = std::min(40, 61 - static_cast<int>(std::ceil(std::log2(pos))) - 1);
    c->scale_bits = bits;
    const double scale = std::ldexp(1.0, bits);
    for (int o = 1; o <= Z; ++o) {
      for (int64_t i = dem->od_ptr[o]; i < dem->od_ptr[o + 1]; ++i) {
        const double v = dem->od_demand[i];
        odest.push_back(static_cast<int>(dem->od_dest[i]));
        odem.push_back(v);
        oq.push_back(v > 0 ? std::llrint(v * scale) : 0);
      }
      optr[o] = static_cast<int>(odest.size());
    }
  }
  c->inv_scale = std::ldexp(1.0, -c->scale_bits);
  c->total_demand = total;
  c->h_od_dem = odem;
  c->nnz = static_cast<long long>(odem.size());
  std::vector<int> src(std::max(Z, 1));
  for (int i = 0; i < Z; ++i) src[i] = i + 1;
  TG_TRY(c->alloc_n(&c->od_ptr, Z + 1));
  TG_TRY(c->alloc_n(&c->od_dest, std::max<size_t>(odest.size(), 1)));
  TG_TRY(c->alloc_n(&c->od_q, std::max<size_t>(oq.size(), 1)));
  TG_TRY(c->alloc_n(&c->od_dem, std::max<size_t>(odem.size(), 1)));
  TG_TRY(c->alloc_n(&c->sources, std::max(Z, 1)));
  TG_CUDA(cudaMemcpy(c->od_ptr, optr.data(), sizeof(int) * (Z + 1), cudaMemcpyHostToDevice));
  if (!odest.empty()) {
    TG_CUDA(cudaMemcpy(c->od_dest, odest.data(), sizeof(int) * odest.size(),
                       cudaMemcpyHostToDevice));
    TG_CUDA(cudaMemcpy(c->od_q, oq.data(), sizeof(long long) * oq.size(), cudaMemcpyHostToDevice));
    TG_CUDA(cudaMemcpy(c->od_dem, odem.data(), sizeof(double) * odem.size(),
                       cudaMemcpyHostToDevice));
  }
  TG_CUDA(cudaMemcpy(c->sources, src.data(), sizeof(int) * src.size(), cudaMemcpyHostToDevice));

  TG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  TG_TRY(c->plan_launches());
  TG_TRY(c->alloc_n(&c->counters, 2));
  TG_TRY(c->alloc_n(&c->err, 1));
  TG_TRY(c->alloc_n(&c->err_info, 2));
  TG_TRY(c->alloc_n(&c->path_stats, 8));
  TG_CUDA(cudaMemset(c->err, 0, sizeof(int)));
  TG_CUDA(cudaMemset(c->path_stats, 0, 8 * sizeof(unsigned long long)));

  // shortest-path label scratch between the two path kernels
  const size_t tb = static_cast<size_t>(n1) * (c->fp64 ? 8 : 4);
  int64_t chunk = opt.chunk_tasks > 0 ? opt.chunk_tasks
                                      : std::max<int64_t>(1, (int64_t(2) << 30) / static_cast<int64_t>(tb));
  chunk = std::max<int64_t>(1, std::min<int64_t>(chunk, 1 << 30));
  c->dist_tasks = std::min<int64_t>(chunk, std::max<int64_t>(Z, 1) * 4096);
  TG_TRY(c->alloc(&c->dist, tb * c->dist_tasks));
  TG_TRY(c->alloc_n(&c->api_e32, M));
  TG_TRY(c->alloc_n(&c->api_e4, static_cast<size_t>(n1) * 4));
  TG_TRY(c->alloc_n(&c->api_r32, M));
  TG_TRY(c->alloc_n(&c->api_w64, M));
  TG_TRY(c->alloc_n(&c->api_yfx, M));
  TG_TRY(c->ensure_scenarios(1));
  std::vector<double> capv(c->h_cap);
  TG_CUDA(cudaMemcpy(c->cap, capv.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
  *out = guard.release();
  return TAPGPU_OK;
}

static int upload_states(Ctx* c, int S, int max_iters, double target) {
  std::vector<ScenState> st(S);
  for (auto& s : st) {
    std::memset(&s, 0, sizeof(s));
    s.max_iters = max_iters;
    s.target_relgap = target;
    s.relgap = DBL_MAX;
    s.best_lb = -DBL_MAX;
  }
  TG_CUDA(cudaMemcpyAsync(c->state, st.data(), sizeof(ScenState) * S, cudaMemcpyHostToDevice,
                          c->stream));
  TG_CUDA(cudaMemsetAsync(c->err, 0, sizeof(int), c->stream));
  return TAPGPU_OK;
}

static int iterate_until_done(Ctx* c, int S, int max_iters, std::vector<ScenState>& st) {
  // iterations per graph launch: enough to hide launch gaps, few enough that
  // finished scenarios do not linger
  int per = c->opt.iters_per_launch > 0 ? c->opt.iters_per_launch : (S == 1 ? 8 : 4);
  std::vector<int> active;
  for (;;) {
    TG_TRY(c->read_states(S, st));
    active.clear();
    for (int s = 0; s < S; ++s)
      if (!st[s].done) active.push_back(s);
    TG_TRY(c->sync_check());
    if (active.empty()) break;
    int n = per;
    if (max_iters > 0) {
      int left = 0;
      for (int s : active) left = std::max(left, max_iters - st[s].iter);
      n = std::max(1, std::min(n, left));
    }
    if (active != c->h_scen_list) {
      TG_CUDA(cudaMemcpyAsync(c->scen_list, active.data(), sizeof(int) * active.size(),
                              cudaMemcpyHostToDevice, c->stream));
      c->h_scen_list = active;
    }
    TG_TRY(c->run_graph(n, static_cast<int>(active.size())));
  }
  return TAPGPU_OK;
}

static void fill_result(const ScenState& s, int err_bits, tapgpu_result* r) {
  r->iterations = s.iter;
  r->error_bits = err_bits;
  r->objective = s.obj;
  r->relgap = s.relgap;
  r->total_cost = s.vht_end;
  r->avg_excess = s.avg_excess;
  r->lambda_last = s.lambda;
}

}  // namespace tapgpu

using tapgpu::Ctx;

extern "C" {

void tapgpu_default_options(tapgpu_options* o) {
  std::memset(o, 0, sizeof(*o));
  o->precision = TAPGPU_FP64;
  o->device = 0;
  o->use_graphs = 1;
}

const char* tapgpu_status_string(int s) {
  switch (s) {
    case TAPGPU_OK: return "ok";
    case TAPGPU_ERR_ARG: return "invalid argument";
    case TAPGPU_ERR_CUDA: return "CUDA error";
    case TAPGPU_ERR_NO_PATH: return "no path for a positive demand";
    case TAPGPU_ERR_NO_CONVERGENCE: return "device loop hit its bound";
    case TAPGPU_ERR_ALLOC: return "allocation failed";
    case TAPGPU_ERR_UNSUPPORTED: return "unsupported size";
    case TAPGPU_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char* tapgpu_last_message(void) { return tapgpu::g_message.c_str(); }

int tapgpu_create(const tapgpu_network* net, const tapgpu_demand* dem, const tapgpu_options* opt,
                  tapgpu_ctx** out) {
  if (!out) return TAPGPU_ERR_ARG;
  *out = nullptr;
  Ctx* c = nullptr;
  int rc = tapgpu::create_impl(net, dem, opt, &c);
  if (rc != TAPGPU_OK) return rc;
  *out = new tapgpu_ctx{c};
  return TAPGPU_OK;
}

void tapgpu_destroy(tapgpu_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->c->device);
  delete ctx->c;
  delete ctx;
}

int tapgpu_set_capacity(tapgpu_ctx* ctx, const double* capacity) {
  if (!ctx || !capacity) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  double min_cap = DBL_MAX;
  for (int k = 0; k < c->M; ++k) {
    const double v = capacity[c->perm[k]];
    if (v > 0 && v < min_cap) min_cap = v;
  }
  for (int k = 0; k < c->M; ++k) {
    const double v = capacity[c->perm[k]];
    c->h_cap[k] = v > 0 ? v : min_cap;
  }
  c->base_dirty = true;
  TG_CUDA(cudaSetDevice(c->device));
  TG_CUDA(cudaMemcpy(c->cap, c->h_cap.data(), sizeof(double) * c->M, cudaMemcpyHostToDevice));
  return TAPGPU_OK;
}

int tapgpu_solve_begin(tapgpu_ctx* ctx, int max_iters, double target_relgap, const double* x0) {
  if (!ctx || (max_iters <= 0 && !(target_relgap > 0))) {
    tapgpu::set_message("need an iteration cap or a positive relative-gap target");
    return TAPGPU_ERR_ARG;
  }
  Ctx* c = ctx->c;
  TG_CUDA(cudaSetDevice(c->device));
  TG_TRY(c->ensure_scenarios(1));
  c->use_dem_scen = false;
  c->use_link_scen = false;
  TG_CUDA(cudaMemcpy(c->cap, c->h_cap.data(), sizeof(double) * c->M, cudaMemcpyHostToDevice));
  std::vector<int> one{0};
  TG_CUDA(cudaMemcpyAsync(c->scen_list, one.data(), sizeof(int), cudaMemcpyHostToDevice, c->stream));
  c->h_scen_list = one;
  TG_TRY(tapgpu::upload_states(c, 1, max_iters, target_relgap));
  if (x0) {
    std::vector<double> xi(c->M);
    for (int k = 0; k < c->M; ++k) xi[k] = x0[c->perm[k]];
    TG_CUDA(cudaMemcpyAsync(c->x, xi.data(), sizeof(double) * c->M, cudaMemcpyHostToDevice,
                            c->stream));
    TG_CUDA(cudaStreamSynchronize(c->stream));
  }
  TG_TRY(c->enqueue_initial(1, x0 != nullptr));
  TG_TRY(c->sync_check());
  c->solve_max_iters = max_iters;
  c->last_nscen = 1;
  return TAPGPU_OK;
}

int tapgpu_solve_advance(tapgpu_ctx* ctx, int max_new_iters, int* done, tapgpu_result* res) {
  if (!ctx || max_new_iters < 1) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  TG_CUDA(cudaSetDevice(c->device));
  std::vector<tapgpu::ScenState> st;
  TG_TRY(c->read_states(1, st));
  if (!st[0].done) {
    int n = max_new_iters;
    if (c->solve_max_iters > 0) n = std::max(1, std::min(n, c->solve_max_iters - st[0].iter));
    TG_TRY(c->run_graph(n, 1));
    TG_TRY(c->read_states(1, st));
  }
  TG_TRY(c->sync_check());
  int e = 0;
  TG_CUDA(cudaMemcpy(&e, c->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (done) *done = st[0].done;
  if (res) tapgpu::fill_result(st[0], e, res);
  return TAPGPU_OK;
}

int tapgpu_solve(tapgpu_ctx* ctx, int max_iters, double target_relgap, const double* x0,
                 tapgpu_result* res) {
  int rc = tapgpu_solve_begin(ctx, max_iters, target_relgap, x0);
  if (rc != TAPGPU_OK) return rc;
  Ctx* c = ctx->c;
  std::vector<tapgpu::ScenState> st;
  TG_TRY(tapgpu::iterate_until_done(c, 1, max_iters, st));
  int e = 0;
  TG_CUDA(cudaMemcpy(&e, c->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (res) tapgpu::fill_result(st[0], e, res);
  return TAPGPU_OK;
}

int tapgpu_get_link_flows(tapgpu_ctx* ctx, int scenario, double* volume, double* cost) {
  if (!ctx) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  if (scenario < 0 || scenario >= c->S_cap) return TAPGPU_ERR_ARG;
  TG_CUDA(cudaSetDevice(c->device));
  TG_CUDA(cudaStreamSynchronize(c->stream));
  std::vector<double> tmp(c->M);
  const size_t off = static_cast<size_t>(scenario) * c->M;
  if (volume) {
    TG_CUDA(cudaMemcpy(tmp.data(), c->x + off, sizeof(double) * c->M, cudaMemcpyDeviceToHost));
    for (int k = 0; k < c->M; ++k) volume[c->perm[k]] = tmp[k];
  }
  if (cost) {
    TG_CUDA(cudaMemcpy(tmp.data(), c->t + off, sizeof(double) * c->M, cudaMemcpyDeviceToHost));
    for (int k = 0; k < c->M; ++k) cost[c->perm[k]] = tmp[k];
  }
  return TAPGPU_OK;
}

int tapgpu_get_link_flows_batch(tapgpu_ctx* ctx, int first, int count, double* volume,
                                double* cost) {
  if (!ctx || count < 1) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  if (first < 0 || static_cast<int64_t>(first) + count > c->S_cap) return TAPGPU_ERR_ARG;
  TG_CUDA(cudaSetDevice(c->device));
  TG_CUDA(cudaStreamSynchronize(c->stream));
  const int M = c->M;
  const size_t off = static_cast<size_t>(first) * M, n = static_cast<size_t>(count) * M;
  bool identity = true;
  for (int k = 0; k < M && identity; ++k) identity = c->perm[k] == k;
  double* outs[2] = {volume, cost};
  const double* srcs[2] = {c->x + off, c->t + off};
  std::vector<double> tmp;
  for (int a = 0; a < 2; ++a) {
    if (!outs[a]) continue;
    if (identity) {  // the caller's link order is the device's: one copy
      TG_CUDA(cudaMemcpy(outs[a], srcs[a], sizeof(double) * n, cudaMemcpyDeviceToHost));
      continue;
    }
    tmp.resize(n);
    TG_CUDA(cudaMemcpy(tmp.data(), srcs[a], sizeof(double) * n, cudaMemcpyDeviceToHost));
    for (int s = 0; s < count; ++s) {
      const double* row = tmp.data() + static_cast<size_t>(s) * M;
      double* out = outs[a] + static_cast<size_t>(s) * M;
      for (int k = 0; k < M; ++k) out[c->perm[k]] = row[k];
    }
  }
  return TAPGPU_OK;
}

int tapgpu_get_trace(tapgpu_ctx* ctx, int scenario, double* rows, int max_rows, int* nrows) {
  if (!ctx || !rows || !nrows) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  if (scenario < 0 || scenario >= c->S_cap) return TAPGPU_ERR_ARG;
  TG_CUDA(cudaSetDevice(c->device));
  tapgpu::ScenState st;
  TG_CUDA(cudaStreamSynchronize(c->stream));
  TG_CUDA(cudaMemcpy(&st, c->state + scenario, sizeof(st), cudaMemcpyDeviceToHost));
  const int n = std::min(std::min(st.iter, c->trace_cap), max_rows);
  if (n > 0)
    TG_CUDA(cudaMemcpy(rows, c->trace + static_cast<size_t>(scenario) * c->trace_cap * tapgpu::kTraceCols,
                       sizeof(double) * n * tapgpu::kTraceCols, cudaMemcpyDeviceToHost));
  *nrows = n;
  return TAPGPU_OK;
}

int tapgpu_solve_scenarios(tapgpu_ctx* ctx, int num_scen, const int64_t* scen_ptr,
                           const int64_t* scen_links, const double* scen_cap, int max_iters,
                           double target_relgap, const double* x0, tapgpu_result* results) {
  if (!ctx || num_scen < 1 || !scen_ptr || (max_iters <= 0 && !(target_relgap > 0))) {
    tapgpu::set_message("bad scenario arguments");
    return TAPGPU_ERR_ARG;
  }
  Ctx* c = ctx->c;
  const int M = c->M;
  // every argument is checked before the context's state changes
  const int64_t nedit = scen_ptr[num_scen] - scen_ptr[0];
  if (nedit > std::numeric_limits<int>::max() - 1) {
    tapgpu::set_message("too many scenario edits in one call");
    return TAPGPU_ERR_ARG;
  }
  if (nedit > 0 && (!scen_links || !scen_cap)) {
    tapgpu::set_message("scenario edits without link or capacity arrays");
    return TAPGPU_ERR_ARG;
  }
  std::vector<int64_t> inv(M);
  for (int k = 0; k < M; ++k) inv[c->perm[k]] = k;
  for (int s = 0; s < num_scen; ++s) {
    if (scen_ptr[s + 1] < scen_ptr[s]) return TAPGPU_ERR_ARG;
    for (int64_t i = scen_ptr[s]; i < scen_ptr[s + 1]; ++i)
      if (scen_links[i] < 0 || scen_links[i] >= M || std::isnan(scen_cap[i])) {
        tapgpu::set_message("scenario link index out of range");
        return TAPGPU_ERR_ARG;
      }
  }
  if (c->dem_scen && c->dem_scen != num_scen) {
    tapgpu::set_message("demand scenarios were set for " + std::to_string(c->dem_scen) +
                        " scenarios, not " + std::to_string(num_scen));
    return TAPGPU_ERR_ARG;
  }
  if (c->link_scen && c->link_scen != num_scen) {
    tapgpu::set_message("link-record scenarios were set for " + std::to_string(c->link_scen) +
                        " scenarios, not " + std::to_string(num_scen));
    return TAPGPU_ERR_ARG;
  }
  TG_CUDA(cudaSetDevice(c->device));
  TG_TRY(c->ensure_scenarios(num_scen));
  c->use_dem_scen = c->dem_scen == num_scen;
  c->use_link_scen = c->link_scen == num_scen;
  c->last_nscen = num_scen;
  // capacities of every scenario, made on the device from the base row and
  // the edits; the host finds each scenario's smallest positive capacity
  // for the zero-capacity fix-up
  if (c->base_dirty) {
    if (!c->base_cap) TG_TRY(c->alloc_n(&c->base_cap, M));
    TG_CUDA(cudaMemcpy(c->base_cap, c->h_cap.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
    c->h_cap_order.resize(M);
    std::iota(c->h_cap_order.begin(), c->h_cap_order.end(), 0);
    std::stable_sort(c->h_cap_order.begin(), c->h_cap_order.end(),
                     [c](int a, int b) { return c->h_cap[a] < c->h_cap[b]; });
    c->base_dirty = false;
  }
  std::vector<int> eptr(num_scen + 1), elink(static_cast<size_t>(std::max<int64_t>(nedit, 1)));
  std::vector<double> evalv(elink.size()), emin(num_scen);
  {
    std::vector<int> seen;  // links edited in this scenario (few)
    int64_t j = 0;
    for (int s = 0; s < num_scen; ++s) {
      eptr[s] = static_cast<int>(j);
      seen.clear();
      for (int64_t i = scen_ptr[s]; i < scen_ptr[s + 1]; ++i, ++j) {
        elink[j] = static_cast<int>(inv[scen_links[i]]);
        evalv[j] = scen_cap[i];
        seen.push_back(elink[j]);
      }
      // smallest positive capacity of the final row: edits (the last edit of
      // a link wins) and the smallest base capacity of a link not edited
      double mn = DBL_MAX;
      for (int64_t i = eptr[s]; i < j; ++i) {
        bool last = true;
        for (int64_t i2 = i + 1; i2 < j; ++i2) last = last && elink[i2] != elink[i];
        if (last && evalv[i] > 0 && evalv[i] < mn) mn = evalv[i];
      }
      for (int k : c->h_cap_order) {
        if (std::find(seen.begin(), seen.end(), k) != seen.end()) continue;
        if (c->absent_in(s, k)) continue;  // not part of this scenario's network
        if (c->h_cap[k] < mn) mn = c->h_cap[k];
        break;
      }
      emin[s] = mn;
    }
    eptr[num_scen] = static_cast<int>(j);
  }
  if (num_scen + 1 > c->ed_scen_cap) {
    if (c->ed_ptr) tapgpu::free_owned(c, c->ed_ptr);
    if (c->ed_min) tapgpu::free_owned(c, c->ed_min);
    c->ed_ptr = nullptr;
    c->ed_min = nullptr;
    TG_TRY(c->alloc_n(&c->ed_ptr, num_scen + 1));
    TG_TRY(c->alloc_n(&c->ed_min, num_scen + 1));
    c->ed_scen_cap = num_scen + 1;
  }
  if (static_cast<int64_t>(elink.size()) > c->ed_cap) {
    if (c->ed_link) tapgpu::free_owned(c, c->ed_link);
    if (c->ed_val) tapgpu::free_owned(c, c->ed_val);
    c->ed_link = nullptr;
    c->ed_val = nullptr;
    TG_TRY(c->alloc_n(&c->ed_link, elink.size()));
    TG_TRY(c->alloc_n(&c->ed_val, elink.size()));
    c->ed_cap = static_cast<int64_t>(elink.size());
  }
  TG_CUDA(cudaMemcpyAsync(c->ed_ptr, eptr.data(), sizeof(int) * eptr.size(),
                          cudaMemcpyHostToDevice, c->stream));
  TG_CUDA(cudaMemcpyAsync(c->ed_link, elink.data(), sizeof(int) * elink.size(),
                          cudaMemcpyHostToDevice, c->stream));
  TG_CUDA(cudaMemcpyAsync(c->ed_val, evalv.data(), sizeof(double) * evalv.size(),
                          cudaMemcpyHostToDevice, c->stream));
  TG_CUDA(cudaMemcpyAsync(c->ed_min, emin.data(), sizeof(double) * emin.size(),
                          cudaMemcpyHostToDevice, c->stream));
  TG_CUDA(tapgpu::launch_scenario_caps(c->cap, c->base_cap, M, num_scen, c->ed_ptr, c->ed_link,
                                       c->ed_val, c->ed_min, c->link_grid, c->stream));
  // the host vectors above must outlive the copies
  TG_CUDA(cudaStreamSynchronize(c->stream));
  std::vector<int> all(num_scen);
  std::iota(all.begin(), all.end(), 0);
  TG_CUDA(cudaMemcpyAsync(c->scen_list, all.data(), sizeof(int) * num_scen,
                          cudaMemcpyHostToDevice, c->stream));
  c->h_scen_list = all;
  TG_TRY(tapgpu::upload_states(c, num_scen, max_iters, target_relgap));
  if (x0) {
    // the warm start once, then copied to every scenario on the device
    std::vector<double> xi(M);
    for (int k = 0; k < M; ++k) xi[k] = x0[c->perm[k]];
    TG_CUDA(cudaMemcpyAsync(c->x, xi.data(), sizeof(double) * M, cudaMemcpyHostToDevice, c->stream));
    TG_CUDA(tapgpu::launch_replicate_rows(c->x, M, num_scen, c->link_grid, c->stream));
    TG_CUDA(cudaStreamSynchronize(c->stream));
    TG_TRY(c->enqueue_initial(num_scen, true));
  } else if (c->use_dem_scen || c->use_link_scen) {
    // every scenario has its own demand or links: load each at its own free flow
    tapgpu::LinkArgs la = c->link_args(num_scen);
    TG_CUDA(tapgpu::launch_set_costs(la, c->link_grid, c->stream));
    TG_TRY(c->enqueue_paths(num_scen, true, c->e32, c->r32, c->w64, c->yfx, true));
    la.pass = 0;
    TG_CUDA(tapgpu::launch_init_flows(la, c->link_grid, c->stream));
  } else {
    // free-flow all-or-nothing does not depend on capacity: load scenario 0
    // once and start every scenario from it
    tapgpu::LinkArgs la = c->link_args(1);
    TG_CUDA(tapgpu::launch_set_costs(la, c->link_grid, c->stream));
    TG_TRY(c->enqueue_paths(1, true, c->e32, c->r32, c->w64, c->yfx, true));
    for (int s = 1; s < num_scen; ++s)
      TG_CUDA(cudaMemcpyAsync(c->yfx + static_cast<size_t>(s) * M, c->yfx,
                              sizeof(unsigned long long) * M, cudaMemcpyDeviceToDevice,
                              c->stream));
    la = c->link_args(num_scen);
    la.pass = 0;
    TG_CUDA(tapgpu::launch_init_flows(la, c->link_grid, c->stream));
  }
  TG_TRY(c->sync_check());
  std::vector<tapgpu::ScenState> st;
  TG_TRY(tapgpu::iterate_until_done(c, num_scen, max_iters, st));
  int e = 0;
  TG_CUDA(cudaMemcpy(&e, c->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (results)
    for (int s = 0; s < num_scen; ++s) tapgpu::fill_result(st[s], e, &results[s]);
  return TAPGPU_OK;
}

int tapgpu_set_scenario_demand(tapgpu_ctx* ctx, int num_scen, const double* demand) {
  if (!ctx || num_scen < 0) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  TG_CUDA(cudaSetDevice(c->device));
  TG_CUDA(cudaStreamSynchronize(c->stream));
  if (c->sc_od_q) tapgpu::free_owned(c, c->sc_od_q);
  if (c->sc_total) tapgpu::free_owned(c, c->sc_total);
  c->sc_od_q = nullptr;
  c->sc_total = nullptr;
  c->dem_scen = 0;
  c->use_dem_scen = false;
  if (c->gexec) {  // captured launches hold the old demand pointers
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  c->g_nscen = -1;
  if (num_scen == 0 || !demand) return TAPGPU_OK;
  const long long nnz = c->nnz;
  if (nnz == 0) {
    tapgpu::set_message("the context has no demand to vary");
    return TAPGPU_ERR_ARG;
  }
  std::vector<double> totals(num_scen);
  double max_pos = 0.0;
  for (int s = 0; s < num_scen; ++s) {
    double tot = 0.0, pos = 0.0;
    for (long long i = 0; i < nnz; ++i) {
      const double v = demand[static_cast<size_t>(s) * nnz + i];
      if (std::isnan(v) || std::isinf(v)) {
        tapgpu::set_message("scenario demand must be finite");
        return TAPGPU_ERR_ARG;
      }
      if (v > 0 && !(c->h_od_dem[i] > 0)) {
        tapgpu::set_message("a demand scenario can only change OD pairs with positive base demand");
        return TAPGPU_ERR_ARG;
      }
      tot += v;  // tap/tap_functions.c:377-386 sums every entry
      if (v > 0) pos += v;
    }
    totals[s] = tot;
    max_pos = std::max(max_pos, pos);
  }
  // keep every node/link total below 2^61 in the shared fixed point
  int bits = 40;
  if (max_pos > 1.0) bits = std::min(40, 61 - static_cast<int>(std::ceil(std::log2(max_pos))) - 1);
  if (bits < c->scale_bits) {
    const double scale = std::ldexp(1.0, bits);
    std::vector<long long> oq(nnz);
    for (long long i = 0; i < nnz; ++i)
      oq[i] = c->h_od_dem[i] > 0 ? std::llrint(c->h_od_dem[i] * scale) : 0;
    TG_CUDA(cudaMemcpy(c->od_q, oq.data(), sizeof(long long) * nnz, cudaMemcpyHostToDevice));
    c->scale_bits = bits;
    c->inv_scale = std::ldexp(1.0, -bits);
  }
  const double scale = std::ldexp(1.0, c->scale_bits);
  std::vector<long long> q(static_cast<size_t>(num_scen) * nnz);
  for (size_t i = 0; i < q.size(); ++i) q[i] = demand[i] > 0 ? std::llrint(demand[i] * scale) : 0;
  TG_TRY(c->alloc_n(&c->sc_od_q, q.size()));
  TG_TRY(c->alloc_n(&c->sc_total, static_cast<size_t>(num_scen)));
  TG_CUDA(cudaMemcpy(c->sc_od_q, q.data(), sizeof(long long) * q.size(), cudaMemcpyHostToDevice));
  TG_CUDA(cudaMemcpy(c->sc_total, totals.data(), sizeof(double) * num_scen, cudaMemcpyHostToDevice));
  c->dem_scen = num_scen;
  return TAPGPU_OK;
}

int tapgpu_set_scenario_links(tapgpu_ctx* ctx, int num_scen, const int64_t* edit_ptr,
                              const int64_t* edit_links, const double* edit_fft,
                              const double* edit_alpha, const double* edit_beta,
                              const int64_t* absent_ptr, const int64_t* absent_links) {
  if (!ctx || num_scen < 0) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  const int M = c->M;
  if (num_scen > 0) {  // every argument is checked before the context's state changes
    if (!edit_ptr || !absent_ptr) {
      tapgpu::set_message("link-record scenarios need edit and absent-link offsets");
      return TAPGPU_ERR_ARG;
    }
    const int64_t ne = edit_ptr[num_scen] - edit_ptr[0];
    const int64_t na = absent_ptr[num_scen] - absent_ptr[0];
    if (ne < 0 || na < 0 || ne > std::numeric_limits<int>::max() - 1 ||
        (ne > 0 && (!edit_links || !edit_fft || !edit_alpha || !edit_beta)) ||
        (na > 0 && !absent_links)) {
      tapgpu::set_message("bad link-record scenario arrays");
      return TAPGPU_ERR_ARG;
    }
    for (int s = 0; s < num_scen; ++s) {
      if (edit_ptr[s + 1] < edit_ptr[s] || absent_ptr[s + 1] < absent_ptr[s]) {
        tapgpu::set_message("link-record scenario offsets not monotone");
        return TAPGPU_ERR_ARG;
      }
      for (int64_t i = edit_ptr[s]; i < edit_ptr[s + 1]; ++i) {
        if (edit_links[i] < 0 || edit_links[i] >= M || !(edit_fft[i] >= 0) ||
            !std::isfinite(edit_fft[i]) || !(edit_alpha[i] >= 0) ||
            !std::isfinite(edit_alpha[i]) || !std::isfinite(edit_beta[i])) {
          tapgpu::set_message("link-record edit " + std::to_string(i) +
                              " has a link out of range or an invalid cost parameter");
          return TAPGPU_ERR_ARG;
        }
      }
      for (int64_t i = absent_ptr[s]; i < absent_ptr[s + 1]; ++i)
        if (absent_links[i] < 0 || absent_links[i] >= M) {
          tapgpu::set_message("absent link index out of range");
          return TAPGPU_ERR_ARG;
        }
    }
  }
  TG_CUDA(cudaSetDevice(c->device));
  TG_CUDA(cudaStreamSynchronize(c->stream));
  void* olds[] = {c->sc_fft, c->sc_alpha, c->sc_beta, c->sc_ipow, c->sc_absent};
  for (void* p : olds) tapgpu::free_owned(c, p);
  c->sc_fft = c->sc_alpha = c->sc_beta = nullptr;
  c->sc_ipow = nullptr;
  c->sc_absent = nullptr;
  c->h_absent.clear();
  c->link_scen = 0;
  c->use_link_scen = false;
  if (c->gexec) {  // captured launches hold the old parameter pointers
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  c->g_nscen = -1;
  if (num_scen == 0) return TAPGPU_OK;

  std::vector<int64_t> inv(M);
  for (int k = 0; k < M; ++k) inv[c->perm[k]] = k;
  const int64_t ne = edit_ptr[num_scen] - edit_ptr[0];
  std::vector<int> eptr(num_scen + 1), elink(static_cast<size_t>(std::max<int64_t>(ne, 1)));
  std::vector<double> efft(elink.size()), ealpha(elink.size()), ebeta(elink.size());
  std::vector<unsigned char> eip(elink.size());
  int64_t j = 0;
  for (int s = 0; s < num_scen; ++s) {
    eptr[s] = static_cast<int>(j);
    for (int64_t i = edit_ptr[s]; i < edit_ptr[s + 1]; ++i, ++j) {
      elink[j] = static_cast<int>(inv[edit_links[i]]);
      efft[j] = edit_fft[i];
      ealpha[j] = edit_alpha[i];
      const double b = edit_beta[i];
      ebeta[j] = b;
      eip[j] = (b >= 0 && b <= 15 && std::floor(b) == b) ? static_cast<unsigned char>(b) : 255;
    }
  }
  eptr[num_scen] = static_cast<int>(j);
  const int words = (M + 31) / 32;
  c->h_absent.assign(static_cast<size_t>(num_scen) * words, 0u);
  for (int s = 0; s < num_scen; ++s)
    for (int64_t i = absent_ptr[s]; i < absent_ptr[s + 1]; ++i) {
      const int k = static_cast<int>(inv[absent_links[i]]);
      c->h_absent[static_cast<size_t>(s) * words + (k >> 5)] |= 1u << (k & 31);
    }
  const size_t rows = static_cast<size_t>(num_scen) * M;
  TG_TRY(c->alloc_n(&c->sc_fft, rows));
  TG_TRY(c->alloc_n(&c->sc_alpha, rows));
  TG_TRY(c->alloc_n(&c->sc_beta, rows));
  TG_TRY(c->alloc_n(&c->sc_ipow, rows));
  TG_TRY(c->alloc_n(&c->sc_absent, c->h_absent.size()));
  int* d_ptr = nullptr;
  int* d_link = nullptr;
  double* d_val = nullptr;
  unsigned char* d_ip = nullptr;
  TG_TRY(c->alloc_n(&d_ptr, eptr.size()));
  TG_TRY(c->alloc_n(&d_link, elink.size()));
  TG_TRY(c->alloc_n(&d_val, 3 * elink.size()));
  TG_TRY(c->alloc_n(&d_ip, elink.size()));
  const size_t ns = elink.size();
  int rc = TAPGPU_OK;
  if (cudaMemcpy(d_ptr, eptr.data(), sizeof(int) * eptr.size(), cudaMemcpyHostToDevice) ||
      cudaMemcpy(d_link, elink.data(), sizeof(int) * ns, cudaMemcpyHostToDevice) ||
      cudaMemcpy(d_val, efft.data(), sizeof(double) * ns, cudaMemcpyHostToDevice) ||
      cudaMemcpy(d_val + ns, ealpha.data(), sizeof(double) * ns, cudaMemcpyHostToDevice) ||
      cudaMemcpy(d_val + 2 * ns, ebeta.data(), sizeof(double) * ns, cudaMemcpyHostToDevice) ||
      cudaMemcpy(d_ip, eip.data(), ns, cudaMemcpyHostToDevice) ||
      cudaMemcpy(c->sc_absent, c->h_absent.data(), sizeof(unsigned) * c->h_absent.size(),
                 cudaMemcpyHostToDevice) ||
      tapgpu::launch_param_rows(c->sc_fft, c->fft, M, num_scen, d_ptr, d_link, d_val,
                                c->link_grid, c->stream) ||
      tapgpu::launch_param_rows(c->sc_alpha, c->alpha, M, num_scen, d_ptr, d_link, d_val + ns,
                                c->link_grid, c->stream) ||
      tapgpu::launch_param_rows(c->sc_beta, c->beta, M, num_scen, d_ptr, d_link, d_val + 2 * ns,
                                c->link_grid, c->stream) ||
      tapgpu::launch_param_rows(c->sc_ipow, c->ipow, M, num_scen, d_ptr, d_link, d_ip,
                                c->link_grid, c->stream) ||
      cudaStreamSynchronize(c->stream)) {
    tapgpu::set_message(std::string("link-record scenario rows: ") +
                        cudaGetErrorString(cudaGetLastError()));
    rc = TAPGPU_ERR_CUDA;
  }
  void* tmp[] = {d_ptr, d_link, d_val, d_ip};
  for (void* p : tmp) tapgpu::free_owned(c, p);
  if (rc != TAPGPU_OK) return rc;
  c->absent_words = words;
  c->link_scen = num_scen;
  return TAPGPU_OK;
}

static int to_device_weights(Ctx* c, const double* weights) {
  std::vector<double> w(c->M);
  std::vector<uint2> wf(c->M), wr(c->M);
  for (int k = 0; k < c->M; ++k) {
    const double v = weights[c->perm[k]];
    if (!(v >= 0) || std::isinf(v)) {
      tapgpu::set_message("link costs must be finite and non-negative");
      return TAPGPU_ERR_ARG;
    }
    w[k] = v;
    const float f = static_cast<float>(v);
    unsigned bits;
    std::memcpy(&bits, &f, sizeof bits);
    wf[k] = make_uint2(static_cast<unsigned>(c->h_head[k]), bits);
    wr[c->h_rpos[k]] = make_uint2(static_cast<unsigned>(c->h_tail[k]), bits);
  }
  {
    double s = 0.0;
    for (int k = 0; k < c->M; ++k) s += w[k];
    const double mean = s / c->M;
    c->api_nf_delta = c->opt.nf_delta > 0 ? c->opt.nf_delta : (mean > 0 ? 16.0 * mean : 1.0);
  }
  TG_CUDA(cudaMemcpyAsync(c->api_r32, wr.data(), sizeof(uint2) * c->M, cudaMemcpyHostToDevice,
                          c->stream));
  TG_CUDA(cudaMemcpyAsync(c->api_w64, w.data(), sizeof(double) * c->M, cudaMemcpyHostToDevice,
                          c->stream));
  TG_CUDA(cudaMemcpyAsync(c->api_e32, wf.data(), sizeof(uint2) * c->M, cudaMemcpyHostToDevice,
                          c->stream));
  std::vector<uint2> w4(static_cast<size_t>(c->n1) * 4, make_uint2(0u, 0u));
  for (int k = 0; k < c->M; ++k)
    if (c->h_ell_pos[k] >= 0) w4[c->h_ell_pos[k]] = make_uint2(c->h_e4x[k], wf[k].y);
  TG_CUDA(cudaMemcpyAsync(c->api_e4, w4.data(), sizeof(uint2) * w4.size(), cudaMemcpyHostToDevice,
                          c->stream));
  TG_CUDA(cudaStreamSynchronize(c->stream));
  return TAPGPU_OK;
}

int tapgpu_sssp(tapgpu_ctx* ctx, const double* weights, const int64_t* srcs, int64_t num_sources,
                double* dist, int64_t* pred) {
  if (!ctx || !weights || (num_sources > 0 && !srcs)) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  for (int64_t i = 0; i < num_sources; ++i)
    if (srcs[i] < 0 || srcs[i] >= c->n1) {
      tapgpu::set_message("source node out of range");
      return TAPGPU_ERR_ARG;
    }
  TG_CUDA(cudaSetDevice(c->device));
  TG_TRY(to_device_weights(c, weights));
  const int n1 = c->n1;
  if (!c->pred_buf) TG_TRY(c->alloc_n(&c->pred_buf, static_cast<size_t>(c->dist_tasks) * n1));
  int* dsrc = nullptr;
  // FP64 labels: a FP32 context's label buffer holds half as many sources
  const int64_t chunk = c->fp64 ? c->dist_tasks : std::max<int64_t>(1, c->dist_tasks / 2);
  TG_TRY(c->alloc_n(&dsrc, static_cast<size_t>(std::max<int64_t>(1, std::min(chunk, num_sources)))));
  std::vector<double> dtmp;
  std::vector<float> ftmp;
  std::vector<int> ptmp;
  int rc = TAPGPU_OK;
  // the API always computes FP64 labels: they equal the reference's bit for bit
  for (int64_t s0 = 0; s0 < num_sources && rc == TAPGPU_OK; s0 += chunk) {
    const int64_t s1 = std::min(num_sources, s0 + chunk);
    const int ns = static_cast<int>(s1 - s0);
    std::vector<int> hs(ns);
    for (int i = 0; i < ns; ++i) hs[i] = static_cast<int>(srcs[s0 + i]);
    if (cudaMemcpyAsync(dsrc, hs.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, c->stream) !=
        cudaSuccess) {
      rc = TAPGPU_ERR_CUDA;
      break;
    }
    tapgpu::PathArgs a = c->path_args(1);
    a.sources = dsrc;
    a.num_sources = ns;
    a.scen_list = nullptr;
    a.state = nullptr;
    a.task_begin = 0;
    a.task_end = ns;
    a.w64 = c->api_w64;
    a.e32 = nullptr;
    a.r4 = nullptr;
    a.r4d = nullptr;
    a.aon_c64 = 0;
    a.do_load = 0;
    a.pred_out = c->pred_buf;
    a.y_fx = c->api_yfx;
    a.nf_delta = c->api_nf_delta;
    const int optin = tapgpu::max_smem_optin(c->device);
    const bool s_smem = tapgpu::sssp_smem_bytes(n1, true, c->sssp_variant, c->M) + 1024 <= static_cast<size_t>(optin);
    const int occ = tapgpu::sssp_occupancy(true, c->sssp_block, s_smem, n1, c->sssp_variant, c->M,
                                           c->opt.global_scratch == 2);
    int grid = std::max(1, std::min(occ * c->num_sms, ns));
    if (!s_smem) {
      const size_t need = tapgpu::sssp_smem_bytes(n1, true, c->sssp_variant, c->M) * static_cast<size_t>(grid);
      if (need > c->path_scratch_bytes) {
        grid = std::max<int>(1, static_cast<int>(c->path_scratch_bytes / tapgpu::sssp_smem_bytes(n1, true, c->sssp_variant, c->M)));
        if (c->path_scratch_bytes == 0) {
          rc = TAPGPU_ERR_UNSUPPORTED;
          break;
        }
      }
    }
    cudaMemsetAsync(c->counters, 0, 2 * sizeof(int), c->stream);
    a.counter = c->counters;
    a.scratch_stride = static_cast<long long>(tapgpu::sssp_smem_bytes(n1, true, c->sssp_variant, c->M));
    if (tapgpu::launch_sssp(a, true, grid, c->sssp_block, s_smem, c->sssp_variant, c->stream) !=
        cudaSuccess) {
      rc = TAPGPU_ERR_CUDA;
      break;
    }
    a.counter = c->counters + 1;
    // FP64 labels: the 16-byte-per-node loading layout, whatever the context's
    const size_t abytes = tapgpu::aon_smem_bytes(n1, true);
    const bool a_smem = abytes + 1024 <= static_cast<size_t>(optin) && !c->opt.global_scratch;
    int agrid = std::max(1, std::min(tapgpu::aon_occupancy(true, c->aon_block, a_smem, n1) *
                                         c->num_sms, ns));
    if (!a_smem) {
      agrid = std::min<int>(agrid, static_cast<int>(c->path_scratch_bytes / abytes));
      if (agrid < 1) {
        rc = TAPGPU_ERR_UNSUPPORTED;
        break;
      }
    }
    a.scratch_stride = static_cast<long long>(abytes);
    if (tapgpu::launch_aon(a, true, agrid, c->aon_block, a_smem, c->stream) != cudaSuccess) {
      rc = TAPGPU_ERR_CUDA;
      break;
    }
    rc = c->sync_check();
    if (rc != TAPGPU_OK) break;
    if (dist) {
      dtmp.resize(static_cast<size_t>(ns) * n1);
      if (cudaMemcpy(dtmp.data(), c->dist, sizeof(double) * dtmp.size(), cudaMemcpyDeviceToHost) !=
          cudaSuccess) {
        rc = TAPGPU_ERR_CUDA;
        break;
      }
      for (size_t i = 0; i < dtmp.size(); ++i)
        dist[static_cast<size_t>(s0) * n1 + i] = std::isinf(dtmp[i]) ? DBL_MAX : dtmp[i];
    }
    if (pred) {
      ptmp.resize(static_cast<size_t>(ns) * n1);
      if (cudaMemcpy(ptmp.data(), c->pred_buf, sizeof(int) * ptmp.size(), cudaMemcpyDeviceToHost) !=
          cudaSuccess) {
        rc = TAPGPU_ERR_CUDA;
        break;
      }
      for (size_t i = 0; i < ptmp.size(); ++i)
        pred[static_cast<size_t>(s0) * n1 + i] = ptmp[i] >= 0 ? c->perm[ptmp[i]] : -1;
    }
  }
  tapgpu::free_owned(c, dsrc);
  if (rc == TAPGPU_ERR_CUDA && tapgpu::g_message.empty())
    tapgpu::set_message(cudaGetErrorString(cudaGetLastError()));
  return rc;
}

int tapgpu_aon(tapgpu_ctx* ctx, const double* weights, double* volume) {
  if (!ctx || !weights || !volume) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  TG_CUDA(cudaSetDevice(c->device));
  TG_TRY(to_device_weights(c, weights));
  TG_CUDA(cudaMemsetAsync(c->api_yfx, 0, sizeof(unsigned long long) * c->M, c->stream));
  TG_CUDA(cudaMemsetAsync(c->err, 0, sizeof(int), c->stream));
  const double solver_delta = c->nf_delta;
  c->nf_delta = c->api_nf_delta;
  const int rc = c->enqueue_paths(1, true, c->fp64 ? nullptr : c->api_e32,
                                  c->fp64 ? nullptr : c->api_r32, c->fp64 ? c->api_w64 : nullptr,
                                  c->api_yfx, false);
  c->nf_delta = solver_delta;
  TG_TRY(rc);
  TG_TRY(c->sync_check());
  std::vector<unsigned long long> y(c->M);
  TG_CUDA(cudaMemcpy(y.data(), c->api_yfx, sizeof(unsigned long long) * c->M,
                     cudaMemcpyDeviceToHost));
  for (int k = 0; k < c->M; ++k)
    volume[c->perm[k]] = static_cast<double>(static_cast<long long>(y[k])) * c->inv_scale;
  return TAPGPU_OK;
}

void* tapgpu_stream(tapgpu_ctx* ctx) { return ctx ? ctx->c->stream : nullptr; }

int tapgpu_run_iterations(tapgpu_ctx* ctx, int iters) {
  if (!ctx || iters < 1) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  TG_CUDA(cudaSetDevice(c->device));
  const int S = c->last_nscen;
  std::vector<tapgpu::ScenState> st;
  TG_TRY(c->read_states(S, st));
  for (auto& s : st) {
    s.done = 0;
    s.max_iters = s.iter + iters;
    s.target_relgap = 0.0;
  }
  TG_CUDA(cudaMemcpyAsync(c->state, st.data(), sizeof(tapgpu::ScenState) * S,
                          cudaMemcpyHostToDevice, c->stream));
  std::vector<int> all(S);
  std::iota(all.begin(), all.end(), 0);
  if (c->h_scen_list != all) {
    TG_CUDA(cudaMemcpyAsync(c->scen_list, all.data(), sizeof(int) * S, cudaMemcpyHostToDevice,
                            c->stream));
    c->h_scen_list = all;
  }
  int per = c->opt.iters_per_launch > 0 ? c->opt.iters_per_launch : 8;
  for (int done = 0; done < iters;) {
    const int n = std::min(per, iters - done);
    TG_TRY(c->run_graph(n, S));
    done += n;
  }
  return TAPGPU_OK;
}

int tapgpu_set_timing(tapgpu_ctx* ctx, int on) {
  if (!ctx) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  TG_CUDA(cudaSetDevice(c->device));
  TG_CUDA(cudaStreamSynchronize(c->stream));
  if (c->gexec) {
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  c->timing = on != 0;
  c->timed.clear();
  c->ev_used = 0;
  for (int i = 0; i < 4; ++i) {
    c->kt_ms[i] = 0.0;
    c->kt_n[i] = 0;
  }
  c->launches = 0;
  TG_CUDA(cudaMemset(c->path_stats, 0, 8 * sizeof(unsigned long long)));
  return TAPGPU_OK;
}

int tapgpu_get_path_stats(tapgpu_ctx* ctx, int64_t* out) {
  if (!ctx || !out) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  TG_CUDA(cudaSetDevice(c->device));
  TG_CUDA(cudaStreamSynchronize(c->stream));
  unsigned long long v[6];
  TG_CUDA(cudaMemcpy(v, c->path_stats, sizeof(v), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 6; ++i) out[i] = static_cast<int64_t>(v[i]);
  return TAPGPU_OK;
}

int tapgpu_get_timing(tapgpu_ctx* ctx, double* ms, int64_t* counts, int64_t* kernel_launches) {
  if (!ctx) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  TG_CUDA(cudaSetDevice(c->device));
  TG_CUDA(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < 4; ++i) {
    if (ms) ms[i] = c->kt_ms[i];
    if (counts) counts[i] = c->kt_n[i];
  }
  if (kernel_launches) *kernel_launches = c->launches;
  return TAPGPU_OK;
}

int tapgpu_profile_iteration(tapgpu_ctx* ctx, int reps, float* ms) {
  if (!ctx || !ms || reps < 1) return TAPGPU_ERR_ARG;
  Ctx* c = ctx->c;
  TG_CUDA(cudaSetDevice(c->device));
  std::vector<tapgpu::ScenState> st;
  TG_TRY(c->read_states(1, st));
  st[0].done = 0;
  st[0].max_iters = 0;
  st[0].target_relgap = 0.0;
  TG_CUDA(cudaMemcpyAsync(c->state, st.data(), sizeof(tapgpu::ScenState), cudaMemcpyHostToDevice,
                          c->stream));
  std::vector<int> one{0};
  TG_CUDA(cudaMemcpyAsync(c->scen_list, one.data(), sizeof(int), cudaMemcpyHostToDevice, c->stream));
  c->h_scen_list = one;
  cudaEvent_t ev[5];
  for (auto& e : ev) TG_CUDA(cudaEventCreate(&e));
  double acc[5] = {0, 0, 0, 0, 0};
  int rc = TAPGPU_OK;
  for (int r = 0; r < reps && rc == TAPGPU_OK; ++r) {
    cudaEventRecord(ev[0], c->stream);
    const int64_t tasks = c->Z;
    tapgpu::PathArgs a = c->path_args(1);
    a.task_end = static_cast<int>(tasks);
    cudaMemsetAsync(c->counters, 0, 2 * sizeof(int), c->stream);
    a.counter = c->counters;
    a.scratch_stride = static_cast<long long>(tapgpu::sssp_smem_bytes(c->n1, c->fp64, c->sssp_variant, c->M));
    a.e32 = c->fp64 ? nullptr : c->e32;
    a.r32 = c->fp64 ? nullptr : c->r32;
    a.w64 = c->fp64 ? c->w64 : nullptr;
    if (tasks > c->dist_tasks) {
      rc = TAPGPU_ERR_UNSUPPORTED;
      break;
    }
    tapgpu::launch_sssp(a, c->fp64, std::min<int64_t>(c->sssp_grid, tasks), c->sssp_block,
                        c->sssp_smem, c->sssp_variant, c->stream);
    cudaEventRecord(ev[1], c->stream);
    a.counter = c->counters + 1;
    a.scratch_stride = static_cast<long long>(tapgpu::aon_smem_bytes(c->n1, c->fp64, c->aon_c64));
    tapgpu::launch_aon(a, c->fp64, std::min<int64_t>(c->aon_grid, tasks), c->aon_block,
                       c->aon_smem, c->stream);
    cudaEventRecord(ev[2], c->stream);
    tapgpu::LinkArgs la = c->link_args(1);
    for (int p = 0; p < tapgpu::kLsPasses; ++p) {
      la.pass = p;
      tapgpu::launch_ls_pass(la, c->ls_grid(1), c->ls_block, c->stream);
    }
    tapgpu::launch_ls_fallback(la, c->stream);
    cudaEventRecord(ev[3], c->stream);
    tapgpu::launch_step(la, c->ls_link_grid, c->ls_block, c->stream);
    cudaEventRecord(ev[4], c->stream);
    if (cudaEventSynchronize(ev[4]) != cudaSuccess) {
      rc = TAPGPU_ERR_CUDA;
      break;
    }
    float t;
    for (int i = 0; i < 4; ++i) {
      cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
      acc[i] += t;
    }
    cudaEventElapsedTime(&t, ev[0], ev[4]);
    acc[4] += t;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc != TAPGPU_OK) return rc;
  TG_TRY(c->sync_check());
  for (int i = 0; i < 5; ++i) ms[i] = static_cast<float>(acc[i] / reps);
  return TAPGPU_OK;
}

}  // extern "C"
