// fw_kernels.cuh - device data layout and kernel entry points of the GB300
// Frank-Wolfe user-equilibrium solver.
//
// Layout in HBM (one network, S scenarios):
//   forward star   row_ptr[n1+1], head[m]            (n1 = N+1 rows, row 0 unused)
//   reverse star   in_ptr[n1+1], in_link[m]          (in-links of a node by link id)
//   link table     tail[m], fft/alpha/beta[m] f64, ipow[m] u8 (integer BPR power)
//   per scenario   cap[S][m], x[S][m], t[S][m], d[S][m] f64, y_fx[S][m] u64,
//                  w32[S][m] f32 or w64[S][m] f64 (shortest-path weights)
//   demand         CSR over source slots: od_ptr[Z+1], od_dest, od_q (fixed point)
//   scratch        dist[chunk][n1] (f32 or f64) between the two path kernels
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tapgpu {

constexpr int kLsPerPass = 12;   // line-search candidates 2^-k evaluated per pass
constexpr int kLsPasses = 5;     // passes captured per iteration (k up to 60)
constexpr int kLsMaxHalvings = 1000;  // tap/tap_functions.c:472
constexpr int kNumSums = 4 + kLsPerPass;  // g0, vht, obj, g(1), g(2^-j) ...
constexpr int kTraceCols = 8;    // obj, relgap, avg_excess, vht, lambda, gap, iter, g0

// error bits written to the device error word
enum : int {
  kErrRounds = 1,      // shortest-path rounds exceeded the node-count bound
  kErrNoPath = 2,      // positive demand with an unreachable destination
  kErrWalk = 4,        // predecessor walk longer than the node count
  kErrPending = 8,     // predecessor tree could not be completed
  kErrLineSearch = 16, // no step found within the halving cap
};

struct Graph {
  int n1, m, first_thru;
  const int* row_ptr;
  const int* head;
  const int* tail;
  const int* in_ptr;
  const int* in_link;
  const int* in_head;  // head node of each reverse-star slot
  const int* out_deg;  // out-degree of each node
};

struct LinkParams {
  const double* fft;
  const double* alpha;
  const double* beta;
  const unsigned char* ipow;  // 0..15: integer power; 255: use pow()
  long long stride;           // 0: one row for every scenario; m: row [scenario][m]
};

struct ScenState {
  int iter;        // FW iterations completed
  int done;        // 1 once the stopping rule holds
  int ls_pending;  // line search still searching
  int ls_next;     // next halving exponent to test
  int max_iters;   // <= 0: no cap
  int pad0, pad1, pad2;
  double target_relgap;
  double relgap, best_lb, obj, gap, lambda, vht, avg_excess, g0;
  double vht_end;  // VHT at the current x with the current costs
  double ls_lo, ls_hi, ls_glo, ls_ghi;  // exact line search: bracket of the root of g
};

// line-search modes
enum : int {
  kLsReference = 0,  // largest 2^-k with g(2^-k) <= 0 (tap/tap_functions.c:469-507)
  kLsExact = 1,      // root of g on [0, 1] (differentiable: used by the adjoint)
};
constexpr int kLsExactPasses = 14;  // bracket shrinks 13x per pass

struct Demand {
  const int* od_ptr;            // [num_sources+1]
  const int* od_dest;           // destination node
  const long long* od_q;        // demand in fixed point (2^-scale_bits units)
  long long q_stride;           // entries per scenario in od_q (0: one demand for all)
  const double* od_dem;         // demand as given (for the no-path check)
  double inv_scale;             // 2^-scale_bits
  double total;                 // total demand (tap/tap_functions.c:377-386)
};

struct PathArgs {
  Graph g;
  const uint2* e32;             // [S][m] {head, f32 weight bits} when fp32 paths
  const uint2* e4;              // [S][n1][4] the first four records of each node, or nullptr
  const uint2* r32;             // [S][m] {tail, f32 weight bits} in reverse-star order
  const uint2* r4;              // [S][n1][4] the first four in-link records of each node
                                //     {link << 16 | tail, f32 weight bits} (unused: +inf
                                //     weight), or nullptr
  const unsigned* r4_more;      // [ceil(n1/32)] bit v: node v has more than four in-links
  const uint4* r4d;             // [S][n1][4] FP64 paths: the first four in-link records of each
                                //     node {link, tail, f64 weight} (unused: +inf), or nullptr
  int aon_c64;                  // FP64 loading in the compact layout (with r4d)
  const double* w64;            // [S][m] when fp64 paths
  const int* sources;           // source nodes
  int num_sources;
  const int* scen_list;         // scenario of each task block (nullptr: scenario 0)
  const ScenState* state;       // skip tasks of finished scenarios (nullptr: never)
  int task_begin, task_end;     // task t: scenario scen_list[t / num_sources],
                                //         source sources[t % num_sources]
  void* dist;                   // [(t - task_begin)][n1]
  int* counter;                 // work counter, zero before launch
  int* err;                     // error bits
  int* err_info;                // [2]: origin, destination of a missing path
  int max_rounds;
  // all-or-nothing only
  Demand dem;
  unsigned long long* y_fx;     // [S][m]
  int* pred_out;                // [(t - task_begin)][n1] predecessor links, optional
  int do_load;                  // 0: predecessors only
  void* scratch;                // per-CTA global scratch when the smem variant does not fit
  long long scratch_stride;     // bytes per CTA
  int all_global;               // global scratch: the queue kernels' bitmaps and ring too
  unsigned long long* stats;    // optional [4]: rounds, tasks, node expansions, -
  double nf_delta;              // near-far threshold step (label units)
};

struct LinkArgs {
  int m;
  int num_scen;                 // scenarios in the launch (grid.y)
  const int* scen_list;         // grid.y -> scenario id (nullptr: identity)
  LinkParams lp;
  const double* cap;            // [S][m]
  double* x;                    // [S][m]
  double* t;                    // [S][m]
  double* d;                    // [S][m]
  unsigned long long* y_fx;     // [S][m]
  uint2* e32;                   // [S][m] packed fp32 edge records, or nullptr
  uint2* e4;                    // [S][n1][4] first four records of each node, or nullptr
  const int* ell_pos;           // [m] slot of link k in its tail's four (-1: beyond the fourth)
  const unsigned* e4x;          // [m] first word of link k's padded record: its head, with the
                                //     tail's out-degree in the upper 16 bits (16-bit queue ring)
  int n1;
  uint2* r32;                   // [S][m] packed fp32 reverse records (with e32)
  uint2* r4;                    // [S][n1][4] first four in-link records of each node, or nullptr
  uint4* r4d;                   // [S][n1][4] the same for FP64 paths {link, tail, weight}, or nullptr
  const int* r4_pos;            // [m] slot of link k among its head's four (-1: beyond the fourth)
  const unsigned* r4x;          // [m] first word of link k's padded reverse record
  const int* head;              // [m] head node of each link (for e32)
  const int* tail;              // [m] tail node of each link (for r32)
  const int* rpos;              // [m] reverse-star slot of each link (for r32)
  double* w64;                  // [S][m] or nullptr
  double* dtdx;                 // [S][m] or nullptr (derivative of the BPR cost)
  double* partials;             // [S][gridDim.x][kNumSums]
  unsigned int* arrive;         // [S] block arrival counters
  ScenState* state;             // [S]
  double* trace;                // [S][trace_cap][kTraceCols] or nullptr
  int trace_cap;
  double inv_scale;             // fixed point -> volume
  double total_demand;
  const double* total_demand_s; // [S] per-scenario totals (demand scenarios) or null
  int pass;                     // line-search pass index
  int* err;
  double* x_hist;               // [S][hist_cap / ckpt_every + 1][m] flows at checkpoints
  double* d_hist;               // [S][hist_cap][m] directions (adjoint tape)
  double* lam_hist;             // [S][hist_cap]
  int hist_cap;
  int ckpt_every;               // flows kept every ckpt_every iterations
  int ls_mode;                  // kLsReference or kLsExact
  int ls_ratio;                 // FP32-path mode: candidates from x/c + lambda d/c (one division)
  const unsigned* absent;       // [S][absent_words] links not in a scenario's network, or null
  int absent_words;             // 32-bit words per scenario of `absent`
};

// launch helpers (implemented in fw_kernels.cu)
// (m: links, used by the small-network variant, whose edge list is held too)
size_t sssp_smem_bytes(int n1, bool fp64, int variant = 0, int m = 0);
// The queue kernels with labels in global memory keep their near/far bitmaps
// and ring in shared memory (these bytes) while they fit.
size_t nfq_split_smem_bytes(int n1, int variant);
bool nfq_split(int n1, int variant);
// c64: FP64 labels in the compact layout (predecessor words in the label slot)
size_t aon_smem_bytes(int n1, bool fp64, bool c64 = false);
bool aon_compact(int n1, bool fp64);  // 10-byte-per-node loading layout
int max_smem_optin(int device);
// shortest-path kernel variants
enum : int {
  kSsspRounds = 1,  // bulk-synchronous label-correction rounds (k_sssp)
  kSsspAsync = 2,   // warp-owned frontier words, no per-round barrier (k_sssp_async)
  kSsspNearFar = 3, // asynchronous near set below a rising threshold (k_sssp_nf)
  kSsspNearFarQueue = 4,  // near-far with a FIFO ring of near nodes (k_sssp_nfq)
  kSsspNearFarQueueWide = 5,  // the same with 32-bit ring entries (chosen above 65535 nodes)
  kSsspSmall = 6,   // Bellman-Ford sweeps over the edge list in shared memory (k_sssp_small;
                    // chosen for networks of at most kSmallNet nodes and links)
};
constexpr int kSmallNet = 4096;
// links up to which one block per scenario runs an iteration's line search
// and step (above it the multi-block passes spread the FP64 work over SMs)
constexpr int kSmallTail = 512;
constexpr int kQueueSlots = 1024;  // ring slots of k_sssp_nfq
cudaError_t launch_sssp(const PathArgs& a, bool fp64, int grid, int block, bool smem,
                        int variant, cudaStream_t s);
cudaError_t launch_aon(const PathArgs& a, bool fp64, int grid, int block, bool smem,
                       cudaStream_t s);
// x = loaded volumes (a.pass == 0) or x as given (a.pass == 1); t = BPR(x); weights; state reset
cudaError_t launch_init_flows(const LinkArgs& a, int grid, cudaStream_t s);
// weights = free-flow times and y_fx = 0 (first all-or-nothing)
cudaError_t launch_set_costs(const LinkArgs& a, int grid, cudaStream_t s);
// line-search passes and the step: `block` kSmallLinkBlock (networks of at
// most kSmallNet links, FP64 work over more SMs) or kLinkBlock
constexpr int kSmallLinkBlock = 64;
cudaError_t launch_ls_pass(const LinkArgs& a, int grid, int block, cudaStream_t s);
cudaError_t launch_ls_fallback(const LinkArgs& a, cudaStream_t s);
cudaError_t launch_step(const LinkArgs& a, int grid, int block, cudaStream_t s);
// small networks (at most kSmallTail links): every line-search pass, the
// fallback and the step in one launch (one block per scenario)
cudaError_t launch_fw_tail_small(const LinkArgs& a, cudaStream_t s);
// capacity rows [nscen][m] = base with each scenario's edits (see fw_kernels.cu)
cudaError_t launch_scenario_caps(double* cap, const double* base, int m, int nscen, const int* ptr,
                                 const int* link, const double* val, const double* min_pos,
                                 int grid, cudaStream_t s);
// parameter rows [nscen][m] = base with each scenario's edits (ptr [nscen+1], link, val)
cudaError_t launch_param_rows(double* rows, const double* base, int m, int nscen, const int* ptr,
                              const int* link, const double* val, int grid, cudaStream_t s);
cudaError_t launch_param_rows(unsigned char* rows, const unsigned char* base, int m, int nscen,
                              const int* ptr, const int* link, const unsigned char* val, int grid,
                              cudaStream_t s);
// rows 1 .. nscen-1 of x [nscen][m] become copies of row 0
cudaError_t launch_replicate_rows(double* x, int m, int nscen, int grid, cudaStream_t s);
cudaError_t launch_fill_records(uint2* p, size_t n, uint2 val, int grid, cudaStream_t s);
cudaError_t launch_fill_records4(uint4* p, size_t n, uint4 val, int grid, cudaStream_t s);
int sssp_occupancy(bool fp64, int block, bool smem, int n1, int variant, int m = 0,
                   bool all_global = false);  // CTAs per SM
int aon_occupancy(bool fp64, int block, bool smem, int n1, bool c64 = false);

}  // namespace tapgpu
