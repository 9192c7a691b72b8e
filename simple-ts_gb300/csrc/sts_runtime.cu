// Device context, set-up sequence, step orchestration (CUDA graph with
// conditional WHILE nodes) and the C ABI of libsts_gb300.so.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <memory>
#include <mutex>
#include <tuple>
#include <algorithm>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

#include "sts_checkpoint.h"
#include "sts_common.cuh"
#include "sts_host.h"
#include "sts_kernels.h"
#include "sts_unet.h"
#include "sts_warmnet.h"
#include "../../include/sts_gb300.h"

using namespace sts;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CU(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(STS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));    \
  } while (0)

// kernel kinds reported by sts_profile_steps
constexpr int kProfileKinds = 8;
// threads per CTA of the fused boundary kernel (32, 64 and 128 measured slower: the wall entries
// gain nothing from more CTAs, and the last CTA's column and row phases run on fewer threads;
// 512 and 1024 slower too: 1200x120 FP64 0.3862 ms per step against 0.3875 and 0.3924)
constexpr int kBndThreads = 256;

}  // namespace

// The temperature-jump wall values read T, the cell density and static data; the slip walls
// and the velocity boundary phases write only u and v, and the pressure-begin phase writes p and
// the cell density on the inlet/outlet columns, and only with the ratio-corrected pressure
// condition (never in an x-periodic domain).  Unless that can meet a local-Kn jump (which reads
// the cell density), the jump values need nothing of those kernels and run beside them.
static bool tjump_beside_walls(uint64_t bits) {
  if (bits & F_PERIODIC) return true;
  return !((bits & F_KN_LOCAL) && (bits & F_PRESSURE_BC) && (bits & F_RATIO_CORRECT));
}

struct sts_ctx {
  Case hc;
  Geo g{};
  Ctl* d_ctl = nullptr;
  Ctl* h_ctl = nullptr;  // pinned mirror
  cudaStream_t s = nullptr;
  sts_options opt{};
  std::vector<void*> allocs;
  dim3 grid, block;
  bool finished = false;
  // graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // the same step without the WHILE node over steps, for launches of one step
  cudaGraph_t graph1 = nullptr;
  cudaGraphExec_t exec1 = nullptr;
  // the one-step graph of sts_step_exchange: the state comes in from host buffers in the first
  // kernel (node n_xin) and goes out to host buffers beside the flux kernel (node n_xout); their
  // buffers are set before every launch
  cudaGraph_t graph1x = nullptr;
  cudaGraphExec_t exec1x = nullptr;
  cudaGraphNode_t n_xin = nullptr, n_xout = nullptr;
  unsigned long long h_step = 0, h_outer = 0;
  // the sweep loop's grid barrier and the case's 32x8 tiles
  LoopCtl* d_lc = nullptr;
  int ntiles = 0;
  bool in_batch = false;  // stepped by an sts_batch, not by sts_step
  std::chrono::steady_clock::time_point t0;
  bool tmp_fresh = true, iter_fresh = true;
  // diagnostics (WriteDragCoefficient, SolveContinuityEquation): the cells of every flagged
  // body with a fluid neighbour in the reference's loop order, the sums, the continuity dumps
  std::vector<int> drag_bodies;  // body index (0-based id) of each list
  int* d_drag_cells = nullptr;
  int* d_drag_first = nullptr;
  double* d_drag_out = nullptr;
  double *d_cont_st = nullptr, *d_cont = nullptr;
  // global conservation sums (made at the first sts_conservation call)
  double *d_cons_part = nullptr, *d_cons_rows = nullptr, *d_cons_out = nullptr;
  bool cd_fresh = true, pu_fresh = true;
  // checkpoint dumps (made at the first save)
  std::unique_ptr<Checkpointer> saver;
  // warm_start 5: the network's correction of the stencil's start (sts_warmnet.cu); the device
  // runs warm_start 4 and these kernels follow the stencil's
  bool warm_net = false;
  std::unique_ptr<UNet> net;
  NetState* d_ns = nullptr;
  NetBuffers nb{};
  int net_slots = 0;
  static constexpr int kNetBatch = 8, kNetBase = 16, kNetLevels = 3;
  float *d_bx = nullptr, *d_bt = nullptr, *d_bw = nullptr, *d_loss = nullptr;
  int* d_bslots = nullptr;
  unsigned long long net_rng = 0x9E3779B97F4A7C15ull;
  cudaStream_t cap = nullptr;  // capture stream of the network's graph nodes

  ~sts_ctx() {
    saver.reset();  // writes out pending saves before the buffers and the stream go
    drop_graphs();
    for (void* p : allocs) cudaFree(p);
    if (h_ctl) cudaFreeHost(h_ctl);
    net.reset();
    if (cap) cudaStreamDestroy(cap);
    if (s) cudaStreamDestroy(s);
  }

  template <class T>
  int alloc(T** p, size_t n) {
    void* q = nullptr;
    CU(cudaMalloc(&q, sizeof(T) * (n ? n : 1)));
    CU(cudaMemsetAsync(q, 0, sizeof(T) * (n ? n : 1), s));
    allocs.push_back(q);
    *p = (T*)q;
    return STS_OK;
  }
  template <class T>
  int upload(T* dst, const std::vector<T>& src) {
    if (!src.empty()) CU(cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, s));
    return STS_OK;
  }
  int read_ctl() {
    CU(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    return STS_OK;
  }
  int check() {
    CU(cudaGetLastError());
    return STS_OK;
  }
  // launches
  void boundary(unsigned ph) { k_boundary<<<1, 1024, 0, s>>>(g, ph, 0, 0); }
  // the fused boundary kernel: one thread per slip-wall entry (and per jump entry when those
  // run beside the velocity and pressure phases)
  bool jump_beside() const { return tjump_beside_walls(g.bits); }
  dim3 bnd_grid() const {
    const int n = g.n_slip_u + g.n_slip_v + (jump_beside() ? g.n_tjump : 0);
    return dim3((unsigned)std::max(1, std::min((n + kBndThreads - 1) / kBndThreads, 4096)));
  }
  // boundary work and fluxes/diffusion of one outer iteration outside the graph; `mark`
  // (optional) brackets the launches for the per-kernel profile
  template <class M>
  void boundary_step(M mark) {
    mark(-1);
    k_bnd_fused<<<bnd_grid(), kBndThreads, 0, s>>>(g, 0ull, 0, jump_beside() ? 1 : 0, 0u);
    mark(5);
    mark(-1);
    flux_kernel()<<<grid, block, 0, s>>>(g, PH_TEMP | PH_PRES);
    mark(6);
  }
  // the learned warm starts' kernels after the start of a step (modes 3 and 4)
  template <class M>
  void warm_launches(M mark) {
    if (g.warm_start == 3) {
      mark(-1);
      k_warm_diff<<<grid, block, 0, s>>>(g);
      k_warm_fit<<<1, 576, 0, s>>>(g);
      k_warm_apply<<<grid, block, 0, s>>>(g);
      mark(0);
    }
  }
  // warm_start 4: the fit and the next step's start, once the step's iterate is final
  template <class M>
  void warm_train(M mark) {
    if (g.warm_start != 4) return;
    mark(-1);
    k_conv_gram<<<grid, block, 0, s>>>(g);
    k_conv_solve<<<2, kConvSolveThreads, 0, s>>>(g);
    k_conv_next<<<grid, block, 0, s>>>(g);
    k_conv_predict<<<grid, block, 0, s>>>(g);
    if (warm_net) net_tail(s);
    mark(0);
  }
  // warm_start 5: the network's kernels after the stencil's, on stream `st` (the context's stream,
  // or a stream that captures them into the step graph)
  void net_tail(cudaStream_t st) {
    const int px = nb.H * nb.W, b = (px + 255) / 256;
    k_net_target<<<b, 256, 0, st>>>(g, d_ns, nb);
    k_net_head<<<1, 1, 0, st>>>(g, d_ns, net_slots);
    k_net_locate<<<dim3((g.Nx + 255) / 256, g.Ny), 256, 0, st>>>(g, d_ns);
    k_net_gather<<<b, 256, 0, st>>>(g, d_ns, nb);
    k_net_commit<<<1, 1, 0, st>>>(g, d_ns, nb);
    net->set_stream(st);
    net->forward(nb.infer_in, 1, nb.infer_out);
    net->set_stream(s);
    k_net_apply<<<b, 256, 0, st>>>(g, d_ns, nb);
  }
  int net_setup(unsigned long long seed);
  bool fast() const { return g.precision >= 1; }
  bool mixed() const { return g.precision >= 2 && !(hc.bits & F_FIXED_SWEEPS); }
  // launch shapes (neither changes any result: every cell is computed on its own and the residual
  // reductions are maxima): the assembly kernel's block and the sweep loop's CTAs per SM, chosen
  // by the autotuner from the run's first steps
  dim3 asm_block{32, 8, 1};
  int sms = 0, pt_per_sm_max = 0, pt_per_sm = 0;  // pt_per_sm 0: as many as fit
  // per candidate: the fastest sample (per assembly launch, per sweep or sweep round), the most
  // robust of the samples against a step disturbed by something else
  struct TuneStat {
    double best = 1e30;
  };
  static constexpr int kTuneRounds = 3;
  int tune_left = 0, tune_idx = 0;
  std::vector<TuneStat> tune_pt, tune_asm;
  static dim3 asm_shape(int k) {
    static const dim3 shapes[3] = {dim3(32, 8), dim3(64, 4), dim3(128, 2)};
    return shapes[k];
  }
  int tune_step(int* done);
  void tune_choose();
  using AsmKernel = void (*)(Geo, unsigned long long, int);
  using FluxKernel = void (*)(Geo, unsigned);
  AsmKernel asm_kernel() const {
    return g.precision == 3 ? k_assemble_df : (fast() ? k_assemble_fast : k_assemble);
  }
  dim3 asm_grid() const {
    return dim3((g.Nx + asm_block.x - 1) / asm_block.x, (g.Ny + asm_block.y - 1) / asm_block.y, g.precision == 3 ? 3 : 1);
  }
  FluxKernel flux_kernel() const {
    return g.precision == 3 ? k_flux_diff_df : (fast() ? k_flux_diff_fast : k_flux_diff);
  }
  using CorrectKernel = void (*)(Geo);
  CorrectKernel correct_kernel() const { return g.precision == 3 ? k_correct_df : k_correct; }
  // the persistent sweep-loop kernel of this context and its grid (CTAs that fit at once)
  using PtKernel = void (*)(Geo, int, LoopCtl*);
  using PtKernelTB = void (*)(Geo, int, LoopCtl*, EMaps);
  PtKernel pt_kernel() const {
    if (mixed()) return g.precision == 3 ? k_pt_loop_mixed_df : k_pt_loop_mixed;
    return fast() ? k_pt_loop_fast : k_pt_loop;
  }
  // temporal blocking of the FP32-correction loop: pt_tb 2 runs two FP32 sweeps per tile load
  // (single cases); pt_tb_forced (sts_set_sweep_blocking) overrides the autotuner's choice
  EMaps emaps{};
  int pt_tb = 0, pt_tb_forced = 0;
  bool tb_available() const { return mixed() && !in_batch && g.eT[0] != nullptr; }
  bool tb_on() const { return pt_tb == 2 && tb_available(); }
  PtKernelTB pt_kernel_tb() const { return g.precision == 3 ? k_pt_loop_mixed_df_tb : k_pt_loop_mixed_tb; }
  const void* pt_func() const { return tb_on() ? (const void*)pt_kernel_tb() : (const void*)pt_kernel(); }
  dim3 pt_grid;
  int size_pt_grid() {
    int dev = 0, per_sm = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pt_func(), 256, 0));
    if (per_sm < 1) return fail(STS_ERR_CUDA, "the sweep-loop kernel does not fit on a multiprocessor");
    pt_per_sm_max = per_sm;
    const int use = (pt_per_sm > 0 && pt_per_sm <= per_sm) ? pt_per_sm : per_sm;
    pt_grid = dim3((unsigned)std::max(1, std::min(ntiles, use * sms)));
    return STS_OK;
  }
  // the sweep loop of one outer iteration outside the graph: one cooperative launch
  int pt_loop() {
    void* args[] = {(void*)&g, (void*)&ntiles, (void*)&d_lc, (void*)&emaps};
    CU(cudaLaunchCooperativeKernel(pt_func(), pt_grid, dim3(32, 8), args, 0, s));
    return STS_OK;
  }
  int make_emaps();
  int build_graph(bool loop, bool xout = false);
  // the step graphs are rebuilt at the next graph step
  void drop_graphs() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (exec1) cudaGraphExecDestroy(exec1);
    if (graph1) cudaGraphDestroy(graph1);
    if (exec1x) cudaGraphExecDestroy(exec1x);
    if (graph1x) cudaGraphDestroy(graph1x);
    exec = exec1 = exec1x = nullptr;
    graph = graph1 = graph1x = nullptr;
    n_xin = n_xout = nullptr;
  }
  // The state is final once the boundary kernel is done (the flux kernel and the end of the step
  // read it; only a time-dependent inflow writes u at the end of the step), so the state can go
  // out beside the flux kernel when the step's kernels sit at the top level of the graph.
  bool xout_in_graph() {
    return hc.cfg.n("N_I") == 1 && !warm_net && !(g.bits & F_U_BY_TIME);
  }
  int write_mesh();
  int write_drag();
  int continuity();
  int step_host(int n, int* done);
  int step_graph(int n, int* done, double* const* state_out = nullptr, const double* const* state_in = nullptr);
  int write_outputs(bool wait_files);
  int wait_outputs();
  int write_logs(bool iterations = true);
  int profile(int n, double* ms, int* cnt, int* done);
};

namespace {

// Adds a kernel node; the argument values are copied into the node.
template <class... P, class... A>
int add_kernel(cudaGraphNode_t* node, cudaGraph_t graph, const std::vector<cudaGraphNode_t>& deps, void (*f)(P...),
               dim3 grid, dim3 block, A... args) {
  std::tuple<P...> vals(args...);
  void* argv[sizeof...(P)];
  std::apply([&](auto&... x) {
    int k = 0;
    ((argv[k++] = (void*)&x), ...);
  }, vals);
  cudaKernelNodeParams p{};
  p.func = (void*)f;
  p.gridDim = grid;
  p.blockDim = block;
  p.sharedMemBytes = 0;
  p.kernelParams = argv;
  CU(cudaGraphAddKernelNode(node, graph, deps.data(), deps.size(), &p));
  return STS_OK;
}

// Sets the arguments of a kernel node of an instantiated graph (for its next launches).
template <class... P, class... A>
int set_kernel_args(cudaGraphExec_t exec, cudaGraphNode_t node, void (*f)(P...), dim3 grid, dim3 block, A... args) {
  std::tuple<P...> vals(args...);
  void* argv[sizeof...(P)];
  std::apply([&](auto&... x) {
    int k = 0;
    ((argv[k++] = (void*)&x), ...);
  }, vals);
  cudaKernelNodeParams p{};
  p.func = (void*)f;
  p.gridDim = grid;
  p.blockDim = block;
  p.sharedMemBytes = 0;
  p.kernelParams = argv;
  CU(cudaGraphExecKernelNodeSetParams(exec, node, &p));
  return STS_OK;
}

// A programmatic edge between two kernel nodes: `to` is launched as soon as every CTA of `from`
// has finished, and its kernel waits (wait_for_predecessor) for `from` to complete, writes
// visible, before it touches memory, so the launch of `to` overlaps the completion of `from`.
// (Launching `to` once every CTA of `from` has begun, cudaGraphKernelNodePortLaunchCompletion,
// measured slower: its waiting CTAs hold resources the predictor's kernels beside them need.)
constexpr unsigned char kPdlPort = cudaGraphKernelNodePortProgrammatic;
int add_pdl_edge(cudaGraph_t graph, cudaGraphNode_t from, cudaGraphNode_t to) {
  cudaGraphEdgeData e{};
  e.from_port = kPdlPort;
  e.to_port = 0;
  e.type = cudaGraphDependencyTypeProgrammatic;
  CU(cudaGraphAddDependencies(graph, &from, &to, &e, 1));
  return STS_OK;
}

int add_while(cudaGraphNode_t* node, cudaGraph_t graph, const std::vector<cudaGraphNode_t>& deps,
              cudaGraphConditionalHandle h, cudaGraph_t* body) {
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  CU(cudaGraphAddNode(node, graph, deps.data(), nullptr, deps.size(), &cp));
  *body = cp.conditional.phGraph_out[0];
  return STS_OK;
}

}  // namespace

// The whole multi-step loop as one graph:
//   WHILE(step) { step_begin -> WHILE(outer) { assemble -> sweep loop (one cooperative kernel) ->
//                 correct -> face_rho -> walls -> boundary -> T-jump -> flux_diff } -> step_end }
// Every decision (sweep count, outer iterations, end of run) is taken on the device.
// loop: the steps in a WHILE node (any number of steps per launch, each ended by the device's
// decision); otherwise one step, its kernels at the top level of the graph (launches of one step:
// a conditional node costs several microseconds per step).  xout (one step, xout_in_graph()): the
// state goes out to host buffers beside the flux kernel, the zero-gradient copies of p and T
// moving from the flux kernel to the end of the boundary kernel.
// One small CTA per SM for the state's way out: it fits beside the flux kernel's resident CTAs
// (their registers leave about 4k per SM), and 64 threads a CTA still keep enough bytes in flight
// to fill the host link.
constexpr int kXoutThreads = 64;

int sts_ctx::build_graph(bool loop, bool xout) {
  cudaGraph_t& top = loop ? graph : (xout ? graph1x : graph1);
  CU(cudaGraphCreate(&top, 0));
  cudaGraphConditionalHandle hs = 0;
  cudaGraph_t b_step = top;
  if (loop) {
    CU(cudaGraphConditionalHandleCreate(&hs, top, 1, cudaGraphCondAssignDefault));
    cudaGraphNode_t n_step;
    if (int r = add_while(&n_step, top, {}, hs, &b_step)) return r;
  }
  // one outer iteration per step (N_I = 1): its kernels go straight into the step's body, without
  // the conditional WHILE node that repeats them (the network's captured kernels keep the node)
  const bool one_outer = hc.cfg.n("N_I") == 1 && !warm_net;
  cudaGraphConditionalHandle ho = 0;
  if (!one_outer) CU(cudaGraphConditionalHandleCreate(&ho, b_step, 1, cudaGraphCondAssignDefault));
  const int outer_cond = one_outer ? 0 : 1;  // the kernels that set the outer node's condition
  cudaGraphNode_t n_begin, n_outer = nullptr, n_end;
  if (xout) {  // one_outer holds: no outer node
    const double* none = nullptr;
    if (int r = add_kernel(&n_begin, b_step, {}, k_step_begin_in, grid, block, g, 0ull, 0, none, none, none, none))
      return r;
    n_xin = n_begin;
  } else if (int r = add_kernel(&n_begin, b_step, {}, k_step_begin, grid, block, g, 1, (unsigned long long)ho,
                                outer_cond)) {
    return r;
  }
  if (g.warm_start == 3) {
    cudaGraphNode_t w[3];
    if (int r = add_kernel(&w[0], b_step, {n_begin}, k_warm_diff, grid, block, g)) return r;
    if (int r = add_kernel(&w[1], b_step, {w[0]}, k_warm_fit, dim3(1), dim3(576), g)) return r;
    if (int r = add_kernel(&w[2], b_step, {w[1]}, k_warm_apply, grid, block, g)) return r;
    n_begin = w[2];
  }
  cudaGraph_t b_outer = b_step;
  if (!one_outer)
    if (int r = add_while(&n_outer, b_step, {n_begin}, ho, &b_outer)) return r;
  cudaGraphNode_t n_asm, n_sw, n_cor, n_rho, n_bnd, n_fd, n_pred = nullptr;
  if (int r = add_kernel(&n_asm, b_outer, one_outer ? std::vector<cudaGraphNode_t>{n_begin} : std::vector<cudaGraphNode_t>{},
                         asm_kernel(), asm_grid(), asm_block, g, (unsigned long long)0, 0))
    return r;
  // warm_start 4: the predictor's kernels (first outer iteration only) beside the assembly
  std::vector<cudaGraphNode_t> before_sweeps{n_asm};

  if (tb_on()) {
    if (int r = add_kernel(&n_sw, b_outer, before_sweeps, pt_kernel_tb(), pt_grid, dim3(32, 8), g, ntiles, d_lc, emaps))
      return r;
  } else if (int r = add_kernel(&n_sw, b_outer, before_sweeps, pt_kernel(), pt_grid, dim3(32, 8), g, ntiles, d_lc)) {
    return r;
  }
  {
    cudaLaunchAttributeValue v{};
    v.cooperative = 1;
    CU(cudaGraphKernelNodeSetAttribute(n_sw, cudaLaunchAttributeCooperative, &v));
  }
  // correct -> face_rho -> boundary -> flux_diff, each launched as soon as its predecessor's CTAs
  // have all finished (programmatic edges; every one of these kernels waits before touching memory)
  if (int r = add_kernel(&n_cor, b_outer, {}, correct_kernel(), grid, block, g)) return r;
  if (int r = add_pdl_edge(b_outer, n_sw, n_cor)) return r;
  if (g.warm_start == 4) {  // the fit and the next step's start, beside the step's last kernels
    cudaGraphNode_t w[4];
    if (int r = add_kernel(&w[0], b_outer, {n_sw}, k_conv_gram, grid, block, g)) return r;
    if (int r = add_kernel(&w[1], b_outer, {w[0]}, k_conv_solve, dim3(2), dim3(kConvSolveThreads), g)) return r;
    if (int r = add_kernel(&w[2], b_outer, {w[0]}, k_conv_next, grid, block, g)) return r;
    if (int r = add_kernel(&w[3], b_outer, {w[1], w[2]}, k_conv_predict, grid, block, g)) return r;
    n_pred = w[3];
    if (warm_net) {  // the network's kernels, captured into the body after the stencil's
      CU(cudaStreamBeginCaptureToGraph(cap, b_outer, &w[3], nullptr, 1, cudaStreamCaptureModeRelaxed));
      net_tail(cap);
      cudaGraph_t captured = nullptr;
      CU(cudaStreamEndCapture(cap, &captured));
    }
  }
  if (int r = add_kernel(&n_rho, b_outer, {}, k_face_rho, grid, block, g)) return r;
  if (int r = add_pdl_edge(b_outer, n_cor, n_rho)) return r;
  const unsigned tail = PH_TEMP | PH_PRES;
  if (int r = add_kernel(&n_bnd, b_outer, {}, k_bnd_fused, bnd_grid(), dim3(kBndThreads), g, (unsigned long long)ho,
                         outer_cond, jump_beside() ? 1 : 0, xout ? tail : 0u))
    return r;
  if (int r = add_pdl_edge(b_outer, n_rho, n_bnd)) return r;
  if (int r = add_kernel(&n_fd, b_outer, {}, flux_kernel(), grid, block, g, xout ? 0u : tail)) return r;
  if (int r = add_pdl_edge(b_outer, n_bnd, n_fd)) return r;
  if (xout)  // the buffers are set before every launch
    if (int r = add_kernel(&n_xout, b_outer, {n_bnd}, k_move4_state_out, dim3(std::max(1, sms)), dim3(kXoutThreads), g,
                           (double*)nullptr, (double*)nullptr, (double*)nullptr, (double*)nullptr))
      return r;
  std::vector<cudaGraphNode_t> before_end{n_outer};
  if (one_outer) {  // every last node of the outer iteration's kernels
    before_end = {n_fd};
    if (n_pred) before_end.push_back(n_pred);
  }
  if (int r = add_kernel(&n_end, b_step, before_end, k_step_end, dim3(1), dim3(1024), g, (unsigned long long)hs,
                         loop ? 1 : 0))
    return r;
  CU(cudaGraphInstantiate(loop ? &exec : (xout ? &exec1x : &exec1), top, 0));
  if (loop) h_step = hs;
  h_outer = ho;
  return STS_OK;
}

int sts_ctx::step_graph(int n, int* done, double* const* state_out, const double* const* state_in) {
  const bool loop = n != 1;
  const bool xout = !loop && state_out && xout_in_graph();
  cudaGraphExec_t& ex = loop ? exec : (xout ? exec1x : exec1);
  if (!ex)
    if (int r = build_graph(loop, xout)) return r;
  const unsigned before = h_ctl->it_counter;
  unsigned left = (unsigned)n;
  CU(cudaMemcpyAsync(&d_ctl->steps_left, &left, sizeof(unsigned), cudaMemcpyHostToDevice, s));
  if (xout) {
    const double* none[4] = {nullptr, nullptr, nullptr, nullptr};
    const double* const* in = state_in ? state_in : none;
    if (int r = set_kernel_args(ex, n_xin, k_step_begin_in, grid, block, g, 0ull, 0, in[0], in[1], in[2], in[3]))
      return r;
    if (int r = set_kernel_args(ex, n_xout, k_move4_state_out, dim3(std::max(1, sms)), dim3(kXoutThreads), g, state_out[0],
                                state_out[1], state_out[2], state_out[3]))
      return r;
  }
  CU(cudaGraphLaunch(ex, s));
  if (state_out && !xout) {  // the new state straight to device-addressable host buffers, before the one sync
    k_move4_state_out<<<std::max(1, std::min((g.Na + 255) / 256, 4 * std::max(sms, 1))), 256, 0, s>>>(
        g, state_out[0], state_out[1], state_out[2], state_out[3]);
    CU(cudaGetLastError());
  }
  if (int r = read_ctl()) return r;
  *done = (int)(h_ctl->it_counter - before);
  return STS_OK;
}

// Kernel-by-kernel variant: the device still decides every sweep; the host only
// checks after each batch of sweep launches whether the loop has stopped.
int sts_ctx::step_host(int n, int* done) {
  const int NI = (int)hc.cfg.n("N_I");
  int k = 0;
  for (; k < n; k++) {
    k_step_begin<<<grid, block, 0, s>>>(g, 1, 0, 0);
    warm_launches([](int) {});
    for (int outer = 0; outer < NI; outer++) {
      asm_kernel()<<<asm_grid(), asm_block, 0, s>>>(g, 0, 0);
      if (int r = pt_loop()) return r;
      correct_kernel()<<<grid, block, 0, s>>>(g);
      k_face_rho<<<grid, block, 0, s>>>(g);
      boundary_step([](int) {});
      if (NI > 1) {
        if (int r = read_ctl()) return r;
        if (!h_ctl->continue_iter) break;
      }
    }
    warm_train([](int) {});
    k_step_end<<<1, 1024, 0, s>>>(g, 0, 0);
    if (int r = check()) return r;
    if (int r = read_ctl()) return r;
    if (!h_ctl->continue_step) {
      k++;
      break;
    }
  }
  *done = k;
  return STS_OK;
}

// One step launched kernel by kernel for the autotuner: the step's assembly kernels run with the
// block shape of candidate tune_idx % 3 and its sweep loops with tune_idx % per_sm_max + 1 CTAs per
// SM; event pairs time both.  The step is a real step (launch shapes do not change results).
int sts_ctx::tune_step(int* done) {
  const int NI = (int)hc.cfg.n("N_I");
  const int npt = (int)tune_pt.size(), nasm = (int)tune_asm.size();
  const bool record = tune_idx >= 0;  // index -1: one warm-up step, not recorded
  const int pc = record ? tune_idx % npt : npt - 1, ac = record ? tune_idx % nasm : 0;
  asm_block = asm_shape(ac);
  pt_per_sm = pc % pt_per_sm_max + 1;
  pt_tb = pt_tb_forced ? pt_tb_forced : (pc >= pt_per_sm_max ? 2 : 1);
  if (int r = size_pt_grid()) return r;
  std::vector<cudaEvent_t> ev;
  auto mark = [&]() {
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    ev.push_back(e);
  };
  k_step_begin<<<grid, block, 0, s>>>(g, 1, 0, 0);
  warm_launches([](int) {});
  int outer = 0;
  for (; outer < NI; outer++) {
    mark();
    asm_kernel()<<<asm_grid(), asm_block, 0, s>>>(g, 0, 0);
    mark();
    if (int r = pt_loop()) return r;
    mark();
    correct_kernel()<<<grid, block, 0, s>>>(g);
    k_face_rho<<<grid, block, 0, s>>>(g);
    boundary_step([](int) {});
    if (NI > 1) {
      if (int r = read_ctl()) return r;
      if (!h_ctl->continue_iter) {
        outer++;
        break;
      }
    }
  }
  warm_train([](int) {});
  k_step_end<<<1, 1024, 0, s>>>(g, 0, 0);
  if (int r = check()) return r;
  if (int r = read_ctl()) return r;
  double t_asm = 0, t_pt = 0;
  for (size_t k = 0; k + 2 < ev.size(); k += 3) {
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ev[k], ev[k + 1]);
    cudaEventElapsedTime(&b, ev[k + 1], ev[k + 2]);
    t_asm += a;
    t_pt += b;
  }
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  if (record) {
    if (outer > 0) tune_asm[ac].best = std::min(tune_asm[ac].best, t_asm / outer);
    if (h_ctl->step_sweeps > 0) tune_pt[pc].best = std::min(tune_pt[pc].best, t_pt / h_ctl->step_sweeps);
  }
  tune_idx++;
  if (--tune_left == 0) tune_choose();
  *done = 1;
  return STS_OK;
}

// The fastest block shape per assembly launch and CTAs per SM per sweep; the graph, built after
// the tuning steps, uses them.
void sts_ctx::tune_choose() {
  int best_a = 0, best_p = (int)tune_pt.size() - 1;
  for (int k = 0; k < (int)tune_asm.size(); k++)
    if (tune_asm[k].best < tune_asm[best_a].best) best_a = k;
  for (int k = 0; k < (int)tune_pt.size(); k++)
    if (tune_pt[k].best < tune_pt[best_p].best) best_p = k;
  asm_block = asm_shape(best_a);
  pt_per_sm = best_p % pt_per_sm_max + 1;
  pt_tb = pt_tb_forced ? pt_tb_forced : (best_p >= pt_per_sm_max ? 2 : 1);
  size_pt_grid();
}

// The TMA tensor maps of the FP32 correction buffers: 2D FP32, rows of Nxe floats, boxes of 40 x 12
// (the tile of 32 x 8 cells with a margin of two, x from 4 cells left of the tile).
int sts_ctx::make_emaps() {
  void* fp = nullptr;
  cudaDriverEntryPointQueryResult q;
  CU(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fp, 12000, cudaEnableDefault, &q));
  if (q != cudaDriverEntryPointSuccess || !fp) return fail(STS_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  auto enc = (PFN_cuTensorMapEncodeTiled_v12000)fp;
  cuuint64_t dims[2] = {(cuuint64_t)g.Nxe, (cuuint64_t)g.Ny};
  cuuint64_t strides[1] = {(cuuint64_t)g.Nxe * sizeof(float)};
  cuuint32_t box[2] = {40, 12}, es[2] = {1, 1};
  for (int b = 0; b < 3; b++)
    for (int f = 0; f < 2; f++) {
      CUtensorMap* m = f ? &emaps.ep[b] : &emaps.eT[b];
      float* base = f ? g.ep[b] : g.eT[b];
      if (enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return fail(STS_ERR_CUDA, "cuTensorMapEncodeTiled failed for a correction buffer");
    }
  return STS_OK;
}

// The launch loop with a CUDA event pair around every kernel: per-kernel device time.
// kinds: 0 step_begin, 1 assemble, 2 sweep loop, 3 correct, 4 face_rho, 5 boundary,
// 6 flux_diff, 7 step_end
int sts_ctx::profile(int n, double* ms, int* cnt, int* done) {
  const int NI = (int)hc.cfg.n("N_I");
  std::vector<cudaEvent_t> ev;
  std::vector<int> kind;
  auto mark = [&](int k) {
    cudaEvent_t a;
    cudaEventCreate(&a);
    cudaEventRecord(a, s);
    ev.push_back(a);
    kind.push_back(k);
  };
  for (int q = 0; q < kProfileKinds; q++) { ms[q] = 0; cnt[q] = 0; }
  int k = 0;
  for (; k < n; k++) {
    mark(-1); k_step_begin<<<grid, block, 0, s>>>(g, 1, 0, 0); mark(0);
    warm_launches(mark);
    for (int outer = 0; outer < NI; outer++) {
      mark(-1);
      asm_kernel()<<<asm_grid(), asm_block, 0, s>>>(g, 0, 0);
      mark(1);
      mark(-1);
      if (int r = pt_loop()) return r;
      mark(2);
      mark(-1); correct_kernel()<<<grid, block, 0, s>>>(g); mark(3);
      mark(-1); k_face_rho<<<grid, block, 0, s>>>(g); mark(4);
      boundary_step(mark);
      if (NI > 1) {
        if (int r = read_ctl()) return r;
        if (!h_ctl->continue_iter) break;
      }
    }
    warm_train(mark);
    mark(-1); k_step_end<<<1, 1024, 0, s>>>(g, 0, 0); mark(7);
    if (int r = check()) return r;
    if (int r = read_ctl()) return r;
    if (!h_ctl->continue_step) { k++; break; }
  }
  CU(cudaStreamSynchronize(s));
  for (size_t q = 1; q < ev.size(); q++) {
    if (kind[q] < 0) continue;
    float t = 0;
    cudaEventElapsedTime(&t, ev[q - 1], ev[q]);
    ms[kind[q]] += t;
    cnt[kind[q]] += 1;
  }
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  *done = k;
  return STS_OK;
}

// The mesh files written while the mesh is built (SIMPLE_TS_MPI.cpp:2252-2259).
int sts_ctx::write_mesh() {
  if (!opt.write_files) return STS_OK;
  const std::string dir = hc.dir + "/";
  write_txt(dir + "x_f.txt", hc.x_f.data(), hc.Nx + 1);
  write_txt(dir + "hx.txt", hc.hx.data(), hc.Nx);
  write_txt(dir + "x_v.txt", hc.x_v.data(), hc.Nx);
  write_txt(dir + "y_f.txt", hc.y_f.data(), hc.Ny + 1);
  write_txt(dir + "hy.txt", hc.hy.data(), hc.Ny);
  write_txt(dir + "y_v.txt", hc.y_v.data(), hc.Ny);
  return STS_OK;
}

// WriteDragCoefficient (SIMPLE_TS_MPI.cpp:8147-8578, serial path): the sums on the device
// (k_drag), the coefficients and the three logs on the host with the reference's arithmetic
// and formats: CD.<body>.txt for the flagged bodies, DataInShortFormat.txt, p_and_u_xb_it.txt.
int sts_ctx::write_drag() {
  if (!opt.write_files) return STS_OK;
  const Config& cf = hc.cfg;
  const int nl = (int)drag_bodies.size();
  std::vector<double> sums(12 * nl + 2, 0.0);
  k_drag<<<1, std::max(32, ((nl + 1 + 31) / 32) * 32), 0, s>>>(g, d_drag_cells, d_drag_first, nl, d_drag_out);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(sums.data(), d_drag_out, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost, s));
  if (int r = read_ctl()) return r;
  const Ctl& c = *h_ctl;
  const std::string dir = hc.dir + "/";
  const bool restart = cf.b("ToReadSolvedDataFromFile");
  const int TypeND = (int)cf.n("TypeOfNonDimensiolization");
  const double Re = cf.d("Re"), Ma = cf.d("Ma"), Kn = cf.d("Kn"), gamma1 = cf.d("gamma1"), T_BC_xb = cf.d("T_BC_xb");
  const double ht = cf.d("ht"), ug = c.u_given_xb_in_it;
  double CD_fr_x = 0, CD_p_x = 0;
  const int w = 30;
  for (int k = 0; k < nl; k++) {
    const double* q = &sums[12 * k];
    double c_CD_p = 0, c_CD_fr = 0;
    if (TypeND == 1) {
      c_CD_p = 1.0 / (ug * ug * (c.p_BC_xb / T_BC_xb));
      c_CD_fr = 2.0 / (Re * ug);
    } else if (TypeND == 2) {
      c_CD_p = 2.0 / (gamma1 * Ma * Ma * (c.p_BC_xb / T_BC_xb));
      c_CD_fr = 2.0 / (Re * ug);
    } else if (TypeND == 3) {
      c_CD_p = 1.0 / (ug * ug * (c.p_BC_xb / T_BC_xb));
      c_CD_fr = (5.0 / 8.0) * std::sqrt(M_PI) * Kn / (ug * ug * (c.p_BC_xb / T_BC_xb));
    }
    const double fb = c_CD_fr * q[0], pb = c_CD_p * q[1], ff = c_CD_fr * q[3], pf = c_CD_p * q[4];
    const double ft = c_CD_fr * q[6], pt = c_CD_p * q[7], fh = c_CD_fr * q[9], ph = c_CD_p * q[10];
    CD_fr_x = (ft / q[8]) + (fb / q[2]);
    CD_p_x = (pf / q[5]) - (ph / q[11]);
    const std::string name = dir + "CD." + std::to_string(drag_bodies[k]) + ".txt";
    std::ofstream o;
    if (cd_fresh && !restart) o.open(name.c_str());
    else o.open(name.c_str(), std::ios::out | std::ios::app);
    if (!restart && cd_fresh) {
      const char* hdr[16] = {"//it (number of step by time) 00", "ht (step by time) 01", "CD_fr_x (CD from friction) 02",
                             "CD_p_x (CD from pressure) 03", "S_for_CD_bottom 04", "S_for_CD_front 05",
                             "S_for_CD_top 06", "S_for_CD_behind 07", "CD_fr_bottom 08", "CD_p_bottom 09",
                             "CD_fr_front 10", "CD_p_front 11", "CD_fr_top 12", "CD_p_top 13", "CD_fr_behind 14",
                             "CD_p_behind 15"};
      for (const char* hh : hdr) o << std::setw(w) << hh;
      o << std::endl;
    }
    o << std::setw(w) << c.it << std::setiosflags(std::ios::scientific) << std::setprecision(10);
    const double vals[15] = {ht, CD_fr_x, CD_p_x, q[2], q[5], q[8], q[11], fb, pb, ff, pf, ft, pt, fh, ph};
    for (double x : vals) o << std::setw(w) << x;
    o << std::endl;
  }
  if (nl > 0) cd_fresh = false;
  if (cf.n("WriteDataInShortFormat_kind") == 1) {
    std::ofstream o((dir + "DataInShortFormat.txt").c_str());
    o << std::setiosflags(std::ios::scientific) << std::setprecision(15) << std::setw(w) << Re << std::setw(w) << Kn
      << std::setw(w) << CD_p_x + CD_fr_x << std::setw(w) << CD_p_x << std::setw(w) << c.u_gas_nd << std::setw(w)
      << sums[12 * nl] << std::setw(w) << sums[12 * nl + 1] << std::setw(w) << c.p_BC_xb << std::setw(w) << c.p_BC_xe
      << std::endl;
  }
  if (hc.bits & F_PRESSURE_BC) {
    const std::string name = dir + "p_and_u_xb_it.txt";
    std::ofstream o;
    if (pu_fresh && !restart) o.open(name.c_str());
    else o.open(name.c_str(), std::ios::out | std::ios::app);
    if (!restart && pu_fresh) {
      const char* hdr[7] = {"//it (number of step by time)", "ht (step by time)", "p_BC_xb", "u_given_xb_in_it",
                            "u_given_xb_in_it_max", "u_given_xb_in_it_mean", "p_correction"};
      for (const char* hh : hdr) o << std::setw(w) << hh;
      o << std::endl;
    }
    o << std::setw(w) << c.it << std::setiosflags(std::ios::scientific) << std::setprecision(15) << std::setw(w) << ht
      << std::setw(w) << c.p_BC_xb << std::setw(w) << c.u_given_xb_in_it << std::setw(w) << c.u_in_max
      << std::setw(w) << c.u_in_mean << std::setw(w) << c.p_correction << std::endl;
    pu_fresh = false;
  }
  return STS_OK;
}

// SolveContinuityEquation (SIMPLE_TS_MPI.cpp:10621-10714, serial path): the fluxes again (as the
// reference does; this is also what the next step's assembly sees), the residuals, the dumps.
int sts_ctx::continuity() {
  k_fluxes<<<grid, block, 0, s>>>(g);
  k_continuity<<<grid, block, 0, s>>>(g, d_cont_st, d_cont);
  CU(cudaGetLastError());
  if (!opt.write_files) return STS_OK;
  const int Na = hc.Na;
  std::vector<double> st(Na), ce(Na);
  CU(cudaMemcpyAsync(st.data(), d_cont_st, sizeof(double) * Na, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(ce.data(), d_cont, sizeof(double) * Na, cudaMemcpyDeviceToHost, s));
  if (int r = read_ctl()) return r;
  const std::string dir = hc.dir + "/", its = num(h_ctl->it);
  const bool bin = hc.cfg.b("ToWriteSolvedDataToBinaryFile"), newf = hc.cfg.b("ToWriteSolvedDataToNewFiles");
  const std::string ext = bin ? ".bin" : ".txt";
  auto put = [&](const std::string& f, const std::vector<double>& a) {
    if (bin) write_bin(f, a.data(), sizeof(double) * Na);
    else write_txt(f, a.data(), Na);
  };
  put(dir + "ContinuityEquation_stationary" + ext, st);
  put(dir + "ContinuityEquation" + ext, ce);
  if (newf) {
    put(dir + "ContinuityEquation_stationary." + its + ext, st);
    put(dir + "ContinuityEquation." + its + ext, ce);
  }
  return STS_OK;
}

// WriteSolvedDataToFile (SIMPLE_TS_MPI.cpp:5564-5731): the wall-temperature overwrite is a
// side effect on the state; then a snapshot of u, v, p, T is taken on the stream and its dumps,
// it_begin.txt and EnteredData.txt are written by the checkpoint thread.  wait_files: return
// only once they are on disk.
int sts_ctx::write_outputs(bool wait_files) {
  boundary(PH_TJUMP | PH_TJUMP_WRITE);
  if (int r = check()) return r;
  if (!opt.write_files) return STS_OK;
  if (int r = read_ctl()) return r;
  if (!saver) saver.reset(new Checkpointer(opt.device, (size_t)hc.Na));
  const unsigned cur = h_ctl->cur;
  const double* src[4] = {g.u, g.v, g.p[cur], g.T[cur]};
  DumpSpec d;
  d.dir = hc.dir;
  d.it = h_ctl->it;
  d.bin = hc.cfg.b("ToWriteSolvedDataToBinaryFile");
  d.newf = hc.cfg.b("ToWriteSolvedDataToNewFiles");
  d.cfg = hc.cfg;
  d.vol = hc.vol_file.data();
  std::string err;
  if (int r = saver->save(s, src, std::move(d), err)) return fail(r, err);
  if (wait_files)
    if (int r = saver->wait(err)) return fail(r, err);
  return STS_OK;
}

// Every checkpoint taken so far is on disk.
int sts_ctx::wait_outputs() {
  std::string err;
  if (saver)
    if (int r = saver->wait(err)) return fail(r, err);
  return STS_OK;
}

// WriteTempDataToFile and WriteIterationsInLoopsToFile (SIMPLE_TS_MPI.cpp:5838-6006).
int sts_ctx::write_logs(bool iterations) {
  if (!opt.write_files) return STS_OK;
  if (int r = read_ctl()) return r;
  const Ctl& c = *h_ctl;
  {
    std::ofstream o;
    if (tmp_fresh && !hc.restart) o.open((hc.dir + "/Tmp.txt").c_str());
    else o.open((hc.dir + "/Tmp.txt").c_str(), std::ios::out | std::ios::app);
    o << "it = " << c.it << "\tit_counter = " << c.it_counter << "\tIter = " << c.Iter << "\tIter_p_c = " << c.Iter_p_c
      << "\tIter_T = " << (unsigned)hc.cfg.n("N_I_T") << std::endl;
    unsigned sum = 0;
    for (unsigned k = 0; k < c.Iter && k < 64; k++) {
      o << "\t" << k << "\t" << c.sweeps[k] << std::setiosflags(std::ios::scientific) << std::setprecision(15) << "\t"
        << c.res_p0[k] << "\t" << c.res_p[k] << "\t" << c.res_T0[k] << "\t" << c.res_T[k] << std::endl;
      sum += c.sweeps[k];
    }
    o << "\t\t" << sum << std::endl;
    o << std::setiosflags(std::ios::scientific) << std::setprecision(15) << "\t" << c.res_u0 << "\t" << c.res_u
      << std::endl
      << "\t" << c.res_v0 << "\t" << c.res_v << std::endl;
    tmp_fresh = false;
  }
  if (iterations) {
    std::ofstream o;
    if (iter_fresh) {
      if (hc.restart) o.open((hc.dir + "/Iterations_in_loops.txt").c_str(), std::ios::out | std::ios::app);
      else {
        o.open((hc.dir + "/Iterations_in_loops.txt").c_str());
        o << "it" << "\tit_counter" << "\tIter" << "\tsum_max_Iter_p_c" << std::endl;
      }
    } else {
      o.open((hc.dir + "/Iterations_in_loops.txt").c_str(), std::ios::out | std::ios::app);
    }
    unsigned sum = 0;
    for (unsigned k = 0; k < c.Iter && k < 64; k++) sum += c.sweeps[k];
    o << c.it << "\t" << c.it_counter << "\t\t" << c.Iter << "\t" << sum << std::endl;
    iter_fresh = false;
  }
  return STS_OK;
}

// warm_start 5: the window (64 x 256 cells, or the mesh rounded down to multiples of 4 when it is
// smaller), a U-Net of 3 levels and 16 base channels over it, a replay ring of 256 windows and
// the training batch buffers; one forward on the context's stream before any graph is built.
int sts_ctx::net_setup(unsigned long long seed) {
  nb.H = std::min(64, g.Ny / 4 * 4);
  nb.W = std::min(256, g.Nx / 4 * 4);
  if (nb.H < 4 || nb.W < 4) return fail(STS_ERR_ARG, "warm_start 5 needs a mesh of at least 4 x 4 cells");
  const size_t px = (size_t)nb.H * nb.W;
  net_slots = 256;
  nb.slot_floats = px * (kNetIn + kNetOut + 1 + kNetOut);
  if (int r = alloc(&nb.replay, nb.slot_floats * net_slots)) return r;
  if (int r = alloc(&nb.infer_in, px * kNetIn)) return r;
  if (int r = alloc(&nb.infer_w, px)) return r;
  if (int r = alloc(&nb.infer_out, px * kNetOut)) return r;
  if (int r = alloc(&d_ns, 1)) return r;
  if (int r = alloc(&d_bx, px * kNetBatch * kNetIn)) return r;
  if (int r = alloc(&d_bt, px * kNetBatch * kNetOut)) return r;
  if (int r = alloc(&d_bw, px * kNetBatch)) return r;
  if (int r = alloc(&d_loss, 1)) return r;
  if (int r = alloc(&d_bslots, kNetBatch)) return r;
  CU(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  net.reset(new UNet(kNetIn, kNetOut, kNetBase, kNetLevels, kNetBatch, nb.H, nb.W, seed, s));
  if (!net->ok()) return fail(STS_ERR_CUDA, std::string("network set-up: ") + net->error());
  CU(net->forward(nb.infer_in, 1, nb.infer_out));
  CU(cudaStreamSynchronize(s));
  return STS_OK;
}

namespace {

// Scratch of one sweep-loop call: the second p and T buffers, the 8 sweep invariants and the
// control block, carved out of one device region of scratch_bytes(Na) bytes.
size_t scratch_bytes(size_t Na) { return sizeof(Ctl) + 256 + 10 * Na * sizeof(double); }

// The sweep loop of sts_pt_sweeps on a given scratch region (no allocation here).
int pt_sweeps_on(const sts_sweep_fields* f, int max_sweeps, int fixed, double tol_p, double tol_T, cudaStream_t s,
                 char* scratch, int* sweeps_done, double* res_p, double* res_T) {
  const size_t Na = (size_t)f->Nx * (size_t)f->Ny;
  Geo g{};
  g.Nx = f->Nx;
  g.Ny = f->Ny;
  g.Na = (int)Na;
  g.bits = (f->periodic ? F_PERIODIC : 0) | (f->given_u_xb ? F_GIVEN_U_XB : 0) | (f->given_u_xe ? F_GIVEN_U_XE : 0) |
           (fixed ? F_FIXED_SWEEPS : 0);
  g.Nx_o0 = f->Nx_o0;
  g.Nx_o1 = f->Nx_o1;
  g.ht = f->ht;
  g.gamma1 = f->gamma1;
  g.MaxError_p_c = tol_p;
  g.MaxError_T = tol_T;
  g.N_I_p_c = max_sweeps;
  g.cls = f->cls;
  g.hx = f->hx; g.hy = f->hy;
  g.Fx = const_cast<double*>(f->Fx); g.Fy = const_cast<double*>(f->Fy);
  g.DTx = const_cast<double*>(f->DTx); g.DTy = const_cast<double*>(f->DTy);
  g.u = const_cast<double*>(f->u); g.v = const_cast<double*>(f->v); g.rho = const_cast<double*>(f->rho);
  g.ScT1 = const_cast<double*>(f->ScT1);
  g.apx = const_cast<double*>(f->apx); g.apy = const_cast<double*>(f->apy);
  g.bpx = const_cast<double*>(f->bpx); g.bpy = const_cast<double*>(f->bpy);
  g.p_pr = const_cast<double*>(f->p_pr); g.T_pr = const_cast<double*>(f->T_pr);
  g.Tw_u = const_cast<double*>(f->Tw_u); g.Tw_v = const_cast<double*>(f->Tw_v);
  Ctl* ctl = (Ctl*)scratch;
  double* arr = (double*)(scratch + ((sizeof(Ctl) + 255) / 256) * 256);
  g.ctl = ctl;
  g.p[0] = f->p;
  g.T[0] = f->T;
  g.p[1] = arr;
  g.T[1] = arr + Na;
  for (int k = 0; k < 8; k++) g.inv[k] = arr + (2 + k) * Na;
  CU(cudaMemsetAsync(ctl, 0, sizeof(Ctl), s));  // buffer index, counters and maxima start at zero
  const dim3 block(32, 8), grid((f->Nx + 31) / 32, (f->Ny + 7) / 8);
  k_sweep_first<<<grid, block, 0, s>>>(g, 0, 0);
  struct { unsigned cur, Iter, Iter_pr1, Iter_pr2, Iter_p_c, it_counter, pt_done; } head{};
  const size_t head_off = offsetof(Ctl, cur);
  if (fixed) {
    for (int q = 1; q < max_sweeps; q++) k_sweep<<<grid, block, 0, s>>>(g, 0, 0);
  } else {
    int launched = 1;
    for (;;) {
      CU(cudaMemcpyAsync(&head, (char*)ctl + head_off, sizeof(head), cudaMemcpyDeviceToHost, s));
      CU(cudaStreamSynchronize(s));
      if (head.pt_done || launched >= max_sweeps) break;
      for (int q = 0; q < 4 && launched < max_sweeps; q++, launched++) k_sweep<<<grid, block, 0, s>>>(g, 0, 0);
    }
  }
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(&head, (char*)ctl + head_off, sizeof(head), cudaMemcpyDeviceToHost, s));
  double rp = 0, rT = 0;
  unsigned status = 0;
  CU(cudaMemcpyAsync(&rp, &ctl->res_p[0], sizeof(double), cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(&rT, &ctl->res_T[0], sizeof(double), cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(&status, &ctl->status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  if (head.cur == 1) {  // an odd number of sweeps left the result in the scratch buffers
    CU(cudaMemcpyAsync(f->p, g.p[1], sizeof(double) * Na, cudaMemcpyDeviceToDevice, s));
    CU(cudaMemcpyAsync(f->T, g.T[1], sizeof(double) * Na, cudaMemcpyDeviceToDevice, s));
    CU(cudaStreamSynchronize(s));
  }
  if (sweeps_done) *sweeps_done = (int)head.Iter_p_c;
  if (res_p) *res_p = rp;
  if (res_T) *res_T = rT;
  if (status & 1u) return fail(STS_ERR_NONFINITE, "a residual became NaN or Inf");
  return STS_OK;
}

int check_sweep_args(const sts_sweep_fields* f, int max_sweeps) {
  if (!f || max_sweeps < 1) return fail(STS_ERR_ARG, "bad argument");
  if (f->Nx < 3 || f->Ny < 3) return fail(STS_ERR_ARG, "mesh must have at least 3 cells in each direction");
  const void* ptrs[] = {f->cls, f->hx, f->hy, f->Fx, f->Fy, f->DTx, f->DTy, f->u, f->v, f->rho, f->ScT1, f->apx,
                        f->apy, f->bpx, f->bpy, f->p_pr, f->T_pr, f->Tw_u, f->Tw_v, f->p, f->T};
  for (const void* q : ptrs)
    if (!q) return fail(STS_ERR_ARG, "null field pointer");
  if (f->Nx_o0 < 0 || f->Nx_o1 > f->Nx) return fail(STS_ERR_ARG, "bad p/T solve range");
  return STS_OK;
}

int open_impl(const char* dir, const sts_options* opt_in, sts_ctx** out) {
  if (!dir || !out) return fail(STS_ERR_ARG, "null argument");
  sts_options opt;
  sts_default_options(&opt);
  if (opt_in) opt = *opt_in;
  std::unique_ptr<sts_ctx> c(new sts_ctx);
  c->opt = opt;
  c->t0 = std::chrono::steady_clock::now();
  std::string err;
  if (opt.precision < 0 || opt.precision > 3) return fail(STS_ERR_ARG, "precision must be 0, 1, 2 or 3");
  if (opt.warm_start < 0 || opt.warm_start > 5) return fail(STS_ERR_ARG, "warm_start must be 0, 1, 2, 3, 4 or 5");
  if (!load_case(dir, opt.fixed_sweeps != 0, c->hc, err)) return fail(STS_ERR_INPUT, err);
  Case& h = c->hc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(STS_ERR_CUDA, "no CUDA device");
  if (opt.device < 0 || opt.device >= ndev) return fail(STS_ERR_ARG, "bad device ordinal");
  CU(cudaSetDevice(opt.device));
  CU(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking));
  CU(cudaMallocHost(&c->h_ctl, sizeof(Ctl)));
  std::memset(c->h_ctl, 0, sizeof(Ctl));
  const int Na = h.Na;
  Geo& g = c->g;
  g.Nx = h.Nx;
  g.Ny = h.Ny;
  g.Na = Na;
  g.bits = h.bits;
  g.Nx_u0 = h.Nx_u[0]; g.Nx_u1 = h.Nx_u[1]; g.Ny_u0 = h.Ny_u[0]; g.Ny_u1 = h.Ny_u[1];
  g.Nx_v0 = h.Nx_v[0]; g.Nx_v1 = h.Nx_v[1]; g.Ny_v0 = h.Ny_v[0]; g.Ny_v1 = h.Ny_v[1];
  g.Nx_o0 = h.Nx_o[0]; g.Nx_o1 = h.Nx_o[1]; g.Ny_o0 = h.Ny_o[0]; g.Ny_o1 = h.Ny_o[1];
  const Config& cf = h.cfg;
  g.ht = cf.d("ht");
  g.gamma1 = cf.d("gamma1");
  g.Kn = cf.d("Kn");
  g.cT1 = h.cT1;
  g.cT2 = h.cT2;
  g.c_Fr_v = h.c_Fr_v;
  g.Re = cf.d("Re");
  g.Ma = cf.d("Ma");
  g.T_BC_xb = cf.d("T_BC_xb");
  g.T_BC_xe = cf.d("T_BC_xe");
  g.u_given_xb_error = cf.d("u_given_xb_error");
  g.p_correction_min = cf.d("p_correction_min");
  g.p_correction_max = cf.d("p_correction_max");
  g.MaxError_Velocities = cf.d("MaxError_Velocities");
  g.MaxError_p_c = cf.d("MaxError_p_c");
  g.MaxError_T = cf.d("MaxError_T");
  g.MaxError_to_stop_program = cf.d("MaxError_to_stop_program");
  g.Nt = cf.d("Nt");
  g.t_BC_b = cf.d("t_BC_b");
  g.t_BC_e = cf.d("t_BC_e");
  g.u_BC_xb_t_BC_b = cf.d("u_BC_xb_t_BC_b");
  g.u_BC_xb_t_BC_e = cf.d("u_BC_xb_t_BC_e");
  g.TypeND = (int)cf.n("TypeOfNonDimensiolization");
  g.N_I = (int)cf.n("N_I");
  g.N_I_p_c = (int)cf.n("N_I_p_c");
  g.p_corr_method = (int)cf.n("p_BC_xb_correction_method");

  // static data
  double *hx, *hy;
  uint8_t* cls;
  uint32_t* vid;
  Body* bodies;
  int *su, *sv, *tj;
  uint8_t *suf, *svf, *tjf, *tjw;
  if (int r = c->alloc(&hx, h.Nx)) return r;
  if (int r = c->alloc(&hy, h.Ny)) return r;
  if (int r = c->alloc(&cls, Na)) return r;
  if (int r = c->alloc(&vid, Na)) return r;
  if (int r = c->alloc(&bodies, h.bodies.size())) return r;
  if (int r = c->alloc(&su, h.slip_u.size())) return r;
  if (int r = c->alloc(&sv, h.slip_v.size())) return r;
  if (int r = c->alloc(&tj, h.tjump.size())) return r;
  if (int r = c->alloc(&suf, h.slip_u.size())) return r;
  if (int r = c->alloc(&svf, h.slip_v.size())) return r;
  if (int r = c->alloc(&tjf, h.tjump.size())) return r;
  if (int r = c->alloc(&tjw, h.tjump.size())) return r;
  std::vector<Body> bv;
  for (const HostBody& b : h.bodies) bv.push_back(b.dev);
  if (int r = c->upload(hx, h.hx)) return r;
  if (int r = c->upload(hy, h.hy)) return r;
  if (int r = c->upload(cls, h.cls)) return r;
  if (int r = c->upload(vid, h.vol_file)) return r;
  if (int r = c->upload(bodies, bv)) return r;
  if (int r = c->upload(su, h.slip_u)) return r;
  if (int r = c->upload(sv, h.slip_v)) return r;
  if (int r = c->upload(tj, h.tjump)) return r;
  if (int r = c->upload(suf, h.slip_u_fin)) return r;
  if (int r = c->upload(svf, h.slip_v_fin)) return r;
  if (int r = c->upload(tjf, h.tjump_fin)) return r;
  if (int r = c->upload(tjw, h.tjump_wr_fin)) return r;
  g.hx = hx; g.hy = hy; g.cls = cls; g.vol_id = vid; g.bodies = bodies;
  g.slip_u = su; g.slip_v = sv; g.tjump = tj;
  g.slip_u_fin = suf; g.slip_v_fin = svf; g.tjump_fin = tjf; g.tjump_wr_fin = tjw;
  g.n_slip_u = (int)h.slip_u.size();
  g.n_slip_v = (int)h.slip_v.size();
  g.n_tjump = (int)h.tjump.size();
  {
    std::vector<unsigned> solved, other;
    for (int j = 0; j < h.Ny; j++)
      for (int i = 0; i < h.Nx; i++)
        ((h.cls[i + j * h.Nx] & 0x30u) ? solved : other).push_back((unsigned)i | ((unsigned)j << 16));
    unsigned *dsol = nullptr, *doth = nullptr;
    if (int r = c->alloc(&dsol, solved.size())) return r;
    if (int r = c->alloc(&doth, other.size())) return r;
    if (int r = c->upload(dsol, solved)) return r;
    if (int r = c->upload(doth, other)) return r;
    g.pt_cells = dsol;
    g.pt_copy = doth;
    g.n_pt_cells = (int)solved.size();
    g.n_pt_copy = (int)other.size();
  }

  // fields
  double** fields[] = {&g.u, &g.v, &g.u_pr, &g.v_pr, &g.p[0], &g.p[1], &g.T[0], &g.T[1], &g.p_pr, &g.T_pr, &g.rho,
                       &g.rho_pr, &g.sqrt_T, &g.rho_u, &g.rho_v, &g.Fx, &g.Fy, &g.D_ux, &g.D_uy, &g.D_vx, &g.D_vy,
                       &g.DTx, &g.DTy, &g.Gamma_xf, &g.Gamma_yf, &g.u_pseudo, &g.v_pseudo, &g.d12, &g.d34, &g.apx,
                       &g.apy, &g.bpx, &g.bpy, &g.ScT1, &g.Tw_u, &g.Tw_v};
  for (double** f : fields)
    if (int r = c->alloc(f, Na)) return r;
  for (int k = 0; k < 9; k++)
    if (int r = c->alloc(&g.inv[k], Na)) return r;
  g.precision = opt.precision;
  {
    // correctly rounded reciprocals (IEEE division here) of the mesh quantities the kernels
    // divide by; the neighbour indices are those of the kernels (periodic wrap in x, the y index
    // above compared with Nx as in the reference's ScT1 code, clamped to the mesh)
    const int Nx = h.Nx, Ny = h.Ny;
    std::vector<double> rhx(Nx), rxm(Nx), rxp(Nx), r3x(Nx), rhy(Ny), rym(Ny), ryp(Ny), r3y(Ny);
    for (int i = 0; i < Nx; i++) {
      const Nb d = neighbours(i, 0, Nx, Ny, h.bits & F_PERIODIC);
      rhx[i] = 1.0 / h.hx[i];
      rxm[i] = 1.0 / (h.hx[d.i_1] + h.hx[i]);
      rxp[i] = 1.0 / (h.hx[i] + h.hx[d.i1]);
      r3x[i] = 1.0 / (h.hx[i] * 3.0);
    }
    for (int j = 0; j < Ny; j++) {
      const int jm = j - (0 < j ? 1 : 0), jp = std::min(j + (j < Nx - 1 ? 1 : 0), Ny - 1);
      rhy[j] = 1.0 / h.hy[j];
      rym[j] = 1.0 / (h.hy[jm] + h.hy[j]);
      ryp[j] = 1.0 / (h.hy[j] + h.hy[jp]);
      r3y[j] = 1.0 / (h.hy[j] * 3.0);
    }
    double* t[8];
    const std::vector<double>* src[8] = {&rhx, &rhy, &rxm, &rxp, &rym, &ryp, &r3x, &r3y};
    for (int k = 0; k < 8; k++) {
      if (int r = c->alloc(&t[k], src[k]->size())) return r;
      if (int r = c->upload(t[k], *src[k])) return r;
    }
    g.rhx = t[0]; g.rhy = t[1]; g.rxx_m = t[2]; g.rxx_p = t[3]; g.ryy_m = t[4]; g.ryy_p = t[5];
    g.r3x = t[6]; g.r3y = t[7];
    g.rht = 1.0 / g.ht;
    g.r3 = 1.0 / 3.0;
    for (int k = 0; k < 7; k++) {  // filled by k_flux_quotients before the first flux kernel
      double* q = nullptr;
      if (int r = c->alloc(&q, Na)) return r;
      if (k < 6) g.fq[k] = q;
      else g.hxy = q;
    }
  }
  // warm_start 5 is warm_start 4 on the device plus the network's kernels
  g.warm_start = opt.warm_start == 5 ? 4 : opt.warm_start;
  c->warm_net = opt.warm_start == 5;
  if (g.warm_start)
    for (int k = 0; k < 2; k++) {
      if (int r = c->alloc(&g.p_m[k], Na)) return r;
      if (int r = c->alloc(&g.T_m[k], Na)) return r;
    }
  if (g.warm_start == 3) {
    for (int k = 0; k < kWarmRing; k++) {
      if (int r = c->alloc(&g.Dp[k], Na)) return r;
      if (int r = c->alloc(&g.DT[k], Na)) return r;
    }
    const size_t nb = (size_t)((h.Nx + 31) / 32) * ((h.Ny + 7) / 8);
    if (int r = c->alloc(&g.warm_part, nb * 18)) return r;  // 2 fields x 9 normal-equation terms
  }
  if (g.warm_start == 4) {
    for (int f = 0; f < 2; f++)
      for (int k = 0; k < kConvRing; k++)
        if (int r = c->alloc(&g.cD[f][k], Na)) return r;
    for (int k = 0; k < 2; k++) {
      if (int r = c->alloc(&g.cact[k], Na)) return r;
      if (int r = c->alloc(&g.cnext[k], Na)) return r;
    }
    const size_t nt = (size_t)((h.Nx + 31) / 32) * ((h.Ny + 7) / 8);
    if (int r = c->alloc(&g.cpart, nt * 2 * kConvTerms)) return r;
    if (int r = c->alloc(&g.crows, nt * 2)) return r;
    if (int r = c->alloc(&g.ctmax, nt * 2)) return r;
    if (int r = c->alloc(&g.cgram, (size_t)kConvWin * 2 * kConvTerms)) return r;
  }
  if (g.precision >= 2) {
    float** f32[] = {&g.c32[0], &g.c32[1], &g.c32[2], &g.c32[3], &g.c32[4], &g.a32[0], &g.a32[1], &g.a32[2], &g.a32[3],
                     &g.T1, &g.hT, &g.q1, &g.den1, &g.dT, &g.dp};
    for (float** f : f32)
      if (int r = c->alloc(f, Na)) return r;
    g.Nxe = (h.Nx + 3) / 4 * 4;
    for (int b = 0; b < 3; b++) {
      if (int r = c->alloc(&g.ep[b], (size_t)g.Nxe * h.Ny)) return r;
      if (int r = c->alloc(&g.eT[b], (size_t)g.Nxe * h.Ny)) return r;
    }
    if (int r = c->make_emaps()) return r;
  }
  if (int r = c->alloc(&c->d_ctl, 1)) return r;
  g.ctl = c->d_ctl;
  if (c->warm_net)
    if (int r = c->net_setup(0x5EED0005ull)) return r;
  if (int r = c->upload(g.u, h.u)) return r;
  if (int r = c->upload(g.v, h.v)) return r;
  if (int r = c->upload(g.p[0], h.p)) return r;
  if (int r = c->upload(g.p[1], h.p)) return r;
  if (int r = c->upload(g.T[0], h.T)) return r;
  if (int r = c->upload(g.T[1], h.T)) return r;
  if (int r = c->upload(g.rho, h.rho)) return r;

  // control block
  Ctl& ct = *c->h_ctl;
  ct.cT = h.cT;
  ct.cPch = h.cPch;
  ct.p_BC_xb = h.p_BC_xb;
  ct.p_BC_xe = h.p_BC_xe;
  ct.u_given_xb = h.u_given_xb;
  ct.u_given_xb_in_it = h.u_given_xb_in_it;
  ct.p_correction = cf.d("p_correction");
  ct.u_gas_nd = cf.d("u_gas_nd");
  ct.it = h.restart ? h.it_begin : 0.0;
  ct.continue_step = 1;
  ct.running = 1;
  CU(cudaMemcpyAsync(c->d_ctl, c->h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, c->s));

  c->block = dim3(32, 8);
  c->grid = dim3((h.Nx + 31) / 32, (h.Ny + 7) / 8);
  c->ntiles = (int)(c->grid.x * c->grid.y);
  if (int r = c->alloc(&c->d_lc, 1)) return r;
  if (int r = c->write_mesh()) return r;
  {
    // drag lists: the cells of each flagged body with a fluid neighbour, in WriteDragCoefficient's
    // loop order (i outer, j inner over the p/T solve range, SIMPLE_TS_MPI.cpp:8203-8206)
    std::vector<int> cells, first(1, 0);
    for (int b = 0; b < (int)h.bodies.size(); b++) {
      if (!h.bodies[b].drag) continue;
      for (int i = h.Nx_o[0]; i < h.Nx_o[1]; i++)
        for (int j = h.Ny_o[0]; j < h.Ny_o[1]; j++) {
          const int node = i + j * h.Nx;
          if ((int)h.vol_file[node] - 1 != b) continue;
          const Nb d = neighbours(i, j, h.Nx, h.Ny, false);
          auto fl = [&](int q) { return cls_fluid(h.cls[q]); };
          if (fl(d.ij_1) || fl(d.i_1j) || fl(d.ij1) || fl(d.i1j)) cells.push_back(node);
        }
      c->drag_bodies.push_back(b);
      first.push_back((int)cells.size());
    }
    if (int r = c->alloc(&c->d_drag_cells, cells.size())) return r;
    if (int r = c->alloc(&c->d_drag_first, first.size())) return r;
    if (int r = c->alloc(&c->d_drag_out, 12 * c->drag_bodies.size() + 2)) return r;
    if (int r = c->upload(c->d_drag_cells, cells)) return r;
    if (int r = c->upload(c->d_drag_first, first)) return r;
    if (cf.b("ToSolveContinuityEquation")) {
      if (int r = c->alloc(&c->d_cont_st, Na)) return r;
      if (int r = c->alloc(&c->d_cont, Na)) return r;
    }
  }
  if (int r = c->size_pt_grid()) return r;
  if (opt.autotune) {
    // candidates of the sweep loop: CTAs per SM, times one or two FP32 sweeps per tile load
    c->tune_pt.assign(c->pt_per_sm_max * (c->mixed() ? 2 : 1), sts_ctx::TuneStat{});
    c->tune_asm.assign(3, sts_ctx::TuneStat{});
    c->tune_idx = -1;  // one warm-up step first
    c->tune_left = 1 + sts_ctx::kTuneRounds * std::max((int)c->tune_pt.size(), 3);
  }
  const dim3 G = c->grid, B = c->block;
  cudaStream_t s = c->s;
  k_flux_quotients<<<G, B, 0, s>>>(g);

  // the rest of main() before the time loop (SIMPLE_TS_MPI.cpp:2833-3227), on the device
  if (!h.restart) {
    k_step_begin<<<G, B, 0, s>>>(g, 0, 0, 0);  // *_pr copies
    k_face_rho<<<G, B, 0, s>>>(g);
    c->boundary(PH_VEL);
    k_step_begin<<<G, B, 0, s>>>(g, 0, 0, 0);
    k_face_rho<<<G, B, 0, s>>>(g);
    if (int r = c->write_outputs(!opt.async_save)) return r;  // the set-up save (SIMPLE_TS_MPI.cpp:2863)
  }
  for (double* f : {g.d12, g.d34, g.apx, g.apy, g.bpx, g.bpy, g.Gamma_yf, g.Gamma_xf, g.Fx, g.Fy, g.u_pseudo,
                    g.v_pseudo, g.D_ux, g.D_uy, g.D_vx, g.D_vy, g.DTx, g.DTy, g.ScT1, g.rho_u, g.rho_v})
    CU(cudaMemsetAsync(f, 0, sizeof(double) * Na, s));
  if (!h.restart) c->boundary(PH_PINIT);
  if (cf.b("ToContinueFromInterpolation")) {
    k_apply_bodies<<<G, B, 0, s>>>(g);
    c->boundary(PH_SLIP_U | PH_SLIP_V | PH_TJUMP | PH_TJUMP_WRITE);
  }
  k_sqrt_rho<<<G, B, 0, s>>>(g, 1);
  k_face_rho<<<G, B, 0, s>>>(g);
  k_step_begin<<<G, B, 0, s>>>(g, 0, 0, 0);
  k_sqrt_rho<<<G, B, 0, s>>>(g, 0);
  k_face_rho<<<G, B, 0, s>>>(g);
  c->boundary(PH_SLIP_U | PH_SLIP_V | PH_VEL | PH_PBEGIN | PH_TJUMP | PH_TEMP | PH_PRES);
  k_flux_diff<<<G, B, 0, s>>>(g, 0);
  if (int r = c->check()) return r;
  if (int r = c->read_ctl()) return r;
  *out = c.release();
  return STS_OK;
}

}  // namespace

extern "C" {

void sts_default_options(sts_options* opt) {
  if (!opt) return;
  opt->fixed_sweeps = 1;
  opt->use_graph = 1;
  opt->device = 0;
  opt->write_files = 1;
  opt->precision = 0;
  opt->warm_start = 0;
  opt->async_save = 1;
  opt->autotune = 1;
}

int sts_open_case(const char* case_dir, const sts_options* opt, sts_ctx** out) {
  g_err.clear();
  if (out) *out = nullptr;
  sts_options o;
  sts_default_options(&o);
  if (opt) o = *opt;
  o.write_files = opt ? opt->write_files : 0;
  return open_impl(case_dir, &o, out);
}

// sts_step; with state_out (device addresses of host buffers), the graph launch is followed by the
// move of the new state into those buffers before its synchronisation, and *moved says whether
// that happened (the autotuner's steps, launched one by one, or a run that had ended, leave it to
// the caller).
// state_in (with state_out, one step in the graph): the state is read from those buffers in the step's
// first kernel; *moved tells whether the step's graph ran with the buffers.
static int step_impl(sts_ctx* ctx, int nsteps, int* steps_done, double* const* state_out, bool* moved,
                     const double* const* state_in = nullptr) {
  if (moved) *moved = false;
  int done = 0;
  if (!ctx->finished && nsteps > 0) {
    CU(cudaSetDevice(ctx->opt.device));
    const unsigned status_before = ctx->h_ctl->status;
    // the autotuner's steps come first (real steps, launched kernel by kernel)
    while (ctx->tune_left > 0 && done < nsteps && !ctx->finished) {
      int d = 0;
      if (int r = ctx->tune_step(&d)) return r;
      done += d;
      if (!ctx->h_ctl->continue_step) ctx->finished = true;
      if (ctx->h_ctl->status & (ST_BARRIER_TIMEOUT | ST_NONFINITE)) break;
    }
    if (done < nsteps && !ctx->finished && !(ctx->h_ctl->status & ~status_before & (ST_BARRIER_TIMEOUT | ST_NONFINITE))) {
      int d = 0;
      int r = ctx->opt.use_graph ? ctx->step_graph(nsteps - done, &d, state_out, state_in) : ctx->step_host(nsteps - done, &d);
      if (r) return r;
      if (ctx->opt.use_graph && state_out && moved) *moved = true;
      done += d;
    }
    if (!ctx->h_ctl->continue_step) ctx->finished = true;
    if (ctx->h_ctl->status & ST_BARRIER_TIMEOUT) {
      ctx->finished = true;  // the device state is no longer consistent
      return fail(STS_ERR_TIMEOUT, "a grid barrier of the sweep loop timed out");
    }
    if (ctx->h_ctl->status & ~status_before & ST_NONFINITE) {
      if (steps_done) *steps_done = done;
      return fail(STS_ERR_NONFINITE, "a residual became NaN or Inf");
    }
  }
  if (steps_done) *steps_done = done;
  return STS_OK;
}

int sts_step(sts_ctx* ctx, int nsteps, int* steps_done) {
  if (!ctx || nsteps < 0) return fail(STS_ERR_ARG, "bad argument");
  if (ctx->in_batch) return fail(STS_ERR_ARG, "the case belongs to a batch: step it with sts_batch_step");
  return step_impl(ctx, nsteps, steps_done, nullptr, nullptr);
}

int sts_step_timed(sts_ctx* ctx, int nsteps, int* steps_done, double* device_ms) {
  if (!ctx || nsteps < 0) return fail(STS_ERR_ARG, "bad argument");
  CU(cudaSetDevice(ctx->opt.device));
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  CU(cudaEventRecord(a, ctx->s));
  int done = 0;
  int r = sts_step(ctx, nsteps, &done);
  cudaEventRecord(b, ctx->s);
  cudaEventSynchronize(b);
  float t = 0;
  cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (device_ms) *device_ms = t;
  if (steps_done) *steps_done = done;
  return r;
}

int sts_profile_steps(sts_ctx* ctx, int nsteps, double* kernel_ms, int* kernel_launches, int* steps_done) {
  if (!ctx || nsteps < 0 || !kernel_ms || !kernel_launches) return fail(STS_ERR_ARG, "bad argument");
  if (ctx->in_batch) return fail(STS_ERR_ARG, "the case belongs to a batch");
  CU(cudaSetDevice(ctx->opt.device));
  int done = 0;
  if (ctx->finished) {
    for (int q = 0; q < kProfileKinds; q++) { kernel_ms[q] = 0; kernel_launches[q] = 0; }
  } else if (int r = ctx->profile(nsteps, kernel_ms, kernel_launches, &done)) {
    return r;
  }
  if (ctx->h_ctl->status & ST_BARRIER_TIMEOUT) {
    ctx->finished = true;
    return fail(STS_ERR_TIMEOUT, "a grid barrier of the sweep loop timed out");
  }
  if (!ctx->h_ctl->continue_step) ctx->finished = true;
  if (steps_done) *steps_done = done;
  return STS_OK;
}

int sts_get_field(sts_ctx* ctx, const char* name, double* out) {
  if (!ctx || !name || !out) return fail(STS_ERR_ARG, "null argument");
  CU(cudaSetDevice(ctx->opt.device));
  // which p/T buffer is current: every step of a single context ends with its control block read
  // back; a batch's case is refreshed here
  if (ctx->in_batch)
    if (int r = ctx->read_ctl()) return r;
  const Geo& g = ctx->g;
  const std::string n(name);
  const unsigned cur = ctx->h_ctl->cur;
  const double* src = nullptr;
  if (n == "hx") { std::memcpy(out, ctx->hc.hx.data(), sizeof(double) * g.Nx); return STS_OK; }
  if (n == "hy") { std::memcpy(out, ctx->hc.hy.data(), sizeof(double) * g.Ny); return STS_OK; }
  if (n == "x_v") { std::memcpy(out, ctx->hc.x_v.data(), sizeof(double) * g.Nx); return STS_OK; }
  if (n == "y_v") { std::memcpy(out, ctx->hc.y_v.data(), sizeof(double) * g.Ny); return STS_OK; }
  struct { const char* k; const double* p; } tab[] = {
      {"u", g.u}, {"v", g.v}, {"p", g.p[cur]}, {"T", g.T[cur]}, {"rho", g.rho}, {"sqrt_T", g.sqrt_T},
      {"p_pr", g.p_pr}, {"T_pr", g.T_pr}, {"u_pr", g.u_pr}, {"v_pr", g.v_pr}, {"rho_pr", g.rho_pr},
      {"rho_u", g.rho_u}, {"rho_v", g.rho_v}, {"Fx", g.Fx}, {"Fy", g.Fy}, {"D_ux", g.D_ux}, {"D_uy", g.D_uy},
      {"D_vx", g.D_vx}, {"D_vy", g.D_vy}, {"DTx", g.DTx}, {"DTy", g.DTy}, {"Gamma_xf", g.Gamma_xf},
      {"Gamma_yf", g.Gamma_yf}, {"ScT1", g.ScT1}, {"apx", g.apx}, {"apy", g.apy}, {"bpx", g.bpx}, {"bpy", g.bpy},
      {"u_pseudo", g.u_pseudo}, {"v_pseudo", g.v_pseudo}, {"d_p_c_12", g.d12}, {"d_p_c_34", g.d34},
      {"Tw_u", g.Tw_u}, {"Tw_v", g.Tw_v}};
  for (auto& t : tab)
    if (n == t.k) src = t.p;
  if (!src) return fail(STS_ERR_ARG, "unknown field " + n);
  CU(cudaMemcpyAsync(out, src, sizeof(double) * g.Na, cudaMemcpyDeviceToHost, ctx->s));
  CU(cudaStreamSynchronize(ctx->s));
  return STS_OK;
}

int sts_set_field(sts_ctx* ctx, const char* name, const double* in) {
  if (!ctx || !name || !in) return fail(STS_ERR_ARG, "null argument");
  CU(cudaSetDevice(ctx->opt.device));
  if (ctx->in_batch)
    if (int r = ctx->read_ctl()) return r;
  const Geo& g = ctx->g;
  const std::string n(name);
  const unsigned cur = ctx->h_ctl->cur;
  double* dst = nullptr;
  if (n == "u") dst = g.u;
  else if (n == "v") dst = g.v;
  else if (n == "p") dst = g.p[cur];
  else if (n == "T") dst = g.T[cur];
  if (!dst) return fail(STS_ERR_ARG, "field cannot be set: " + n);
  CU(cudaMemcpyAsync(dst, in, sizeof(double) * g.Na, cudaMemcpyHostToDevice, ctx->s));
  if (g.warm_start && (n == "p" || n == "T")) {
    // the warm start's history no longer describes the state: it starts over
    static const unsigned zero = 0;
    CU(cudaMemcpyAsync(&g.ctl->warm_ready, &zero, sizeof(unsigned), cudaMemcpyHostToDevice, ctx->s));
  }
  CU(cudaStreamSynchronize(ctx->s));
  return STS_OK;
}

// Device addresses of host buffers the device can read and write directly (memory pinned by
// cudaHostAlloc / cudaMallocHost or registered with cudaHostRegister); false for any other
// memory, which then goes through the copy engines.
static bool mapped_host(const void* const* ptrs, void** dev, int n) {
  for (int k = 0; k < n; k++) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, ptrs[k]) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
    dev[k] = a.devicePointer;
  }
  return true;
}

// 256-thread CTAs, at most four per multiprocessor (a grid-stride pass covers the rest)
static int move_grid(int n, int sms) { return std::max(1, std::min((n + 255) / 256, 4 * std::max(sms, 1))); }

// sts_set_state's work queued on the context's stream, without its synchronisation.
static int set_state_queue(sts_ctx* ctx, const double* u_in, const double* v_in, const double* p_in,
                           const double* T_in) {
  const Geo& g = ctx->g;
  const unsigned cur = ctx->h_ctl->cur;
  const size_t bytes = sizeof(double) * g.Na;
  const void* hp[4] = {u_in, v_in, p_in, T_in};
  void* dp[4];
  if (mapped_host(hp, dp, 4)) {
    k_move4<<<move_grid(g.Na, ctx->sms), 256, 0, ctx->s>>>((const double*)dp[0], (const double*)dp[1], (const double*)dp[2],
                                                 (const double*)dp[3], g.u, g.v, g.p[cur], g.T[cur], g.Na);
    CU(cudaGetLastError());
  } else {
    CU(cudaMemcpyAsync(g.u, u_in, bytes, cudaMemcpyHostToDevice, ctx->s));
    CU(cudaMemcpyAsync(g.v, v_in, bytes, cudaMemcpyHostToDevice, ctx->s));
    CU(cudaMemcpyAsync(g.p[cur], p_in, bytes, cudaMemcpyHostToDevice, ctx->s));
    CU(cudaMemcpyAsync(g.T[cur], T_in, bytes, cudaMemcpyHostToDevice, ctx->s));
  }
  if (g.warm_start) {
    static const unsigned zero = 0;
    CU(cudaMemcpyAsync(&g.ctl->warm_ready, &zero, sizeof(unsigned), cudaMemcpyHostToDevice, ctx->s));
  }
  return STS_OK;
}

int sts_set_state(sts_ctx* ctx, const double* u_in, const double* v_in, const double* p_in, const double* T_in) {
  if (!ctx || !u_in || !v_in || !p_in || !T_in) return fail(STS_ERR_ARG, "null argument");
  CU(cudaSetDevice(ctx->opt.device));
  if (ctx->in_batch)
    if (int r = ctx->read_ctl()) return r;
  if (int r = set_state_queue(ctx, u_in, v_in, p_in, T_in)) return r;
  CU(cudaStreamSynchronize(ctx->s));
  return STS_OK;
}

int sts_get_state(sts_ctx* ctx, double* u_out, double* v_out, double* p_out, double* T_out) {
  if (!ctx || !u_out || !v_out || !p_out || !T_out) return fail(STS_ERR_ARG, "null argument");
  CU(cudaSetDevice(ctx->opt.device));
  if (ctx->in_batch)
    if (int r = ctx->read_ctl()) return r;
  const Geo& g = ctx->g;
  const unsigned cur = ctx->h_ctl->cur;
  const size_t bytes = sizeof(double) * g.Na;
  const void* hp[4] = {u_out, v_out, p_out, T_out};
  void* dp[4];
  if (mapped_host(hp, dp, 4)) {
    k_move4<<<move_grid(g.Na, ctx->sms), 256, 0, ctx->s>>>(g.u, g.v, g.p[cur], g.T[cur], (double*)dp[0], (double*)dp[1],
                                                 (double*)dp[2], (double*)dp[3], g.Na);
    CU(cudaGetLastError());
  } else {
    CU(cudaMemcpyAsync(u_out, g.u, bytes, cudaMemcpyDeviceToHost, ctx->s));
    CU(cudaMemcpyAsync(v_out, g.v, bytes, cudaMemcpyDeviceToHost, ctx->s));
    CU(cudaMemcpyAsync(p_out, g.p[cur], bytes, cudaMemcpyDeviceToHost, ctx->s));
    CU(cudaMemcpyAsync(T_out, g.T[cur], bytes, cudaMemcpyDeviceToHost, ctx->s));
  }
  CU(cudaStreamSynchronize(ctx->s));
  return STS_OK;
}

int sts_step_exchange(sts_ctx* ctx, int nsteps, const double* u_in, const double* v_in, const double* p_in,
                      const double* T_in, double* u_out, double* v_out, double* p_out, double* T_out,
                      int* steps_done) {
  if (!ctx || nsteps < 0 || !u_in || !v_in || !p_in || !T_in || !u_out || !v_out || !p_out || !T_out)
    return fail(STS_ERR_ARG, "bad argument");
  if (ctx->in_batch) return fail(STS_ERR_ARG, "the case belongs to a batch: step it with sts_batch_step");
  if (steps_done) *steps_done = 0;
  CU(cudaSetDevice(ctx->opt.device));
  const void* hout[4] = {u_out, v_out, p_out, T_out};
  const void* hin[4] = {u_in, v_in, p_in, T_in};
  void *dout[4], *din[4];
  const bool direct = mapped_host(hout, dout, 4);
  // one step in the exchange graph, both sides device-addressable: the state comes in in the
  // step's first kernel, otherwise ahead of the step
  const bool fused_in = direct && nsteps == 1 && ctx->opt.use_graph && ctx->tune_left == 0 && !ctx->finished &&
                        ctx->xout_in_graph() && mapped_host(hin, din, 4);
  if (fused_in) {
    if (ctx->g.warm_start) {  // as sts_set_state: the warm start's history begins again
      static const unsigned zero = 0;
      CU(cudaMemcpyAsync(&ctx->g.ctl->warm_ready, &zero, sizeof(unsigned), cudaMemcpyHostToDevice, ctx->s));
    }
  } else if (int r = set_state_queue(ctx, u_in, v_in, p_in, T_in)) {
    return r;
  }
  bool moved = false;
  const int r = step_impl(ctx, nsteps, steps_done, direct ? (double* const*)dout : nullptr, &moved,
                          fused_in ? (const double* const*)din : nullptr);
  if (r != STS_OK && r != STS_ERR_NONFINITE) return r;
  if (!moved) {
    if (fused_in)  // no step ran: the state still goes in
      if (int q = set_state_queue(ctx, u_in, v_in, p_in, T_in)) return q;
    CU(cudaStreamSynchronize(ctx->s));  // the inputs are read (a run that had ended takes no step)
    if (int q = sts_get_state(ctx, u_out, v_out, p_out, T_out)) return q;
  }
  return r;
}

int sts_dims(sts_ctx* ctx, int* Nx, int* Ny) {
  if (!ctx) return fail(STS_ERR_ARG, "null context");
  if (Nx) *Nx = ctx->g.Nx;
  if (Ny) *Ny = ctx->g.Ny;
  return STS_OK;
}

int sts_stats(sts_ctx* ctx, double* out) {
  if (!ctx || !out) return fail(STS_ERR_ARG, "null argument");
  if (int r = ctx->read_ctl()) return r;
  const Ctl& c = *ctx->h_ctl;
  const unsigned I = c.Iter ? (c.Iter - 1 < 64 ? c.Iter - 1 : 63) : 0;
  out[0] = c.Iter; out[1] = c.Iter_p_c; out[2] = c.res_p0[I]; out[3] = c.res_p[I]; out[4] = c.res_T0[I];
  out[5] = c.res_T[I]; out[6] = c.res_u; out[7] = c.res_v; out[8] = c.it;
  return STS_OK;
}

int sts_sweep_history(sts_ctx* ctx, unsigned int* out, int cap, int* n_out) {
  if (!ctx || !out || cap < 0) return fail(STS_ERR_ARG, "bad argument");
  if (int r = ctx->read_ctl()) return r;
  const Ctl& c = *ctx->h_ctl;
  const unsigned avail = c.hist_n < 4096u ? c.hist_n : 4096u;
  const unsigned n = (unsigned)cap < avail ? (unsigned)cap : avail;
  for (unsigned k = 0; k < n; k++) out[k] = c.hist_sweeps[(c.hist_n - n + k) % 4096u];
  if (n_out) *n_out = (int)n;
  return STS_OK;
}

int sts_autotune_result(sts_ctx* ctx, int* steps_left, int* ctas_per_sm, int* asm_block_x, int* asm_block_y) {
  if (!ctx) return fail(STS_ERR_ARG, "null context");
  if (steps_left) *steps_left = ctx->tune_left;
  if (ctas_per_sm) *ctas_per_sm = ctx->pt_per_sm > 0 ? ctx->pt_per_sm : ctx->pt_per_sm_max;
  if (asm_block_x) *asm_block_x = (int)ctx->asm_block.x;
  if (asm_block_y) *asm_block_y = (int)ctx->asm_block.y;
  return STS_OK;
}

int sts_write_outputs(sts_ctx* ctx) {
  if (!ctx) return fail(STS_ERR_ARG, "null context");
  CU(cudaSetDevice(ctx->opt.device));
  const int w = ctx->opt.write_files;
  ctx->opt.write_files = 1;
  const int r = ctx->write_outputs(true);
  ctx->opt.write_files = w;
  return r;
}

int sts_write_outputs_async(sts_ctx* ctx) {
  if (!ctx) return fail(STS_ERR_ARG, "null context");
  if (ctx->in_batch) return fail(STS_ERR_ARG, "the case belongs to a batch");
  CU(cudaSetDevice(ctx->opt.device));
  const int w = ctx->opt.write_files;
  ctx->opt.write_files = 1;
  const int r = ctx->write_outputs(false);
  ctx->opt.write_files = w;
  return r;
}

int sts_wait_outputs(sts_ctx* ctx) {
  if (!ctx) return fail(STS_ERR_ARG, "null context");
  CU(cudaSetDevice(ctx->opt.device));
  return ctx->wait_outputs();
}

int sts_run_case(const char* case_dir, const sts_options* opt) {
  sts_options o;
  sts_default_options(&o);
  if (opt) o = *opt;
  sts_ctx* ctx = nullptr;
  g_err.clear();
  const time_t time_solve_start = time(nullptr);  // SIMPLE_TS_MPI.cpp:1799
  if (int r = open_impl(case_dir, &o, &ctx)) return r;
  std::unique_ptr<sts_ctx> guard(ctx);
  const Config& cf = ctx->hc.cfg;
  // The reference's wall-clock limit: the run ends after the first step that ends at or after
  // time_solve_stop = start + max_time_for_solve hours (SIMPLE_TS_MPI.cpp:2010, :4443).  The host
  // checks it between chunks of steps; a chunk is cut to the steps that fit in the time left
  // (one step once the limit is closer than a step), so the run stops at the reference's step up
  // to the resolution of time(NULL).
  const double time_solve_stop = (double)time_solve_start + cf.d("max_time_for_solve") * 3600.0;
  double s_per_step = 0;  // wall seconds per step, from the last chunk
  const long save_every = cf.n("Nt_save_solved_data") > 0 ? cf.n("Nt_save_solved_data") : 1;
  const long log_every = cf.n("Nt_save_temp_data") > 0 ? cf.n("Nt_save_temp_data") : 1;
  const long drag_every = cf.n("Nt_save_DragCoefficient") > 0 ? cf.n("Nt_save_DragCoefficient") : 1;
  const bool cont = cf.b("ToSolveContinuityEquation");
  // the continuity dumps of every step's last outer iteration (SIMPLE_TS_MPI.cpp:4588-4591) only
  // outlive the step when they go to per-step files
  const bool cont_each_step = cont && cf.b("ToWriteSolvedDataToNewFiles");
  long save_c = 0, log_c = 0, drag_c = 0;
  while (!ctx->finished) {
    long chunk = std::min(save_every - save_c, std::min(log_every - log_c, drag_every - drag_c));
    if (cont_each_step) chunk = 1;
    {
      const double left = time_solve_stop - (double)time(nullptr);
      if (left <= 0 || s_per_step <= 0) chunk = 1;
      else chunk = std::max(1L, std::min(chunk, (long)(left / s_per_step)));
    }
    int done = 0;
    const auto c0 = std::chrono::steady_clock::now();
    const int r = sts_step(ctx, (int)chunk, &done);
    if (r && r != STS_ERR_NONFINITE) return r;
    if (done > 0) s_per_step = std::chrono::duration<double>(std::chrono::steady_clock::now() - c0).count() / done;
    save_c += done;
    log_c += done;
    drag_c += done;
    // the reference's order after a step: saves (with the continuity dumps), drag, logs
    if (cont_each_step && done > 0 && save_c < save_every)
      if (int q = ctx->continuity()) return q;
    if (save_c >= save_every) {
      if (int q = ctx->write_outputs(!o.async_save)) return q;
      if (cont)
        if (int q = ctx->continuity()) return q;
      save_c = 0;
    }
    if (drag_c >= drag_every) {
      if (int q = ctx->write_drag()) return q;
      drag_c = 0;
    }
    if (log_c >= log_every) {
      if (int q = ctx->write_logs()) return q;
      log_c = 0;
    }
    if (done == 0) break;
    if ((double)time(nullptr) >= time_solve_stop) break;  // SIMPLE_TS_MPI.cpp:4443
  }
  // after the loop (SIMPLE_TS_MPI.cpp:4695-4714)
  const double hours = std::chrono::duration<double>(std::chrono::steady_clock::now() - ctx->t0).count() / 3600.0;
  ctx->hc.cfg.set("max_time_for_solve", hours);
  if (int q = ctx->write_outputs(true)) return q;  // also waits for the periodic saves
  if (cont)
    if (int q = ctx->continuity()) return q;
  if (int q = ctx->write_drag()) return q;
  if (int q = ctx->write_logs(false)) return q;  // the final log writes Tmp.txt only (SIMPLE_TS_MPI.cpp:4714)
  return STS_OK;
}

int sts_pt_sweeps(const sts_sweep_fields* f, int max_sweeps, int fixed_sweeps, double tol_p, double tol_T,
                  void* stream, int* sweeps_done, double* res_p, double* res_T) {
  g_err.clear();
  if (int r = check_sweep_args(f, max_sweeps)) return r;
  cudaStream_t s = (cudaStream_t)stream;
  char* scratch = nullptr;
  CU(cudaMallocAsync((void**)&scratch, scratch_bytes((size_t)f->Nx * f->Ny), s));
  const int r = pt_sweeps_on(f, max_sweeps, fixed_sweeps, tol_p, tol_T, s, scratch, sweeps_done, res_p, res_T);
  cudaFreeAsync(scratch, s);
  cudaStreamSynchronize(s);
  return r;
}

}  // extern "C"

namespace {

// Scratch of sts_pt_sweeps_noalloc: one fixed array per GPU that loads the library, laid out
// like the allocated scratch of sts_pt_sweeps (control block, then 10 fields of Nx*Ny doubles).
constexpr size_t kNoAllocBytes = sizeof(Ctl) + 256 + 10 * (size_t)STS_NOALLOC_MAX_CELLS * sizeof(double);
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch on the current device.  In host code the array's name only
// stands in for the symbol; it is not a device address.  The address is looked up on every call
// (cudaGetSymbolAddress is cheap) so that a device reset or another context never leaves a stale
// pointer behind.
int noalloc_scratch(char** out) {
  void* p = nullptr;
  CU(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  *out = (char*)p;
  return STS_OK;
}

}  // namespace

extern "C" {

int sts_pt_sweeps_noalloc(const sts_sweep_fields* f, int max_sweeps, int fixed_sweeps, double tol_p, double tol_T,
                          void* stream, int* sweeps_done, double* res_p, double* res_T) {
  g_err.clear();
  if (int r = check_sweep_args(f, max_sweeps)) return r;
  if ((size_t)f->Nx * (size_t)f->Ny > (size_t)STS_NOALLOC_MAX_CELLS)
    return fail(STS_ERR_ARG, "mesh of " + std::to_string((size_t)f->Nx * f->Ny) +
                                 " cells exceeds the no-allocation limit of " + std::to_string(STS_NOALLOC_MAX_CELLS) +
                                 " cells; use sts_pt_sweeps");
  char* scratch = nullptr;
  if (int r = noalloc_scratch(&scratch)) return r;
  return pt_sweeps_on(f, max_sweeps, fixed_sweeps, tol_p, tol_T, (cudaStream_t)stream, scratch, sweeps_done, res_p,
                      res_T);
}

int sts_conservation(sts_ctx* ctx, double* out5) {
  if (!ctx || !out5) return fail(STS_ERR_ARG, "null argument");
  CU(cudaSetDevice(ctx->opt.device));
  const Geo& g = ctx->g;
  const int nch = (g.Nx + kConsChunk - 1) / kConsChunk;
  if (!ctx->d_cons_part) {
    if (int r = ctx->alloc(&ctx->d_cons_part, (size_t)g.Ny * nch * kConsQ)) return r;
    if (int r = ctx->alloc(&ctx->d_cons_rows, (size_t)g.Ny * kConsQ)) return r;
    if (int r = ctx->alloc(&ctx->d_cons_out, (size_t)kConsQ)) return r;
  }
  k_cons_partial<<<dim3((nch + 31) / 32, g.Ny), 32, 0, ctx->s>>>(g, ctx->h_ctl->cur, ctx->d_cons_part, nch);
  k_cons_final<<<1, 256, 0, ctx->s>>>(g.Ny, nch, ctx->d_cons_part, ctx->d_cons_rows, ctx->d_cons_out);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(out5, ctx->d_cons_out, sizeof(double) * kConsQ, cudaMemcpyDeviceToHost, ctx->s));
  CU(cudaStreamSynchronize(ctx->s));
  return STS_OK;
}

int sts_set_sweep_blocking(sts_ctx* ctx, int k) {
  if (!ctx || k < 0 || k > 2) return fail(STS_ERR_ARG, "k must be 0, 1 or 2");
  if (k == 2 && !ctx->tb_available())
    return fail(STS_ERR_ARG, "two sweeps per tile load need a single case with FP32 correction sweeps");
  CU(cudaSetDevice(ctx->opt.device));
  CU(cudaStreamSynchronize(ctx->s));
  ctx->pt_tb_forced = k;
  if (k) ctx->pt_tb = k;
  if (int r = ctx->size_pt_grid()) return r;
  ctx->drop_graphs();  // the graphs are rebuilt with the new sweep-loop kernel at the next step
  return STS_OK;
}

int sts_get_sweep_blocking(sts_ctx* ctx, int* k) {
  if (!ctx || !k) return fail(STS_ERR_ARG, "null argument");
  *k = ctx->tb_on() ? 2 : 1;
  return STS_OK;
}

int sts_warm_net_train(sts_ctx* ctx, int iters, float lr, float* loss_out) {
  if (!ctx || iters < 0) return fail(STS_ERR_ARG, "bad argument");
  if (!ctx->warm_net) return fail(STS_ERR_ARG, "the context does not use warm_start 5");
  CU(cudaSetDevice(ctx->opt.device));
  NetState h{};
  CU(cudaMemcpyAsync(&h, ctx->d_ns, sizeof(NetState), cudaMemcpyDeviceToHost, ctx->s));
  CU(cudaStreamSynchronize(ctx->s));
  // completed pairs: slots 0 .. count-1, or the whole ring but the slot being filled
  const int B = sts_ctx::kNetBatch, S = ctx->net_slots;
  const int n = (int)std::min<unsigned>(h.count, (unsigned)S);
  if (n < 1) return fail(STS_ERR_ARG, "no training pairs yet: step the case first");
  const int pending = h.have_win ? h.slot : -1;
  const int px = ctx->nb.H * ctx->nb.W;
  float loss = 0.f;
  for (int it = 0; it < iters; it++) {
    int slots[sts_ctx::kNetBatch];
    for (int b = 0; b < B; b++) {
      int q;
      do {
        ctx->net_rng = ctx->net_rng * 6364136223846793005ull + 1442695040888963407ull;
        q = (int)((ctx->net_rng >> 33) % (unsigned long long)n);
      } while (n > 1 && q == pending && h.count >= (unsigned)S);
      slots[b] = q;
    }
    CU(cudaMemcpyAsync(ctx->d_bslots, slots, sizeof(slots), cudaMemcpyHostToDevice, ctx->s));
    k_net_batch<<<std::max(1, std::min((B * px + 255) / 256, 4096)), 256, 0, ctx->s>>>(ctx->nb, ctx->d_bslots, B,
                                                                                     ctx->d_bx, ctx->d_bt, ctx->d_bw);
    CU(ctx->net->forward(ctx->d_bx, B, nullptr));
    CU(ctx->net->backward_mse(ctx->d_bt, ctx->d_bw, B, ctx->d_loss));
    CU(ctx->net->adam(lr));
    if (it + 1 == iters) CU(cudaMemcpyAsync(&loss, ctx->d_loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->s));
    CU(cudaStreamSynchronize(ctx->s));  // the slot list on the host stack is reused
  }
  unsigned e = 0;
  CU(cudaMemcpy(&e, ctx->net->error_flag(), sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (e) return fail(STS_ERR_TIMEOUT, "a tensor-core GEMM pipeline wait gave up");
  if (loss_out) *loss_out = loss;
  return STS_OK;
}

int sts_warm_net_eval(sts_ctx* ctx, float* loss_net, float* loss_zero) {
  if (!ctx || !ctx->warm_net) return fail(STS_ERR_ARG, "the context does not use warm_start 5");
  CU(cudaSetDevice(ctx->opt.device));
  NetState h{};
  CU(cudaMemcpyAsync(&h, ctx->d_ns, sizeof(NetState), cudaMemcpyDeviceToHost, ctx->s));
  CU(cudaStreamSynchronize(ctx->s));
  const int B = sts_ctx::kNetBatch, S = ctx->net_slots;
  const int n = (int)std::min<unsigned>(h.count, (unsigned)S);
  const int pending = (h.have_win && h.count >= (unsigned)S) ? h.slot : -1;
  const int px = ctx->nb.H * ctx->nb.W;
  double sn = 0, sz = 0;
  int batches = 0;
  for (int q0 = 0; q0 < n; q0 += B) {
    int slots[sts_ctx::kNetBatch];
    int m = 0;
    for (int q = q0; q < n && m < B; q++)
      if (q != pending) slots[m++] = q;
    if (m == 0) continue;
    for (int b = m; b < B; b++) slots[b] = slots[b % m];  // a short last batch repeats its pairs
    CU(cudaMemcpyAsync(ctx->d_bslots, slots, sizeof(slots), cudaMemcpyHostToDevice, ctx->s));
    k_net_batch<<<std::max(1, std::min((B * px + 255) / 256, 4096)), 256, 0, ctx->s>>>(ctx->nb, ctx->d_bslots, B,
                                                                                     ctx->d_bx, ctx->d_bt, ctx->d_bw);
    float l[2] = {0.f, 0.f};
    CU(ctx->net->forward(ctx->d_bx, B, nullptr));
    CU(ctx->net->loss(ctx->d_bt, ctx->d_bw, B, ctx->d_loss, false));
    CU(cudaMemcpyAsync(&l[0], ctx->d_loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->s));
    CU(ctx->net->loss(ctx->d_bt, ctx->d_bw, B, ctx->d_loss, true));
    CU(cudaMemcpyAsync(&l[1], ctx->d_loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->s));
    CU(cudaStreamSynchronize(ctx->s));
    sn += l[0];
    sz += l[1];
    batches++;
  }
  if (!batches) return fail(STS_ERR_ARG, "no training pairs yet: step the case first");
  if (loss_net) *loss_net = (float)(sn / batches);
  if (loss_zero) *loss_zero = (float)(sz / batches);
  return STS_OK;
}

int sts_warm_net_enable(sts_ctx* ctx, int on) {
  if (!ctx || !ctx->warm_net) return fail(STS_ERR_ARG, "the context does not use warm_start 5");
  CU(cudaSetDevice(ctx->opt.device));
  const unsigned v = on ? 1u : 0u;
  CU(cudaMemcpyAsync(&ctx->d_ns->enabled, &v, sizeof(unsigned), cudaMemcpyHostToDevice, ctx->s));
  CU(cudaStreamSynchronize(ctx->s));
  return STS_OK;
}

int sts_warm_net_info(sts_ctx* ctx, int* pairs, int* win_h, int* win_w, long long* nparams) {
  if (!ctx || !ctx->warm_net) return fail(STS_ERR_ARG, "the context does not use warm_start 5");
  CU(cudaSetDevice(ctx->opt.device));
  NetState h{};
  CU(cudaMemcpyAsync(&h, ctx->d_ns, sizeof(NetState), cudaMemcpyDeviceToHost, ctx->s));
  CU(cudaStreamSynchronize(ctx->s));
  if (pairs) *pairs = (int)h.count;
  if (win_h) *win_h = ctx->nb.H;
  if (win_w) *win_w = ctx->nb.W;
  if (nparams) *nparams = ctx->net->param_count();
  return STS_OK;
}

int sts_warm_net_gate(sts_ctx* ctx, int* steps_on_p, int* steps_on_T) {
  if (!ctx || !ctx->warm_net) return fail(STS_ERR_ARG, "the context does not use warm_start 5");
  CU(cudaSetDevice(ctx->opt.device));
  NetState h{};
  CU(cudaMemcpyAsync(&h, ctx->d_ns, sizeof(NetState), cudaMemcpyDeviceToHost, ctx->s));
  CU(cudaStreamSynchronize(ctx->s));
  if (steps_on_p) *steps_on_p = (int)h.steps_on[0];
  if (steps_on_T) *steps_on_T = (int)h.steps_on[1];
  return STS_OK;
}

int sts_warm_net_params(sts_ctx* ctx, float* out, const float* in) {
  if (!ctx || !ctx->warm_net) return fail(STS_ERR_ARG, "the context does not use warm_start 5");
  CU(cudaSetDevice(ctx->opt.device));
  if (out) CU(ctx->net->get_params(out));
  if (in) CU(ctx->net->set_params(in));
  return STS_OK;
}

int sts_sync(sts_ctx* ctx) {
  if (!ctx) return fail(STS_ERR_ARG, "null context");
  CU(cudaStreamSynchronize(ctx->s));
  return STS_OK;
}

void sts_destroy(sts_ctx* ctx) {
  if (ctx && !ctx->in_batch) delete ctx;  // a batch's cases are released with the batch
}

const char* sts_last_error(void) { return g_err.c_str(); }

int sts_inspect_case(const char* case_dir, int* Nx, int* Ny, unsigned int* vol_out, unsigned char* cls_out,
                     double* hx_out, double* hy_out, double* xv_out, double* yv_out) {
  if (!case_dir) return fail(STS_ERR_ARG, "null argument");
  Case h;
  std::string err;
  if (!load_case(case_dir, true, h, err)) return fail(STS_ERR_INPUT, err);
  if (Nx) *Nx = h.Nx;
  if (Ny) *Ny = h.Ny;
  if (vol_out) std::memcpy(vol_out, h.vol_id.data(), sizeof(unsigned) * h.Na);
  if (cls_out) std::memcpy(cls_out, h.cls.data(), h.Na);
  if (hx_out) std::memcpy(hx_out, h.hx.data(), sizeof(double) * h.Nx);
  if (hy_out) std::memcpy(hy_out, h.hy.data(), sizeof(double) * h.Ny);
  if (xv_out) std::memcpy(xv_out, h.x_v.data(), sizeof(double) * h.Nx);
  if (yv_out) std::memcpy(yv_out, h.y_v.data(), sizeof(double) * h.Ny);
  return STS_OK;
}

int sts_check_double_float(unsigned long long n, unsigned long long seed, int device, double* max_rel_err) {
  if (!max_rel_err) return fail(STS_ERR_ARG, "null argument");
  CU(cudaSetDevice(device));
  unsigned long long* d = nullptr;
  CU(cudaMalloc(&d, 5 * sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(d, 0, 5 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    k_check_df<<<1216, 256>>>(n, seed, d);
    e = cudaGetLastError();
  }
  unsigned long long h[5] = {0, 0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(STS_ERR_CUDA, std::string("sts_check_double_float: ") + cudaGetErrorString(e));
  for (int q = 0; q < 5; q++) std::memcpy(&max_rel_err[q], &h[q], sizeof(double));
  return STS_OK;
}

int sts_check_division(unsigned long long n, unsigned long long seed, int device, unsigned long long* mismatches) {
  if (!mismatches) return fail(STS_ERR_ARG, "null argument");
  CU(cudaSetDevice(device));
  unsigned long long* d = nullptr;
  CU(cudaMalloc(&d, sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(d, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) {
    k_check_division<<<1216, 256>>>(n, seed, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(mismatches, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(STS_ERR_CUDA, std::string("sts_check_division: ") + cudaGetErrorString(e));
  return STS_OK;
}

int sts_check_barrier_timeout(int device, int skip_cta, unsigned spin_limit, int rounds) {
  if (rounds < 1 || spin_limit < 1) return fail(STS_ERR_ARG, "bad argument");
  CU(cudaSetDevice(device));
  int sms = 0;
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  if (skip_cta >= sms) return fail(STS_ERR_ARG, "skip_cta beyond the grid (one CTA per multiprocessor)");
  LoopCtl* lc = nullptr;
  CU(cudaMalloc(&lc, sizeof(LoopCtl)));
  LoopCtl h{};
  cudaError_t e = cudaMemset(lc, 0, sizeof(LoopCtl));
  if (e == cudaSuccess) {
    void* args[] = {(void*)&lc, (void*)&skip_cta, (void*)&spin_limit, (void*)&rounds};
    e = cudaLaunchCooperativeKernel((const void*)k_barrier_probe, dim3(sms), dim3(32, 8), args, 0, nullptr);
  }
  if (e == cudaSuccess) e = cudaMemcpy(&h, lc, sizeof(LoopCtl), cudaMemcpyDeviceToHost);
  cudaFree(lc);
  if (e != cudaSuccess) return fail(STS_ERR_CUDA, std::string("sts_check_barrier_timeout: ") + cudaGetErrorString(e));
  if (h.status & ST_BARRIER_TIMEOUT) return fail(STS_ERR_TIMEOUT, "a grid barrier timed out");
  return STS_OK;
}

int sts_fp64_rates(int device, double* gops) {
  if (!gops) return fail(STS_ERR_ARG, "null argument");
  CU(cudaSetDevice(device));
  int sms = 0;
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int blocks = 4 * sms, threads = 256, iters = 256;
  double* d = nullptr;
  CU(cudaMalloc(&d, sizeof(double) * blocks * threads));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int op = 0; op < 3 && e == cudaSuccess; op++) {
    float best = 0.0f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
      cudaEventRecord(e0);
      k_fp64_rate<<<blocks, threads>>>(op, iters, 0.99999999, 1e-12, d);
      cudaEventRecord(e1);
      e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaGetLastError();
      float ms = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e == cudaSuccess && rep > 0 && (best == 0.0f || ms < best)) best = ms;  // rep 0 warms up
    }
    gops[op] = best > 0.0f ? (double)blocks * threads * iters * 8 / ((double)best * 1e6) : 0.0;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d);
  if (e != cudaSuccess) return fail(STS_ERR_CUDA, std::string("sts_fp64_rates: ") + cudaGetErrorString(e));
  return STS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches: many independent cases advanced together, every kernel of a step launched once
// for all of them (CTA z = case) and the sweep loops of all cases in one cooperative launch.
// ---------------------------------------------------------------------------
struct sts_batch {
  std::vector<sts_ctx*> cases;
  cudaStream_t s = nullptr;
  std::vector<void*> allocs;
  Geo* d_geos = nullptr;
  int* d_tile_case = nullptr;
  int* d_tile_first = nullptr;
  LoopCtl* d_lc = nullptr;
  int ncases = 0, ntiles = 0, precision = 0;
  bool fixed = true;
  dim3 cell_grid, bnd_grid, pt_grid;
  int jump_beside = 1;  // every case's jump entries run beside its velocity and pressure phases
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<unsigned> counter_before;

  ~sts_batch() {
    if (h_flag) cudaFreeHost(h_flag);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void* p : allocs) cudaFree(p);
    if (s) cudaStreamDestroy(s);
    for (sts_ctx* c : cases) delete c;
  }
  template <class T>
  int alloc(T** p, size_t n) {
    void* q = nullptr;
    CU(cudaMalloc(&q, sizeof(T) * (n ? n : 1)));
    allocs.push_back(q);
    *p = (T*)q;
    return STS_OK;
  }
  bool fast() const { return precision >= 1; }
  using PtKernel = void (*)(const Geo*, const int*, const int*, int, int, LoopCtl*);
  PtKernel pt_kernel() const {
    if (precision >= 2 && !fixed) return precision == 3 ? kb_pt_loop_mixed_df : kb_pt_loop_mixed;
    return fast() ? kb_pt_loop_fast : kb_pt_loop;
  }
  int build_graph();
  int step_host(int n);
  bool use_graph = true;
  bool warm3 = false, warm4 = false;
  unsigned* d_flag = nullptr;
  unsigned* h_flag = nullptr;
  // launch shapes (autotuned as for a single case: assembly block, sweep-loop CTAs per SM)
  dim3 asm_block{32, 8, 1};
  int max_nx = 1, max_ny = 1, sms = 0, per_sm_max = 0, per_sm = 0;
  int tune_left = 0, tune_idx = -1;
  std::vector<sts_ctx::TuneStat> tune_pt, tune_asm;
  dim3 asm_grid() const {
    return dim3((max_nx + asm_block.x - 1) / asm_block.x, (max_ny + asm_block.y - 1) / asm_block.y,
                (unsigned)ncases * (precision == 3 ? 3u : 1u));
  }
  void size_pt() {
    const int use = (per_sm > 0 && per_sm <= per_sm_max) ? per_sm : per_sm_max;
    pt_grid = dim3((unsigned)std::max(1, std::min(ntiles, use * sms)));
  }
  void launch_assemble() {
    if (precision == 3) kb_assemble_df<<<asm_grid(), asm_block, 0, s>>>(d_geos, 0ull, 0);
    else if (fast()) kb_assemble_fast<<<asm_grid(), asm_block, 0, s>>>(d_geos, 0ull, 0);
    else kb_assemble<<<asm_grid(), asm_block, 0, s>>>(d_geos, 0ull, 0);
  }
  int tune_step();
};

// The batched step loop launched kernel by kernel (for per-kernel profiling): the same kernels
// as the graph, the loop condition read back after every step.
int sts_batch::step_host(int n) {
  const dim3 blk(32, 8);
  const Geo* G = d_geos;
  for (int k = 0; k < n; k++) {
    kb_step_begin<<<cell_grid, blk, 0, s>>>(G);
    if (warm3) {
      kb_warm_diff<<<cell_grid, blk, 0, s>>>(G);
      kb_warm_fit<<<dim3(1, 1, ncases), 576, 0, s>>>(G);
      kb_warm_apply<<<cell_grid, blk, 0, s>>>(G);
    }
    launch_assemble();
    const int* tc = d_tile_case;
    const int* tf = d_tile_first;
    void* args[] = {(void*)&G, (void*)&tc, (void*)&tf, (void*)&ncases, (void*)&ntiles, (void*)&d_lc};
    CU(cudaLaunchCooperativeKernel((const void*)pt_kernel(), pt_grid, blk, args, 0, s));
    (precision == 3 ? kb_correct_df : kb_correct)<<<cell_grid, blk, 0, s>>>(G);
    kb_face_rho<<<cell_grid, blk, 0, s>>>(G);
    kb_bnd_fused<<<bnd_grid, kBndThreads, 0, s>>>(G, 0ull, 0, jump_beside);
    if (precision == 3) kb_flux_diff_df<<<cell_grid, blk, 0, s>>>(G, PH_TEMP | PH_PRES);
    else if (fast()) kb_flux_diff_fast<<<cell_grid, blk, 0, s>>>(G, PH_TEMP | PH_PRES);
    else kb_flux_diff<<<cell_grid, blk, 0, s>>>(G, PH_TEMP | PH_PRES);
    if (warm4) {
      kb_conv_gram<<<cell_grid, blk, 0, s>>>(G);
      kb_conv_solve<<<dim3(2, 1, ncases), kConvSolveThreads, 0, s>>>(G);
      kb_conv_next<<<cell_grid, blk, 0, s>>>(G);
      kb_conv_predict<<<cell_grid, blk, 0, s>>>(G);
    }
    kb_step_end<<<dim3(1, 1, ncases), 1024, 0, s>>>(G, 0ull, 0);
    kb_continue<<<1, 256, 0, s>>>(G, ncases, 0ull, d_flag);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(h_flag, d_flag, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    if (!*h_flag) break;
  }
  return STS_OK;
}

// One batched step for the autotuner, launched kernel by kernel: the assembly with block shape
// tune_idx % 3, the sweep loop with tune_idx % per_sm_max + 1 CTAs per SM, both timed by event pairs;
// the loop is compared per round (the most sweeps any case took).  A real step.
int sts_batch::tune_step() {
  const bool record = tune_idx >= 0;
  const int npt = (int)tune_pt.size(), nasm = (int)tune_asm.size();
  const int pc = record ? tune_idx % npt : npt - 1, ac = record ? tune_idx % nasm : 0;
  asm_block = sts_ctx::asm_shape(ac);
  per_sm = pc + 1;
  size_pt();
  cudaEvent_t ev[3];
  for (cudaEvent_t& e : ev) CU(cudaEventCreate(&e));
  const dim3 blk(32, 8);
  const Geo* G = d_geos;
  kb_set_steps<<<1, 256, 0, s>>>(G, ncases, 1u);
  kb_step_begin<<<cell_grid, blk, 0, s>>>(G);
  if (warm3) {
    kb_warm_diff<<<cell_grid, blk, 0, s>>>(G);
    kb_warm_fit<<<dim3(1, 1, ncases), 576, 0, s>>>(G);
    kb_warm_apply<<<cell_grid, blk, 0, s>>>(G);
  }
  CU(cudaEventRecord(ev[0], s));
  launch_assemble();
  CU(cudaEventRecord(ev[1], s));
  const int* tc = d_tile_case;
  const int* tf = d_tile_first;
  void* args[] = {(void*)&G, (void*)&tc, (void*)&tf, (void*)&ncases, (void*)&ntiles, (void*)&d_lc};
  CU(cudaLaunchCooperativeKernel((const void*)pt_kernel(), pt_grid, blk, args, 0, s));
  CU(cudaEventRecord(ev[2], s));
  (precision == 3 ? kb_correct_df : kb_correct)<<<cell_grid, blk, 0, s>>>(G);
  kb_face_rho<<<cell_grid, blk, 0, s>>>(G);
  kb_bnd_fused<<<bnd_grid, kBndThreads, 0, s>>>(G, 0ull, 0, jump_beside);
  if (precision == 3) kb_flux_diff_df<<<cell_grid, blk, 0, s>>>(G, PH_TEMP | PH_PRES);
  else if (fast()) kb_flux_diff_fast<<<cell_grid, blk, 0, s>>>(G, PH_TEMP | PH_PRES);
  else kb_flux_diff<<<cell_grid, blk, 0, s>>>(G, PH_TEMP | PH_PRES);
  if (warm4) {
    kb_conv_gram<<<cell_grid, blk, 0, s>>>(G);
    kb_conv_solve<<<dim3(2, 1, ncases), kConvSolveThreads, 0, s>>>(G);
    kb_conv_next<<<cell_grid, blk, 0, s>>>(G);
    kb_conv_predict<<<cell_grid, blk, 0, s>>>(G);
  }
  kb_step_end<<<dim3(1, 1, ncases), 1024, 0, s>>>(G, 0ull, 0);
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(s));
  float ta = 0, tp = 0;
  cudaEventElapsedTime(&ta, ev[0], ev[1]);
  cudaEventElapsedTime(&tp, ev[1], ev[2]);
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  unsigned rounds = 0;
  for (sts_ctx* c : cases) {
    if (int r = c->read_ctl()) return r;
    rounds = std::max(rounds, c->h_ctl->step_sweeps);
  }
  if (record) {
    tune_asm[ac].best = std::min(tune_asm[ac].best, (double)ta);
    if (rounds > 0) tune_pt[pc].best = std::min(tune_pt[pc].best, (double)tp / rounds);
  }
  tune_idx++;
  if (--tune_left == 0) {
    int best_a = 0, best_p = npt - 1;
    for (int k = 0; k < nasm; k++)
      if (tune_asm[k].best < tune_asm[best_a].best) best_a = k;
    for (int k = 0; k < npt; k++)
      if (tune_pt[k].best < tune_pt[best_p].best) best_p = k;
    asm_block = sts_ctx::asm_shape(best_a);
    per_sm = best_p + 1;
    size_pt();
    if (use_graph) {  // rebuilt with the chosen shapes
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      exec = nullptr;
      graph = nullptr;
      if (int r = build_graph()) return r;
    }
  }
  return STS_OK;
}

int sts_batch::build_graph() {
  CU(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle hs;
  CU(cudaGraphConditionalHandleCreate(&hs, graph, 1, cudaGraphCondAssignDefault));
  cudaGraphNode_t n_step;
  cudaGraph_t b;
  if (int r = add_while(&n_step, graph, {}, hs, &b)) return r;
  const dim3 blk(32, 8);
  const Geo* G = d_geos;
  cudaGraphNode_t n[11];
  if (int r = add_kernel(&n[0], b, {}, kb_step_begin, cell_grid, blk, G)) return r;
  if (warm3) {
    cudaGraphNode_t w[3];
    if (int r = add_kernel(&w[0], b, {n[0]}, kb_warm_diff, cell_grid, blk, G)) return r;
    if (int r = add_kernel(&w[1], b, {w[0]}, kb_warm_fit, dim3(1, 1, ncases), dim3(576), G)) return r;
    if (int r = add_kernel(&w[2], b, {w[1]}, kb_warm_apply, cell_grid, blk, G)) return r;
    n[0] = w[2];
  }
  if (int r = add_kernel(&n[1], b, {n[0]}, precision == 3 ? kb_assemble_df : (fast() ? kb_assemble_fast : kb_assemble),
                         asm_grid(), asm_block, G, (unsigned long long)0, 0))
    return r;
  if (int r = add_kernel(&n[2], b, {n[1]}, pt_kernel(), pt_grid, blk, G, (const int*)d_tile_case,
                         (const int*)d_tile_first, ncases, ntiles, d_lc))
    return r;
  {
    cudaLaunchAttributeValue v{};
    v.cooperative = 1;
    CU(cudaGraphKernelNodeSetAttribute(n[2], cudaLaunchAttributeCooperative, &v));
  }
  if (int r = add_kernel(&n[3], b, {n[2]}, precision == 3 ? kb_correct_df : kb_correct, cell_grid, blk, G)) return r;
  if (int r = add_kernel(&n[4], b, {n[3]}, kb_face_rho, cell_grid, blk, G)) return r;
  if (int r = add_kernel(&n[6], b, {n[4]}, kb_bnd_fused, bnd_grid, dim3(kBndThreads), G, (unsigned long long)0, 0,
                         jump_beside))
    return r;
  if (int r = add_kernel(&n[8], b, {n[6]}, precision == 3 ? kb_flux_diff_df : (fast() ? kb_flux_diff_fast : kb_flux_diff),
                         cell_grid, blk, G,
                         (unsigned)(PH_TEMP | PH_PRES)))
    return r;
  std::vector<cudaGraphNode_t> before_end{n[8]};
  if (warm4) {  // the fit and the next step's start, beside the step's last kernels
    cudaGraphNode_t w[4];
    if (int r = add_kernel(&w[0], b, {n[2]}, kb_conv_gram, cell_grid, blk, G)) return r;
    if (int r = add_kernel(&w[1], b, {w[0]}, kb_conv_solve, dim3(2, 1, ncases), dim3(kConvSolveThreads), G)) return r;
    if (int r = add_kernel(&w[2], b, {w[0]}, kb_conv_next, cell_grid, blk, G)) return r;
    if (int r = add_kernel(&w[3], b, {w[1], w[2]}, kb_conv_predict, cell_grid, blk, G)) return r;
    before_end.push_back(w[3]);
  }
  if (int r = add_kernel(&n[9], b, before_end, kb_step_end, dim3(1, 1, ncases), dim3(1024), G, (unsigned long long)0, 0))
    return r;
  if (int r = add_kernel(&n[10], b, {n[9]}, kb_continue, dim3(1), dim3(256), G, ncases, (unsigned long long)hs,
                         (unsigned*)nullptr))
    return r;
  CU(cudaGraphInstantiate(&exec, graph, 0));
  return STS_OK;
}

extern "C" {

int sts_open_batch(const char* const* case_dirs, int ncases, const sts_options* opt_in, sts_batch** out) {
  if (opt_in && opt_in->warm_start == 5) return fail(STS_ERR_ARG, "warm_start 5 is not available in batches");
  g_err.clear();
  if (out) *out = nullptr;
  if (!case_dirs || !out || ncases < 1) return fail(STS_ERR_ARG, "bad argument");
  if (ncases > kMaxBatchCases) return fail(STS_ERR_ARG, "too many cases for one batch");
  sts_options opt;
  sts_default_options(&opt);
  if (opt_in) opt = *opt_in;
  opt.write_files = 0;
  std::unique_ptr<sts_batch> b(new sts_batch);
  b->use_graph = opt.use_graph != 0;
  b->precision = opt.precision;
  b->fixed = opt.fixed_sweeps != 0;
  for (int k = 0; k < ncases; k++) {
    if (!case_dirs[k]) return fail(STS_ERR_ARG, "null case directory");
    sts_ctx* c = nullptr;
    if (int r = open_impl(case_dirs[k], &opt, &c)) return r;
    c->in_batch = true;
    b->cases.push_back(c);
    if ((int)c->hc.cfg.n("N_I") != 1)
      return fail(STS_ERR_ARG, std::string("batched cases need N_I = 1: ") + case_dirs[k]);
  }
  CU(cudaSetDevice(opt.device));
  CU(cudaDeviceSynchronize());  // every case's set-up is done
  CU(cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking));
  b->ncases = ncases;
  std::vector<Geo> geos;
  std::vector<int> tile_case, tile_first;
  unsigned gx = 1, gy = 1, wx = 1;
  for (int k = 0; k < ncases; k++) {
    sts_ctx* c = b->cases[k];
    geos.push_back(c->g);
    tile_first.push_back((int)tile_case.size());
    for (int t = 0; t < c->ntiles; t++) tile_case.push_back(k);
    gx = std::max(gx, c->grid.x);
    gy = std::max(gy, c->grid.y);
    b->max_nx = std::max(b->max_nx, c->g.Nx);
    b->max_ny = std::max(b->max_ny, c->g.Ny);
    wx = std::max(wx, c->bnd_grid().x);
    if (!c->jump_beside()) b->jump_beside = 0;
  }
  b->ntiles = (int)tile_case.size();
  b->warm3 = opt.warm_start == 3;
  b->warm4 = opt.warm_start == 4;
  if (int r = b->alloc(&b->d_geos, ncases)) return r;
  if (int r = b->alloc(&b->d_tile_case, tile_case.size())) return r;
  if (int r = b->alloc(&b->d_tile_first, tile_first.size())) return r;
  if (int r = b->alloc(&b->d_lc, 1)) return r;
  CU(cudaMemcpy(b->d_geos, geos.data(), sizeof(Geo) * ncases, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(b->d_tile_case, tile_case.data(), sizeof(int) * tile_case.size(), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(b->d_tile_first, tile_first.data(), sizeof(int) * tile_first.size(), cudaMemcpyHostToDevice));
  CU(cudaMemset(b->d_lc, 0, sizeof(LoopCtl)));
  b->cell_grid = dim3(gx, gy, (unsigned)ncases);
  b->bnd_grid = dim3(wx, 1, (unsigned)ncases);
  int sms = 0, per_sm = 0;
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, opt.device));
  CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b->pt_kernel(), 256, 0));
  if (per_sm < 1) return fail(STS_ERR_CUDA, "the sweep-loop kernel does not fit on a multiprocessor");
  b->sms = sms;
  b->per_sm_max = per_sm;
  b->size_pt();
  if (opt.autotune) {
    b->tune_pt.assign(per_sm, sts_ctx::TuneStat{});
    b->tune_asm.assign(3, sts_ctx::TuneStat{});
    b->tune_left = 1 + sts_ctx::kTuneRounds * std::max(per_sm, 3);
  }
  if (int r = b->alloc(&b->d_flag, 1)) return r;
  CU(cudaMallocHost(&b->h_flag, sizeof(unsigned)));
  if (b->use_graph)
    if (int r = b->build_graph()) return r;
  *out = b.release();
  return STS_OK;
}

int sts_batch_step(sts_batch* b, int nsteps, int* steps_done) {
  if (!b || nsteps < 0) return fail(STS_ERR_ARG, "bad argument");
  int done = 0;
  if (nsteps > 0) {
    sts_ctx* c0 = b->cases[0];
    CU(cudaSetDevice(c0->opt.device));
    std::vector<unsigned> before(b->ncases), status_before(b->ncases);
    for (int k = 0; k < b->ncases; k++) {
      before[k] = b->cases[k]->h_ctl->it_counter;
      status_before[k] = b->cases[k]->h_ctl->status;
    }
    for (sts_ctx* c : b->cases) CU(cudaStreamSynchronize(c->s));  // field uploads of the cases land first
    // the autotuner's steps come first (real steps, launched kernel by kernel)
    int tuned = 0;
    while (b->tune_left > 0 && tuned < nsteps) {
      if (int r = b->tune_step()) return r;
      tuned++;
      bool any = false;
      for (sts_ctx* c : b->cases) any = any || c->h_ctl->continue_step;
      if (!any) break;
    }
    if (tuned < nsteps) {
      kb_set_steps<<<1, 256, 0, b->s>>>(b->d_geos, b->ncases, (unsigned)(nsteps - tuned));
      CU(cudaGetLastError());
      if (b->use_graph) {
        CU(cudaGraphLaunch(b->exec, b->s));
      } else if (int r = b->step_host(nsteps - tuned)) {
        return r;
      }
    }
    CU(cudaStreamSynchronize(b->s));
    bool nonfinite = false;
    for (int k = 0; k < b->ncases; k++) {
      sts_ctx* c = b->cases[k];
      if (int r = c->read_ctl()) return r;
      done = std::max(done, (int)(c->h_ctl->it_counter - before[k]));
      if (!c->h_ctl->continue_step) c->finished = true;
      if (c->h_ctl->status & ST_BARRIER_TIMEOUT) return fail(STS_ERR_TIMEOUT, "a grid barrier of the sweep loop timed out");
      if (c->h_ctl->status & ~status_before[k] & ST_NONFINITE) nonfinite = true;
    }
    if (nonfinite) {
      if (steps_done) *steps_done = done;
      return fail(STS_ERR_NONFINITE, "a residual became NaN or Inf in at least one case");
    }
  }
  if (steps_done) *steps_done = done;
  return STS_OK;
}

int sts_batch_step_timed(sts_batch* b, int nsteps, int* steps_done, double* device_ms) {
  if (!b || nsteps < 0) return fail(STS_ERR_ARG, "bad argument");
  CU(cudaSetDevice(b->cases[0]->opt.device));
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  CU(cudaEventRecord(e0, b->s));
  int done = 0;
  const int r = sts_batch_step(b, nsteps, &done);
  cudaEventRecord(e1, b->s);
  cudaEventSynchronize(e1);
  float t = 0;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (device_ms) *device_ms = t;
  if (steps_done) *steps_done = done;
  return r;
}

int sts_batch_case(sts_batch* b, int index, sts_ctx** out) {
  if (!b || !out || index < 0 || index >= b->ncases) return fail(STS_ERR_ARG, "bad case index");
  *out = b->cases[index];
  return STS_OK;
}

void sts_batch_destroy(sts_batch* b) { delete b; }

int sts_batch_autotune_result(sts_batch* b, int* steps_left, int* ctas_per_sm, int* asm_block_x, int* asm_block_y) {
  if (!b) return fail(STS_ERR_ARG, "null batch");
  if (steps_left) *steps_left = b->tune_left;
  if (ctas_per_sm) *ctas_per_sm = b->per_sm > 0 ? b->per_sm : b->per_sm_max;
  if (asm_block_x) *asm_block_x = (int)b->asm_block.x;
  if (asm_block_y) *asm_block_y = (int)b->asm_block.y;
  return STS_OK;
}

}  // extern "C"
