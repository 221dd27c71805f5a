// sayram_engine.cu -- host runtime and C-ABI of the GB300 Sayram-2D hot path.
//
// An Engine owns one batch of instances (a single Solver is a batch of one): the padded device
// layout, the chunk/tile work lists, the per-step launch sequence and the optional CUDA graph.
// Every public function returns a status code and records a message for sayram_last_error().
#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "host_errors.h"
#include "sayram_gpu.h"
#include "sayram_ops.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define SG_CUDA(call)                                                                      \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(SAYRAM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));    \
  } while (0)

long long round_up(long long a, long long m) { return (a + m - 1) / m * m; }

using sg::Ctl;
using sg::InstDev;
using sg::InstState;

}  // namespace

struct sayram_batch_s {
  sayram_options opt{};
  int dev = 0;
  int nsm = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t cstream = nullptr;           // host copies of sayram_batch_step_host, in pieces
  cudaStream_t tstream = nullptr;           // its layout transforms in, beside the assembly of earlier pieces
  std::vector<cudaEvent_t> piece_ev;        // one per piece and direction
  int n = 0;
  std::vector<InstDev> hinst;
  long long ncell = 0;      // padded storage cells (capacity)
  int cap_slots = 0, cap_chunks = 0, cap_tiles = 0;
  int pmax = 4;             // widest row pitch the SpMV kernels must stage
  int* d_dyn = nullptr;     // [nchunks, ntiles, ninst] read by the kernels
  std::vector<int> h_chunk, h_tile;
  std::vector<std::pair<void*, int>> cell_arrays;  // every per-cell array and its element size
  long long nreal = 0;      // real cells (packed alpha-major size)
  int nchunks = 0, ntiles = 0;
  size_t bytes = 0;
  bool mixed = false;  // FP32 Krylov with (hi, lo) coefficients
  bool dwm = false;    // double-word wide arithmetic (otherwise IEEE FP64)

  // device memory
  std::vector<void*> allocs;
  InstDev* d_inst = nullptr;
  InstState* d_st = nullptr;
  Ctl* d_ctl = nullptr;
  Ctl* h_ctl = nullptr;  // pinned mirror
  int* d_chunk = nullptr;
  int* d_tile = nullptr;
  double *d_xe = nullptr, *d_ye = nullptr, *d_wx = nullptr, *d_wy = nullptr, *d_dirv = nullptr;
  double* d_part = nullptr;
  double* d_stage = nullptr;   // 6 * max instance cells (setup) / packed field (get/set)
  long long ycap_ = 0;         // y-edge table length
  double* d_tab = nullptr;     // D table (3 * n_alpha * n_energy), grown on demand
  long long tab_cap = 0;
  double* d_rows = nullptr;    // D-table row factors p, dlogE/dp, its square (3 * ycap_)
  long long stage_cells = 0;
  sg::Geo geo{};
  sg::Fields fl{};
  sg::Coef<double> c64{};
  sg::Coef<float> c32{};
  sg::Kry<double> k64{};
  sg::Kry<float> k32{};
  sg::Common cm{};

  // timing
  bool timing = false;
  std::vector<std::string> tnames;
  std::vector<double> tms;
  std::vector<long long> tcount;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::vector<cudaEvent_t> evpool;
  size_t evused = 0;
  cudaEvent_t slots[8] = {};
  // per-step CUDA graph with device-side loops (built on the first graph step)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  // the same step without its prefix (counter reset, k_begin, k_assemble) and its polish, for the
  // host-buffer step that assembles piece by piece while the state is still being copied in and
  // polishes piece by piece while the finished pieces are copied out
  cudaGraph_t graph_solve = nullptr;
  cudaGraphExec_t gexec_solve = nullptr;

  ~sayram_batch_s() { release(); }

  void release() {
    if (dev >= 0) cudaSetDevice(dev);
    drop_graph();
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    if (d_tab) cudaFree(d_tab);
    if (d_rows) cudaFree(d_rows);
    d_tab = d_rows = nullptr;
    tab_cap = 0;
    if (h_ctl) cudaFreeHost(h_ctl);
    h_ctl = nullptr;
    for (auto e : evpool) cudaEventDestroy(e);
    evpool.clear();
    for (auto& e : slots)
      if (e) cudaEventDestroy(e), e = nullptr;
    for (auto e : piece_ev) cudaEventDestroy(e);
    piece_ev.clear();
    if (cstream) cudaStreamDestroy(cstream);
    cstream = nullptr;
    if (tstream) cudaStreamDestroy(tstream);
    tstream = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }

  template <typename T>
  int alloc(T** p, long long count) {
    void* q = nullptr;
    const size_t nb = (size_t)std::max<long long>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, nb);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(SAYRAM_ERR_OOM, "cudaMalloc of " + std::to_string(nb) + " bytes failed: " +
                                      cudaGetErrorString(e));
    }
    allocs.push_back(q);
    bytes += nb;
    e = cudaMemsetAsync(q, 0, nb, stream);
    if (e != cudaSuccess) return fail(SAYRAM_ERR_CUDA, cudaGetErrorString(e));
    *p = (T*)q;
    return SAYRAM_OK;
  }

  // ---- timing helpers
  int tid(const char* name) {
    for (size_t k = 0; k < tnames.size(); ++k)
      if (tnames[k] == name) return (int)k;
    tnames.push_back(name);
    tms.push_back(0.0);
    tcount.push_back(0);
    return (int)tnames.size() - 1;
  }
  cudaEvent_t ev() {
    if (evused == evpool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      evpool.push_back(e);
    }
    return evpool[evused++];
  }
  template <typename F>
  void launch(const char* name, F&& f) {
    if (!timing) {
      f();
      return;
    }
    cudaEvent_t a = ev(), b = ev();
    cudaEventRecord(a, stream);
    f();
    cudaEventRecord(b, stream);
    pending.push_back({tid(name), {a, b}});
  }
  void collect_timing() {
    for (auto& p : pending) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, p.second.first, p.second.second);
      tms[p.first] += ms;
      tcount[p.first] += 1;
    }
    pending.clear();
    evused = 0;
  }

  // launch shape of the streaming kernels: cells per chunk (one block iteration) and blocks per SM
  int chunk = 2048;
  int gmult = 16;
  int grid_stream() const { return std::max(1, std::min(cap_chunks, nsm * gmult)); }
  int nchunks_of(int nx, int ny) const {
    const long long cells = round_up((long long)ny * round_up(nx, 4), 4);
    return (int)((cells + chunk - 1) / chunk);
  }
  // dynamic shared memory of the SpMV kernels: the chunk plus one row above and below
  template <typename T>
  size_t smem_spmv() const { return (size_t)(chunk + 2 * pmax) * sizeof(T); }
  // the residual and polish kernels stage the 8-byte wide solution
  size_t smem_wide() const { return (size_t)(chunk + 2 * pmax) * 8; }
  template <typename T, typename C, typename A, int CH>
  int prep_kernels() {
    const int b1 = (int)smem_spmv<T>(), b2 = (int)smem_wide();
    if (b1 > 227 * 1024 || b2 > 227 * 1024) return fail(SAYRAM_ERR_ARG, "rows too wide for the shared-memory stencil");
    SG_CUDA(cudaFuncSetAttribute(sg::k_bicg1<T, CH>, cudaFuncAttributeMaxDynamicSharedMemorySize, b1));
    SG_CUDA(cudaFuncSetAttribute(sg::k_bicg2<T, CH>, cudaFuncAttributeMaxDynamicSharedMemorySize, b1));
    SG_CUDA(cudaFuncSetAttribute(sg::k_resid<T, C, A, CH>, cudaFuncAttributeMaxDynamicSharedMemorySize, b2));
    SG_CUDA(cudaFuncSetAttribute(sg::k_polish<C, A, CH>, cudaFuncAttributeMaxDynamicSharedMemorySize, b2));
    SG_CUDA(cudaFuncSetAttribute(sg::k_solve_coop<T, C, A, CH, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, b2));
    SG_CUDA(cudaFuncSetAttribute(sg::k_solve_coop<T, C, A, CH, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, b2));
    return SAYRAM_OK;
  }
  // The cooperative solve (k_solve_coop) replaces the graph's refinement loops when every chunk
  // gets a block of its own in one wave of co-resident blocks (a fixed instance list; the server's
  // lanes set coop = 0). Returns its grid (negative: the 4-blocks-per-SM form), or 0 when the
  // loops of separate kernels are used.
  int coop = 1;
  template <typename T, typename C, typename A, int CH>
  int coop_grid() {
    if (!coop || nchunks < 1) return 0;
    int can = 0;
    if (cudaDeviceGetAttribute(&can, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !can) {
      cudaGetLastError();
      return 0;
    }
    int per_sm2 = 0, per_sm4 = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, sg::k_solve_coop<T, C, A, CH, 2>, sg::kThreads,
                                                      smem_wide()) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm4, sg::k_solve_coop<T, C, A, CH, 4>, sg::kThreads,
                                                      smem_wide()) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    if ((long long)nchunks <= (long long)per_sm2 * nsm) return nchunks;
    if ((long long)nchunks <= (long long)per_sm4 * nsm) return -nchunks;
    return 0;
  }
  template <typename T, typename C, typename A, int CH>
  int launch_coop(int sgrid, const sg::Coef<C>& cfull, const sg::Coef<T>& ck, const sg::Kry<T>& kr) {
    const int grid = sgrid < 0 ? -sgrid : sgrid;
    sg::Common c2 = cm;
    c2.use_cond = 2;
    c2.guard_refine = opt.max_refine + 1;
    c2.guard_iters = opt.max_iters + 1;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(sg::kThreads);
    cfg.dynamicSmemBytes = smem_wide();
    cfg.stream = stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (sgrid > 0)
      SG_CUDA(cudaLaunchKernelEx(&cfg, sg::k_solve_coop<T, C, A, CH, 2>, c2, fl, cfull, ck, kr, opt.tol,
                                 opt.inner_tol, opt.max_refine, opt.max_iters));
    else
      SG_CUDA(cudaLaunchKernelEx(&cfg, sg::k_solve_coop<T, C, A, CH, 4>, c2, fl, cfull, ck, kr, opt.tol,
                                 opt.inner_tol, opt.max_refine, opt.max_iters));
    return SAYRAM_OK;
  }
  // dispatch of the per-step sequence on precision and chunk size (graph: build it; else: run it)
  template <typename T, typename C, typename A>
  int run_chunked(const sg::Coef<C>& cf, const sg::Coef<T>& ck, const sg::Kry<T>& kr, bool as_graph, bool prefix) {
    switch (chunk) {
      case 1024: return as_graph ? build_graph<T, C, A, 1024>(cf, ck, kr, prefix) : step_once<T, C, A, 1024>(cf, ck, kr);
      case 2048: return as_graph ? build_graph<T, C, A, 2048>(cf, ck, kr, prefix) : step_once<T, C, A, 2048>(cf, ck, kr);
      default: return as_graph ? build_graph<T, C, A, 4096>(cf, ck, kr, prefix) : step_once<T, C, A, 4096>(cf, ck, kr);
    }
  }
  int run_mode(bool as_graph, bool prefix = true) {
    return dwm ? run_chunked<float, float, sg::DWA>(c32, c32, k32, as_graph, prefix)
           : mixed ? run_chunked<float, float, sg::F64A>(c32, c32, k32, as_graph, prefix)
                   : run_chunked<double, double, sg::F64A>(c64, c64, k64, as_graph, prefix);
  }
  // the step prefix outside a graph: counter reset, k_begin, then k_assemble over tiles [t0, t1)
  int launch_begin() {
    SG_CUDA(cudaMemsetAsync(d_ctl, 0, 2 * sizeof(int), stream));
    sg::k_begin<<<(n + 255) / 256, 256, 0, stream>>>(cm);
    SG_CUDA(cudaGetLastError());
    return SAYRAM_OK;
  }
  int launch_assemble(int t0, int t1) {
    if (dwm)
      sg::k_assemble<float, sg::DWA><<<grid_tiles(), sg::kAsmThreads, 0, stream>>>(cm, geo, fl, c32, t0, t1);
    else if (mixed)
      sg::k_assemble<float, sg::F64A><<<grid_tiles(), sg::kAsmThreads, 0, stream>>>(cm, geo, fl, c32, t0, t1);
    else
      sg::k_assemble<double, sg::F64A><<<grid_tiles(), sg::kAsmThreads, 0, stream>>>(cm, geo, fl, c64, t0, t1);
    SG_CUDA(cudaGetLastError());
    return SAYRAM_OK;
  }
  // the polish over chunks [c0, c1) (whole instances; c1 < 0: all)
  template <typename C, typename A>
  int launch_polish_t(const sg::Coef<C>& cf, int c0, int c1) {
    const int gs = grid_stream();
    const size_t sm = smem_wide();
    if (chunk == 1024)
      sg::k_polish<C, A, 1024><<<gs, sg::kThreads, sm, stream>>>(cm, fl, cf, c0, c1);
    else if (chunk == 2048)
      sg::k_polish<C, A, 2048><<<gs, sg::kThreads, sm, stream>>>(cm, fl, cf, c0, c1);
    else
      sg::k_polish<C, A, 4096><<<gs, sg::kThreads, sm, stream>>>(cm, fl, cf, c0, c1);
    SG_CUDA(cudaGetLastError());
    return SAYRAM_OK;
  }
  int launch_polish(int c0, int c1) {
    return dwm ? launch_polish_t<float, sg::DWA>(c32, c0, c1)
           : mixed ? launch_polish_t<float, sg::F64A>(c32, c0, c1)
                   : launch_polish_t<double, sg::F64A>(c64, c0, c1);
  }
  // the refinement loop of one step as a graph (no prefix, no polish)
  int ensure_solve_graph() {
    if (gexec_solve) return SAYRAM_OK;
    int rc = run_mode(true, false);
    if (rc) drop_graph();
    return rc;
  }
  int launch_solve() {
    int rc = ensure_solve_graph();
    if (rc) return rc;
    SG_CUDA(cudaGraphLaunch(gexec_solve, stream));
    return SAYRAM_OK;
  }
  void drop_graph() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    if (gexec_solve) cudaGraphExecDestroy(gexec_solve);
    if (graph_solve) cudaGraphDestroy(graph_solve);
    gexec = gexec_solve = nullptr;
    graph = graph_solve = nullptr;
  }
  int autotune(int steps, int* best_chunk, int* best_grid);
  int set_dtable(int idx, const sayram_dtable* t);
  struct Tuned {
    int chunk, gmult;
    double ms_per_step;
  };
  std::vector<Tuned> tune_log;
  // Assembly grid: many short-lived blocks (96 per SM, each a few dozen tiles) rather than one
  // or two waves of blocks that each walk hundreds of tiles. On the 4096-instance batch, with 5
  // resident blocks per SM, the launch took 6.09 ms with 8 launched per SM, 6.15 with 5 (one
  // wave), 5.85 with 10, 5.60 with 20, 5.40 with 40, 5.27 with 64 and 5.32 with one block per
  // tile; with 6 resident, 5.22 with 48, 5.16 with 64 and 5.09 with 96.
  int grid_tiles() const { return std::max(1, std::min(cap_tiles, nsm * sg::kAsmGridPerSm)); }
  int n_enabled() const {
    int k = 0;
    for (int b = 0; b < n && b < (int)hinst.size(); ++b) k += hinst[b].enabled ? 1 : 0;
    return k;
  }

  int build(const sayram_problem* probs, int count, const sayram_options* o);
  int set_options(const sayram_options* o);
  int init_device();
  int alloc_storage(long long cells, int slots, int chunks_cap, int tiles_cap, long long xcap, long long ycap,
                    long long dcap, long long stage_cap);
  int zero_region(long long begin, long long end);
  int place(int b, const sayram_problem& p, long long base, int xe_off, int ye_off, const int dir_off[4],
            long long hoff);
  int rebuild_lists();
  int upload_instance(int b, const sayram_problem& p, bool coeffs, bool f0);
  int run_steps(int nsteps);
  int launch_steps(int nsteps);  // queue steps on the stream (no status read-back)
  int read_ctl();
  int finish_status();
  template <typename T, typename C, typename A, int CH>
  int step_once(const sg::Coef<C>& cfull, const sg::Coef<T>& ck, const sg::Kry<T>& kr);
  template <typename T, typename C, typename A, int CH>
  int build_graph(const sg::Coef<C>& cfull, const sg::Coef<T>& ck, const sg::Kry<T>& kr, bool prefix);
  int last_captured(cudaGraphNode_t* node);
  // wide (8-byte) table entries: a double, or a (hi, lo) float pair in double-word mode
  double wide(double v) const {
    if (!dwm) return v;
    const float h = (float)v, l = (float)(v - (double)h);
    double out;
    float pr[2] = {h, l};
    std::memcpy(&out, pr, sizeof(out));
    return out;
  }
  double unwide(double w) const {
    if (!dwm) return w;
    float pr[2];
    std::memcpy(pr, &w, sizeof(pr));
    return (double)pr[0] + (double)pr[1];
  }
};

static int validate_problem(const sayram_problem& p) {
  if (p.nx < 1 || p.ny < 1) return fail(SAYRAM_ERR_ARG, "Grid2D: x_edges/y_edges must have size >= 2.");
  if ((long long)p.nx * p.ny > (1LL << 31)) return fail(SAYRAM_ERR_ARG, "grid too large");
  if (!p.x_edges || !p.y_edges) return fail(SAYRAM_ERR_ARG, "missing edges");
  for (int i = 0; i < p.nx; ++i)
    if (!(p.x_edges[i + 1] > p.x_edges[i]))
      return fail(SAYRAM_ERR_ARG, "Grid2D: x_edges must be strictly increasing at i=" + std::to_string(i));
  for (int j = 0; j < p.ny; ++j)
    if (!(p.y_edges[j + 1] > p.y_edges[j]))
      return fail(SAYRAM_ERR_ARG, "Grid2D: y_edges must be strictly increasing at j=" + std::to_string(j));
  if (!(p.dt > 0) || !std::isfinite(p.dt)) return fail(SAYRAM_ERR_ARG, "dt must be positive");
  if (!p.G || !p.Dxx || !p.Dxy || !p.Dyy || !p.inv_tau || !p.f0)
    return fail(SAYRAM_ERR_ARG, "missing coefficient or initial-state array");
  for (int s = 0; s < 4; ++s) {
    if (p.bc[s] != SAYRAM_DIRICHLET && p.bc[s] != SAYRAM_ZEROFLUX)
      return fail(SAYRAM_ERR_ARG, "unknown boundary type");
    if (p.bc[s] == SAYRAM_DIRICHLET && !p.dirichlet[s])
      return fail(SAYRAM_ERR_ARG, "Dirichlet BC: missing value.");  // Solver.cc:393
  }
  return SAYRAM_OK;
}

int sayram_batch_s::set_options(const sayram_options* o) {
  sayram_default_options(&opt);
  if (o) opt = *o;
  if (opt.precision != SAYRAM_FP64 && opt.precision != SAYRAM_FP32_REFINE && opt.precision != SAYRAM_FP32_REFINE_DW)
    return fail(SAYRAM_ERR_ARG, "unknown precision");
  if (!(opt.tol > 0)) opt.tol = opt.precision == SAYRAM_FP64 ? 1e-12 : 1e-11;
  if (opt.inner_tol < 0) opt.inner_tol = 0;
  if (opt.max_iters < 1) opt.max_iters = 1;
  if (opt.max_refine < 2) opt.max_refine = 2;
  if (opt.precond != SAYRAM_PRECOND_JACOBI && opt.precond != SAYRAM_PRECOND_ALPHA_LINE)
    return fail(SAYRAM_ERR_ARG, "unknown preconditioner");
  mixed = opt.precision != SAYRAM_FP64;
  dwm = opt.precision == SAYRAM_FP32_REFINE_DW;
  return SAYRAM_OK;
}

int sayram_batch_s::init_device() {
  dev = opt.device;
  int ndev = 0;
  SG_CUDA(cudaGetDeviceCount(&ndev));
  if (dev < 0 || dev >= ndev) return fail(SAYRAM_ERR_ARG, "no such CUDA device");
  SG_CUDA(cudaSetDevice(dev));
  SG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  SG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  SG_CUDA(cudaStreamCreateWithFlags(&cstream, cudaStreamNonBlocking));
  SG_CUDA(cudaStreamCreateWithFlags(&tstream, cudaStreamNonBlocking));
  return SAYRAM_OK;
}

// Device storage for `cells` padded cells, `slots` instances, the work lists and the per-instance
// tables (edges, weights, Dirichlet values; capacities in entries).
int sayram_batch_s::alloc_storage(long long cells, int slots, int chunks_cap, int tiles_cap, long long xcap,
                                  long long ycap, long long dcap, long long stage_cap) {
  int rc;
  // k_assemble indexes cells with 32-bit ints (2^31 cells would need ~330 GB of device memory)
  if (cells >= (1LL << 31) - 1) return fail(SAYRAM_ERR_ARG, "a batch holds at most 2^31 - 2 padded cells");
#define SG_ALLOC(p, cnt) \
  if ((rc = alloc(&(p), (cnt))) != SAYRAM_OK) return rc
  ncell = cells;
  cap_slots = slots;
  cap_chunks = chunks_cap;
  cap_tiles = tiles_cap;
  stage_cells = stage_cap;
  SG_ALLOC(d_inst, slots);
  SG_ALLOC(d_st, slots);
  SG_ALLOC(d_ctl, 1);
  SG_ALLOC(d_dyn, 4);
  SG_ALLOC(d_chunk, chunks_cap);
  SG_ALLOC(d_tile, tiles_cap);
  SG_ALLOC(d_xe, xcap);
  SG_ALLOC(d_ye, ycap);
  ycap_ = ycap;
  SG_ALLOC(d_wx, 2 * xcap);
  SG_ALLOC(d_wy, 2 * ycap);
  SG_ALLOC(d_dirv, std::max<long long>(dcap, 1));
  SG_ALLOC(d_part, 4LL * chunks_cap);
  SG_ALLOC(d_stage, stage_cap);
  cell_arrays.clear();
  double** geos[10] = {&geo.aAx, &geo.aBx, &geo.Sx, &geo.aAy, &geo.aBy, &geo.Sy, &geo.ukk, &geo.sdiag, &geo.G,
                       &geo.decay};
  for (auto g : geos) {
    SG_ALLOC(*g, cells);
    cell_arrays.push_back({*g, 8});
  }
  double** fs[9] = {&fl.f, &fl.fh[0], &fl.fh[1], &fl.fh[2], &fl.invD, &fl.R, &fl.colsum, &fl.y64[0], &fl.y64[1]};
  for (auto f : fs) {
    SG_ALLOC(*f, cells);
    cell_arrays.push_back({*f, 8});
  }
  if (mixed) {
    float** cs[8] = {&c32.cw, &c32.ce, &c32.cs, &c32.cn, &c32.lw, &c32.le, &c32.ls, &c32.ln};
    for (auto c : cs) {
      SG_ALLOC(*c, cells);
      cell_arrays.push_back({*c, 4});
    }
    float** ks[8] = {&k32.r, &k32.rh, &k32.t, &k32.x, &k32.p[0], &k32.p[1], &k32.v[0], &k32.v[1]};
    for (auto k : ks) {
      SG_ALLOC(*k, cells);
      cell_arrays.push_back({*k, 4});
    }
  } else {
    double** cs[4] = {&c64.cw, &c64.ce, &c64.cs, &c64.cn};
    for (auto c : cs) {
      SG_ALLOC(*c, cells);
      cell_arrays.push_back({*c, 8});
    }
    double** ks[8] = {&k64.r, &k64.rh, &k64.t, &k64.x, &k64.p[0], &k64.p[1], &k64.v[0], &k64.v[1]};
    for (auto k : ks) {
      SG_ALLOC(*k, cells);
      cell_arrays.push_back({*k, 8});
    }
  }
#undef SG_ALLOC
  SG_CUDA(cudaMallocHost(&h_ctl, sizeof(Ctl)));
  std::memset(h_ctl, 0, sizeof(Ctl));
  hinst.assign(slots, InstDev{});
  cm = sg::Common{};
  cm.inst = d_inst;
  cm.st = d_st;
  cm.ctl = d_ctl;
  cm.chunk_inst = d_chunk;
  cm.tile_inst = d_tile;
  cm.wx = d_wx;
  cm.wy = d_wy;
  cm.dirv = d_dirv;
  cm.part = d_part;
  cm.dyn = d_dyn;
  cm.hist_cap = sg::kOrder;
  cm.precond = opt.precond;
  fl.decay = geo.decay;
  return SAYRAM_OK;
}

// Zeroes cells [begin, end) of every per-cell array (a reused region must start at zero).
int sayram_batch_s::zero_region(long long begin, long long end) {
  for (auto& a : cell_arrays)
    SG_CUDA(cudaMemsetAsync((char*)a.first + begin * a.second, 0, (size_t)(end - begin) * a.second, stream));
  return SAYRAM_OK;
}

// Places instance b at cell index `base` (cell (0,0); one pad row precedes it) with its tables
// at the given offsets, uploads the tables and coefficients and runs the set-up kernel.
int sayram_batch_s::place(int b, const sayram_problem& p, long long base, int xe_off, int ye_off,
                          const int dir_off[4], long long hoff) {
  InstDev& I = hinst[b];
  std::memset(&I, 0, sizeof(I));
  I.nx = p.nx;
  I.ny = p.ny;
  I.pitch = (int)round_up(p.nx, 4);
  if (I.pitch > pmax) {
    if (gexec) return fail(SAYRAM_ERR_STATE, "instance wider than the rows the step graph was built for");
    pmax = I.pitch;
  }
  I.enabled = 1;
  for (int s = 0; s < 4; ++s) I.bc[s] = p.bc[s];
  I.base = base;
  I.hoff = hoff;
  I.ntx = (p.nx + sg::kTX - 1) / sg::kTX;
  I.nty = (p.ny + sg::kTY - 1) / sg::kTY;
  I.nchunks = nchunks_of(p.nx, p.ny);
  I.xe = xe_off;
  I.ye = ye_off;
  for (int s = 0; s < 4; ++s) I.dir[s] = p.bc[s] == SAYRAM_DIRICHLET ? dir_off[s] : -1;
  I.dt = p.dt;
  // tables: edges, bilinear weights of Solver.cc:333-336, Dirichlet vertex values
  std::vector<double> wx(2 * (p.nx + 1), 0.0), wy(2 * (p.ny + 1), 0.0);
  for (int i = 1; i < p.nx; ++i) {
    const double xv = p.x_edges[i];
    const double xl = 0.5 * (p.x_edges[i - 1] + p.x_edges[i]), xr = 0.5 * (p.x_edges[i] + p.x_edges[i + 1]);
    wx[2 * i] = wide((xr - xv) / (xr - xl));
    wx[2 * i + 1] = wide((xv - xl) / (xr - xl));
  }
  for (int j = 1; j < p.ny; ++j) {
    const double yv = p.y_edges[j];
    const double yb = 0.5 * (p.y_edges[j - 1] + p.y_edges[j]), yt = 0.5 * (p.y_edges[j] + p.y_edges[j + 1]);
    wy[2 * j] = wide((yt - yv) / (yt - yb));
    wy[2 * j + 1] = wide((yv - yb) / (yt - yb));
  }
  SG_CUDA(cudaMemcpyAsync(d_xe + xe_off, p.x_edges, sizeof(double) * (p.nx + 1), cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaMemcpyAsync(d_ye + ye_off, p.y_edges, sizeof(double) * (p.ny + 1), cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaMemcpyAsync(d_wx + 2LL * xe_off, wx.data(), sizeof(double) * wx.size(), cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaMemcpyAsync(d_wy + 2LL * ye_off, wy.data(), sizeof(double) * wy.size(), cudaMemcpyHostToDevice, stream));
  for (int s = 0; s < 4; ++s)
    if (I.dir[s] >= 0) {
      const int m = (s <= 1) ? p.ny + 1 : p.nx + 1;
      std::vector<double> v(m);
      for (int k = 0; k < m; ++k) v[k] = wide(p.dirichlet[s][k]);
      SG_CUDA(cudaMemcpyAsync(d_dirv + I.dir[s], v.data(), sizeof(double) * m, cudaMemcpyHostToDevice, stream));
    }
  SG_CUDA(cudaMemcpyAsync(d_inst + b, &I, sizeof(InstDev), cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaMemsetAsync(d_st + b, 0, sizeof(InstState), stream));
  return upload_instance(b, p, true, true);
}

// Work lists of the enabled instances, in slot order: chunks of `chunk` cells and 32x16 tiles.
int sayram_batch_s::rebuild_lists() {
  h_chunk.clear();
  h_tile.clear();
  int ninst = 0;
  for (int b = 0; b < cap_slots; ++b) {
    InstDev& I = hinst[b];
    if (!I.enabled) continue;
    ninst = b + 1;
    I.nchunks = nchunks_of(I.nx, I.ny);
    I.chunk0 = (int)h_chunk.size();
    for (int k = 0; k < I.nchunks; ++k) h_chunk.push_back(b);
    I.tile0 = (int)h_tile.size();
    for (int k = 0; k < I.ntx * I.nty; ++k) h_tile.push_back(b);
  }
  if ((int)h_chunk.size() > cap_chunks || (int)h_tile.size() > cap_tiles)
    return fail(SAYRAM_ERR_STATE, "work lists exceed their capacity");
  nchunks = (int)h_chunk.size();
  ntiles = (int)h_tile.size();
  n = std::max(n, ninst);
  const int dyn[4] = {nchunks, ntiles, cap_slots, 0};
  SG_CUDA(cudaMemcpyAsync(d_inst, hinst.data(), sizeof(InstDev) * cap_slots, cudaMemcpyHostToDevice, stream));
  if (nchunks) SG_CUDA(cudaMemcpyAsync(d_chunk, h_chunk.data(), sizeof(int) * nchunks, cudaMemcpyHostToDevice, stream));
  if (ntiles) SG_CUDA(cudaMemcpyAsync(d_tile, h_tile.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, stream));
  // the dyn counts travel by value too: pageable source, so the copy completes before return
  SG_CUDA(cudaMemcpyAsync(d_dyn, dyn, sizeof(dyn), cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaStreamSynchronize(stream));
  cm.nchunks = nchunks;
  cm.ntiles = ntiles;
  cm.ninst = cap_slots;
  return SAYRAM_OK;
}

int sayram_batch_s::build(const sayram_problem* probs, int count, const sayram_options* o) {
  int rc = set_options(o);
  if (rc) return rc;
  for (int b = 0; b < count; ++b) {
    rc = validate_problem(probs[b]);
    if (rc) return fail(rc, "instance " + std::to_string(b) + ": " + g_err);
  }
  if ((rc = init_device())) return rc;
  // compact layout: instances back to back, each with a pad row above and below
  std::vector<long long> base(count), hoff(count);
  std::vector<int> xoffv(count), yoffv(count), doffv(4 * count);
  long long cursor = 0, h = 0, maxcells = 0;
  int chunks = 0, tiles = 0, xoff = 0, yoff = 0, doff = 0;
  for (int b = 0; b < count; ++b) {
    const sayram_problem& p = probs[b];
    const long long pitch = round_up(p.nx, 4);
    base[b] = cursor + pitch;
    cursor += round_up((long long)(p.ny + 2) * pitch, 32);
    hoff[b] = h;
    h += (long long)p.nx * p.ny;
    chunks += (int)((round_up((long long)p.ny * pitch, 4) + 1023) / 1024);  // room for any chunk size
    tiles += ((p.nx + sg::kTX - 1) / sg::kTX) * ((p.ny + sg::kTY - 1) / sg::kTY);
    xoffv[b] = xoff;
    xoff += p.nx + 1;
    yoffv[b] = yoff;
    yoff += p.ny + 1;
    for (int s = 0; s < 4; ++s) {
      doffv[4 * b + s] = doff;
      if (p.bc[s] == SAYRAM_DIRICHLET) doff += (s <= 1) ? p.ny + 1 : p.nx + 1;
    }
    maxcells = std::max(maxcells, (long long)p.nx * p.ny);
  }
  nreal = h;
  // default launch shape: the largest chunk that still leaves two chunks per SM (measured over
  // single 128^2..2048^2 instances and mixed batches of 19..200: larger chunks pay below that,
  // when too few blocks share the stream, and above it, from fewer, longer block latencies)
  chunk = 1024;
  for (int c : {4096, 2048}) {
    long long nch = 0;
    for (int b = 0; b < count; ++b)
      nch += (round_up((long long)probs[b].ny * round_up(probs[b].nx, 4), 4) + c - 1) / c;
    if (nch >= 2LL * nsm) {
      chunk = c;
      break;
    }
  }
  if ((rc = alloc_storage(cursor + 64, count, chunks, tiles, xoff, yoff, doff, std::max(6 * maxcells, nreal))))
    return rc;
  n = count;
  for (int b = 0; b < count; ++b)
    if ((rc = place(b, probs[b], base[b], xoffv[b], yoffv[b], &doffv[4 * b], hoff[b]))) return rc;
  if ((rc = rebuild_lists())) return rc;
  SG_CUDA(cudaStreamSynchronize(stream));
  return SAYRAM_OK;
}

// Copies one instance's coefficient fields (and f0) into the staging buffer and runs k_setup.
int sayram_batch_s::upload_instance(int b, const sayram_problem& p, bool coeffs, bool f0) {
  const long long nc = (long long)p.nx * p.ny;
  const double* src[6] = {p.G, p.Dxx, p.Dxy, p.Dyy, p.inv_tau, p.f0};
  int mask = 0;
  for (int k = 0; k < 6; ++k) {
    const bool want = (k < 5) ? coeffs : f0;
    if (!want || !src[k]) continue;
    SG_CUDA(cudaMemcpyAsync(d_stage + k * nc, src[k], sizeof(double) * nc, cudaMemcpyHostToDevice, stream));
    mask |= 1 << k;
  }
  if (coeffs && (mask & 31) != 31) return fail(SAYRAM_ERR_ARG, "all coefficient fields are required");
  const int threads = 256;
  const int blocks = (int)std::min<long long>((nc + threads - 1) / threads, (long long)nsm * 8);
  if (dwm)
    sg::k_setup<sg::DWA><<<blocks, threads, 0, stream>>>(cm, geo, fl.f, d_stage, d_xe, d_ye, b, mask);
  else
    sg::k_setup<sg::F64A><<<blocks, threads, 0, stream>>>(cm, geo, fl.f, d_stage, d_xe, d_ye, b, mask);
  SG_CUDA(cudaGetLastError());
  // the staging buffer is reused by the next upload: keep the stream ordered
  SG_CUDA(cudaStreamSynchronize(stream));
  return SAYRAM_OK;
}

int sayram_batch_s::read_ctl() {
  SG_CUDA(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream));
  SG_CUDA(cudaStreamSynchronize(stream));
  return SAYRAM_OK;
}

template <typename T, typename C, typename A, int CH>
int sayram_batch_s::step_once(const sg::Coef<C>& cfull, const sg::Coef<T>& ck, const sg::Kry<T>& kr) {
  using namespace sg;
  const int gs = grid_stream(), gt = grid_tiles();
  int prc = prep_kernels<T, C, A, CH>();
  if (prc) return prc;
  SG_CUDA(cudaMemsetAsync(d_ctl, 0, 2 * sizeof(int), stream));
  launch("begin", [&] { k_begin<<<(n + 255) / 256, 256, 0, stream>>>(cm); });
  launch("assemble", [&] { k_assemble<C, A><<<gt, kAsmThreads, 0, stream>>>(cm, geo, fl, cfull, 0, -1); });
  int cgrid = coop_grid<T, C, A, CH>();
  if (cgrid != 0) {
    int crc = SAYRAM_OK;
    launch("solve_coop", [&] { crc = launch_coop<T, C, A, CH>(cgrid, cfull, ck, kr); });
    if (crc) {  // refused: the loops of separate kernels from now on
      cudaGetLastError();
      g_err.clear();
      coop = 0;
      cgrid = 0;
    }
  }
  for (int o = 0; cgrid == 0 && o < opt.max_refine; ++o) {
    launch("resid", [&] {
      k_resid<T, C, A, CH><<<gs, kThreads, smem_wide(), stream>>>(cm, fl, cfull, kr, opt.tol, opt.inner_tol, opt.max_refine);
    });
    SG_CUDA(cudaGetLastError());
    if (o == opt.max_refine - 1) break;
    int rc = read_ctl();
    if (rc) return rc;
    if (h_ctl->n_outer == 0) break;
    for (int it = 0; it < opt.max_iters; ++it) {
      // per-kernel timing also splits the Krylov time by how many instances are still
      // iterating: "krylov_tail10" holds the iterations in which fewer than 10 % are
      bool tail = false;
      if (timing) {
        if (it > 0) {
          rc = read_ctl();
          if (rc) return rc;
          if (h_ctl->n_inner == 0) break;
        }
        tail = 10LL * h_ctl->n_inner < (long long)n_enabled();
      }
      launch(tail ? "krylov_tail10" : "krylov_rest", [&] {
        launch("bicg1", [&] { k_bicg1<T, CH><<<gs, kThreads, smem_spmv<T>(), stream>>>(cm, ck, kr); });
        launch("bicg2", [&] { k_bicg2<T, CH><<<gs, kThreads, smem_spmv<T>(), stream>>>(cm, ck, kr); });
        launch("bicg3", [&] { k_bicg3<T, CH><<<gs, kThreads, 0, stream>>>(cm, kr, opt.max_iters); });
      });
      SG_CUDA(cudaGetLastError());
      if (!timing && (it < 4 || (it & 3) == 3)) {
        rc = read_ctl();
        if (rc) return rc;
        if (h_ctl->n_inner == 0) break;
      }
    }
  }
  launch("polish", [&] { k_polish<C, A, CH><<<gs, kThreads, smem_wide(), stream>>>(cm, fl, cfull, 0, -1); });
  SG_CUDA(cudaGetLastError());
  return SAYRAM_OK;
}

int sayram_batch_s::last_captured(cudaGraphNode_t* node) {
  cudaStreamCaptureStatus cs;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  SG_CUDA(cudaStreamGetCaptureInfo(stream, &cs, nullptr, nullptr, &deps, nullptr, &nd));
  if (cs != cudaStreamCaptureStatusActive || nd != 1) return fail(SAYRAM_ERR_CUDA, "unexpected capture state");
  *node = deps[0];
  return SAYRAM_OK;
}

// One step as a graph: memset + begin + assemble, WHILE(outer){ resid, WHILE(inner){ k1 k2 k3 } },
// polish. The WHILE conditions are set on the device by the residual and Krylov kernels.
template <typename T, typename C, typename A, int CH>
int sayram_batch_s::build_graph(const sg::Coef<C>& cfull, const sg::Coef<T>& ck, const sg::Kry<T>& kr, bool prefix) {
  using namespace sg;
  const int gs = grid_stream(), gt = grid_tiles();
  int prc = prep_kernels<T, C, A, CH>();
  if (prc) return prc;
  const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  cudaGraph_t g = nullptr;
  SG_CUDA(cudaGraphCreate(&g, 0));
  (prefix ? graph : graph_solve) = g;
  int rc;
  const int cgrid = coop_grid<T, C, A, CH>();
  if (cgrid != 0) {
    // [memset, begin, assemble,] the cooperative solve[, polish]
    SG_CUDA(cudaStreamBeginCaptureToGraph(stream, g, nullptr, nullptr, 0, mode));
    if (prefix) {
      cudaMemsetAsync(d_ctl, 0, 2 * sizeof(int), stream);
      k_begin<<<(n + 255) / 256, 256, 0, stream>>>(cm);
      k_assemble<C, A><<<gt, kAsmThreads, 0, stream>>>(cm, geo, fl, cfull, 0, -1);
    }
    // a capture that refuses the cooperative launch or does not keep it cooperative falls back
    // to the loops of separate kernels
    bool coop_node = launch_coop<T, C, A, CH>(cgrid, cfull, ck, kr) == SAYRAM_OK;
    cudaGraphNode_t cnode = nullptr;
    if (coop_node) coop_node = last_captured(&cnode) == SAYRAM_OK;
    if (coop_node) {
      cudaLaunchAttributeValue cv = {};
      coop_node = cudaGraphKernelNodeGetAttribute(cnode, cudaLaunchAttributeCooperative, &cv) == cudaSuccess &&
                  cv.cooperative;
    }
    if (coop_node && prefix) k_polish<C, A, CH><<<gs, kThreads, smem_wide(), stream>>>(cm, fl, cfull, 0, -1);
    cudaGraph_t gc = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(stream, &gc);
    if (!coop_node || ce != cudaSuccess) {
      cudaGetLastError();
      g_err.clear();
      cudaGraphDestroy(g);
      (prefix ? graph : graph_solve) = nullptr;
      coop = 0;
      return build_graph<T, C, A, CH>(cfull, ck, kr, prefix);
    }
    SG_CUDA(cudaGraphInstantiate(prefix ? &gexec : &gexec_solve, g, 0));
    return SAYRAM_OK;
  }
  cudaGraphConditionalHandle hout, hin;
  SG_CUDA(cudaGraphConditionalHandleCreate(&hout, g, 1, cudaGraphCondAssignDefault));
  Common c2 = cm;
  c2.use_cond = 1;
  c2.h_outer = hout;
  c2.guard_refine = opt.max_refine + 1;
  c2.guard_iters = opt.max_iters + 1;
  // prefix
  cudaGraphNode_t pre = nullptr;
  if (prefix) {
    SG_CUDA(cudaStreamBeginCaptureToGraph(stream, g, nullptr, nullptr, 0, mode));
    cudaMemsetAsync(d_ctl, 0, 2 * sizeof(int), stream);
    k_begin<<<(n + 255) / 256, 256, 0, stream>>>(c2);
    k_assemble<C, A><<<gt, kAsmThreads, 0, stream>>>(c2, geo, fl, cfull, 0, -1);
    if ((rc = last_captured(&pre))) { cudaStreamEndCapture(stream, &g); return rc; }
    SG_CUDA(cudaStreamEndCapture(stream, &g));
  }
  // outer WHILE
  cudaGraphNodeParams op = {};
  op.type = cudaGraphNodeTypeConditional;
  op.conditional.handle = hout;
  op.conditional.type = cudaGraphCondTypeWhile;
  op.conditional.size = 1;
  cudaGraphNode_t outer;
  SG_CUDA(cudaGraphAddNode(&outer, g, prefix ? &pre : nullptr, nullptr, prefix ? 1 : 0, &op));
  cudaGraph_t obody = op.conditional.phGraph_out[0];
  SG_CUDA(cudaGraphConditionalHandleCreate(&hin, obody, 0, cudaGraphCondAssignDefault));
  c2.h_inner = hin;
  cudaGraphNode_t rnode;
  SG_CUDA(cudaStreamBeginCaptureToGraph(stream, obody, nullptr, nullptr, 0, mode));
  k_resid<T, C, A, CH><<<gs, kThreads, smem_wide(), stream>>>(c2, fl, cfull, kr, opt.tol, opt.inner_tol, opt.max_refine);
  if ((rc = last_captured(&rnode))) { cudaStreamEndCapture(stream, &obody); return rc; }
  SG_CUDA(cudaStreamEndCapture(stream, &obody));
  // inner WHILE inside the outer body
  cudaGraphNodeParams ip = {};
  ip.type = cudaGraphNodeTypeConditional;
  ip.conditional.handle = hin;
  ip.conditional.type = cudaGraphCondTypeWhile;
  ip.conditional.size = 1;
  cudaGraphNode_t inner;
  SG_CUDA(cudaGraphAddNode(&inner, obody, &rnode, nullptr, 1, &ip));
  cudaGraph_t ibody = ip.conditional.phGraph_out[0];
  SG_CUDA(cudaStreamBeginCaptureToGraph(stream, ibody, nullptr, nullptr, 0, mode));
  k_bicg1<T, CH><<<gs, kThreads, smem_spmv<T>(), stream>>>(c2, ck, kr);
  k_bicg2<T, CH><<<gs, kThreads, smem_spmv<T>(), stream>>>(c2, ck, kr);
  k_bicg3<T, CH><<<gs, kThreads, 0, stream>>>(c2, kr, opt.max_iters);
  SG_CUDA(cudaStreamEndCapture(stream, &ibody));
  // suffix (the solve-only graph leaves the polish to its caller)
  if (prefix) {
    SG_CUDA(cudaStreamBeginCaptureToGraph(stream, g, &outer, nullptr, 1, mode));
    k_polish<C, A, CH><<<gs, kThreads, smem_wide(), stream>>>(c2, fl, cfull, 0, -1);
    SG_CUDA(cudaStreamEndCapture(stream, &g));
  }
  SG_CUDA(cudaGraphInstantiate(prefix ? &gexec : &gexec_solve, g, 0));
  return SAYRAM_OK;
}

int sayram_batch_s::run_steps(int nsteps) {
  int rc = launch_steps(nsteps);
  if (rc) return rc;
  SG_CUDA(cudaStreamSynchronize(stream));
  if (timing) collect_timing();
  return finish_status();
}

int sayram_batch_s::launch_steps(int nsteps) {
  if (nsteps < 0) return fail(SAYRAM_ERR_ARG, "nsteps must be >= 0");
  SG_CUDA(cudaSetDevice(dev));
  const bool use_graph = opt.use_graph && !timing;
  if (use_graph && !gexec) {
    int rc = run_mode(true);
    if (rc) {
      drop_graph();
      return rc;
    }
  }
  for (int s = 0; s < nsteps; ++s) {
    if (use_graph) {
      SG_CUDA(cudaGraphLaunch(gexec, stream));
      continue;
    }
    int rc = run_mode(false);
    if (rc) return rc;
  }
  return SAYRAM_OK;
}

namespace {
// Albert_Young's unit conversion (utils.h:12-20, common.h:41-43), host libm: the device kernel
// reads these per-row values so that its arithmetic is a fixed sequence of IEEE operations.
constexpr double kC = 1.0;          // gC
constexpr double kE0 = 0.511875;    // gE0 [MeV]
constexpr double kPi = 3.141592653589793238462;  // gPI
double host_e2p(double E, double E0) { return std::sqrt(E * (E + 2 * E0)) / kC; }
double host_dlogE_dp(double logE, double E0) {
  const double E = std::exp(logE);
  return host_e2p(E, kE0) * kC * kC / (E * (E + E0));
}
}  // namespace

// Interpolates Dxx, Dxy, Dyy from a D table at every cell centre of instance idx (all instances
// when idx < 0), as Albert_Young(_LC)::constructD does, and re-derives the face factors from them
// and the stored G. The step graph reads the factors from memory, so it stays valid.
int sayram_batch_s::set_dtable(int idx, const sayram_dtable* t) {
  if (!t || t->n_alpha < 2 || t->n_energy < 2 || !t->alpha0_deg || !t->energy || !t->Daa || !t->Dap || !t->Dpp)
    return fail(SAYRAM_ERR_ARG, "D table: needs n_alpha, n_energy >= 2 and all five arrays");
  if (idx >= n) return fail(SAYRAM_ERR_ARG, "instance index out of range");
  if (idx >= 0 && !hinst[idx].enabled) return fail(SAYRAM_ERR_STATE, "instance slot is empty");
  const int na = t->n_alpha, ne = t->n_energy;
  const double a0 = t->alpha0_deg[0], a1 = t->alpha0_deg[na - 1];
  const double e0 = t->energy[0], e1 = t->energy[ne - 1];
  if (!(a1 > a0) || !(e0 > 0.0) || !(e1 > e0) || !std::isfinite(a0) || !std::isfinite(a1) || !std::isfinite(e1))
    return fail(SAYRAM_ERR_ARG, "D table: alpha0 and energy axes must increase from end to end, energies > 0");
  SG_CUDA(cudaSetDevice(dev));
  SG_CUDA(cudaStreamSynchronize(stream));
  const long long nt = 3LL * na * ne;
  if (nt > tab_cap) {
    double* q = nullptr;
    if (cudaMalloc(&q, sizeof(double) * nt) != cudaSuccess) {
      cudaGetLastError();
      return fail(SAYRAM_ERR_OOM, "D table: no device memory for the table");
    }
    if (d_tab) cudaFree(d_tab);
    d_tab = q;
    tab_cap = nt;
  }
  if (!d_rows) {
    if (cudaMalloc(&d_rows, sizeof(double) * 3 * std::max<long long>(ycap_, 1)) != cudaSuccess) {
      cudaGetLastError();
      d_rows = nullptr;
      return fail(SAYRAM_ERR_OOM, "D table: no device memory for the row factors");
    }
  }
  const size_t tb = sizeof(double) * (size_t)na * ne;
  SG_CUDA(cudaMemcpyAsync(d_tab, t->Daa, tb, cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaMemcpyAsync(d_tab + (long long)na * ne, t->Dap, tb, cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaMemcpyAsync(d_tab + 2LL * na * ne, t->Dpp, tb, cudaMemcpyHostToDevice, stream));
  // row factors of the selected instances, from their y edges
  std::vector<double> ye(ycap_), rows(3 * ycap_, 0.0);
  SG_CUDA(cudaMemcpyAsync(ye.data(), d_ye, sizeof(double) * ycap_, cudaMemcpyDeviceToHost, stream));
  SG_CUDA(cudaStreamSynchronize(stream));
  for (int b = (idx < 0 ? 0 : idx); b < (idx < 0 ? n : idx + 1); ++b) {
    const InstDev& I = hinst[b];
    if (!I.enabled) continue;
    for (int j = 0; j < I.ny; ++j) {
      const double logE = 0.5 * (ye[I.ye + j] + ye[I.ye + j + 1]);
      const double dl = host_dlogE_dp(logE, kE0);
      rows[I.ye + j] = host_e2p(std::exp(logE), kE0);
      rows[ycap_ + I.ye + j] = dl;
      rows[2 * ycap_ + I.ye + j] = std::pow(dl, 2);
    }
  }
  SG_CUDA(cudaMemcpyAsync(d_rows, rows.data(), sizeof(double) * rows.size(), cudaMemcpyHostToDevice, stream));
  sg::DTab dt{};
  dt.na = na;
  dt.ne = ne;
  dt.xmin = a0 * kPi / 180;
  dt.xmax = a1 * kPi / 180;
  dt.lymin = std::log(e0);
  dt.lymax = std::log(e1);
  const double gme = kE0 / (kC * kC);
  dt.denorm = gme * gme * kC * kC;
  dt.Daa = d_tab;
  dt.Dap = d_tab + (long long)na * ne;
  dt.Dpp = d_tab + 2LL * na * ne;
  dt.rp = d_rows;
  dt.rdl = d_rows + ycap_;
  dt.rdl2 = d_rows + 2 * ycap_;
  const int t0 = idx < 0 ? 0 : hinst[idx].tile0;
  const int t1 = idx < 0 ? ntiles : hinst[idx].tile0 + hinst[idx].ntx * hinst[idx].nty;
  if (t1 > t0) {
    const int blocks = std::min(t1 - t0, nsm * 8);
    if (dwm)
      sg::k_dtable<sg::DWA><<<blocks, 256, 0, stream>>>(cm, geo, dt, d_xe, d_ye, t0, t1);
    else
      sg::k_dtable<sg::F64A><<<blocks, 256, 0, stream>>>(cm, geo, dt, d_xe, d_ye, t0, t1);
    SG_CUDA(cudaGetLastError());
  }
  SG_CUDA(cudaStreamSynchronize(stream));
  return SAYRAM_OK;
}

// Times `steps` steps of every launch shape (cells per chunk x blocks per SM) from the same
// state and keeps the fastest; f, the history of earlier states, the extrapolated start (in the
// y buffers) and the per-instance state are restored afterwards, so tuning does not advance the
// simulation.
int sayram_batch_s::autotune(int steps, int* best_chunk, int* best_grid) {
  if (steps < 1) steps = 1;
  SG_CUDA(cudaSetDevice(dev));
  constexpr int kSnap = 3 + sg::kHist;
  double* snap = nullptr;  // f, the history states and both y buffers
  if (cudaMalloc(&snap, sizeof(double) * kSnap * ncell) != cudaSuccess) {
    cudaGetLastError();
    return fail(SAYRAM_ERR_OOM, "autotune: no room for the state snapshot");
  }
  double* const saved[kSnap] = {fl.f, fl.fh[0], fl.fh[1], fl.fh[2], fl.y64[0], fl.y64[1]};
  std::vector<InstState> hs(cap_slots);
  for (int k = 0; k < kSnap; ++k)
    SG_CUDA(cudaMemcpyAsync(snap + k * ncell, saved[k], sizeof(double) * ncell, cudaMemcpyDeviceToDevice, stream));
  SG_CUDA(cudaMemcpyAsync(hs.data(), d_st, sizeof(InstState) * cap_slots, cudaMemcpyDeviceToHost, stream));
  SG_CUDA(cudaStreamSynchronize(stream));
  auto restore = [&]() -> int {
    for (int k = 0; k < kSnap; ++k)
      SG_CUDA(cudaMemcpyAsync(saved[k], snap + k * ncell, sizeof(double) * ncell, cudaMemcpyDeviceToDevice, stream));
    SG_CUDA(cudaMemcpyAsync(d_st, hs.data(), sizeof(InstState) * cap_slots, cudaMemcpyHostToDevice, stream));
    SG_CUDA(cudaStreamSynchronize(stream));
    return SAYRAM_OK;
  };
  cudaEvent_t e0, e1;
  SG_CUDA(cudaEventCreate(&e0));
  SG_CUDA(cudaEventCreate(&e1));
  // blocks per SM: more blocks than fit at once balance the uneven chunks better (on the 4096-
  // instance batch: 23.2, 21.8, 21.0, 20.8 ms per step for 8, 12, 32, 48)
  const int chunks[3] = {1024, 2048, 4096}, grids[4] = {8, 16, 32, 64};
  const bool timing_was = timing;
  timing = false;  // per-kernel events would split the graph into a host loop
  double best = 1e300;
  int bc = chunk, bg = gmult, rc = SAYRAM_OK;
  tune_log.clear();
  for (int ci = 0; ci < 3 && rc == SAYRAM_OK; ++ci)
    for (int gi = 0; gi < 4 && rc == SAYRAM_OK; ++gi) {
      chunk = chunks[ci];
      gmult = grids[gi];
      drop_graph();
      if ((rc = rebuild_lists())) break;
      if ((rc = launch_steps(1))) break;  // builds the graph, warms up
      if ((rc = restore())) break;
      cudaEventRecord(e0, stream);
      if ((rc = launch_steps(steps))) break;
      cudaEventRecord(e1, stream);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      tune_log.push_back({chunk, gmult, (double)ms / steps});
      if (ms < best) {
        best = ms;
        bc = chunk;
        bg = gmult;
      }
      if ((rc = restore())) break;
    }
  chunk = bc;
  gmult = bg;
  drop_graph();
  int rc2 = rebuild_lists();
  if (!rc2) rc2 = restore();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(snap);
  timing = timing_was;
  if (rc) return rc;
  if (rc2) return rc2;
  if (best_chunk) *best_chunk = bc;
  if (best_grid) *best_grid = bg;
  return SAYRAM_OK;
}

int sayram_batch_s::finish_status() {
  std::vector<InstState> hs(n);
  SG_CUDA(cudaMemcpyAsync(hs.data(), d_st, sizeof(InstState) * n, cudaMemcpyDeviceToHost, stream));
  SG_CUDA(cudaStreamSynchronize(stream));
  int worst = SAYRAM_OK;
  for (int b = 0; b < n; ++b) {
    if (!hinst[b].enabled || hs[b].steps == 0) continue;
    if (hs[b].status == sg::ST_NEGATIVE) worst = SAYRAM_ERR_NEGATIVE;
    else if (hs[b].status == sg::ST_NOT_CONVERGED && worst == SAYRAM_OK) worst = SAYRAM_ERR_NOT_CONVERGED;
  }
  if (worst == SAYRAM_ERR_NEGATIVE) return fail(worst, "a negative cell survived the positivity polish");
  if (worst == SAYRAM_ERR_NOT_CONVERGED) return fail(worst, "a step ended above the residual target");
  return SAYRAM_OK;
}

namespace sg {
int host_fail(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace sg

// ================================================================================== C-ABI
extern "C" {

const char* sayram_last_error(void) { return g_err.c_str(); }
const char* sayram_version(void) { return "sayram-gb300 0.1 (sm_103a)"; }

void sayram_default_options(sayram_options* o) {
  if (!o) return;
  o->precision = SAYRAM_FP64;
  o->tol = 0.0;
  o->inner_tol = -1.0;
  o->max_iters = 500;
  o->max_refine = 6;
  o->device = 0;
  o->use_graph = 1;
  o->precond = SAYRAM_PRECOND_ALPHA_LINE;
}

void* sayram_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    g_err = "cudaMallocHost failed";
    return nullptr;
  }
  return p;
}
void sayram_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int sayram_batch_create(const sayram_problem* probs, int n, const sayram_options* opt, sayram_batch* out) {
  if (!out) return fail(SAYRAM_ERR_ARG, "null output handle");
  *out = nullptr;
  if (!probs || n < 1) return fail(SAYRAM_ERR_ARG, "empty batch");
  sayram_batch_s* b = new (std::nothrow) sayram_batch_s();
  if (!b) return fail(SAYRAM_ERR_OOM, "host allocation failed");
  sayram_options o;
  sayram_default_options(&o);
  if (opt) o = *opt;
  if (o.inner_tol < 0) o.inner_tol = (o.precision != SAYRAM_FP64) ? 1e-4 : 0.0;
  int rc = b->build(probs, n, &o);
  if (rc) {
    std::string msg = g_err;
    delete b;
    return fail(rc, msg);
  }
  *out = b;
  g_err.clear();
  return SAYRAM_OK;
}

int sayram_batch_size(sayram_batch b) { return b ? b->n : 0; }

int sayram_batch_step(sayram_batch b, int nsteps) {
  if (!b) return fail(SAYRAM_ERR_ARG, "null handle");
  return b->run_steps(nsteps);
}

// The instances are split into about kPieces runs at instance boundaries (a small first run);
// while the copy engine moves one run between host and staging memory (cstream), the layout
// kernel transforms the run before it (stream). Copies go through the copy engine, which is
// faster than kernels reading host memory over the CPU-GPU link (208 against 153 GB/s on GB300).
int sayram_batch_step_host(sayram_batch b, int nsteps, const double* f_in, double* f_out) {
  if (!b) return fail(SAYRAM_ERR_ARG, "null handle");
  if (nsteps < 0) return fail(SAYRAM_ERR_ARG, "nsteps must be >= 0");
  SG_CUDA(cudaSetDevice(b->dev));
  constexpr int kPieces = 16;  // per call, 8 / 12 / 16 runs: 17.3 / 17.0 / 17.0 ms (4096 instances)
  struct Piece {
    long long off, len;  // doubles of the packed host array
    int t0, t1;          // tiles
    int c0, c1;          // chunks
  };
  std::vector<Piece> pieces;
  {
    // the first run is small (a quarter of the others): its copy in is what the first assembly
    // waits for, and its polish is what the first copy out waits for; the rest are about equal
    const long long target = (b->nreal + kPieces - 1) / kPieces;
    const long long first = (b->nreal + 4 * kPieces - 1) / (4 * kPieces);
    int a = 0;
    while (a < b->n) {
      long long len = 0;
      int e = a;
      const long long want = pieces.empty() ? first : target;
      while (e < b->n && (len < want || e == a)) {
        len += (long long)b->hinst[e].nx * b->hinst[e].ny;
        ++e;
      }
      const sg::InstDev& A = b->hinst[a];
      const sg::InstDev& E = b->hinst[e - 1];
      pieces.push_back({A.hoff, len, A.tile0, E.tile0 + E.ntx * E.nty, A.chunk0, E.chunk0 + E.nchunks});
      a = e;
    }
  }
  const size_t np = pieces.size();
  while (b->piece_ev.size() < 3 * np + 1) {
    cudaEvent_t e;
    SG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b->piece_ev.push_back(e);
  }
  const int gt = b->grid_tiles();
  auto field_in = [&](const Piece& pc, cudaStream_t s) {
    b->launch("field_in", [&] {
      if (b->dwm)
        sg::k_field_in<sg::DWA><<<gt, sg::kFieldThreads, 0, s>>>(b->cm, b->fl.f, b->d_stage, 1, pc.t0, pc.t1);
      else
        sg::k_field_in<sg::F64A><<<gt, sg::kFieldThreads, 0, s>>>(b->cm, b->fl.f, b->d_stage, 1, pc.t0, pc.t1);
    });
  };
  auto field_out = [&](const Piece& pc) {
    b->launch("field_out", [&] {
      if (b->dwm)
        sg::k_field_out<sg::DWA><<<gt, 256, 0, b->stream>>>(b->cm, b->d_stage, b->fl.f, pc.t0, pc.t1);
      else
        sg::k_field_out<sg::F64A><<<gt, 256, 0, b->stream>>>(b->cm, b->d_stage, b->fl.f, pc.t0, pc.t1);
    });
  };
  auto copy_in = [&](size_t k) -> int {  // H2D of piece k on the copy stream, then an event
    const Piece& pc = pieces[k];
    SG_CUDA(cudaMemcpyAsync(b->d_stage + pc.off, f_in + pc.off, sizeof(double) * pc.len, cudaMemcpyHostToDevice,
                            b->cstream));
    SG_CUDA(cudaEventRecord(b->piece_ev[k], b->cstream));
    return SAYRAM_OK;
  };
  auto copy_out = [&](size_t k) -> int {  // after piece k's transform: D2H on the copy stream
    const Piece& pc = pieces[k];
    SG_CUDA(cudaEventRecord(b->piece_ev[np + k], b->stream));
    SG_CUDA(cudaStreamWaitEvent(b->cstream, b->piece_ev[np + k], 0));
    SG_CUDA(cudaMemcpyAsync(f_out + pc.off, b->d_stage + pc.off, sizeof(double) * pc.len, cudaMemcpyDeviceToHost,
                            b->cstream));
    return SAYRAM_OK;
  };
  // An instance whose state changed restarts its extrapolation history; one given back its own
  // current state (a host round trip) keeps it (k_field_in compares bit for bit).
  int rc = SAYRAM_OK;
  const bool split = b->opt.use_graph && !b->timing && nsteps >= 1 && np >= 2 && (f_in || f_out);
  if (split) {
    // Graph stepping with host buffers: the first step's assembly runs piece by piece behind the
    // copies in (each piece's tiles as soon as its cells have landed), and the last step's
    // polish runs piece by piece ahead of the copies out; in between, graphs. Every piece holds
    // whole instances, so the per-instance reductions stay inside one launch.
    if ((rc = b->ensure_solve_graph())) return rc;
    if (nsteps > 2 && (rc = b->launch_steps(0))) return rc;  // builds the full step's graph up front
    for (int s = 0; s < nsteps; ++s) {
      const bool head = s == 0 && f_in, tail = s == nsteps - 1 && f_out;
      if (!head && !tail) {
        if ((rc = b->launch_steps(1))) return rc;
        continue;
      }
      if (head) {
        // the transforms run on their own stream, so that piece k+1's transform overlaps piece
        // k's assembly (different instances); it starts after everything queued so far
        SG_CUDA(cudaEventRecord(b->piece_ev[3 * np], b->stream));
        SG_CUDA(cudaStreamWaitEvent(b->tstream, b->piece_ev[3 * np], 0));
      }
      if ((rc = b->launch_begin())) return rc;
      if (head) {
        for (size_t k = 0; k < np; ++k)
          if ((rc = copy_in(k))) return rc;
        for (size_t k = 0; k < np; ++k) {
          SG_CUDA(cudaStreamWaitEvent(b->tstream, b->piece_ev[k], 0));
          field_in(pieces[k], b->tstream);
          SG_CUDA(cudaEventRecord(b->piece_ev[2 * np + k], b->tstream));
        }
        for (size_t k = 0; k < np; ++k) {
          SG_CUDA(cudaStreamWaitEvent(b->stream, b->piece_ev[2 * np + k], 0));
          if ((rc = b->launch_assemble(pieces[k].t0, pieces[k].t1))) return rc;
        }
      } else if ((rc = b->launch_assemble(0, -1))) {
        return rc;
      }
      if ((rc = b->launch_solve())) return rc;
      if (tail) {
        for (size_t k = 0; k < np; ++k) {
          if ((rc = b->launch_polish(pieces[k].c0, pieces[k].c1))) return rc;
          field_out(pieces[k]);
          if ((rc = copy_out(k))) return rc;
        }
      } else if ((rc = b->launch_polish(0, -1))) {
        return rc;
      }
    }
    SG_CUDA(cudaStreamSynchronize(b->cstream));
    SG_CUDA(cudaStreamSynchronize(b->stream));
    return b->finish_status();
  }
  if (f_in) {
    for (size_t k = 0; k < np; ++k) {
      if ((rc = copy_in(k))) return rc;
      SG_CUDA(cudaStreamWaitEvent(b->stream, b->piece_ev[k], 0));
      field_in(pieces[k], b->stream);
    }
  }
  rc = b->run_steps(nsteps);
  if (rc != SAYRAM_OK && rc != SAYRAM_ERR_NOT_CONVERGED && rc != SAYRAM_ERR_NEGATIVE) return rc;
  if (f_out) {
    for (size_t k = 0; k < np; ++k) {
      field_out(pieces[k]);
      int rc2 = copy_out(k);
      if (rc2) return rc2;
    }
    SG_CUDA(cudaStreamSynchronize(b->cstream));
    SG_CUDA(cudaStreamSynchronize(b->stream));
    if (b->timing) b->collect_timing();
  }
  return rc;
}

int sayram_batch_get_f(sayram_batch b, int idx, double* f_out) {
  if (!b || !f_out || idx < 0 || idx >= b->n) return fail(SAYRAM_ERR_ARG, "bad handle, index or buffer");
  SG_CUDA(cudaSetDevice(b->dev));
  const InstDev& I = b->hinst[idx];
  // rows of the padded layout -> alpha-major on the host
  std::vector<double> rows((size_t)I.ny * I.pitch);
  SG_CUDA(cudaMemcpyAsync(rows.data(), b->fl.f + I.base, sizeof(double) * rows.size(), cudaMemcpyDeviceToHost, b->stream));
  SG_CUDA(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < I.nx; ++i)
    for (int j = 0; j < I.ny; ++j) f_out[(size_t)i * I.ny + j] = b->unwide(rows[(size_t)j * I.pitch + i]);
  return SAYRAM_OK;
}

int sayram_batch_set_f(sayram_batch b, int idx, const double* f) {
  if (!b || !f || idx < 0 || idx >= b->n) return fail(SAYRAM_ERR_ARG, "bad handle, index or buffer");
  SG_CUDA(cudaSetDevice(b->dev));
  const InstDev& I = b->hinst[idx];
  std::vector<double> rows((size_t)I.ny * I.pitch, 0.0);
  for (int i = 0; i < I.nx; ++i)
    for (int j = 0; j < I.ny; ++j) rows[(size_t)j * I.pitch + i] = b->wide(f[(size_t)i * I.ny + j]);
  SG_CUDA(cudaMemcpyAsync(b->fl.f + I.base, rows.data(), sizeof(double) * rows.size(), cudaMemcpyHostToDevice, b->stream));
  SG_CUDA(cudaMemsetAsync((char*)(b->d_st + idx) + offsetof(InstState, nhist), 0, sizeof(int), b->stream));
  SG_CUDA(cudaStreamSynchronize(b->stream));
  return SAYRAM_OK;
}

int sayram_batch_set_dirichlet(sayram_batch b, int idx, int side, const double* v, int n) {
  if (!b || !v || idx < 0 || idx >= b->n || side < 0 || side > 3)
    return fail(SAYRAM_ERR_ARG, "bad handle, index, side or buffer");
  const InstDev& I = b->hinst[idx];
  if (I.dir[side] < 0) return fail(SAYRAM_ERR_ARG, "side is not Dirichlet");
  const int m = (side <= 1) ? I.ny + 1 : I.nx + 1;
  if (n != m) return fail(SAYRAM_ERR_ARG, "expected " + std::to_string(m) + " vertex values");
  SG_CUDA(cudaSetDevice(b->dev));
  std::vector<double> wv(m);
  for (int k = 0; k < m; ++k) wv[k] = b->wide(v[k]);
  SG_CUDA(cudaMemcpyAsync(b->d_dirv + I.dir[side], wv.data(), sizeof(double) * m, cudaMemcpyHostToDevice, b->stream));
  SG_CUDA(cudaStreamSynchronize(b->stream));
  return SAYRAM_OK;
}

int sayram_batch_set_coeffs(sayram_batch b, int idx, const double* G, const double* Dxx, const double* Dxy,
                            const double* Dyy, const double* inv_tau) {
  if (!b || idx < 0 || idx >= b->n) return fail(SAYRAM_ERR_ARG, "bad handle or index");
  SG_CUDA(cudaSetDevice(b->dev));
  const InstDev& I = b->hinst[idx];
  const long long nc = (long long)I.nx * I.ny;
  // fields not given keep their current values: fetch them back is not possible (only derived
  // factors are stored), so all five are required unless the caller passes every one.
  if (!G || !Dxx || !Dxy || !Dyy || !inv_tau)
    return fail(SAYRAM_ERR_ARG, "set_coeffs needs all of G, Dxx, Dxy, Dyy, inv_tau");
  sayram_problem p{};
  p.nx = I.nx;
  p.ny = I.ny;
  p.G = G;
  p.Dxx = Dxx;
  p.Dxy = Dxy;
  p.Dyy = Dyy;
  p.inv_tau = inv_tau;
  (void)nc;
  return b->upload_instance(idx, p, true, false);
}

int sayram_batch_stats(sayram_batch b, int idx, sayram_stats* out) {
  if (!b || !out || idx < 0 || idx >= b->n) return fail(SAYRAM_ERR_ARG, "bad handle, index or buffer");
  SG_CUDA(cudaSetDevice(b->dev));
  InstState s;
  SG_CUDA(cudaMemcpyAsync(&s, b->d_st + idx, sizeof(s), cudaMemcpyDeviceToHost, b->stream));
  SG_CUDA(cudaStreamSynchronize(b->stream));
  out->steps = s.steps;
  out->t = (double)s.steps * b->hinst[idx].dt;
  out->status = s.steps == 0 ? SAYRAM_OK
                : s.status == sg::ST_NEGATIVE ? SAYRAM_ERR_NEGATIVE
                : s.status == sg::ST_NOT_CONVERGED ? SAYRAM_ERR_NOT_CONVERGED : SAYRAM_OK;
  out->refinements = s.refines;
  out->iterations = s.iters_total;
  out->rel_residual = s.rel;
  out->min_f = s.min_f;
  out->clamped = s.clamped;
  out->mass_drift = s.mass_drift;
  out->total_iterations = s.cum_iters;
  out->total_refinements = s.cum_refines;
  return SAYRAM_OK;
}

int sayram_batch_export_system(sayram_batch b, int idx, double* M5, double* R) {
  if (!b || !M5 || !R || idx < 0 || idx >= b->n) return fail(SAYRAM_ERR_ARG, "bad handle, index or buffer");
  SG_CUDA(cudaSetDevice(b->dev));
  const InstDev& I = b->hinst[idx];
  if (b->dwm)
    sg::k_assemble<float, sg::DWA><<<b->grid_tiles(), sg::kAsmThreads, 0, b->stream>>>(b->cm, b->geo, b->fl, b->c32, 0, -1);
  else if (b->mixed)
    sg::k_assemble<float, sg::F64A><<<b->grid_tiles(), sg::kAsmThreads, 0, b->stream>>>(b->cm, b->geo, b->fl, b->c32, 0, -1);
  else
    sg::k_assemble<double, sg::F64A><<<b->grid_tiles(), sg::kAsmThreads, 0, b->stream>>>(b->cm, b->geo, b->fl, b->c64, 0, -1);
  SG_CUDA(cudaGetLastError());
  const size_t rows = (size_t)I.ny * I.pitch;
  std::vector<double> invD(rows), Rr(rows), c[4];
  SG_CUDA(cudaMemcpyAsync(invD.data(), b->fl.invD + I.base, rows * 8, cudaMemcpyDeviceToHost, b->stream));
  SG_CUDA(cudaMemcpyAsync(Rr.data(), b->fl.R + I.base, rows * 8, cudaMemcpyDeviceToHost, b->stream));
  for (int k = 0; k < 4; ++k) {
    c[k].resize(rows);
    if (b->mixed) {
      std::vector<float> hi(rows), lo(rows);
      float* hs[4] = {b->c32.cw, b->c32.ce, b->c32.cs, b->c32.cn};
      float* ls[4] = {b->c32.lw, b->c32.le, b->c32.ls, b->c32.ln};
      SG_CUDA(cudaMemcpyAsync(hi.data(), hs[k] + I.base, rows * 4, cudaMemcpyDeviceToHost, b->stream));
      SG_CUDA(cudaMemcpyAsync(lo.data(), ls[k] + I.base, rows * 4, cudaMemcpyDeviceToHost, b->stream));
      SG_CUDA(cudaStreamSynchronize(b->stream));
      for (size_t q = 0; q < rows; ++q) c[k][q] = (double)hi[q] + (double)lo[q];
    } else {
      double* ds[4] = {b->c64.cw, b->c64.ce, b->c64.cs, b->c64.cn};
      SG_CUDA(cudaMemcpyAsync(c[k].data(), ds[k] + I.base, rows * 8, cudaMemcpyDeviceToHost, b->stream));
    }
  }
  SG_CUDA(cudaStreamSynchronize(b->stream));
  const int nx = I.nx, ny = I.ny, P = I.pitch;
  const size_t N = (size_t)nx * ny;
  auto Dof = [&](int i, int j) { return 1.0 / b->unwide(invD[(size_t)j * P + i]); };
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const size_t K = (size_t)j * nx + i, q = (size_t)j * P + i;
      M5[K] = Dof(i, j);
      M5[N + K] = i > 0 ? -c[0][q] * Dof(i - 1, j) : 0.0;
      M5[2 * N + K] = i < nx - 1 ? -c[1][q] * Dof(i + 1, j) : 0.0;
      M5[3 * N + K] = j > 0 ? -c[2][q] * Dof(i, j - 1) : 0.0;
      M5[4 * N + K] = j < ny - 1 ? -c[3][q] * Dof(i, j + 1) : 0.0;
      R[K] = b->unwide(Rr[q]);
    }
  return SAYRAM_OK;
}

size_t sayram_batch_device_bytes(sayram_batch b) { return b ? b->bytes : 0; }
void* sayram_batch_stream(sayram_batch b) { return b ? (void*)b->stream : nullptr; }

int sayram_batch_record_event(sayram_batch b, int slot) {
  if (!b || slot < 0 || slot >= 8) return fail(SAYRAM_ERR_ARG, "bad handle or slot");
  SG_CUDA(cudaSetDevice(b->dev));
  if (!b->slots[slot]) SG_CUDA(cudaEventCreate(&b->slots[slot]));
  SG_CUDA(cudaEventRecord(b->slots[slot], b->stream));
  return SAYRAM_OK;
}

int sayram_batch_elapsed_ms(sayram_batch b, int slot0, int slot1, double* ms) {
  if (!b || !ms || slot0 < 0 || slot0 >= 8 || slot1 < 0 || slot1 >= 8 || !b->slots[slot0] || !b->slots[slot1])
    return fail(SAYRAM_ERR_ARG, "bad handle or unrecorded slot");
  SG_CUDA(cudaEventSynchronize(b->slots[slot1]));
  float f = 0.f;
  SG_CUDA(cudaEventElapsedTime(&f, b->slots[slot0], b->slots[slot1]));
  *ms = f;
  return SAYRAM_OK;
}

int sayram_batch_enable_timing(sayram_batch b, int enable) {
  if (!b) return fail(SAYRAM_ERR_ARG, "null handle");
  b->timing = enable != 0;
  for (auto& t : b->tms) t = 0.0;
  for (auto& c : b->tcount) c = 0;
  return SAYRAM_OK;
}

int sayram_batch_kernel_times(sayram_batch b, const char** names, double* total_ms, long long* launches, int cap) {
  if (!b) return fail(SAYRAM_ERR_ARG, "null handle");
  const int m = (int)b->tnames.size();
  for (int k = 0; k < m && k < cap; ++k) {
    if (names) names[k] = b->tnames[k].c_str();
    if (total_ms) total_ms[k] = b->tms[k];
    if (launches) launches[k] = b->tcount[k];
  }
  return m;
}

int sayram_batch_autotune(sayram_batch b, int steps, int* chunk_out, int* blocks_per_sm_out) {
  if (!b) return fail(SAYRAM_ERR_ARG, "null handle");
  return b->autotune(steps, chunk_out, blocks_per_sm_out);
}

int sayram_batch_set_dtable(sayram_batch b, int idx, const sayram_dtable* t) {
  if (!b) return fail(SAYRAM_ERR_ARG, "null handle");
  return b->set_dtable(idx, t);
}

int sayram_set_dtable(sayram_solver s, const sayram_dtable* t) { return sayram_batch_set_dtable(s, 0, t); }

int sayram_batch_set_coop(sayram_batch b, int on) {
  if (!b) return fail(SAYRAM_ERR_ARG, "null handle");
  SG_CUDA(cudaSetDevice(b->dev));
  SG_CUDA(cudaStreamSynchronize(b->stream));
  b->coop = on ? 1 : 0;
  b->drop_graph();
  return SAYRAM_OK;
}

int sayram_batch_set_launch_shape(sayram_batch b, int chunk, int blocks_per_sm) {
  if (!b) return fail(SAYRAM_ERR_ARG, "null handle");
  if (chunk != 1024 && chunk != 2048 && chunk != 4096) return fail(SAYRAM_ERR_ARG, "chunk must be 1024, 2048 or 4096");
  if (blocks_per_sm < 1 || blocks_per_sm > 64) return fail(SAYRAM_ERR_ARG, "blocks_per_sm must be in [1, 64]");
  SG_CUDA(cudaSetDevice(b->dev));
  SG_CUDA(cudaStreamSynchronize(b->stream));
  b->chunk = chunk;
  b->gmult = blocks_per_sm;
  b->drop_graph();
  return b->rebuild_lists();
}

int sayram_batch_get_launch_shape(sayram_batch b, int* chunk, int* blocks_per_sm) {
  if (!b) return fail(SAYRAM_ERR_ARG, "null handle");
  if (chunk) *chunk = b->chunk;
  if (blocks_per_sm) *blocks_per_sm = b->gmult;
  return SAYRAM_OK;
}

int sayram_batch_tuning_log(sayram_batch b, int* chunks, int* blocks_per_sm, double* ms_per_step, int cap) {
  if (!b) return fail(SAYRAM_ERR_ARG, "null handle");
  const int m = (int)b->tune_log.size();
  for (int k = 0; k < m && k < cap; ++k) {
    if (chunks) chunks[k] = b->tune_log[k].chunk;
    if (blocks_per_sm) blocks_per_sm[k] = b->tune_log[k].gmult;
    if (ms_per_step) ms_per_step[k] = b->tune_log[k].ms_per_step;
  }
  return m;
}

long long sayram_batch_launches(sayram_batch b) {
  if (!b) return -1;
  if (cudaSetDevice(b->dev) != cudaSuccess) return -1;
  Ctl c;
  if (cudaMemcpyAsync(&c, b->d_ctl, sizeof(c), cudaMemcpyDeviceToHost, b->stream) != cudaSuccess) return -1;
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return -1;
  return (long long)c.launches;
}

void sayram_batch_destroy(sayram_batch b) { delete b; }

size_t sayram_instance_bytes(int nx, int ny, int precision) {
  const long long pitch = round_up(nx, 4);
  const long long cells = round_up((long long)(ny + 2) * pitch, 32);
  const long long per = 19 * 8 + (precision != SAYRAM_FP64 ? 8 * 4 + 8 * 4 : 4 * 8 + 8 * 8) + 8;
  return (size_t)(cells * per + 4096);
}

// ---- single instance (class Solver drop-in)
int sayram_create(const sayram_problem* p, const sayram_options* opt, sayram_solver* out) {
  return sayram_batch_create(p, 1, opt, out);
}
int sayram_update(sayram_solver s) { return sayram_batch_step(s, 1); }
int sayram_step(sayram_solver s, int nsteps) { return sayram_batch_step(s, nsteps); }
double sayram_t(sayram_solver s) {
  sayram_stats st;
  if (!s || sayram_batch_stats(s, 0, &st) != SAYRAM_OK) return 0.0;
  return st.t;
}
int sayram_get_f(sayram_solver s, double* f_out) { return sayram_batch_get_f(s, 0, f_out); }
int sayram_set_f(sayram_solver s, const double* f) { return sayram_batch_set_f(s, 0, f); }
int sayram_set_dirichlet(sayram_solver s, int side, const double* v, int n) {
  return sayram_batch_set_dirichlet(s, 0, side, v, n);
}
int sayram_set_coeffs(sayram_solver s, const double* G, const double* Dxx, const double* Dxy,
                      const double* Dyy, const double* inv_tau) {
  return sayram_batch_set_coeffs(s, 0, G, Dxx, Dxy, Dyy, inv_tau);
}
int sayram_get_stats(sayram_solver s, sayram_stats* out) { return sayram_batch_stats(s, 0, out); }
void sayram_destroy(sayram_solver s) { sayram_batch_destroy(s); }

}  // extern "C"


// ================================================================================== server
namespace {

double now_seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
  long long id = 0;
  int nsteps = 0;
  double t_submit = 0.0;
  sayram_problem p{};
  std::vector<double> xe, ye, G, Dxx, Dxy, Dyy, itau, f0, dir[4];
  void own(const sayram_problem& q) {
    const size_t nc = (size_t)q.nx * q.ny;
    xe.assign(q.x_edges, q.x_edges + q.nx + 1);
    ye.assign(q.y_edges, q.y_edges + q.ny + 1);
    G.assign(q.G, q.G + nc);
    Dxx.assign(q.Dxx, q.Dxx + nc);
    Dxy.assign(q.Dxy, q.Dxy + nc);
    Dyy.assign(q.Dyy, q.Dyy + nc);
    itau.assign(q.inv_tau, q.inv_tau + nc);
    f0.assign(q.f0, q.f0 + nc);
    p = q;
    p.x_edges = xe.data();
    p.y_edges = ye.data();
    p.G = G.data();
    p.Dxx = Dxx.data();
    p.Dxy = Dxy.data();
    p.Dyy = Dyy.data();
    p.inv_tau = itau.data();
    p.f0 = f0.data();
    for (int s = 0; s < 4; ++s) {
      if (q.bc[s] == SAYRAM_DIRICHLET) {
        const int m = (s <= 1) ? q.ny + 1 : q.nx + 1;
        dir[s].assign(q.dirichlet[s], q.dirichlet[s] + m);
        p.dirichlet[s] = dir[s].data();
      } else {
        p.dirichlet[s] = nullptr;
      }
    }
  }
};

struct Result {
  std::vector<double> f;
  sayram_stats st{};
  double t_submit = 0.0, t_done = 0.0;
};

long long region_cells(int nx, int ny) { return round_up((long long)(ny + 2) * round_up(nx, 4), 32); }

}  // namespace

// One lane of the server: an engine with its own stream, arena, slots and queue. A lane runs one
// step at a time; the server launches every idle lane that has work and collects each lane when
// its step has finished, so lanes of small and of large instances advance at their own pace.
struct ServerLane {
  sayram_batch_s eng;
  sayram_server_config cfg{};
  long long arena = 0;
  std::map<long long, long long> free_;  // offset -> length (cells), coalesced
  struct Slot {
    bool used = false;
    long long id = 0, begin = 0, len = 0;
    int nsteps = 0, done = 0, nx = 0, ny = 0;
    double t_submit = 0.0;
  };
  std::vector<Slot> slots;
  std::deque<Request*> waiting;
  sayram_server_info info{};
  bool dirty = false;
  bool inflight = false;         // a step has been launched and not yet collected
  cudaEvent_t done_ev = nullptr;  // recorded after the step's launches
  double t_launch = 0.0, t_begin = 0.0;

  ~ServerLane() {
    if (inflight && done_ev) cudaEventSynchronize(done_ev);  // the engine's arrays outlive its step
    for (Request* r : waiting) delete r;
    if (done_ev) cudaEventDestroy(done_ev);
  }

  bool take(long long len, long long* off) {  // first fit
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= len) {
        *off = it->first;
        const long long rest = it->second - len, start = it->first + len;
        free_.erase(it);
        if (rest > 0) free_[start] = rest;
        return true;
      }
    }
    return false;
  }
  void give(long long off, long long len) {
    auto it = free_.emplace(off, len).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }

  int admit_one(Request* r, int slot, long long off) {
    const int ms = cfg.max_side + 1;
    int dir_off[4];
    for (int s2 = 0; s2 < 4; ++s2) dir_off[s2] = (slot * 4 + s2) * ms;
    const long long len = region_cells(r->p.nx, r->p.ny);
    int rc = eng.zero_region(off, off + len);
    if (rc) return rc;
    rc = eng.place(slot, r->p, off + round_up(r->p.nx, 4), slot * ms, slot * ms, dir_off, 0);
    if (rc) return rc;
    Slot& S = slots[slot];
    S.used = true;
    S.id = r->id;
    S.begin = off;
    S.len = len;
    S.nsteps = r->nsteps;
    S.done = 0;
    S.nx = r->p.nx;
    S.ny = r->p.ny;
    S.t_submit = r->t_submit;
    info.admitted++;
    info.resident++;
    info.arena_cells_used += (double)len;
    return SAYRAM_OK;
  }

  int admit() {
    int scanned = 0;
    for (auto it = waiting.begin(); it != waiting.end() && scanned < 9;) {
      Request* r = *it;
      int slot = -1;
      for (int k = 0; k < cfg.max_slots; ++k)
        if (!slots[k].used) {
          slot = k;
          break;
        }
      if (slot < 0) break;
      long long off;
      if (!take(region_cells(r->p.nx, r->p.ny), &off)) {
        ++it;
        ++scanned;
        continue;
      }
      int rc = admit_one(r, slot, off);
      if (rc) return rc;
      delete r;
      it = waiting.erase(it);
      info.waiting--;
      dirty = true;
    }
    return SAYRAM_OK;
  }

  // admission, work lists, then the step's launches (not waited for)
  int launch() {
    SG_CUDA(cudaSetDevice(eng.dev));
    const double t0 = now_seconds();
    int rc = admit();
    if (rc) return rc;
    const double ta = now_seconds();
    info.admit_seconds += ta - t0;
    if (dirty) {
      if ((rc = eng.rebuild_lists())) return rc;
      dirty = false;
    }
    const double tl = now_seconds();
    info.lists_seconds += tl - ta;
    if (info.resident == 0) return SAYRAM_OK;
    if ((rc = eng.launch_steps(1))) return rc;
    SG_CUDA(cudaEventRecord(done_ev, eng.stream));
    inflight = true;
    t_begin = t0;
    t_launch = tl;
    return SAYRAM_OK;
  }

  // 1 if the launched step has finished, 0 if not yet, < 0 on a CUDA error
  int ready() {
    const cudaError_t e = cudaEventQuery(done_ev);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    fail(SAYRAM_ERR_CUDA, std::string("server step: ") + cudaGetErrorString(e));
    return -1;
  }

  // after the step: completions (state rows back to the host), then free their slots
  int finish(std::map<long long, Result>& results, int* ncomp) {
    if (ncomp) *ncomp = 0;
    SG_CUDA(cudaSetDevice(eng.dev));
    inflight = false;
    const double ts = now_seconds();
    info.step_seconds += ts - t_launch;
    info.ticks++;
    info.instance_steps += info.resident;
    std::vector<int> fin;
    for (int k = 0; k < cfg.max_slots; ++k)
      if (slots[k].used && ++slots[k].done >= slots[k].nsteps) fin.push_back(k);
    std::vector<std::vector<double>> rows(fin.size());
    std::vector<InstState> sts(fin.size());
    for (size_t q = 0; q < fin.size(); ++q) {
      const InstDev& I = eng.hinst[fin[q]];
      rows[q].resize((size_t)I.ny * I.pitch);
      SG_CUDA(cudaMemcpyAsync(rows[q].data(), eng.fl.f + I.base, sizeof(double) * rows[q].size(),
                              cudaMemcpyDeviceToHost, eng.stream));
      SG_CUDA(cudaMemcpyAsync(&sts[q], eng.d_st + fin[q], sizeof(InstState), cudaMemcpyDeviceToHost, eng.stream));
    }
    SG_CUDA(cudaStreamSynchronize(eng.stream));
    const double t1 = now_seconds();
    info.busy_seconds += t1 - t_begin;
    info.collect_seconds += t1 - ts;
    for (size_t q = 0; q < fin.size(); ++q) {
      Slot& S = slots[fin[q]];
      InstDev& I = eng.hinst[fin[q]];
      Result& R = results[S.id];
      R.f.resize((size_t)S.nx * S.ny);
      for (int i = 0; i < S.nx; ++i)
        for (int j = 0; j < S.ny; ++j) R.f[(size_t)i * S.ny + j] = eng.unwide(rows[q][(size_t)j * I.pitch + i]);
      const InstState& hs = sts[q];
      R.st.steps = hs.steps;
      R.st.t = (double)hs.steps * I.dt;
      R.st.status = hs.status == sg::ST_NEGATIVE ? SAYRAM_ERR_NEGATIVE
                    : hs.status == sg::ST_NOT_CONVERGED ? SAYRAM_ERR_NOT_CONVERGED : SAYRAM_OK;
      R.st.refinements = hs.refines;
      R.st.iterations = hs.iters_total;
      R.st.rel_residual = hs.rel;
      R.st.min_f = hs.min_f;
      R.st.clamped = hs.clamped;
      R.st.mass_drift = hs.mass_drift;
      R.st.total_iterations = hs.cum_iters;
      R.st.total_refinements = hs.cum_refines;
      R.t_submit = S.t_submit;
      R.t_done = t1;
      I.enabled = 0;
      give(S.begin, S.len);
      info.arena_cells_used -= (double)S.len;
      S.used = false;
      info.resident--;
      info.completed++;
      dirty = true;
    }
    if (ncomp) *ncomp = (int)fin.size();
    return SAYRAM_OK;
  }

  // sizes the lane's arrays from its share of the budget (tables, staging, lists, cell arena)
  int create(const sayram_server_config& c, const sayram_options* opt) {
    cfg = c;
    sayram_batch_s& e = eng;
    // the lane's step graph outlives changes of its instance list; the cooperative solve's grid
    // is sized to the list it was built for
    e.coop = 0;
    int rc = e.set_options(opt);
    if (!rc) rc = e.init_device();
    if (rc) return rc;
    SG_CUDA(cudaEventCreateWithFlags(&done_ev, cudaEventDisableTiming));
    const long long ms = c.max_side + 1;
    const double table_bytes = (double)c.max_slots * ms * (1 + 1 + 2 + 2 + 4) * 8.0;
    const double stage_bytes = 6.0 * (double)c.max_side * c.max_side * 8.0;
    const double per_cell = (double)sayram_instance_bytes(64, 64, e.opt.precision) /
                            (double)region_cells(64, 64);  // bytes per arena cell (all arrays)
    const double avail = c.hbm_budget_bytes - table_bytes - stage_bytes - 64.0 * 1048576.0;
    const long long cells = (long long)(avail / (per_cell + 4.0 / 1024 * 2 + 8.0 * 4 / 1024));
    if (cells < region_cells(1, 1) + 64) return fail(SAYRAM_ERR_BUDGET, "HBM budget too small for any instance");
    const long long side_tiles = (long long)c.max_slots * (c.max_side / sg::kTX + c.max_side / sg::kTY + 2);
    const int chunks_cap = (int)std::min<long long>(cells / 1024 + c.max_slots + 1, 1LL << 30);
    const int tiles_cap = (int)std::min<long long>(cells / (sg::kTX * sg::kTY) + side_tiles, 1LL << 30);
    rc = e.alloc_storage(cells + 64, c.max_slots, chunks_cap, tiles_cap, (long long)c.max_slots * ms,
                         (long long)c.max_slots * ms, 4LL * c.max_slots * ms,
                         std::max<long long>(6LL * c.max_side * c.max_side, 1));
    if (rc) return rc;
    e.n = c.max_slots;
    e.pmax = (int)round_up(c.max_side, 4);
    if ((rc = e.rebuild_lists())) return rc;
    arena = cells;
    free_[0] = cells;
    slots.resize(c.max_slots);
    info.arena_cells = (double)cells;
    info.device_bytes = (double)e.bytes;
    return SAYRAM_OK;
  }

  // SAYRAM_OK if a request of this grid can ever run in the lane
  int accepts(int nx, int ny) const {
    if (nx > cfg.max_side || ny > cfg.max_side) return fail(SAYRAM_ERR_BUDGET, "grid side exceeds the server's max_side");
    if (region_cells(nx, ny) > arena) return fail(SAYRAM_ERR_BUDGET, "request larger than the HBM budget");
    return SAYRAM_OK;
  }
};

// The server: one lane, or two -- instances with max(nx, ny) <= split in the first (its own
// share of the budget and of the tables), the rest in the second.
struct sayram_server_s {
  std::vector<std::unique_ptr<ServerLane>> lanes;
  int split = 0;
  double wait_seconds = 600.0;  // longest host wait of one tick for a lane's step
  std::map<long long, Result> results;
  long long next_id = 1;

  ServerLane* lane_for(int nx, int ny) {
    if (lanes.size() > 1 && std::max(nx, ny) <= split && lanes[0]->accepts(nx, ny) == SAYRAM_OK)
      return lanes[0].get();
    return lanes.back().get();
  }

  int tick(int* ncomp) {
    if (ncomp) *ncomp = 0;
    int rc;
    for (auto& L : lanes)
      if (!L->inflight && (rc = L->launch())) return rc;
    bool any = false;
    for (auto& L : lanes) any = any || L->inflight;
    if (!any) return SAYRAM_OK;
    // wait for the first lane whose step finishes, then collect every finished lane (a step
    // takes milliseconds; one that has not finished after wait_seconds is reported, and a later
    // tick waits for it again)
    const double t_wait = now_seconds();
    int total = 0;
    for (;;) {
      bool done = false;
      for (auto& L : lanes) {
        if (!L->inflight) continue;
        const int r = L->ready();
        if (r < 0) return SAYRAM_ERR_CUDA;
        if (r == 0) continue;
        int n = 0;
        if ((rc = L->finish(results, &n))) return rc;
        total += n;
        done = true;
      }
      if (done) break;
      if (now_seconds() - t_wait > wait_seconds)
        return fail(SAYRAM_ERR_TIMEOUT, "server step still running after " + std::to_string(wait_seconds) +
                                            " s (the next tick waits for it again)");
      std::this_thread::yield();
    }
    if (ncomp) *ncomp = total;
    return SAYRAM_OK;
  }
};

extern "C" {

int sayram_server_create(const sayram_server_config* cfg, const sayram_options* opt, sayram_server* out) {
  if (!out || !cfg) return fail(SAYRAM_ERR_ARG, "null config or output handle");
  *out = nullptr;
  sayram_server_config c = *cfg;
  if (c.max_slots <= 0) c.max_slots = 4096;
  if (c.max_side <= 0) c.max_side = 1024;
  if (!(c.hbm_budget_bytes > 0)) return fail(SAYRAM_ERR_ARG, "HBM budget must be positive");
  const int nl = c.lanes >= 2 ? 2 : 1;
  const int split = c.lane_split_side > 0 ? c.lane_split_side : 128;
  const double frac = c.lane_small_fraction > 0 && c.lane_small_fraction < 1 ? c.lane_small_fraction : 0.25;
  if (nl == 2 && split >= c.max_side) return fail(SAYRAM_ERR_ARG, "lane_split_side must be below max_side");
  std::unique_ptr<sayram_server_s> s(new (std::nothrow) sayram_server_s());
  if (!s) return fail(SAYRAM_ERR_OOM, "host allocation failed");
  s->split = split;
  s->wait_seconds = c.wait_seconds > 0 ? c.wait_seconds : 600.0;
  for (int k = 0; k < nl; ++k) {
    sayram_server_config lc = c;
    if (nl == 2) {
      lc.hbm_budget_bytes = c.hbm_budget_bytes * (k == 0 ? frac : 1.0 - frac);
      if (k == 0) lc.max_side = split;
    }
    std::unique_ptr<ServerLane> L(new (std::nothrow) ServerLane());
    if (!L) return fail(SAYRAM_ERR_OOM, "host allocation failed");
    int rc = L->create(lc, opt);
    if (rc) {
      std::string m = g_err;
      L.reset();
      s.reset();
      return fail(rc, m);
    }
    s->lanes.push_back(std::move(L));
  }
  *out = s.release();
  g_err.clear();
  return SAYRAM_OK;
}

int sayram_server_submit(sayram_server s, const sayram_problem* p, int nsteps, long long* id_out) {
  if (!s || !p || nsteps < 1) return fail(SAYRAM_ERR_ARG, "bad server, problem or step count");
  int rc = validate_problem(*p);
  if (rc) return rc;
  ServerLane* L = s->lane_for(p->nx, p->ny);
  if ((rc = L->accepts(p->nx, p->ny))) return rc;
  Request* r = new (std::nothrow) Request();
  if (!r) return fail(SAYRAM_ERR_OOM, "host allocation failed");
  r->own(*p);
  r->nsteps = nsteps;
  r->id = s->next_id++;
  r->t_submit = now_seconds();
  L->waiting.push_back(r);
  L->info.submitted++;
  L->info.waiting++;
  if (id_out) *id_out = r->id;
  return SAYRAM_OK;
}

int sayram_server_tick(sayram_server s, int* n_completed) {
  if (!s) return fail(SAYRAM_ERR_ARG, "null server");
  return s->tick(n_completed);
}

int sayram_server_poll(sayram_server s, long long id, double* f_out, sayram_stats* st, double* t_submit,
                       double* t_done) {
  if (!s) return fail(SAYRAM_ERR_ARG, "null server");
  auto it = s->results.find(id);
  if (it == s->results.end()) return fail(SAYRAM_ERR_STATE, "request not completed");
  if (f_out) std::memcpy(f_out, it->second.f.data(), sizeof(double) * it->second.f.size());
  if (st) *st = it->second.st;
  if (t_submit) *t_submit = it->second.t_submit;
  if (t_done) *t_done = it->second.t_done;
  s->results.erase(it);
  return SAYRAM_OK;
}

int sayram_server_info_get(sayram_server s, sayram_server_info* out) {
  if (!s || !out) return fail(SAYRAM_ERR_ARG, "null server or output");
  sayram_server_info t{};
  for (auto& L : s->lanes) {  // sums over the lanes (their step times overlap)
    const sayram_server_info& i = L->info;
    t.submitted += i.submitted;
    t.admitted += i.admitted;
    t.completed += i.completed;
    t.waiting += i.waiting;
    t.resident += i.resident;
    t.ticks += i.ticks;
    t.instance_steps += i.instance_steps;
    t.device_bytes += (double)L->eng.bytes;
    t.arena_cells += i.arena_cells;
    t.arena_cells_used += i.arena_cells_used;
    t.busy_seconds += i.busy_seconds;
    t.admit_seconds += i.admit_seconds;
    t.lists_seconds += i.lists_seconds;
    t.step_seconds += i.step_seconds;
    t.collect_seconds += i.collect_seconds;
  }
  *out = t;
  return SAYRAM_OK;
}

int sayram_server_completed_ids(sayram_server s, long long* ids, int cap) {
  if (!s || (!ids && cap > 0)) return 0;
  int n = 0;
  for (auto& kv : s->results) {
    if (n >= cap) break;
    ids[n++] = kv.first;
  }
  return n;
}

void sayram_server_destroy(sayram_server s) { delete s; }

}  // extern "C"

// ================================================================================== no allocation
// sayram_step_noalloc: the FP64 single-instance step for callers that cannot allocate device
// memory (see the header). Its working arrays live in one file-scope device array that the CUDA
// runtime creates when the module loads; this path calls no cudaMalloc / cudaFree /
// cudaMallocHost and no allocating library routine.
namespace {

constexpr long long kNoAllocCells = 73728;  // padded cells: round_up((ny+2)*round_up(nx,4), 32) + 64
constexpr int kNoAllocMaxSide = 4096;       // nx, ny limit (host tables are on the stack)
constexpr int kNoAllocChunk = 1024;  // cells per chunk of the streaming kernels on this path
constexpr int kNoAllocMaxChunks = (int)(kNoAllocCells / kNoAllocChunk) + 2;
constexpr int kNoAllocMaxTiles = 8192;
constexpr size_t kNoAllocTableBytes = 1u << 20;
constexpr size_t kNoAllocBytes = kNoAllocTableBytes + (size_t)kNoAllocCells * 27 * sizeof(double);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
unsigned char* g_noalloc_base[128] = {};  // device address of g_noalloc_scratch, per device

// Per-cell set-up from separate coefficient arrays (alpha-major) in the caller's device memory:
// sg::setup_cell, the same per-cell definition k_setup uses (k_setup reads one packed staging
// buffer instead).
__global__ void k_setup_fields(sg::Common cm, sg::Geo geo, const double* G, const double* Dxx,
                               const double* Dxy, const double* Dyy, const double* itau,
                               const double* xe, const double* ye) {
  const sg::InstDev I = cm.inst[0];
  const long long ncell = (long long)I.nx * I.ny;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c / I.ny), j = (int)(c % I.ny);
    const long long K = I.base + (long long)j * I.pitch + i;
    sg::setup_cell<sg::F64A>(geo, K, xe[i], xe[i + 1], ye[j], ye[j + 1], I.dt, G[c], Dxx[c], Dxy[c], Dyy[c], itau[c]);
  }
}

// Carves the scratch array into the typed regions of one instance.
struct NoAllocLayout {
  unsigned char* cur;
  unsigned char* end;
  template <typename T>
  T* take(long long count) {
    const size_t nb = ((size_t)count * sizeof(T) + 255) & ~(size_t)255;
    if (cur + nb > end) return nullptr;
    T* p = reinterpret_cast<T*>(cur);
    cur += nb;
    return p;
  }
};

int noalloc_device_base(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (dev < 0 || dev >= 128) return fail(SAYRAM_ERR_ARG, "device ordinal out of range");
  if (!g_noalloc_base[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(SAYRAM_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_noalloc_base[dev] = (unsigned char*)ptr;
  }
  *out = g_noalloc_base[dev];
  return SAYRAM_OK;
}

}  // namespace

extern "C" int sayram_step_noalloc(const sayram_problem* pd, const sayram_options* opt, int nsteps,
                                   const double* f_in, double* f_out, void* stream_ptr,
                                   sayram_stats* stats_out) {
  using namespace sg;
  if (!pd || !f_in || !f_out || nsteps < 0) return fail(SAYRAM_ERR_ARG, "null problem/buffer or negative nsteps");
  const int nx = pd->nx, ny = pd->ny;
  if (nx < 1 || ny < 1) return fail(SAYRAM_ERR_ARG, "Grid2D: x_edges/y_edges must have size >= 2.");
  const long long pitch = round_up(nx, 4);
  const long long padded = round_up((long long)(ny + 2) * pitch, 32) + 64;
  if (nx > kNoAllocMaxSide || ny > kNoAllocMaxSide || padded > kNoAllocCells)
    return fail(SAYRAM_ERR_ARG, "sayram_step_noalloc: grid " + std::to_string(nx) + "x" + std::to_string(ny) +
                                    " exceeds the fixed scratch (needs round_up((ny+2)*round_up(nx,4),32)+64 <= " +
                                    std::to_string(kNoAllocCells) + " cells and nx, ny <= " +
                                    std::to_string(kNoAllocMaxSide) + "; 256x256 fits)");
  if (!pd->x_edges || !pd->y_edges || !pd->G || !pd->Dxx || !pd->Dxy || !pd->Dyy || !pd->inv_tau)
    return fail(SAYRAM_ERR_ARG, "missing device array in the problem");
  if (!(pd->dt > 0) || !std::isfinite(pd->dt)) return fail(SAYRAM_ERR_ARG, "dt must be positive");
  for (int s = 0; s < 4; ++s) {
    if (pd->bc[s] != SAYRAM_DIRICHLET && pd->bc[s] != SAYRAM_ZEROFLUX) return fail(SAYRAM_ERR_ARG, "unknown boundary type");
    if (pd->bc[s] == SAYRAM_DIRICHLET && !pd->dirichlet[s]) return fail(SAYRAM_ERR_ARG, "Dirichlet BC: missing value.");
  }
  sayram_options o;
  sayram_default_options(&o);
  if (opt) o = *opt;
  if (o.precision != SAYRAM_FP64) return fail(SAYRAM_ERR_ARG, "sayram_step_noalloc runs the FP64 path only");
  if (!(o.tol > 0)) o.tol = 1e-12;
  if (o.inner_tol < 0) o.inner_tol = 0.0;
  if (o.max_iters < 1) o.max_iters = 1;
  if (o.max_refine < 2) o.max_refine = 2;
  int dev = 0;
  SG_CUDA(cudaGetDevice(&dev));
  unsigned char* base = nullptr;
  int rc = noalloc_device_base(dev, &base);
  if (rc) return rc;
  cudaStream_t stream = (cudaStream_t)stream_ptr;
  int nsm = 0;
  SG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));

  // ---- host tables (stack), the same layout rules as sayram_batch_create for one instance
  InstDev I;
  std::memset(&I, 0, sizeof(I));
  I.nx = nx;
  I.ny = ny;
  I.pitch = (int)pitch;
  I.enabled = 1;
  for (int s = 0; s < 4; ++s) I.bc[s] = pd->bc[s];
  I.base = pitch;
  I.hoff = 0;
  I.chunk0 = 0;
  I.nchunks = (int)((round_up((long long)ny * pitch, 4) + kNoAllocChunk - 1) / kNoAllocChunk);
  I.tile0 = 0;
  I.ntx = (nx + kTX - 1) / kTX;
  I.nty = (ny + kTY - 1) / kTY;
  if (I.nchunks > kNoAllocMaxChunks || I.ntx * I.nty > kNoAllocMaxTiles)
    return fail(SAYRAM_ERR_ARG, "sayram_step_noalloc: grid exceeds the fixed work tables");
  I.xe = 0;
  I.ye = 0;
  int doff = 0;
  for (int s = 0; s < 4; ++s) {
    I.dir[s] = pd->bc[s] == SAYRAM_DIRICHLET ? doff : -1;
    if (pd->bc[s] == SAYRAM_DIRICHLET) doff += (s <= 1) ? ny + 1 : nx + 1;
  }
  I.dt = pd->dt;
  static thread_local double hxe[kNoAllocMaxSide + 1], hye[kNoAllocMaxSide + 1];
  static thread_local double hwx[2 * (kNoAllocMaxSide + 1)], hwy[2 * (kNoAllocMaxSide + 1)];
  static thread_local int hchunk[kNoAllocMaxChunks], htile[kNoAllocMaxTiles];

  // ---- carve the scratch array
  NoAllocLayout lay{base, base + kNoAllocBytes};
  InstDev* d_inst = lay.take<InstDev>(1);
  InstState* d_st = lay.take<InstState>(1);
  Ctl* d_ctl = lay.take<Ctl>(1);
  int* d_chunk = lay.take<int>(kNoAllocMaxChunks);
  int* d_tile = lay.take<int>(kNoAllocMaxTiles);
  double* d_wx = lay.take<double>(2 * (nx + 1));
  double* d_wy = lay.take<double>(2 * (ny + 1));
  double* d_dirv = lay.take<double>(doff > 0 ? doff : 1);
  double* d_part = lay.take<double>(4LL * kNoAllocMaxChunks);
  unsigned char* tables_end = lay.cur;
  if (!d_part || tables_end > base + kNoAllocTableBytes) return fail(SAYRAM_ERR_ARG, "tables exceed the scratch");
  lay.cur = base + kNoAllocTableBytes;
  Geo geo{};
  Fields fl{};
  Coef<double> co{};
  Kry<double> kr{};
  double** cellarrs[27] = {&geo.aAx, &geo.aBx, &geo.Sx, &geo.aAy, &geo.aBy, &geo.Sy, &geo.ukk, &geo.sdiag,
                           &fl.f, &fl.fh[0], &fl.invD, &fl.R, &fl.colsum, &fl.y64[0], &fl.y64[1],
                           &co.cw, &co.ce, &co.cs, &co.cn,
                           &kr.r, &kr.rh, &kr.t, &kr.x, &kr.p[0], &kr.p[1], &kr.v[0], &kr.v[1]};
  for (auto a : cellarrs) {
    *a = lay.take<double>(kNoAllocCells);
    if (!*a) return fail(SAYRAM_ERR_ARG, "cell arrays exceed the scratch");
  }
  fl.fh[1] = fl.fh[2] = fl.fh[0];  // one history buffer: linear extrapolation (hist_cap = 1);
                                    // geo.decay / fl.decay stay null (no loss compensation here)
  unsigned char* used_end = lay.cur;

  // ---- every call starts from zero: padding, pad rows, state and counters must be 0
  SG_CUDA(cudaMemsetAsync(base, 0, (size_t)(used_end - base), stream));
  SG_CUDA(cudaMemcpyAsync(hxe, pd->x_edges, sizeof(double) * (nx + 1), cudaMemcpyDeviceToHost, stream));
  SG_CUDA(cudaMemcpyAsync(hye, pd->y_edges, sizeof(double) * (ny + 1), cudaMemcpyDeviceToHost, stream));
  SG_CUDA(cudaStreamSynchronize(stream));
  for (int i = 0; i < nx; ++i)
    if (!(hxe[i + 1] > hxe[i])) return fail(SAYRAM_ERR_ARG, "Grid2D: x_edges must be strictly increasing at i=" + std::to_string(i));
  for (int j = 0; j < ny; ++j)
    if (!(hye[j + 1] > hye[j])) return fail(SAYRAM_ERR_ARG, "Grid2D: y_edges must be strictly increasing at j=" + std::to_string(j));
  for (int k = 0; k < 2 * (kNoAllocMaxSide + 1) && k < 2 * (nx + 1); ++k) hwx[k] = 0.0;
  for (int k = 0; k < 2 * (kNoAllocMaxSide + 1) && k < 2 * (ny + 1); ++k) hwy[k] = 0.0;
  for (int i = 1; i < nx; ++i) {  // bilinear weights of Solver.cc:333-336
    const double xv = hxe[i], xl = 0.5 * (hxe[i - 1] + hxe[i]), xr = 0.5 * (hxe[i] + hxe[i + 1]);
    hwx[2 * i] = (xr - xv) / (xr - xl);
    hwx[2 * i + 1] = (xv - xl) / (xr - xl);
  }
  for (int j = 1; j < ny; ++j) {
    const double yv = hye[j], yb = 0.5 * (hye[j - 1] + hye[j]), yt = 0.5 * (hye[j] + hye[j + 1]);
    hwy[2 * j] = (yt - yv) / (yt - yb);
    hwy[2 * j + 1] = (yv - yb) / (yt - yb);
  }
  for (int k = 0; k < I.nchunks; ++k) hchunk[k] = 0;
  for (int k = 0; k < I.ntx * I.nty; ++k) htile[k] = 0;
  SG_CUDA(cudaMemcpyAsync(d_inst, &I, sizeof(I), cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaMemcpyAsync(d_chunk, hchunk, sizeof(int) * I.nchunks, cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaMemcpyAsync(d_tile, htile, sizeof(int) * I.ntx * I.nty, cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaMemcpyAsync(d_wx, hwx, sizeof(double) * 2 * (nx + 1), cudaMemcpyHostToDevice, stream));
  SG_CUDA(cudaMemcpyAsync(d_wy, hwy, sizeof(double) * 2 * (ny + 1), cudaMemcpyHostToDevice, stream));
  for (int s = 0; s < 4; ++s)
    if (I.dir[s] >= 0)
      SG_CUDA(cudaMemcpyAsync(d_dirv + I.dir[s], pd->dirichlet[s], sizeof(double) * ((s <= 1) ? ny + 1 : nx + 1),
                              cudaMemcpyDeviceToDevice, stream));
  Common cm{};
  cm.inst = d_inst;
  cm.st = d_st;
  cm.ctl = d_ctl;
  cm.hist_cap = 1;
  cm.chunk_inst = d_chunk;
  cm.nchunks = I.nchunks;
  cm.tile_inst = d_tile;
  cm.ntiles = I.ntx * I.nty;
  cm.ninst = 1;
  cm.wx = d_wx;
  cm.wy = d_wy;
  cm.dirv = d_dirv;
  cm.part = d_part;
  // the caller's edges are read directly by the setup kernel
  const long long ncell = (long long)nx * ny;
  const int sblocks = (int)std::min<long long>((ncell + 255) / 256, (long long)nsm * 8);
  k_setup_fields<<<sblocks, 256, 0, stream>>>(cm, geo, pd->G, pd->Dxx, pd->Dxy, pd->Dyy, pd->inv_tau,
                                             pd->x_edges, pd->y_edges);
  SG_CUDA(cudaGetLastError());
  const int gt = std::max(1, std::min(cm.ntiles, nsm * kAsmGridPerSm));
  const int gs = std::max(1, std::min(cm.nchunks, nsm * 16));
  k_field_in<F64A><<<gt, kFieldThreads, 0, stream>>>(cm, fl.f, f_in, 0, 0, -1);
  const size_t smem_na = (size_t)(kNoAllocChunk + 2 * pitch) * sizeof(double);
  SG_CUDA(cudaFuncSetAttribute(k_bicg1<double, kNoAllocChunk>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_na));
  SG_CUDA(cudaFuncSetAttribute(k_bicg2<double, kNoAllocChunk>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_na));
  SG_CUDA(cudaFuncSetAttribute(k_resid<double, double, F64A, kNoAllocChunk>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_na));
  SG_CUDA(cudaFuncSetAttribute(k_polish<double, F64A, kNoAllocChunk>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_na));
  SG_CUDA(cudaGetLastError());
  Ctl hctl;
  for (int s = 0; s < nsteps; ++s) {
    SG_CUDA(cudaMemsetAsync(d_ctl, 0, 2 * sizeof(int), stream));
    k_begin<<<1, 32, 0, stream>>>(cm);
    k_assemble<double, F64A><<<gt, kAsmThreads, 0, stream>>>(cm, geo, fl, co, 0, -1);
    for (int r = 0; r < o.max_refine; ++r) {
      k_resid<double, double, F64A, kNoAllocChunk><<<gs, kThreads, smem_na, stream>>>(cm, fl, co, kr, o.tol, o.inner_tol, o.max_refine);
      SG_CUDA(cudaGetLastError());
      if (r == o.max_refine - 1) break;
      SG_CUDA(cudaMemcpyAsync(&hctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream));
      SG_CUDA(cudaStreamSynchronize(stream));
      if (hctl.n_outer == 0) break;
      for (int it = 0; it < o.max_iters; ++it) {
        k_bicg1<double, kNoAllocChunk><<<gs, kThreads, smem_na, stream>>>(cm, co, kr);
        k_bicg2<double, kNoAllocChunk><<<gs, kThreads, smem_na, stream>>>(cm, co, kr);
        k_bicg3<double, kNoAllocChunk><<<gs, kThreads, 0, stream>>>(cm, kr, o.max_iters);
        SG_CUDA(cudaGetLastError());
        if (it < 4 || (it & 3) == 3) {
          SG_CUDA(cudaMemcpyAsync(&hctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream));
          SG_CUDA(cudaStreamSynchronize(stream));
          if (hctl.n_inner == 0) break;
        }
      }
    }
    k_polish<double, F64A, kNoAllocChunk><<<gs, kThreads, smem_na, stream>>>(cm, fl, co, 0, -1);
    SG_CUDA(cudaGetLastError());
  }
  k_field_out<F64A><<<gt, 256, 0, stream>>>(cm, f_out, fl.f, 0, -1);
  SG_CUDA(cudaGetLastError());
  InstState hs;
  SG_CUDA(cudaMemcpyAsync(&hs, d_st, sizeof(hs), cudaMemcpyDeviceToHost, stream));
  SG_CUDA(cudaStreamSynchronize(stream));
  if (stats_out) {
    stats_out->steps = hs.steps;
    stats_out->t = (double)hs.steps * pd->dt;
    stats_out->status = hs.steps == 0 ? SAYRAM_OK
                        : hs.status == ST_NEGATIVE ? SAYRAM_ERR_NEGATIVE
                        : hs.status == ST_NOT_CONVERGED ? SAYRAM_ERR_NOT_CONVERGED : SAYRAM_OK;
    stats_out->refinements = hs.refines;
    stats_out->iterations = hs.iters_total;
    stats_out->rel_residual = hs.rel;
    stats_out->min_f = hs.min_f;
    stats_out->clamped = hs.clamped;
    stats_out->mass_drift = hs.mass_drift;
    stats_out->total_iterations = hs.cum_iters;
    stats_out->total_refinements = hs.cum_refines;
  }
  if (hs.steps > 0 && hs.status == ST_NEGATIVE) return fail(SAYRAM_ERR_NEGATIVE, "a negative cell survived the positivity polish");
  if (hs.steps > 0 && hs.status == ST_NOT_CONVERGED) return fail(SAYRAM_ERR_NOT_CONVERGED, "a step ended above the residual target");
  return SAYRAM_OK;
}
