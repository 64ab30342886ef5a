// fvs_batch.cu — many independent cases in one launch.
//
// The cases' meshes are packed as a disjoint union (each case's cells and
// edge slots contiguous, fvs_layout.hpp), so the per-item device code of the
// single-mesh path serves unchanged; what is per case is the free stream
// (boundary records carry the case index), the residual norm (cell tiles
// never straddle cases) and convergence (converged cases are dropped from
// the tile lists).  Launch forms:
//  - one cooperative launch of k_persistent advances all active cases by a
//    chunk of RK steps, with bounded grid barriers between the phases,
//    captured once in a CUDA graph and replayed;
//  - a CUDA graph of one step's tile launches (one block per tile and
//    phase), replayed once per step;
//  - for first-order mixed batches, either form with the fused stage (each
//    cell evaluates its own faces' fluxes: one phase per stage).
// The launch shape (form, block size, tile length, resident blocks per SM)
// comes from an autotuner that times the candidates on the batch itself,
// and the run-to-target calls try shapes again as the active set shrinks.
//
// The reference runs one case per process (src/fvs2d.f90); the batch has no
// counterpart there beyond running time_integration on each case.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "df64.cuh"
#include "fvs_internal.hpp"
#include "fvs_layout.hpp"

using namespace fvs;

namespace {

thread_local std::string g_batch_create_error;

__global__ void kb_scatter_in(const double* __restrict__ ref, const int* __restrict__ perm, double* __restrict__ dev, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2* s = reinterpret_cast<const double2*>(ref) + 2 * (size_t)i;
  double2* t = reinterpret_cast<double2*>(dev) + 2 * (size_t)perm[i];
  t[0] = s[0];
  t[1] = s[1];
}

__global__ void kb_gather_out(const double* __restrict__ dev, const int* __restrict__ perm, double* __restrict__ ref, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2* s = reinterpret_cast<const double2*>(dev) + 2 * (size_t)perm[i];
  double2* t = reinterpret_cast<double2*>(ref) + 2 * (size_t)i;
  t[0] = s[0];
  t[1] = s[1];
}

bool same_scheme(const fvs_options& a, const fvs_options& b) {
  return a.gamma == b.gamma && a.dt == b.dt && a.cfl == b.cfl && a.steady == b.steady && a.vortex == b.vortex &&
         a.ntstart == b.ntstart && a.grad_method == b.grad_method && a.lsq_stencil == b.lsq_stencil &&
         a.lsq_pow == b.lsq_pow && a.limiter == b.limiter && a.reconst == b.reconst && a.umuscl == b.umuscl &&
         a.flux == b.flux && a.rk_nstages == b.rk_nstages && a.rk_order == b.rk_order && a.ssprk == b.ssprk &&
         a.precision == b.precision;
}

}  // namespace

struct fvs_batch {
  int ncases = 0;
  std::vector<HostMesh> hm;
  std::vector<fvs_options> opt;
  fvs_options base;
  std::string err;
  const KernelSet* ks = nullptr;
  bool mixed = false;
  int prec = FVS_PREC_FP64;
  cudaStream_t stream = nullptr;
  DeviceArena arena;
  DevView d;  // the current precision's view
  // views of the other precisions, built on first use (the precision ladder)
  struct Variant {
    bool built = false;
    DevView d;
    int block = 256, tile = 1024, bps = 1;
    bool tiled = false;
  } var[4];
  int nc = 0, ne = 0;
  std::vector<int> coff, eoff, cnum, enumv;  // per-case cell / edge-slot ranges
  std::vector<double> pinf;                 // [ncases][4]
  int* d_perm = nullptr;                    // concatenated reference -> device cell maps
  std::vector<int> ref_off;                 // offset of each case in d_perm
  double* d_stage = nullptr;
  double* d_backup = nullptr;               // state saved around the autotuner
  std::vector<StageParams> stages;
  // launch shape and plan
  int block = 256, tile = 1024, bps = 1, nsm = 0;
  int4* d_cell_tiles = nullptr;
  int2* d_edge_tiles = nullptr;
  int4* d_case_tiles = nullptr;
  double* d_tile_partials = nullptr;
  double* d_case_norms = nullptr;
  int* d_step0 = nullptr;
  int* d_case_count = nullptr;  // per active case: tiles of the last stage finished (graph form)
  GridBarrier* d_bar = nullptr;
  int cap_cell_tiles = 0, cap_edge_tiles = 0;
  int norm_cap = 1024;
  double budget_s = 4.0;
  PersistPlan plan;
  std::vector<char> active;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = -1;
  bool plan_dirty = true, use_graph = true;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t eva = nullptr, evb = nullptr;  // around one chunk's launches (shape trials)
  bool retune = true;                         // shape trials as the active set shrinks
  int* h_step0 = nullptr;
  DcView dc;  // defect-correction arrays, allocated on first use
  // launch mode: false = one cooperative persistent launch per chunk, true =
  // a CUDA graph of one step's tile launches, replayed once per step
  bool tiled = false;
  cudaGraphExec_t tgraph = nullptr;     // one step, current plan and precision
  cudaGraphExec_t tgraph_dc = nullptr;  // one defect-correction step
  // fused first-order stages (flux per cell, one phase per stage) where they
  // apply, in the mixed phase (fuse) and in defect correction (fuse_dc);
  // second buffers of the primitives and of the correction tangents
  bool fuse = true, fuse_dc = false;
  void* pv2_mem = nullptr;
  void* dp2_mem = nullptr;
  std::vector<int> group;  // cases of one group stop together (first to converge)

  ~fvs_batch() {
    if (graph) cudaGraphExecDestroy(graph);
    if (tgraph) cudaGraphExecDestroy(tgraph);
    if (tgraph_dc) cudaGraphExecDestroy(tgraph_dc);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (eva) cudaEventDestroy(eva);
    if (evb) cudaEventDestroy(evb);
    if (h_step0) cudaFreeHost(h_step0);
    arena.release();
    if (stream) cudaStreamDestroy(stream);
  }
  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* where) {
    err = std::string(where) + ": " + cudaGetErrorString(e);
    return FVS_ERR_CUDA;
  }
};

namespace {

template <typename T>
int build_batch_device(fvs_batch* B, DevView& d) {
  Layout<T> L;
  std::string err;
  const bool fold_w = d.grad_method == FVS_GRAD_LSQ && B->prec != FVS_PREC_FP64_STRICT;
  const bool first = B->coff.empty();
  for (int c = 0; c < B->ncases; c++) {
    int rc = append_case(L, B->hm[c], fold_w, c, err);
    if (rc) return B->fail(rc, "case " + std::to_string(c) + ": " + err);
    if (first) {
      B->coff.push_back(L.case_coff[c]);
      B->eoff.push_back(L.case_eoff[c]);
      B->cnum.push_back(B->hm[c].nc);
      B->enumv.push_back((int)(B->hm[c].edge_intr.size() + B->hm[c].b_edge.size()));
    }
  }
  B->nc = L.nc;
  B->ne = L.ne;
  B->ref_off = B->coff;  // L.perm is appended case by case in the same order
  if (!upload_layout(B->arena, L, d)) return B->fail(FVS_ERR_NOMEM, "device allocation or upload of the batch meshes failed");
  if (first && !B->arena.upload(B->d_perm, L.perm)) return B->fail(FVS_ERR_NOMEM, "upload of the cell maps failed");
  double* dp = nullptr;
  if (!B->arena.upload(dp, B->pinf)) return B->fail(FVS_ERR_NOMEM, "upload of the free streams failed");
  d.case_pinf = dp;
  if (!alloc_work<T>(B->arena, d, L.nc, L.ne, (L.nc + 255) / 256, 16))
    return B->fail(FVS_ERR_NOMEM, "device allocation of the batch state failed");
  std::vector<T> phi0(L.nc, T(d.first_order ? 0.0 : 1.0));
  if (cudaMemcpy(d.phi, phi0.data(), sizeof(T) * L.nc, cudaMemcpyHostToDevice) != cudaSuccess)
    return B->fail(FVS_ERR_CUDA, "phi upload failed");
  std::vector<double> dtl(L.nc, B->base.dt);
  if (cudaMemcpy(d.dtl, dtl.data(), 8 * dtl.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return B->fail(FVS_ERR_CUDA, "dt upload failed");
  return FVS_OK;
}

int build_for(fvs_batch* B, int prec, DevView& d) {
  if (prec == FVS_PREC_MIXED) return build_batch_device<float>(B, d);
  if (prec == FVS_PREC_FP64_DF) return build_batch_device<df64>(B, d);
  return build_batch_device<double>(B, d);
}

int alloc_batch_buffers(fvs_batch* B) {
  void* p;
  bool ok = B->arena.alloc(p, 32 * (size_t)B->nc);
  B->d_stage = static_cast<double*>(p);
  ok = ok && B->arena.alloc(p, 32 * (size_t)B->nc);
  B->d_backup = static_cast<double*>(p);
  ok = ok && B->arena.alloc(p, 32 * (size_t)B->ncases * B->norm_cap);
  B->d_case_norms = static_cast<double*>(p);
  ok = ok && B->arena.alloc(p, sizeof(GridBarrier));
  B->d_bar = static_cast<GridBarrier*>(p);
  ok = ok && B->arena.alloc(p, 16);
  B->d_step0 = static_cast<int*>(p);
  ok = ok && B->arena.alloc(p, 16 * (size_t)B->ncases);
  B->d_case_tiles = static_cast<int4*>(p);
  ok = ok && B->arena.alloc(p, 16 * (size_t)B->ncases);
  B->d_case_count = static_cast<int*>(p);
  return ok ? FVS_OK : B->fail(FVS_ERR_NOMEM, "device allocation of the batch buffers failed");
}

void init_view_constants(fvs_batch* B, DevView& d) {
  const fvs_options& ob = B->base;
  d.gamma = ob.gamma; d.gm1 = ob.gamma - 1.0; d.igm1 = 1.0 / (ob.gamma - 1.0);
  d.ggm1 = ob.gamma / (ob.gamma - 1.0);
  d.khalf = ob.umuscl / 2.0; d.nkhalf = -ob.umuscl / 2.0; d.omk = 1.0 - ob.umuscl; d.cfl = ob.cfl;
  set_fp32_constants(d);
  d.limiter = ob.limiter; d.grad_method = ob.grad_method; d.first_order = ob.reconst == FVS_RECON_UPWIND1;
  d.vortex = ob.vortex; d.vx = ob.vortex_x; d.vy = ob.vortex_y; d.vkappa = ob.vortex_kappa;
  for (int k = 0; k < 4; k++) { d.vinf[k] = ob.vortex_inf[k]; d.pinf[k] = B->pinf[k]; }
  mms_constants(d.mc);
  d.dt = ob.dt;
}

const KernelSet* kernels_for(int prec) {
  return prec == FVS_PREC_MIXED         ? &kernels_mixed()
         : prec == FVS_PREC_FP64_STRICT ? &kernels_fp64_strict()
         : prec == FVS_PREC_FP64_DF     ? &kernels_fp64_df()
                                        : &kernels_fp64_fast();
}

void set_batch_stages(fvs_batch* B) {
  const fvs_options& o = B->base;
  double hr[5], c[5], dts[5];
  rk_coefficients(o, o.dt, hr, c, dts);
  B->stages.clear();
  const int ns = o.rk_nstages;
  for (int k = 1; k <= ns; k++) {
    StageParams sp;
    sp.stage = k; sp.nstages = ns; sp.steady = o.steady; sp.last = (k == ns);
    sp.mode = (ns == 3 && o.ssprk) ? MODE_SSP3 : (o.ssprk ? MODE_SSP42 : MODE_RK);
    sp.h = hr[k]; sp.coef = c[k]; sp.dts = dts[k];
    if (sp.mode == MODE_SSP42) sp.cst = (k == 4) ? 1.0 / 4.0 : 1.0 / 3.0;
    else if (sp.mode == MODE_RK) sp.cst = (k == 3) ? 1.0 : (k == 4 ? 1.0 / 6.0 : 1.0 / 2.0);
    else sp.cst = 1.0;
    if (sp.mode == MODE_SSP3) {
      static const double A[4] = {0, 0.0, 0.75, 1.0 / 3.0}, Bw[4] = {0, 1.0, 0.25, 2.0 / 3.0};
      sp.a = A[k]; sp.b = Bw[k];
    }
    sp.set_pairs();
    B->stages.push_back(sp);
  }
  B->d.dt = o.dt;
}

void drop_tiled_graphs(fvs_batch* B) {
  if (B->tgraph) cudaGraphExecDestroy(B->tgraph);
  if (B->tgraph_dc) cudaGraphExecDestroy(B->tgraph_dc);
  B->tgraph = B->tgraph_dc = nullptr;
}

// a graph of whatever `enqueue` launches on the batch's stream
template <typename F>
cudaError_t capture_graph(fvs_batch* B, cudaGraphExec_t* out, F enqueue) {
  cudaGraph_t g;
  cudaError_t e = cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t le = enqueue();
  e = cudaStreamEndCapture(B->stream, &g);
  if (e != cudaSuccess) return e;
  if (le != cudaSuccess) {
    cudaGraphDestroy(g);
    return le;
  }
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  return e;
}

// The fused first-order stage: mixed precision, first order and an even
// number of stages (each step then ends in the primary primitive buffer).
bool fusable(const fvs_batch* B) { return B->base.reconst == FVS_RECON_UPWIND1 && B->stages.size() % 2 == 0; }

int apply_fusion(fvs_batch* B) {
  B->d.Pv2 = nullptr;
  if (!(B->fuse && fusable(B) && B->prec == FVS_PREC_MIXED)) return FVS_OK;
  if (!B->pv2_mem && !B->arena.alloc(B->pv2_mem, 16 * (size_t)B->nc))
    return B->fail(FVS_ERR_NOMEM, "second primitive buffer");
  B->d.Pv2 = B->pv2_mem;
  return FVS_OK;
}

// tile lists of the active cases for the current tile length
int build_plan(fvs_batch* B) {
  if (int rc = apply_fusion(B)) return rc;
  std::vector<int4> ct, cases;
  std::vector<int2> et;
  for (int c = 0; c < B->ncases; c++) {
    if (!B->active[c]) continue;
    const int first = (int)ct.size();
    for (int a = B->coff[c]; a < B->coff[c] + B->cnum[c]; a += B->tile)
      ct.push_back(make_int4(a, std::min(a + B->tile, B->coff[c] + B->cnum[c]), c, (int)cases.size()));
    for (int a = B->eoff[c]; a < B->eoff[c] + B->enumv[c]; a += B->tile)
      et.push_back(make_int2(a, std::min(a + B->tile, B->eoff[c] + B->enumv[c])));
    cases.push_back(make_int4(c, first, (int)ct.size(), B->cnum[c]));
  }
  void* p;
  if ((int)ct.size() > B->cap_cell_tiles) {
    const int cap = (int)ct.size() * 2;
    if (!B->arena.alloc(p, 16 * (size_t)cap)) return B->fail(FVS_ERR_NOMEM, "tile list allocation");
    B->d_cell_tiles = static_cast<int4*>(p);
    if (!B->arena.alloc(p, 32 * (size_t)cap)) return B->fail(FVS_ERR_NOMEM, "tile partial allocation");
    B->d_tile_partials = static_cast<double*>(p);
    B->cap_cell_tiles = cap;
  }
  if ((int)et.size() > B->cap_edge_tiles) {
    const int cap = (int)et.size() * 2;
    if (!B->arena.alloc(p, 8 * (size_t)cap)) return B->fail(FVS_ERR_NOMEM, "tile list allocation");
    B->d_edge_tiles = static_cast<int2*>(p);
    B->cap_edge_tiles = cap;
  }
  cudaError_t e = cudaSuccess;
  if (!ct.empty()) e = cudaMemcpy(B->d_cell_tiles, ct.data(), 16 * ct.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !et.empty()) e = cudaMemcpy(B->d_edge_tiles, et.data(), 8 * et.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !cases.empty()) e = cudaMemcpy(B->d_case_tiles, cases.data(), 16 * cases.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return B->cuda_fail(e, "plan upload");
  PersistPlan& P = B->plan;
  P.tile = B->tile;
  P.nstages = (int)B->stages.size();
  for (int k = 0; k < P.nstages; k++) P.sp[k] = B->stages[k];
  P.t1 = 0.0;
  P.step0_dev = B->d_step0;
  P.cell_tiles = B->d_cell_tiles;
  P.ncell_tiles = (int)ct.size();
  P.edge_tiles = B->d_edge_tiles;
  P.nedge_tiles = (int)et.size();
  P.case_tiles = B->d_case_tiles;
  P.ncase_active = (int)cases.size();
  P.case_count = B->d_case_count;
  P.tile_partials = B->d_tile_partials;
  P.case_norms = B->d_case_norms;
  P.norm_cap = B->norm_cap;
  P.bar = B->d_bar;
  int clk = 0;
  cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  P.budget = (long long)(B->budget_s * (clk > 0 ? clk : 2000000) * 1000.0);
  if (B->graph) {
    cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
  }
  drop_tiled_graphs(B);
  B->graph_steps = -1;
  B->plan_dirty = false;
  return FVS_OK;
}

int grid_size(fvs_batch* B) {
  const int occ = B->ks->persistent_occupancy(B->d, B->block);
  return std::max(1, std::min(B->bps, occ)) * B->nsm;
}

// one chunk of nsteps steps starting at global step step0 (graph replay);
// timed: events recorded on the stream around the chunk's launches
int launch_chunk(fvs_batch* B, int nsteps, int step0, bool timed = false) {
  if (B->plan_dirty) {
    int rc = build_plan(B);
    if (rc) return rc;
  }
  if (B->plan.ncell_tiles == 0) return FVS_OK;
  *B->h_step0 = step0;
  cudaError_t e = cudaMemcpyAsync(B->d_step0, B->h_step0, sizeof(int), cudaMemcpyHostToDevice, B->stream);
  if (e != cudaSuccess) return B->cuda_fail(e, "step upload");
  if (B->tiled) {
    // the step counter on the device advances at the end of each step
    B->plan.nsteps = 1;
    if (!B->tgraph) {
      e = capture_graph(B, &B->tgraph, [&]() { return B->ks->tiled_step(B->d, B->plan, B->block, B->stream); });
      if (e != cudaSuccess) return B->cuda_fail(e, "tiled step capture");
    }
    e = cudaMemsetAsync(B->d_bar, 0, sizeof(GridBarrier), B->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(B->d_case_count, 0, sizeof(int) * (size_t)B->ncases, B->stream);
    if (timed) cudaEventRecord(B->eva, B->stream);
    for (int i = 0; i < nsteps && e == cudaSuccess; i++) e = cudaGraphLaunch(B->tgraph, B->stream);
    if (timed) cudaEventRecord(B->evb, B->stream);
    return e == cudaSuccess ? FVS_OK : B->cuda_fail(e, "tiled step launch");
  }
  const int grid = grid_size(B);
  B->plan.nsteps = nsteps;
  if (B->use_graph && B->graph_steps != nsteps) {
    if (B->graph) { cudaGraphExecDestroy(B->graph); B->graph = nullptr; }
    cudaGraph_t g;
    e = cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaMemsetAsync(B->d_bar, 0, sizeof(GridBarrier), B->stream);
      cudaError_t le = B->ks->persistent(B->d, B->plan, grid, B->block, B->stream);
      e = cudaStreamEndCapture(B->stream, &g);
      if (le == cudaSuccess && e == cudaSuccess) {
        e = cudaGraphInstantiate(&B->graph, g, 0);
        cudaGraphDestroy(g);
      } else if (e == cudaSuccess) {
        cudaGraphDestroy(g);
        e = le;
      }
    }
    if (e != cudaSuccess || !B->graph) {
      // capture of cooperative launches unavailable: launch directly
      cudaGetLastError();
      B->use_graph = false;
      B->graph = nullptr;
    } else {
      B->graph_steps = nsteps;
    }
  }
  if (timed) cudaEventRecord(B->eva, B->stream);
  if (B->use_graph) {
    e = cudaGraphLaunch(B->graph, B->stream);
    if (e != cudaSuccess) return B->cuda_fail(e, "cudaGraphLaunch");
  } else {
    e = cudaMemsetAsync(B->d_bar, 0, sizeof(GridBarrier), B->stream);
    if (e == cudaSuccess) e = B->ks->persistent(B->d, B->plan, grid, B->block, B->stream);
    if (e != cudaSuccess) return B->cuda_fail(e, "persistent launch");
  }
  if (timed) cudaEventRecord(B->evb, B->stream);
  return FVS_OK;
}

// A launch shape of the batched kernels.
struct LaunchShape {
  bool tiled, fuse;
  int block, tile, bps;
};

// Online choice of the launch shape as cases converge and the active set
// shrinks (the best shape of a small set differs from that of the full
// batch: fewer, shorter tiles, fewer blocks to synchronise).  Once the active
// cells fall to half of those at the last choice (or at once, when `now`),
// the next chunks run one candidate shape each for a few steps, timed on the
// device, and the fastest is kept.  Every trial step is a step of the run:
// nothing is repeated or discarded.
class ShapeTrials {
 public:
  ShapeTrials(fvs_batch* b, bool dc, bool now) : b_(b) {
    if (!b->retune) return;
    const LaunchShape cur = {b->tiled, b->fuse, b->block, b->tile, b->bps};
    cand_.push_back(cur);
    // separate phases: large tiles at high occupancy suit large active sets,
    // short tiles and few blocks small ones; tiles as long as the block run
    // one item per thread (the single-mesh kernels' shape)
    const bool sep = dc ? b->fuse : false;
    for (const LaunchShape& s : {LaunchShape{false, sep, 256, 1024, 2}, LaunchShape{false, sep, 256, 1024, 4},
                                 LaunchShape{false, sep, 256, 256, 1}, LaunchShape{false, sep, 128, 256, 2},
                                 LaunchShape{true, sep, 256, 4096, 1}, LaunchShape{true, sep, 256, 1024, 1},
                                 LaunchShape{true, sep, 128, 256, 1}, LaunchShape{true, sep, 256, 256, 1},
                                 LaunchShape{true, sep, 128, 128, 1}})
      cand_.push_back(s);
    // the fused first-order stage (two blocks of 256 per SM at most)
    if (!dc && b->prec == FVS_PREC_MIXED && fusable(b))
      for (const LaunchShape& s : {LaunchShape{false, true, 256, 256, 1}, LaunchShape{false, true, 128, 256, 2},
                                   LaunchShape{false, true, 256, 1024, 2}, LaunchShape{true, true, 128, 256, 1}})
        cand_.push_back(s);
    us_.assign(cand_.size(), 0.f);
    cells_ = active_cells();
    if (now) next_ = 0;
  }
  bool trialling() const { return next_ >= 0; }
  // before a chunk: apply the candidate under trial; the chunk length
  int before_chunk(int n) {
    if (next_ < 0) return n;
    apply(cand_[next_]);
    return std::min(n, kTrialSteps);
  }
  // after a chunk of n steps, its events synchronised
  void after_chunk(int n) {
    if (next_ < 0) return;
    float ms = 0.f;
    cudaEventSynchronize(b_->evb);
    const bool ok = cudaEventElapsedTime(&ms, b_->eva, b_->evb) == cudaSuccess;
    cudaGetLastError();
    us_[next_] = ok ? 1000.f * ms / std::max(1, n) : 1e30f;
    if (++next_ < (int)cand_.size()) return;
    int best = 0;
    for (int k = 1; k < (int)cand_.size(); k++)
      if (us_[k] < us_[best]) best = k;
    apply(cand_[best]);
    cand_[0] = cand_[best];
    next_ = -1;
  }
  // after the active set changed
  void active_changed() {
    if (cand_.empty() || next_ >= 0) return;
    const long long c = active_cells();
    if (2 * c <= cells_) {
      cells_ = c;
      next_ = 0;
    }
  }

 private:
  static constexpr int kTrialSteps = 20;
  long long active_cells() const {
    long long n = 0;
    for (int c = 0; c < b_->ncases; c++)
      if (b_->active[c]) n += b_->cnum[c];
    return n;
  }
  void apply(const LaunchShape& s) {
    if (s.tiled == b_->tiled && s.fuse == b_->fuse && s.block == b_->block && s.tile == b_->tile && s.bps == b_->bps)
      return;
    b_->tiled = s.tiled; b_->fuse = s.fuse; b_->block = s.block; b_->tile = s.tile; b_->bps = s.bps;
    b_->plan_dirty = true;
  }
  fvs_batch* b_;
  std::vector<LaunchShape> cand_;
  std::vector<float> us_;
  long long cells_ = 0;
  int next_ = -1;
};

// View of precision prec: the current one, or a variant built on first use
// from the stored host meshes (same device order as every other variant).
int variant_view(fvs_batch* B, int prec, DevView** out) {
  if (prec == B->prec) {
    *out = &B->d;
    return FVS_OK;
  }
  fvs_batch::Variant& v = B->var[prec];
  if (!v.built) {
    init_view_constants(B, v.d);
    const int cur = B->prec;  // build_batch_device reads the precision
    B->prec = prec;
    int rc = build_for(B, prec, v.d);
    B->prec = cur;
    if (rc) return rc;
    v.built = true;
    v.block = B->block; v.tile = B->tile; v.bps = B->bps;
  }
  *out = &v.d;
  return FVS_OK;
}

int check_barrier(fvs_batch* B) {
  GridBarrier gb;
  cudaError_t e = cudaMemcpyAsync(&gb, B->d_bar, sizeof gb, cudaMemcpyDeviceToHost, B->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
  if (e != cudaSuccess) return B->cuda_fail(e, "persistent kernel");
  if (gb.err) return B->fail(FVS_ERR_TIMEOUT, "a grid barrier of the persistent kernel ran out of its wait budget");
  return FVS_OK;
}

}  // namespace

extern "C" {

int fvs_batch_create(const fvs_mesh* meshes, const fvs_options* opts, int32_t ncases, int32_t host_threads,
                     fvs_batch** out) {
  NvtxRange nv("fvs batch setup");
  if (!out) return FVS_ERR_INVALID;
  *out = nullptr;
  if (!meshes || !opts || ncases <= 0) {
    g_batch_create_error = "invalid batch description";
    return FVS_ERR_INVALID;
  }
  const fvs_options& o0 = opts[0];
  for (int c = 1; c < ncases; c++)
    if (!same_scheme(o0, opts[c])) {
      g_batch_create_error = "case " + std::to_string(c) + ": all cases of a batch share the scheme (only Mach and angle of attack differ)";
      return FVS_ERR_INVALID;
    }
  const char* unsupported = o0.grad_method != FVS_GRAD_LSQ             ? "batches run LSQ gradients"
                            : o0.dt_from_cfl                            ? "batches run a fixed dt or steady time stepping"
                            : o0.flux != 1                              ? "batches run the Roe flux"
                            : (o0.rk_nstages < 3 || o0.rk_nstages > 4) ? "batches run 3- or 4-stage Runge-Kutta schemes"
                                                                        : nullptr;
  if (unsupported) {
    g_batch_create_error = unsupported;
    return FVS_ERR_INVALID;
  }
  std::unique_ptr<fvs_batch> B(new fvs_batch());
  B->ncases = ncases;
  B->opt.assign(opts, opts + ncases);
  B->base = o0;
  if (B->base.reconst != FVS_RECON_UMUSCL) B->base.umuscl = 0.0;
  B->hm.resize(ncases);
  // host preprocessing of the cases in parallel
  std::vector<std::string> errs(ncases);
  std::vector<int> rcs(ncases, 0);
  std::atomic<int> next(0);
  int nth = host_threads > 0 ? host_threads : (int)std::max(1u, std::thread::hardware_concurrency());
  nth = std::min(nth, ncases);
  std::vector<std::thread> pool;
  for (int t = 0; t < nth; t++)
    pool.emplace_back([&]() {
      for (int c = next++; c < ncases; c = next++) {
        fvs_options oc = opts[c];
        if (oc.reconst != FVS_RECON_UMUSCL) oc.umuscl = 0.0;
        rcs[c] = build_host_mesh(&meshes[c], &oc, B->hm[c], errs[c]);
      }
    });
  for (auto& th : pool) th.join();
  for (int c = 0; c < ncases; c++)
    if (rcs[c]) {
      g_batch_create_error = "case " + std::to_string(c) + ": " + errs[c];
      return rcs[c];
    }
  B->pinf.resize(4 * (size_t)ncases);
  for (int c = 0; c < ncases; c++) {
    const double aoa = opts[c].aoa_inf_deg * 3.141592653589793238462643383279502884 / 180.0;
    B->pinf[4 * c] = 1.0;
    B->pinf[4 * c + 1] = opts[c].mach_inf * std::cos(aoa);
    B->pinf[4 * c + 2] = opts[c].mach_inf * std::sin(aoa);
    B->pinf[4 * c + 3] = 1.0 / opts[c].gamma;
  }
  B->prec = o0.precision;
  B->mixed = o0.precision == FVS_PREC_MIXED;
  B->ks = kernels_for(o0.precision);
  cudaError_t e = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { g_batch_create_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e); return FVS_ERR_CUDA; }
  cudaMallocHost(&B->h_step0, 16);
  cudaEventCreate(&B->ev0);
  cudaEventCreate(&B->ev1);
  cudaEventCreate(&B->eva);
  cudaEventCreate(&B->evb);
  cudaDeviceGetAttribute(&B->nsm, cudaDevAttrMultiProcessorCount, 0);
  init_view_constants(B.get(), B->d);
  int rc = build_for(B.get(), B->prec, B->d);
  if (!rc) rc = alloc_batch_buffers(B.get());
  if (rc) { g_batch_create_error = B->err; return rc; }
  set_batch_stages(B.get());
  B->active.assign(ncases, 1);
  if (B->ks->persistent_occupancy(B->d, B->block) <= 0) {
    g_batch_create_error = "no persistent kernel for this scheme";
    return FVS_ERR_INVALID;
  }
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { g_batch_create_error = std::string("batch setup: ") + cudaGetErrorString(e); return FVS_ERR_CUDA; }
  *out = B.release();
  return FVS_OK;
}

void fvs_batch_destroy(fvs_batch* b) { delete b; }

const char* fvs_batch_last_error(const fvs_batch* b) { return b ? b->err.c_str() : g_batch_create_error.c_str(); }

int fvs_batch_info(const fvs_batch* b, int32_t* ncells, int32_t* nedges, int32_t* launch4) {
  if (!b) return FVS_ERR_INVALID;
  if (ncells) *ncells = b->nc;
  if (nedges) *nedges = b->ne;
  if (launch4) {
    launch4[0] = b->block;
    launch4[1] = b->tile;
    launch4[2] = b->bps;
    launch4[3] = (b->use_graph ? 1 : 0) | (b->tiled ? 2 : 0) | (b->d.Pv2 ? 4 : 0);
  }
  return FVS_OK;
}

int fvs_batch_set_state(fvs_batch* b, int32_t icase, const double* cvar) {
  if (!b || !cvar || icase < 0 || icase >= b->ncases) return FVS_ERR_INVALID;
  const int n = b->cnum[icase];
  cudaError_t e = cudaMemcpyAsync(b->d_stage, cvar, 32 * (size_t)n, cudaMemcpyHostToDevice, b->stream);
  if (e != cudaSuccess) return b->cuda_fail(e, "state upload");
  kb_scatter_in<<<(n + 255) / 256, 256, 0, b->stream>>>(b->d_stage, b->d_perm + b->ref_off[icase], b->d.U, n);
  // primitives with the kernel set's own conversion (the same rounding as
  // the update kernel produces them)
  b->ks->cvar2pvar(b->d, b->stream);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  return e == cudaSuccess ? FVS_OK : b->cuda_fail(e, "set_state");
}

int fvs_batch_get_state(fvs_batch* b, int32_t icase, double* cvar) {
  if (!b || !cvar || icase < 0 || icase >= b->ncases) return FVS_ERR_INVALID;
  const int n = b->cnum[icase];
  kb_gather_out<<<(n + 255) / 256, 256, 0, b->stream>>>(b->d.U, b->d_perm + b->ref_off[icase], b->d_stage, n);
  cudaError_t e = cudaMemcpyAsync(cvar, b->d_stage, 32 * (size_t)n, cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  return e == cudaSuccess ? FVS_OK : b->cuda_fail(e, "get_state");
}

int fvs_batch_init_state(fvs_batch* b) {
  if (!b) return FVS_ERR_INVALID;
  // free stream of each case (src/initialize.f90:36-44)
  for (int c = 0; c < b->ncases; c++) {
    const double* p = &b->pinf[4 * c];
    const double g = b->opt[c].gamma;
    double u[4] = {p[0], p[0] * p[1], p[0] * p[2], p[3] / (g - 1.0) + 0.5 * p[0] * (p[1] * p[1] + p[2] * p[2])};
    std::vector<double> cv(4 * (size_t)b->cnum[c]);
    for (int i = 0; i < b->cnum[c]; i++) std::memcpy(&cv[4 * i], u, sizeof u);
    int rc = fvs_batch_set_state(b, c, cv.data());
    if (rc) return rc;
  }
  return FVS_OK;
}

// Switches the batch to another arithmetic (the precision ladder: a mixed
// phase followed by an FP64 phase).  The other precision's device layout is
// built on first use from the stored host meshes; the FP64 state is copied.
int fvs_batch_set_precision(fvs_batch* b, int32_t precision) {
  if (!b || precision < 0 || precision > 3) return FVS_ERR_INVALID;
  if (precision == b->prec) return FVS_OK;
  fvs_batch::Variant& cur = b->var[b->prec];
  cur.built = true;
  cur.d = b->d;
  cur.block = b->block; cur.tile = b->tile; cur.bps = b->bps; cur.tiled = b->tiled;
  fvs_batch::Variant& nxt = b->var[precision];
  const int old_prec = b->prec;
  b->prec = precision;
  if (!nxt.built) {
    init_view_constants(b, nxt.d);
    int rc = build_for(b, precision, nxt.d);
    if (rc) {
      b->prec = old_prec;
      return rc;
    }
    nxt.built = true;
    nxt.block = b->block; nxt.tile = b->tile; nxt.bps = b->bps; nxt.tiled = b->tiled;
  }
  cudaError_t e = cudaMemcpyAsync(nxt.d.U, cur.d.U, 32 * (size_t)b->nc, cudaMemcpyDeviceToDevice, b->stream);
  if (e != cudaSuccess) return b->cuda_fail(e, "state copy");
  b->d = nxt.d;
  b->ks = kernels_for(precision);
  b->mixed = precision == FVS_PREC_MIXED;
  b->block = nxt.block; b->tile = nxt.tile; b->bps = nxt.bps; b->tiled = nxt.tiled;
  b->ks->cvar2pvar(b->d, b->stream);
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  drop_tiled_graphs(b);
  b->graph_steps = -1;
  b->plan_dirty = true;
  e = cudaStreamSynchronize(b->stream);
  return e == cudaSuccess ? FVS_OK : b->cuda_fail(e, "precision switch");
}

int fvs_batch_set_groups(fvs_batch* b, const int32_t* group) {
  if (!b) return FVS_ERR_INVALID;
  if (!group) {
    b->group.clear();
    return FVS_OK;
  }
  b->group.assign(group, group + b->ncases);
  return FVS_OK;
}

int fvs_batch_set_mode(fvs_batch* b, int32_t mode) {
  if (!b || mode < 0 || mode > (FVS_BATCH_TILED | FVS_BATCH_UNFUSED | FVS_BATCH_DC_FUSED | FVS_BATCH_FIXED_SHAPE))
    return FVS_ERR_INVALID;
  b->tiled = (mode & FVS_BATCH_TILED) != 0;
  b->fuse = (mode & FVS_BATCH_UNFUSED) == 0;
  b->fuse_dc = (mode & FVS_BATCH_DC_FUSED) != 0;
  b->retune = (mode & FVS_BATCH_FIXED_SHAPE) == 0;
  b->plan_dirty = true;
  return FVS_OK;
}

int fvs_batch_set_barrier_budget(fvs_batch* b, double seconds) {
  if (!b || seconds < 0) return FVS_ERR_INVALID;
  b->budget_s = seconds;
  b->plan_dirty = true;
  return FVS_OK;
}

int fvs_batch_set_launch(fvs_batch* b, int32_t block, int32_t tile, int32_t blocks_per_sm) {
  if (!b || (block != 64 && block != 128 && block != 256) || tile < block || blocks_per_sm < 1) return FVS_ERR_INVALID;
  if (b->ks->persistent_occupancy(b->d, block) <= 0) return b->fail(FVS_ERR_INVALID, "block size does not fit");
  b->block = block;
  b->tile = tile;
  b->bps = blocks_per_sm;
  b->plan_dirty = true;
  return FVS_OK;
}

// nsteps steps of every active case; norms (optional) [ncases][nsteps][4]
int fvs_batch_steps(fvs_batch* b, int32_t nsteps, double* norms, float* ms) {
  NvtxRange nv("fvs batch steps");
  if (!b || nsteps <= 0 || nsteps > b->norm_cap) return FVS_ERR_INVALID;
  cudaEventRecord(b->ev0, b->stream);
  int rc = launch_chunk(b, nsteps, 0);
  if (rc) return rc;
  cudaEventRecord(b->ev1, b->stream);
  if ((rc = check_barrier(b))) return rc;
  if (ms) cudaEventElapsedTime(ms, b->ev0, b->ev1);
  if (norms) {
    std::vector<double> all(4 * (size_t)b->ncases * b->norm_cap);
    cudaError_t e = cudaMemcpy(all.data(), b->d_case_norms, 8 * all.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return b->cuda_fail(e, "norm download");
    for (int c = 0; c < b->ncases; c++)
      std::memcpy(norms + 4 * (size_t)c * nsteps, &all[4 * (size_t)c * b->norm_cap], 32 * (size_t)nsteps);
  }
  return FVS_OK;
}

// Candidate launch shapes timed on the batch itself; the state is restored.
int fvs_batch_autotune(fvs_batch* b, int32_t trial_steps, float* best_ms) {
  NvtxRange nv("fvs batch autotune");
  if (!b || trial_steps <= 0 || trial_steps > b->norm_cap) return FVS_ERR_INVALID;
  cudaError_t e = cudaMemcpy(b->d_backup, b->d.U, 32 * (size_t)b->nc, cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) return b->cuda_fail(e, "state backup");
  const int blocks[2] = {128, 256};
  const int tiles_per_block[3] = {1, 4, 16};
  float best = 1e30f;
  int bb = b->block, bt = b->tile, bp = b->bps;
  bool btiled = b->tiled, bfuse = b->fuse;
  // the fused first-order stage is timed against the separate phases where
  // it applies
  const int nfuse = (b->prec == FVS_PREC_MIXED && fusable(b)) ? 2 : 1;
  for (int fz = 0; fz < nfuse; fz++)
  for (int mode = 0; mode < 2; mode++)
  for (int blk : blocks) {
    if (nfuse == 2) b->fuse = fz == 1;
    if (int rc = apply_fusion(b)) return rc;  // the occupancy below is the variant's
    const int occ = b->ks->persistent_occupancy(b->d, blk);
    if (occ <= 0) continue;
    const int bps_list[3] = {1, std::max(1, occ / 2), occ};
    for (int tpb : tiles_per_block)
      for (int q = 0; q < 3; q++) {
        if (q > 0 && bps_list[q] == bps_list[q - 1]) continue;
        if (mode == 1 && q > 0) continue;  // blocks per SM do not apply to tile launches
        b->block = blk;
        b->tile = blk * tpb;
        b->bps = bps_list[q];
        b->tiled = mode == 1;
        b->plan_dirty = true;
        float ms = 0.f;
        int rc = fvs_batch_steps(b, 1, nullptr, nullptr);  // warm-up, graph capture
        if (!rc) rc = fvs_batch_steps(b, trial_steps, nullptr, &ms);
        if (rc) return rc;
        if (ms < best) {
          best = ms;
          bb = blk; bt = blk * tpb; bp = bps_list[q]; btiled = b->tiled; bfuse = b->fuse;
        }
      }
  }
  b->block = bb;
  b->tile = bt;
  b->bps = bp;
  b->tiled = btiled;
  b->fuse = bfuse;
  b->plan_dirty = true;
  e = cudaMemcpy(b->d.U, b->d_backup, 32 * (size_t)b->nc, cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) return b->cuda_fail(e, "state restore");
  // primitives of the restored state
  b->ks->cvar2pvar(b->d, b->stream);
  e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return b->cuda_fail(e, "autotune restore");
  if (best_ms) *best_ms = best / trial_steps;
  return FVS_OK;
}

// A case that converged ends the other cases of its group at the same step
// (several starts of one problem raced against each other).
void stop_group(fvs_batch* b, int c, int at, std::vector<int>& done) {
  if (b->group.empty()) return;
  for (int k = 0; k < b->ncases; k++)
    if (k != c && b->active[k] && b->group[k] == b->group[c]) {
      b->active[k] = 0;
      done[k] = at;
    }
}

// Steps all cases until each one's RMS(dU_rho) falls to drop x its first
// value (or max_steps).  steps_done[c] = the step at which case c reached the
// drop (max_steps if it did not); first/last [ncases][4] norms.
static int run_until(fvs_batch* b, int32_t max_steps, double drop, const double* levels, int32_t chunk,
                     int32_t* steps_done, double* first, double* last, float* ms) {
  if (!b || max_steps <= 0 || chunk <= 0 || chunk > b->norm_cap) return FVS_ERR_INVALID;
  const int nc = b->ncases;
  std::vector<double> f(4 * (size_t)nc, -1.0), l(4 * (size_t)nc, 0.0);
  std::vector<int> done(nc, max_steps);
  std::fill(b->active.begin(), b->active.end(), 1);
  b->plan_dirty = true;
  std::vector<double> all(4 * (size_t)nc * b->norm_cap);
  std::vector<int> conv_now;
  cudaEventRecord(b->ev0, b->stream);
  int step = 0, rc = FVS_OK;
  bool nonfinite = false;
  // shapes chosen for a shrunken active set last for this run only
  const LaunchShape start = {b->tiled, b->fuse, b->block, b->tile, b->bps};
  ShapeTrials trials(b, false, false);
  while (step < max_steps) {
    const int n = trials.before_chunk(std::min(chunk, max_steps - step));
    if ((rc = launch_chunk(b, n, step, trials.trialling()))) break;
    if ((rc = check_barrier(b))) break;
    cudaError_t e = cudaMemcpy(all.data(), b->d_case_norms, 8 * all.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { rc = b->cuda_fail(e, "norm download"); break; }
    bool changed = false;
    int nact = 0;
    for (int c = 0; c < nc; c++) {
      if (!b->active[c]) continue;
      for (int s = 0; s < n; s++) {
        const double* v = &all[4 * ((size_t)c * b->norm_cap + (step + s) % b->norm_cap)];
        if (!std::isfinite(v[0])) { nonfinite = true; b->active[c] = 0; done[c] = step + s + 1; changed = true; break; }
        if (f[4 * c] < 0) std::memcpy(&f[4 * c], v, 32);
        std::memcpy(&l[4 * c], v, 32);
        // converged when every component is at its target (one component can
        // dip under its level while an oscillating mode passes through zero)
        bool conv = true;
        for (int k = 0; k < 4; k++) conv = conv && v[k] <= (levels ? levels[4 * c + k] : drop * f[4 * c + k]);
        if (conv) {
          done[c] = step + s + 1;
          b->active[c] = 0;
          changed = true;
          conv_now.push_back(c);
          break;
        }
      }
    }
    // the earliest converged case of a group ends the group
    std::sort(conv_now.begin(), conv_now.end(), [&](int x, int y) { return done[x] < done[y]; });
    for (int c : conv_now) stop_group(b, c, done[c], done);
    conv_now.clear();
    for (int c = 0; c < nc; c++) nact += b->active[c];
    step += n;
    if (nact == 0) break;
    trials.after_chunk(n);
    if (changed) {
      b->plan_dirty = true;
      trials.active_changed();
    }
  }
  cudaEventRecord(b->ev1, b->stream);
  cudaEventSynchronize(b->ev1);
  if (ms) cudaEventElapsedTime(ms, b->ev0, b->ev1);
  b->tiled = start.tiled; b->fuse = start.fuse; b->block = start.block; b->tile = start.tile; b->bps = start.bps;
  std::fill(b->active.begin(), b->active.end(), 1);
  b->plan_dirty = true;
  if (steps_done) std::memcpy(steps_done, done.data(), 4 * (size_t)nc);
  if (first) std::memcpy(first, f.data(), 32 * (size_t)nc);
  if (last) std::memcpy(last, l.data(), 32 * (size_t)nc);
  if (rc) return rc;
  return nonfinite ? b->fail(FVS_ERR_NONFINITE, "a case's residual norm is not finite") : FVS_OK;
}

// Defect-correction run of a first-order steady batch to absolute per-case
// levels [ncases][4].  Each chunk of `chunk` steps: fold the correction into
// the FP64 state, evaluate the FP64 residual and local dt there, then iterate
// the correction in one cooperative launch with the linearised residual.
// The norms are the RMS of the correction increments per step.  Leaves the
// batch in FP64 with the folded state.
int fvs_batch_run_to_level_dc(fvs_batch* b, int32_t max_steps, const double* levels, int32_t chunk,
                              int32_t* steps_done, double* first, double* last, float* ms) {
  NvtxRange nv("fvs batch defect correction");
  if (!b || !levels || max_steps <= 0 || chunk <= 0 || chunk > b->norm_cap) return FVS_ERR_INVALID;
  if (!b->base.steady || b->base.reconst != FVS_RECON_UPWIND1)
    return b->fail(FVS_ERR_INVALID, "defect correction runs first-order steady batches");
  int rc = fvs_batch_set_precision(b, FVS_PREC_FP64);
  if (rc) return rc;
  DevView* d32 = nullptr;
  if ((rc = variant_view(b, FVS_PREC_MIXED, &d32))) return rc;
  DevView& d64 = b->d;
  const size_t n4 = 16 * (size_t)b->nc;
  if (!b->dc.D) {
    void* p[6];
    for (int k = 0; k < 6; k++)
      if (!b->arena.alloc(p[k], k < 5 ? n4 : 4 * (size_t)b->nc)) return b->fail(FVS_ERR_NOMEM, "defect-correction arrays");
    b->dc.D = static_cast<float*>(p[0]); b->dc.D0 = static_cast<float*>(p[1]);
    b->dc.DF = static_cast<float*>(p[2]); b->dc.dP = static_cast<float*>(p[3]);
    b->dc.R0 = static_cast<float*>(p[4]); b->dc.dtl = static_cast<float*>(p[5]);
  }
  cudaError_t e = cudaMemsetAsync(b->dc.D, 0, n4, b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->dc.dP, 0, n4, b->stream);
  if (e != cudaSuccess) return b->cuda_fail(e, "defect-correction reset");
  const DcKernels& K = dc_kernels();
  const KernelSet& K64 = kernels_fp64_fast();
  // launch shape of the mixed variant (tuned there when the batch ran mixed)
  const fvs_batch::Variant& vm = b->var[FVS_PREC_MIXED];
  const int sb = b->block, st = b->tile, sp = b->bps;
  const bool stl = b->tiled;
  if (vm.built) { b->block = vm.block; b->tile = vm.tile; b->bps = vm.bps; b->tiled = vm.tiled; }
  const bool fuse_dc = b->fuse_dc && fusable(b);
  if (fuse_dc && !b->dp2_mem && !b->arena.alloc(b->dp2_mem, 16 * (size_t)b->nc))
    return b->fail(FVS_ERR_NOMEM, "second tangent buffer");
  b->dc.dP2 = fuse_dc ? static_cast<float*>(b->dp2_mem) : nullptr;
  if (K.occupancy(b->dc, b->block) <= 0) return b->fail(FVS_ERR_INVALID, "no resident block for the defect-correction kernel");
  const int nc = b->ncases;
  std::vector<double> f(4 * (size_t)nc, -1.0), l(4 * (size_t)nc, 0.0);
  std::vector<int> done(nc, max_steps);
  std::fill(b->active.begin(), b->active.end(), 1);
  b->plan_dirty = true;
  std::vector<double> all(4 * (size_t)nc * b->norm_cap);
  std::vector<int> conv_now;
  cudaEventRecord(b->ev0, b->stream);
  int step = 0;
  bool nonfinite = false;
  ShapeTrials trials(b, true, true);
  while (step < max_steps) {
    const int n = trials.before_chunk(std::min(chunk, max_steps - step));
    if (b->plan_dirty && (rc = build_plan(b))) break;
    const int occ = K.occupancy(b->dc, b->block);
    if (occ <= 0) { rc = b->fail(FVS_ERR_INVALID, "no resident block for the defect-correction kernel"); break; }
    const int grid = std::max(1, std::min(b->bps, occ)) * b->nsm;
    // base state of the chunk: fold, FP64 residual and wave speeds, FP32 copies
    K.fold(*d32, b->dc, d64.U, b->stream);
    K64.cvar2pvar(d64, b->stream);
    K64.flux(d64, 0.0, true, b->stream);
    K64.residual_out(d64, b->stream);
    K.base(*d32, b->dc, d64.U, d64.resid, d64.ws, b->stream);
    *b->h_step0 = step;
    e = cudaMemcpyAsync(b->d_step0, b->h_step0, sizeof(int), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_bar, 0, sizeof(GridBarrier), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_case_count, 0, sizeof(int) * (size_t)b->ncases, b->stream);
    if (b->tiled) {
      b->plan.nsteps = 1;
      if (e == cudaSuccess && !b->tgraph_dc)
        e = capture_graph(b, &b->tgraph_dc, [&]() { return K.tiled_step(*d32, b->plan, b->dc, b->block, b->stream); });
      if (trials.trialling()) cudaEventRecord(b->eva, b->stream);
      for (int i = 0; i < n && e == cudaSuccess; i++) e = cudaGraphLaunch(b->tgraph_dc, b->stream);
    } else {
      b->plan.nsteps = n;
      if (trials.trialling()) cudaEventRecord(b->eva, b->stream);
      if (e == cudaSuccess) e = K.persistent(*d32, b->plan, b->dc, grid, b->block, b->stream);
    }
    if (trials.trialling()) cudaEventRecord(b->evb, b->stream);
    if (e != cudaSuccess) { rc = b->cuda_fail(e, "defect-correction chunk"); break; }
    if ((rc = check_barrier(b))) break;
    e = cudaMemcpy(all.data(), b->d_case_norms, 8 * all.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { rc = b->cuda_fail(e, "norm download"); break; }
    bool changed = false;
    int nact = 0;
    for (int c = 0; c < nc; c++) {
      if (!b->active[c]) continue;
      for (int s = 0; s < n; s++) {
        const double* v = &all[4 * ((size_t)c * b->norm_cap + (step + s) % b->norm_cap)];
        if (!std::isfinite(v[0])) { nonfinite = true; b->active[c] = 0; done[c] = step + s + 1; changed = true; break; }
        if (f[4 * c] < 0) std::memcpy(&f[4 * c], v, 32);
        std::memcpy(&l[4 * c], v, 32);
        bool conv = true;
        for (int k = 0; k < 4; k++) conv = conv && v[k] <= levels[4 * c + k];
        if (conv) {
          done[c] = step + s + 1;
          b->active[c] = 0;
          changed = true;
          conv_now.push_back(c);
          break;
        }
      }
    }
    // the earliest converged case of a group ends the group
    std::sort(conv_now.begin(), conv_now.end(), [&](int x, int y) { return done[x] < done[y]; });
    for (int c : conv_now) stop_group(b, c, done[c], done);
    conv_now.clear();
    for (int c = 0; c < nc; c++) nact += b->active[c];
    step += n;
    if (nact == 0) break;
    trials.after_chunk(n);
    if (changed) {
      b->plan_dirty = true;
      trials.active_changed();
    }
  }
  // the last correction into the FP64 state
  K.fold(*d32, b->dc, d64.U, b->stream);
  K64.cvar2pvar(d64, b->stream);
  cudaEventRecord(b->ev1, b->stream);
  e = cudaEventSynchronize(b->ev1);
  if (!rc && e != cudaSuccess) rc = b->cuda_fail(e, "defect-correction run");
  if (ms) cudaEventElapsedTime(ms, b->ev0, b->ev1);
  b->block = sb; b->tile = st; b->bps = sp; b->tiled = stl;
  std::fill(b->active.begin(), b->active.end(), 1);
  b->plan_dirty = true;
  if (steps_done) std::memcpy(steps_done, done.data(), 4 * (size_t)nc);
  if (first) std::memcpy(first, f.data(), 32 * (size_t)nc);
  if (last) std::memcpy(last, l.data(), 32 * (size_t)nc);
  if (rc) return rc;
  return nonfinite ? b->fail(FVS_ERR_NONFINITE, "a case's residual norm is not finite") : FVS_OK;
}

int fvs_batch_run_to_drop(fvs_batch* b, int32_t max_steps, double drop, int32_t chunk, int32_t* steps_done,
                          double* first, double* last, float* ms) {
  return run_until(b, max_steps, drop, nullptr, chunk, steps_done, first, last, ms);
}

int fvs_batch_run_to_level(fvs_batch* b, int32_t max_steps, const double* levels, int32_t chunk, int32_t* steps_done,
                           double* first, double* last, float* ms) {
  NvtxRange nv("fvs batch run to level");
  if (!levels) return FVS_ERR_INVALID;
  return run_until(b, max_steps, 0.0, levels, chunk, steps_done, first, last, ms);
}

}  // extern "C"
