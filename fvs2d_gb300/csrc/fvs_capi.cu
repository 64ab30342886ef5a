// fvs_capi.cu — the C-ABI of include/fvs2d.h: handle life cycle, device
// layout (reverse Cuthill-McKee cell order, edge slots, gather lists), the
// per-step CUDA graph and the host<->device copies.
//
// Reference procedures replaced (see include/fvs2d.h for the mapping):
//   compute_residual   src/residual.f90:23-177   -> fvs_residual
//   time_integration   src/runge_kutta.f90:94-114 -> fvs_time_integration
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "df64.cuh"
#include "fp64_fast.cuh"
#include "fvs_internal.hpp"
#include "fvs_layout.hpp"
#include "fvs_tiles.hpp"

using namespace fvs;

namespace {

thread_local std::string g_create_error;

__global__ void k_scatter_in(const double* __restrict__ ref, const int* __restrict__ perm, double* __restrict__ dev, int nc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const double2* s = reinterpret_cast<const double2*>(ref) + 2 * (size_t)i;
  double2* t = reinterpret_cast<double2*>(dev) + 2 * (size_t)perm[i];
  t[0] = s[0];
  t[1] = s[1];
}

__global__ void k_gather_out(const double* __restrict__ dev, const int* __restrict__ perm, double* __restrict__ ref, int nc,
                             int width) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  for (int k = 0; k < width; k++) ref[(size_t)width * i + k] = dev[(size_t)width * perm[i] + k];
}

template <typename T>
__global__ void k_gather_out_t(const T* __restrict__ dev, const int* __restrict__ perm, double* __restrict__ ref, int nc, int width) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  for (int k = 0; k < width; k++) ref[(size_t)width * i + k] = double(dev[(size_t)width * perm[i] + k]);
}

// Wall pressure coefficient, normal velocity and loads of one slip-wall
// boundary (write_inst_cp_un, src/io.f90:340-446).  One block: every thread
// evaluates the face values of its edges into `edges` [n][4] = (xf, cp,
// cp_cell, un); thread 0 then sums in edge order into sums[7] = (cn, ca, cn1,
// ca1, |un|max, sum un^2, sum |un|).  __dmul_rn / __dadd_rn / __dsub_rn round
// each product and sum on its own (no multiply-add contraction), in the
// reference's evaluation order.
template <typename T>
__global__ void k_wall_loads(DevView d, int g0, int n, double c2, double p_inf, double* edges, double* sums) {
  const T* P = static_cast<const T*>(d.Pv);
  const T* GX = static_cast<const T*>(d.Gx);
  const T* GY = static_cast<const T*>(d.Gy);
  const T* DL = static_cast<const T*>(d.edL);
  const T* NR = static_cast<const T*>(d.enrm);
  const T* AR = static_cast<const T*>(d.earea);
  const T* XY = static_cast<const T*>(d.exy);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int g = g0 + i, c = d.ecell[g].x;
    const double dx = double(DL[2 * g]), dy = double(DL[2 * g + 1]);
    double w[4];
    for (int v = 1; v < 4; v++)
      w[v] = __dadd_rn(__dadd_rn(double(P[4 * c + v]), __dmul_rn(dx, double(GX[4 * c + v]))),
                       __dmul_rn(dy, double(GY[4 * c + v])));
    const double nx = double(NR[2 * g]), ny = double(NR[2 * g + 1]);
    double* e = edges + 4 * (size_t)i;
    e[0] = double(XY[2 * g]);
    e[1] = __dmul_rn(c2, __dsub_rn(w[3], p_inf));
    e[2] = __dmul_rn(c2, __dsub_rn(double(P[4 * c + 3]), p_inf));
    e[3] = __dadd_rn(__dmul_rn(w[1], nx), __dmul_rn(w[2], ny));
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double cn = 0, ca = 0, cn1 = 0, ca1 = 0, un_max = 0, un_l2 = 0, un_l1 = 0;
  for (int i = 0; i < n; i++) {
    const int g = g0 + i;
    const double* e = edges + 4 * (size_t)i;
    const double nx = double(NR[2 * g]), ny = double(NR[2 * g + 1]), af = double(AR[g]);
    cn = __dadd_rn(cn, __dmul_rn(__dmul_rn(e[1], ny), af));
    ca = __dadd_rn(ca, __dmul_rn(__dmul_rn(e[1], nx), af));
    cn1 = __dadd_rn(cn1, __dmul_rn(__dmul_rn(e[2], ny), af));
    ca1 = __dadd_rn(ca1, __dmul_rn(__dmul_rn(e[2], nx), af));
    const double a = fabs(e[3]);
    un_l2 = __dadd_rn(un_l2, __dmul_rn(e[3], e[3]));
    un_l1 = __dadd_rn(un_l1, a);
    un_max = un_max > a ? un_max : a;
  }
  sums[0] = cn; sums[1] = ca; sums[2] = cn1; sums[3] = ca1;
  sums[4] = un_max; sums[5] = un_l2; sums[6] = un_l1;
}

// out[5i..5i+4] = rcp_nr(x), 1/x, rsqrt_nr(x), sqrt_nr(x), sqrt(x)
__global__ void k_check_fp64_math(const double* __restrict__ x, int n, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = x[i];
  double* o = out + 5 * (size_t)i;
  o[0] = rcp_nr(v);
  o[1] = 1.0 / v;
  o[2] = rsqrt_nr(v);
  o[3] = sqrt_nr(v);
  o[4] = sqrt(v);
}

}  // namespace

struct fvs_handle {
  HostMesh hm;
  fvs_options o;
  double pvar_inf[4];
  std::string err;
  const KernelSet* ks = nullptr;
  bool mixed = false;
  bool df = false;  // double-float kernels (FVS_PREC_FP64_DF)
  cudaStream_t stream = nullptr;
  DeviceArena arena;
  DevView d;
  std::vector<int> perm;   // reference cell -> device cell
  int* d_perm = nullptr;   // device copy of perm
  double* d_stage = nullptr;  // [nc][4] reference-order staging
  double* h_small = nullptr;  // pinned scratch for control words
  std::vector<StageParams> stages;
  double dt = 0;
  bool dt_ready = false;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int nblk = 0;
  int launches_per_step = 0;
  bool host_only = false;
  double* d_wall = nullptr;  // wall-load scratch, allocated on first use
  size_t wall_cap = 0;
  // index-checking kernels (FVS2D_BOUNDS=1): their error word
  bool bounds = false;
  // fused RK stage (mixed and double-float): cells in tile order, one
  // launch per stage (k_tile_stage)
  bool fused = false;
  int tile_mode = 0;  // 1: the whole stage per tile; 2: flux + update per tile; 3: bulk-copy whole stage
  TileView tv;
  TileDmaView dv;
  bool gb_stale = true;  // the gather buffer does not hold the current primitives
  // d with one norm partial per tile block, for the fused stage
  DevView tile_view() const {
    DevView v = d;
    v.nblk_red = tv.ntiles;
    return v;
  }

  ~fvs_handle() {
    if (d_wall) cudaFree(d_wall);
    if (graph) cudaGraphExecDestroy(graph);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    arena.release();
    if (h_small) cudaFreeHost(h_small);
    if (stream) cudaStreamDestroy(stream);
  }

  int fail(int code, const std::string& msg) {
    err = msg;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* where) {
    err = std::string(where) + ": " + cudaGetErrorString(e);
    return FVS_ERR_CUDA;
  }
};

namespace {

// The fused RK stage runs for mixed and double-float handles when the
// environment variable FVS2D_TILE_STAGE is "1" at fvs_create.  It is off by
// default: on GB300 the three separate kernels are faster (1,048,576-cell
// vortex, per SSP-RK3 step: mixed 0.262 against 0.310 ms, double-float 0.656
// against 1.014 ms), because each tile block runs its four phases one after
// the other between barriers, latency-bound at 24-40 resident warps per SM.
// FVS2D_TILE_STAGE=2 selects the lighter fusion: the gradient kernel as
// before, then face flux and update in one launch per tile
// (k_tile_flux_update).  Returns the mode: 0 none, 1 full, 2 flux + update.
// FVS2D_TILE_STAGE=3 selects the bulk-copy form (k_tile_dma; mixed handles
// with LSQ gradients).
int want_fused(const fvs_handle* H) {
  if (H->o.precision != FVS_PREC_MIXED && H->o.precision != FVS_PREC_FP64_DF) return 0;
  const char* e = std::getenv("FVS2D_TILE_STAGE");
  if (!e || e[1] != 0) return 0;
  if (e[0] == '3') return (H->o.precision == FVS_PREC_MIXED && H->o.grad_method == FVS_GRAD_LSQ) ? 3 : 0;
  return e[0] == '1' ? 1 : e[0] == '2' ? 2 : 0;
}

// Tile plan of a fused handle from its device-order layout: plan arrays,
// the extra primitive buffers (two in all for an even number of stages,
// three for an odd one, so that every step starts and ends in Pv) and the
// tile block's shared memory.  Returns false (handle stays unfused) when a
// tile block would need more shared memory than a block may have.
template <typename T>
int build_tiles(fvs_handle* H, const Layout<T>& L, const std::vector<int>& tile_start, bool& ok, TilePlan& P) {
  ok = false;
  std::string err;
  int rc = build_tile_plan(tile_start, L.ecell, L.cf, L.st_ptr, L.st_cell, P, err);
  if (rc) return H->fail(rc, err);
  P.tile_cells = tile_cells_setting();
  err = check_tile_plan(P, L.nc, L.ne, L.ecell, L.cf, L.st_ptr);
  if (!err.empty()) return H->fail(FVS_ERR_MESH, "tile plan: " + err);
  TileView& tv = H->tv;
  tv.ntiles = P.ntiles;
  tv.lmax = P.lmax;
  tv.gmax = P.gmax;
  tv.fmax = P.fmax;
  tv.smem_bytes = H->ks->tile_smem(P.lmax, P.gmax, P.fmax);
  if (tv.smem_bytes == 0) return FVS_OK;
  int *c0, *h0, *nh1, *halo, *g0, *lsp, *s0, *f0, *face;
  uint16_t* lst;
  uint32_t* flr;
  int2* lcf;
  DeviceArena& A = H->arena;
  bool up = A.upload(c0, P.c0) && A.upload(h0, P.h0) && A.upload(nh1, P.nh1) && A.upload(halo, P.halo) &&
            A.upload(g0, P.g0) && A.upload(lsp, P.lsp) && A.upload(s0, P.s0) && A.upload(lst, P.lst) &&
            A.upload(f0, P.f0) && A.upload(face, P.face) && A.upload(flr, P.flr) && A.upload(lcf, P.lcf);
  tv.c0 = c0; tv.h0 = h0; tv.nh1 = nh1; tv.halo = halo; tv.g0 = g0; tv.lsp = lsp; tv.s0 = s0; tv.lst = lst;
  tv.f0 = f0; tv.face = face; tv.flr = flr; tv.lcf = lcf;
  // tile-major face records and gradient-cell records
  std::vector<T> fgeo(8 * P.face.size(), T(0));
  for (size_t f = 0; f < P.face.size(); f++) {
    const int e = P.face[f];
    T* g = &fgeo[8 * f];
    g[0] = L.enrm[2 * (size_t)e]; g[1] = L.enrm[2 * (size_t)e + 1]; g[2] = L.earea[e];
    g[3] = L.edL[2 * (size_t)e]; g[4] = L.edL[2 * (size_t)e + 1];
    g[5] = L.edR[2 * (size_t)e]; g[6] = L.edR[2 * (size_t)e + 1];
  }
  std::vector<int2> gcell(P.lsp.size(), make_int2(0, 0));
  for (int t = 0; t < P.ntiles; t++) {
    const int b = P.c0[t], n = P.c0[t + 1] - b, ng = P.g0[t + 1] - P.g0[t] - 1;
    for (int i = 0; i < ng; i++) {
      const int gid = i < n ? b + i : P.halo[P.h0[t] + i - n];
      gcell[P.g0[t] + i] = make_int2(gid, L.st_ptr[gid]);
    }
  }
  T* dfgeo;
  int2* dgcell;
  up = up && A.upload(dfgeo, fgeo) && A.upload(dgcell, gcell);
  tv.fgeo = dfgeo;
  tv.gcell = dgcell;
  // one norm partial per tile block (tiles hold at least tile_cells / 2
  // cells, so there can be more tiles than 256-cell blocks)
  if (P.ntiles > H->nblk) {
    void* q = nullptr;
    if (!A.alloc(q, 32 * (size_t)P.ntiles)) return H->fail(FVS_ERR_NOMEM, "norm partials of the tile plan");
    H->d.partials = static_cast<double*>(q);
  }
  tv.nbuf = H->o.rk_nstages % 2 == 0 ? 2 : 3;
  tv.Pbuf[0] = H->d.Pv;
  for (int k = 1; k < tv.nbuf && up; k++) up = A.alloc(tv.Pbuf[k], sizeof(T) * 4 * (size_t)L.nc);
  if (!up) return H->fail(FVS_ERR_NOMEM, "device allocation or upload of the tile plan failed");
  ok = true;
  return FVS_OK;
}

// The bulk-copy plan of a fused handle (mode 3): segments, coefficients in
// tile order, gather buffers, the error word and the shared-memory layout;
// every copy's alignment and extent checked.  ok = false leaves the handle
// on the separate kernels (a block would need too much shared memory).
template <typename T>
int build_tile_dma_view(fvs_handle* H, const Layout<T>& L, const TilePlan& P, bool& ok) {
  ok = false;
  std::string err;
  TileDma D;
  build_tile_dma(P, L.st_ptr, L.nc, D);
  err = check_tile_dma(P, D, (int)sizeof(T), L.nc, L.st_cell.size());
  if (!err.empty()) return H->fail(FVS_ERR_MESH, "bulk-copy tile plan: " + err);
  std::vector<T> coef(2 * D.coef_src.size(), T(0));
  for (size_t k = 0; k < D.coef_src.size(); k++)
    if (D.coef_src[k] >= 0) {
      coef[2 * k] = L.st_coef[2 * (size_t)D.coef_src[k]];
      coef[2 * k + 1] = L.st_coef[2 * (size_t)D.coef_src[k] + 1];
    }
  TileDmaView& dv = H->dv;
  dv.smax = D.smax; dv.pmax = D.pmax; dv.rmax = D.rmax; dv.qmax = D.qmax;
  const DmaSmem m = dma_smem((int)sizeof(T), P.lmax, P.gmax, P.fmax, D.smax, D.pmax, D.rmax, D.qmax);
  dv.o_P = (unsigned)m.P; dv.o_Fg = (unsigned)m.Fg; dv.o_C = (unsigned)m.C; dv.o_L = (unsigned)m.L;
  dv.o_S = (unsigned)m.S; dv.o_R = (unsigned)m.Rr; dv.o_Q = (unsigned)m.Q; dv.o_Gx = (unsigned)m.Gx;
  dv.o_Gy = (unsigned)m.Gy; dv.o_Ph = (unsigned)m.Ph; dv.o_F = (unsigned)m.F;
  dv.smem_bytes = m.total;
  if (H->ks->tile_dma_smem(H->tv, dv) == 0) return FVS_OK;
  DeviceArena& A = H->arena;
  int *gb0, *sb0, *pb0, *rb0, *cb0, *dptr, *dpos;
  uint16_t *lst, *lsp;
  uint32_t* flr;
  int2* lcf;
  T* dcoef;
  bool up = A.upload(gb0, D.gb0) && A.upload(sb0, D.sb0) && A.upload(pb0, D.pb0) && A.upload(rb0, D.rb0) &&
            A.upload(cb0, D.cb0) && A.upload(lst, D.lst) && A.upload(lsp, D.lsp) && A.upload(flr, D.flr) &&
            A.upload(lcf, D.lcf) && A.upload(dcoef, coef) && A.upload(dptr, D.dptr) && A.upload(dpos, D.dpos);
  dv.gb0 = gb0; dv.sb0 = sb0; dv.pb0 = pb0; dv.rb0 = rb0; dv.cb0 = cb0; dv.lst = lst; dv.lsp = lsp; dv.flr = flr;
  dv.lcf = lcf; dv.coef = dcoef; dv.dptr = dptr; dv.dpos = dpos;
  const size_t gbytes = sizeof(T) * 4 * (size_t)D.gb0.back();
  for (int k = 0; k < H->tv.nbuf && up; k++) up = A.alloc(dv.GB[k], gbytes);
  void* e = nullptr;
  up = up && A.alloc(e, 16);
  dv.err = static_cast<int*>(e);
  if (!up) return H->fail(FVS_ERR_NOMEM, "device allocation or upload of the bulk-copy plan failed");
  ok = true;
  return FVS_OK;
}

// Builds every device array of the handle from the host mesh.
template <typename T>
int build_device(fvs_handle* H) {
  Layout<T> L;
  std::string err;
  const bool fold_w = H->o.precision != FVS_PREC_FP64_STRICT;
  const int fuse = want_fused(H);
  std::vector<int> tile_start;
  int rc;
  if (fuse) {
    // tiles of compact patches (recursive coordinate bisection), reverse
    // Cuthill-McKee order within each tile
    const std::vector<int> order = rcb_tile_order(H->hm, rcm_order(H->hm), tile_cells_setting(), tile_start);
    rc = append_case(L, H->hm, fold_w, 0, err, &order);
  } else {
    rc = append_case(L, H->hm, fold_w, 0, err);
  }
  if (rc) return H->fail(rc, err);
  H->perm = L.perm;
  DevView& d = H->d;
  int* dperm = nullptr;
  if (!upload_layout(H->arena, L, d) || !H->arena.upload(dperm, L.perm))
    return H->fail(FVS_ERR_NOMEM, "device allocation or upload of the mesh failed");
  H->d_perm = dperm;
  H->nblk = (L.nc + 255) / 256;
  void* p;
  if (!alloc_work<T>(H->arena, d, L.nc, L.ne, H->nblk, 4096) || !H->arena.alloc(p, 32 * (size_t)L.nc))
    return H->fail(FVS_ERR_NOMEM, "device allocation of the state failed");
  H->d_stage = static_cast<double*>(p);
  // phi: 0 for first order, 1 without a limiter (src/gradient_limiter.f90:30-40)
  std::vector<T> phi0(L.nc, T(H->o.reconst == FVS_RECON_UPWIND1 ? 0.0 : 1.0));
  if (cudaMemcpy(d.phi, phi0.data(), sizeof(T) * L.nc, cudaMemcpyHostToDevice) != cudaSuccess)
    return H->fail(FVS_ERR_CUDA, "phi upload failed");
  if (fuse && H->ks->tile_stage) {
    TilePlan P;
    rc = build_tiles<T>(H, L, tile_start, H->fused, P);
    if (rc) return rc;
    H->tile_mode = H->fused ? fuse : 0;
    if (H->tile_mode == 3) {
      bool ok = false;
      rc = build_tile_dma_view<T>(H, L, P, ok);
      if (rc) return rc;
      if (!ok) H->tile_mode = 0;
    }
  }
  return FVS_OK;
}

void set_stages(fvs_handle* H) {
  const fvs_options& o = H->o;
  double hr[5], c[5], dts[5];
  rk_coefficients(o, H->dt, hr, c, dts);
  H->stages.clear();
  const int ns = o.rk_nstages;
  for (int k = 1; k <= ns; k++) {
    StageParams sp;
    sp.stage = k; sp.nstages = ns; sp.steady = o.steady; sp.last = (k == ns);
    sp.mode = (ns == 3 && o.ssprk) ? MODE_SSP3 : (o.ssprk ? MODE_SSP42 : MODE_RK);
    sp.h = hr[k]; sp.coef = c[k]; sp.dts = dts[k];
    if (sp.mode == MODE_SSP42) sp.cst = (k == 4) ? 1.0 / 4.0 : 1.0 / 3.0;             // :380-381
    else if (sp.mode == MODE_RK) sp.cst = (k == 3) ? 1.0 : (k == 4 ? 1.0 / 6.0 : 1.0 / 2.0);  // :300-302
    else sp.cst = 1.0;
    if (sp.mode == MODE_SSP3) {
      static const double A[4] = {0, 0.0, 0.75, 1.0 / 3.0}, B[4] = {0, 1.0, 0.25, 2.0 / 3.0};
      sp.a = A[k]; sp.b = B[k];
    }
    sp.set_pairs();
    H->stages.push_back(sp);
  }
  H->d.dt = H->dt;
}

void enqueue_step(fvs_handle* H) {
  const KernelSet& K = *H->ks;
  cudaStream_t s = H->stream;
  K.begin_step(H->d, s);
  if (H->tile_mode == 1) {
    const DevView dv = H->tile_view();
    for (size_t k = 0; k < H->stages.size(); k++) K.tile_stage(dv, H->tv, H->stages[k], (int)k, s);
    return;
  }
  if (H->tile_mode == 3) {
    const DevView dv = H->tile_view();
    for (size_t k = 0; k < H->stages.size(); k++) K.tile_dma_stage(dv, H->tv, H->dv, H->stages[k], (int)k, s);
    return;
  }
  if (H->tile_mode == 2) {
    for (size_t k = 0; k < H->stages.size(); k++) {
      DevView dk = H->tile_view();
      dk.Pv = H->tv.Pbuf[k % H->tv.nbuf];
      K.gradient(dk, s);
      K.tile_fu_stage(dk, H->tv, H->stages[k], (int)k, s);
    }
    return;
  }
  for (const StageParams& sp : H->stages) {
    K.gradient(H->d, s);
    K.flux(H->d, sp.dts, sp.steady && sp.stage == 1, s);
    K.update(H->d, sp, s);
  }
}

int count_launches(const fvs_handle* H) {
  // k_begin_step, then gradient (second order), flux and update per stage,
  // or one fused tile stage; the last stage also reduces the norms
  const int grad = H->d.first_order ? 0 : 1;
  int per_stage = (H->tile_mode == 1 || H->tile_mode == 3) ? 1 : H->tile_mode == 2 ? grad + 1 : grad + 2;
  return 1 + per_stage * (int)H->stages.size();
}

int ensure_graph(fvs_handle* H, int steps_per_graph) {
  if (H->graph && H->graph_steps == steps_per_graph) return FVS_OK;
  if (H->graph) { cudaGraphExecDestroy(H->graph); H->graph = nullptr; }
  cudaGraph_t g;
  cudaError_t e = cudaStreamBeginCapture(H->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return H->cuda_fail(e, "cudaStreamBeginCapture");
  for (int i = 0; i < steps_per_graph; i++) enqueue_step(H);
  e = cudaStreamEndCapture(H->stream, &g);
  if (e != cudaSuccess) return H->cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&H->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return H->cuda_fail(e, "cudaGraphInstantiate");
  H->graph_steps = steps_per_graph;
  return FVS_OK;
}

int check_launch(fvs_handle* H, const char* where) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FVS_OK : H->cuda_fail(e, where);
}

// index-checking handles: FVS_ERR_BOUNDS for a recorded violation (the word
// is cleared, so later calls report later violations); call after the
// stream has been synchronised
int bounds_report(fvs_handle* H) {
  if (!H->bounds) return FVS_OK;
  int w[4];
  cudaError_t e = cudaMemcpy(w, H->d.bounds_err, sizeof w, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return H->cuda_fail(e, "bounds word download");
  if (!w[0]) return FVS_OK;
  static const char* site[] = {"?", "stencil cell", "edge left cell", "edge right cell", "gather slot"};
  cudaMemset(H->d.bounds_err, 0, sizeof w);
  return H->fail(FVS_ERR_BOUNDS, std::string("index-checking kernels: ") + site[(w[1] >= 1 && w[1] <= 4) ? w[1] : 0] +
                                     " index " + std::to_string(w[2]) + " outside its array of " + std::to_string(w[3]));
}

// residual of the current device state at `time` (stage-free): fills d.resid, d.ws
int device_residual(fvs_handle* H, double time) {
  NvtxRange nv("fvs residual (gradient, flux, gather)");
  H->h_small[0] = time;
  cudaError_t e = cudaMemcpyAsync(H->d.tctl + 1, H->h_small, sizeof(double), cudaMemcpyHostToDevice, H->stream);
  if (e != cudaSuccess) return H->cuda_fail(e, "time upload");
  H->ks->cvar2pvar(H->d, H->stream);
  H->ks->gradient(H->d, H->stream);
  H->ks->flux(H->d, 0.0, true, H->stream);
  H->ks->residual_out(H->d, H->stream);
  return check_launch(H, "residual kernels");
}

int ensure_dt(fvs_handle* H, double t1) {
  if (H->dt_ready) return FVS_OK;
  if (H->o.dt_from_cfl && !H->o.steady) {
    int rc = device_residual(H, t1);
    if (rc) return rc;
    std::vector<double> ws(H->hm.nc);
    cudaError_t e = cudaMemcpyAsync(ws.data(), H->d.ws, sizeof(double) * ws.size(), cudaMemcpyDeviceToHost, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e != cudaSuccess) return H->cuda_fail(e, "ws download");
    double dmin = 0.0;
    for (int o = 0; o < H->hm.nc; o++) {
      double dd = H->o.cfl * H->hm.vol[o] / (0.5 * ws[H->perm[o]]);
      if (o == 0 || dd < dmin) dmin = dd;
    }
    H->dt = dmin;
  }
  set_stages(H);
  if (H->graph) { cudaGraphExecDestroy(H->graph); H->graph = nullptr; }
  H->dt_ready = true;
  return FVS_OK;
}

int state_in(fvs_handle* H, const double* cvar) {
  NvtxRange nv("fvs state upload");
  const size_t bytes = 32 * (size_t)H->hm.nc;
  cudaError_t e = cudaMemcpyAsync(H->d_stage, cvar, bytes, cudaMemcpyHostToDevice, H->stream);
  if (e != cudaSuccess) return H->cuda_fail(e, "state upload");
  k_scatter_in<<<(H->hm.nc + 255) / 256, 256, 0, H->stream>>>(H->d_stage, H->d_perm, H->d.U, H->hm.nc);
  H->ks->cvar2pvar(H->d, H->stream);
  H->gb_stale = true;
  return check_launch(H, "state scatter");
}

int state_out(fvs_handle* H, const double* dev, double* host, int width) {
  NvtxRange nv("fvs state download");
  const int nc = H->hm.nc;
  k_gather_out<<<(nc + 255) / 256, 256, 0, H->stream>>>(dev, H->d_perm, H->d_stage, nc, width);
  cudaError_t e = cudaMemcpyAsync(host, H->d_stage, sizeof(double) * width * (size_t)nc, cudaMemcpyDeviceToHost, H->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  return e == cudaSuccess ? FVS_OK : H->cuda_fail(e, "state download");
}

template <typename T>
int typed_out(fvs_handle* H, const void* dev, double* host, int width) {
  const int nc = H->hm.nc;
  k_gather_out_t<T><<<(nc + 255) / 256, 256, 0, H->stream>>>(static_cast<const T*>(dev), H->d_perm, H->d_stage, nc, width);
  cudaError_t e = cudaMemcpyAsync(host, H->d_stage, sizeof(double) * width * (size_t)nc, cudaMemcpyDeviceToHost, H->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  return e == cudaSuccess ? FVS_OK : H->cuda_fail(e, "array download");
}

int validate_options(const fvs_options* o, std::string& err) {
  if (o->flux != 1) { err = "only the Roe flux (1) exists (src/input.f90:269-277)"; return FVS_ERR_INVALID; }
  if (o->grad_method < 1 || o->grad_method > 3) { err = "grad_method must be 1, 2 or 3"; return FVS_ERR_INVALID; }
  if (o->limiter < 0 || o->limiter > 3) { err = "limiter must be 0..3"; return FVS_ERR_INVALID; }
  if (o->reconst < 1 || o->reconst > 3) { err = "reconst must be 1..3"; return FVS_ERR_INVALID; }
  if (o->limiter != FVS_LIM_NONE && o->grad_method != FVS_GRAD_LSQ && o->reconst != FVS_RECON_UPWIND1) {
    err = "the limiter reads the LSQ stencil (src/gradient_limiter.f90:54): use LSQ gradients";
    return FVS_ERR_INVALID;
  }
  const int ns = o->rk_nstages;
  bool ok = (ns == 4 && o->rk_order >= 1 && o->rk_order <= 4 && (!o->ssprk || o->rk_order == 2)) || (ns == 3 && o->ssprk);
  if (!ok) { err = "RK coefficients exist for 4 stages (SSP: order 2) and the SSP-RK3 extension only"; return FVS_ERR_INVALID; }
  if (o->precision < 0 || o->precision > 3) { err = "precision must be 0, 1, 2 or 3"; return FVS_ERR_INVALID; }
  if (!(o->gamma > 1.0)) { err = "gamma must be > 1"; return FVS_ERR_INVALID; }
  return FVS_OK;
}

}  // namespace

// ===========================================================================
// C-ABI
// ===========================================================================
extern "C" {

int fvs_options_default(fvs_options* o) {
  if (!o) return FVS_ERR_INVALID;
  std::memset(o, 0, sizeof(*o));
  o->gamma = 1.4; o->mach_inf = 0.5; o->aoa_inf_deg = 0.0; o->dt = 0.01; o->cfl = 1.0;
  o->steady = 0; o->vortex = 0; o->ntstart = 1;
  o->grad_method = FVS_GRAD_LSQ; o->lsq_stencil = FVS_LSQ_FN; o->lsq_pow = 0.0;
  o->limiter = FVS_LIM_NONE; o->reconst = FVS_RECON_UPWIND2; o->umuscl = 0.0; o->flux = 1;
  o->rk_nstages = 4; o->rk_order = 4; o->ssprk = 0;
  o->vortex_x = 5.0; o->vortex_y = 5.0; o->vortex_kappa = 1.0;
  o->vortex_inf[0] = 1.0; o->vortex_inf[1] = 0.2; o->vortex_inf[2] = 0.0; o->vortex_inf[3] = 1.0;
  o->dt_from_cfl = 0; o->precision = FVS_PREC_FP64; o->diverge_factor = 0.0;
  return FVS_OK;
}

int fvs_create(const fvs_mesh* mesh, const fvs_options* opt, fvs_handle** out) {
  if (!out) return FVS_ERR_INVALID;
  *out = nullptr;
  if (!mesh || !opt || mesh->nnodes <= 0 || mesh->ncells_tri < 0 || mesh->ncells_quad < 0 ||
      mesh->ncells_tri + mesh->ncells_quad <= 0 || !mesh->node_xy || (mesh->ncells_tri && !mesh->tri_nodes) ||
      (mesh->ncells_quad && !mesh->quad_nodes) || mesh->nbndries < 0 ||
      (mesh->nbndries && (!mesh->bndry_ncells || !mesh->bndry_type || !mesh->bndry_cells))) {
    g_create_error = "invalid mesh description";
    return FVS_ERR_INVALID;
  }
  std::string err;
  int rc = validate_options(opt, err);
  if (rc) { g_create_error = err; return rc; }
  std::unique_ptr<fvs_handle> H(new fvs_handle());
  H->o = *opt;
  if (H->o.reconst != FVS_RECON_UMUSCL) H->o.umuscl = 0.0;  // src/input.f90:250,254
  {
    NvtxRange nv("fvs host setup (grid_data, stencils)");
    rc = build_host_mesh(mesh, &H->o, H->hm, err);
  }
  if (rc) { g_create_error = err; return rc; }
  // free stream, src/data_solution.f90:55-63
  const double aoa = H->o.aoa_inf_deg * 3.141592653589793238462643383279502884 / 180.0;
  H->pvar_inf[0] = 1.0;
  H->pvar_inf[1] = H->o.mach_inf * std::cos(aoa);
  H->pvar_inf[2] = H->o.mach_inf * std::sin(aoa);
  H->pvar_inf[3] = 1.0 / H->o.gamma;
  H->mixed = H->o.precision == FVS_PREC_MIXED;
  H->df = H->o.precision == FVS_PREC_FP64_DF;
  H->ks = H->o.precision == FVS_PREC_FP64_STRICT ? &kernels_fp64_strict()
          : H->mixed ? &kernels_mixed() : H->df ? &kernels_fp64_df() : &kernels_fp64_fast();
  {
    const char* e = std::getenv("FVS2D_BOUNDS");
    H->bounds = H->o.precision == FVS_PREC_FP64 && e && e[0] == '1' && e[1] == 0;
    if (H->bounds) H->ks = &kernels_fp64_bounds();
  }
  cudaError_t e = cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { g_create_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e); return FVS_ERR_CUDA; }
  if (cudaMallocHost(&H->h_small, 64) != cudaSuccess) { g_create_error = "pinned allocation failed"; return FVS_ERR_NOMEM; }
  cudaEventCreate(&H->ev0);
  cudaEventCreate(&H->ev1);
  DevView& d = H->d;
  d.gamma = H->o.gamma;
  d.khalf = H->o.umuscl / 2.0;
  d.nkhalf = -H->o.umuscl / 2.0;
  d.omk = 1.0 - H->o.umuscl;
  d.cfl = H->o.cfl;
  d.gm1 = H->o.gamma - 1.0;
  d.igm1 = 1.0 / (H->o.gamma - 1.0);
  d.ggm1 = H->o.gamma / (H->o.gamma - 1.0);
  set_fp32_constants(d);
  d.limiter = H->o.limiter;
  d.grad_method = H->o.grad_method;
  d.first_order = H->o.reconst == FVS_RECON_UPWIND1;
  d.vortex = H->o.vortex;
  d.vx = H->o.vortex_x; d.vy = H->o.vortex_y; d.vkappa = H->o.vortex_kappa;
  for (int k = 0; k < 4; k++) { d.vinf[k] = H->o.vortex_inf[k]; d.pinf[k] = H->pvar_inf[k]; }
  mms_constants(d.mc);
  {
    NvtxRange nv("fvs device layout and upload");
    rc = H->mixed ? build_device<float>(H.get()) : H->df ? build_device<df64>(H.get()) : build_device<double>(H.get());
  }
  if (rc) { g_create_error = H->err; return rc; }
  if (H->ks->update_wave) {
    const int ns = H->o.rk_nstages;
    d.upd_grid = H->ks->update_wave((ns == 3 && H->o.ssprk) ? MODE_SSP3 : (H->o.ssprk ? MODE_SSP42 : MODE_RK));
  }
  if (H->bounds) {
    void* p = nullptr;
    if (!H->arena.alloc(p, 4 * sizeof(int))) { g_create_error = "bounds word allocation failed"; return FVS_ERR_NOMEM; }
    d.bounds_err = static_cast<int*>(p);
  }
  H->dt = H->o.dt;
  // steady runs start from dt_local = dt (src/runge_kutta.f90:73-76)
  {
    std::vector<double> dtl(H->hm.nc, H->o.dt);
    cudaMemcpy(d.dtl, dtl.data(), 8 * dtl.size(), cudaMemcpyHostToDevice);
  }
  if (!(H->o.dt_from_cfl && !H->o.steady)) {
    set_stages(H.get());
    H->dt_ready = true;
  } else {
    set_stages(H.get());
  }
  H->launches_per_step = count_launches(H.get());
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { g_create_error = std::string("setup: ") + cudaGetErrorString(e); return FVS_ERR_CUDA; }
  *out = H.release();
  return FVS_OK;
}

int fvs_create_host(const fvs_mesh* mesh, const fvs_options* opt, fvs_handle** out) {
  if (!out) return FVS_ERR_INVALID;
  *out = nullptr;
  if (!mesh || !opt || mesh->nnodes <= 0 || mesh->ncells_tri < 0 || mesh->ncells_quad < 0 ||
      mesh->ncells_tri + mesh->ncells_quad <= 0 || !mesh->node_xy || (mesh->ncells_tri && !mesh->tri_nodes) ||
      (mesh->ncells_quad && !mesh->quad_nodes) || mesh->nbndries < 0 ||
      (mesh->nbndries && (!mesh->bndry_ncells || !mesh->bndry_type || !mesh->bndry_cells))) {
    g_create_error = "invalid mesh description";
    return FVS_ERR_INVALID;
  }
  std::string err;
  int rc = validate_options(opt, err);
  if (rc) { g_create_error = err; return rc; }
  std::unique_ptr<fvs_handle> H(new fvs_handle());
  H->o = *opt;
  if (H->o.reconst != FVS_RECON_UMUSCL) H->o.umuscl = 0.0;
  rc = build_host_mesh(mesh, &H->o, H->hm, err);
  if (rc) { g_create_error = err; return rc; }
  H->host_only = true;
  H->dt = H->o.dt;
  *out = H.release();
  return FVS_OK;
}

void fvs_destroy(fvs_handle* h) { delete h; }

const char* fvs_last_error(const fvs_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int fvs_get_sizes(const fvs_handle* h, fvs_sizes* s) {
  if (!h || !s) return FVS_ERR_INVALID;
  const HostMesh& m = h->hm;
  std::memset(s, 0, sizeof(*s));
  s->nnodes = m.nnodes; s->ncells = m.nc; s->ncells_tri = m.ntri; s->ncells_quad = m.nquad;
  s->nedges = m.ne; s->nedges_intr = (int)m.edge_intr.size(); s->nedges_bndr = (int)m.edge_bndr.size();
  s->ncells_intr = (int)m.cell_intr.size(); s->ncells_bndr = (int)m.cell_bndr.size(); s->nbndries = m.nb;
  s->stencil_len = (int)m.st_cell.size(); s->nstages = h->o.rk_nstages;
  s->heff1 = m.heff1; s->heff2 = m.heff2; s->vol_sum = m.vol1; s->vol_green = m.vol2; s->dt = h->dt;
  return FVS_OK;
}

int fvs_export_size(const fvs_handle* h, const char* name, int64_t* nbytes) {
  if (!h || !name || !nbytes) return FVS_ERR_INVALID;
  return export_array(h->hm, name, nullptr, nbytes);
}

int fvs_export(const fvs_handle* h, const char* name, void* dst, int64_t nbytes) {
  if (!h || !name || !dst) return FVS_ERR_INVALID;
  return export_array(h->hm, name, dst, &nbytes);
}

int fvs_init_state(fvs_handle* h) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h) return FVS_ERR_INVALID;
  // initialize_solution, src/initialize.f90:19-90 (ntstart <= 1)
  if (h->o.ntstart > 1)
    return h->fail(FVS_ERR_INVALID, "ntstart > 1 restarts from continuation files (src/initialize.f90:56-77): "
                                    "read them on the host and call fvs_set_state");
  const int nc = h->hm.nc;
  std::vector<double> cv(4 * (size_t)nc);
  const double g = h->o.gamma, t0 = double(h->o.ntstart - 1) * h->o.dt;
  for (int ic = 0; ic < nc; ic++) {
    double pv[4];
    if (h->o.ntstart < 1) std::memcpy(pv, &h->hm.mms_sol[4 * ic], sizeof pv);
    else if (h->o.vortex) vortex_state(h->o, t0, h->hm.xc[ic], h->hm.yc[ic], pv);
    else std::memcpy(pv, h->pvar_inf, sizeof pv);
    double* u = &cv[4 * ic];
    u[0] = pv[0];
    u[1] = pv[0] * pv[1];
    u[2] = pv[0] * pv[2];
    u[3] = pv[3] / (g - 1.0) + 0.5 * pv[0] * (pv[1] * pv[1] + pv[2] * pv[2]);
  }
  return fvs_set_state(h, cv.data());
}

int fvs_set_state(fvs_handle* h, const double* cvar) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h || !cvar) return FVS_ERR_INVALID;
  int rc = state_in(h, cvar);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  return e == cudaSuccess ? FVS_OK : h->cuda_fail(e, "set_state");
}

int fvs_get_state(fvs_handle* h, double* cvar) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h || !cvar) return FVS_ERR_INVALID;
  return state_out(h, h->d.U, cvar, 4);
}

int fvs_residual(fvs_handle* h, double time, double* resid, double* ws_nrml) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h) return FVS_ERR_INVALID;
  int rc = device_residual(h, time);
  if (rc) return rc;
  if (resid && (rc = state_out(h, h->d.resid, resid, 4))) return rc;
  if (ws_nrml && (rc = state_out(h, h->d.ws, ws_nrml, 1))) return rc;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "residual");
  return bounds_report(h);
}

int fvs_get_gradient(fvs_handle* h, double* grad, double* phi) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h) return FVS_ERR_INVALID;
  const int nc = h->hm.nc;
  int rc = FVS_OK;
  if (grad) {
    if (h->mixed) {
      if ((rc = typed_out<float>(h, h->d.Gx, grad, 4))) return rc;
      if ((rc = typed_out<float>(h, h->d.Gy, grad + 4 * (size_t)nc, 4))) return rc;
    } else if (h->df) {
      if ((rc = typed_out<df64>(h, h->d.Gx, grad, 4))) return rc;
      if ((rc = typed_out<df64>(h, h->d.Gy, grad + 4 * (size_t)nc, 4))) return rc;
    } else {
      if ((rc = typed_out<double>(h, h->d.Gx, grad, 4))) return rc;
      if ((rc = typed_out<double>(h, h->d.Gy, grad + 4 * (size_t)nc, 4))) return rc;
    }
  }
  if (phi)
    rc = h->mixed ? typed_out<float>(h, h->d.phi, phi, 1)
         : h->df  ? typed_out<df64>(h, h->d.phi, phi, 1)
                  : typed_out<double>(h, h->d.phi, phi, 1);
  return rc;
}

// bulk-copy handles: the gather buffer the first stage reads, from the
// current primitives, when the state changed since the last step
int refill_gather(fvs_handle* h) {
  if (h->tile_mode != 3 || !h->gb_stale) return FVS_OK;
  cudaError_t e = h->ks->tile_dma_fill(h->d, h->dv, 0, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "gather buffer fill");
  h->gb_stale = false;
  return FVS_OK;
}

// bulk-copy handles: FVS_ERR_TIMEOUT when a block's wait for its copies ran
// out (the word is cleared); call after the stream has been synchronised
int dma_report(fvs_handle* h) {
  if (h->tile_mode != 3) return FVS_OK;
  int w = 0;
  cudaError_t e = cudaMemcpy(&w, h->dv.err, sizeof w, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return h->cuda_fail(e, "bulk-copy error word download");
  if (!w) return FVS_OK;
  cudaMemset(h->dv.err, 0, sizeof w);
  h->gb_stale = true;
  return h->fail(FVS_ERR_TIMEOUT, "a tile block's wait for its bulk copies ran out");
}

static int run_steps(fvs_handle* h, double t1, int nsteps, double* resnorm, float* ms) {
  NvtxRange nv("fvs time integration (graph replays)");
  int rc = ensure_dt(h, t1);
  if (rc) return rc;
  if ((rc = ensure_graph(h, 1))) return rc;
  if ((rc = refill_gather(h))) return rc;
  // control words: t1, steps done = 0
  h->h_small[0] = t1;
  reinterpret_cast<int*>(h->h_small + 1)[0] = 0;  // steps done
  reinterpret_cast<int*>(h->h_small + 1)[1] = 0;  // blocks done in the current last stage
  cudaError_t e = cudaMemcpyAsync(h->d.tctl, h->h_small, sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h->d.stepctl, h->h_small + 1, 2 * sizeof(int), cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "step control upload");
  if (ms) cudaEventRecord(h->ev0, h->stream);
  const int cap = h->d.norm_cap;
  int done = 0;
  while (done < nsteps) {
    int chunk = std::min(cap, nsteps - done);
    for (int i = 0; i < chunk; i++) {
      e = cudaGraphLaunch(h->graph, h->stream);
      if (e != cudaSuccess) return h->cuda_fail(e, "cudaGraphLaunch");
    }
    if (resnorm) {
      e = cudaMemcpyAsync(resnorm + 4 * (size_t)done, h->d.norms, 32 * (size_t)chunk, cudaMemcpyDeviceToHost, h->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
      if (e != cudaSuccess) return h->cuda_fail(e, "norm download");
    }
    done += chunk;
  }
  if (ms) {
    cudaEventRecord(h->ev1, h->stream);
    e = cudaEventSynchronize(h->ev1);
    if (e != cudaSuccess) return h->cuda_fail(e, "event sync");
    cudaEventElapsedTime(ms, h->ev0, h->ev1);
  }
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "time integration");
  if ((rc = bounds_report(h))) return rc;
  if ((rc = dma_report(h))) return rc;
  if (resnorm) {
    for (size_t i = 0; i < 4 * (size_t)nsteps; i++)
      if (!std::isfinite(resnorm[i])) return h->fail(FVS_ERR_NONFINITE, "residual norm is not finite at step " + std::to_string(i / 4 + 1));
  } else {
    // no norms requested (device-resident stepping): the last step's norms
    // from the device ring; a non-finite state stays non-finite, so the last
    // step shows whether any step went bad
    double last[4];
    e = cudaMemcpy(last, h->d.norms + 4 * (size_t)((nsteps - 1) % cap), sizeof last, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cuda_fail(e, "norm download");
    for (int k = 0; k < 4; k++)
      if (!std::isfinite(last[k]))
        return h->fail(FVS_ERR_NONFINITE, "residual norm is not finite after step " + std::to_string(nsteps));
  }
  return FVS_OK;
}

int fvs_time_integration(fvs_handle* h, double t1, int32_t nsteps, double* resnorm) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h || nsteps < 0) return FVS_ERR_INVALID;
  if (nsteps == 0) return FVS_OK;
  return run_steps(h, t1, nsteps, resnorm, nullptr);
}

int fvs_run_to_drop(fvs_handle* h, double t1, int32_t max_steps, double drop, int32_t check_every, int32_t* steps_done,
                    double* resnorm) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h || max_steps <= 0 || check_every <= 0) return FVS_ERR_INVALID;
  std::vector<double> buf(4 * (size_t)max_steps);
  double first = 0;
  int done = 0;
  int rc = FVS_OK;
  while (done < max_steps) {
    int n = std::min(check_every, max_steps - done);
    double tstart = t1 + double(done) * h->dt;
    rc = run_steps(h, tstart, n, buf.data() + 4 * (size_t)done, nullptr);
    if (done == 0 && rc == FVS_OK) first = buf[0];
    done += n;
    if (rc) break;
    double last = buf[4 * (size_t)(done - 1)];
    if (h->o.diverge_factor > 0 && last > h->o.diverge_factor * first) {
      rc = h->fail(FVS_ERR_DIVERGED, "residual grew past diverge_factor");
      break;
    }
    bool hit = false;
    int at = done;
    for (int i = done - n; i < done; i++)
      if (buf[4 * (size_t)i] <= drop * first) { hit = true; at = i + 1; break; }
    if (hit) { done = at; break; }
  }
  if (steps_done) *steps_done = done;
  if (resnorm) std::memcpy(resnorm, buf.data(), 32 * (size_t)done);
  return rc;
}

int fvs_vortex_error(fvs_handle* h, double time, double* e) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h || !e) return FVS_ERR_INVALID;
  const HostMesh& m = h->hm;
  std::vector<double> cv(4 * (size_t)m.nc);
  int rc = fvs_get_state(h, cv.data());
  if (rc) return rc;
  // error_isentropic_vortex, src/mms.f90:271-365
  const double g = h->o.gamma;
  double mx[4] = {0, 0, 0, 0}, l1[4] = {0, 0, 0, 0}, l2[4] = {0, 0, 0, 0}, L2 = 0;
  for (int ic : m.cell_intr) {
    double pv[4], ex[4], d[4];
    vortex_state(h->o, time, m.xc[ic], m.yc[ic], pv);
    ex[0] = pv[0]; ex[1] = pv[0] * pv[1]; ex[2] = pv[0] * pv[2];
    ex[3] = pv[3] / (g - 1.0) + 0.5 * ex[0] * (pv[1] * pv[1] + pv[2] * pv[2]);
    for (int v = 0; v < 4; v++) {
      d[v] = std::fabs(cv[4 * ic + v] - ex[v]);
      if (d[v] > mx[v]) mx[v] = d[v];
      l1[v] = l1[v] + d[v];
      l2[v] = l2[v] + d[v] * d[v];
    }
    L2 = L2 + d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + d[3] * d[3];
  }
  const double n = double(m.cell_intr.size());
  for (int v = 0; v < 4; v++) { e[3 * v] = mx[v]; e[3 * v + 1] = l1[v] / n; e[3 * v + 2] = std::sqrt(l2[v] / n); }
  e[12] = std::sqrt(L2 / n);
  return FVS_OK;
}

int fvs_wall_loads(fvs_handle* h, int32_t ib, double* edge_out, double* loads) {
  NvtxRange nv("fvs wall loads");
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h || !loads) return FVS_ERR_INVALID;
  const HostMesh& m = h->hm;
  if (ib < 1 || ib > m.nb) return h->fail(FVS_ERR_INVALID, "boundary index out of range");
  if (m.b_type[ib - 1] != FVS_BC_SLIP_WALL) return h->fail(FVS_ERR_INVALID, "wall loads need a slip_wall boundary");
  const int n = m.b_eptr[ib] - m.b_eptr[ib - 1];
  if (n <= 0) return h->fail(FVS_ERR_INVALID, "boundary has no edges");
  if (m.st_ptr.empty()) return h->fail(FVS_ERR_INVALID, "no gradient operator");
  const size_t need = 4 * (size_t)n + 8;
  if (need > h->wall_cap) {
    if (h->d_wall) cudaFree(h->d_wall);
    h->d_wall = nullptr;
    h->wall_cap = 0;
    cudaError_t e = cudaMalloc(&h->d_wall, sizeof(double) * need);
    if (e != cudaSuccess) return h->cuda_fail(e, "wall-load scratch");
    h->wall_cap = need;
  }
  // gradient_cellcntr_1var (src/gradient.f90:75-96): the configured gradient
  // without limiter, of the current state, also for first-order runs
  DevView g = h->d;
  g.first_order = 0;
  g.limiter = FVS_LIM_NONE;
  h->ks->cvar2pvar(h->d, h->stream);
  h->ks->gradient(g, h->stream);
  const double mach = h->o.mach_inf, c2 = 2.0 / (mach * mach);
  const int g0 = h->d.nint + m.b_eptr[ib - 1];
  double* sums = h->d_wall + 4 * (size_t)n;
  if (h->mixed) k_wall_loads<float><<<1, 256, 0, h->stream>>>(h->d, g0, n, c2, h->pvar_inf[3], h->d_wall, sums);
  else if (h->df) k_wall_loads<df64><<<1, 256, 0, h->stream>>>(h->d, g0, n, c2, h->pvar_inf[3], h->d_wall, sums);
  else k_wall_loads<double><<<1, 256, 0, h->stream>>>(h->d, g0, n, c2, h->pvar_inf[3], h->d_wall, sums);
  int rc = check_launch(h, "wall-load kernels");
  if (rc) return rc;
  double s[7];
  cudaError_t e = cudaMemcpyAsync(s, sums, sizeof s, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && edge_out)
    e = cudaMemcpyAsync(edge_out, h->d_wall, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "wall-load download");
  const double un_l2 = std::sqrt(s[5] / double(n)), un_l1 = s[6] / double(n);
  // cosd / sind of the angle of attack in degrees
  const double a = h->o.aoa_inf_deg * 3.141592653589793238462643383279502884 / 180.0;
  const double ca = std::cos(a), sa = std::sin(a);
  loads[0] = s[0] * ca - s[1] * sa;
  loads[1] = s[0] * sa + s[1] * ca;
  loads[2] = s[2] * ca - s[3] * sa;
  loads[3] = s[2] * sa + s[3] * ca;
  loads[4] = s[4]; loads[5] = un_l2; loads[6] = un_l1;
  loads[7] = s[0]; loads[8] = s[1]; loads[9] = s[2]; loads[10] = s[3];
  return FVS_OK;
}

int fvs_mms_source(fvs_handle* h, double* src) {
  if (!h || !src) return FVS_ERR_INVALID;
  std::memcpy(src, h->hm.mms_src.data(), sizeof(double) * h->hm.mms_src.size());
  return FVS_OK;
}

int fvs_steps_device(fvs_handle* h, int32_t nsteps, float* ms) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h || nsteps <= 0) return FVS_ERR_INVALID;
  return run_steps(h, 0.0, nsteps, nullptr, ms);
}

int fvs_profile_step(fvs_handle* h, int32_t cap, int32_t* n, char* names, float* ms) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h || !n || !names || !ms) return FVS_ERR_INVALID;
  int rc = ensure_dt(h, 0.0);
  if (rc) return rc;
  const KernelSet& K = *h->ks;
  cudaStream_t s = h->stream;
  std::vector<cudaEvent_t> ev;
  std::vector<std::string> nm;
  auto mark = [&](const std::string& label) {
    cudaEvent_t x;
    cudaEventCreate(&x);
    cudaEventRecord(x, s);
    ev.push_back(x);
    nm.push_back(label);
  };
  if ((rc = refill_gather(h))) return rc;
  mark("start");
  K.begin_step(h->d, s);
  if (h->tile_mode == 1) {
    const DevView dv = h->tile_view();
    for (size_t k = 0; k < h->stages.size(); k++) {
      K.tile_stage(dv, h->tv, h->stages[k], (int)k, s);
      mark("tile_stage");
    }
  } else if (h->tile_mode == 3) {
    const DevView dv = h->tile_view();
    for (size_t k = 0; k < h->stages.size(); k++) {
      K.tile_dma_stage(dv, h->tv, h->dv, h->stages[k], (int)k, s);
      mark("tile_dma_stage");
    }
  } else if (h->tile_mode == 2) {
    for (size_t k = 0; k < h->stages.size(); k++) {
      DevView dk = h->tile_view();
      dk.Pv = h->tv.Pbuf[k % h->tv.nbuf];
      K.gradient(dk, s);
      if (!dk.first_order) mark("gradient");
      K.tile_fu_stage(dk, h->tv, h->stages[k], (int)k, s);
      mark("tile_flux_update");
    }
  } else {
    for (const StageParams& sp : h->stages) {
      K.gradient(h->d, s);
      mark("gradient");
      K.flux(h->d, sp.dts, sp.steady && sp.stage == 1, s);
      mark("flux");
      K.update(h->d, sp, s);
      mark("update");
    }
  }
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return h->cuda_fail(e, "profile step");
  int m = 0;
  for (size_t i = 1; i < ev.size() && m < cap; i++, m++) {
    std::snprintf(names + 32 * m, 32, "%s", nm[i].c_str());
    cudaEventElapsedTime(&ms[m], ev[i - 1], ev[i]);
  }
  for (cudaEvent_t x : ev) cudaEventDestroy(x);
  *n = m;
  return FVS_OK;
}

int fvs_launches_per_step(const fvs_handle* h, int32_t* n) {
  if (!h || !n) return FVS_ERR_INVALID;
  *n = h->launches_per_step;
  return FVS_OK;
}

int fvs_debug_set_gather(fvs_handle* h, int32_t cell, int32_t entry, int32_t value) {
  if (!h) return FVS_ERR_INVALID;
  if (!h->bounds) return h->fail(FVS_ERR_INVALID, "fvs_debug_set_gather needs an index-checking handle (FVS2D_BOUNDS=1)");
  if (cell < 1 || cell > h->hm.nc || entry < 0 || entry > 3) return h->fail(FVS_ERR_INVALID, "cell or entry out of range");
  int* p = reinterpret_cast<int*>(const_cast<int4*>(h->d.cflist) + h->perm[cell - 1]) + entry;
  // the kernels read the list from memory at every launch, so a captured
  // step graph sees the new entry
  cudaError_t e = cudaMemcpy(p, &value, sizeof value, cudaMemcpyHostToDevice);
  return e == cudaSuccess ? FVS_OK : h->cuda_fail(e, "gather entry upload");
}

int fvs_tile_plan_info(const fvs_mesh* mesh, const fvs_options* opt, int32_t* info) {
  if (!mesh || !opt || !info) return FVS_ERR_INVALID;
  std::string err;
  int rc = validate_options(opt, err);
  if (rc) { g_create_error = err; return rc; }
  fvs_options o = *opt;
  if (o.reconst != FVS_RECON_UMUSCL) o.umuscl = 0.0;
  HostMesh hm;
  rc = build_host_mesh(mesh, &o, hm, err);
  if (rc) { g_create_error = err; return rc; }
  std::vector<int> tile_start;
  const std::vector<int> order = rcb_tile_order(hm, rcm_order(hm), tile_cells_setting(), tile_start);
  Layout<float> L;
  rc = append_case(L, hm, true, 0, err, &order);
  if (rc) { g_create_error = err; return rc; }
  TilePlan P;
  rc = build_tile_plan(tile_start, L.ecell, L.cf, L.st_ptr, L.st_cell, P, err);
  if (rc) { g_create_error = err; return rc; }
  P.tile_cells = tile_cells_setting();
  const std::string bad = check_tile_plan(P, L.nc, L.ne, L.ecell, L.cf, L.st_ptr);
  info[0] = P.ntiles; info[1] = P.lmax; info[2] = P.gmax; info[3] = P.fmax; info[4] = bad.empty() ? 1 : 0;
  info[5] = (int32_t)P.halo.size();
  if (!bad.empty()) { g_create_error = bad; return FVS_ERR_MESH; }
  // the bulk-copy form's segments (mixed: 4-byte values)
  TileDma D;
  build_tile_dma(P, L.st_ptr, L.nc, D);
  const std::string bad2 = check_tile_dma(P, D, 4, L.nc, L.st_cell.size());
  const DmaSmem m = dma_smem(4, P.lmax, P.gmax, P.fmax, D.smax, D.pmax, D.rmax, D.qmax);
  info[6] = (int32_t)m.total; info[7] = bad2.empty() ? 1 : 0;
  if (!bad2.empty()) { g_create_error = "bulk-copy plan: " + bad2; return FVS_ERR_MESH; }
  return FVS_OK;
}

int fvs_check_fp64_math(const double* x, int32_t n, double* out) {
  if (!x || !out || n <= 0) return FVS_ERR_INVALID;
  double* d = nullptr;
  const size_t nb = sizeof(double) * (size_t)n;
  if (cudaMalloc(&d, 6 * nb) != cudaSuccess) return FVS_ERR_NOMEM;
  cudaError_t e = cudaMemcpy(d, x, nb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_check_fp64_math<<<(n + 255) / 256, 256>>>(d, n, d + n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d + n, 5 * nb, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? FVS_OK : FVS_ERR_CUDA;
}

int fvs_device_state(fvs_handle* h, void** dptr) {
  if (h && h->host_only) return h->fail(FVS_ERR_INVALID, "host-only handle (fvs_create_host) has no device state");
  if (!h || !dptr) return FVS_ERR_INVALID;
  *dptr = h->d.U;
  return FVS_OK;
}

}  // extern "C"
