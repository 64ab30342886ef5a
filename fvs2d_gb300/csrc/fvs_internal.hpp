// fvs_internal.hpp — structures shared by the host setup (fvs_setup.cpp),
// the C-ABI (fvs_capi.cpp) and the device kernels (fvs_kernels.cuh).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/fvs2d.h"

namespace fvs {

// NVTX range over a host-side phase (setup, upload, stepping, download):
// visible in a profiler's timeline, free when no tool is attached
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// ---------------------------------------------------------------------------
// Host mesh in the reference's numbering, 0-based, "-1" where the reference
// stores 0 (no neighbour / boundary).  Built by build_host_mesh() so that
// every connectivity and geometry array is bit-identical to grid_data
// (src/grid_procs.f90:170-794) and the gradient setups.
// ---------------------------------------------------------------------------
struct HostMesh {
  int nnodes = 0, ntri = 0, nquad = 0, nc = 0;
  double Lx = 0, Ly = 0, xmin = 0, ymin = 0;
  std::vector<double> xn, yn;
  std::vector<int8_t> nvrt;
  std::vector<int> cnode;     // [nc][4]
  std::vector<int> nghbr;     // [nc][4]
  std::vector<int> nghbre;    // [nc][4]
  std::vector<int> cedge;     // [nc][4]
  std::vector<double> nrmlsign;  // [nc][4]
  std::vector<double> xc, yc, vol;
  std::vector<int> nd_ptr, nd_cell;  // node -> cells, in ascending cell order
  int ne = 0;
  std::vector<int> en1, en2, ec1, ec2;
  std::vector<double> ex, ey, ea, enx, eny, etx, ety;
  std::vector<int> cell_intr, cell_bndr, edge_intr, edge_bndr, bedge_cell;
  int nb = 0;
  std::vector<int> b_type, b_cptr, b_cell, b_eptr, b_edge;  // CSR per boundary
  double heff1 = 0, heff2 = 0, vol1 = 0, vol2 = 0;
  // gradient operator (reference order)
  int grad_method = 0;
  std::vector<int> st_ptr, st_cell;  // CSR
  std::vector<double> st_coef;       // LSQ/GGCB: [len][2]; GGNB: [len]
  std::vector<double> st_w;          // LSQ weights
  std::vector<int8_t> st_node;       // GGNB: local node of each entry
  std::vector<double> coef0;         // GGCB/GGNB [nc][2]
  std::vector<double> coefedg;       // GGNB [nc][4][2]
  std::vector<double> eps2;          // limiter eps^2 per cell
  std::vector<double> mms_sol, mms_src;  // [nc][4]
};

// options derived once per handle
struct Scheme {
  fvs_options o;
  double pvar_inf[4];
  double mc[16];  // MMS constants
  double h_rk[5], rk_coef[5], dts[5];
};

int build_host_mesh(const fvs_mesh* m, const fvs_options* o, HostMesh& hm, std::string& err);
void mms_constants(double* mc);
void mms_euler2d(const double* mc, double gamma, double xc, double yc, double* sol, double* rhs);
void vortex_state(const fvs_options& o, double t, double x, double y, double* pv);
void rk_coefficients(const fvs_options& o, double dt, double* h_rk, double* rk_coef, double* dts);
int export_array(const HostMesh& hm, const char* name, void* dst, int64_t* nbytes);

// ---------------------------------------------------------------------------
// Device view.  Arrays are in device order (cells renumbered by reverse
// Cuthill-McKee, interior edges sorted by their first device cell, boundary
// edges after them in the reference's processing order).  "T" arrays hold the
// compute type of the path: double for FP64, float for MIXED.
// ---------------------------------------------------------------------------
enum StageMode : int {
  MODE_RK = 0,        // time_integ_RK / time_integ_RK_steady
  MODE_SSP42 = 1,     // time_integ_SSPRK / time_integ_SSPRK_steady
  MODE_SSP3 = 2,      // SSP-RK3 extension (Shu-Osher)
};

struct DevView {
  int nc = 0, nint = 0, nedge = 0, nblk_red = 0;
  // cells
  double* U = nullptr;      // [nc] x 4 conservative state
  double* U0 = nullptr;     // [nc] x 4 state at the start of the step
  double* F = nullptr;      // [nc] x 4 RK accumulator (fcvar)
  void* Pv = nullptr;       // [nc] x 4 primitives (T)
  void* Pv2 = nullptr;      // [nc] x 4 second primitive buffer of the fused first-order
                            // stage (mixed batches; null: separate flux and update phases)
  void* Gx = nullptr;       // [nc] x 4 d/dx primitives (T)
  void* Gy = nullptr;       // [nc] x 4 d/dy primitives (T)
  void* phi = nullptr;      // [nc] limiter (T)
  double* ws = nullptr;     // [nc] sum 0.5(|un|+a)A
  double* dtl = nullptr;    // [nc] local time step
  double* resid = nullptr;  // [nc] x 4 residual (standalone residual only)
  const double* vol = nullptr;
  const double* rvol = nullptr;  // 1/vol (MIXED only)
  const void* eps2 = nullptr;    // [nc] (T)
  const int4* cflist = nullptr;  // [nc] signed flux slots, reference summation order
  const void* cpos = nullptr;    // [nc][4] x 2 face-centre offsets (T) for the limiter
  const int8_t* nvrt = nullptr;
  const int* st_ptr = nullptr;
  const int* st_cell = nullptr;
  const void* st_coef = nullptr;  // LSQ/GGCB [len] x 2 (T); GGNB [len] (T)
  const void* st_w = nullptr;     // LSQ [len] (T)
  const int8_t* st_node = nullptr;
  const void* coef0 = nullptr;    // [nc] x 2 (T)
  const void* coefedg = nullptr;  // [nc][4] x 2 (T)
  // edges
  const int2* ecell = nullptr;    // (L,R) device cell ids; R = -1 on boundary edges
  const void* enrm = nullptr;     // [nedge] x 2 unit normal (T)
  const void* earea = nullptr;    // [nedge] (T)
  const void* edL = nullptr;      // [nedge] x 2 xf - xcL (T)
  const void* edR = nullptr;      // [nint] x 2 xf - xcR (T)
  const int* ebtype = nullptr;    // [nedge] boundary record: type | case << 4 (boundary slots only)
  const void* exy = nullptr;      // [nedge] x 2 face centre (T) (boundary slots only)
  const double* case_pinf = nullptr;  // [ncases][4] free stream per case (batched meshes)
  void* eflux = nullptr;          // [nedge] x 4 flux*area (T)
  void* ews = nullptr;            // [nedge] ws_max*area (T)
  // reduction and step control
  double* partials = nullptr;     // [nblk_red] x 4
  double* norms = nullptr;        // [norm_cap] x 4
  int norm_cap = 0;
  int* bounds_err = nullptr;      // [4] index-checking kernels: flag, site, index, extent
  int* stepctl = nullptr;         // [0] = steps done in this call
  int upd_grid = 0;               // blocks of the last stage's update launch, which strides over the cells
                                  // (one wave of resident blocks; 0: one block per 256 cells)
  double* tctl = nullptr;         // [0] = t1, [1] = told of the current step
  // scheme
  double gamma = 1.4, khalf = 0, nkhalf = 0, omk = 1, cfl = 1, dt = 0;
  double gm1 = 0.4, igm1 = 2.5, ggm1 = 3.5;  // gamma-1, 1/(gamma-1) and gamma/(gamma-1)
  // the same constants rounded once on the host for the FP32 kernels
  float fgamma = 1.4f, fgm1 = 0.4f, figm1 = 2.5f, fkhalf = 0, fnkhalf = 0, fomk = 1, fggm1 = 3.5f;
  // and split into FP32 pairs (hi, lo) for the double-float kernels
  float dgamma[2] = {1.4f, 0}, dgm1[2] = {0.4f, 0}, digm1[2] = {2.5f, 0}, dkhalf[2] = {0, 0}, dnkhalf[2] = {0, 0},
        domk[2] = {1, 0}, dggm1[2] = {3.5f, 0};
  const void* volT = nullptr;    // [nc] 1/vol in the compute type (GG gradients)
  int limiter = 0, grad_method = 3, first_order = 0, vortex = 0;
  double vx = 0, vy = 0, vkappa = 0, vinf[4] = {0, 0, 0, 0};
  double pinf[4] = {0, 0, 0, 0};
  double mc[16];
};

// FP32 constants of the scheme: rounded, and split into (hi, lo) pairs
inline void set_fp32_constants(DevView& d) {
  auto split = [](double x, float* o) {
    o[0] = float(x);
    o[1] = float(x - double(o[0]));
  };
  d.fgamma = float(d.gamma); d.fgm1 = float(d.gm1); d.figm1 = float(d.igm1);
  d.fkhalf = float(d.khalf); d.fnkhalf = float(d.nkhalf); d.fomk = float(d.omk); d.fggm1 = float(d.ggm1);
  split(d.gamma, d.dgamma); split(d.gm1, d.dgm1); split(d.igm1, d.digm1);
  split(d.khalf, d.dkhalf); split(d.nkhalf, d.dnkhalf); split(d.omk, d.domk); split(d.ggm1, d.dggm1);
}

// Device view of a TilePlan (fvs_tiles.hpp) for the fused RK stage: one
// thread block per tile keeps the primitives of the tile and its halo, the
// gradients of the tile and its first halo layer and the tile's face fluxes
// in shared memory.  Arrays as in TilePlan; Pbuf: the primitive buffers the
// stages alternate between (Pbuf[0] is DevView::Pv).
struct TileView {
  int ntiles = 0, lmax = 0, gmax = 0, fmax = 0;
  const int* c0 = nullptr;
  const int* h0 = nullptr;
  const int* nh1 = nullptr;
  const int* halo = nullptr;
  const int* g0 = nullptr;
  const int* lsp = nullptr;
  const int* s0 = nullptr;
  const uint16_t* lst = nullptr;
  const int* f0 = nullptr;
  const int* face = nullptr;
  const uint32_t* flr = nullptr;
  const int2* lcf = nullptr;
  const void* fgeo = nullptr;   // per tile face, 8 T: nx, ny, length, xf-xcL, yf-ycL, xf-xcR, yf-ycR, 0
  const int2* gcell = nullptr;  // per gradient cell (lsp layout): device cell, first global stencil entry
  void* Pbuf[3] = {nullptr, nullptr, nullptr};
  int nbuf = 2;
  size_t smem_bytes = 0;  // dynamic shared memory of one block
};

// Device view of a TileDma plan (fvs_tiles.hpp): the bulk-copy form of the
// fused stage.  GB: the gather buffers the stages alternate between (the
// same parity as TileView::Pbuf), coef: stencil coefficients in tile order
// (pairs of the compute type); err: set when a bounded wait for the bulk
// copies ran out.
struct TileDmaView {
  const int* gb0 = nullptr;
  const int* sb0 = nullptr;
  const int* pb0 = nullptr;
  const int* rb0 = nullptr;
  const int* cb0 = nullptr;
  const uint16_t* lst = nullptr;
  const uint16_t* lsp = nullptr;
  const uint32_t* flr = nullptr;
  const int2* lcf = nullptr;
  const void* coef = nullptr;
  const int* dptr = nullptr;
  const int* dpos = nullptr;
  void* GB[3] = {nullptr, nullptr, nullptr};
  int smax = 0, pmax = 0, rmax = 0, qmax = 0;
  int* err = nullptr;
  size_t smem_bytes = 0;
  // shared-memory regions of a block, byte offsets (fvs_tiles.hpp dma_smem):
  // mbarrier at 0, primitives, face records, coefficients, stencil lists,
  // stencil offsets, face cells, gather lists, gradients x / y, limiter,
  // face fluxes
  unsigned o_P = 0, o_Fg = 0, o_C = 0, o_L = 0, o_S = 0, o_R = 0, o_Q = 0, o_Gx = 0, o_Gy = 0, o_Ph = 0, o_F = 0;
};

struct StageParams {
  int stage = 1, nstages = 4, mode = MODE_RK, steady = 0, last = 0;
  double h = 0;       // h_rk(stage) (unsteady)
  double cst = 0;     // steady multiplier of dt_local
  double coef = 1;    // rk_coef(stage)
  double a = 0, b = 1;  // SSP3 Shu-Osher weights
  double dts = 0;     // stage time offset from told
  // h, cst, coef, a, b as pairs of FP32 numbers (hi, lo) for the
  // double-float update; set_pairs() fills them from the doubles
  float hp[2] = {0, 0}, cstp[2] = {0, 0}, coefp[2] = {1, 0}, ap[2] = {0, 0}, bp[2] = {1, 0};
  void set_pairs() {
    const double src[5] = {h, cst, coef, a, b};
    float* dst[5] = {hp, cstp, coefp, ap, bp};
    for (int i = 0; i < 5; i++) {
      dst[i][0] = (float)src[i];
      dst[i][1] = (float)(src[i] - (double)dst[i][0]);
    }
  }
};

// Software grid barrier of the persistent kernel.  Every wait is bounded by a
// clock64() budget; a wait that runs out sets err, every block leaves at its
// next barrier and the host reports FVS_ERR_TIMEOUT.  (A two-level variant,
// blocks meeting first in 64 groups, measured 3-5 % slower on a 16-case
// sweep: with at most a few hundred resident blocks one counter suffices.)
struct GridBarrier {
  unsigned int count;
  unsigned int gen;
  int err;
  int pad;
};

// Work plan of the persistent kernel: nsteps RK steps over tile lists.
// Cell tiles never straddle two cases, so each tile's partial norm belongs
// to one case.  Only the tiles of active (not yet converged) cases are listed.
struct PersistPlan {
  int nsteps = 1, nstages = 4;
  StageParams sp[4];
  double t1 = 0;
  const int* step0_dev = nullptr;        // device word: global index of the launch's first step;
                                         // told = t1 + (step0 + s) * dt
  const int4* cell_tiles = nullptr;      // x = first cell, y = end, z = case
  int ncell_tiles = 0;
  const int2* edge_tiles = nullptr;      // x = first edge slot, y = end
  int nedge_tiles = 0;
  int tile = 0;                          // tile length (cells or edge slots)
  const int4* case_tiles = nullptr;      // x = case, y = first cell tile, z = end tile, w = cells of the case
                                         // (cell_tiles[t].w = the index of t's case in case_tiles)
  int ncase_active = 0;
  int* case_count = nullptr;             // [case_tiles] tiles of the step's last stage done (graph form)
  double* tile_partials = nullptr;       // [ncell_tiles][4]
  double* case_norms = nullptr;          // [ncases][norm_cap][4]
  int norm_cap = 0;
  GridBarrier* bar = nullptr;
  long long budget = 0;                  // clock64 cycles one barrier wait may take
};

// Kernel launchers, one set per arithmetic variant (strict FP64, FP64 with
// FMA, mixed).  All launch on the given stream; none synchronises.
struct KernelSet {
  const char* name;
  void (*begin_step)(const DevView&, cudaStream_t);
  void (*cvar2pvar)(const DevView&, cudaStream_t);
  void (*gradient)(const DevView&, cudaStream_t);
  // ws_out: also store the wave-speed records (a steady scheme's first stage
  // and residual evaluations read them)
  void (*flux)(const DevView&, double dts, bool ws_out, cudaStream_t);
  void (*update)(const DevView&, const StageParams&, cudaStream_t);
  void (*residual_out)(const DevView&, cudaStream_t);
  // persistent kernel (LSQ gradients): resident blocks per SM for a block
  // size (0: the scheme has no persistent variant), and the cooperative launch
  int (*persistent_occupancy)(const DevView&, int block);
  cudaError_t (*persistent)(const DevView&, const PersistPlan&, int grid, int block, cudaStream_t);
  // one step of the same tile work as separate launches (for graph capture)
  cudaError_t (*tiled_step)(const DevView&, const PersistPlan&, int block, cudaStream_t);
  // fused RK stage over the tiles of a TileView (mixed and double-float
  // builds; null elsewhere): stage k (0-based) reads Pbuf[k % nbuf] and
  // writes Pbuf[(k + 1) % nbuf]; dts is the stage's time offset
  cudaError_t (*tile_stage)(const DevView&, const TileView&, const StageParams&, int k, cudaStream_t);
  // shared memory of one tile block for the plan's largest tile (bytes)
  size_t (*tile_smem)(int lmax, int gmax, int fmax);
  // face flux + RK update of stage k over the tiles (gradients from the
  // separate gradient kernel); d.Pv is the stage's input buffer
  cudaError_t (*tile_fu_stage)(const DevView&, const TileView&, const StageParams&, int k, cudaStream_t);
  // bulk-copy fused stage (mixed build; null elsewhere), its shared memory
  // for a plan (0: too large, or the build has none), and the fill of a
  // gather buffer from the primitives (before the first stage after a new
  // state)
  cudaError_t (*tile_dma_stage)(const DevView&, const TileView&, const TileDmaView&, const StageParams&, int k,
                                cudaStream_t);
  size_t (*tile_dma_smem)(const TileView&, const TileDmaView&);
  cudaError_t (*tile_dma_fill)(const DevView&, const TileDmaView&, int buf, cudaStream_t);
  // blocks of 256 threads of the update kernel of an RK mode resident on the
  // device at once (0: unknown); queried before any graph capture
  int (*update_wave)(int mode);
};
// Defect correction of a first-order steady batch (mixed build): per chunk
// the FP64 residual R0 of the base state is evaluated once; the RK stages
// then iterate a correction dU of the base with the linearised residual
// R0 + J dU, J dU evaluated in FP32 by forward-mode differentiation of the
// Roe flux.  Arrays are [nc][4] FP32 in device order.
struct DcView {
  float* D = nullptr;    // correction dU
  float* D0 = nullptr;   // correction at the start of the step
  float* DF = nullptr;   // stage accumulator (fcvar)
  float* dP = nullptr;   // primitive tangent of dU at the base state
  float* dP2 = nullptr;  // second tangent buffer of the fused stage (null: separate
                         // J dU and update phases)
  float* R0 = nullptr;   // FP64 residual of the base state, rounded to FP32
  float* dtl = nullptr;  // [nc] local time step at the base state (FP32)
};

struct DcKernels {
  // U64 += dU; dU = dP = 0 (all cells)
  void (*fold)(const DevView& d32, const DcView& c, double* U64, cudaStream_t);
  // FP32 primitives of the base, R0 from the FP64 residual, local dt from
  // the FP64 wave speeds (all cells)
  void (*base)(const DevView& d32, const DcView& c, const double* U64, const double* resid64, const double* ws64,
               cudaStream_t);
  int (*occupancy)(const DcView& c, int block);
  cudaError_t (*persistent)(const DevView& d32, const PersistPlan& p, const DcView& c, int grid, int block,
                            cudaStream_t);
  cudaError_t (*tiled_step)(const DevView& d32, const PersistPlan& p, const DcView& c, int block, cudaStream_t);
};
const DcKernels& dc_kernels();

const KernelSet& kernels_fp64_strict();
const KernelSet& kernels_fp64_fast();
const KernelSet& kernels_mixed();
const KernelSet& kernels_fp64_df();
const KernelSet& kernels_fp64_bounds();

}  // namespace fvs
