// fvs_tiles.hpp — tile decomposition of one mesh for the fused RK stage
// (host side).
//
// The fused stage kernel (k_tile_stage in fvs_kernels.cuh) runs one thread
// block per tile: a set of at most TILE_CELLS cells, contiguous in device
// order, whose primitives, gradients and face fluxes it keeps in shared
// memory.  For that the cells are numbered tile by tile (rcb_tile_order):
// recursive coordinate bisection of the cell centroids, always across the
// longer side of the current box at the median, until a part holds at most
// TILE_CELLS cells.  The parts are compact patches, so a tile's halo is its
// perimeter; consecutive tiles are neighbours, so halo reads hit in L2.
//
// Per tile t (build_tile_plan, from the device-order layout):
//   cells      [c0[t], c0[t+1])                      the tile's own cells
//   halo1      face neighbours outside the tile       (need gradients)
//   halo2      stencil cells of tile + halo1 outside both (need primitives)
//   local numbering: tile cells 0..n-1, halo1, halo2 (uint16)
//   lst        local index of every stencil entry of the gradient cells
//              (tile + halo1), in the global stencil's entry order
//   faces      every edge slot touching a tile cell, once, ascending slot;
//              flr = local L | local R << 16 (0xFFFF: boundary slot)
//   lcf        per tile cell the four signed slot references of the global
//              gather list (reference summation order) as local faces
// Cut faces (one cell in the tile, one in halo1) are evaluated by both tiles
// that touch them, each for its own cell.
#pragma once

#include <algorithm>
#include <cstdlib>
#include <cstdint>
#include <numeric>
#include <string>
#include <vector>

#include "fvs_internal.hpp"

namespace fvs {

constexpr int TILE_CELLS = 512;

// tile size: TILE_CELLS, or FVS2D_TILE_CELLS (64..4096) from the environment
inline int tile_cells_setting() {
  const char* e = std::getenv("FVS2D_TILE_CELLS");
  const int v = e ? std::atoi(e) : 0;
  return (v >= 64 && v <= 4096) ? v : TILE_CELLS;
}

// reference cell -> local device index: tiles of at most tile_cells cells by
// recursive coordinate bisection; within a tile, cells in the order of
// `within` (a local order such as reverse Cuthill-McKee), which keeps the
// tile's own loads close together
inline std::vector<int> rcb_tile_order(const HostMesh& h, const std::vector<int>& within, int tile_cells,
                                       std::vector<int>& tile_start) {
  const int nc = h.nc;
  std::vector<int> idx(nc);
  std::iota(idx.begin(), idx.end(), 0);
  struct Part { int b, e; };
  std::vector<Part> stack{{0, nc}};
  std::vector<Part> tiles;
  while (!stack.empty()) {
    const Part p = stack.back();
    stack.pop_back();
    if (p.e - p.b <= tile_cells) {
      tiles.push_back(p);
      continue;
    }
    double xl = 1e300, xh = -1e300, yl = 1e300, yh = -1e300;
    for (int i = p.b; i < p.e; i++) {
      const int c = idx[i];
      xl = std::min(xl, h.xc[c]); xh = std::max(xh, h.xc[c]);
      yl = std::min(yl, h.yc[c]); yh = std::max(yh, h.yc[c]);
    }
    const bool byx = (xh - xl) >= (yh - yl);
    const int m = p.b + (p.e - p.b) / 2;
    // median split with a total order (coordinate, then cell id): the same
    // tiles on every host
    std::nth_element(idx.begin() + p.b, idx.begin() + m, idx.begin() + p.e, [&](int a, int b) {
      const double ka = byx ? h.xc[a] : h.yc[a], kb = byx ? h.xc[b] : h.yc[b];
      return ka != kb ? ka < kb : a < b;
    });
    // depth first, lower half first: consecutive tiles are neighbours
    stack.push_back({m, p.e});
    stack.push_back({p.b, m});
  }
  std::vector<int> perm(nc);
  tile_start.assign(1, 0);
  int next = 0;
  for (const Part& t : tiles) {
    std::sort(idx.begin() + t.b, idx.begin() + t.e, [&](int a, int b) { return within[a] < within[b]; });
    for (int i = t.b; i < t.e; i++) perm[idx[i]] = next++;
    tile_start.push_back(next);
  }
  return perm;
}

struct TilePlan {
  int ntiles = 0, tile_cells = TILE_CELLS;
  int lmax = 0, gmax = 0, fmax = 0;  // largest local cell, gradient cell and face counts
  std::vector<int> c0;               // [ntiles + 1]
  std::vector<int> h0;               // [ntiles + 1] offsets into halo
  std::vector<int> nh1;              // [ntiles]
  std::vector<int> halo;             // device cells: halo1 then halo2 of each tile
  std::vector<int> g0;               // [ntiles + 1] offsets into lsp (one per gradient cell + 1 per tile)
  std::vector<int> lsp;              // per gradient cell: offset of its entries in lst (from s0[t])
  std::vector<int> s0;               // [ntiles + 1] offsets into lst
  std::vector<uint16_t> lst;         // local stencil entries
  std::vector<int> f0;               // [ntiles + 1] offsets into face / flr
  std::vector<int> face;             // edge slot of each tile face
  std::vector<uint32_t> flr;         // local L | local R << 16
  std::vector<int2> lcf;             // [nc] four int16 signed local face refs (+-(f+1)), packed in pairs
};

// Builds the plan from device-order connectivity: cells [tile_start[t],
// tile_start[t+1]) form tile t; ecell, cf (signed 1-based slots) and the
// stencil CSR (st_ptr, st_cell) are in device numbering.
inline int build_tile_plan(const std::vector<int>& tile_start, const std::vector<int2>& ecell,
                           const std::vector<int4>& cf, const std::vector<int>& st_ptr,
                           const std::vector<int>& st_cell, TilePlan& P, std::string& err) {
  const int nt = (int)tile_start.size() - 1;
  const int nc = tile_start.back();
  P = TilePlan();
  P.ntiles = nt;
  P.c0 = tile_start;
  P.h0.assign(1, 0);
  P.g0.assign(1, 0);
  P.s0.assign(1, 0);
  P.f0.assign(1, 0);
  P.lcf.assign(nc, make_int2(0, 0));
  std::vector<int> local(nc, -1);  // device cell -> local index within the current tile
  for (int t = 0; t < nt; t++) {
    const int b = tile_start[t], e = tile_start[t + 1], n = e - b;
    std::vector<int> cells;  // local -> device cell
    cells.reserve(2 * n);
    for (int c = b; c < e; c++) {
      local[c] = (int)cells.size();
      cells.push_back(c);
    }
    // faces of the tile's cells, each once, by slot
    std::vector<int> fl;
    for (int c = b; c < e; c++) {
      const int* s = reinterpret_cast<const int*>(&cf[c]);
      for (int k = 0; k < 4; k++)
        if (s[k] != 0) fl.push_back((s[k] > 0 ? s[k] : -s[k]) - 1);
    }
    std::sort(fl.begin(), fl.end());
    fl.erase(std::unique(fl.begin(), fl.end()), fl.end());
    // halo1: the other cell of every face
    for (int s : fl)
      for (int c : {ecell[s].x, ecell[s].y})
        if (c >= 0 && local[c] < 0) {
          local[c] = (int)cells.size();
          cells.push_back(c);
        }
    const int ng = (int)cells.size(), h1 = ng - n;
    // halo2: stencil cells of the gradient cells (tile + halo1)
    for (int i = 0; i < ng; i++)
      for (int k = st_ptr[cells[i]]; k < st_ptr[cells[i] + 1]; k++) {
        const int c = st_cell[k];
        if (local[c] < 0) {
          local[c] = (int)cells.size();
          cells.push_back(c);
        }
      }
    const int nl = (int)cells.size();
    if (nl > 0xFFFE) {
      err = "a tile's halo exceeds 65534 cells";
      return FVS_ERR_MESH;
    }
    for (int i = n; i < nl; i++) P.halo.push_back(cells[i]);
    P.h0.push_back((int)P.halo.size());
    P.nh1.push_back(h1);
    // local stencils of the gradient cells
    int off = 0;
    for (int i = 0; i < ng; i++) {
      P.lsp.push_back(off);
      for (int k = st_ptr[cells[i]]; k < st_ptr[cells[i] + 1]; k++, off++) P.lst.push_back((uint16_t)local[st_cell[k]]);
    }
    P.lsp.push_back(off);
    P.g0.push_back((int)P.lsp.size());
    P.s0.push_back((int)P.lst.size());
    // faces and their local cells
    std::vector<int> lface(fl.size());
    for (size_t f = 0; f < fl.size(); f++) {
      const int s = fl[f];
      const uint32_t l = (uint32_t)local[ecell[s].x];
      const uint32_t r = ecell[s].y >= 0 ? (uint32_t)local[ecell[s].y] : 0xFFFFu;
      P.face.push_back(s);
      P.flr.push_back(l | (r << 16));
    }
    P.f0.push_back((int)P.face.size());
    // gather lists in local faces (same entries, same order)
    for (int c = b; c < e; c++) {
      const int* s = reinterpret_cast<const int*>(&cf[c]);
      int16_t q[4] = {0, 0, 0, 0};
      for (int k = 0; k < 4; k++) {
        if (s[k] == 0) continue;
        const int slot = (s[k] > 0 ? s[k] : -s[k]) - 1;
        const int f = (int)(std::lower_bound(fl.begin(), fl.end(), slot) - fl.begin());
        if (f + 1 > 0x7FFF) {
          err = "a tile has more than 32766 faces";
          return FVS_ERR_MESH;
        }
        q[k] = (int16_t)(s[k] > 0 ? f + 1 : -(f + 1));
      }
      P.lcf[c] = make_int2((int)((uint16_t)q[0] | ((uint32_t)(uint16_t)q[1] << 16)),
                           (int)((uint16_t)q[2] | ((uint32_t)(uint16_t)q[3] << 16)));
    }
    P.lmax = std::max(P.lmax, nl);
    P.gmax = std::max(P.gmax, ng);
    P.fmax = std::max(P.fmax, (int)fl.size());
    for (int c : cells) local[c] = -1;
  }
  return FVS_OK;
}

// Checks every index the fused stage kernel derives from a plan against the
// extents it uses them for (shared-memory arrays of lmax / gmax / fmax
// entries, the device-order arrays of nc cells and ne edge slots).
// Returns an empty string when all hold, else the first violation.
inline std::string check_tile_plan(const TilePlan& P, int nc, int ne, const std::vector<int2>& ecell,
                                   const std::vector<int4>& cf, const std::vector<int>& st_ptr) {
  auto bad = [](const char* what, int t) { return std::string(what) + " (tile " + std::to_string(t) + ")"; };
  if ((int)P.c0.size() != P.ntiles + 1 || P.c0[0] != 0 || P.c0[P.ntiles] != nc) return "tile ranges do not cover the cells";
  for (int t = 0; t < P.ntiles; t++) {
    const int b = P.c0[t], n = P.c0[t + 1] - b;
    const int nh = P.h0[t + 1] - P.h0[t], nl = n + nh, ng = n + P.nh1[t], nf = P.f0[t + 1] - P.f0[t];
    if (n <= 0 || n > P.tile_cells) return bad("tile size outside 1..tile_cells", t);
    if (P.nh1[t] < 0 || P.nh1[t] > nh) return bad("halo1 count", t);
    if (nl > P.lmax || ng > P.gmax || nf > P.fmax || nl > 0xFFFE) return bad("counts above the plan maxima", t);
    for (int i = P.h0[t]; i < P.h0[t + 1]; i++)
      if (P.halo[i] < 0 || P.halo[i] >= nc || (P.halo[i] >= b && P.halo[i] < b + n)) return bad("halo cell", t);
    if (P.g0[t + 1] - P.g0[t] != ng + 1) return bad("gradient offset count", t);
    const int ns = P.s0[t + 1] - P.s0[t];
    for (int i = 0; i < ng; i++) {
      const int gid = i < n ? b + i : P.halo[P.h0[t] + i - n];
      const int o0 = P.lsp[P.g0[t] + i], o1 = P.lsp[P.g0[t] + i + 1];
      if (o0 < 0 || o1 > ns || o1 - o0 != st_ptr[gid + 1] - st_ptr[gid]) return bad("stencil offsets", t);
      for (int k = o0; k < o1; k++)
        if ((int)P.lst[P.s0[t] + k] >= nl) return bad("stencil entry outside the local cells", t);
    }
    for (int f = P.f0[t]; f < P.f0[t + 1]; f++) {
      const int s = P.face[f];
      if (s < 0 || s >= ne) return bad("face slot", t);
      const int l = (int)(P.flr[f] & 0xFFFFu), r = (int)(P.flr[f] >> 16);
      if (l >= ng) return bad("face left cell outside the gradient cells", t);
      if ((ecell[s].y < 0) != (r == 0xFFFF) || (r != 0xFFFF && r >= ng)) return bad("face right cell", t);
    }
    for (int c = b; c < b + n; c++) {
      const int* g = reinterpret_cast<const int*>(&cf[c]);
      const int16_t q[4] = {(int16_t)(P.lcf[c].x & 0xFFFF), (int16_t)((unsigned)P.lcf[c].x >> 16),
                            (int16_t)(P.lcf[c].y & 0xFFFF), (int16_t)((unsigned)P.lcf[c].y >> 16)};
      for (int k = 0; k < 4; k++) {
        if ((g[k] == 0) != (q[k] == 0) || (g[k] > 0) != (q[k] > 0)) return bad("gather entry", t);
        if (q[k] == 0) continue;
        const int f = (q[k] > 0 ? q[k] : -q[k]) - 1;
        if (f >= nf || P.face[P.f0[t] + f] != (g[k] > 0 ? g[k] : -g[k]) - 1) return bad("gather face", t);
      }
    }
  }
  return std::string();
}

// ---------------------------------------------------------------------------
// Bulk-copy form of the fused stage (FVS2D_TILE_STAGE=3)
// ---------------------------------------------------------------------------
// Every input of a tile block is one contiguous segment that a single
// cp.async.bulk brings into shared memory: the primitives of the tile's
// local cells (a gather buffer with one record per local cell, which every
// stage fills for the next one: each cell's new primitives go to its home
// record and to its record in every tile that holds it as a halo), the face
// records, the stencil coefficients, local stencil lists, stencil offsets,
// face cells and gather lists.  Each segment starts on a 16-byte boundary and
// has a multiple of 16 bytes (the bulk copy's rule): entry counts are padded.
struct TileDma {
  std::vector<int> gb0;        // [ntiles + 1] gather segment, in cell records (4 values)
  std::vector<int> sb0;        // [ntiles + 1] stencil entries (multiple of 8)
  std::vector<int> pb0;        // [ntiles + 1] stencil offsets, uint16 (multiple of 8)
  std::vector<int> rb0;        // [ntiles + 1] face cells, uint32 (multiple of 4)
  std::vector<int> cb0;        // [ntiles + 1] gather lists, int2 (multiple of 2)
  std::vector<uint16_t> lst;   // local cell of each stencil entry
  std::vector<uint16_t> lsp;   // per gradient cell: first entry (ng + 1 values)
  std::vector<uint32_t> flr;   // local L | local R << 16
  std::vector<int2> lcf;       // per tile cell: four int16 signed local face refs
  std::vector<int> coef_src;   // global stencil entry of each padded entry (-1: padding)
  std::vector<int> dptr, dpos; // per device cell: its gather records (home first)
  int smax = 0, pmax = 0, rmax = 0, qmax = 0;  // largest padded segment lengths
};

inline int pad_to(int n, int m) { return (n + m - 1) / m * m; }

inline void build_tile_dma(const TilePlan& P, const std::vector<int>& st_ptr, int nc, TileDma& D) {
  D = TileDma();
  D.gb0.assign(1, 0); D.sb0.assign(1, 0); D.pb0.assign(1, 0); D.rb0.assign(1, 0); D.cb0.assign(1, 0);
  std::vector<std::vector<int>> pos(nc);
  for (int t = 0; t < P.ntiles; t++) {
    const int b = P.c0[t], n = P.c0[t + 1] - b;
    const int nh = P.h0[t + 1] - P.h0[t], nl = n + nh, ng = n + P.nh1[t];
    const int nf = P.f0[t + 1] - P.f0[t], ns = P.s0[t + 1] - P.s0[t];
    // gather records: home records first in each cell's list
    for (int i = 0; i < nl; i++) {
      const int c = i < n ? b + i : P.halo[P.h0[t] + i - n];
      if (i < n) pos[c].insert(pos[c].begin(), D.gb0.back() + i);
      else pos[c].push_back(D.gb0.back() + i);
    }
    D.gb0.push_back(D.gb0.back() + nl);
    // stencil entries with their coefficients' global entry index
    const int nsp = pad_to(ns, 8);
    for (int k = 0; k < nsp; k++) D.lst.push_back(k < ns ? P.lst[P.s0[t] + k] : 0);
    for (int i = 0; i < ng; i++) {
      const int gid = i < n ? b + i : P.halo[P.h0[t] + i - n];
      const int cnt = P.lsp[P.g0[t] + i + 1] - P.lsp[P.g0[t] + i];
      for (int j = 0; j < cnt; j++) D.coef_src.push_back(st_ptr[gid] + j);
    }
    for (int k = ns; k < nsp; k++) D.coef_src.push_back(-1);
    D.sb0.push_back(D.sb0.back() + nsp);
    D.smax = std::max(D.smax, nsp);
    const int npp = pad_to(ng + 1, 8);
    for (int i = 0; i < npp; i++) D.lsp.push_back(i <= ng ? (uint16_t)P.lsp[P.g0[t] + i] : 0);
    D.pb0.push_back(D.pb0.back() + npp);
    D.pmax = std::max(D.pmax, npp);
    const int nfp = pad_to(nf, 4);
    for (int f = 0; f < nfp; f++) D.flr.push_back(f < nf ? P.flr[P.f0[t] + f] : 0u);
    D.rb0.push_back(D.rb0.back() + nfp);
    D.rmax = std::max(D.rmax, nfp);
    const int nq = pad_to(n, 2);
    for (int i = 0; i < nq; i++) D.lcf.push_back(i < n ? P.lcf[b + i] : make_int2(0, 0));
    D.cb0.push_back(D.cb0.back() + nq);
    D.qmax = std::max(D.qmax, nq);
  }
  D.dptr.assign(1, 0);
  for (int c = 0; c < nc; c++) {
    for (int q : pos[c]) D.dpos.push_back(q);
    D.dptr.push_back((int)D.dpos.size());
  }
}

// Shared-memory layout of a bulk-copy tile block, in bytes from the start
// (every region on a 16-byte boundary).  R: bytes of one value (4 or 8).
struct DmaSmem {
  size_t mbar, P, Fg, C, L, S, Rr, Q, Gx, Gy, Ph, F, total;
};
inline size_t al16(size_t x) { return (x + 15) / 16 * 16; }
inline DmaSmem dma_smem(int R, int lmax, int gmax, int fmax, int smax, int pmax, int rmax, int qmax) {
  DmaSmem m;
  size_t o = 0;
  m.mbar = o; o += 16;
  m.P = o; o = al16(o + (size_t)lmax * 4 * R);
  m.Fg = o; o = al16(o + (size_t)fmax * 8 * R);
  m.C = o; o = al16(o + (size_t)smax * 2 * R);
  m.L = o; o = al16(o + (size_t)smax * 2);
  m.S = o; o = al16(o + (size_t)pmax * 2);
  m.Rr = o; o = al16(o + (size_t)rmax * 4);
  m.Q = o; o = al16(o + (size_t)qmax * 8);
  m.Gx = o; o = al16(o + (size_t)gmax * 4 * R);
  m.Gy = o; o = al16(o + (size_t)gmax * 4 * R);
  m.Ph = o; o = al16(o + (size_t)gmax * R);
  m.F = o; o = al16(o + (size_t)fmax * 5 * R);
  // the norm reduction reuses [Gx, ...) : at least 4 x 256 doubles
  if (o - m.Gx < 4 * 256 * sizeof(double)) o = m.Gx + 4 * 256 * sizeof(double);
  m.total = o;
  return m;
}

// Checks what the bulk copies and the kernel's indexing rely on: segment
// starts and byte sizes multiples of 16, segments within their arrays and
// within the shared-memory regions, gather records within the buffer, every
// stencil offset within the tile's entries.  Empty string when all hold.
inline std::string check_tile_dma(const TilePlan& P, const TileDma& D, int R, int nc, size_t nstencil) {
  auto bad = [](const char* what, int t) { return std::string(what) + " (tile " + std::to_string(t) + ")"; };
  const int ntot = D.gb0.back();
  for (int t = 0; t < P.ntiles; t++) {
    const int n = P.c0[t + 1] - P.c0[t], nl = n + P.h0[t + 1] - P.h0[t], ng = n + P.nh1[t];
    const int nf = P.f0[t + 1] - P.f0[t];
    const int ns = D.sb0[t + 1] - D.sb0[t], np = D.pb0[t + 1] - D.pb0[t];
    const int nr = D.rb0[t + 1] - D.rb0[t], nq = D.cb0[t + 1] - D.cb0[t];
    if (D.gb0[t + 1] - D.gb0[t] != nl || nl > P.lmax) return bad("gather segment", t);
    if (((size_t)D.gb0[t] * 4 * R) % 16 || ((size_t)nl * 4 * R) % 16) return bad("gather alignment", t);
    if (((size_t)P.f0[t] * 8 * R) % 16 || nf > P.fmax) return bad("face record alignment", t);
    if (ns % 8 || D.sb0[t] % 8 || ns > D.smax) return bad("stencil segment", t);
    if (np % 8 || D.pb0[t] % 8 || np < ng + 1 || np > D.pmax) return bad("stencil offset segment", t);
    if (nr % 4 || D.rb0[t] % 4 || nr < nf || nr > D.rmax) return bad("face cell segment", t);
    if (nq % 2 || D.cb0[t] % 2 || nq < n || nq > D.qmax) return bad("gather list segment", t);
    for (int i = 0; i <= ng; i++)
      if (D.lsp[D.pb0[t] + i] > ns || (i > 0 && D.lsp[D.pb0[t] + i] < D.lsp[D.pb0[t] + i - 1]))
        return bad("stencil offsets", t);
    for (int k = 0; k < ns; k++) {
      if (D.lst[D.sb0[t] + k] >= nl) return bad("stencil entry", t);
      const int src = D.coef_src[D.sb0[t] + k];
      if (src < -1 || src >= (int)nstencil) return bad("coefficient entry", t);
    }
    for (int f = 0; f < nf; f++)
      if (D.flr[D.rb0[t] + f] != P.flr[P.f0[t] + f]) return bad("face cells", t);
  }
  if ((int)D.dptr.size() != nc + 1) return "gather record lists";
  for (int c = 0; c < nc; c++) {
    if (D.dptr[c + 1] <= D.dptr[c]) return "a cell without a home record";
    for (int j = D.dptr[c]; j < D.dptr[c + 1]; j++)
      if (D.dpos[j] < 0 || D.dpos[j] >= ntot) return "gather record outside the buffer";
  }
  return std::string();
}

}  // namespace fvs
