// fvs_layout.hpp — device layout of one or many meshes (host side).
//
// A mesh is appended to a Layout in device order: its cells renumbered by
// reverse Cuthill-McKee and placed after the cells already present, its
// interior edge slots sorted by their first device cell, then its boundary
// slots in the reference's processing order.  A single-mesh handle holds one
// mesh; a batch holds the disjoint union of all its cases, which is again a
// mesh, so every kernel serves both.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "fvs_internal.hpp"

namespace fvs {

// device allocations owned by one handle
struct DeviceArena {
  std::vector<void*> allocs;
  ~DeviceArena() { release(); }
  void release() {
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
  }
  template <typename V>
  bool upload(V*& dst, const std::vector<V>& src) {
    dst = nullptr;
    if (src.empty()) return true;
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(V) * src.size()) != cudaSuccess) return false;
    allocs.push_back(p);
    if (cudaMemcpy(p, src.data(), sizeof(V) * src.size(), cudaMemcpyHostToDevice) != cudaSuccess) return false;
    dst = static_cast<V*>(p);
    return true;
  }
  bool alloc(void*& dst, size_t bytes) {
    dst = nullptr;
    if (bytes == 0) bytes = 16;
    if (cudaMalloc(&dst, bytes) != cudaSuccess) return false;
    allocs.push_back(dst);
    return cudaMemset(dst, 0, bytes) == cudaSuccess;
  }
};

inline double minimg(double d, double L) { return L > 0 ? d - L * std::nearbyint(d / L) : d; }

// reverse Cuthill-McKee over face neighbours: BFS from a pseudo-peripheral
// cell, neighbours visited by increasing degree, order reversed.  Returns
// reference cell -> local device index.
inline std::vector<int> rcm_order(const HostMesh& h) {
  const int nc = h.nc;
  std::vector<int> deg(nc, 0);
  for (int ic = 0; ic < nc; ic++)
    for (int k = 0; k < h.nvrt[ic]; k++) deg[ic] += h.nghbr[4 * ic + k] >= 0;
  std::vector<int> order;
  order.reserve(nc);
  std::vector<char> seen(nc, 0);
  std::vector<int> level(nc, -1);
  auto farthest = [&](int s) {
    std::vector<int> q{s};
    std::fill(level.begin(), level.end(), -1);
    level[s] = 0;
    for (size_t i = 0; i < q.size(); i++) {
      int c = q[i];
      for (int k = 0; k < h.nvrt[c]; k++) {
        int n = h.nghbr[4 * c + k];
        if (n >= 0 && level[n] < 0) {
          level[n] = level[c] + 1;
          q.push_back(n);
        }
      }
    }
    int best = q.back();
    for (int c : q)
      if (level[c] == level[q.back()] && deg[c] < deg[best]) best = c;
    return best;
  };
  int next_unseen = 0;
  while ((int)order.size() < nc) {
    while (seen[next_unseen]) next_unseen++;
    int start = next_unseen;
    for (int ic = next_unseen; ic < nc; ic++)
      if (!seen[ic] && deg[ic] < deg[start]) start = ic;
    start = farthest(farthest(start));
    size_t head = order.size();
    order.push_back(start);
    seen[start] = 1;
    int nb[4];
    while (head < order.size()) {
      int c = order[head++];
      int m = 0;
      for (int k = 0; k < h.nvrt[c]; k++) {
        int n = h.nghbr[4 * c + k];
        if (n >= 0 && !seen[n]) nb[m++] = n;
      }
      // at most 4 neighbours: insertion sort by (degree, index), a total order
      for (int i = 1; i < m; i++)
        for (int j = i; j > 0 && (deg[nb[j]] != deg[nb[j - 1]] ? deg[nb[j]] < deg[nb[j - 1]] : nb[j] < nb[j - 1]); j--)
          std::swap(nb[j], nb[j - 1]);
      for (int i = 0; i < m; i++) {
        seen[nb[i]] = 1;
        order.push_back(nb[i]);
      }
    }
  }
  std::reverse(order.begin(), order.end());
  std::vector<int> perm(nc);
  for (int i = 0; i < nc; i++) perm[order[i]] = i;
  return perm;
}

// host copies of the device arrays, in device order
template <typename T>
struct Layout {
  int nc = 0, ne = 0, nint = 0;  // nint: interior slots of all cases
  std::vector<int> perm;         // appended case by case: reference cell -> device cell
  std::vector<int> case_coff, case_eoff;
  std::vector<int2> ecell;
  std::vector<T> enrm, earea, edL, edR, exy;
  std::vector<int> ebtype;
  std::vector<int4> cf;
  std::vector<double> vol, rvol;
  std::vector<T> rvolT, eps2, cpos;
  std::vector<int8_t> nvrt;
  std::vector<int> st_ptr{0}, st_cell;
  std::vector<T> st_coef, st_w, coef0, coefedg;
  std::vector<int8_t> st_node;
};

// Appends one mesh (case index `cs`) to the layout.  fold_w: LSQ weights
// multiplied into the coefficients (the FP64 and mixed kernels).  order:
// reference cell -> local device index (default: reverse Cuthill-McKee).
template <typename T>
int append_case(Layout<T>& L, const HostMesh& h, bool fold_w, int cs, std::string& err,
                const std::vector<int>* order = nullptr) {
  const int nc = h.nc, coff = L.nc, eoff = L.ne;
  const std::vector<int> lperm = order ? *order : rcm_order(h);
  std::vector<int> perm(nc), iperm(nc);
  for (int i = 0; i < nc; i++) {
    perm[i] = coff + lperm[i];
    iperm[lperm[i]] = i;
  }
  const int nint = (int)h.edge_intr.size(), nbe = (int)h.b_edge.size(), ne = nint + nbe;
  L.case_coff.push_back(coff);
  L.case_eoff.push_back(eoff);
  // interior edge slots sorted by their first device cell (stable)
  std::vector<int> eorder(nint);
  std::iota(eorder.begin(), eorder.end(), 0);
  std::stable_sort(eorder.begin(), eorder.end(), [&](int a, int b) {
    int ea = h.edge_intr[a], eb = h.edge_intr[b];
    return std::min(lperm[h.ec1[ea]], lperm[h.ec2[ea]]) < std::min(lperm[h.ec1[eb]], lperm[h.ec2[eb]]);
  });
  std::vector<int> slot_of_intr(nint);
  for (int s = 0; s < nint; s++) slot_of_intr[eorder[s]] = eoff + s;
  L.ecell.resize(eoff + ne);
  L.enrm.resize(2 * (size_t)(eoff + ne));
  L.earea.resize(eoff + ne);
  L.edL.resize(2 * (size_t)(eoff + ne));
  L.edR.resize(2 * (size_t)(eoff + ne), T(0));
  L.exy.resize(2 * (size_t)(eoff + ne), T(0));
  L.ebtype.resize(eoff + ne, 0);
  for (int s = 0; s < nint; s++) {
    const int ie = h.edge_intr[eorder[s]], g = eoff + s;
    const int cl = h.ec1[ie], cr = h.ec2[ie];
    L.ecell[g] = make_int2(perm[cl], perm[cr]);
    L.enrm[2 * g] = T(h.enx[ie]);
    L.enrm[2 * g + 1] = T(h.eny[ie]);
    L.earea[g] = T(h.ea[ie]);
    L.edL[2 * g] = T(minimg(h.ex[ie] - h.xc[cl], h.Lx));
    L.edL[2 * g + 1] = T(minimg(h.ey[ie] - h.yc[cl], h.Ly));
    L.edR[2 * g] = T(minimg(h.ex[ie] - h.xc[cr], h.Lx));
    L.edR[2 * g + 1] = T(minimg(h.ey[ie] - h.yc[cr], h.Ly));
  }
  // boundary slots in the reference's processing order; edge i of boundary
  // ib is paired with bndry(ib)%cell(i) (src/residual.f90:114-125)
  std::vector<int> bcell_of(nbe);
  for (int ib = 0, k = 0; ib < h.nb; ib++)
    for (int i = h.b_eptr[ib]; i < h.b_eptr[ib + 1]; i++, k++) {
      const int ie = h.b_edge[i], cl = h.b_cell[h.b_cptr[ib] + (i - h.b_eptr[ib])], g = eoff + nint + k;
      bcell_of[k] = cl;
      L.ecell[g] = make_int2(perm[cl], -1);
      L.enrm[2 * g] = T(h.enx[ie]);
      L.enrm[2 * g + 1] = T(h.eny[ie]);
      L.earea[g] = T(h.ea[ie]);
      L.edL[2 * g] = T(minimg(h.ex[ie] - h.xc[cl], h.Lx));
      L.edL[2 * g + 1] = T(minimg(h.ey[ie] - h.yc[cl], h.Ly));
      L.ebtype[g] = h.b_type[ib] | (cs << 4);
      L.exy[2 * g] = T(h.ex[ie]);
      L.exy[2 * g + 1] = T(h.ey[ie]);
    }
  // gather lists in the reference's summation order: interior edges in
  // edge_intr order (+ to c1, - to c2), then the boundary edges
  L.cf.resize(coff + nc, make_int4(0, 0, 0, 0));
  std::vector<int> ncf(nc, 0);
  auto push = [&](int cell, int v) -> bool {
    const int lc = perm[cell] - coff;
    if (ncf[lc] >= 4) return false;
    reinterpret_cast<int*>(&L.cf[coff + lc])[ncf[lc]++] = v;
    return true;
  };
  for (int i = 0; i < nint; i++) {
    const int ie = h.edge_intr[i], s = slot_of_intr[i];
    if (!push(h.ec1[ie], s + 1) || !push(h.ec2[ie], -(s + 1))) {
      err = "a cell has more than 4 flux contributions";
      return FVS_ERR_MESH;
    }
  }
  for (int k = 0; k < nbe; k++)
    if (!push(bcell_of[k], eoff + nint + k + 1)) {
      err = "a cell has more than 4 flux contributions";
      return FVS_ERR_MESH;
    }
  // cell arrays in device order
  L.vol.resize(coff + nc);
  L.rvol.resize(coff + nc);
  L.rvolT.resize(coff + nc);
  L.eps2.resize(coff + nc);
  L.nvrt.resize(coff + nc);
  L.cpos.resize(8 * (size_t)(coff + nc), T(0));
  for (int o = 0; o < nc; o++) {
    const int dc = perm[o];
    L.vol[dc] = h.vol[o];
    L.rvol[dc] = 1.0 / h.vol[o];
    L.rvolT[dc] = T(1.0 / h.vol[o]);
    L.eps2[dc] = T(h.eps2[o]);
    L.nvrt[dc] = h.nvrt[o];
    for (int k = 0; k < h.nvrt[o]; k++) {
      const int je = h.cedge[4 * o + k];
      L.cpos[8 * (size_t)dc + 2 * k] = T(minimg(h.ex[je] - h.xc[o], h.Lx));
      L.cpos[8 * (size_t)dc + 2 * k + 1] = T(minimg(h.ey[je] - h.yc[o], h.Ly));
    }
  }
  // stencils in device order, per-cell entry order kept
  const bool ggnb = h.grad_method == FVS_GRAD_GGNB;
  fold_w = fold_w && h.grad_method == FVS_GRAD_LSQ;
  for (int lc = 0; lc < nc; lc++) {
    const int o = iperm[lc];
    for (int k = h.st_ptr[o]; k < h.st_ptr[o + 1]; k++) {
      L.st_cell.push_back(perm[h.st_cell[k]]);
      if (ggnb) {
        L.st_coef.push_back(T(h.st_coef[k]));
        L.st_node.push_back(h.st_node[k]);
      } else if (fold_w) {
        // FP64 / mixed: the LSQ weight folded into the coefficients (in FP64)
        L.st_coef.push_back(T(h.st_coef[2 * k] * h.st_w[k]));
        L.st_coef.push_back(T(h.st_coef[2 * k + 1] * h.st_w[k]));
      } else {
        L.st_coef.push_back(T(h.st_coef[2 * k]));
        L.st_coef.push_back(T(h.st_coef[2 * k + 1]));
      }
      if (!h.st_w.empty()) L.st_w.push_back(T(h.st_w[k]));
    }
    L.st_ptr.push_back((int)L.st_cell.size());
  }
  if (!h.coef0.empty()) {
    L.coef0.resize(2 * (size_t)(coff + nc));
    for (int o = 0; o < nc; o++) {
      L.coef0[2 * perm[o]] = T(h.coef0[2 * o]);
      L.coef0[2 * perm[o] + 1] = T(h.coef0[2 * o + 1]);
    }
  }
  if (!h.coefedg.empty()) {
    L.coefedg.resize(8 * (size_t)(coff + nc));
    for (int o = 0; o < nc; o++)
      for (int k = 0; k < 8; k++) L.coefedg[8 * (size_t)perm[o] + k] = T(h.coefedg[8 * o + k]);
  }
  L.perm.insert(L.perm.end(), perm.begin(), perm.end());
  L.nc += nc;
  L.ne += ne;
  L.nint += nint;
  return FVS_OK;
}

// Uploads the mesh arrays of a layout and points the view at them.
template <typename T>
bool upload_layout(DeviceArena& A, const Layout<T>& L, DevView& d) {
  bool ok = true;
  double *dvol, *drvol;
  int4* dcf;
  int8_t *dnv, *dsn;
  int *dsp, *dsc, *deb;
  int2* dec;
  T *t_rvol, *t_eps2, *t_cpos, *t_coef, *t_w, *t_c0, *t_ce, *t_nrm, *t_area, *t_edL, *t_edR, *t_exy;
  ok = ok && A.upload(dvol, L.vol) && A.upload(drvol, L.rvol) && A.upload(dcf, L.cf) && A.upload(dnv, L.nvrt);
  ok = ok && A.upload(dsp, L.st_ptr) && A.upload(dsc, L.st_cell) && A.upload(dsn, L.st_node) && A.upload(dec, L.ecell);
  ok = ok && A.upload(deb, L.ebtype) && A.upload(t_rvol, L.rvolT) && A.upload(t_eps2, L.eps2);
  ok = ok && A.upload(t_cpos, L.cpos) && A.upload(t_coef, L.st_coef) && A.upload(t_w, L.st_w);
  ok = ok && A.upload(t_c0, L.coef0) && A.upload(t_ce, L.coefedg) && A.upload(t_nrm, L.enrm) && A.upload(t_area, L.earea);
  ok = ok && A.upload(t_edL, L.edL) && A.upload(t_edR, L.edR) && A.upload(t_exy, L.exy);
  if (!ok) return false;
  d.nc = L.nc;
  d.nint = L.nint;
  d.nedge = L.ne;
  d.vol = dvol; d.rvol = drvol; d.cflist = dcf; d.nvrt = dnv; d.st_ptr = dsp; d.st_cell = dsc; d.st_node = dsn;
  d.ecell = dec; d.ebtype = deb; d.volT = t_rvol; d.eps2 = t_eps2; d.cpos = t_cpos; d.st_coef = t_coef; d.st_w = t_w;
  d.coef0 = t_c0; d.coefedg = t_ce; d.enrm = t_nrm; d.earea = t_area; d.edL = t_edL; d.edR = t_edR; d.exy = t_exy;
  return true;
}

// Allocates the state and work arrays of a view with nc cells, ne edges.
template <typename T>
bool alloc_work(DeviceArena& A, DevView& d, int nc, int ne, int nblk, int norm_cap) {
  void* p;
  bool ok = true;
  const size_t n4 = 4 * (size_t)nc;
  d.nblk_red = nblk;
  d.norm_cap = norm_cap;
#define FVS_ALLOC(field, type, bytes) \
  ok = ok && A.alloc(p, bytes);       \
  d.field = static_cast<type>(p)
  FVS_ALLOC(U, double*, 8 * n4);
  FVS_ALLOC(U0, double*, 8 * n4);
  FVS_ALLOC(F, double*, 8 * n4);
  FVS_ALLOC(resid, double*, 8 * n4);
  FVS_ALLOC(ws, double*, 8 * (size_t)nc);
  FVS_ALLOC(dtl, double*, 8 * (size_t)nc);
  FVS_ALLOC(Pv, void*, sizeof(T) * n4);
  FVS_ALLOC(Gx, void*, sizeof(T) * n4);
  FVS_ALLOC(Gy, void*, sizeof(T) * n4);
  FVS_ALLOC(phi, void*, sizeof(T) * (size_t)nc);
  FVS_ALLOC(eflux, void*, sizeof(T) * 4 * (size_t)ne);
  FVS_ALLOC(ews, void*, sizeof(T) * (size_t)ne);
  FVS_ALLOC(partials, double*, 32 * (size_t)nblk);
  FVS_ALLOC(norms, double*, 32 * (size_t)norm_cap);
  FVS_ALLOC(stepctl, int*, 16);
  FVS_ALLOC(tctl, double*, 16);
#undef FVS_ALLOC
  return ok;
}

}  // namespace fvs
