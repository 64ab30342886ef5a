// fvs_setup.cpp — host-side mesh preprocessing for the device path.
//
// Produces, from the arrays grid_read/grid_bc_read load, the connectivity,
// geometry and gradient operators of the reference bit-for-bit:
//   grid_data            src/grid_procs.f90:170-794
//   grid_data_verify     src/grid_procs.f90:814-852
//   setup_fn / setup_nn  src/gradient_lsq.f90:70-365 (+ verify :490-529)
//   GG-cell setup        src/gradient_ggcb.f90:48-110
//   GG-node setup        src/gradient_ggnb.f90:49-177
// The algorithms differ from the reference where only speed is at stake
// (edge neighbours come from a hash of directed edges instead of scanning the
// cells around a node) and agree where the numbering depends on the order
// (edges are created in cell order and local-edge order exactly as the
// reference does).  All floating-point expressions keep the reference's
// evaluation order; this file is compiled with -ffp-contract=off.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <unordered_map>

#include "fvs_internal.hpp"

namespace fvs {

static const double kPi = 3.141592653589793238462643383279502884;

namespace {

inline double unwrap(double v, double ref, double L) { return L > 0 ? v - L * std::nearbyint((v - ref) / L) : v; }
inline double minimg(double d, double L) { return L > 0 ? d - L * std::nearbyint(d / L) : d; }
inline double wrap_into(double v, double lo, double L) {
  if (L > 0) {
    if (v < lo) v += L;
    else if (v >= lo + L) v -= L;
  }
  return v;
}

// ---------------------------------------------------------------------------
// kdtree2 semantics (src/kdtree2.f90): mean split on the widest coordinate,
// buckets of at most 13 points, best-first search with a max-heap of the n
// closest squared distances, results heap-sorted by distance.  Ties between
// equidistant cells resolve exactly as in kdtree2, which matters because the
// LSQ-fn stencil takes the first unused cells of the sorted list.
// ---------------------------------------------------------------------------
class KdTree {
 public:
  struct Hit { double dis; int idx; };

  KdTree(const std::vector<double>& x, const std::vector<double>& y) : x_(x), y_(y) {
    int n = (int)x.size();
    ind_.resize(n);
    std::iota(ind_.begin(), ind_.end(), 0);
    nodes_.reserve(2 * (size_t)n / 6 + 16);
    root_ = build(0, n - 1, -1);
  }

  // n nearest points to (qx,qy), sorted ascending by squared distance
  void nearest(double qx, double qy, int n, std::vector<Hit>& out) const {
    Search s{qx, qy, n, 0, 1.79769313486231570815e+308, {}};
    s.heap.assign(n + 1, Hit{0.0, -1});
    search(s, root_);
    heapsort(s.heap, n);
    out.assign(s.heap.begin() + 1, s.heap.begin() + 1 + n);
  }

 private:
  struct Box { double lo, hi; };
  struct Node {
    int cut_dim = -1;
    double cut_val = 0, cut_left = 0, cut_right = 0;
    int l = 0, u = 0, left = -1, right = -1;
    Box box[2];
  };
  struct Search {
    double qx, qy;
    int nn, nfound;
    double ball;
    std::vector<Hit> heap;  // 1-based
  };

  double coord(int c, int i) const { return c == 0 ? x_[i] : y_[i]; }

  Box spread(int c, int l, int u) const {
    double smin = coord(c, ind_[l]), smax = smin;
    int i = l + 2;
    for (; i <= u; i += 2) {
      double a = coord(c, ind_[i - 1]), b = coord(c, ind_[i]);
      if (a > b) std::swap(a, b);
      if (smin > a) smin = a;
      if (smax < b) smax = b;
    }
    if (i == u + 1) {
      double last = coord(c, ind_[u]);
      if (smin > last) smin = last;
      if (smax < last) smax = last;
    }
    return Box{smin, smax};
  }

  int partition(int c, double alpha, int l, int u) {
    int lb = l, rb = u;
    while (lb < rb) {
      if (coord(c, ind_[lb]) <= alpha) ++lb;
      else { std::swap(ind_[lb], ind_[rb]); --rb; }
    }
    return coord(c, ind_[lb]) <= alpha ? lb : lb - 1;
  }

  int build(int l, int u, int parent) {
    if (u < l) return -1;
    int id = (int)nodes_.size();
    nodes_.emplace_back();
    if (u - l <= 12) {
      Node& nd = nodes_[id];
      nd.box[0] = spread(0, l, u);
      nd.box[1] = spread(1, l, u);
      nd.l = l; nd.u = u;
      return id;
    }
    Box b[2];
    for (int c = 0; c < 2; c++)
      b[c] = (parent < 0 || nodes_[parent].cut_dim == c) ? spread(c, l, u) : nodes_[parent].box[c];
    int c = (b[1].hi - b[1].lo > b[0].hi - b[0].lo) ? 1 : 0;
    double s = 0.0;
    for (int k = l; k <= u; k++) s = s + coord(c, ind_[k]);
    double avg = s / (double)(u - l + 1);
    {
      Node& nd = nodes_[id];
      nd.box[0] = b[0]; nd.box[1] = b[1];
      nd.cut_val = avg; nd.cut_dim = c; nd.l = l; nd.u = u;
    }
    int m = partition(c, avg, l, u);
    int left = build(l, m, id);
    int right = build(m + 1, u, id);
    Node& nd = nodes_[id];
    nd.left = left; nd.right = right;
    if (right < 0) {
      nd.box[0] = nodes_[left].box[0]; nd.box[1] = nodes_[left].box[1];
      nd.cut_left = nodes_[left].box[c].hi; nd.cut_val = nd.cut_left;
    } else if (left < 0) {
      nd.box[0] = nodes_[right].box[0]; nd.box[1] = nodes_[right].box[1];
      nd.cut_right = nodes_[right].box[c].lo; nd.cut_val = nd.cut_right;
    } else {
      nd.cut_right = nodes_[right].box[c].lo;
      nd.cut_left = nodes_[left].box[c].hi;
      nd.cut_val = (nd.cut_left + nd.cut_right) / 2;
      for (int k = 0; k < 2; k++) {
        nd.box[k].hi = std::fmax(nodes_[left].box[k].hi, nodes_[right].box[k].hi);
        nd.box[k].lo = std::fmin(nodes_[left].box[k].lo, nodes_[right].box[k].lo);
      }
    }
    return id;
  }

  static double heap_insert(Search& s, double dis, int idx) {
    int i = ++s.nfound;
    while (i > 1) {
      int p = i / 2;
      if (dis > s.heap[p].dis) { s.heap[i] = s.heap[p]; i = p; }
      else break;
    }
    s.heap[i] = Hit{dis, idx};
    return s.heap[1].dis;
  }

  static double heap_replace_max(Search& s, double dis, int idx) {
    int n = s.nfound, parent = 1, child = 2;
    while (child <= n) {
      double pc = s.heap[child].dis;
      if (child < n && pc < s.heap[child + 1].dis) { child++; pc = s.heap[child].dis; }
      if (dis >= pc) break;
      s.heap[parent] = s.heap[child];
      parent = child; child = 2 * parent;
    }
    s.heap[parent] = Hit{dis, idx};
    return s.heap[1].dis;
  }

  void terminal(Search& s, const Node& nd) const {
    double ball = s.ball;
    for (int i = nd.l; i <= nd.u; i++) {
      int p = ind_[i];
      double d = x_[p] - s.qx, sd = 0.0;
      sd = sd + d * d;
      if (sd > ball) continue;
      d = y_[p] - s.qy;
      sd = sd + d * d;
      if (sd > ball) continue;
      if (s.nfound < s.nn) {
        double top = heap_insert(s, sd, p);
        if (s.nfound == s.nn) ball = top;
      } else {
        ball = heap_replace_max(s, sd, p);
      }
    }
    s.ball = ball;
  }

  static double dist2_box(double q, const Box& b) {
    if (q > b.hi) return (q - b.hi) * (q - b.hi);
    if (q < b.lo) return (b.lo - q) * (b.lo - q);
    return 0.0;
  }

  void search(Search& s, int id) const {
    const Node& nd = nodes_[id];
    if (nd.left < 0 || nd.right < 0) { terminal(s, nd); return; }
    double q = nd.cut_dim == 0 ? s.qx : s.qy, dis;
    int closer, farther;
    if (q < nd.cut_val) { closer = nd.left; farther = nd.right; dis = (nd.cut_right - q) * (nd.cut_right - q); }
    else { closer = nd.right; farther = nd.left; dis = (nd.cut_left - q) * (nd.cut_left - q); }
    search(s, closer);
    double ball = s.ball;
    if (dis <= ball) {
      int other = 1 - nd.cut_dim;
      dis = dis + dist2_box(other == 0 ? s.qx : s.qy, nd.box[other]);
      if (dis > ball) return;
      search(s, farther);
    }
  }

  static void heapsort(std::vector<Hit>& a, int n) {
    if (n <= 1) return;
    int il = n / 2 + 1, ir = n;
    for (;;) {
      Hit v;
      if (il > 1) v = a[--il];
      else {
        v = a[ir]; a[ir] = a[1];
        if (--ir == 1) { a[1] = v; return; }
      }
      int i = il, j = 2 * il;
      while (j <= ir) {
        if (j < ir && a[j].dis < a[j + 1].dis) j++;
        if (v.dis < a[j].dis) { a[i] = a[j]; i = j; j += j; }
        else j = ir + 1;
      }
      a[i] = v;
    }
  }

  const std::vector<double>& x_;
  const std::vector<double>& y_;
  std::vector<int> ind_;
  std::vector<Node> nodes_;
  int root_ = -1;
};

// LSQ normal-equation coefficients for one cell (identical arithmetic in
// setup_fn :137-201 and setup_nn :292-338)
bool lsq_cell_coeffs(HostMesh& h, int ic, double pw) {
  int b = h.st_ptr[ic], n = h.st_ptr[ic + 1] - b;
  if (n > 64) return false;
  double d[64][2];
  for (int k = 0; k < n; k++) {
    int jc = h.st_cell[b + k];
    double dx = minimg(h.xc[jc] - h.xc[ic], h.Lx), dy = minimg(h.yc[jc] - h.yc[ic], h.Ly);
    double dis = std::sqrt(dx * dx + dy * dy);
    double w = 0.0;
    if (dis > 0.0) w = 1.0 / std::pow(dis, pw);
    h.st_w[b + k] = w;
    d[k][0] = w * dx;
    d[k][1] = w * dy;
  }
  double g[2][2];
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) {
      double s = 0.0;
      for (int k = 0; k < n; k++) s = s + d[k][i] * d[k][j];
      g[i][j] = s;
    }
  double det = g[0][0] * g[1][1] - g[0][1] * g[1][0];
  double gi[2][2] = {{1.0 / det * g[1][1], -1.0 / det * g[0][1]}, {-1.0 / det * g[1][0], 1.0 / det * g[0][0]}};
  for (int k = 0; k < n; k++)
    for (int i = 0; i < 2; i++) h.st_coef[2 * (b + k) + i] = (0.0 + gi[i][0] * d[k][0]) + gi[i][1] * d[k][1];
  return true;
}

}  // namespace

// ---------------------------------------------------------------------------
void mms_constants(double* mc) {
  const double v[16] = {1.12, 0.15, 3.12 * kPi, 2.92 * kPi, 1.32, 0.06, 2.09 * kPi, 3.12 * kPi,
                        1.18, 0.03, 2.15 * kPi, 3.32 * kPi, 1.62, 0.31, 3.79 * kPi, 2.98 * kPi};
  std::memcpy(mc, v, sizeof(v));
}

static double msol(const double* m, int nx, int ny, double x, double y) {
  double arg = m[2] * x + m[3] * y;
  if (nx + ny == 0) return m[0] + m[1] * std::sin(arg);
  double pw = (nx ? m[2] : 1.0) * (ny ? m[3] : 1.0);  // ax**nx * ay**ny for nx+ny == 1
  return pw * m[1] * std::cos(arg);
}

void mms_euler2d(const double* mc, double g, double xc, double yc, double* sol, double* rhs) {
  double r = msol(mc, 0, 0, xc, yc), u = msol(mc + 4, 0, 0, xc, yc);
  double v = msol(mc + 8, 0, 0, xc, yc), p = msol(mc + 12, 0, 0, xc, yc);
  sol[0] = r; sol[1] = u; sol[2] = v; sol[3] = p;
  double rx = msol(mc, 1, 0, xc, yc), ux = msol(mc + 4, 1, 0, xc, yc);
  double vx = msol(mc + 8, 1, 0, xc, yc), px = msol(mc + 12, 1, 0, xc, yc);
  double ry = msol(mc, 0, 1, xc, yc), uy = msol(mc + 4, 0, 1, xc, yc);
  double vy = msol(mc + 8, 0, 1, xc, yc), py = msol(mc + 12, 0, 1, xc, yc);
  double rH = g / (g - 1.0) * p + r * u * u / 2.0 + r * v * v / 2.0;
  double rHx = g / (g - 1.0) * px + rx * (u * u + v * v) / 2.0 + r * (u * ux + v * vx);
  double rHy = g / (g - 1.0) * py + ry * (u * u + v * v) / 2.0 + r * (u * uy + v * vy);
  rhs[0] = rx * u + u * rx + ry * v + r * vy;
  rhs[1] = rx * u * u + 2.0 * r * u * ux + ry * u * v + r * uy * v + r * u * vy + px;
  rhs[2] = rx * u * v + r * ux * v + r * u * vx + ry * v * v + 2.0 * r * v * vy + py;
  rhs[3] = u * rHx + ux * rH + v * rHy + vy * rH;
}

void vortex_state(const fvs_options& o, double t, double x, double y, double* pv) {
  double g = o.gamma, K = o.vortex_kappa;
  double T_inf = o.vortex_inf[3] / o.vortex_inf[0];
  double dx = x - (o.vortex_x + o.vortex_inf[1] * t);
  double dy = y - (o.vortex_y + o.vortex_inf[2] * t);
  double r = std::sqrt(dx * dx + dy * dy);
  double q = K / (2.0 * kPi);
  double u = o.vortex_inf[1] - q * dy * std::exp(0.5 * (1.0 - r * r));
  double v = o.vortex_inf[2] + q * dx * std::exp(0.5 * (1.0 - r * r));
  double temp = T_inf - (q * q) * (g - 1.0) / (2.0 * g) * std::exp(1.0 - r * r);
  double rho = std::pow(temp, 1.0 / (g - 1.0));
  pv[0] = rho; pv[1] = u; pv[2] = v; pv[3] = std::pow(rho, g);
}

// runge_kutta_init, src/runge_kutta.f90:25-67 (+ SSP-RK3 stage times)
void rk_coefficients(const fvs_options& o, double dt, double* h, double* c, double* dts) {
  for (int k = 0; k < 5; k++) { h[k] = 0; c[k] = 0; dts[k] = 0; }
  if (o.rk_nstages == 4) {
    static const double tab[4][4] = {{3.60897, 2.04, 0.34206, 0.00897}, {0.11, 3.92, 1.86, 0.11},
                                     {0.65, 2.7, 2.0, 0.65}, {1.0, 2.0, 2.0, 1.0}};
    const double* r = tab[o.rk_order - 1];
    h[1] = dt / 2.0; h[2] = dt / 2.0; h[3] = dt; h[4] = dt / 6.0;
    c[1] = r[0]; c[2] = r[1]; c[3] = r[2]; c[4] = r[3];
    dts[1] = 0.0; dts[2] = 0.5 * dt; dts[3] = 0.5 * dt; dts[4] = dt;  // told, t12, t12, tnew
    if (o.rk_order == 2 && o.ssprk) {
      h[1] = dt / 3.0; h[2] = dt / 3.0; h[3] = dt / 3.0; h[4] = dt / 4.0;
      c[1] = c[2] = c[3] = c[4] = 1.0;
      dts[1] = 0.0; dts[2] = dt / 3.0; dts[3] = dt * 2.0 / 3.0; dts[4] = dt;
    }
  } else if (o.rk_nstages == 3) {
    h[1] = h[2] = h[3] = dt;
    c[1] = c[2] = c[3] = 1.0;
    dts[1] = 0.0; dts[2] = dt; dts[3] = dt / 2.0;
  }
}

// ---------------------------------------------------------------------------
int build_host_mesh(const fvs_mesh* m, const fvs_options* o, HostMesh& h, std::string& err) {
  h.nnodes = m->nnodes; h.ntri = m->ncells_tri; h.nquad = m->ncells_quad;
  const int nc = h.nc = h.ntri + h.nquad;
  h.Lx = m->period_x > 0 ? m->period_x : 0.0;
  h.Ly = m->period_y > 0 ? m->period_y : 0.0;
  h.xn.resize(h.nnodes); h.yn.resize(h.nnodes);
  for (int i = 0; i < h.nnodes; i++) { h.xn[i] = m->node_xy[2 * i]; h.yn[i] = m->node_xy[2 * i + 1]; }
  if (h.Lx > 0 || h.Ly > 0) {
    h.xmin = *std::min_element(h.xn.begin(), h.xn.end());
    h.ymin = *std::min_element(h.yn.begin(), h.yn.end());
  }
  h.nvrt.assign(nc, 0);
  h.cnode.assign(4 * (size_t)nc, -1);
  for (int i = 0; i < h.ntri; i++) {
    h.nvrt[i] = 3;
    for (int k = 0; k < 3; k++) h.cnode[4 * i + k] = m->tri_nodes[3 * i + k] - 1;
  }
  for (int i = 0; i < h.nquad; i++) {
    int ic = h.ntri + i;
    h.nvrt[ic] = 4;
    for (int k = 0; k < 4; k++) h.cnode[4 * ic + k] = m->quad_nodes[4 * i + k] - 1;
  }
  for (int ic = 0; ic < nc; ic++)
    for (int k = 0; k < h.nvrt[ic]; k++)
      if (h.cnode[4 * ic + k] < 0 || h.cnode[4 * ic + k] >= h.nnodes) {
        err = "cell " + std::to_string(ic + 1) + " references node " + std::to_string(h.cnode[4 * ic + k] + 1) + " out of range";
        return FVS_ERR_MESH;
      }

  // centroids and volumes (:185-227); periodic vertices unwrapped against node 1
  h.xc.resize(nc); h.yc.resize(nc); h.vol.resize(nc);
  for (int ic = 0; ic < nc; ic++) {
    const int nv = h.nvrt[ic];
    const int* cn = &h.cnode[4 * ic];
    double X[4], Y[4];
    for (int k = 0; k < nv; k++) { X[k] = unwrap(h.xn[cn[k]], h.xn[cn[0]], h.Lx); Y[k] = unwrap(h.yn[cn[k]], h.yn[cn[0]], h.Ly); }
    double sx = 0.0, sy = 0.0;
    for (int k = 0; k < nv; k++) { sx = sx + X[k]; sy = sy + Y[k]; }
    h.xc[ic] = wrap_into(sx / (double)nv, h.xmin, h.Lx);
    h.yc[ic] = wrap_into(sy / (double)nv, h.ymin, h.Ly);
    auto tri = [](double x1, double x2, double x3, double y1, double y2, double y3) {
      return 0.5 * (((x1 * (y2 - y3)) + (x2 * (y3 - y1))) + (x3 * (y1 - y2)));
    };
    h.vol[ic] = tri(X[0], X[1], X[2], Y[0], Y[1], Y[2]);
    if (nv == 4) h.vol[ic] = h.vol[ic] + tri(X[0], X[2], X[3], Y[0], Y[2], Y[3]);
  }
  {
    double at = 0.0;
    for (int ic = 0; ic < nc; ic++) at = at + h.vol[ic];
    h.heff1 = std::sqrt(at / (double)nc);
    at = 0.0;
    for (int ic = 0; ic < nc; ic++) at = at + std::sqrt(h.vol[ic]);
    h.heff2 = at / (double)nc;
  }

  // node -> cells in ascending cell order (:273-296)
  h.nd_ptr.assign(h.nnodes + 1, 0);
  for (int ic = 0; ic < nc; ic++)
    for (int k = 0; k < h.nvrt[ic]; k++) h.nd_ptr[h.cnode[4 * ic + k] + 1]++;
  for (int i = 0; i < h.nnodes; i++) h.nd_ptr[i + 1] += h.nd_ptr[i];
  h.nd_cell.resize(h.nd_ptr[h.nnodes]);
  {
    std::vector<int> fill(h.nd_ptr.begin(), h.nd_ptr.end() - 1);
    for (int ic = 0; ic < nc; ic++)
      for (int k = 0; k < h.nvrt[ic]; k++) h.nd_cell[fill[h.cnode[4 * ic + k]]++] = ic;
  }

  // edge neighbours (:325-366).  Local edge k of a cell runs node(k) ->
  // node(k+1); its neighbour is the cell holding the reversed directed edge
  // and is stored at slot (k+2) mod nvrt.
  h.nghbr.assign(4 * (size_t)nc, -1);
  std::vector<int> partner(4 * (size_t)nc, -1);  // cell*4+local edge of the twin
  {
    std::unordered_map<uint64_t, int> dir;
    dir.reserve(4 * (size_t)nc);
    auto key = [](int a, int b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; };
    for (int ic = 0; ic < nc; ic++) {
      const int nv = h.nvrt[ic];
      for (int k = 0; k < nv; k++) {
        int a = h.cnode[4 * ic + k], b = h.cnode[4 * ic + (k + 1) % nv];
        if (!dir.emplace(key(a, b), 4 * ic + k).second) {
          err = "directed edge " + std::to_string(a + 1) + "->" + std::to_string(b + 1) +
                " appears in two cells (inconsistent orientation or non-manifold mesh)";
          return FVS_ERR_MESH;
        }
      }
    }
    for (int ic = 0; ic < nc; ic++) {
      const int nv = h.nvrt[ic];
      for (int k = 0; k < nv; k++) {
        int a = h.cnode[4 * ic + k], b = h.cnode[4 * ic + (k + 1) % nv];
        auto it = dir.find(key(b, a));
        if (it != dir.end()) {
          int jc = it->second / 4;
          h.nghbr[4 * ic + (k + 2) % nv] = jc;
          partner[4 * ic + k] = it->second;
        }
      }
    }
    // two cells sharing two edges would make the reference's twin lookup
    // (first matching neighbour slot, :508-518) ambiguous
    for (int ic = 0; ic < nc; ic++) {
      const int nv = h.nvrt[ic];
      for (int a = 0; a < nv; a++)
        for (int b = a + 1; b < nv; b++)
          if (h.nghbr[4 * ic + a] >= 0 && h.nghbr[4 * ic + a] == h.nghbr[4 * ic + b]) {
            err = "cells " + std::to_string(ic + 1) + " and " + std::to_string(h.nghbr[4 * ic + a] + 1) + " share two edges";
            return FVS_ERR_MESH;
          }
    }
  }
  // nghbre (:373-395): neighbour across local edge e
  h.nghbre.assign(4 * (size_t)nc, -1);
  for (int ic = 0; ic < nc; ic++) {
    const int nv = h.nvrt[ic];
    for (int k = 0; k < nv; k++) h.nghbre[4 * ic + k] = h.nghbr[4 * ic + (k + 2) % nv];
  }

  // edges in creation order (:401-624): ascending cell, local edge order
  h.cedge.assign(4 * (size_t)nc, -1);
  for (int ic = 0; ic < nc; ic++) {
    const int nv = h.nvrt[ic];
    for (int k = 0; k < nv; k++) {
      int nb = h.nghbr[4 * ic + (k + 2) % nv];
      if (nb > ic || nb < 0) {
        h.cedge[4 * ic + k] = h.ne++;
        h.en1.push_back(h.cnode[4 * ic + k]);
        h.en2.push_back(h.cnode[4 * ic + (k + 1) % nv]);
        h.ec1.push_back(ic);
        h.ec2.push_back(nb);
      } else {
        h.cedge[4 * ic + k] = h.cedge[partner[4 * ic + k]];
      }
    }
  }
  const int ne = h.ne;
  // edge geometry (:630-647)
  h.ex.resize(ne); h.ey.resize(ne); h.ea.resize(ne); h.enx.resize(ne); h.eny.resize(ne); h.etx.resize(ne); h.ety.resize(ne);
  for (int i = 0; i < ne; i++) {
    double x1 = h.xn[h.en1[i]], y1 = h.yn[h.en1[i]];
    double x2 = unwrap(h.xn[h.en2[i]], x1, h.Lx), y2 = unwrap(h.yn[h.en2[i]], y1, h.Ly);
    double dx = x2 - x1, dy = y2 - y1;
    double a = std::sqrt(dx * dx + dy * dy);
    h.ea[i] = a;
    h.ex[i] = wrap_into(0.5 * (x1 + x2), h.xmin, h.Lx);
    h.ey[i] = wrap_into(0.5 * (y1 + y2), h.ymin, h.Ly);
    h.enx[i] = dy / a; h.eny[i] = -dx / a;
    h.etx[i] = dx / a; h.ety[i] = dy / a;
  }
  // nrmlsign (:672-691)
  h.nrmlsign.assign(4 * (size_t)nc, 1.0);
  for (int ic = 0; ic < nc; ic++)
    for (int k = 0; k < h.nvrt[ic]; k++)
      if (h.ec1[h.cedge[4 * ic + k]] != ic) h.nrmlsign[4 * ic + k] = -1.0;

  // boundaries
  h.nb = m->nbndries;
  h.b_type.resize(h.nb);
  h.b_cptr.assign(h.nb + 1, 0);
  for (int ib = 0; ib < h.nb; ib++) {
    h.b_type[ib] = m->bndry_type[ib];
    h.b_cptr[ib + 1] = h.b_cptr[ib] + m->bndry_ncells[ib];
    int t = h.b_type[ib];
    if (t != FVS_BC_FREESTREAM && t != FVS_BC_SLIP_WALL && t != FVS_BC_DIRICHLET) {
      err = "boundary " + std::to_string(ib + 1) + ": type " + std::to_string(t) +
            " not implemented (src/residual.f90:206-220)";
      return FVS_ERR_INVALID;
    }
  }
  h.b_cell.resize(h.b_cptr[h.nb]);
  for (int i = 0; i < h.b_cptr[h.nb]; i++) {
    h.b_cell[i] = m->bndry_cells[i] - 1;
    if (h.b_cell[i] < 0 || h.b_cell[i] >= nc) { err = "boundary cell id out of range"; return FVS_ERR_MESH; }
  }
  // interior / boundary cells (:697-728)
  for (int ic = 0; ic < nc; ic++) {
    bool interior = true;
    for (int k = 0; k < h.nvrt[ic]; k++) if (h.nghbre[4 * ic + k] < 0) interior = false;
    (interior ? h.cell_intr : h.cell_bndr).push_back(ic);
  }
  if ((int)h.cell_bndr.size() != h.b_cptr[h.nb]) {
    err = "boundary cells determined " + std::to_string(h.cell_bndr.size()) + " != " +
          std::to_string(h.b_cptr[h.nb]) + " listed in .bc (grid_data)";
    return FVS_ERR_MESH;
  }
  // interior / boundary edges (:733-791)
  for (int i = 0; i < ne; i++) {
    if (h.ec2[i] < 0) { h.edge_bndr.push_back(i); h.bedge_cell.push_back(h.ec1[i]); }
    else h.edge_intr.push_back(i);
  }
  h.b_eptr.assign(h.nb + 1, 0);
  for (int ib = 0; ib < h.nb; ib++) {
    for (int i = h.b_cptr[ib]; i < h.b_cptr[ib + 1]; i++) {
      int ic = h.b_cell[i];
      for (int k = 0; k < h.nvrt[ic]; k++) {
        int je = h.cedge[4 * ic + k];
        if (h.ec1[je] == ic && h.ec2[je] < 0) h.b_edge.push_back(je);
      }
    }
    h.b_eptr[ib + 1] = (int)h.b_edge.size();
    int nbe = h.b_eptr[ib + 1] - h.b_eptr[ib], nbc = h.b_cptr[ib + 1] - h.b_cptr[ib];
    if (nbe != nbc) {
      err = "boundary " + std::to_string(ib + 1) + " has " + std::to_string(nbe) + " edges for " + std::to_string(nbc) +
            " cells: the reference pairs edge i with cell i (src/residual.f90:114-125)";
      return FVS_ERR_MESH;
    }
  }
  if ((int)h.b_edge.size() != (int)h.edge_bndr.size()) {
    err = "boundary edges determined " + std::to_string(h.edge_bndr.size()) + " != " + std::to_string(h.b_edge.size()) +
          " read (grid_data)";
    return FVS_ERR_MESH;
  }
  // grid_data_verify sums (:824-840)
  h.vol1 = 0.0;
  for (int ic = 0; ic < nc; ic++) h.vol1 = h.vol1 + h.vol[ic];
  h.vol2 = 0.0;
  for (int ic = 0; ic < nc; ic++) {
    double v = 0.0;
    for (int k = 0; k < h.nvrt[ic]; k++) {
      int je = h.cedge[4 * ic + k];
      double nx = h.enx[je] * h.nrmlsign[4 * ic + k];
      v = v + ((nx * h.ex[je]) * h.ea[je]);
    }
    h.vol2 = h.vol2 + v;
  }

  // gradient operator (src/gradient.f90:18-38)
  h.grad_method = o->grad_method;
  h.st_ptr.assign(nc + 1, 0);
  if (o->grad_method == FVS_GRAD_LSQ && o->lsq_stencil != FVS_LSQ_NN) {
    // setup_fn (:70-131): face neighbours, boundary slots padded with the
    // nearest cell centres that are neither the cell nor a neighbour
    for (int ic = 0; ic < nc; ic++) h.st_ptr[ic + 1] = h.st_ptr[ic] + h.nvrt[ic];
    h.st_cell.assign(h.st_ptr[nc], -1);
    std::unique_ptr<KdTree> tree;
    std::vector<KdTree::Hit> hits;
    for (int ic = 0; ic < nc; ic++) {
      const int nv = h.nvrt[ic], b = h.st_ptr[ic];
      int slots[4], nslot = 0;
      for (int k = 0; k < nv; k++) {
        int jc = h.nghbr[4 * ic + k];
        if (jc < 0) slots[nslot++] = k;
        else h.st_cell[b + k] = jc;
      }
      if (nslot == 0) continue;
      if (nslot > 2) {
        err = "setup_fn: cell " + std::to_string(ic + 1) + " has more than 2 boundary edges";
        return FVS_ERR_MESH;
      }
      if (!tree) tree.reset(new KdTree(h.xc, h.yc));
      tree->nearest(h.xc[ic], h.yc[ic], 8, hits);
      int nt = 0;
      for (int i = 0; i < 8 && nt < nslot; i++) {
        int jc = hits[i].idx;
        if (jc == ic || jc < 0) continue;
        bool used = false;
        for (int k = 0; k < nv; k++) used = used || h.nghbr[4 * ic + k] == jc;
        if (!used) h.st_cell[b + slots[nt++]] = jc;
      }
      if (nt < nslot) {
        err = "setup_fn: cell " + std::to_string(ic + 1) + " found too few padding cells";
        return FVS_ERR_MESH;
      }
    }
  } else if (o->grad_method == FVS_GRAD_LSQ) {
    // setup_nn (:214-269): sorted unique cells around the cell's nodes
    std::vector<int> tmp;
    for (int ic = 0; ic < nc; ic++) {
      tmp.clear();
      for (int k = 0; k < h.nvrt[ic]; k++) {
        int v = h.cnode[4 * ic + k];
        for (int j = h.nd_ptr[v]; j < h.nd_ptr[v + 1]; j++) if (h.nd_cell[j] != ic) tmp.push_back(h.nd_cell[j]);
      }
      std::sort(tmp.begin(), tmp.end());
      tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
      h.st_cell.insert(h.st_cell.end(), tmp.begin(), tmp.end());
      h.st_ptr[ic + 1] = (int)h.st_cell.size();
    }
  }
  if (o->grad_method == FVS_GRAD_LSQ) {
    h.st_coef.assign(2 * h.st_cell.size(), 0.0);
    h.st_w.assign(h.st_cell.size(), 0.0);
    for (int ic = 0; ic < nc; ic++)
      if (!lsq_cell_coeffs(h, ic, o->lsq_pow)) { err = "LSQ stencil longer than 64 cells"; return FVS_ERR_MESH; }
    // grad_lsq_verify (:490-529)
    const bool per = h.Lx > 0 || h.Ly > 0;
    for (int ic = 0; ic < nc; ic++) {
      double dfx = 0.0, dfy = 0.0;
      for (int k = h.st_ptr[ic]; k < h.st_ptr[ic + 1]; k++) {
        int jc = h.st_cell[k];
        double diff = per ? 1.0 * minimg(h.yc[jc] - h.yc[ic], h.Ly) + 2.0 * minimg(h.xc[jc] - h.xc[ic], h.Lx)
                          : 1.0 * h.yc[jc] + 2.0 * h.xc[jc] - (1.0 * h.yc[ic] + 2.0 * h.xc[ic]);
        dfx = dfx + h.st_coef[2 * k] * diff * h.st_w[k];
        dfy = dfy + h.st_coef[2 * k + 1] * diff * h.st_w[k];
      }
      if (std::fabs(dfx - 2.0) > 1.0e-10 || std::fabs(dfy - 1.0) > 1.0e-10) {
        char buf[200];
        std::snprintf(buf, sizeof buf, "LSQ coefficients are not correct at cell %d: df/dx=%.17g df/dy=%.17g (grad_lsq_verify)",
                      ic + 1, dfx, dfy);
        err = buf;
        return FVS_ERR_MESH;
      }
    }
  } else if (o->grad_method == FVS_GRAD_GGCB) {
    // GG-cell (src/gradient_ggcb.f90:48-110): distance-weighted face values
    for (int ic = 0; ic < nc; ic++) h.st_ptr[ic + 1] = h.st_ptr[ic] + h.nvrt[ic];
    h.st_cell.assign(h.st_ptr[nc], -1);
    h.st_coef.assign(2 * (size_t)h.st_ptr[nc], 0.0);
    h.coef0.assign(2 * (size_t)nc, 0.0);
    for (int ic = 0; ic < nc; ic++) {
      double c0x = 0.0, c0y = 0.0;
      for (int k = 0; k < h.nvrt[ic]; k++) {
        int je = h.cedge[4 * ic + k], s = h.st_ptr[ic] + k;
        double af = h.ea[je], nxf = h.enx[je] * h.nrmlsign[4 * ic + k], nyf = h.eny[je] * h.nrmlsign[4 * ic + k];
        double dx = minimg(h.ex[je] - h.xc[ic], h.Lx), dy = minimg(h.ey[je] - h.yc[ic], h.Ly);
        double d0 = std::sqrt(dx * dx + dy * dy);
        int other = ic;
        if (h.ec1[je] >= 0 && h.ec1[je] != ic) other = h.ec1[je];
        else if (h.ec2[je] >= 0 && h.ec2[je] != ic) other = h.ec2[je];
        h.st_cell[s] = other;
        dx = minimg(h.ex[je] - h.xc[other], h.Lx); dy = minimg(h.ey[je] - h.yc[other], h.Ly);
        double d1 = std::sqrt(dx * dx + dy * dy);
        c0x = c0x + d1 / (d0 + d1) * nxf * af;
        c0y = c0y + d1 / (d0 + d1) * nyf * af;
        h.st_coef[2 * s] = d0 / (d0 + d1) * nxf * af;
        h.st_coef[2 * s + 1] = d0 / (d0 + d1) * nyf * af;
      }
      h.coef0[2 * ic] = c0x; h.coef0[2 * ic + 1] = c0y;
    }
  } else {
    // GG-node (src/gradient_ggnb.f90:49-177): inverse-distance node values
    std::vector<double> idw(h.nnodes);
    for (int v = 0; v < h.nnodes; v++) {
      double idt = 0.0;
      for (int j = h.nd_ptr[v]; j < h.nd_ptr[v + 1]; j++) {
        int ic = h.nd_cell[j];
        double dx = minimg(h.xc[ic] - h.xn[v], h.Lx), dy = minimg(h.yc[ic] - h.yn[v], h.Ly);
        idt = idt + 1.0 / std::sqrt(dx * dx + dy * dy);
      }
      idw[v] = 1.0 / idt;
    }
    h.coef0.assign(2 * (size_t)nc, 0.0);
    h.coefedg.assign(8 * (size_t)nc, 0.0);
    for (int ic = 0; ic < nc; ic++) {
      double c0x = 0.0, c0y = 0.0;
      for (int k = 0; k < h.nvrt[ic]; k++) {
        int je = h.cedge[4 * ic + k];
        double af = h.ea[je], nxf = h.enx[je] * h.nrmlsign[4 * ic + k], nyf = h.eny[je] * h.nrmlsign[4 * ic + k];
        int v1 = h.en1[je], v2 = h.en2[je];
        double dx = minimg(h.xc[ic] - h.xn[v1], h.Lx), dy = minimg(h.yc[ic] - h.yn[v1], h.Ly);
        double w1 = 1.0 / std::sqrt(dx * dx + dy * dy);
        dx = minimg(h.xc[ic] - h.xn[v2], h.Lx); dy = minimg(h.yc[ic] - h.yn[v2], h.Ly);
        double w2 = 1.0 / std::sqrt(dx * dx + dy * dy);
        c0x = c0x + af * nxf / 2.0 * (w1 * idw[v1] + w2 * idw[v2]);
        c0y = c0y + af * nyf / 2.0 * (w1 * idw[v1] + w2 * idw[v2]);
      }
      h.coef0[2 * ic] = c0x; h.coef0[2 * ic + 1] = c0y;
      for (int in = 0; in < h.nvrt[ic]; in++) {
        int v = h.cnode[4 * ic + in];
        double ax = 0.0, ay = 0.0;
        for (int k = 0; k < h.nvrt[ic]; k++) {
          int je = h.cedge[4 * ic + k];
          for (int j = 0; j < 2; j++) {
            if ((j == 0 ? h.en1[je] : h.en2[je]) != v) continue;
            double af = h.ea[je], nxf = h.enx[je] * h.nrmlsign[4 * ic + k], nyf = h.eny[je] * h.nrmlsign[4 * ic + k];
            ax = ax + af * nxf / 2.0;
            ay = ay + af * nyf / 2.0;
          }
        }
        h.coefedg[8 * ic + 2 * in] = ax; h.coefedg[8 * ic + 2 * in + 1] = ay;
        for (int j = h.nd_ptr[v]; j < h.nd_ptr[v + 1]; j++) {
          int jc = h.nd_cell[j];
          double dx = minimg(h.xc[jc] - h.xn[v], h.Lx), dy = minimg(h.yc[jc] - h.yn[v], h.Ly);
          double cnb = idw[v] / std::sqrt(dx * dx + dy * dy);
          h.st_cell.push_back(jc);
          h.st_coef.push_back(jc == ic ? 0.0 : cnb);
          h.st_node.push_back((int8_t)in);
        }
      }
      h.st_ptr[ic + 1] = (int)h.st_cell.size();
    }
  }

  // limiter eps^2 = (K h)^3 with h = 2 sqrt(vol/pi) (src/gradient_limiter.f90:113-126)
  h.eps2.resize(nc);
  for (int ic = 0; ic < nc; ic++) {
    double hh = 2.0 * std::sqrt(h.vol[ic] / kPi);
    double t = (o->limiter == FVS_LIM_ALBADA ? 0.3 : 5.0) * hh;
    h.eps2[ic] = t * t * t;
  }
  // manufactured solution at cell centres (src/mms.f90:105-114)
  double mc[16];
  mms_constants(mc);
  h.mms_sol.resize(4 * (size_t)nc);
  h.mms_src.resize(4 * (size_t)nc);
  for (int ic = 0; ic < nc; ic++) mms_euler2d(mc, o->gamma, h.xc[ic], h.yc[ic], &h.mms_sol[4 * ic], &h.mms_src[4 * ic]);
  return FVS_OK;
}

// ---------------------------------------------------------------------------
// Named exports in the reference's numbering (1-based ids, 0 = none,
// 0-based CSR offsets); the same names as the CPU oracle's export table.
int export_array(const HostMesh& h, const char* name, void* dst, int64_t* nbytes) {
  const int nc = h.nc, ne = h.ne;
  int32_t* I = static_cast<int32_t*>(dst);
  double* D = static_cast<double*>(dst);
  auto want = [&](int64_t n) -> int {
    if (!dst) { *nbytes = n; return 1; }
    if (*nbytes < n) return -1;
    return 0;
  };
  auto id1 = [](int v) { return v + 1; };  // -1 -> 0
  std::string s(name);
  int r;
#define FVS_EXPORT(cond, bytes, body)            \
  if (cond) {                                    \
    if ((r = want(bytes)) != 0) return r > 0 ? FVS_OK : FVS_ERR_INVALID; \
    body;                                        \
    return FVS_OK;                               \
  }
  FVS_EXPORT(s == "cell_xy", 16LL * nc, for (int i = 0; i < nc; i++) { D[2 * i] = h.xc[i]; D[2 * i + 1] = h.yc[i]; })
  FVS_EXPORT(s == "cell_vol", 8LL * nc, for (int i = 0; i < nc; i++) D[i] = h.vol[i])
  FVS_EXPORT(s == "cell_nghbr", 16LL * nc, for (int i = 0; i < 4 * nc; i++) I[i] = (i % 4) < h.nvrt[i / 4] ? id1(h.nghbr[i]) : -1)
  FVS_EXPORT(s == "cell_nghbre", 16LL * nc, for (int i = 0; i < 4 * nc; i++) I[i] = (i % 4) < h.nvrt[i / 4] ? id1(h.nghbre[i]) : -1)
  FVS_EXPORT(s == "cell_edge", 16LL * nc, for (int i = 0; i < 4 * nc; i++) I[i] = (i % 4) < h.nvrt[i / 4] ? id1(h.cedge[i]) : -1)
  FVS_EXPORT(s == "cell_nrmlsign", 32LL * nc, for (int i = 0; i < 4 * nc; i++) D[i] = (i % 4) < h.nvrt[i / 4] ? h.nrmlsign[i] : 0.0)
  FVS_EXPORT(s == "edge_nodes", 8LL * ne, for (int i = 0; i < ne; i++) { I[2 * i] = h.en1[i] + 1; I[2 * i + 1] = h.en2[i] + 1; })
  FVS_EXPORT(s == "edge_cells", 8LL * ne, for (int i = 0; i < ne; i++) { I[2 * i] = id1(h.ec1[i]); I[2 * i + 1] = id1(h.ec2[i]); })
  FVS_EXPORT(s == "edge_geom", 56LL * ne, for (int i = 0; i < ne; i++) {
    double* g = D + 7 * i;
    g[0] = h.ex[i]; g[1] = h.ey[i]; g[2] = h.ea[i]; g[3] = h.enx[i]; g[4] = h.eny[i]; g[5] = h.etx[i]; g[6] = h.ety[i];
  })
  FVS_EXPORT(s == "edge_intr", 4LL * h.edge_intr.size(), for (size_t i = 0; i < h.edge_intr.size(); i++) I[i] = h.edge_intr[i] + 1)
  FVS_EXPORT(s == "edge_bndr", 4LL * h.edge_bndr.size(), for (size_t i = 0; i < h.edge_bndr.size(); i++) I[i] = h.edge_bndr[i] + 1)
  FVS_EXPORT(s == "bedge_cell", 4LL * h.bedge_cell.size(), for (size_t i = 0; i < h.bedge_cell.size(); i++) I[i] = h.bedge_cell[i] + 1)
  FVS_EXPORT(s == "cell_intr", 4LL * h.cell_intr.size(), for (size_t i = 0; i < h.cell_intr.size(); i++) I[i] = h.cell_intr[i] + 1)
  FVS_EXPORT(s == "cell_bndr", 4LL * h.cell_bndr.size(), for (size_t i = 0; i < h.cell_bndr.size(); i++) I[i] = h.cell_bndr[i] + 1)
  FVS_EXPORT(s == "bndry_edges", 4LL * h.b_edge.size(), for (size_t i = 0; i < h.b_edge.size(); i++) I[i] = h.b_edge[i] + 1)
  FVS_EXPORT(s == "stencil_ptr", 4LL * (nc + 1), for (int i = 0; i <= nc; i++) I[i] = h.st_ptr[i])
  FVS_EXPORT(s == "stencil_cell", 4LL * h.st_cell.size(), for (size_t i = 0; i < h.st_cell.size(); i++) I[i] = h.st_cell[i] + 1)
  FVS_EXPORT(s == "stencil_coef", 8LL * h.st_coef.size(), std::memcpy(D, h.st_coef.data(), 8 * h.st_coef.size()))
  FVS_EXPORT(s == "stencil_w" && !h.st_w.empty(), 8LL * h.st_w.size(), std::memcpy(D, h.st_w.data(), 8 * h.st_w.size()))
  FVS_EXPORT(s == "coef0" && !h.coef0.empty(), 8LL * h.coef0.size(), std::memcpy(D, h.coef0.data(), 8 * h.coef0.size()))
  FVS_EXPORT(s == "coefedg" && !h.coefedg.empty(), 8LL * h.coefedg.size(), std::memcpy(D, h.coefedg.data(), 8 * h.coefedg.size()))
  FVS_EXPORT(s == "eps2", 8LL * nc, std::memcpy(D, h.eps2.data(), 8 * (size_t)nc))
#undef FVS_EXPORT
  return FVS_ERR_INVALID;
}

}  // namespace fvs
