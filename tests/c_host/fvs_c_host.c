/* fvs_c_host.c - a compiled host program driving the C-ABI of fvs2d.h the
 * way the Fortran host does through ISO_C_BINDING: it fills fvs_mesh from
 * its own arrays (1-based node and cell ids, as the reference's grid reader
 * leaves them), creates a handle, sets the state, calls the drop-in for
 * time_integration (src/runge_kutta.f90:94) and reads the state back.
 *
 * Input: a binary case file
 *   int32 nnodes, ntri, nquad, nbndries, nbcells
 *   float64 node_xy[nnodes][2]
 *   int32 tri[ntri][3], quad[nquad][4]
 *   int32 bndry_ncells[nbndries], bndry_type[nbndries], bndry_cells[nbcells]
 *   float64 mach_inf, aoa_inf_deg, dt
 *   float64 cvar[ntri + nquad][4]          initial conservative state
 * Arguments: case file, output file, number of steps, FVS_PREC_* value.
 * Output: the state after the steps as raw float64 [ncells][4] in the output
 * file, and one line per step on stdout with its four RMS(dU) norms. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "fvs2d.h"

static int read_n(FILE* f, void* p, size_t bytes) { return bytes == 0 || fread(p, 1, bytes, f) == bytes; }

static void* alloc_n(size_t bytes) { return malloc(bytes > 0 ? bytes : 1); }

int main(int argc, char** argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: %s case.bin state_out.bin nsteps precision\n", argv[0]);
    return 2;
  }
  const int nsteps = atoi(argv[3]);
  FILE* f = fopen(argv[1], "rb");
  int32_t hdr[5];
  if (!f || !read_n(f, hdr, sizeof hdr) || nsteps <= 0) {
    fprintf(stderr, "cannot read %s\n", argv[1]);
    return 2;
  }
  const int32_t nnodes = hdr[0], ntri = hdr[1], nquad = hdr[2], nb = hdr[3], nbc = hdr[4];
  const int32_t ncells = ntri + nquad;
  double* xy = alloc_n(16 * (size_t)nnodes);
  int32_t* tri = alloc_n(12 * (size_t)ntri);
  int32_t* quad = alloc_n(16 * (size_t)nquad);
  int32_t* bn = alloc_n(4 * (size_t)nb);
  int32_t* bt = alloc_n(4 * (size_t)nb);
  int32_t* bc = alloc_n(4 * (size_t)nbc);
  double flow[3];
  double* cvar = alloc_n(32 * (size_t)ncells);
  double* norms = alloc_n(32 * (size_t)nsteps);
  int ok = read_n(f, xy, 16 * (size_t)nnodes) && read_n(f, tri, 12 * (size_t)ntri) &&
           read_n(f, quad, 16 * (size_t)nquad) && read_n(f, bn, 4 * (size_t)nb) && read_n(f, bt, 4 * (size_t)nb) &&
           read_n(f, bc, 4 * (size_t)nbc) && read_n(f, flow, sizeof flow) && read_n(f, cvar, 32 * (size_t)ncells);
  fclose(f);
  if (!ok) {
    fprintf(stderr, "truncated case file %s\n", argv[1]);
    return 2;
  }

  fvs_mesh m;
  m.nnodes = nnodes;
  m.ncells_tri = ntri;
  m.ncells_quad = nquad;
  m.node_xy = xy;
  m.tri_nodes = tri;
  m.quad_nodes = nquad > 0 ? quad : NULL;
  m.nbndries = nb;
  m.bndry_ncells = bn;
  m.bndry_type = bt;
  m.bndry_cells = bc;
  m.period_x = 0.0;
  m.period_y = 0.0;

  fvs_options o;
  fvs_options_default(&o);
  o.mach_inf = flow[0];
  o.aoa_inf_deg = flow[1];
  o.dt = flow[2];
  o.steady = 0;
  o.precision = atoi(argv[4]);

  fvs_handle* h = NULL;
  int rc = fvs_create(&m, &o, &h);
  if (rc != FVS_OK) {
    fprintf(stderr, "fvs_create: %d %s\n", rc, fvs_last_error(NULL));
    return 1;
  }
  if ((rc = fvs_set_state(h, cvar)) != FVS_OK || (rc = fvs_time_integration(h, 0.0, nsteps, norms)) != FVS_OK ||
      (rc = fvs_get_state(h, cvar)) != FVS_OK) {
    fprintf(stderr, "fvs call failed: %d %s\n", rc, fvs_last_error(h));
    fvs_destroy(h);
    return 1;
  }
  fvs_destroy(h);

  FILE* g = fopen(argv[2], "wb");
  if (!g || fwrite(cvar, 32, (size_t)ncells, g) != (size_t)ncells) {
    fprintf(stderr, "cannot write %s\n", argv[2]);
    return 2;
  }
  fclose(g);
  for (int s = 0; s < nsteps; s++)
    printf("%.17g %.17g %.17g %.17g\n", norms[4 * s], norms[4 * s + 1], norms[4 * s + 2], norms[4 * s + 3]);
  free(xy);
  free(tri);
  free(quad);
  free(bn);
  free(bt);
  free(bc);
  free(cvar);
  free(norms);
  return 0;
}
