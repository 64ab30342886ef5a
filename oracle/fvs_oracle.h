/*
 * fvs_oracle.h — CPU oracle for fvs2d's residual-and-update loop.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference leg of bench.py may load this library, and only
 * as the checker.  The product (fvs2d_gb300) never links or calls it.
 *
 * It restates the Fortran reference in source loop order, with 1-based
 * arrays, built with -O2 -ffp-contract=off (no FMA contraction).  Parity
 * status: the reference ships no golden outputs and cannot be compiled
 * here (no Fortran compiler, no MPI), so parity against the reference's own
 * numbers is UNPINNED.  The oracle is pinned by the reference's built-in
 * known-answer checks: LSQ linear exactness (src/gradient_lsq.f90:490-529),
 * the Green-theorem area identity and boundary counts
 * (src/grid_procs.f90:722-728,785-791,824-840), MMS truncation error
 * decreasing with h (src/test.f90:481-519) and vortex error norms
 * (src/mms.f90:271-365).
 */
#ifndef FVS_ORACLE_H
#define FVS_ORACLE_H
#include "../include/fvs2d.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc orc;

int  orc_create(const fvs_mesh* m, const fvs_options* o, orc** out, char* err, int errlen);
void orc_destroy(orc* c);
int  orc_sizes(const orc* c, fvs_sizes* s);
int  orc_export_size(const orc* c, const char* name, int64_t* nbytes);
int  orc_export(const orc* c, const char* name, void* dst, int64_t nbytes);
int  orc_init_state(orc* c);
int  orc_set_state(orc* c, const double* cvar);
int  orc_get_state(const orc* c, double* cvar);
/* nthreads <= 1: the reference's sequential edge loop.  nthreads > 1: a
 * race-free OpenMP variant (per-edge flux buffer + per-cell gather in the
 * reference's summation order) that gives bit-identical results. */
int  orc_residual(orc* c, double time, double* resid, double* ws, int nthreads);
int  orc_get_gradient(const orc* c, double* grad, double* phi);
int  orc_wall_loads(orc* c, int ib, double* edge_out, double* loads);
int  orc_time_integration(orc* c, double t1, int nsteps, double* resnorm, int nthreads);
int  orc_vortex_error(orc* c, double time, double* err13);
int  orc_mms_source(const orc* c, double* src);
double orc_dt(const orc* c);

#ifdef __cplusplus
}
#endif
#endif
