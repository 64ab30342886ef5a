"""Small seeded cases shared by the parity tests (sizes the oracle finishes in
well under a second)."""
from __future__ import annotations

import math

from fvs2d_gb300 import Options, meshgen

GAMMA = 1.4
# isentropic vortex of the benchmark cases: centre (0,0), K=5, rho=p=1,
# Mach 0.5 along +x
VORTEX = dict(vortex=True, vortex_x=0.0, vortex_y=0.0, vortex_kappa=5.0,
              vortex_inf=(1.0, 0.5 * math.sqrt(GAMMA), 0.0, 1.0))


def periodic_vortex(n=24, jitter=0.0, **kw):
    """Periodic vortex box with SSP-RK3 and a CFL-derived dt (extensions)."""
    mesh = meshgen.periodic_square(n, n, jitter=jitter)
    o = Options(**VORTEX, rk_nstages=3, rk_order=3, ssprk=True, cfl=0.8, dt_from_cfl=True)
    return mesh, o.replace(**kw)


def dirichlet_vortex(nx=20, ny=16, **kw):
    """Reference-parity variant: exact-vortex Dirichlet box, classic RK4."""
    mesh = meshgen.dirichlet_square(nx, ny, jitter=0.2)
    o = Options(**VORTEX, rk_nstages=4, rk_order=4, ssprk=False, dt=0.02)
    return mesh, o.replace(**kw)


def airfoil(nw=64, nr=24, **kw):
    """Steady transonic O-grid: slip wall + free stream, SSP-RK(4,2), local dt,
    LSQ-fn + Venkatakrishnan."""
    mesh = meshgen.naca0012_ogrid(nw, nr)
    o = Options(mach_inf=0.8, aoa_inf_deg=1.25, steady=True, cfl=1.25, rk_nstages=4, rk_order=2, ssprk=True,
                grad_method=3, lsq_stencil="fn", limiter=1, dt=0.01)
    return mesh, o.replace(**kw)


def periodic_mixed(n=18, jitter=0.2, **kw):
    """Periodic vortex on a mixed mesh: every third column of quads kept."""
    mesh = meshgen.periodic_square(n, n, jitter=jitter, quad_every=3)
    o = Options(**VORTEX, rk_nstages=3, rk_order=3, ssprk=True, cfl=0.8, dt_from_cfl=True)
    return mesh, o.replace(**kw)


def airfoil_quads(nw=64, nr=20, **kw):
    """The transonic O-grid as quadrilaterals (like the reference's example
    mesh), steady SSP-RK(4,2), LSQ-fn + Venkatakrishnan."""
    mesh = meshgen.naca0012_ogrid(nw, nr, quads=True)
    o = Options(mach_inf=0.8, aoa_inf_deg=1.25, steady=True, cfl=1.25, rk_nstages=4, rk_order=2, ssprk=True,
                grad_method=3, lsq_stencil="fn", limiter=1, dt=0.01)
    return mesh, o.replace(**kw)


def mms_box(nx=16, ny=16, **kw):
    """Manufactured-solution box (ntstart=0, Dirichlet MMS boundary)."""
    mesh = meshgen.dirichlet_square(nx, ny, x0=0.0, y0=0.0, lx=1.0, ly=1.0, jitter=0.1)
    o = Options(ntstart=0, vortex=False, rk_nstages=4, rk_order=4, dt=1e-3)
    return mesh, o.replace(**kw)
