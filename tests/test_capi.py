"""The C-ABI library loads and exports every entry point include/fvs2d.h
declares (no device call here), and the input-file parser mirrors input_read."""
import ctypes as C
import os
import re

import pytest

from fvs2d_gb300 import Options, capi, read_input

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:int|void|const char\*)\s+\**(fvs_\w+)\s*\(", text, flags=re.M)
    return names


def test_every_declared_symbol_is_exported():
    lib = capi.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
        assert n in capi.SIGNATURES, f"{n} missing from the ctypes table"


def test_options_default_matches_python_defaults():
    lib = capi.load()
    o = capi.FvsOptions()
    assert lib.fvs_options_default(C.byref(o)) == 0
    assert o.gamma == 1.4 and o.grad_method == 3 and o.reconst == 2 and o.rk_nstages == 4 and o.flux == 1


def test_device_calls_rejected_on_host_handle():
    from fvs2d_gb300 import meshgen
    lib = capi.load()
    m = capi.MeshArrays(meshgen.dirichlet_square(4, 4))
    o = Options().to_struct()
    h = C.c_void_p()
    assert lib.fvs_create_host(C.byref(m.struct), C.byref(o), C.byref(h)) == 0
    try:
        assert lib.fvs_init_state(h) == capi.FVS_ERR_INVALID
        assert b"host-only" in lib.fvs_last_error(h)
    finally:
        lib.fvs_destroy(h)


def test_invalid_arguments():
    lib = capi.load()
    h = C.c_void_p()
    assert lib.fvs_create(None, None, C.byref(h)) == capi.FVS_ERR_INVALID
    assert lib.fvs_last_error(None)
    assert lib.fvs_get_sizes(None, None) == capi.FVS_ERR_INVALID


INPUT_TEMPLATE = """===
\tFlow & Simulation Parameters
===
{grid}    --- Grid base file name without extension
2.e5      --- Reynolds number
{mach}       --- Free-stream Mach number
{aoa}       --- Free-stream flow angle (deg)
1.4d0     --- gamma (cp/cv)
~~~
0.01      --- Time-step: dt
4000      --- Number of total time-steps: ntimes
50        --- Number of output solutions: nsaves
{ntstart}         --- Starting time-step
{steady},1.25\t\t--- compute steady flow, CFL number
{vortex}         --- compute isentropic vortex
~~~
T,T,F,F\t\t--- Output variables(T/F): rho, u, v, p
s4\t\t\t\t--- Format for transient output files
===
\tTemporal & Spatial Discretization Schemes
===
{grad}  --- cell-center gradient scheme
{lim}         --- gradient limiter scheme
{recon}  --- face reconstruction scheme
1         --- inviscid flux scheme
~~~
4         --- Number of stages for R-K time-integration
{order}         --- Order of accuracy of R-K time-integration
{ssp}         --- Strong stability preserving formulation for R-K
"""
VORTEX_FILE = "5.0,5.0 --- x/y center\n1.0     --- Strength\n1.0     --- rho\n0.2     --- u\n0.0     --- v\n1.0     --- p\n"


def write_input(tmp_path, **kw):
    vals = dict(grid="naca0012_omesh-x", mach="0.8", aoa="1.25", ntstart="1", steady="T", vortex="F",
                grad="3,nn,0.0", lim="1", recon="2,0.3333", order="2", ssp="T")
    vals.update(kw)
    p = tmp_path / "fvs2d.input"
    p.write_text(INPUT_TEMPLATE.format(**vals))
    (tmp_path / "fvs2d.vortex").write_text(VORTEX_FILE)
    return str(p)


def test_read_input(tmp_path):
    o = read_input(write_input(tmp_path))
    assert o.grid_base == "naca0012_omesh"
    assert (o.mach_inf, o.aoa_inf_deg, o.gamma, o.dt, o.cfl) == (0.8, 1.25, 1.4, 0.01, 1.25)
    assert o.steady and not o.vortex and o.grad_method == 3 and o.lsq_stencil == "nn" and o.limiter == 1
    assert o.reconst == 2 and o.umuscl == 0.0  # kappa forced to 0 for methods 1-2 (src/input.f90:254)
    assert o.rk_nstages == 4 and o.rk_order == 2 and o.ssprk


def test_read_input_vortex_and_mms(tmp_path):
    o = read_input(write_input(tmp_path, vortex="T", steady="F", recon="3,0.3333", grad="3,fn,1.0"))
    assert o.vortex and o.vortex_x == 5.0 and o.vortex_inf == (1.0, 0.2, 0.0, 1.0)
    assert o.reconst == 3 and o.umuscl == 0.3333 and o.lsq_pow == 1.0
    o = read_input(write_input(tmp_path, vortex="T", ntstart="0"))
    assert not o.vortex  # ntstart=0 (MMS) switches the vortex off (src/input.f90:140)


@pytest.mark.parametrize("bad", [dict(grad="4,fn,0.0"), dict(grad="3,xx,0.0"), dict(lim="5"), dict(recon="4,0.0")])
def test_read_input_errors(tmp_path, bad):
    with pytest.raises(ValueError):
        read_input(write_input(tmp_path, **bad))


def test_reference_example_inputs(reference_examples):
    o = read_input(os.path.join(reference_examples, "naca0012_ogrid", "fvs2d.input"))
    assert o.grid_base == "naca0012_omesh" and o.steady and o.lsq_stencil == "nn" and o.ssprk and o.rk_order == 2
    o = read_input(os.path.join(reference_examples, "isentropic_vortex", "fvs2d.input"))
    assert o.vortex and o.grid_base == "vortex" and o.vortex_x == 5.0 and o.vortex_inf[1] == 0.2


def test_batch_rejects_invalid_descriptions():
    """fvs_batch_create checks the batch on the host before any device work:
    no cases, cases with different schemes, schemes the batched kernels do
    not run, and a broken mesh in one case (reported with its index)."""
    from fvs2d_gb300 import meshgen
    from fvs2d_gb300.batch import Batch
    from fvs2d_gb300.solver import FvsError
    lib = capi.load()
    h = C.c_void_p()
    assert lib.fvs_batch_create(None, None, 0, 0, C.byref(h)) == capi.FVS_ERR_INVALID
    assert lib.fvs_batch_last_error(None)
    m = meshgen.dirichlet_square(6, 6)
    base = Options(grad_method=3, steady=True, cfl=1.0, rk_nstages=4)
    bad = [
        ([m, m], [base, base.replace(cfl=0.5)], capi.FVS_ERR_INVALID, b"share the scheme"),
        ([m], [base.replace(grad_method=1)], capi.FVS_ERR_INVALID, b"LSQ"),
        ([m], [base.replace(rk_nstages=2)], capi.FVS_ERR_INVALID, b"stage"),
    ]
    broken = meshgen.dirichlet_square(6, 6)
    broken.tri_nodes[3, 1] = 10**6
    bad.append(([m, broken], [base, base], capi.FVS_ERR_MESH, b"case 1:"))
    for meshes, opts, code, words in bad:
        with pytest.raises(FvsError) as e:
            Batch(meshes, opts, host_threads=2)
        assert e.value.code == code, (e.value.code, str(e.value))
        assert words.decode() in str(e.value), str(e.value)
