"""Checkpoint files in the reference's IOS layout (save / cont, .cd + .s8).

The expected control-file text below is written out from the FORMAT
statements of writecd (src/ios_unstrc.f90:229-247) and the save-file
arguments of io_init (src/io.f90:93-113); the column checks are the ones
readcd applies (src/ios_unstrc.f90:489-501).
"""
from __future__ import annotations

import struct

import numpy as np
import pytest

from fvs2d_gb300 import ios

EXPECTED_SAVE_CD = (
    "     number of nodes = 6\n"
    "     number of cells = 7\n"
    "     number of parameters =     4\n"
    "     number of timesteps  =     1\n"
    "\n"
    "     Information about file :   (  4  info lines )\n"
    "   " + "number of time-step computed =    100".ljust(72) + "\n"
    "   " + "conservatve variables are saved in cell centers".ljust(72) + "\n"
    "   " + "#ncells and #nodes are replaced".ljust(72) + "\n"
    "   " + " ".ljust(72) + "\n"
    "      Information about parameters :\n"
    "   " + "rho".ljust(72) + "\n"
    "   " + "rhou".ljust(72) + "\n"
    "   " + "rhov".ljust(72) + "\n"
    "   " + "rhoE".ljust(72) + "\n"
    "  Numbers of timesteps :\n"
    "         150\n")


def _state(n, seed=0):
    rng = np.random.default_rng(seed)
    u = rng.uniform(0.5, 2.0, (n, 4))
    u[:, 1:3] -= 1.2
    return u


def test_save_control_text_matches_the_fortran_formats(tmp_path):
    u = _state(6)
    p_cd, p_s = ios.write_save(str(tmp_path), u, nnodes=7, ntstart=51, ntimes=100)
    assert p_cd.endswith("save.cd") and p_s.endswith("save.s8")
    assert open(p_cd).read() == EXPECTED_SAVE_CD


def test_control_columns_as_readcd_reads_them():
    text = ios.format_cd(ios.ControlData(123456, 789, ["a", "b"], ["x"], list(range(1, 14))))
    L = text.split("\n")
    assert L[0][:23] == "     number of nodes = " and int(L[0][23:]) == 123456
    assert L[1][:23] == "     number of cells = " and int(L[1][23:]) == 789
    assert int(L[2][28:33]) == 2 and int(L[3][28:33]) == 13
    assert L[4] == ""
    assert int(L[5][33:36]) == 1
    # six time-step numbers per line, each (2x,i10)
    assert L[-3] == "".join(f"  {t:10d}" for t in range(7, 13))
    cd = ios.parse_cd(text)
    assert (cd.m1, cd.m2, cd.params, cd.info, cd.itimes) == (123456, 789, ["a", "b"], ["x"], list(range(1, 14)))


def test_save_records_are_big_endian_fp64_one_parameter_per_record(tmp_path):
    n = 5
    u = _state(n, 1)
    _, p_s = ios.write_save(str(tmp_path), u, nnodes=9, ntstart=1, ntimes=3)
    raw = open(p_s, "rb").read()
    assert len(raw) == 4 * n * 8  # no record markers
    for k in range(4):
        for i in range(n):
            assert raw[8 * (k * n + i):8 * (k * n + i + 1)] == struct.pack(">d", u[i, k])


def test_save_then_cont_round_trip_is_bit_exact(tmp_path):
    u = _state(37, 2)
    ios.write_save(str(tmp_path), u, nnodes=30, ntstart=1, ntimes=10, base="cont")
    v = ios.read_cont(str(tmp_path), 37, 30)
    assert np.array_equal(u, v)


def test_s4_variant_rounds_to_fp32(tmp_path):
    u = _state(11, 3)
    _, p_s = ios.write_save(str(tmp_path), u, nnodes=4, ntstart=1, ntimes=1, base="cont", imach=1)
    assert p_s.endswith(".s4")
    v = ios.read_cont(str(tmp_path), 11, 4, imach=1)
    assert np.array_equal(v, u.astype(np.float32).astype(np.float64))


def test_restart_checks(tmp_path):
    u = _state(8, 4)
    ios.write_save(str(tmp_path), u, nnodes=12, ntstart=1, ntimes=1, base="cont")
    with pytest.raises(ios.IosError, match="does not match"):
        ios.read_cont(str(tmp_path), 9, 12)
    with pytest.raises(ios.IosError, match="does not match"):
        ios.read_cont(str(tmp_path), 8, 13)
    with pytest.raises(ios.IosError, match="not found"):
        ios.read_cont(str(tmp_path), 8, 12, base="missing")
    # a file with two time steps, or not four parameters, is refused
    cd = ios.ControlData(8, 12, list(ios.SAVE_PARAMS), [], [1, 2])
    (tmp_path / "two.cd").write_text(ios.format_cd(cd))
    ios.write_records(str(tmp_path / "two.s8"), [u[:, k] for k in range(4)] * 2)
    with pytest.raises(ios.IosError, match="nt>1"):
        ios.read_cont(str(tmp_path), 8, 12, base="two")
    cd = ios.ControlData(8, 12, ["rho", "rhou", "rhov"], [], [1])
    (tmp_path / "three.cd").write_text(ios.format_cd(cd))
    ios.write_records(str(tmp_path / "three.s8"), [u[:, k] for k in range(3)])
    with pytest.raises(ios.IosError, match="parameters"):
        ios.read_cont(str(tmp_path), 8, 12, base="three")
    # a data file shorter than its control data says
    (tmp_path / "short.cd").write_text(ios.format_cd(ios.save_control(8, 12, 1, 1)))
    ios.write_records(str(tmp_path / "short.s8"), [u[:, 0]])
    with pytest.raises(ios.IosError, match="beyond the end"):
        ios.read_cont(str(tmp_path), 8, 12, base="short")
    with pytest.raises(ios.IosError, match="truncated"):
        ios.parse_cd("     number of nodes = 1\n")
