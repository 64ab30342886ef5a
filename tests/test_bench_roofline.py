"""The roofline bookkeeping of bench.py (no GPU): the algorithmic bytes per
launch on the 1,048,576-cell vortex (1,572,864 edge slots), the ideal
bytes per cell-stage of each precision, and the figures the bench line reads
from the committed ncu summary (profiles/ncu_traffic.txt)."""
import bench
from fvs2d_gb300 import PREC_FP64, PREC_FP64_DF, PREC_MIXED

NC, NE = 1048576, 1572864


def test_algorithmic_bytes_per_launch():
    # FP64 (T = 8): gradient 160 B per cell; flux 96 B per edge slot + 104 B
    # per cell; update 152 B per cell + 32 B per edge slot
    assert bench.algorithmic_bytes("gradient", NC, NE, 8) == 160 * NC
    assert bench.algorithmic_bytes("flux", NC, NE, 8) == 96 * NE + 104 * NC == 260046848
    assert bench.algorithmic_bytes("update", NC, NE, 8) == 152 * NC + 32 * NE
    # mixed (T = 4): the update's FP64 state moves 64 B per stage on average
    assert bench.algorithmic_bytes("gradient", NC, NE, 4) == 88 * NC
    assert bench.algorithmic_bytes("flux", NC, NE, 4) == 52 * NE + 52 * NC
    assert bench.algorithmic_bytes("update", NC, NE, 4) == 100 * NC + 16 * NE
    assert bench.algorithmic_bytes("other", NC, NE, 8) == 0.0


def test_ideal_stage_bytes_per_precision():
    # FP64 state (U, U0 read, U written) 96 B + cell geometry + LSQ-fn
    # coefficients + geometry of 1.5 faces
    assert bench.step_bytes(PREC_FP64) == 96 + 36 + 48 + 72 == 252
    assert bench.step_bytes(PREC_FP64_DF) == 252
    assert bench.step_bytes(PREC_MIXED) == 96 + 24 + 24 + 42 == 186


def test_committed_ncu_summary_is_read():
    for kernel in ("flux", "gradient", "update"):
        for prec in ("fp64", "mixed", "fp64_df"):
            key = f"{kernel}:{prec}"
            traffic = bench.traffic_from_profile(key)
            assert traffic is not None and traffic > 5e7, key
            frac = bench.fp64_pipe_frac(key)
            assert frac is not None and 0.0 <= frac <= 1.0, key
            assert bench.pipe_note(key), key
    # the FP64 flux is bound by the FP64 pipe, its DRAM traffic below the
    # algorithmic bytes
    assert bench.fp64_pipe_frac("flux:fp64") > 0.8
    assert bench.traffic_from_profile("flux:fp64") < bench.algorithmic_bytes("flux", NC, NE, 8)
    assert bench.traffic_from_profile("nothing:fp64") is None
