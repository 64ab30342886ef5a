"""The FP32-pair arithmetic of the device code, restated with numpy float32
(IEEE round to nearest) and checked against exact sums on the CPU: the
norm partials' block reduction (two_sum accumulation per thread, then
pair_add over a shuffle-down tree of 32 lanes and over the warps;
fvs_kernels.cuh NormAcc / block_pairs4) and the two cheaper double-float
forms of the Roe flux (dadd_s, dfma; df64.cuh), whose errors are bounded by
~2^-47 of their operands."""
import math
from fractions import Fraction

import numpy as np

F = np.float32


def two_sum_acc(h, lo, x):
    s = (h + x).astype(F)
    bp = (s - h).astype(F)
    lo = (lo + ((h - (s - bp)).astype(F) + (x - bp).astype(F)).astype(F)).astype(F)
    return s, lo


def pair_add(h, lo, h2, l2):
    s = (h + h2).astype(F)
    bp = (s - h).astype(F)
    e = (((h - (s - bp)).astype(F) + (h2 - bp).astype(F)).astype(F) + (lo + l2).astype(F)).astype(F)
    hn = (s + e).astype(F)
    return hn, (e - (hn - s).astype(F)).astype(F)


def shuffle_down_sum(h, lo):
    """32 lanes on the last axis combined as __shfl_down_sync does; lane 0."""
    for o in (16, 8, 4, 2, 1):
        h2, l2 = h.copy(), lo.copy()
        h2[..., :32 - o], l2[..., :32 - o] = h[..., o:], lo[..., o:]
        h, lo = pair_add(h, lo, h2, l2)
    return h[..., 0], lo[..., 0]


def block_sums(x, per_thread=1):
    """Block partials of 256-thread blocks as the update kernel forms them."""
    cpb = 256 * per_thread
    nb = -(-len(x) // cpb)
    xx = np.zeros(nb * cpb, F)
    xx[:len(x)] = x
    xx = xx.reshape(nb, per_thread, 256)
    h, lo = np.zeros((nb, 256), F), np.zeros((nb, 256), F)
    for j in range(per_thread):
        h, lo = two_sum_acc(h, lo, xx[:, j, :])
    hw, lw = shuffle_down_sum(h.reshape(nb, 8, 32), lo.reshape(nb, 8, 32))  # per warp
    H, L = np.zeros((nb, 32), F), np.zeros((nb, 32), F)
    H[:, :8], L[:, :8] = hw, lw
    return shuffle_down_sum(H, L)


def test_norm_pairs_sum_to_near_exact():
    rng = np.random.default_rng(7)
    n = 300_000
    # squared FP32 increments spanning six decades, as at a vortex core and
    # in the free stream around it
    x = ((rng.standard_normal(n) * 10.0 ** rng.uniform(-6, 0, n)) ** 2).astype(F)
    exact = math.fsum(float(v) for v in x)
    for per_thread in (1, 3):
        hb, lb = block_sums(x, per_thread)
        # the last block: 256 threads stride over the partials, then the tree
        nbp = -(-len(hb) // 256) * 256
        H, L = np.zeros(nbp, F), np.zeros(nbp, F)
        H[:len(hb)], L[:len(lb)] = hb, lb
        h, lo = np.zeros(256, F), np.zeros(256, F)
        for r in range(nbp // 256):
            h, lo = pair_add(h, lo, H[r * 256:(r + 1) * 256], L[r * 256:(r + 1) * 256])
        hw, lw = shuffle_down_sum(h.reshape(8, 32), lo.reshape(8, 32))
        HH, LL = np.zeros(32, F), np.zeros(32, F)
        HH[:8], LL[:8] = hw, lw
        h0, l0 = shuffle_down_sum(HH, LL)
        got = float(h0) + float(l0)
        assert abs(got - exact) <= 1e-13 * exact, (per_thread, got, exact)
    # a plain FP32 sum of the same squares is far off: the pairs are needed
    assert abs(float(np.sum(x, dtype=F)) - exact) > 1e-8 * exact


def split(v):
    hi = np.float32(v)
    return hi, np.float32(v - float(hi))


def exact(h, lo):
    return Fraction(float(h)) + Fraction(float(lo))


def fmaf(a, b, c):
    """IEEE fused multiply-add in FP32, by exact rationals."""
    return np.float32(float(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))))


def fast_two_sum(a, b):
    s = np.float32(a + b)
    return s, np.float32(b - np.float32(s - a))


def two_sum(a, b):
    s = np.float32(a + b)
    bp = np.float32(s - a)
    return s, np.float32(np.float32(a - np.float32(s - bp)) + np.float32(b - bp))


def dadd_s(a, b):
    s, e = two_sum(a[0], b[0])
    return fast_two_sum(s, np.float32(e + np.float32(a[1] + b[1])))


def dfma(a, b, c):
    p = np.float32(a[0] * b[0])
    pe = fmaf(a[0], b[0], -p)
    cross = fmaf(a[0], b[1], np.float32(a[1] * b[0]))
    s, e = two_sum(p, c[0])
    return fast_two_sum(s, np.float32(e + np.float32(np.float32(pe + cross) + c[1])))


def test_sloppy_sum_and_fused_multiply_add_bounds():
    rng = np.random.default_rng(11)
    tol = 2.0 ** -46
    for _ in range(1500):
        a = split(rng.standard_normal() * 10.0 ** rng.uniform(-3, 3))
        b = split(rng.standard_normal() * 10.0 ** rng.uniform(-3, 3))
        c = split(rng.standard_normal() * 10.0 ** rng.uniform(-3, 3))
        ea, eb, ec = exact(*a), exact(*b), exact(*c)
        s = dadd_s(a, b)
        assert abs(exact(*s) - (ea + eb)) <= tol * (abs(ea) + abs(eb))
        f = dfma(a, b, c)
        assert abs(exact(*f) - (ea * eb + ec)) <= tol * (abs(ea * eb) + abs(ec))
        # like-signed sums (the only kind the flux gives dadd_s): relative
        # to the result as well
        pa = (a[0], a[1]) if a[0] >= 0 else (-a[0], -a[1])
        pb = (b[0], b[1]) if b[0] >= 0 else (-b[0], -b[1])
        s2 = dadd_s(pa, pb)
        exact_like = abs(ea) + abs(eb)
        assert abs(exact(*s2) - exact_like) <= tol * exact_like
