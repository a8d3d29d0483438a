"""The erfc and exp approximations compiled into the pair kernels, read from
their source tables and evaluated on the CPU against scipy / numpy: the FP32
fit (pair_math.cuh TCP_ERFC_Q, float32 Horner as the kernels evaluate it), and
the FP64 segment erfcx and 2^(i/64) tables (erfcx64_table.inc)."""
import pathlib
import re

import numpy as np
import pytest
from scipy.special import erfc

CSRC = pathlib.Path(__file__).resolve().parents[1] / "tcp_allpair_gb300" / "csrc"
SRC = (CSRC / "pair_math.cuh").read_text()


def _floats(block):
    return [float(v.rstrip("f")) for v in re.findall(r"-?\d+\.\d+e[-+]\d+f?|-?\d+\.\d+", block)]


def fp32_table():
    p = float(re.search(r"constexpr double kErfcP = ([0-9.]+);", SRC).group(1))
    deg = int(re.search(r"constexpr int kErfcDeg = (\d+);", SRC).group(1))
    block = re.search(r"#define TCP_ERFC_Q\s*\\\s*\{(.*?)\}", SRC, re.S).group(1)
    c = _floats(block)
    assert len(c) == deg + 1
    return p, c


def test_fp32_fit_in_float32():
    p, c = fp32_table()
    x = np.linspace(0.0, 4.5, 100001).astype(np.float32)
    t = (np.float32(1.0) / (np.float32(1.0) + np.float32(p) * x)).astype(np.float32)
    q = np.full_like(t, np.float32(c[0]))
    for ck in c[1:]:   # fused multiply-add: exact product, one rounding
        q = (q.astype(np.float64) * t.astype(np.float64) + np.float64(np.float32(ck))).astype(np.float32)
    approx = np.exp(-x.astype(np.float64) ** 2) * (t.astype(np.float64) * q.astype(np.float64))
    ref = erfc(x.astype(np.float64))
    rel = np.abs(approx - ref) / ref
    assert rel.max() < 6e-7
    assert np.sqrt(np.mean(rel ** 2)) < 2e-7


def test_fp32_degree5_fit_on_the_ewald_range():
    """The degree-5 Q (TCP_ERFC5_Q, kErfc5P) of the Newton-3 kernels' Ewald
    term on [0, kErfc5Xmax], float32 Horner as the kernels evaluate it; the
    host uses it only where alpha rc <= kErfc5Xmax."""
    p = float(re.search(r"constexpr double kErfc5P = ([0-9.]+);", SRC).group(1))
    xmax = float(re.search(r"constexpr double kErfc5Xmax = ([0-9.]+);", SRC).group(1))
    deg = int(re.search(r"constexpr int kErfc5Deg = (\d+);", SRC).group(1))
    c = _floats(re.search(r"#define TCP_ERFC5_Q\s*\\\s*\{(.*?)\}", SRC, re.S).group(1))
    assert len(c) == deg + 1 and xmax >= 3.46          # covers alpha rc for a 1e-6 Ewald error
    x = np.linspace(0.0, xmax, 100001).astype(np.float32)
    t = (np.float32(1.0) / (np.float32(1.0) + np.float32(p) * x)).astype(np.float32)
    q = np.full_like(t, np.float32(c[0]))
    for ck in c[1:]:
        q = (q.astype(np.float64) * t.astype(np.float64) + np.float64(np.float32(ck))).astype(np.float32)
    approx = np.exp(-x.astype(np.float64) ** 2) * (t.astype(np.float64) * q.astype(np.float64))
    ref = erfc(x.astype(np.float64))
    rel = np.abs(approx - ref) / ref
    assert rel.max() < 1e-6
    assert np.sqrt(np.mean(rel ** 2)) < 4e-7


@pytest.mark.parametrize("y", [1e-6, 0.01, 0.1, 0.25])
def test_kelbg_close_series(y):
    """The Taylor forms of kelbg_close (pair_math.cuh) against direct FP64."""
    from scipy.special import erf
    z = np.linspace(1e-6, 0.25, 200)
    x = np.sqrt(z)
    one_m_g = -np.expm1(-y)
    ser = y * (((((-y / 720 + 1 / 120) * y - 1 / 24) * y + 1 / 6) * y - 0.5) * y + 1)
    assert abs(ser - one_m_g) / one_m_g < 1e-7
    H = [2.63393830e-05, -2.08959105e-04, 1.44663996e-03, -8.54832702e-03, 4.17918210e-02,
         -1.61197024e-01, 4.51351667e-01, -7.52252778e-01]
    block = re.search(r"float hz = (.*?)num_f", SRC, re.S).group(1)
    assert _floats(block) == pytest.approx(H, rel=1e-8)
    hz = np.polyval(H, z)
    h = x * z * hz
    href = 2 / np.sqrt(np.pi) * x * np.exp(-z) - erf(x)
    assert np.max(np.abs(h - href) / np.abs(href)) < 1e-7


def fp64_segment_tables():
    inc = (CSRC / "erfcx64_table.inc").read_text()
    deg = int(re.search(r"kEwqDeg = (\d+)", inc).group(1))
    nseg = int(re.search(r"kEwqSeg = (\d+)", inc).group(1))
    nexp = int(re.search(r"kExpTab = (\d+)", inc).group(1))
    block = re.search(r"kEwqTab\[\d+\]\[\d+\] = \{(.*?)\};", inc, re.S).group(1)
    rows = re.findall(r"\{([^{}]*)\}", block)
    tab = np.array([[float(v) for v in r.split(",")] for r in rows])
    assert tab.shape == (deg + 1, nseg)
    e2 = np.array([float(v) for v in
                   re.search(r"kExp2Tab\[\d+\] = \{(.*?)\};", inc, re.S).group(1).split(",")])
    assert len(e2) == nexp
    return tab, e2


def test_fp64_segment_ewald_q():
    """ewald_q (pair_math.cuh): Q(x) = erfcx(x) + 2x/sqrt(pi) by the degree-9
    segment polynomial at the nearest multiple of 1/8 on [0, 9]; the Ewald force
    term exp(-x^2) Q(x) and erfc(x) = exp(-x^2) (Q(x) - 2x/sqrt(pi))."""
    tab, _ = fp64_segment_tables()
    x = np.concatenate([np.linspace(0.0, 9.0, 40001), [9.0 + 1e-13]])
    j = np.rint(8.0 * x).astype(int)
    h = x - j / 8.0
    assert np.all(np.abs(h) <= 1 / 16 + 1e-15) and j.max() < tab.shape[1]
    q = tab[-1, j]
    for k in range(tab.shape[0] - 2, -1, -1):
        q = q * h + tab[k, j]
    g = np.exp(-x * x)
    c = 2.0 / np.sqrt(np.pi)
    force = erfc(x) + c * x * g
    assert np.max(np.abs(g * q - force) / force) < 2e-15
    sel = x <= 6.0
    assert np.max(np.abs(g * (q - c * x) - erfc(x))[sel] / erfc(x)[sel]) < 5e-14


def _fma(a, b, c):
    """a * b + c with one rounding (exact rationals, then the nearest double)."""
    from fractions import Fraction
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def test_fp64_table_exp():
    """exp_neg_tab (pair_math.cuh) step by step with fused multiply-adds:
    2^(k/256) (1 + p(f)) with the 2^(i/256) table, against numpy's exp on [0, 700)."""
    _, e2 = fp64_segment_tables()
    n = len(e2)
    assert n == 256 and np.max(np.abs(e2 / np.exp2(np.arange(n) / n) - 1)) < 2.3e-16
    rng = np.random.default_rng(5)
    M = 6755399441055744.0
    hi, lo = 0.0027076061740622863, 9.058776616587108e-20
    worst = 0.0
    for z in np.concatenate([rng.uniform(0.0, 80.0, 1500), rng.uniform(80.0, 699.0, 500), [0.0, 1e-300]]):
        kd = _fma(z, -369.3299304675746, M)
        k = int(kd - M)
        kf = kd - M
        f = _fma(-kf, hi, -z)
        f = _fma(-kf, lo, f)
        q = _fma(f, 1.0 / 24.0, 1.0 / 6.0)
        q = _fma(q, f, 0.5)
        q = _fma(q, f, 1.0)
        v = _fma(e2[k & 255], q * f, e2[k & 255]) * 2.0 ** (k >> 8)
        worst = max(worst, abs(v / np.exp(-z) - 1))
    assert worst < 5e-16
