"""CPU checks of the arithmetic two device kernels rely on, restated step for
step in Python (the GPU parity tests cover the kernels themselves):

* `ll_ldexp` (dqmc_gb300/csrc/k_ozaki.cu): a 64-bit integer v times 2^e as a
  double, on the integer units and without branches: |v| normalised to bit 63,
  the 53 high bits rounded to nearest even at bit 11, a carry out of the
  significand stepping the exponent by addition.  It must equal the correctly
  rounded float(v) * 2^e inside the exponent window -1022 <= e <= 960.
* `det_laplace` (dqmc_gb300/csrc/k_local.cu): det of a 4x4 complex matrix by
  the Laplace expansion over the 2x2 minors of rows {0, 1} and {2, 3}, with the
  lane layout of the kernel (top minors in lanes 0-5, bottom minors in lanes
  6-11, products in lanes 0-5, a three-level butterfly sum).
"""
import math
import struct

import numpy as np

MASK64 = (1 << 64) - 1


def clz64(m):
    return 64 - m.bit_length()


def ll_ldexp(v, e):
    """The kernel's steps on Python integers (64-bit wrap-around where the
    kernel relies on it)."""
    sgn = (v & MASK64) & (1 << 63)
    m = (-v if v < 0 else v) & MASK64
    lz = clz64(m) & 63
    mn = (m << lz) & MASK64
    q = mn >> 11
    rem = mn & 0x7FF
    q += 1 if (rem + (q & 1)) > 0x400 else 0
    be = 63 - lz + e + 1023
    bits = sgn | ((((be - 1) << 52) + q) & MASK64)
    if m == 0:
        return 0.0
    return struct.unpack("<d", struct.pack("<Q", bits & MASK64))[0]


def reference(v, e):
    return math.ldexp(float(v), e)   # float(int) rounds to nearest even


def test_ll_ldexp_random_and_edges():
    rng = np.random.default_rng(11)
    cases = []
    for _ in range(20000):
        nb = int(rng.integers(1, 64))
        v = int(rng.integers(0, 1 << 62)) >> (62 - min(nb, 62))
        if rng.integers(2):
            v = -v
        cases.append((v, int(rng.integers(-300, 300))))
    # ties and carries around the 53-bit boundary, powers of two, the largest magnitudes
    for sh in range(0, 11):
        base = ((1 << 53) - 1) << sh
        for d in (-(1 << max(sh - 1, 0)), -1, 0, 1, 1 << max(sh - 1, 0)):
            cases.append((base + d, 7))
            cases.append((-(base + d), -9))
    for k in range(1, 63):
        for d in (-1, 0, 1):
            cases.append(((1 << k) + d, 3))
    cases += [((1 << 63) - 1, 0), (-(1 << 63) + 1, 0), (1, -1022), (-1, 960), (0, 5)]
    for v, e in cases:
        got, want = ll_ldexp(v, e), reference(v, e)
        assert struct.pack("<d", got) == struct.pack("<d", want), (v, e, got, want)


def det_laplace_lanes(M):
    pa = [0, 0, 0, 1, 1, 2]
    pb = [1, 2, 3, 2, 3, 3]
    m = [M[l // 4, l % 4] if l < 16 else 0j for l in range(32)]
    minor = []
    for lane in range(32):
        mi = lane if lane < 12 else 0
        pr, pp = (0, mi) if mi < 6 else (2, mi - 6)
        e00, e01 = m[4 * pr + pa[pp]], m[4 * pr + pb[pp]]
        e10, e11 = m[4 * (pr + 1) + pa[pp]], m[4 * (pr + 1) + pb[pp]]
        minor.append(e00 * e11 - e01 * e10)
    term = []
    for lane in range(32):
        bc = minor[11 - lane if lane < 6 else 0]
        t = minor[lane] * bc if lane < 6 else 0j
        term.append(-t if lane in (1, 4) else t)
    for o in (4, 2, 1):
        term = [term[l] + term[l ^ o] for l in range(32)]
    return term[0]


def test_det_laplace_lane_layout():
    rng = np.random.default_rng(12)
    for _ in range(500):
        M = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
        d, ref = det_laplace_lanes(M), np.linalg.det(M)
        assert abs(d - ref) <= 1e-12 * max(1.0, abs(ref)), (d, ref)
    # M = I + Delta (I - G) near the identity, the regime of the local updates
    for _ in range(200):
        D = 0.1 * (rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))
        G = 0.5 * (rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))
        M = np.eye(4) + D @ (np.eye(4) - G)
        assert abs(det_laplace_lanes(M) - np.linalg.det(M)) <= 1e-14 * abs(np.linalg.det(M)) * 10
