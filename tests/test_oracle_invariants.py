"""Structural invariants of the CPU oracle, restated from the reference's
tests (test/tests_O3.jl:211-263, 283-332; test/tests_linalg.jl:37-60) plus
the free-fermion limit (test/tests_freefermions.jl:71-98 checks it against
ED; here against the closed form G = (1 + B_M ... B_1)^-1)."""
import dataclasses

import numpy as np
import pytest

from oracle import dqmc_ref as R


@pytest.fixture(scope="module")
def mc(golden, small_params):
    m = R.DQMCRef(small_params, golden["randconf"])
    m.init()
    return m


def test_udt_properties():
    rng = np.random.default_rng(1234)
    x = rng.random((10, 10))
    u, d, t = R.decompose_udt(x.astype(np.complex128))
    assert np.allclose(u @ u.conj().T, np.eye(10))
    assert sorted(int(np.sum(np.abs(t[:, j]) == 0)) for j in range(10)) == list(range(10))
    assert np.allclose(u @ np.diag(d) @ t, x)
    assert np.all(np.diff(d) <= 1e-12 * d[0])   # pivoting orders |R_kk|


def test_slice_matrix_inverses(mc):
    n = mc.n
    rng = np.random.default_rng(7)
    A = rng.random((n, n)) + 1j * rng.random((n, n))
    B = mc.slice_matrix(3, 1.0)
    Binv = mc.slice_matrix(3, -1.0)
    assert np.allclose(B @ Binv, np.eye(n), atol=1e-12)
    Ares = B.conj().T @ A
    assert np.allclose(mc.multiply_daggered_B_left(3, A.copy()), Ares, atol=1e-12)
    X = A.copy()
    mc.multiply_B_left(3, X)
    mc.multiply_B_inv_left(3, X)
    assert np.allclose(X, A, atol=1e-12)
    mc.multiply_B_right(3, X)
    mc.multiply_B_inv_right(3, X)
    assert np.allclose(X, A, atol=1e-12)
    assert np.allclose(mc.multiply_B_right(3, np.eye(n, dtype=complex)), B, atol=1e-14)
    assert np.allclose(mc.multiply_B_inv_right(3, np.eye(n, dtype=complex)), Binv, atol=1e-14)


def test_init_greens_matches_fresh(mc):
    # tests_O3.jl:212-213
    assert mc.current_slice == mc.M and mc.direction == -1
    assert np.max(np.abs(mc.greens - mc.calc_greens(mc.current_slice))) < 1e-12


def test_wrapping(mc):
    # tests_O3.jl:232-238
    g = mc.calc_greens(2)
    assert np.allclose(mc.wrap_greens(g, 2, 1), mc.calc_greens(3), atol=1e-12)
    assert np.allclose(mc.wrap_greens(g, 2, -1), mc.calc_greens(1), atol=1e-12)


def test_propagation_within_bounds(golden, small_params):
    # tests_O3.jl:252-263, for two directions and a stabilisation inside the chain
    p = dataclasses.replace(small_params, slices=20, safe_mult=5)
    phi = R.synthetic_field(p.N, p.slices, 11)
    m = R.DQMCRef(p, phi)
    m.init()
    m.propagate()
    steps = 0
    while not (m.current_slice == m.M and m.direction == -1):
        assert np.max(np.abs(m.calc_greens(m.current_slice) - m.greens)) < 1e-12
        m.propagate()
        steps += 1
    assert steps == 2 * m.M - 1
    assert max(d for _, _, d in m.instability) < 1e-10


def test_free_fermions_closed_form(small_params):
    p = dataclasses.replace(small_params, lambda_=0.0, slices=20)
    m = R.DQMCRef(p, R.synthetic_field(p.N, p.slices, 3))
    m.init()
    Bchain = np.eye(m.n, dtype=complex)
    for sl in range(1, m.M + 1):
        Bchain = m.slice_matrix(sl) @ Bchain
    # G(slice M) = [1 + B_{M-1}...B_1 B_M]^-1
    BM = m.slice_matrix(m.M)
    G_exact = np.linalg.inv(np.eye(m.n) + np.linalg.inv(BM) @ Bchain @ BM)
    assert np.allclose(m.greens, G_exact, atol=1e-10)


def test_local_update_consistency(mc):
    """update_greens! yields the fresh G of the updated field (Sherman-Morrison)."""
    rng = np.random.default_rng(5)
    N = mc.N
    m = R.DQMCRef(mc.p, mc.phi.copy())
    m.init()
    delta = rng.uniform(-0.2, 0.2, size=(3, N))
    rate = m.local_updates(delta, rng.uniform(size=N))
    assert 0 < rate <= 1
    assert np.max(np.abs(m.greens - m.calc_greens(m.current_slice))) < 1e-10
    assert np.isclose(m.boson_action_value, R.boson_action(m.p, m.phi), rtol=1e-12)


def test_force_formula_matches_finite_differences(small_params):
    """The adjoint force formula d log|det M|/d phi = -Re tr(G_ii E^-1 dE) and
    the boson-action gradient against central differences (h = 1e-5) of the
    log-weight parts on random entries."""
    p = dataclasses.replace(small_params, slices=10, lambda_=1.0, r=1.0, c=1.0, u=1.0)
    phi = R.synthetic_field(p.N, p.slices, 21)
    m = R.DQMCRef(p, phi)
    gl = R.force_logdetM(m)
    gb = R.force_boson(p, phi)
    rng = np.random.default_rng(22)
    h = 1e-5
    for _ in range(6):
        a, i, l = rng.integers(3), rng.integers(p.N), rng.integers(p.slices)
        vals = []
        for sgn in (1, -1):
            ph = phi.copy()
            ph[a, i, l] += sgn * h
            mm = R.DQMCRef(p, ph)
            vals.append(R.log_weight_parts(mm))
        fd_logdet = (vals[0][0] - vals[1][0]) / (2 * h)
        fd_boson = (vals[0][1] - vals[1][1]) / (2 * h)
        assert abs(gl[a, i, l] - fd_logdet) <= 1e-6 * max(1.0, abs(fd_logdet))
        assert abs(gb[a, i, l] - fd_boson) <= 1e-6 * max(1.0, abs(fd_boson))


def test_time_displaced_greens_at_safe_slices(small_params):
    """measure_tdgfs! at the safe_mult slices against the direct formulas
    G(tau, 0) = B(tau-1, 1) G0 and G(0, tau) = -(1 - G0) B(tau-1, 1)^-1
    (effective -> true), G0 = [1 + B(M, 1)]^-1 (src/fermion_measurements.jl:1343-1403,
    calc_tdgf_direct :1527-1550)."""
    p = dataclasses.replace(small_params, slices=20, safe_mult=5)
    m = R.DQMCRef(p, R.synthetic_field(p.N, p.slices, 3))
    Gt0, G0t = m.measure_tdgfs()
    n = p.n
    B = [m.slice_matrix(t) for t in range(1, p.slices + 1)]

    def chain(a, b):
        X = np.eye(n, dtype=complex)
        for t in range(b, a + 1):
            X = B[t - 1] @ X
        return X

    G0 = np.linalg.inv(np.eye(n) + chain(p.slices, 1))
    for tau in range(1, p.slices + 1, p.safe_mult):
        want = m.effective_greens2greens(chain(tau - 1, 1) @ G0)
        assert np.max(np.abs(Gt0[tau - 1] - want)) < 1e-12
        want0 = m.effective_greens2greens(-(np.eye(n) - G0) @ np.linalg.inv(chain(tau - 1, 1)))
        assert np.max(np.abs(G0t[tau - 1] - want0)) < 1e-10 * max(1.0, np.max(np.abs(want0)))


@pytest.mark.parametrize("seed", [1234, 99])
def test_udt_inversion_identities(seed):
    """tests_linalg.jl:119-174 ("UDT and UDV inversion business", well-conditioned)
    restated for the oracle: with X = U D T and Y = Uy Dy Ty from decompose_udt of
    uniform random complex matrices (the size of the reference's test G, 64 x 64),
    inv_one_plus_udt_scalettar gives (I + X)^-1 and inv_sum_udts_scalettar gives
    (X + Y)^-1 to round-off; and, with D spread over 1e-12..1e12 (the regime the
    scale separation exists for), [1 + U D T]^-1 still matches a 50-digit inverse."""
    rng = np.random.default_rng(seed)
    n = 64
    X = rng.uniform(size=(n, n)) + 1j * rng.uniform(size=(n, n))
    Y = rng.uniform(size=(n, n)) + 1j * rng.uniform(size=(n, n))
    u, d, t = R.decompose_udt(X.copy())
    uy, dy, ty = R.decompose_udt(Y.copy())
    assert np.allclose(u @ np.diag(d) @ t, X, atol=1e-12)
    assert np.allclose(R.inv_one_plus_udt_scalettar(u, d, t), np.linalg.inv(np.eye(n) + X), atol=1e-10)
    assert np.allclose(R.inv_sum_udts_scalettar(u, d, t, uy, dy, ty), np.linalg.inv(X + Y), atol=1e-10)
    # badly scaled (16 x 16): D from 1e12 to 1e-12, reference inverse in 50-digit arithmetic
    mpmath = pytest.importorskip("mpmath")
    m = 16
    us, _, ts = R.decompose_udt(X[:m, :m].copy())
    d2 = np.logspace(12, -12, m)
    mpmath.mp.dps = 50
    U = mpmath.matrix([[mpmath.mpc(z.real, z.imag) for z in row] for row in us])
    T = mpmath.matrix([[mpmath.mpc(z.real, z.imag) for z in row] for row in ts])
    Dm = mpmath.diag([mpmath.mpf(x) for x in d2])
    inv = (mpmath.eye(m) + U * Dm * T) ** -1
    want = np.array([[complex(inv[i, j]) for j in range(m)] for i in range(m)])
    got = R.inv_one_plus_udt_scalettar(us, d2, ts)
    assert np.max(np.abs(got - want)) / max(1.0, np.max(np.abs(want))) < 1e-10
