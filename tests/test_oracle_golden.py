"""Pins the CPU oracle against the reference's golden data and literal known
answers (test/tests_O3.jl, test/tests_O3_measurements.jl, test/tests_linalg.jl).
"""
import dataclasses

import numpy as np

from oracle import dqmc_ref as R


def test_lattice_tables(golden):
    # tests_O3.jl:268-272
    assert np.array_equal(R.neighbors_table(4) + 1, golden["lit_neighbors_L4"])
    assert np.array_equal(R.time_neighbors_table(10) + 1, golden["lit_time_neighbors_M10"])


def test_checkerboard_corners(golden):
    # tests_O3.jl:96
    A, B = R.four_site_corners(4)
    assert np.array_equal(A + 1, golden["lit_corners_A"])
    assert np.array_equal(B + 1, golden["lit_corners_B"])


def test_checkerboard_matrices(golden, small_params):
    # tests_O3.jl:98-111 (bit-exact: same products of cosh/sinh)
    cb = R.checkerboard_matrices(small_params)
    for g in (0, 1):
        assert np.allclose(cb[("full", False)][g].toarray(), golden[f"nob_chkr_hop{g + 1}"], rtol=0, atol=1e-15)
        assert np.allclose(cb[("full", True)][g].toarray(), golden[f"nob_chkr_hop_inv{g + 1}"], rtol=0, atol=1e-15)
        assert np.allclose(cb[("half", False)][g].toarray(), golden[f"nob_chkr_hop_half{g + 1}"], rtol=0, atol=1e-15)
        assert np.allclose(cb[("half", True)][g].toarray(), golden[f"nob_chkr_hop_half_inv{g + 1}"], rtol=0,
                           atol=1e-15)
    for key, name in (("mu", "nob_chkr_mu"), ("mu_inv", "nob_chkr_mu_inv"), ("mu_half", "nob_chkr_mu_half"),
                      ("mu_half_inv", "nob_chkr_mu_half_inv")):
        assert np.allclose(np.diag(cb[key]), golden[name], rtol=0, atol=1e-15)


def test_checkerboard_error_quadratic(small_params):
    # tests_O3.jl:75-91: |exp(-dtau/2 T) - chkr_half_A chkr_half_B sqrt(mu)| <= dtau^2
    for dt in (0.1, 0.01, 0.001, 0.0001, 0.00001):
        p = dataclasses.replace(small_params, delta_tau=dt)
        _, eT, _ = R.hopping_matrices(p)
        cb = R.checkerboard_matrices(p)
        chk = (cb[("half", False)][0] @ cb[("half", False)][1]).toarray() * np.sqrt(cb["mu"])[None, :]
        assert np.max(np.abs(eT - chk)) <= dt ** 2


def test_interaction_matrices(golden, small_params):
    # tests_O3.jl:156-163
    rc = golden["randconf"]
    assert np.allclose(R.interaction_matrix_exp(small_params, rc[:, :, 2], 1.0).toarray(), golden["nob_eVplus"],
                       rtol=0, atol=1e-15)
    assert np.allclose(R.interaction_matrix_exp(small_params, rc[:, :, 2], -1.0).toarray(), golden["nob_eVminus"],
                       rtol=0, atol=1e-15)
    assert np.allclose(R.interaction_op(small_params, golden["lit_expop_op"], 1.0), golden["nob_eVexpop"],
                       rtol=0, atol=1e-15)


def test_boson_action(golden, small_params):
    # tests_O3.jl:50-58
    rc = golden["randconf"]
    nb, tn = R.neighbors_table(4), R.time_neighbors_table(10)
    assert np.isclose(R.boson_action(small_params, rc), golden["lit_boson_action_randconf"], rtol=1e-14)
    dS = R.boson_action_diff(small_params, rc, nb, tn, 2, 9, golden["lit_new_op"])
    assert np.isclose(dS, golden["lit_boson_action_diff_site3_slice10"], rtol=1e-12)
    pe = dataclasses.replace(small_params, edrun=True)
    assert np.isclose(R.boson_action(pe, rc), golden["lit_boson_action_randconf_edrun"], rtol=1e-14)
    dS = R.boson_action_diff(pe, rc, nb, tn, 2, 9, golden["lit_new_op"])
    assert np.isclose(dS, golden["lit_boson_action_diff_site3_slice10_edrun"], rtol=1e-12)


def test_calculate_greens_kat(golden):
    # tests_O3.jl:217-227: G from stored UDTs equals the dumped greens
    G, ld = R.greens_from_udts(golden["Ul"], golden["Dl"], golden["Tl"], golden["Ur"], golden["Dr"], golden["Tr"])
    assert np.max(np.abs(G - golden["greens"])) < 1e-12
    # logdet = -sum log d (unitary and unit-triangular factors have |det| = 1)
    assert np.isfinite(ld)


def test_multiply_safely(golden):
    # tests_linalg.jl:105-113
    u, d, t = golden["B_QR_U"], golden["B_QR_D"], golden["B_QR_T"]
    U, D, T = R.multiply_safely(u, d, t, u, d, t)
    assert np.isclose(D.max(), golden["lit_msafe_maxD"], rtol=1e-10)
    assert np.isclose(D.min(), golden["lit_msafe_minD"], rtol=1e-6)


def test_boson_measurements(golden):
    # tests_O3_measurements.jl:1-9
    rc = golden["randconf"]
    assert np.allclose(R.measure_chi_dynamic(rc), golden["chi_dyn"], rtol=1e-13, atol=1e-14)
    assert np.isclose(R.measure_chi_static(rc), golden["lit_chi_static_randconf"], rtol=1e-14)
    m2, m4 = R.measure_binder_factors(rc)
    assert np.isclose(m2, golden["lit_binder_m2"], rtol=1e-14)
    assert np.isclose(m4, golden["lit_binder_m4"], rtol=1e-14)
    # measure_op literals of tests_O3_measurements.jl:7-9 (the reference's own tolerances)
    a, b = R.measure_op(rc)
    assert np.isclose(a, 0.5080018386458331, rtol=1.5e-8)
    assert np.allclose(b, [0.514548, 0.536541, 0.472916], atol=1e-4)


def _etpc_etcdc_loops(L, G):
    """Literal transcription of the reference loops (origins outer, then the
    displacement; src/fermion_measurements.jl:388-424, 592-630), pure Python."""
    N = L * L
    site = lambda x, y: (y % L) + L * (x % L)
    js = ((2, 0, 0, 2), (2, 0, 3, 1), (1, 3, 0, 2), (1, 3, 3, 1))
    Pp = np.zeros((L, L)); Pm = np.zeros((L, L))
    Cp = np.zeros((L, L), complex); Cm = np.zeros((L, L), complex)
    for x in range(L):
        for y in range(L):
            for x0 in range(L):
                for y0 in range(L):
                    r1 = site(x0 + x, y0 + y); r3 = site(x0, y0)
                    ev = []
                    for j in js:
                        i1, i2, i3, i4 = j[0] * N + r1, j[1] * N + r1, j[2] * N + r3, j[3] * N + r3
                        ev.append((G[i1, i4] * G[i2, i3] - G[i1, i3] * G[i2, i4]).real)
                    Pm[y, x] += ev[0] - ev[1] - ev[2] + ev[3]
                    Pp[y, x] += ev[0] + ev[1] + ev[2] + ev[3]
    for x0 in range(L):
        for y0 in range(L):
            for s1 in (0, 2):
                for s2 in (0, 2):
                    for x in range(L):
                        for y in range(L):
                            ri = site(x0 + x, y0 + y); r0 = site(x0, y0)

                            def ev(j1, j2, j3, j4):
                                i1, i2, i3, i4 = (j1 - 1) * N + ri, (j2 - 1) * N + ri, (j3 - 1) * N + r0, (j4 - 1) * N + r0
                                unc = (float(i1 == i2) - G[i2, i1]) * (float(i3 == i4) - G[i4, i3])
                                return unc + (float(i1 == i4) - G[i4, i1]) * G[i2, i3]
                            e1, e2 = ev(1 + s1, 1 + s1, 1 + s2, 1 + s2), ev(1 + s1, 1 + s1, 2 + s2, 2 + s2)
                            e3, e4 = ev(2 + s1, 2 + s1, 1 + s2, 1 + s2), ev(2 + s1, 2 + s1, 2 + s2, 2 + s2)
                            Cm[y, x] += e1 - e2 - e3 + e4
                            Cp[y, x] += e1 + e2 + e3 + e4
    return Pp / N, Pm / N, Cp / N, Cm / N


def test_equal_time_correlators(golden, small_params):
    """tests_O3_measurements.jl:220-249 on the reference's own G (O3.jld
    `greens`, made true by effective_greens2greens!): ETPC reflection
    symmetric within 1e-3, ETCDC imaginary parts below 1e-12 and reflection
    symmetric within 1e-3; the vectorised restatement equals a literal
    transcription of the reference loops."""
    ref = R.DQMCRef(small_params, golden["randconf"])
    g = ref.effective_greens2greens(golden["greens"])
    Pp, Pm = R.measure_etpc(4, g)
    Cp, Cm = R.measure_etcdc(4, g)
    assert R.is_reflection_symmetric(Pm, tol=1e-3) and R.is_reflection_symmetric(Pp, tol=1e-3)
    assert np.max(np.imag(Cm)) < 1e-12 and np.max(np.imag(Cp)) < 1e-12
    assert R.is_reflection_symmetric(Cm, tol=1e-3) and R.is_reflection_symmetric(Cp, tol=1e-3)
    lp, lm, lcp, lcm = _etpc_etcdc_loops(4, g)
    for a, b in ((Pp, lp), (Pm, lm), (Cp, lcp), (Cm, lcm)):
        assert np.max(np.abs(a - b)) < 1e-13


def test_zero_frequency_pairing(golden, small_params):
    """tests_O3_measurements.jl:251-268 for the reference's test configuration:
    ZFPC of the time-displaced G reflection symmetric within 1e-3, and ZFPC of
    M copies of the equal-time G equal to M times ETPC."""
    ref = R.DQMCRef(small_params, golden["randconf"])
    ref.init()
    g = ref.effective_greens2greens(ref.greens)
    Gt0, _ = ref.measure_tdgfs()
    Pp, Pm = R.measure_zfpc(4, Gt0)
    assert R.is_reflection_symmetric(Pm, tol=1e-3) and R.is_reflection_symmetric(Pp, tol=1e-3)
    M = small_params.slices
    zp, zm = R.measure_zfpc(4, [g] * M)
    ep, em = R.measure_etpc(4, g)
    assert np.allclose(zp / M, ep, rtol=1e-12, atol=1e-14) and np.allclose(zm / M, em, rtol=1e-12, atol=1e-14)


def test_zero_frequency_charge_density(golden, small_params):
    """tests_O3_measurements.jl:270-282 for the reference's test configuration:
    ZFCDC imaginary parts below 1e-12, C- reflection symmetric within 1e-3 and
    C+ within 2e-3; the vectorised restatement equals a literal transcription of
    the reference loops (tau, origin, spins, displacement)."""
    ref = R.DQMCRef(small_params, golden["randconf"])
    ref.init()
    g = ref.effective_greens2greens(ref.greens)
    Gt0, G0t = ref.measure_tdgfs()
    Cp, Cm = R.measure_zfcdc(4, g, Gt0, G0t)
    assert np.max(np.imag(Cm)) < 1e-12 and np.max(np.imag(Cp)) < 1e-12
    assert R.is_reflection_symmetric(Cm, tol=1e-3) and R.is_reflection_symmetric(Cp, tol=2e-3)
    L, N = 4, 16
    site = lambda x, y: (y % L) + L * (x % L)
    lp = np.zeros((L, L), complex); lm = np.zeros((L, L), complex)
    for tau in range(small_params.slices):
        for x0 in range(L):
            for y0 in range(L):
                for s1 in (0, 2):
                    for s2 in (0, 2):
                        for x in range(L):
                            for y in range(L):
                                ri, r0 = site(x0 + x, y0 + y), site(x0, y0)

                                def ev(j1, j3):
                                    i1, i3 = (j1 - 1) * N + ri, (j3 - 1) * N + r0
                                    unc = (1.0 - g[i1, i1]) * (1.0 - g[i3, i3])
                                    return unc + (-G0t[tau][i3, i1]) * Gt0[tau][i1, i3]
                                e1, e2 = ev(1 + s1, 1 + s2), ev(1 + s1, 2 + s2)
                                e3, e4 = ev(2 + s1, 1 + s2), ev(2 + s1, 2 + s2)
                                lm[y, x] += e1 - e2 - e3 + e4
                                lp[y, x] += e1 + e2 + e3 + e4
    assert np.max(np.abs(Cp - lp / N)) < 1e-12 and np.max(np.abs(Cm - lm / N)) < 1e-12


def test_zero_frequency_current_current(golden, small_params):
    """tests_O3_measurements.jl:286-302 for the reference's test system: Lambda_xx
    and Lambda_yy with imaginary parts below 1e-12, reflection symmetric within
    2e-3 and 1e-2.  (The superfluid-density literal of that test, 0.0515709...,
    belongs to the field that init!(mc) draws from Julia's seeded RNG and is not
    reproducible here.)  Also: rho_s from the real DFT equals the direct cosine
    sums of its definition."""
    ref = R.DQMCRef(small_params, golden["randconf"])
    ref.init()
    g = ref.effective_greens2greens(ref.greens)
    Gt0, G0t = ref.measure_tdgfs()
    T = ref.T.toarray() if hasattr(ref.T, "toarray") else np.asarray(ref.T)
    lxx, lyy = R.measure_zfccc(4, T, g, Gt0, G0t)
    assert np.max(np.imag(lxx)) < 1e-12 and np.max(np.imag(lyy)) < 1e-12
    assert R.is_reflection_symmetric(lxx, tol=2e-3) and R.is_reflection_symmetric(lyy, tol=1e-2)
    L = 4
    c = np.cos(2 * np.pi * np.arange(L) / L)
    direct = 0.25 * (np.sum(np.real(lxx) * c[None, :]) - np.sum(np.real(lxx) * c[:, None]))
    assert abs(R.measure_sfdensity(lxx) - direct) < 1e-14
