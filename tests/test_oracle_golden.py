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
