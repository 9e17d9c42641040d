"""Parity of the CUDA library (through the C ABI) with the CPU oracle.

Tolerances: FP64 results must agree with the oracle within 1e-10 relative
(max-norm, relative to max |G| = O(1)); accept/reject sequences and the final
field must be identical wherever the acceptance margin |p_acc - u| exceeds
1e-9 (both codes compute p_acc in FP64 with different summation orders).
"""
import dataclasses

import numpy as np
import pytest

from oracle import dqmc_ref as R

pytestmark = pytest.mark.gpu

TOL = 1e-10


def relerr(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(1.0, float(np.max(np.abs(b)))))


def api_params(p: R.Params, all_checks=True, greens_method="scales"):
    from dqmc_gb300.api import ModelParams
    return ModelParams(L=p.L, slices=p.slices, safe_mult=p.safe_mult, delta_tau=p.delta_tau, lambda_=p.lambda_,
                       r=p.r, c=p.c, u=p.u, mu1=p.mu1, mu2=p.mu2, hoppings=tuple(p.hoppings), box=p.box,
                       all_checks=all_checks, greens_method=greens_method)


# calculate_greens formulations: D-scale separation with one LU (default) and
# the reference's two pivoted QRs; both must reproduce the oracle
METHODS = ["scales", "two_qr"]


@pytest.fixture(scope="module")
def lib():
    from dqmc_gb300 import build
    build.build()
    from dqmc_gb300 import api
    return api


# the L=4, beta=4 (M=40) workload: lambda=1, r=c=u=1, box 0.2
P_L4 = R.Params(L=4, slices=40, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5, mu2=-0.5,
              box=0.2)


def test_multiply_B_all_modes(lib, golden, small_params):
    p = small_params
    ref = R.DQMCRef(p, golden["randconf"])
    gpu = lib.DQMC(api_params(p), golden["randconf"])
    rng = np.random.default_rng(1)
    A = rng.standard_normal((p.n, p.n)) + 1j * rng.standard_normal((p.n, p.n))
    for sl in (1, 3, 10):
        for name in ("multiply_B_left", "multiply_B_right", "multiply_B_inv_left", "multiply_B_inv_right",
                     "multiply_daggered_B_left"):
            want = getattr(ref, name)(sl, A.copy())
            got = getattr(gpu, name)(sl, A)
            assert relerr(got, want) < 1e-13, (sl, name, relerr(got, want))


@pytest.mark.parametrize("method", METHODS)
def test_calculate_greens_kat(lib, golden, small_params, method):
    # tests_O3.jl:217-227 through the C ABI
    gpu = lib.DQMC(api_params(small_params, greens_method=method), golden["randconf"])
    G, ld = gpu.calculate_greens_udt(golden["Ul"], golden["Dl"], golden["Tl"], golden["Ur"], golden["Dr"],
                                     golden["Tr"])
    assert relerr(G, golden["greens"]) < TOL
    _, ld_ref = R.greens_from_udts(golden["Ul"], golden["Dl"], golden["Tl"], golden["Ur"], golden["Dr"],
                                   golden["Tr"])
    assert abs(ld - ld_ref) < 1e-9 * max(1.0, abs(ld_ref))


def test_decompose_udt(lib, small_params):
    gpu = lib.DQMC(api_params(small_params), R.synthetic_field(16, 10, 0))
    rng = np.random.default_rng(3)
    n = small_params.n
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * np.logspace(0, 12, n)[None, :]
    U, D, T = gpu.decompose_udt(A)
    Ur, Dr, Tr = R.decompose_udt(A)
    assert np.allclose(U.conj().T @ U, np.eye(n), atol=1e-13)
    assert np.allclose((U * D[None, :]) @ T, A, rtol=0, atol=1e-12 * np.max(np.abs(A)))
    assert np.allclose(D, Dr, rtol=1e-10)
    assert np.allclose(np.abs(T), np.abs(Tr), atol=1e-10)


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("cfg", ["small", "l4"])
def test_init_and_full_propagation(lib, golden, small_params, cfg, method):
    p = small_params if cfg == "small" else P_L4
    phi = golden["randconf"] if cfg == "small" else R.synthetic_field(p.N, p.slices, 100)
    ref = R.DQMCRef(p, phi)
    ref.init()
    gpu = lib.DQMC(api_params(p, greens_method=method), phi)
    gpu.init()
    assert gpu.state == (ref.current_slice, ref.direction)
    assert relerr(gpu.greens, ref.greens) < TOL
    assert abs(gpu.log_det - ref.log_det) < 1e-9 * max(1.0, abs(ref.log_det))
    # one full down + up pass, G compared at every slice (tests_O3.jl:252-263)
    for _ in range(2 * p.slices):
        ref.propagate()
        gpu.propagate()
        assert gpu.state == (ref.current_slice, ref.direction)
        assert relerr(gpu.greens, ref.greens) < TOL, gpu.state


@pytest.mark.parametrize("method", METHODS)
def test_calc_greens_from_scratch(lib, golden, small_params, method):
    p = P_L4
    phi = R.synthetic_field(p.N, p.slices, 5)
    ref = R.DQMCRef(p, phi)
    gpu = lib.DQMC(api_params(p, greens_method=method), phi)
    gpu.init()
    for sl in (1, 7, 20, 40):
        G, ld = gpu.calc_greens_and_logdet(sl)
        Gr, ldr = ref.calc_greens_and_logdet(sl)
        assert relerr(G, Gr) < TOL
        assert abs(ld - ldr) < 1e-9 * max(1.0, abs(ldr))


def test_wrap_greens(lib, small_params):
    p = P_L4
    phi = R.synthetic_field(p.N, p.slices, 6)
    ref = R.DQMCRef(p, phi)
    gpu = lib.DQMC(api_params(p), phi)
    gpu.init()
    g = ref.calc_greens(12)
    for d in (1, -1):
        assert relerr(gpu.wrap_greens(g, 12, d), ref.wrap_greens(g, 12, d)) < 1e-13


def _compare_updates(ref, gpu, delta, u, margin=1e-9):
    rate_g, acc_g, det_g, pacc_g = gpu.local_updates(delta, u, return_details=True)
    rec = []
    rate_r = ref.local_updates(delta, u, record=rec)
    acc_r = np.array([r[2] for r in rec])
    det_r = np.array([r[3] for r in rec])
    pacc_r = np.array([r[4] for r in rec])
    safe = np.abs(pacc_r - u) > margin
    assert np.array_equal(acc_g[safe], acc_r[safe])
    assert np.allclose(det_g, det_r, rtol=1e-10, atol=0)
    return rate_g, rate_r


def test_local_updates_one_slice(lib, golden, small_params):
    p = dataclasses.replace(P_L4)
    phi = R.synthetic_field(p.N, p.slices, 7)
    ref = R.DQMCRef(p, phi)
    ref.init()
    gpu = lib.DQMC(api_params(p), phi)
    gpu.init()
    delta, u = R.synthetic_streams(p.N, 1, p.box, 8)
    _compare_updates(ref, gpu, delta[0], u[0])
    assert relerr(gpu.greens, ref.greens) < TOL
    assert np.array_equal(gpu.get_field(), ref.phi)
    assert abs(gpu.boson_action - ref.boson_action_value) < 1e-10 * abs(ref.boson_action_value)


@pytest.mark.parametrize("delay,method", [(1, "scales"), (4, "scales"), (8, "scales"), (16, "scales"),
                                          (32, "scales"), (1, "two_qr"), (16, "two_qr")])
def test_sweep_l4_accept_sequence(lib, delay, method):
    """L=4, beta=4: one full sweep (M update calls) on shared streams, with
    immediate rank-4 updates (delay 1) and delayed rank-k updates."""
    p = P_L4
    phi = R.synthetic_field(p.N, p.slices, 2024)
    delta, u = R.synthetic_streams(p.N, p.slices, p.box, 2025)
    ref = R.DQMCRef(p, phi)
    ref.init()
    rec = []
    ref.sweep(p.slices, delta, u, record=rec)
    mp = api_params(p, greens_method=method)
    mp.delay = delay
    gpu = lib.DQMC(mp, phi)
    gpu.init()
    res = gpu.sweep(p.slices, delta, u, return_accepted=True)
    acc_r = np.array([r[2] for r in rec]).reshape(p.slices, p.N)
    margin = np.abs(np.array([r[4] - r[5] for r in rec])).reshape(p.slices, p.N)
    assert np.array_equal(res["accepted_mask"], acc_r), f"min margin {margin.min():.3e}"
    assert np.array_equal(gpu.get_field(), ref.phi)
    assert relerr(gpu.greens, ref.greens) < TOL
    assert gpu.state == (ref.current_slice, ref.direction)
    assert res["max_instability"] < 1e-7
    assert abs(gpu.boson_action - ref.boson_action_value) < 1e-10 * abs(ref.boson_action_value)


@pytest.mark.parametrize("delay", [1, 16])
def test_sweep_l10_shapes(lib, delay):
    """L=10, M=100: 15 update calls crossing a stabilisation,
    immediate and delayed (k = 16) updates."""
    p = R.Params(L=10, slices=100, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5,
                 mu2=-0.5, box=0.2)
    calls = 15
    phi = R.synthetic_field(p.N, p.slices, 31)
    delta, u = R.synthetic_streams(p.N, calls, p.box, 32)
    ref = R.DQMCRef(p, phi)
    ref.init()
    rec = []
    ref.sweep(calls, delta, u, record=rec)
    mp = api_params(p)
    mp.delay = delay
    gpu = lib.DQMC(mp, phi)
    gpu.init()
    res = gpu.sweep(calls, delta, u, return_accepted=True)
    acc_r = np.array([r[2] for r in rec]).reshape(calls, p.N)
    assert np.array_equal(res["accepted_mask"], acc_r)
    assert np.array_equal(gpu.get_field(), ref.phi)
    assert relerr(gpu.greens, ref.greens) < TOL


def test_measurement_hook(lib):
    p = P_L4
    phi = R.synthetic_field(p.N, p.slices, 77)
    ref = R.DQMCRef(p, phi)
    ref.init()
    gpu = lib.DQMC(api_params(p), phi)
    gpu.init()
    m = gpu.measure()
    Gt = ref.measured_greens()
    assert relerr(m["greens"], Gt) < TOL
    assert abs(m["occupation"] - float(np.mean(1 - np.diag(Gt)).real)) < 1e-12
    assert abs(m["e_kin"] - ref.kinetic_energy(Gt)) < 1e-10 * max(1.0, abs(ref.kinetic_energy(Gt)))


# ---------------------------------------------------------------------------
# mixed-precision form (split-BF16 tensor-core GEMMs)
# ---------------------------------------------------------------------------
MIXED_TOL = 1e-8   # max |G_mixed - G_FP64| target of the mixed form


@pytest.mark.parametrize("L", [4, 16])
def test_split_bf16_gemm_accuracy(lib, L):
    from dqmc_gb300.api import ModelParams
    p = ModelParams(L=L, slices=10, safe_mult=10, precision="mixed")
    gpu = lib.DQMC(p, R.synthetic_field(p.N, p.slices, 9))
    n = p.n
    rng = np.random.default_rng(11)
    # rows and columns over many decades, as in the UDT products
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * np.logspace(-8, 8, n)[:, None]
    B = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * np.logspace(5, -5, n)[None, :]
    C_ref = A @ B
    C_fp64 = gpu.gemm_check(A, B, 0)
    C_oz = gpu.gemm_check(A, B, 1)
    scale = np.abs(A) @ np.abs(B)                       # elementwise error scale
    assert np.max(np.abs(C_fp64 - C_ref) / scale) < 1e-14
    assert np.max(np.abs(C_oz - C_ref) / scale) < 1e-8


@pytest.mark.parametrize("delay", [1, 16])
def test_mixed_sweep_matches_fp64(lib, delay):
    p = P_L4
    phi = R.synthetic_field(p.N, p.slices, 555)
    delta, u = R.synthetic_streams(p.N, p.slices, p.box, 556)
    ref = R.DQMCRef(p, phi)
    ref.init()
    rec = []
    ref.sweep(p.slices, delta, u, record=rec)
    mp = api_params(p)
    mp.precision = "mixed"
    mp.delay = delay
    gpu = lib.DQMC(mp, phi)
    gpu.init()
    res = gpu.sweep(p.slices, delta, u, return_accepted=True)
    acc_r = np.array([r[2] for r in rec]).reshape(p.slices, p.N)
    margin = np.abs(np.array([r[4] - r[5] for r in rec])).reshape(p.slices, p.N)
    # the accept sequence must be identical; a flip is reported with its margin
    if not np.array_equal(res["accepted_mask"], acc_r):
        c, i = np.argwhere(res["accepted_mask"] != acc_r)[0]
        pytest.fail(f"first flip at call {c}, site {i}: margin |p_acc - u| = {margin[c, i]:.3e}")
    assert np.array_equal(gpu.get_field(), ref.phi)
    assert relerr(gpu.greens, ref.greens) < MIXED_TOL


def test_mixed_l10_greens_error(lib):
    """Mixed form at L=10, M=100: |G_mixed - G_FP64| after 15 update calls
    (delayed k = 16) with the accept sequences compared where the margin is
    above the mixed-form error."""
    p = R.Params(L=10, slices=100, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5,
                 mu2=-0.5, box=0.2)
    calls = 15
    phi = R.synthetic_field(p.N, p.slices, 31)
    delta, u = R.synthetic_streams(p.N, calls, p.box, 32)
    out = {}
    for prec in ("fp64", "mixed"):
        mp = api_params(p)
        mp.precision = prec
        mp.delay = 16
        g = lib.DQMC(mp, phi)
        g.init()
        res = g.sweep(calls, delta, u, return_accepted=True)
        out[prec] = (g.greens, res["accepted_mask"], g.get_field())
        g.close()
    assert np.array_equal(out["fp64"][1], out["mixed"][1])
    assert relerr(out["mixed"][0], out["fp64"][0]) < MIXED_TOL


# ---------------------------------------------------------------------------
# adjoint force (gradient of log|det M| and S_boson)
# ---------------------------------------------------------------------------
def test_force_matches_oracle(lib):
    p = R.Params(L=4, slices=20, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5,
                 mu2=-0.5, box=0.2)
    phi = R.synthetic_field(p.N, p.slices, 61)
    gpu = lib.DQMC(api_params(p), phi)
    gpu.init()
    gl, gb = gpu.force()
    assert gpu.state == (p.slices, -1)
    ref = R.DQMCRef(p, phi)
    gl_r = R.force_logdetM(ref)
    gb_r = R.force_boson(p, phi)
    assert np.max(np.abs(gl - gl_r)) < 1e-10 * max(1.0, np.max(np.abs(gl_r)))
    assert np.max(np.abs(gb - gb_r)) < 1e-12 * max(1.0, np.max(np.abs(gb_r)))


def test_force_l12_finite_differences(lib):
    """L=12, beta=10 (M=100): the adjoint force against
    central differences (h=1e-5) of log|det M| = -log|det G| computed from
    scratch by the library, on 200 random entries (1e-6 relative)."""
    p = R.Params(L=12, slices=100, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5,
                 mu2=-0.5, box=0.2)
    phi = R.synthetic_field(p.N, p.slices, 71)
    gpu = lib.DQMC(api_params(p), phi)
    gpu.init()
    gl, gb = gpu.force()
    rng = np.random.default_rng(72)
    h = 1e-5
    for _ in range(200):
        a, i, l = rng.integers(3), rng.integers(p.N), rng.integers(p.slices)
        f = []
        for sgn in (1, -1):
            ph = phi.copy()
            ph[a, i, l] += sgn * h
            gpu.set_field(ph)
            _, ld = gpu.calc_greens_and_logdet(1)
            f.append(-ld)
        fd = (f[0] - f[1]) / (2 * h)
        assert abs(gl[a, i, l] - fd) <= 1e-6 * max(1.0, abs(fd)), (a, i, l, gl[a, i, l], fd)


def test_langevin_steps(lib):
    """100 Langevin steps (eps = 1e-3) on S_b - log|det M| with a local sweep
    after every 10th (the L=12 schedule, here at L=4, M=40): the field stays
    finite and the tracked boson action matches a recomputation."""
    p = P_L4
    gpu = lib.DQMC(api_params(p), R.synthetic_field(p.N, p.slices, 81))
    gpu.init()
    rng = np.random.default_rng(82)
    delta, u = R.synthetic_streams(p.N, 10 * p.slices, p.box, 83)
    for step in range(100):
        phi = gpu.langevin_step(1e-3, rng)
        assert np.all(np.isfinite(phi))
        if step % 10 == 9:
            k = step // 10
            gpu.sweep(p.slices, delta[k * p.slices:(k + 1) * p.slices], u[k * p.slices:(k + 1) * p.slices])
            gpu.init(gpu.get_field())
    assert np.isfinite(gpu.log_det)
    assert abs(gpu.boson_action - R.boson_action(p, gpu.get_field())) < 1e-9 * abs(gpu.boson_action)


# ---------------------------------------------------------------------------
# global update (src/global_updates.jl:18-58)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("force_accept", [True, False])
def test_global_update(lib, force_accept):
    p = P_L4
    phi = R.synthetic_field(p.N, p.slices, 91)
    shift = np.array([0.05, -0.03, 0.02])
    u = 0.0 if force_accept else 1.0 - 1e-15
    ref = R.DQMCRef(p, phi)
    ref.init()
    acc_r, pacc_r = ref.global_update(shift, u)
    gpu = lib.DQMC(api_params(p), phi)
    gpu.init()
    acc_g, pacc_g = gpu.global_update(shift, u)
    assert abs(pacc_g - pacc_r) < 1e-9 * max(1.0, pacc_r)
    if pacc_r < 1.0 - 1e-9:
        assert acc_g == acc_r == force_accept
    assert np.allclose(gpu.get_field(), ref.phi, rtol=0, atol=1e-15)
    assert relerr(gpu.greens, ref.greens) < TOL
    assert abs(gpu.boson_action - ref.boson_action_value) < 1e-10 * abs(ref.boson_action_value)
    # the sweep continues from the (possibly restored) state
    delta, uu = R.synthetic_streams(p.N, 3, p.box, 92)
    ref.sweep(3, delta, uu)
    gpu.sweep(3, delta, uu)
    assert relerr(gpu.greens, ref.greens) < TOL


# ---------------------------------------------------------------------------
# batches of independent chains (dqmc_batch_*)
# ---------------------------------------------------------------------------
def test_batch_matches_single_chains(lib):
    """Three chains of different sizes swept concurrently give exactly the
    results of the same chains swept one by one."""
    torch = pytest.importorskip("torch")
    sizes = [4, 6, 4]
    M, calls = 20, 20
    plist, fields, streams = [], [], []
    for k, L in enumerate(sizes):
        p = R.Params(L=L, slices=M, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5,
                     mu2=-0.5, box=0.2)
        plist.append(p)
        fields.append(R.synthetic_field(p.N, M, 300 + k))
        streams.append(R.synthetic_streams(p.N, calls, p.box, 400 + k))
    batch = lib.Batch([api_params(p) for p in plist], fields)
    batch.init()
    dev_d, dev_u = [], []
    for p, (delta, u) in zip(plist, streams):
        d = np.ascontiguousarray(np.transpose(delta, (0, 2, 1)))
        dev_d.append(torch.from_numpy(d).cuda())
        dev_u.append(torch.from_numpy(np.ascontiguousarray(u)).cuda())
    torch.cuda.synchronize()
    stats = batch.sweep_device(calls, [t.data_ptr() for t in dev_d], [t.data_ptr() for t in dev_u])
    for k, p in enumerate(plist):
        single = lib.DQMC(api_params(p), fields[k])
        single.init()
        res = single.sweep(calls, streams[k][0], streams[k][1])
        assert stats[k]["accepted"] == res["accepted"]
        assert relerr(batch.chains[k].greens, single.greens) < 1e-12
        assert np.array_equal(batch.chains[k].get_field(), single.get_field())
        single.close()
    batch.close()


def _tdgf_params(cfg, small_params):
    # ref_test: the reference's test system (M = safe_mult = 10), where fill_tdgf!
    # propagates slices 6..10 from the not yet filled (zero) slice 5
    return {"small": dataclasses.replace(small_params, slices=20, safe_mult=5), "ref_test": small_params,
            "l4": P_L4}[cfg]


@pytest.mark.parametrize("cfg,prec", [("small", "fp64"), ("ref_test", "fp64"), ("l4", "fp64"), ("l4", "mixed")])
def test_time_displaced_greens(lib, golden, small_params, cfg, prec):
    """measure_tdgfs! (time-displaced G(tau, 0) and -G(0, tau) for every slice)
    against the oracle's restatement; mixed form within 1e-8."""
    p = _tdgf_params(cfg, small_params)
    phi = R.synthetic_field(p.N, p.slices, 41)
    ref = R.DQMCRef(p, phi)
    gt0_r, g0t_r = ref.measure_tdgfs()
    mp = api_params(p)
    mp.precision = prec
    gpu = lib.DQMC(mp, phi)
    gpu.init()
    gt0, g0t = gpu.measure_tdgfs()
    tol = TOL if prec == "fp64" else 1e-8
    for tau in range(p.slices):
        assert relerr(gt0[tau], gt0_r[tau]) < tol, (tau, relerr(gt0[tau], gt0_r[tau]))
        assert relerr(g0t[tau], g0t_r[tau]) < tol, (tau, relerr(g0t[tau], g0t_r[tau]))


@pytest.mark.parametrize("tune", ["lu_small=0", "lu_small=0,lu_cluster=16", "lu_small=0,lu_cluster=8",
                                  "lu_small=4096"])
@pytest.mark.parametrize("L,prec", [(6, "fp64"), (10, "fp64"), (10, "mixed")])
def test_lu_blocked_and_unblocked(lib, monkeypatch, tune, L, prec):
    """calculate_greens through the blocked LU (panels of 64 columns, ragged last
    panel at n = 400; the panels on a cluster of 16 or 8 CTAs, or on the
    cooperative grid) and through the unblocked cooperative LU, selected per
    handle by DQMC_TUNE; all reproduce the oracle (1e-10 FP64, 1e-8 mixed)."""
    monkeypatch.setenv("DQMC_TUNE", tune)
    p = dataclasses.replace(P_L4, L=L, slices=20)
    phi = R.synthetic_field(p.N, p.slices, 31 + L)
    ref = R.DQMCRef(p, phi)
    prm = api_params(p)
    prm.precision = prec
    gpu = lib.DQMC(prm, phi)
    try:
        gpu.init()
        tol = TOL if prec == "fp64" else 1e-8
        for sl in (1, 10, 20):
            G, ld = gpu.calc_greens_and_logdet(sl)
            Gr, ldr = ref.calc_greens_and_logdet(sl)
            assert relerr(G, Gr) < tol
            assert abs(ld - ldr) < 10 * tol * max(1.0, abs(ldr))
    finally:
        gpu.close()


@pytest.mark.parametrize("L", [4, 8])
def test_equal_time_correlators(lib, L):
    """dqmc_measure_equal_time against the oracle's measure_etpc / measure_etcdc
    (src/fermion_measurements.jl:388-424, 592-630): on a given true G and on
    the measurement hook's G of the current slice (1e-12 and 1e-10 relative)."""
    p = dataclasses.replace(P_L4, L=L, slices=20)
    phi = R.synthetic_field(p.N, p.slices, 71 + L)
    ref = R.DQMCRef(p, phi)
    ref.init()
    gpu = lib.DQMC(api_params(p), phi)
    try:
        gpu.init()
        g_true = ref.measured_greens()
        want = R.measure_etpc(L, g_true) + R.measure_etcdc(L, g_true)
        # given G: only the summation order differs; hook G: the GPU's own G (TOL)
        for got, tol in ((gpu.measure_equal_time(g_true), 1e-12), (gpu.measure_equal_time(), TOL)):
            for a, b in zip(got, want):
                assert relerr(a, b) < tol
    finally:
        gpu.close()


@pytest.mark.parametrize("cfg", ["ref_test", "l4"])
def test_zero_frequency_pairing(lib, small_params, cfg):
    """dqmc_measure_zfpc (measure_zfpc!, src/fermion_measurements.jl:500-541) on
    the device's own G(tau, 0) and on the oracle's G(tau, 0) passed in,
    against the oracle (1e-10 relative)."""
    p = _tdgf_params(cfg, small_params)
    phi = R.synthetic_field(p.N, p.slices, 43)
    ref = R.DQMCRef(p, phi)
    gt0_r, _ = ref.measure_tdgfs()
    want = R.measure_zfpc(p.L, gt0_r)
    gpu = lib.DQMC(api_params(p), phi)
    try:
        gpu.init()
        for got in (gpu.measure_zfpc(), gpu.measure_zfpc(gt0_r)):
            for a, b in zip(got, want):
                assert relerr(a, b) < TOL
    finally:
        gpu.close()


@pytest.mark.parametrize("cfg", ["ref_test", "l4"])
def test_zero_frequency_charge_density(lib, small_params, cfg):
    """dqmc_measure_zfcdc (measure_zfcdc!, src/fermion_measurements.jl:688-743):
    all inputs on the device (hook G, device time-displaced G) against the
    oracle (1e-10 relative), and the oracle's inputs passed in (1e-12)."""
    p = _tdgf_params(cfg, small_params)
    phi = R.synthetic_field(p.N, p.slices, 47)
    ref = R.DQMCRef(p, phi)
    ref.init()
    g = ref.measured_greens()
    gt0_r, g0t_r = ref.measure_tdgfs()
    want = R.measure_zfcdc(p.L, g, gt0_r, g0t_r)
    gpu = lib.DQMC(api_params(p), phi)
    try:
        gpu.init()
        for got, tol in ((gpu.measure_zfcdc(), TOL), (gpu.measure_zfcdc(g, gt0_r, g0t_r), 1e-12)):
            for a, b in zip(got, want):
                assert relerr(a, b) < tol
    finally:
        gpu.close()


@pytest.mark.parametrize("cfg", ["ref_test", "l4"])
def test_zero_frequency_current_current(lib, small_params, cfg):
    """dqmc_measure_zfccc (measure_zfccc!, src/fermion_measurements.jl:814-888,
    and measure_sfdensity :911-920) against the oracle: all inputs on the device
    (1e-10 relative) and the oracle's inputs passed in (1e-12)."""
    p = _tdgf_params(cfg, small_params)
    phi = R.synthetic_field(p.N, p.slices, 53)
    ref = R.DQMCRef(p, phi)
    ref.init()
    g = ref.measured_greens()
    gt0_r, g0t_r = ref.measure_tdgfs()
    T = ref.T.toarray() if hasattr(ref.T, "toarray") else np.asarray(ref.T)
    lxx_r, lyy_r = R.measure_zfccc(p.L, T, g, gt0_r, g0t_r)
    rho_r = R.measure_sfdensity(lxx_r)
    gpu = lib.DQMC(api_params(p), phi)
    try:
        gpu.init()
        for (lxx, lyy, rho), tol in ((gpu.measure_zfccc(), TOL), (gpu.measure_zfccc(g, gt0_r, g0t_r), 1e-12)):
            assert relerr(lxx, lxx_r) < tol and relerr(lyy, lyy_r) < tol
            assert abs(rho - rho_r) < tol * max(1.0, float(np.max(np.abs(lxx_r))))
    finally:
        gpu.close()


def _binned(x, nbins=4):
    """Mean and standard error of the mean from nbins equal bins."""
    b = np.asarray(x, dtype=float).reshape(nbins, -1).mean(axis=1)
    return float(b.mean()), float(b.std(ddof=1) / np.sqrt(nbins))


def test_observables_agree_within_binned_errors(lib):
    """Observable agreement: boson susceptibility chi_static
    (src/boson_measurements.jl:6-32) and the fermion kinetic energy from the
    measurement hook's true G, recorded at the measurement point (slice M,
    direction -1) after each of 24 up-down sweeps at L=4, M=40 from the same
    field and streams on the GPU and in the oracle.  The binned means agree
    within their binned errors; since the accept sequences are identical, the
    series themselves agree to round-off (1e-9 relative)."""
    p = P_L4
    phi = R.synthetic_field(p.N, p.slices, 91)
    n_ud, calls = 24, 2 * p.slices
    delta, u = R.synthetic_streams(p.N, n_ud * calls, p.box, 92)
    ref = R.DQMCRef(p, phi)
    ref.init()
    gpu = lib.DQMC(api_params(p, all_checks=False), phi)
    try:
        gpu.init()
        ek_g, ek_r, chi_g, chi_r = [], [], [], []
        for s in range(n_ud):
            sl = slice(s * calls, (s + 1) * calls)
            gpu.sweep(calls, delta[sl], u[sl])
            ref.sweep(calls, delta[sl], u[sl])
            ek_g.append(gpu.measure()["e_kin"])
            ek_r.append(ref.kinetic_energy(ref.measured_greens()))
            chi_g.append(R.measure_chi_static(gpu.get_field()))
            chi_r.append(R.measure_chi_static(ref.phi))
        for a, b in ((ek_g, ek_r), (chi_g, chi_r)):
            (ma, ea), (mb, eb) = _binned(a), _binned(b)
            assert abs(ma - mb) <= 2.0 * np.hypot(ea, eb) + 1e-12
            assert np.allclose(a, b, rtol=1e-9, atol=1e-12)
    finally:
        gpu.close()


# ---------------------------------------------------------------------------
# hybrid Monte Carlo move (leapfrog with the adjoint force, Metropolis on dH)
# ---------------------------------------------------------------------------
P_HMC = R.Params(L=4, slices=20, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5,
                 mu2=-0.5, box=0.2)


@pytest.mark.parametrize("u", [0.0, 1.0 - 1e-15])
def test_hmc_update_matches_oracle(lib, u):
    """One HMC move (3 leapfrog steps, eps = 0.01) from the same field and
    momenta: dH and the acceptance probability exp(-dH) agree with the
    oracle's restatement within 1e-9, the decision is the same, and the state
    after the move (field, G, action) is the oracle's (accepted trajectory or
    restored field)."""
    p = P_HMC
    # a field near equilibrium (|phi| <= 0.2): dH > 0 here, so u = 0 accepts
    # and u = 1 - 1e-15 rejects (restore path)
    phi = 0.2 * R.synthetic_field(p.N, p.slices, 95)
    pi = np.random.default_rng(96).standard_normal((3, p.N, p.slices))
    ref = R.DQMCRef(p, phi)
    acc_r, dh_r = R.hmc_update(ref, pi, 3, 0.01, u)
    assert dh_r > 0 and acc_r == (u == 0.0)
    gpu = lib.DQMC(api_params(p), phi)
    try:
        gpu.init()
        acc_g, dh_g = gpu.hmc_update(pi, 3, 0.01, u)
        assert abs(dh_g - dh_r) < 1e-9, (dh_g, dh_r)
        assert abs(np.exp(-dh_g) - np.exp(-dh_r)) < 1e-9
        assert acc_g == acc_r
        assert gpu.state == (p.slices, -1)
        assert np.allclose(gpu.get_field(), ref.phi, rtol=0, atol=1e-12)
        assert relerr(gpu.greens, ref.greens) < TOL
        assert abs(gpu.boson_action - R.boson_action(p, ref.phi)) < 1e-10 * abs(gpu.boson_action)
        # the chain continues from the state the move left
        delta, uu = R.synthetic_streams(p.N, 3, p.box, 97)
        ref.sweep(3, delta, uu)
        gpu.sweep(3, delta, uu)
        assert relerr(gpu.greens, ref.greens) < TOL
    finally:
        gpu.close()


def test_hmc_energy_error_scales_as_eps_squared(lib):
    """Leapfrog over a fixed trajectory length tau = 0.1: halving the step
    size divides |dH| by about 4 (second-order integrator)."""
    p = P_HMC
    phi = R.synthetic_field(p.N, p.slices, 98)
    pi = np.random.default_rng(99).standard_normal((3, p.N, p.slices))
    gpu = lib.DQMC(api_params(p), phi)
    try:
        dh = []
        for eps, steps in ((0.02, 5), (0.01, 10), (0.005, 20)):
            gpu.init(phi)
            _, d = gpu.hmc_update(pi, steps, eps, 1.0 - 1e-15)
            dh.append(abs(d))
        r1, r2 = dh[0] / dh[1], dh[1] / dh[2]
        assert 3.0 < r1 < 5.3 and 3.0 < r2 < 5.3, (dh, r1, r2)
    finally:
        gpu.close()


def test_rrule_log_weight(lib):
    """The reverse rule of phi -> log|det M| + S_b: value against the oracle's
    log_weight_parts, pullback against the oracle's dense gradient (scaled by
    the cotangent)."""
    p = P_HMC
    phi = R.synthetic_field(p.N, p.slices, 61)
    gpu = lib.DQMC(api_params(p), phi)
    try:
        y, pullback = gpu.rrule_log_weight(phi)
        ref = R.DQMCRef(p, phi)
        ldm, sb = R.log_weight_parts(ref)
        assert abs(y - (ldm + sb)) < 1e-10 * abs(ldm + sb)
        g = pullback(2.5)
        want = 2.5 * (R.force_logdetM(ref) + R.force_boson(p, phi))
        assert np.max(np.abs(g - want)) < 1e-10 * max(1.0, np.max(np.abs(want)))
    finally:
        gpu.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_round_loop_graph_matches_fixed_rounds(lib, prec):
    """Delayed rounds (k = 16, L = 8, one sweep of M = 40 calls): the captured
    sweep, whose WHILE node repeats [round, flush] only while sites remain,
    against the launch-by-launch path with the fixed bound of N/k + 1 rounds
    per slice.  Same accept mask, field and G bit for bit; the graph runs
    fewer rounds, and its launch counts follow the rounds that ran: per call
    one prepare plus a delayed kernel and a condition kernel per round (local
    kind), and the same flush launches per round as the fixed path."""
    p = R.Params(L=8, slices=40, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5,
                 mu2=-0.5, box=0.2)
    calls = p.slices
    phi = R.synthetic_field(p.N, p.slices, 4040)
    delta, u = R.synthetic_streams(p.N, calls, p.box, 4041)
    chains = []
    try:
        for timed in (True, False):
            mp = api_params(p)
            mp.precision, mp.delay = prec, 16
            c = lib.DQMC(mp, phi)
            chains.append(c)
            c.init()
            c.reset_timing(timed)        # timing on: launch by launch, fixed rounds; off: graph replay
            res = c.sweep(calls, delta, u, return_accepted=True)
            kinds = c.timing()["kinds"]
            c.reset_timing(False)
            c.res, c.kinds = res, kinds
        fixed, graph = chains
        assert np.array_equal(graph.res["accepted_mask"], fixed.res["accepted_mask"])
        assert np.array_equal(graph.get_field(), fixed.get_field())
        assert np.array_equal(graph.greens, fixed.greens)
        r_fixed = (p.N + 15) // 16 + 1
        loc_f, fl_f = fixed.kinds["local_updates"]["launches"], fixed.kinds["flush"]["launches"]
        loc_g, fl_g = graph.kinds["local_updates"]["launches"], graph.kinds["flush"]["launches"]
        assert loc_f == calls * (1 + r_fixed)
        per_round = fl_f // (calls * r_fixed)
        assert per_round * calls * r_fixed == fl_f and per_round >= 1
        rounds = (loc_g - calls) // 2
        assert loc_g == calls + 2 * rounds
        assert fl_g == rounds * per_round
        assert calls <= rounds < calls * r_fixed
        print(f"{prec}: {rounds} rounds run against {calls * r_fixed} fixed")
    finally:
        for c in chains:
            c.close()
