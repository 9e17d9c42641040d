"""Parity at the headline lattice and in the configurations the benchmark runs.

* L=16, beta=20 (M=200, n=1024) in the plain FP64 form against the oracle,
  across one stabilisation: identical accept sequence and field, G within
  1e-10 relative (immediate rank-4 and delayed rank-16 updates).
* L=16, beta=20 mixed form (split-BF16 GEMMs, delayed k=16) against the plain
  FP64 form over 10 sweeps (10 M update calls): identical accept sequences
  (any flip is reported with its margin |p_acc - u|) and max|G - G_FP64|
  <= 1e-8 after every sweep.
* The batched form as benchmarked (mixed, autotuned delay, L in {6,8,10,12},
  M=80, 8 chains in flight on capped cooperative grids): bit-identical to the
  same chains swept one by one with the same grids, and one chain against
  the oracle across a stabilisation.
* The adjoint force against central finite differences of the oracle's own
  log-weight (log|det M| and S_boson) at L=6, M=20.
"""
import dataclasses

import numpy as np
import pytest

from oracle import dqmc_ref as R

pytestmark = pytest.mark.gpu

TOL = 1e-10          # FP64 form against the oracle (relative to max |G|)
MIXED_TOL = 1e-8     # mixed form against the FP64 form


def relerr(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(1.0, float(np.max(np.abs(b)))))


def api_params(p: R.Params, **kw):
    from dqmc_gb300.api import ModelParams
    mp = ModelParams(L=p.L, slices=p.slices, safe_mult=p.safe_mult, delta_tau=p.delta_tau, lambda_=p.lambda_,
                     r=p.r, c=p.c, u=p.u, mu1=p.mu1, mu2=p.mu2, hoppings=tuple(p.hoppings), box=p.box)
    return dataclasses.replace(mp, **kw)


@pytest.fixture(scope="module")
def lib():
    from dqmc_gb300 import build
    build.build()
    from dqmc_gb300 import api
    return api


# L=16, beta=20: the headline lattice (lambda = r = c = u = 1, box 0.2)
P_L16 = R.Params(L=16, slices=200, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5,
                 mu2=-0.5, box=0.2)
L16_CALLS = 12       # from slice 200 down to 188: crosses the stabilisation at the 190/191 boundary


@pytest.fixture(scope="module")
def oracle_l16():
    p = P_L16
    phi = R.synthetic_field(p.N, p.slices, 1600)
    delta, u = R.synthetic_streams(p.N, L16_CALLS, p.box, 1601)
    ref = R.DQMCRef(p, phi)
    ref.init()
    rec = []
    ref.sweep(L16_CALLS, delta, u, record=rec)
    acc = np.array([r[2] for r in rec]).reshape(L16_CALLS, p.N)
    margin = np.abs(np.array([r[4] - r[5] for r in rec])).reshape(L16_CALLS, p.N)
    return dict(phi=phi, delta=delta, u=u, acc=acc, margin=margin, greens=ref.greens.copy(), field=ref.phi.copy(),
                state=(ref.current_slice, ref.direction), action=ref.boson_action_value)


@pytest.mark.parametrize("delay", [1, 16])
def test_l16_fp64_matches_oracle_across_stabilisation(lib, oracle_l16, delay):
    o = oracle_l16
    p = P_L16
    gpu = lib.DQMC(api_params(p, delay=delay), o["phi"])
    try:
        gpu.init()
        res = gpu.sweep(L16_CALLS, o["delta"], o["u"], return_accepted=True)
        mask = res["accepted_mask"]
        if not np.array_equal(mask, o["acc"]):
            c, s = np.argwhere(mask != o["acc"])[0]
            pytest.fail(f"first flip at call {c}, site {s}: margin |p_acc - u| = {o['margin'][c, s]:.3e}")
        assert np.array_equal(gpu.get_field(), o["field"])
        assert gpu.state == o["state"]
        assert relerr(gpu.greens, o["greens"]) < TOL
        assert res["max_instability"] < 1e-7
        assert abs(gpu.boson_action - o["action"]) < 1e-10 * abs(o["action"])
        assert 0.3 < o["acc"].mean() < 0.9
    finally:
        gpu.close()


def test_l16_mixed_ten_sweeps_match_fp64(lib):
    """Mixed form (k=16, as benchmarked) against the FP64 form (immediate
    rank-4, as benchmarked) over 10 sweeps of M update calls."""
    p = P_L16
    sweeps, M, N = 10, p.slices, p.N
    phi = R.synthetic_field(N, M, 1610)
    delta, u = R.synthetic_streams(N, sweeps * M, p.box, 1611)
    fp = lib.DQMC(api_params(p, delay=1), phi)
    mx = lib.DQMC(api_params(p, precision="mixed", delay=16), phi)
    try:
        fp.init()
        mx.init()
        errs = []
        for s in range(sweeps):
            acc_f = np.zeros((M, N), dtype=bool)
            pacc_f = np.zeros((M, N))
            for c in range(M):
                k = s * M + c
                _, acc_f[c], _, pacc_f[c] = fp.update(delta[k], u[k], return_details=True)
            res = mx.sweep(M, delta[s * M:(s + 1) * M], u[s * M:(s + 1) * M], return_accepted=True)
            acc_m = res["accepted_mask"]
            if not np.array_equal(acc_m, acc_f):
                c, i = np.argwhere(acc_m != acc_f)[0]
                margin = abs(pacc_f[c, i] - u[s * M + c, i])
                pytest.fail(f"sweep {s}: first flip at call {c}, site {i}, margin |p_acc - u| = {margin:.3e}")
            assert fp.state == mx.state
            err = relerr(mx.greens, fp.greens)
            errs.append(err)
            assert err <= MIXED_TOL, (s, err)
        assert np.array_equal(mx.get_field(), fp.get_field())
        print(f"max|G_mixed - G_FP64| per sweep: {['%.1e' % e for e in errs]}")
    finally:
        fp.close()
        mx.close()


def test_batched_benchmark_config(lib):
    """The batched configuration the benchmark runs: mixed form, delay picked
    by the autotuner, L in {6, 8, 10, 12}, M = 80, 8 chains in flight with
    capped cooperative grids, over one full sweep of M calls.  Every chain is
    bit-identical to the same chain swept alone on the same grid shapes,
    after the first 12 calls and after the sweep; after 12 calls the L=12
    chain matches the oracle (FP64) across a stabilisation within the
    mixed-form tolerance, with an identical field (hence accept sequence)."""
    torch = pytest.importorskip("torch")
    sizes = [12, 10, 8, 6, 12, 10, 8, 6]
    M, calls, inflight = 80, 12, 8
    plist, fields, streams = [], [], []
    for k, L in enumerate(sizes):
        p = R.Params(L=L, slices=M, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5,
                     mu2=-0.5, box=0.2)
        plist.append(p)
        fields.append(R.synthetic_field(p.N, M, 700 + k))
        streams.append(R.synthetic_streams(p.N, M, p.box, 800 + k))
    mps = [api_params(p, precision="mixed", inflight=inflight) for p in plist]
    batch = lib.Batch(mps, fields, autotune=True)
    singles = []
    try:
        assert all(batch.params[i].delay in (8, 16, 32) for i in range(len(sizes)))
        batch.init()
        dev_d, dev_u = [], []
        for (delta, u) in streams:
            dev_d.append(torch.from_numpy(np.ascontiguousarray(np.transpose(delta, (0, 2, 1)))).cuda())
            dev_u.append(torch.from_numpy(np.ascontiguousarray(u)).cuda())
        torch.cuda.synchronize()
        stats = batch.sweep_device(calls, [t.data_ptr() for t in dev_d], [t.data_ptr() for t in dev_u])
        for k, p in enumerate(plist):
            single = lib.DQMC(batch.params[k], fields[k])
            singles.append(single)
            single.init()
            res = single.sweep(calls, streams[k][0][:calls], streams[k][1][:calls])
            assert stats[k]["accepted"] == res["accepted"], k
            assert np.array_equal(batch.chains[k].greens, single.greens), k
            assert np.array_equal(batch.chains[k].get_field(), single.get_field()), k
        ref = R.DQMCRef(plist[0], fields[0])
        ref.init()
        ref.sweep(calls, streams[0][0][:calls], streams[0][1][:calls])
        assert np.array_equal(batch.chains[0].get_field(), ref.phi)
        assert relerr(batch.chains[0].greens, ref.greens) < MIXED_TOL
        # the rest of the sweep (M - 12 more calls, through the stabilisations
        # and the turn at slice 1): still bit-identical to the chains alone
        rest = M - calls
        stats = batch.sweep_device(rest, [t.data_ptr() + calls * t.shape[1] * t.shape[2] * 8 for t in dev_d],
                                   [t.data_ptr() + calls * t.shape[1] * 8 for t in dev_u])
        for k, single in enumerate(singles):
            res = single.sweep(rest, streams[k][0][calls:], streams[k][1][calls:])
            assert stats[k]["accepted"] == res["accepted"], k
            assert np.array_equal(batch.chains[k].greens, singles[k].greens), k
            assert np.array_equal(batch.chains[k].get_field(), singles[k].get_field()), k
    finally:
        for single in singles:
            single.close()
        batch.close()


def test_force_finite_differences_of_oracle_log_weight(lib):
    """d log|det M|/d phi and d S_boson/d phi of the adjoint kernel against
    central differences (h = 1e-5) of the oracle's log-weight parts
    (log_weight_parts: log|det M| = -log|det G| from scratch, and S_boson)
    on 100 random entries, 1e-6 relative."""
    p = R.Params(L=6, slices=20, delta_tau=0.1, safe_mult=10, lambda_=1.0, r=1.0, c=1.0, u=1.0, mu1=-0.5,
                 mu2=-0.5, box=0.2)
    phi = R.synthetic_field(p.N, p.slices, 66)
    gpu = lib.DQMC(api_params(p), phi)
    try:
        gpu.init()
        gl, gb = gpu.force()
    finally:
        gpu.close()
    rng = np.random.default_rng(67)
    h = 1e-5
    ref = R.DQMCRef(p, phi)
    worst = 0.0
    for _ in range(100):
        a, i, l = rng.integers(3), rng.integers(p.N), rng.integers(p.slices)
        parts = []
        for sgn in (1, -1):
            ref.phi = phi.copy()
            ref.phi[a, i, l] += sgn * h
            parts.append(R.log_weight_parts(ref))
        fd_ld = (parts[0][0] - parts[1][0]) / (2 * h)
        fd_sb = (parts[0][1] - parts[1][1]) / (2 * h)
        e_ld = abs(gl[a, i, l] - fd_ld) / max(1.0, abs(fd_ld))
        e_sb = abs(gb[a, i, l] - fd_sb) / max(1.0, abs(fd_sb))
        worst = max(worst, e_ld, e_sb)
        assert e_ld <= 1e-6, (a, i, l, gl[a, i, l], fd_ld)
        assert e_sb <= 1e-6, (a, i, l, gb[a, i, l], fd_sb)
    print(f"worst relative difference to the oracle's finite differences: {worst:.2e}")
