"""dqmc_local_updates_noalloc: the entry point for callers that cannot let the
library allocate GPU memory (their own allocator owns every device buffer, or
they run inside a fixed memory budget).  It must give the same result as the
handle-based dqmc_local_updates on the same state and streams, call after
call, while using only its static scratch array.

This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from oracle.dqmc_ref import synthetic_field, synthetic_streams

TOL = 1e-10   # same FP64 tolerance as the other parity tests


def _params(api, L=4, M=40):
    return api.ModelParams(L=L, slices=M, safe_mult=10, delta_tau=0.1, lambda_=1.0, r=1.0, c=1.0, u=1.0,
                           mu1=-0.5, mu2=-0.5, box=0.2)


def test_noalloc_rejects_sizes_beyond_static_scratch():
    from dqmc_gb300 import api, build
    build.build()
    lib = api.load_library()
    p = _params(api, L=18, M=10).to_c()          # n = 1296 > 1024
    dummy = ctypes.c_void_p(16)                    # never dereferenced: the size check comes first
    rc = lib.dqmc_local_updates_noalloc(ctypes.byref(p), dummy, dummy, 1, dummy, dummy, None, dummy, None)
    assert rc == -7


@pytest.mark.gpu
@pytest.mark.parametrize("L,M,steps", [(4, 40, 0), (4, 40, 3), (16, 20, 0), (16, 20, 5)])
def test_noalloc_matches_handle_path_two_calls(L, M, steps):
    """Two calls in a row at n = 64 and at the static limit n = 1024, at the
    slice after init (M) and at a slice `steps` propagations further down."""
    torch = pytest.importorskip("torch")
    from dqmc_gb300 import api, build
    build.build()
    lib = api.load_library()
    mp = _params(api, L, M)
    N, n = mp.N, mp.n
    chain = api.DQMC(mp, synthetic_field(N, M, 4242 + L))
    chain.init()
    for _ in range(steps):
        chain.propagate()
    slice1 = chain.current_slice
    assert slice1 == M - steps
    dev = torch.device("cuda:0")

    def to_dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    G_d = to_dev(np.asfortranarray(chain.greens).ravel(order="F").view(np.float64))
    phi_d = to_dev(chain.get_field().ravel(order="F"))
    act_d = torch.tensor([chain.boson_action], dtype=torch.float64, device=dev)
    acc_d = torch.zeros(N, dtype=torch.uint8, device=dev)
    cp = mp.to_c()
    delta, unif = synthetic_streams(N, 2, mp.box, 4343 + L)
    for call in range(2):
        # existing entry point (handle owns its memory)
        _, acc_ref, _, _ = chain.local_updates(delta[call], unif[call], return_details=True)
        # allocation-free entry point on caller-owned device buffers
        d_d = to_dev(np.asfortranarray(delta[call]).ravel(order="F"))
        u_d = to_dev(unif[call])
        torch.cuda.synchronize()
        rc = lib.dqmc_local_updates_noalloc(ctypes.byref(cp), ctypes.c_void_p(G_d.data_ptr()),
                                            ctypes.c_void_p(phi_d.data_ptr()), slice1,
                                            ctypes.c_void_p(d_d.data_ptr()), ctypes.c_void_p(u_d.data_ptr()),
                                            ctypes.c_void_p(acc_d.data_ptr()), ctypes.c_void_p(act_d.data_ptr()),
                                            None)
        assert rc == 0, f"call {call}: status {rc}"
        G_na = G_d.cpu().numpy().view(np.complex128).reshape((n, n), order="F")
        G_ref = chain.greens
        assert np.max(np.abs(G_na - G_ref)) < TOL * max(1.0, np.max(np.abs(G_ref))), f"call {call}"
        assert np.array_equal(acc_d.cpu().numpy().astype(bool), acc_ref), f"call {call}"
        assert acc_ref.any(), "no acceptance: the update path was not exercised"
        phi_na = phi_d.cpu().numpy().reshape((3, N, M), order="F")
        assert np.allclose(phi_na, chain.get_field(), rtol=0, atol=TOL), f"call {call}"
        assert abs(act_d.item() - chain.boson_action) < TOL * abs(chain.boson_action), f"call {call}"
    chain.close()


@pytest.mark.gpu
def test_noalloc_rejects_host_array():
    """A host (numpy) array where a device array is expected is an argument
    error, returned before anything is launched; the device arrays are left
    untouched."""
    torch = pytest.importorskip("torch")
    from dqmc_gb300 import api, build
    build.build()
    lib = api.load_library()
    mp = _params(api, 4, 10)
    N, n, M = mp.N, mp.n, mp.slices
    dev = torch.device("cuda:0")
    G_host = np.zeros(2 * n * n)
    phi_d = torch.zeros(3 * N * M, dtype=torch.float64, device=dev)
    d_d = torch.zeros(3 * N, dtype=torch.float64, device=dev)
    u_d = torch.full((N,), 0.5, dtype=torch.float64, device=dev)
    act_d = torch.zeros(1, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    cp = mp.to_c()
    rc = lib.dqmc_local_updates_noalloc(ctypes.byref(cp), ctypes.c_void_p(G_host.ctypes.data),
                                        ctypes.c_void_p(phi_d.data_ptr()), 1, ctypes.c_void_p(d_d.data_ptr()),
                                        ctypes.c_void_p(u_d.data_ptr()), None, ctypes.c_void_p(act_d.data_ptr()),
                                        None)
    assert rc == -1
    assert act_d.item() == 0.0
