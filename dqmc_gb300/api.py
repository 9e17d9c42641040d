"""Python host binding of the C ABI (include/dqmc_gpu.h) through ctypes.

`DQMC` mirrors the reference's hot-path API on `AbstractDQMC`
(src/QMC.jl, src/dqmc_framework.jl, src/stack.jl, src/local_updates.jl):
`init`, `propagate`, `wrap_greens`, `calculate_greens`, `calc_greens`,
`local_updates`, `update`, `multiply_B_left` & co., `calc_boson_action`.
Every call goes to the CUDA library; there is no CPU fallback: if the
library is missing or no GPU is visible the constructor raises.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdqmc_gpu.so")

DQMC_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "non-finite value", -4: "singular M",
          -5: "device wait timed out", -6: "invalid state", -7: "size exceeds the static scratch (n > 1024)"}

B_LEFT, B_RIGHT, B_INV_LEFT, B_INV_RIGHT, B_DAG_LEFT = 0, 1, 2, 3, 4


class DQMCError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class CParams(ctypes.Structure):
    _fields_ = [("L", ctypes.c_int32), ("slices", ctypes.c_int32), ("safe_mult", ctypes.c_int32),
                ("opdim", ctypes.c_int32), ("delta_tau", ctypes.c_double), ("lambda_", ctypes.c_double),
                ("r", ctypes.c_double), ("c", ctypes.c_double), ("u", ctypes.c_double),
                ("mu1", ctypes.c_double), ("mu2", ctypes.c_double), ("hoppings", ctypes.c_double * 4),
                ("all_checks", ctypes.c_int32), ("precision", ctypes.c_int32), ("device", ctypes.c_int32),
                ("ozaki_bits", ctypes.c_int32), ("delay", ctypes.c_int32), ("greens_method", ctypes.c_int32),
                ("inflight", ctypes.c_int32), ("reserved", ctypes.c_int32 * 1)]


class CStats(ctypes.Structure):
    _fields_ = [("proposals", ctypes.c_int64), ("accepted", ctypes.c_int64), ("acc_rate", ctypes.c_double),
                ("max_instability", ctypes.c_double), ("device_ms", ctypes.c_double)]


KERNEL_KINDS = ["slice_cols", "slice_rows", "local_updates", "zgemm", "qrp", "apply_q", "trsm", "misc",
                "ozaki_gemm", "flush", "lu"]
NK = len(KERNEL_KINDS)


class CTiming(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double * NK), ("launches", ctypes.c_int64 * NK), ("flops", ctypes.c_double * NK),
                ("bytes", ctypes.c_double * NK), ("kernel_launches", ctypes.c_int64)]


# every symbol the header declares, with its argument types
_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.c_int32
SIGNATURES = {
    "dqmc_version": ([], ctypes.c_char_p),
    "dqmc_create": ([ctypes.POINTER(CParams), ctypes.POINTER(_P)], ctypes.c_int),
    "dqmc_destroy": ([_P], ctypes.c_int),
    "dqmc_last_error": ([_P], ctypes.c_char_p),
    "dqmc_set_field": ([_P, _D], ctypes.c_int),
    "dqmc_get_field": ([_P, _D], ctypes.c_int),
    "dqmc_init": ([_P], ctypes.c_int),
    "dqmc_propagate": ([_P], ctypes.c_int),
    "dqmc_get_state": ([_P, ctypes.POINTER(_I32), ctypes.POINTER(_I32)], ctypes.c_int),
    "dqmc_local_updates": ([_P, _D, _D, ctypes.c_void_p, _D, _D, _D], ctypes.c_int),
    "dqmc_update": ([_P, _D, _D, ctypes.c_void_p, _D, _D, _D], ctypes.c_int),
    "dqmc_sweep": ([_P, _I32, _D, _D, ctypes.c_void_p, ctypes.POINTER(CStats)], ctypes.c_int),
    "dqmc_sweep_device": ([_P, _I32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.POINTER(CStats)], ctypes.c_int),
    "dqmc_get_greens": ([_P, _D, ctypes.POINTER(_I32), ctypes.POINTER(_I32)], ctypes.c_int),
    "dqmc_set_greens": ([_P, _D], ctypes.c_int),
    "dqmc_calc_greens": ([_P, _I32, _D, _D], ctypes.c_int),
    "dqmc_wrap_greens": ([_P, _D, _I32, _I32], ctypes.c_int),
    "dqmc_calculate_greens_udt": ([_P, _D, _D, _D, _D, _D, _D, _D, _D], ctypes.c_int),
    "dqmc_decompose_udt": ([_P, _D, _D, _D, _D], ctypes.c_int),
    "dqmc_logdet": ([_P, _D], ctypes.c_int),
    "dqmc_multiply_B": ([_P, _I32, _I32, _D], ctypes.c_int),
    "dqmc_boson_action": ([_P, _D], ctypes.c_int),
    "dqmc_calc_boson_action": ([_P, _D], ctypes.c_int),
    "dqmc_measure": ([_P, _D, _D, _D], ctypes.c_int),
    "dqmc_measure_equal_time": ([_P, _D, _D, _D, _D, _D, ctypes.c_int32], ctypes.c_int),
    "dqmc_measure_zfpc": ([_P, _D, _D, _D, ctypes.c_int32], ctypes.c_int),
    "dqmc_measure_zfcdc": ([_P, _D, _D, _D, _D, _D, ctypes.c_int32], ctypes.c_int),
    "dqmc_measure_zfccc": ([_P, _D, _D, _D, _D, _D, _D, ctypes.c_int32], ctypes.c_int),
    "dqmc_get_timing": ([_P, ctypes.POINTER(CTiming)], ctypes.c_int),
    "dqmc_reset_timing": ([_P, _I32], ctypes.c_int),
    "dqmc_peak_fp64": ([_I32, _D], ctypes.c_int),
    "dqmc_gemm_check": ([_P, _I32, _D, _D, _D], ctypes.c_int),
    "dqmc_force": ([_P, _D, _D], ctypes.c_int),
    "dqmc_measure_tdgfs": ([_P, _D, _D, _I32], ctypes.c_int),
    "dqmc_global_update": ([_P, _D, ctypes.c_double, ctypes.POINTER(_I32), _D], ctypes.c_int),
    "dqmc_hmc_update": ([_P, _D, _I32, ctypes.c_double, ctypes.c_double, ctypes.POINTER(_I32), _D], ctypes.c_int),
    "dqmc_batch_create": ([ctypes.POINTER(CParams), _I32, ctypes.POINTER(_P)], ctypes.c_int),
    "dqmc_batch_destroy": ([_P], ctypes.c_int),
    "dqmc_batch_handle": ([_P, _I32, ctypes.POINTER(_P)], ctypes.c_int),
    "dqmc_batch_sweep": ([_P, _I32, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                          ctypes.POINTER(CStats)], ctypes.c_int),
    "dqmc_local_updates_noalloc": ([ctypes.POINTER(CParams), ctypes.c_void_p, ctypes.c_void_p, _I32,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p], ctypes.c_int),
}

_lib = None


def load_library(path: str = LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m dqmc_gb300.build` "
                          "(or __graft_entry__.build())")
    lib = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


@dataclasses.dataclass
class ModelParams:
    """Subset of the reference's `Params` (src/parameters.jl:4-80)."""
    L: int = 4
    slices: int = 40
    safe_mult: int = 10
    delta_tau: float = 0.1
    lambda_: float = 1.0
    r: float = 1.0
    c: float = 1.0
    u: float = 1.0
    mu1: float = -0.5
    mu2: float = -0.5
    hoppings: tuple = (1.0, 0.5, -0.5, -1.0)
    box: float = 0.2
    all_checks: bool = True
    device: int = -1
    precision: str = "fp64"        # "fp64" or "mixed"
    ozaki_bits: int = 0            # mantissa bits per GEMM operand in the mixed form (0 = default 40)
    delay: int = 0                 # delayed-update depth (0/1 = immediate rank-4)
    greens_method: str = "scales"  # calculate_greens: "scales" (D-scale separation + LU) or "two_qr" (reference)
    inflight: int = 0              # batches: chains swept at the same time (0 = min(count, 8))

    @property
    def N(self):
        return self.L * self.L

    @property
    def n(self):
        return 4 * self.L * self.L

    def to_c(self) -> CParams:
        p = CParams()
        p.L, p.slices, p.safe_mult, p.opdim = self.L, self.slices, self.safe_mult, 3
        p.delta_tau, p.lambda_, p.r, p.c, p.u = self.delta_tau, self.lambda_, self.r, self.c, self.u
        p.mu1, p.mu2 = self.mu1, self.mu2
        for k in range(4):
            p.hoppings[k] = self.hoppings[k]
        p.all_checks = 1 if self.all_checks else 0
        p.precision = {"fp64": 0, "mixed": 1}[self.precision]
        p.device = self.device
        p.ozaki_bits = self.ozaki_bits
        p.delay = self.delay
        if self.greens_method not in ("scales", "two_qr"):
            raise ValueError("greens_method must be 'scales' or 'two_qr'")
        p.greens_method = 0 if self.greens_method == "scales" else 1
        p.inflight = self.inflight
        return p


def _dptr(a):
    return a.ctypes.data_as(_D)


def _cplx_in(a, n):
    a = np.asarray(a, dtype=np.complex128)
    assert a.shape == (n, n)
    return np.asfortranarray(a)


def peak_fp64_tflops(device=0):
    """Measured FP64 FMA throughput of `device` in TFLOP/s."""
    lib = load_library()
    out = ctypes.c_double()
    rc = lib.dqmc_peak_fp64(int(device), ctypes.byref(out))
    if rc != DQMC_OK:
        raise DQMCError(rc, "dqmc_peak_fp64 failed")
    return out.value


class DQMC:
    """One Markov chain on the GPU.  Method names follow the reference."""

    def __init__(self, params: ModelParams, phi=None):
        self.lib = load_library()
        self.p = params
        self.N, self.n, self.M = params.N, params.n, params.slices
        h = ctypes.c_void_p()
        rc = self.lib.dqmc_create(ctypes.byref(params.to_c()), ctypes.byref(h))
        if rc != DQMC_OK:
            raise DQMCError(rc, "dqmc_create failed (unsupported parameters or no usable GPU)")
        self.h = h
        if phi is not None:
            self.set_field(phi)

    def close(self):
        if getattr(self, "h", None) and getattr(self, "_owned", True):
            self.lib.dqmc_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != DQMC_OK:
            raise DQMCError(rc, self.lib.dqmc_last_error(self.h).decode())

    # ---- field / state --------------------------------------------------
    def set_field(self, phi):
        phi = np.asfortranarray(np.asarray(phi, dtype=np.float64))
        assert phi.shape == (3, self.N, self.M)
        self._check(self.lib.dqmc_set_field(self.h, _dptr(phi)))

    def get_field(self):
        out = np.zeros((3, self.N, self.M), order="F")
        self._check(self.lib.dqmc_get_field(self.h, _dptr(out)))
        return out

    def init(self, phi=None):
        """init!(mc, start_conf) (src/dqmc_framework.jl:156-177)."""
        if phi is not None:
            self.set_field(phi)
        self._check(self.lib.dqmc_init(self.h))

    def propagate(self):
        self._check(self.lib.dqmc_propagate(self.h))

    @property
    def state(self):
        s, d = _I32(), _I32()
        self._check(self.lib.dqmc_get_state(self.h, ctypes.byref(s), ctypes.byref(d)))
        return s.value, d.value

    @property
    def current_slice(self):
        return self.state[0]

    @property
    def direction(self):
        return self.state[1]

    # ---- Green's functions ------------------------------------------------
    @property
    def greens(self):
        out = np.zeros((self.n, self.n), dtype=np.complex128, order="F")
        self._check(self.lib.dqmc_get_greens(self.h, out.ctypes.data_as(_D), None, None))
        return out

    @greens.setter
    def greens(self, G):
        G = _cplx_in(G, self.n)
        self._check(self.lib.dqmc_set_greens(self.h, G.ctypes.data_as(_D)))

    def calc_greens_and_logdet(self, slice1):
        out = np.zeros((self.n, self.n), dtype=np.complex128, order="F")
        ld = ctypes.c_double()
        self._check(self.lib.dqmc_calc_greens(self.h, int(slice1), out.ctypes.data_as(_D), ctypes.byref(ld)))
        return out, ld.value

    def calc_greens(self, slice1):
        return self.calc_greens_and_logdet(slice1)[0]

    def wrap_greens(self, G, slice1, direction):
        out = np.array(_cplx_in(G, self.n), order="F", copy=True)
        self._check(self.lib.dqmc_wrap_greens(self.h, out.ctypes.data_as(_D), int(slice1), int(direction)))
        return out

    def calculate_greens_udt(self, Ul, Dl, Tl, Ur, Dr, Tr):
        n = self.n
        args = [_cplx_in(x, n) for x in (Ul, Tl, Ur, Tr)]
        Dl = np.ascontiguousarray(Dl, dtype=np.float64)
        Dr = np.ascontiguousarray(Dr, dtype=np.float64)
        G = np.zeros((n, n), dtype=np.complex128, order="F")
        ld = ctypes.c_double()
        self._check(self.lib.dqmc_calculate_greens_udt(
            self.h, args[0].ctypes.data_as(_D), _dptr(Dl), args[1].ctypes.data_as(_D),
            args[2].ctypes.data_as(_D), _dptr(Dr), args[3].ctypes.data_as(_D), G.ctypes.data_as(_D),
            ctypes.byref(ld)))
        return G, ld.value

    def decompose_udt(self, A):
        n = self.n
        A = _cplx_in(A, n)
        U = np.zeros((n, n), dtype=np.complex128, order="F")
        T = np.zeros((n, n), dtype=np.complex128, order="F")
        D = np.zeros(n)
        self._check(self.lib.dqmc_decompose_udt(self.h, A.ctypes.data_as(_D), U.ctypes.data_as(_D), _dptr(D),
                                                T.ctypes.data_as(_D)))
        return U, D, T

    @property
    def log_det(self):
        ld = ctypes.c_double()
        self._check(self.lib.dqmc_logdet(self.h, ctypes.byref(ld)))
        return ld.value

    # ---- slice matrices ---------------------------------------------------
    def _mulB(self, which, slice1, A):
        out = np.array(_cplx_in(A, self.n), order="F", copy=True)
        self._check(self.lib.dqmc_multiply_B(self.h, which, int(slice1), out.ctypes.data_as(_D)))
        return out

    def multiply_B_left(self, slice1, A):
        return self._mulB(B_LEFT, slice1, A)

    def multiply_B_right(self, slice1, A):
        return self._mulB(B_RIGHT, slice1, A)

    def multiply_B_inv_left(self, slice1, A):
        return self._mulB(B_INV_LEFT, slice1, A)

    def multiply_B_inv_right(self, slice1, A):
        return self._mulB(B_INV_RIGHT, slice1, A)

    def multiply_daggered_B_left(self, slice1, A):
        return self._mulB(B_DAG_LEFT, slice1, A)

    def slice_matrix(self, slice1, power=1.0):
        eye = np.eye(self.n, dtype=np.complex128)
        return self.multiply_B_left(slice1, eye) if power > 0 else self.multiply_B_inv_left(slice1, eye)

    # ---- updates ----------------------------------------------------------
    def local_updates(self, delta, unif, return_details=False):
        """local_updates (src/local_updates.jl:1-38) with fixed-slot streams
        delta (3, N) and unif (N,); returns the acceptance rate."""
        delta = np.asfortranarray(np.asarray(delta, dtype=np.float64).reshape(3, self.N))
        unif = np.ascontiguousarray(unif, dtype=np.float64).reshape(self.N)
        acc = np.zeros(self.N, dtype=np.uint8)
        det = np.zeros(self.N, dtype=np.complex128)
        pacc = np.zeros(self.N)
        rate = ctypes.c_double()
        self._check(self.lib.dqmc_local_updates(self.h, _dptr(delta), _dptr(unif), acc.ctypes.data_as(ctypes.c_void_p),
                                                det.ctypes.data_as(_D), _dptr(pacc), ctypes.byref(rate)))
        if return_details:
            return rate.value, acc.astype(bool), det, pacc
        return rate.value

    def update(self, delta, unif, return_details=False):
        """update (src/dqmc_framework.jl:500-517), global updates off."""
        self.propagate()
        return self.local_updates(delta, unif, return_details)

    def sweep(self, n_calls, delta_stream, unif_stream, return_accepted=False):
        delta_stream = np.ascontiguousarray(np.asarray(delta_stream, dtype=np.float64).reshape(n_calls, 3, self.N))
        # per call the (3, N) block is column-major: component fastest
        d = np.ascontiguousarray(np.transpose(delta_stream, (0, 2, 1)))
        u = np.ascontiguousarray(unif_stream, dtype=np.float64).reshape(n_calls, self.N)
        acc = np.zeros((n_calls, self.N), dtype=np.uint8) if return_accepted else None
        st = CStats()
        self._check(self.lib.dqmc_sweep(self.h, int(n_calls), _dptr(d), _dptr(u),
                                        acc.ctypes.data_as(ctypes.c_void_p) if acc is not None else None,
                                        ctypes.byref(st)))
        res = dict(proposals=st.proposals, accepted=st.accepted, acc_rate=st.acc_rate,
                   max_instability=st.max_instability, device_ms=st.device_ms)
        if return_accepted:
            res["accepted_mask"] = acc.astype(bool)
        return res

    # ---- action / measurements --------------------------------------------
    @property
    def boson_action(self):
        s = ctypes.c_double()
        self._check(self.lib.dqmc_boson_action(self.h, ctypes.byref(s)))
        return s.value

    def calc_boson_action(self):
        s = ctypes.c_double()
        self._check(self.lib.dqmc_calc_boson_action(self.h, ctypes.byref(s)))
        return s.value

    def measure(self):
        G = np.zeros((self.n, self.n), dtype=np.complex128, order="F")
        occ, ek = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.dqmc_measure(self.h, G.ctypes.data_as(_D), ctypes.byref(occ), ctypes.byref(ek)))
        return dict(greens=G, occupation=occ.value, e_kin=ek.value)

    def measure_equal_time(self, greens=None):
        """measure_etpc! and measure_etcdc! (src/fermion_measurements.jl:388-424,
        592-630) of the true G `greens` (n x n), or of the measurement hook's G
        when None.  Returns (etpc_plus, etpc_minus, etcdc_plus, etcdc_minus),
        each L x L indexed [y, x] by the displacement."""
        L = self.p.L
        g = None
        if greens is not None:
            g = np.asfortranarray(np.asarray(greens, dtype=np.complex128).reshape(self.n, self.n))
        pp = np.zeros((L, L), order="F")
        pm = np.zeros((L, L), order="F")
        cp = np.zeros((L, L), dtype=np.complex128, order="F")
        cm = np.zeros((L, L), dtype=np.complex128, order="F")
        self._check(self.lib.dqmc_measure_equal_time(self.h, g.ctypes.data_as(_D) if g is not None else None,
                                                     pp.ctypes.data_as(_D), pm.ctypes.data_as(_D),
                                                     cp.ctypes.data_as(_D), cm.ctypes.data_as(_D), 0))
        return pp, pm, cp, cm

    def measure_zfpc(self, gt0=None):
        """measure_zfpc! (src/fermion_measurements.jl:500-541) over G(tau, 0)
        given as an (M, n, n) array (as measure_tdgfs returns), or computed on
        the device when None.  Returns (zfpc_plus, zfpc_minus), L x L [y, x]."""
        L = self.p.L
        g = None
        if gt0 is not None:
            # (M, n, n) row-major per block -> column-major n x n blocks
            g = np.ascontiguousarray(np.asarray(gt0, dtype=np.complex128).transpose(0, 2, 1))
        pp = np.zeros((L, L), order="F")
        pm = np.zeros((L, L), order="F")
        self._check(self.lib.dqmc_measure_zfpc(self.h, g.ctypes.data_as(_D) if g is not None else None,
                                               pp.ctypes.data_as(_D), pm.ctypes.data_as(_D), 0))
        return pp, pm

    def measure_zfcdc(self, greens=None, gt0=None, g0t=None):
        """measure_zfcdc! (src/fermion_measurements.jl:688-743) from the true
        equal-time G (None: the hook's G) and the (M, n, n) arrays that
        measure_tdgfs returns (None: computed on the device).  Returns
        (zfcdc_plus, zfcdc_minus), L x L complex [y, x]."""
        L = self.p.L
        if (gt0 is None) != (g0t is None):
            raise ValueError("pass both gt0 and g0t or neither")

        def blocks(a):
            return np.ascontiguousarray(np.asarray(a, dtype=np.complex128).transpose(0, 2, 1))
        g = None if greens is None else np.asfortranarray(np.asarray(greens, dtype=np.complex128))
        a = None if gt0 is None else blocks(gt0)
        b = None if g0t is None else blocks(g0t)
        cp = np.zeros((L, L), dtype=np.complex128, order="F")
        cm = np.zeros((L, L), dtype=np.complex128, order="F")
        ptr = lambda x: x.ctypes.data_as(_D) if x is not None else None
        self._check(self.lib.dqmc_measure_zfcdc(self.h, ptr(g), ptr(a), ptr(b), ptr(cp), ptr(cm), 0))
        return cp, cm

    def measure_zfccc(self, greens=None, gt0=None, g0t=None):
        """measure_zfccc! (src/fermion_measurements.jl:814-888) and
        measure_sfdensity (:911-920), inputs as measure_zfcdc.  Returns
        (zfccc_xx, zfccc_yy, sfdensity), the arrays L x L complex [y, x]."""
        L = self.p.L
        if (gt0 is None) != (g0t is None):
            raise ValueError("pass both gt0 and g0t or neither")

        def blocks(a):
            return np.ascontiguousarray(np.asarray(a, dtype=np.complex128).transpose(0, 2, 1))
        g = None if greens is None else np.asfortranarray(np.asarray(greens, dtype=np.complex128))
        a = None if gt0 is None else blocks(gt0)
        b = None if g0t is None else blocks(g0t)
        lxx = np.zeros((L, L), dtype=np.complex128, order="F")
        lyy = np.zeros((L, L), dtype=np.complex128, order="F")
        rho = ctypes.c_double()
        ptr = lambda x: x.ctypes.data_as(_D) if x is not None else None
        self._check(self.lib.dqmc_measure_zfccc(self.h, ptr(g), ptr(a), ptr(b), ptr(lxx), ptr(lyy),
                                                ctypes.byref(rho), 0))
        return lxx, lyy, rho.value

    def global_update(self, shift, u):
        """global_update (src/global_updates.jl:18-58) with a fixed-slot shift
        (3,) and uniform u; returns (accepted, p_acc)."""
        sh = np.ascontiguousarray(shift, dtype=np.float64).reshape(3)
        acc, pa = _I32(), ctypes.c_double()
        self._check(self.lib.dqmc_global_update(self.h, _dptr(sh), float(u), ctypes.byref(acc), ctypes.byref(pa)))
        return bool(acc.value), pa.value

    def hmc_update(self, momenta, n_steps, eps, u):
        """Hybrid Monte Carlo move on S_b - log|det M| with fixed-slot momenta
        (3, N, M), n_steps leapfrog steps of size eps and Metropolis uniform u;
        returns (accepted, dH).  Needs the state (M, -1) and keeps it."""
        pi = np.asfortranarray(np.asarray(momenta, dtype=np.float64).reshape(3, self.N, self.M))
        acc, dh = _I32(), ctypes.c_double()
        self._check(self.lib.dqmc_hmc_update(self.h, _dptr(pi), int(n_steps), float(eps), float(u),
                                             ctypes.byref(acc), ctypes.byref(dh)))
        return bool(acc.value), dh.value

    def force(self):
        """(d log|det M|/d phi, d S_boson/d phi), each (3, N, M); needs the
        state (slice M, direction -1) and returns to it."""
        gl = np.zeros((3, self.N, self.M), order="F")
        gb = np.zeros((3, self.N, self.M), order="F")
        self._check(self.lib.dqmc_force(self.h, _dptr(gl), _dptr(gb)))
        return gl, gb

    def log_weight(self):
        """log|det M| + S_b of the current field (state (M, -1)), with
        log|det M| = -log|det G| of the fresh G at slice M."""
        return -self.log_det + self.boson_action

    def rrule_log_weight(self, phi):
        """Reverse rule of phi -> log|det M(phi)| + S_b(phi), the counterpart
        of a ChainRulesCore rrule: sets the field and rebuilds the stack, and
        returns (y, pullback) with pullback(dy) = dy * (dlog|det M|/dphi +
        dS_b/dphi) from the adjoint force (dqmc_force).  The chain is left in
        the state (M, -1) of phi."""
        self.init(phi)
        y = self.log_weight()
        gl, gb = self.force()

        def pullback(dy):
            return float(dy) * (gl + gb)
        return y, pullback

    def langevin_step(self, eps, rng):
        """One Langevin move on the effective action S_b - log|det M|:
        phi <- phi - eps (dS_b - dlog|det M|) + sqrt(2 eps) eta, then the stack
        is rebuilt (dqmc_init)."""
        gl, gb = self.force()
        phi = self.get_field()
        phi = phi - eps * (gb - gl) + np.sqrt(2.0 * eps) * rng.standard_normal(phi.shape)
        self.init(phi)
        return phi

    def gemm_check(self, A, B, mode):
        """C = A B with the FP64 kernel (mode 0) or the split-BF16 GEMM (mode 1)."""
        n = self.n
        A, B = _cplx_in(A, n), _cplx_in(B, n)
        C = np.zeros((n, n), dtype=np.complex128, order="F")
        self._check(self.lib.dqmc_gemm_check(self.h, int(mode), A.ctypes.data_as(_D), B.ctypes.data_as(_D),
                                             C.ctypes.data_as(_D)))
        return C

    def measure_tdgfs(self):
        """measure_tdgfs! (src/fermion_measurements.jl:1343-1403): time-displaced
        Green's functions of the current field as two (M, n, n) arrays,
        Gt0[tau-1] = G(tau, 0) and G0t[tau-1] = -G(0, tau)."""
        M, n = self.M, self.n
        gt0 = np.empty((M, n, n), dtype=np.complex128)
        g0t = np.empty((M, n, n), dtype=np.complex128)
        self._check(self.lib.dqmc_measure_tdgfs(self.h, gt0.ctypes.data_as(_D), g0t.ctypes.data_as(_D), 0))
        # each slice's matrix is column-major
        return gt0.transpose(0, 2, 1), g0t.transpose(0, 2, 1)

    def timing(self):
        """Per kernel kind: device ms, launches, algorithmic flops and bytes."""
        t = CTiming()
        self._check(self.lib.dqmc_get_timing(self.h, ctypes.byref(t)))
        kinds = {k: dict(ms=t.ms[i], launches=t.launches[i], flops=t.flops[i], bytes=t.bytes[i])
                 for i, k in enumerate(KERNEL_KINDS)}
        return dict(kinds=kinds, kernel_launches=t.kernel_launches)

    def reset_timing(self, enable=True):
        self._check(self.lib.dqmc_reset_timing(self.h, 1 if enable else 0))


def tune_delay(params: ModelParams, candidates=(8, 16, 32), calls=None, seed=12345):
    """Delayed-update depth autotuner: times `calls` update() calls (default
    two stabilisation intervals) of one chain of `params` for every candidate
    k on a seeded synthetic field and proposal stream, after one untimed
    pass, and returns (fastest k, {k: seconds})."""
    rng = np.random.default_rng(seed)
    N, M = params.N, params.slices
    calls = calls or min(M, 2 * params.safe_mult)
    phi = rng.uniform(-1.0, 1.0, size=(3, N, M))
    delta = rng.uniform(-params.box, params.box, size=(calls, 3, N))
    unif = rng.uniform(size=(calls, N))
    times = {}
    for k in candidates:
        chain = DQMC(dataclasses.replace(params, delay=int(k)), phi)
        chain.init()
        chain.sweep(calls, delta, unif)
        t0 = time.perf_counter()
        chain.sweep(calls, delta, unif)
        times[int(k)] = time.perf_counter() - t0
        chain.close()
    best = min(times, key=times.get)
    return best, times


class Batch:
    """Independent chains sharing one GPU (dqmc_batch_*).  `chains[i]` is a
    DQMC view of chain i for the single-chain calls.  autotune=True picks the
    delayed-update depth per distinct (L, slices, precision) with tune_delay
    (the choices are kept in `tuned`)."""

    def __init__(self, params_list, fields=None, autotune=False, candidates=(8, 16, 32)):
        self.tuned = {}
        if autotune:
            tuned = []
            for p in params_list:
                key = (p.L, p.slices, p.precision)
                if key not in self.tuned:
                    self.tuned[key] = tune_delay(p, candidates)
                tuned.append(dataclasses.replace(p, delay=self.tuned[key][0]))
            params_list = tuned
        self.lib = load_library()
        arr = (CParams * len(params_list))(*[p.to_c() for p in params_list])
        b = ctypes.c_void_p()
        rc = self.lib.dqmc_batch_create(arr, len(params_list), ctypes.byref(b))
        if rc != DQMC_OK:
            raise DQMCError(rc, "dqmc_batch_create failed")
        self.b = b
        self.params = list(params_list)
        self.chains = []
        for i, p in enumerate(params_list):
            h = ctypes.c_void_p()
            self.lib.dqmc_batch_handle(self.b, i, ctypes.byref(h))
            c = DQMC.__new__(DQMC)
            c.lib, c.p, c.N, c.n, c.M, c.h = self.lib, p, p.N, p.n, p.slices, h
            c._owned = False
            self.chains.append(c)
        if fields is not None:
            for c, f in zip(self.chains, fields):
                c.set_field(f)

    def init(self):
        for c in self.chains:
            c.init()

    def sweep_device(self, n_calls, delta_ptrs, unif_ptrs):
        """n_calls update() calls on every chain; *_ptrs are device addresses
        (ints) of each chain's streams.  Returns a list of stats dicts."""
        C = len(self.chains)
        dp = (ctypes.c_void_p * C)(*delta_ptrs)
        up = (ctypes.c_void_p * C)(*unif_ptrs)
        st = (CStats * C)()
        rc = self.lib.dqmc_batch_sweep(self.b, int(n_calls), dp, up, st)
        if rc != DQMC_OK:
            raise DQMCError(rc, "dqmc_batch_sweep failed")
        return [dict(proposals=s.proposals, accepted=s.accepted, acc_rate=s.acc_rate,
                     max_instability=s.max_instability, device_ms=s.device_ms) for s in st]

    def close(self):
        if getattr(self, "b", None):
            self.lib.dqmc_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
