"""CPU oracle for the O(3) spin-fermion DQMC sweep hot path (TEST INFRASTRUCTURE ONLY).

This module is a plain numpy/scipy FP64 restatement of the reference algorithm
(carstenbauer/dqmc, Julia).  It exists to check the CUDA library; it is never
part of the product path.  Only `tests/`, `__graft_entry__.smoke()` and the
`cpu_baseline` / `--impl reference` legs of `bench.py` may import it.

Parity status: pinned.  The restatement is checked against the reference's own
golden data (`test/data/O3.jld`, `test/data/linalg.jld`, decoded into
`tests/golden/*.npz` by `tests/golden/make_golden.py`) and against the literal
known answers written in the reference's test files (`test/tests_O3.jl`,
`test/tests_O3_measurements.jl`, `test/tests_linalg.jl`).

Reference files restated here (paths within carstenbauer/dqmc):
  * src/stack.jl:251-499 (stack, propagate, calculate_greens);
  * src/local_updates.jl:1-95, src/action.jl:1-100, src/interactions.jl:35-141;
  * src/slice_matrices.jl:25-226, src/hoppings.jl:16-95, src/hoppings_checkerboard.jl:4-136,
    src/lattice.jl:105-153;
  * src/linalg.jl:20-61, 195-339, 512-567 (UDT, multiply_safely, inverses of UDT sums);
  * src/fermion_measurements.jl:363-920 (equal-time and zero-frequency correlators),
    964-1142 (from-scratch G, effective -> true G), 1343-1523 (time-displaced G);
  * src/boson_measurements.jl:6-32, src/global_updates.jl:18-58,
    src/dqmc_framework.jl:152-177, 500-517.

Conventions (identical to the reference):
  * sites are 0-based here; site s = y + L*x  (reference: `sql = reshape(1:N, L, L)`,
    src/lattice.jl:109);
  * G is n x n complex128 with n = 4N, index = f*N + site, flavours (x, y, x, y)
    for the hopping bands (src/hoppings_checkerboard.jl:95-103);
  * the boson field phi has shape (3, N, M) (src/parameters.jl:19);
  * time slices are 1-based in the public methods, as in the reference.

The LAPACK routines used (`geqp3` via `scipy.linalg.qr(pivoting=True)`, `getrf`)
are the ones Julia's LinearAlgebra calls for `qr(A, Val(true))`, `\\`, `inv`
and `det`; results agree with the reference to round-off, not bit for bit.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sps


# ---------------------------------------------------------------------------
# parameters  (src/parameters.jl:4-80, subset used by the hot path)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Params:
    L: int = 4
    slices: int = 10
    delta_tau: float = 0.1
    safe_mult: int = 10
    lambda_: float = 1.0
    r: float = 1.0
    c: float = 1.0
    u: float = 1.0
    mu1: float = -0.5
    mu2: float = -0.5
    hoppings: tuple = (1.0, 0.5, -0.5, -1.0)   # "tx_x,ty_x,tx_y,ty_y"
    box: float = 0.2
    edrun: bool = False
    checkerboard: bool = True                   # CBAssaad (True) or CBFalse (False)

    @property
    def N(self):
        return self.L * self.L

    @property
    def flv(self):
        return 4

    @property
    def n(self):
        return 4 * self.N

    def t(self):
        """t[bond dir (0=hor,1=ver), band (0=x,1=y)], column-major reshape
        of the HOPPINGS string (src/lattice.jl:59)."""
        h = self.hoppings
        return np.array([[h[0], h[2]], [h[1], h[3]]], dtype=np.float64)


# ---------------------------------------------------------------------------
# lattice  (src/lattice.jl:105-153)
# ---------------------------------------------------------------------------
def neighbors_table(L):
    """(4, N) table of (up, right, down, left) neighbours, 0-based.
    Follows src/lattice.jl:109-118 (circshift of the column-major site grid)."""
    N = L * L
    nb = np.zeros((4, N), dtype=np.int64)
    for x in range(L):
        for y in range(L):
            s = y + L * x
            nb[0, s] = (y + 1) % L + L * x          # up
            nb[1, s] = y + L * ((x + 1) % L)        # right
            nb[2, s] = (y - 1) % L + L * x          # down
            nb[3, s] = y + L * ((x - 1) % L)        # left
    return nb


def time_neighbors_table(M):
    """(2, M) table, row 0 = later slice, row 1 = earlier slice, 0-based,
    periodic (src/lattice.jl:144-153)."""
    tn = np.zeros((2, M), dtype=np.int64)
    for s in range(M):
        tn[0, s] = 0 if s == M - 1 else s + 1
        tn[1, s] = M - 1 if s == 0 else s - 1
    return tn


def four_site_corners(L):
    """Bottom-left corners of the A and B plaquette groups, 0-based.
    src/hoppings_checkerboard.jl:4-18: A at odd (1-based) x,y, x outer loop;
    B = up(right(A))."""
    nb = neighbors_table(L)
    A = []
    for x in range(0, L, 2):
        for y in range(0, L, 2):
            A.append(y + L * x)
    A = np.array(A, dtype=np.int64)
    B = nb[0, nb[1, A]]
    return A, B


def plaquettes(L):
    """(group, corner) -> (i, j, m, n) site quadruples, i = corner, j = up(i),
    m = right(i), n = right(j) (src/hoppings_checkerboard.jl:37-40)."""
    nb = neighbors_table(L)
    A, B = four_site_corners(L)
    out = []
    for corners in (A, B):
        q = []
        for i in corners:
            j = nb[0, i]
            m = nb[1, i]
            n = nb[1, j]
            q.append((i, j, m, n))
        out.append(np.array(q, dtype=np.int64))
    return out


# ---------------------------------------------------------------------------
# hopping matrices  (src/hoppings.jl:16-95, src/hoppings_checkerboard.jl:20-136)
# ---------------------------------------------------------------------------
def hopping_matrices(p: Params):
    """Dense T (mu included) for both bands and exp(-+dtau/2 T), block-diagonal
    over flavours (x, y, x, y).  src/hoppings.jl:16-95."""
    L, N = p.L, p.N
    t = p.t()
    nb = neighbors_table(L)
    Tx = np.diag(np.full(N, -p.mu1))
    Ty = np.diag(np.full(N, -p.mu2))
    for src in range(N):
        for k in (1, 3):           # horizontal neighbours (right, left)
            trg = nb[k, src]
            Tx[trg, src] += -t[0, 0]
            Ty[trg, src] += -t[0, 1]
        for k in (0, 2):           # vertical neighbours (up, down)
            trg = nb[k, src]
            Tx[trg, src] += -t[1, 0]
            Ty[trg, src] += -t[1, 1]
    eTx_m = sla.expm(-0.5 * p.delta_tau * Tx)
    eTy_m = sla.expm(-0.5 * p.delta_tau * Ty)
    eTx_p = sla.expm(0.5 * p.delta_tau * Tx)
    eTy_p = sla.expm(0.5 * p.delta_tau * Ty)
    T = sla.block_diag(Tx, Ty, Tx, Ty)
    eT = sla.block_diag(eTx_m, eTy_m, eTx_m, eTy_m)
    eTinv = sla.block_diag(eTx_p, eTy_p, eTx_p, eTy_p)
    return T, eT, eTinv


def _four_site_exp(p: Params, quads, tflv, prefac, inverse):
    """Product over one plaquette group of the 4-site hopping exponentials
    for band `tflv` (src/hoppings_checkerboard.jl:20-63)."""
    N = p.N
    t = p.t()
    th, tv = t[0, tflv], t[1, tflv]
    fac = -prefac * p.delta_tau
    if inverse:
        fac = -fac
    ch, sh = math.cosh(fac * -th), math.sinh(fac * -th)
    cv, sv = math.cosh(fac * -tv), math.sinh(fac * -tv)
    Mx = sps.identity(N, dtype=np.float64, format="lil")
    for (i, j, m, n) in quads:
        P = sps.identity(N, dtype=np.float64, format="lil")
        for a in (i, j, m, n):
            P[a, a] = ch * cv
        for (a, b) in ((i, n), (j, m), (m, j), (n, i)):
            P[a, b] = sh * sv
        for (a, b) in ((i, j), (j, i), (m, n), (n, m)):
            P[a, b] = ch * sv
        for (a, b) in ((i, m), (j, n), (m, i), (n, j)):
            P[a, b] = sh * cv
        Mx = (Mx.tocsr() @ P.tocsr()).tolil()
    return Mx.tocsr()


def checkerboard_matrices(p: Params):
    """chkr_hop_half[g], chkr_hop[g] (+ inverses) for groups g = A (0), B (1),
    block-diagonal over (x, y, x, y), and the mu diagonals.
    src/hoppings_checkerboard.jl:65-136."""
    quads = plaquettes(p.L)
    out = {}
    for name, prefac in (("half", 0.5), ("full", 1.0)):
        for inv in (False, True):
            mats = []
            for g in range(2):
                ex = _four_site_exp(p, quads[g], 0, prefac, inv)
                ey = _four_site_exp(p, quads[g], 1, prefac, inv)
                mats.append(sps.block_diag((ex, ey, ex, ey), format="csr"))
            out[(name, inv)] = mats
    N = p.N
    muv = np.concatenate([np.full(N, p.mu1), np.full(N, p.mu2)] * 2)
    out["mu"] = np.exp(-p.delta_tau * -muv)
    out["mu_inv"] = np.exp(p.delta_tau * -muv)
    out["mu_half"] = np.exp(-0.5 * p.delta_tau * -muv)
    out["mu_half_inv"] = np.exp(0.5 * p.delta_tau * -muv)
    return out


# ---------------------------------------------------------------------------
# interactions  (src/interactions.jl:35-141)
# ---------------------------------------------------------------------------
def interaction_op(p: Params, op, power):
    """4x4 block exp(-power*dtau*V(op)) for one site (src/interactions.jl:102-141)."""
    nrm = math.sqrt(op[0] * op[0] + op[1] * op[1] + op[2] * op[2])
    sh = power * math.sinh(p.lambda_ * p.delta_tau * nrm) / nrm
    C = math.cosh(p.lambda_ * p.delta_tau * nrm)
    S = (1j * op[1] - op[0]) * sh
    R = (-op[2]) * sh
    e = np.zeros((4, 4), dtype=np.complex128)
    e[0, 0] = C; e[0, 1] = S; e[1, 0] = np.conj(S); e[1, 1] = C
    e[0, 3] = R; e[1, 2] = -R
    e[2, 1] = -R; e[2, 2] = C; e[2, 3] = np.conj(S)
    e[3, 0] = R; e[3, 2] = S; e[3, 3] = C
    return e


def interaction_matrix_exp(p: Params, phi_slice, power):
    """Sparse n x n exp(-power*dtau*V(slice)) built from per-site C, S, R
    (src/interactions.jl:35-88).  phi_slice has shape (3, N)."""
    N = p.N
    nrm = np.sqrt(np.sum(phi_slice * phi_slice, axis=0))
    sh = np.sinh(p.lambda_ * p.delta_tau * nrm) / nrm
    C = np.cosh(p.lambda_ * p.delta_tau * nrm).astype(np.complex128)
    S = (1j * phi_slice[1] - phi_slice[0]) * power * sh
    R = ((-phi_slice[2]) * power * sh).astype(np.complex128)
    rows, cols, vals = [], [], []

    def put(a, b, v):
        rows.append(np.arange(N) + a * N)
        cols.append(np.arange(N) + b * N)
        vals.append(v)

    put(0, 0, C); put(0, 1, S); put(1, 0, np.conj(S)); put(1, 1, C)
    put(0, 3, R); put(1, 2, -R); put(2, 1, -R); put(2, 2, C)
    put(2, 3, np.conj(S)); put(3, 0, R); put(3, 2, S); put(3, 3, C)
    return sps.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(4 * N, 4 * N))


# ---------------------------------------------------------------------------
# boson action  (src/action.jl:1-100)
# ---------------------------------------------------------------------------
def boson_action(p: Params, phi):
    """src/action.jl:1-52."""
    L, M = p.L, phi.shape[2]
    S = 0.0
    if not p.edrun:
        h = phi.reshape((3, L, L, M), order="F")
        t = h - np.roll(h, -1, axis=3)
        S += 0.5 / p.delta_tau * 1.0 / p.c ** 2 * np.sum(t * t)
        for ax in (1, 2):
            t = h - np.roll(h, -1, axis=ax)
            S += p.delta_tau * 0.5 * np.sum(t * t)
    sq = np.sum(phi * phi, axis=0)
    S += np.sum(p.delta_tau * p.r / 2.0 * sq)
    if not p.edrun:
        S += np.sum(p.delta_tau * p.u / 4.0 * sq * sq)
    return float(S)


def boson_action_diff(p: Params, phi, nb, tn, site, slice0, new_op):
    """Delta S_boson for changing phi[:, site, slice0] to new_op.
    src/action.jl:57-100 (slice0 is 0-based)."""
    old = phi[:, site, slice0]
    diff = new_op - old
    old_sq = float(old @ old)
    new_sq = float(new_op @ new_op)
    sq_diff = new_sq - old_sq
    pow4_diff = new_sq * new_sq - old_sq * old_sq
    op_earlier = phi[:, site, tn[1, slice0]]
    op_later = phi[:, site, tn[0, slice0]]
    op_time = op_later + op_earlier
    op_space = np.zeros(3)
    for k in range(4):
        op_space = op_space + phi[:, nb[k, site], slice0]
    dS = 0.0
    if not p.edrun:
        dS += 1.0 / (p.delta_tau * p.c ** 2) * (sq_diff - float(op_time @ diff))
        dS += 0.5 * p.delta_tau * (4 * sq_diff - 2.0 * float(op_space @ diff))
        dS += p.delta_tau * (0.5 * p.r * sq_diff + 0.25 * p.u * pow4_diff)
    else:
        dS += p.delta_tau * (0.5 * p.r * sq_diff)
    return dS


# ---------------------------------------------------------------------------
# UDT linear algebra  (src/linalg.jl:20-39, 61, 101-107, 237-283)
# ---------------------------------------------------------------------------
def decompose_udt(A):
    """Column-pivoted QR (LAPACK geqp3): A = U diag(D) T with D = |Re R_ii|,
    T = (D^-1 R)[:, invperm(p)].  src/linalg.jl:20-39."""
    Q, R, piv = sla.qr(A, pivoting=True)
    D = np.abs(np.real(np.diag(R))).copy()
    R = R / D[:, None]
    inv = np.empty_like(piv)
    inv[piv] = np.arange(len(piv))
    return Q, D, R[:, inv]


def multiply_safely(Ul, Dl, Tl, Ur, Dr, Tr):
    """src/linalg.jl:101-107."""
    mat = Tl @ Ur
    mat = Dl[:, None] * mat
    mat = mat * Dr[None, :]
    U, D, T = decompose_udt(mat)
    return Ul @ U, D, T @ Tr


def inv_one_plus_two_udts(Ul, Dl, Tl, Ur, Dr, Tr):
    """[1 + Ul Dl Tl (Ur Dr Tr)^H]^-1 as (U, d, T) with G = U diag(d) T
    after the final swap of roles used by calculate_greens.
    src/stack.jl:338-369 (same algorithm as src/linalg.jl:237-283)."""
    tmp = Tl @ Tr.conj().T
    tmp = tmp * Dr[None, :]
    tmp = Dl[:, None] * tmp
    U, D, T = decompose_udt(tmp)
    U = Ul @ U
    tmp2 = T @ Ur.conj().T
    # myrdiv!(tmp, U', tmp2): tmp = U' / tmp2 = (tmp2' \ U)'   (src/linalg.jl:61)
    tmp = sla.solve(tmp2.conj().T, U).conj().T
    tmp[np.diag_indices_from(tmp)] += D
    u, d, t = decompose_udt(tmp)
    Tt = sla.inv(t @ tmp2)
    Ut = (U @ u).conj().T
    d = 1.0 / d
    return Tt, d, Ut        # G = Tt diag(d) Ut


def greens_from_udts(Ul, Dl, Tl, Ur, Dr, Tr):
    """G and logdet as calculate_greens + calculate_logdet
    (src/stack.jl:338-385)."""
    Tt, d, Ut = inv_one_plus_two_udts(Ul, Dl, Tl, Ur, Dr, Tr)
    G = Tt @ (d[:, None] * Ut)
    logdet = float(np.real(_logdet(Ut) + np.sum(np.log(d)) + _logdet(Tt)))
    return G, logdet


def inv_one_plus_udt_scalettar(U, D, T):
    """[1 + U D T]^-1 with the scales separated (src/linalg.jl:310-339)."""
    Dp = np.maximum(D, 1.0)
    Dm = np.minimum(D, 1.0)
    Dpinv = 1.0 / Dp
    l = sla.solve(T, np.diag(Dpinv).astype(np.complex128))     # T \ Diagonal(Dpinv)
    r = U * Dm[None, :] + l
    u, d, t = decompose_udt(r)
    r = sla.solve(t, np.diag(1.0 / d).astype(np.complex128))     # t \ Diagonal(1/d)
    l = r @ u.conj().T
    l = Dpinv[:, None] * l
    u, d, t = decompose_udt(l)
    l = sla.solve(T, u)
    l = l * d[None, :]
    return l @ t


def inv_sum_udts_scalettar(Ua, Da, Ta, Ub, Db, Tb):
    """[Ua Da Ta + Ub Db Tb]^-1 with the scales separated (src/linalg.jl:512-567)."""
    Dap, Dam = np.maximum(Da, 1.0), np.minimum(Da, 1.0)
    Dbp, Dbm = np.maximum(Db, 1.0), np.minimum(Db, 1.0)
    mat1 = sla.solve(Tb.T, Ta.T).T                              # Ta / Tb
    mat1 = mat1 * (Dam[:, None] / Dbp[None, :])
    mat2 = Ua.conj().T @ Ub
    mat2 = mat2 * (Dbm[None, :] / Dap[:, None])
    mat1 = mat1 + mat2
    U, D, T = decompose_udt(mat1)
    T = D[:, None] * T
    mat1 = sla.solve(T, U.conj().T)                              # T \ U'
    mat1 = mat1 / Dbp[:, None] / Dap[None, :]
    U, D, T = decompose_udt(mat1)
    mat1 = sla.solve(Tb, U)
    mat2 = T @ Ua.conj().T
    return (mat1 * D[None, :]) @ mat2


def _logdet(A):
    sign, ld = np.linalg.slogdet(A)
    return ld  # real part of log(det A)


# ---------------------------------------------------------------------------
# the DQMC state machine
# ---------------------------------------------------------------------------
class DQMCRef:
    """CPU restatement of `DQMC` for the CBAssaad (or CBFalse) O(3) model
    without B-field.  Method names follow the reference."""

    def __init__(self, p: Params, phi=None):
        assert p.L % 2 == 0 or not p.checkerboard, "CBAssaad needs even L"
        assert p.slices % p.safe_mult == 0
        self.p = p
        self.N = p.N
        self.n = p.n
        self.M = p.slices
        self.nb = neighbors_table(p.L)
        self.tn = time_neighbors_table(p.slices)
        self.T, self.eT, self.eTinv = hopping_matrices(p)
        self.cb = checkerboard_matrices(p)
        self.phi = np.zeros((3, self.N, self.M)) if phi is None else np.array(phi, dtype=np.float64)
        self.boson_action_value = 0.0
        self.greens = np.zeros((self.n, self.n), dtype=np.complex128)
        self.log_det = 0.0
        self.current_slice = 0
        self.direction = 1
        self.delta_i = np.zeros((4, 4), dtype=np.complex128)
        self.Mmat = np.zeros((4, 4), dtype=np.complex128)
        self.n_elements = self.M // p.safe_mult + 1
        self.ranges = [range(1 + (i - 1) * p.safe_mult, i * p.safe_mult + 1)
                       for i in range(1, self.n_elements)]
        self.instability = []

    # ---- slice matrices (src/slice_matrices.jl:25-226) -------------------
    def eV(self, slice1, power):
        return interaction_matrix_exp(self.p, self.phi[:, :, slice1 - 1], power)

    def multiply_B_left(self, slice1, A):
        if not self.p.checkerboard:
            B = self.eT @ (self.eT @ self.eV(slice1, 1.0).toarray())
            A[...] = B @ A
            return A
        hh, hf = self.cb[("half", False)], self.cb[("full", False)]
        A[...] = self.eV(slice1, 1.0) @ A
        A *= self.cb["mu"][:, None]
        A[...] = hh[1] @ A
        A[...] = hf[0] @ A
        A[...] = hh[1] @ A
        return A

    def multiply_B_right(self, slice1, A):
        if not self.p.checkerboard:
            B = self.eT @ (self.eT @ self.eV(slice1, 1.0).toarray())
            A[...] = A @ B
            return A
        hh, hf = self.cb[("half", False)], self.cb[("full", False)]
        A[...] = (hh[1].T @ A.T).T
        A[...] = (hf[0].T @ A.T).T
        A[...] = (hh[1].T @ A.T).T
        A *= self.cb["mu"][None, :]
        A[...] = (self.eV(slice1, 1.0).T @ A.T).T
        return A

    def multiply_B_inv_left(self, slice1, A):
        if not self.p.checkerboard:
            B = self.eV(slice1, -1.0) @ (self.eTinv @ self.eTinv)
            A[...] = B @ A
            return A
        hh, hf = self.cb[("half", True)], self.cb[("full", True)]
        A[...] = hh[1] @ A
        A[...] = hf[0] @ A
        A[...] = hh[1] @ A
        A *= self.cb["mu_inv"][:, None]
        A[...] = self.eV(slice1, -1.0) @ A
        return A

    def multiply_B_inv_right(self, slice1, A):
        if not self.p.checkerboard:
            B = self.eV(slice1, -1.0) @ (self.eTinv @ self.eTinv)
            A[...] = A @ B
            return A
        hh, hf = self.cb[("half", True)], self.cb[("full", True)]
        A[...] = (self.eV(slice1, -1.0).T @ A.T).T
        A *= self.cb["mu_inv"][None, :]
        A[...] = (hh[1].T @ A.T).T
        A[...] = (hf[0].T @ A.T).T
        A[...] = (hh[1].T @ A.T).T
        return A

    def multiply_daggered_B_left(self, slice1, A):
        if not self.p.checkerboard:
            B = self.eT @ (self.eT @ self.eV(slice1, 1.0).toarray())
            A[...] = B.conj().T @ A
            return A
        hh, hf = self.cb[("half", False)], self.cb[("full", False)]
        A[...] = hh[1].T @ A          # real hopping factors: dagger == transpose
        A[...] = hf[0].T @ A
        A[...] = hh[1].T @ A
        A *= self.cb["mu"][:, None]
        A[...] = self.eV(slice1, 1.0) @ A   # eV is Hermitian
        return A

    def slice_matrix(self, slice1, power=1.0):
        A = np.eye(self.n, dtype=np.complex128)
        if power > 0:
            return self.multiply_B_left(slice1, A)
        return self.multiply_B_inv_left(slice1, A)

    # ---- wrapping (src/stack.jl:316-332) ---------------------------------
    def wrap_greens_inplace(self, gf, curr_slice, direction):
        if direction == -1:
            self.multiply_B_inv_left(curr_slice - 1, gf)
            self.multiply_B_right(curr_slice - 1, gf)
        else:
            self.multiply_B_left(curr_slice, gf)
            self.multiply_B_inv_right(curr_slice, gf)
        return gf

    def wrap_greens(self, gf, curr_slice, direction):
        return self.wrap_greens_inplace(np.array(gf, dtype=np.complex128), curr_slice, direction)

    # ---- stack (src/stack.jl:251-313) ------------------------------------
    def initialize_stack(self):
        n, ne = self.n, self.n_elements
        self.u_stack = np.zeros((ne, n, n), dtype=np.complex128)
        self.d_stack = np.zeros((ne, n))
        self.t_stack = np.zeros((ne, n, n), dtype=np.complex128)
        eye = np.eye(n, dtype=np.complex128)
        self.Ul, self.Ur, self.Tl, self.Tr = eye.copy(), eye.copy(), eye.copy(), eye.copy()
        self.Dl, self.Dr = np.ones(n), np.ones(n)

    def build_stack(self):
        n = self.n
        self.u_stack[0] = np.eye(n)
        self.d_stack[0] = 1.0
        self.t_stack[0] = np.eye(n)
        for i in range(1, len(self.ranges) + 1):
            self.add_slice_sequence_left(i)
        self.current_slice = self.M + 1
        self.direction = -1

    def add_slice_sequence_left(self, idx):
        """Updates stack[idx+1] from stack[idx] (1-based idx); src/stack.jl:278-293."""
        k = idx - 1
        curr_U = self.u_stack[k].copy()
        for sl in self.ranges[idx - 1]:
            self.multiply_B_left(sl, curr_U)
        curr_U = curr_U * self.d_stack[k][None, :]
        U, D, T = decompose_udt(curr_U)
        self.u_stack[k + 1] = U
        self.d_stack[k + 1] = D
        self.t_stack[k + 1] = T @ self.t_stack[k]

    def add_slice_sequence_right(self, idx):
        """Updates stack[idx] from stack[idx+1] (1-based idx); src/stack.jl:299-313."""
        k = idx - 1
        curr_U = self.u_stack[k + 1].copy()
        for sl in reversed(self.ranges[idx - 1]):
            self.multiply_daggered_B_left(sl, curr_U)
        curr_U = curr_U * self.d_stack[k + 1][None, :]
        U, D, T = decompose_udt(curr_U)
        self.u_stack[k] = U
        self.d_stack[k] = D
        self.t_stack[k] = T @ self.t_stack[k + 1]

    def calculate_greens(self):
        """src/stack.jl:338-369; logdet as src/stack.jl:377-385."""
        self.greens, self.log_det = greens_from_udts(self.Ul, self.Dl, self.Tl,
                                                     self.Ur, self.Dr, self.Tr)

    def _set_l(self, k):
        self.Ul, self.Dl, self.Tl = self.u_stack[k].copy(), self.d_stack[k].copy(), self.t_stack[k].copy()

    def _set_r(self, k):
        self.Ur, self.Dr, self.Tr = self.u_stack[k].copy(), self.d_stack[k].copy(), self.t_stack[k].copy()

    def propagate(self):
        """src/stack.jl:391-499 (including the always-executed wrap of
        greens_temp on the way up, :420, and the all_checks comparison)."""
        p = self.p
        s = p.safe_mult
        n = self.n
        if self.direction == 1:
            if self.current_slice % s == 0:
                self.current_slice += 1
                if self.current_slice == 1:
                    self._set_r(0)
                    self.u_stack[0] = np.eye(n); self.d_stack[0] = 1.0; self.t_stack[0] = np.eye(n)
                    self._set_l(0)
                    self.calculate_greens()
                elif 1 < self.current_slice <= self.M:
                    idx = (self.current_slice - 1) // s
                    self._set_r(idx)
                    self.add_slice_sequence_left(idx)
                    self._set_l(idx)
                    greens_temp = self.greens.copy()
                    self.wrap_greens_inplace(greens_temp, self.current_slice - 1, 1)
                    self.calculate_greens()
                    self.instability.append((self.current_slice, 1,
                                             float(np.max(np.abs(greens_temp - self.greens)))))
                else:
                    idx = self.n_elements - 1
                    self.add_slice_sequence_left(idx)
                    self.direction = -1
                    self.current_slice = self.M + 1
                    self.propagate()
            else:
                self.wrap_greens_inplace(self.greens, self.current_slice, 1)
                self.current_slice += 1
        else:
            if (self.current_slice - 1) % s == 0:
                self.current_slice -= 1
                if self.current_slice == self.M:
                    self._set_l(self.n_elements - 1)
                    e = self.n_elements - 1
                    self.u_stack[e] = np.eye(n); self.d_stack[e] = 1.0; self.t_stack[e] = np.eye(n)
                    self._set_r(e)
                    self.calculate_greens()
                    self.wrap_greens_inplace(self.greens, self.current_slice + 1, -1)
                elif 0 < self.current_slice < self.M:
                    idx = self.current_slice // s + 1
                    self._set_l(idx - 1)
                    self.add_slice_sequence_right(idx)
                    self._set_r(idx - 1)
                    greens_temp = self.greens.copy()
                    self.calculate_greens()
                    self.instability.append((self.current_slice, -1,
                                             float(np.max(np.abs(greens_temp - self.greens)))))
                    self.wrap_greens_inplace(self.greens, self.current_slice + 1, -1)
                else:
                    idx = 1
                    self.add_slice_sequence_right(idx)
                    self.direction = 1
                    self.current_slice = 0
                    self.propagate()
            else:
                self.wrap_greens_inplace(self.greens, self.current_slice, -1)
                self.current_slice -= 1

    # ---- init (src/dqmc_framework.jl:156-177) ----------------------------
    def init(self, phi=None):
        if phi is not None:
            self.phi = np.array(phi, dtype=np.float64)
        self.boson_action_value = boson_action(self.p, self.phi)
        self.initialize_stack()
        self.build_stack()
        self.propagate()

    # ---- local updates (src/local_updates.jl:1-95) -----------------------
    def calc_detratio(self, i, new_op):
        """src/local_updates.jl:42-59; i is the 0-based site."""
        N = self.N
        sl = self.current_slice - 1
        e1 = interaction_op(self.p, self.phi[:, i, sl], -1.0)
        e2 = interaction_op(self.p, new_op, 1.0)
        self.delta_i = e1 @ e2 - np.eye(4)
        Mtmp = np.eye(4) - self.greens[i::N, i::N]
        self.Mmat = np.eye(4) + self.delta_i @ Mtmp
        return complex(np.linalg.det(self.Mmat))

    def update_greens(self, i):
        """src/local_updates.jl:61-95; i is the 0-based site."""
        N = self.N
        A = self.greens[:, i::N].copy()
        for k in range(4):
            A[i + k * N, k] -= 1.0
        A = A @ np.linalg.inv(self.Mmat)
        B = self.delta_i @ self.greens[i::N, :]
        self.greens += A @ B

    def local_updates(self, delta, uniforms, record=None):
        """One local-update pass over all sites of the current slice
        (src/local_updates.jl:1-38) with fixed-slot streams: delta has
        shape (3, N) (the proposal shifts, already in [-box, box]) and
        uniforms shape (N,).  The uniform of site i is consumed only when
        p_acc <= 1, exactly as `p_acc > 1.0 || rand() < p_acc`."""
        N = self.N
        sl = self.current_slice - 1
        acc = 0
        for i in range(N):
            new_op = self.phi[:, i, sl] + delta[:, i]
            dS = boson_action_diff(self.p, self.phi, self.nb, self.tn, i, sl, new_op)
            exp_dS = math.exp(-dS)
            detratio = self.calc_detratio(i, new_op)
            p_acc = exp_dS * detratio.real
            accepted = p_acc > 1.0 or uniforms[i] < p_acc
            if record is not None:
                record.append((self.current_slice, i, accepted, detratio, p_acc, float(uniforms[i])))
            if accepted:
                acc += 1
                self.phi[:, i, sl] = new_op
                self.boson_action_value += -math.log(exp_dS)
                self.update_greens(i)
        return acc / N

    def global_update(self, shift, u):
        """src/global_updates.jl:18-58 with a fixed-slot shift (3,) (already in
        [-box_global, box_global]) and Metropolis uniform u.  Needs the state
        (M, -1).  Returns (accepted, p_acc)."""
        assert self.current_slice == self.M and self.direction == -1
        S_old = self.boson_action_value
        backup = (self.u_stack.copy(), self.d_stack.copy(), self.t_stack.copy(), self.greens.copy(),
                  self.log_det, self.phi.copy())
        for k in range(3):
            self.phi[k, :, :] += shift[k]
        self.build_stack()
        self.propagate()
        self.boson_action_value = boson_action(self.p, self.phi)
        p_boson = math.exp(-(self.boson_action_value - S_old))
        p_fermion = math.exp(backup[4] - self.log_det)
        p_acc = p_boson * p_fermion
        if p_acc > 1.0 or u < p_acc:
            return True, p_acc
        self.boson_action_value = S_old
        self.u_stack, self.d_stack, self.t_stack, self.greens, self.log_det, self.phi = backup
        return False, p_acc

    def update(self, delta, uniforms, record=None):
        """src/dqmc_framework.jl:500-517 with global updates off."""
        self.propagate()
        return self.local_updates(delta, uniforms, record)

    def sweep(self, n_calls, delta_stream, u_stream, record=None):
        """n_calls update() calls; delta_stream (n_calls, 3, N), u_stream (n_calls, N)."""
        acc = 0.0
        for c in range(n_calls):
            acc += self.update(delta_stream[c], u_stream[c], record)
        return acc / max(n_calls, 1)

    # ---- from-scratch G (src/fermion_measurements.jl:964-1101) -----------
    def calc_Bchain(self, start, stop):
        n = self.n
        U = np.eye(n, dtype=np.complex128); D = np.ones(n); T = np.eye(n, dtype=np.complex128)
        for k in range(start, stop + 1):
            self.multiply_B_left(k, U)
            if k % self.p.safe_mult == 0 or k == stop:
                U = U * D[None, :]
                U, D, Tn = decompose_udt(U)
                T = Tn @ T
        return U, D, T

    def calc_Bchain_dagger(self, start, stop):
        n = self.n
        U = np.eye(n, dtype=np.complex128); D = np.ones(n); T = np.eye(n, dtype=np.complex128)
        for k in range(stop, start - 1, -1):
            self.multiply_daggered_B_left(k, U)
            if k % self.p.safe_mult == 0 or k == start:
                U = U * D[None, :]
                U, D, Tn = decompose_udt(U)
                T = Tn @ T
        return U, D, T

    def calc_greens_and_logdet(self, slice1):
        n = self.n
        Ur, Dr, Tr = self.calc_Bchain_dagger(slice1, self.M)
        if slice1 - 1 >= 1:
            Ul, Dl, Tl = self.calc_Bchain(1, slice1 - 1)
        else:
            Ul = np.eye(n, dtype=np.complex128); Dl = np.ones(n); Tl = np.eye(n, dtype=np.complex128)
        Tt, d, Ut = inv_one_plus_two_udts(Ul, Dl, Tl, Ur, Dr, Tr)
        ld = float(np.real(_logdet(Tt) + np.sum(np.log(d)) + _logdet(Ut)))
        return Tt @ (d[:, None] * Ut), ld

    def calc_greens(self, slice1):
        return self.calc_greens_and_logdet(slice1)[0]

    # ---- measurement hooks -----------------------------------------------
    def effective_greens2greens(self, G):
        """src/fermion_measurements.jl:1125-1142."""
        hh, hhi = self.cb[("half", False)], self.cb[("half", True)]
        G = np.array(G, dtype=np.complex128)
        for g in (1, 0):
            G = (hh[g].T @ G.T).T
        for g in (1, 0):
            G = hhi[g] @ G
        return G

    def measured_greens(self):
        """The true G pushed by _measure_observables! at slice M, dir -1
        (src/dqmc_framework.jl:378-381)."""
        g = self.wrap_greens(self.greens, self.current_slice, 1)
        return self.effective_greens2greens(g)

    # ---- time-displaced Green's functions (src/fermion_measurements.jl:1343-1516) ----
    def calc_Bchain_udts(self, invert, direction):
        """calc_Bchain_udts! (src/fermion_measurements.jl:1411-1488): UDTs of
        the B chains at the safe_mult ranges.  direction 'left': B(tau, 1) =
        B(tau)...B(1) (invert: its inverse, accumulated from the right);
        'right': B(beta, tau) = B(beta)...B(tau) (invert: its inverse,
        accumulated from the left).  Lists indexed by range i (0-based), in the
        reference's order after its final reverse for 'right'."""
        s, M, n = self.p.safe_mult, self.M, self.n
        ranges = [list(range(i * s + 1, (i + 1) * s + 1)) for i in range(M // s)]
        rightmult = (direction == "right" and not invert) or (direction == "left" and invert)
        order = list(range(len(ranges)))
        if direction == "right":
            order = order[::-1]
        us, ds, ts = [], [], []
        for i, ridx in enumerate(order):
            if i == 0:
                cur = np.eye(n, dtype=np.complex128)
            else:
                cur = (ts[i - 1] if rightmult else us[i - 1]).copy()
            seq = ranges[ridx][::-1] if direction == "right" else ranges[ridx]
            for sl in seq:
                if not invert:
                    if direction == "left":
                        self.multiply_B_left(sl, cur)
                    else:
                        self.multiply_B_right(sl, cur)
                else:
                    if direction == "left":
                        self.multiply_B_inv_right(sl, cur)
                    else:
                        self.multiply_B_inv_left(sl, cur)
            if i != 0:
                cur = ds[i - 1][:, None] * cur if rightmult else cur * ds[i - 1][None, :]
            U, D, T = decompose_udt(cur)
            if not rightmult:
                us.append(U)
                ts.append(T if i == 0 else T @ ts[i - 1])
            else:
                ts.append(T)
                us.append(U if i == 0 else us[i - 1] @ U)
            ds.append(D)
        if direction == "right":
            us.reverse(), ds.reverse(), ts.reverse()
        return us, ds, ts

    def fill_tdgf(self, Gt0, G0t):
        """fill_tdgf! (src/fermion_measurements.jl:1497-1523): propagate from the
        safe_mult slices to the others; Gt0, G0t are lists indexed by slice-1."""
        s, M = self.p.safe_mult, self.M
        safe = set(range(1, M + 1, s))
        Mhalf = M // 2 + 1
        for tau in range(Mhalf, M + 1):
            if tau in safe:
                continue
            Gt0[tau - 1] = self.multiply_B_left(tau, Gt0[tau - 2].copy())
            G0t[tau - 1] = self.multiply_B_inv_right(tau, G0t[tau - 2].copy())
        for tau in range(Mhalf - 1, 0, -1):
            if tau in safe:
                continue
            Gt0[tau - 1] = self.multiply_B_inv_left(tau + 1, Gt0[tau].copy())
            G0t[tau - 1] = self.multiply_B_right(tau + 1, G0t[tau].copy())

    def measure_tdgfs(self):
        """measure_tdgfs! (src/fermion_measurements.jl:1343-1403): Gt0[tau] and
        G0t[tau] (tau = 1..M, returned as (M, n, n) arrays) for the current field."""
        s, M = self.p.safe_mult, self.M
        BT0Inv = self.calc_Bchain_udts(True, "left")
        BBetaT = self.calc_Bchain_udts(False, "right")
        BT0 = self.calc_Bchain_udts(False, "left")
        BBetaTInv = self.calc_Bchain_udts(True, "right")
        # zero blocks as allocate_tdgfs! (:1247-1248): when M/2 is not a multiple
        # of safe_mult, fill_tdgf! starts from a slice it has not filled yet
        Gt0 = [np.zeros((self.n, self.n), dtype=np.complex128) for _ in range(M)]
        G0t = [np.zeros((self.n, self.n), dtype=np.complex128) for _ in range(M)]
        for i, tau in enumerate(range(1, M + 1, s)):
            if i != 0:
                g1 = inv_sum_udts_scalettar(BT0Inv[0][i - 1], BT0Inv[1][i - 1], BT0Inv[2][i - 1],
                                            BBetaT[0][i], BBetaT[1][i], BBetaT[2][i])
                g2 = inv_sum_udts_scalettar(BT0[0][i - 1], BT0[1][i - 1], BT0[2][i - 1],
                                            BBetaTInv[0][i], BBetaTInv[1][i], BBetaTInv[2][i])
            else:
                g1 = inv_one_plus_udt_scalettar(BBetaT[0][0], BBetaT[1][0], BBetaT[2][0])
                g2 = inv_one_plus_udt_scalettar(BBetaTInv[0][0], BBetaTInv[1][0], BBetaTInv[2][0])
            Gt0[tau - 1] = self.effective_greens2greens(g1)
            G0t[tau - 1] = self.effective_greens2greens(g2)
        self.fill_tdgf(Gt0, G0t)
        return np.array(Gt0), -np.array(G0t)

    def kinetic_energy(self, G_true):
        """E_kin = sum_ij T_ij <c_i^dag c_j> with <c_i^dag c_j> = delta_ij - G_ji.
        Not an observable of the reference; defined here from its hopping
        matrix (src/hoppings.jl:85) and G convention."""
        cdc = np.eye(self.n) - G_true.T
        return float(np.real(np.sum(self.T * cdc)))


# ---------------------------------------------------------------------------
# equal-time fermion correlators (src/fermion_measurements.jl:363-653)
# ---------------------------------------------------------------------------
def _site_pbc(L, x, y):
    """siteidx (src/fermion_measurements.jl:7-12), 0-based: sql[y, x] = y + L x with PBC."""
    return np.mod(y, L) + L * np.mod(x, L)


def _origins(L):
    x0, y0 = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
    return x0.ravel(), y0.ravel()


def measure_etpc(L, G):
    """measure_etpc! (src/fermion_measurements.jl:388-424) with _pc_ev (:435-449)
    for opdim 3 (G accessed directly, :23-26).  Flavours xu, yd, xd, yu are
    0, 1, 2, 3 here; index = flavour N + site.  Returns (P_plus, P_minus), each
    L x L real with [y, x] the displacement, averaged over the origins r0."""
    N = L * L
    xu, yd, xd, yu = 0, 1, 2, 3
    js = ((xd, xu, xu, xd), (xd, xu, yu, yd), (yd, yu, xu, xd), (yd, yu, yu, yd))
    x0, y0 = _origins(L)
    r0 = _site_pbc(L, x0, y0)
    Pp = np.zeros((L, L))
    Pm = np.zeros((L, L))
    for x in range(L):
        for y in range(L):
            ri = _site_pbc(L, x0 + x, y0 + y)
            ev = []
            for j in js:
                i1, i2, i3, i4 = j[0] * N + ri, j[1] * N + ri, j[2] * N + r0, j[3] * N + r0
                ev.append(np.real(G[i1, i4] * G[i2, i3] - G[i1, i3] * G[i2, i4]))
            Pm[y, x] = np.sum(ev[0] - ev[1] - ev[2] + ev[3]) / N
            Pp[y, x] = np.sum(ev[0] + ev[1] + ev[2] + ev[3]) / N
    return Pp, Pm


def measure_etcdc(L, G):
    """measure_etcdc! (src/fermion_measurements.jl:592-630) with _etcdc_ev
    (:641-653): bands X = 1, Y = 2 and spins UP = 0, DOWN = 2 give the 1-based
    flavour band + spin.  Returns (C_plus, C_minus), L x L complex, [y, x] the
    displacement, averaged over the origins."""
    N = L * L
    X, Y = 1, 2
    x0, y0 = _origins(L)
    r0 = _site_pbc(L, x0, y0)
    Cp = np.zeros((L, L), dtype=np.complex128)
    Cm = np.zeros((L, L), dtype=np.complex128)

    def ev(ri, j1, j2, j3, j4):
        i1, i2 = (j1 - 1) * N + ri, (j2 - 1) * N + ri
        i3, i4 = (j3 - 1) * N + r0, (j4 - 1) * N + r0
        uncorr = ((i1 == i2) - G[i2, i1]) * ((i3 == i4) - G[i4, i3])
        return uncorr + ((i1 == i4) - G[i4, i1]) * G[i2, i3]

    for s1 in (0, 2):
        for s2 in (0, 2):
            for x in range(L):
                for y in range(L):
                    ri = _site_pbc(L, x0 + x, y0 + y)
                    e1 = ev(ri, X + s1, X + s1, X + s2, X + s2)
                    e2 = ev(ri, X + s1, X + s1, Y + s2, Y + s2)
                    e3 = ev(ri, Y + s1, Y + s1, X + s2, X + s2)
                    e4 = ev(ri, Y + s1, Y + s1, Y + s2, Y + s2)
                    Cm[y, x] += np.sum(e1 - e2 - e3 + e4)
                    Cp[y, x] += np.sum(e1 + e2 + e3 + e4)
    return Cp / N, Cm / N


def measure_zfpc(L, Gt0s):
    """measure_zfpc! (src/fermion_measurements.jl:500-541): the pairing
    correlators of measure_etpc summed over G(tau, 0), tau = 1..M (origin mean
    only, no division by M).  Returns (P_plus, P_minus)."""
    Pp = np.zeros((L, L))
    Pm = np.zeros((L, L))
    for g in Gt0s:
        a, b = measure_etpc(L, g)
        Pp += a
        Pm += b
    return Pp, Pm


def measure_zfcdc(L, greens, Gt0s, G0ts):
    """measure_zfcdc! (src/fermion_measurements.jl:688-743) with _zfcdc_ev
    (:753-766): greens is one true equal-time G (used as G(tau) and G(0) for
    every tau), Gt0s[tau] = G(tau, 0) and G0ts[tau] the reference's stored
    -G(0, tau).  Summed over tau = 1..M and averaged over the origins.
    Returns (C_plus, C_minus), L x L complex indexed [y, x]."""
    N = L * L
    X, Y = 1, 2
    x0, y0 = _origins(L)
    r0 = _site_pbc(L, x0, y0)
    Cp = np.zeros((L, L), dtype=np.complex128)
    Cm = np.zeros((L, L), dtype=np.complex128)
    for Gt0, G0t in zip(Gt0s, G0ts):
        Gtau = G0 = greens

        def ev(ri, j1, j2, j3, j4):
            i1, i2 = (j1 - 1) * N + ri, (j2 - 1) * N + ri
            i3, i4 = (j3 - 1) * N + r0, (j4 - 1) * N + r0
            uncorr = ((i1 == i2) - Gtau[i2, i1]) * ((i3 == i4) - G0[i4, i3])
            return uncorr + (-G0t[i4, i1]) * Gt0[i2, i3]

        for s1 in (0, 2):
            for s2 in (0, 2):
                for x in range(L):
                    for y in range(L):
                        ri = _site_pbc(L, x0 + x, y0 + y)
                        e1 = ev(ri, X + s1, X + s1, X + s2, X + s2)
                        e2 = ev(ri, X + s1, X + s1, Y + s2, Y + s2)
                        e3 = ev(ri, Y + s1, Y + s1, X + s2, X + s2)
                        e4 = ev(ri, Y + s1, Y + s1, Y + s2, Y + s2)
                        Cm[y, x] += np.sum(e1 - e2 - e3 + e4)
                        Cp[y, x] += np.sum(e1 + e2 + e3 + e4)
    return Cp / N, Cm / N


def measure_zfccc(L, T, greens, Gt0s, G0ts):
    """measure_zfccc! (src/fermion_measurements.jl:814-888): zero-frequency
    current-current correlators from the hopping matrix T (n x n, the
    reference's mc.l.hopping_matrix), one true equal-time G, G(tau, 0) and the
    stored -G(0, tau).  Returns (Lambda_xx, Lambda_yy), L x L complex [y, x],
    summed over tau, averaged over the origins and negated (i^2)."""
    N = L * L
    x0, y0 = _origins(L)
    r0 = _site_pbc(L, x0, y0)
    out = []
    for dx, dy in ((1, 0), (0, 1)):
        lam = np.zeros((L, L), dtype=np.complex128)
        r0p = _site_pbc(L, x0 + dx, y0 + dy)
        for Gt0, G0t in zip(Gt0s, G0ts):
            Gtau = G0 = greens
            for f1 in range(4):
                for f2 in range(4):
                    for x in range(L):
                        for y in range(L):
                            ri = _site_pbc(L, x0 + x, y0 + y)
                            rj = _site_pbc(L, x0 + x + dx, y0 + y + dy)
                            ais, ajs = f1 * N + ri, f1 * N + rj
                            a0, a0p = f2 * N + r0, f2 * N + r0p
                            tij, tji = T[ais, ajs], T[ajs, ais]
                            t00p, t0p0 = T[a0, a0p], T[a0p, a0]
                            v = (tij * Gtau[ajs, ais] - tji * Gtau[ais, ajs]) * \
                                (t00p * G0[a0p, a0] - t0p0 * G0[a0, a0p])
                            v = v - tij * t00p * G0t[a0p, ais] * Gt0[ajs, a0] \
                                + tij * t0p0 * G0t[a0, ais] * Gt0[ajs, a0p] \
                                + tji * t00p * G0t[a0p, ajs] * Gt0[ais, a0] \
                                - tji * t0p0 * G0t[a0, ajs] * Gt0[ais, a0p]
                            lam[y, x] += np.sum(v)
        out.append(lam / -N)
    return out[0], out[1]


def measure_sfdensity(lambda_xx):
    """measure_sfdensity (src/fermion_measurements.jl:911-920): with q the real
    2D DFT of Re Lambda_xx (first index y), rho_s = (Re q[0, 1] - Re q[1, 0]) / 4."""
    q = np.fft.rfft2(np.real(np.asarray(lambda_xx)).T).T   # halve the first (y) axis, as Julia's rfft
    return 0.25 * (np.real(q[0, 1]) - np.real(q[1, 0]))


def is_reflection_symmetric(a, tol=1e-12):
    """is_reflection_symmetric (src/fermion_measurements.jl:179-201): the inner
    block a[1:, 1:] equals its reversal along each axis, and the first row and
    column without their corner equal their reversals, within tol (the
    reference compares the maximum of the signed difference)."""
    a = np.asarray(a)
    inner = a[1:, 1:]
    parts = [inner - np.flip(inner, axis=0), inner - np.flip(inner, axis=1),
             a[0, 1:] - a[0, 1:][::-1], a[1:, 0] - a[1:, 0][::-1]]
    return all(np.max(np.real(d)) < tol and np.max(np.imag(d)) < tol for d in parts)


# ---------------------------------------------------------------------------
# gradients of the log-weight (not in the reference; built from its pieces)
# ---------------------------------------------------------------------------
def interaction_op_derivs(p: Params, op):
    """E = exp(-dtau V(op)) (power +1) of one site and dE/dop_a, a = 0..2,
    from C = cosh(x), S = (i op2 - op1) sh, R = -op3 sh, sh = sinh(x)/|op|,
    x = lambda dtau |op| (src/interactions.jl:102-141)."""
    nrm = math.sqrt(op[0] ** 2 + op[1] ** 2 + op[2] ** 2)
    x = p.lambda_ * p.delta_tau * nrm
    sh = math.sinh(x) / nrm
    C = math.cosh(x)
    dsh = (p.lambda_ * p.delta_tau * C - sh) / nrm ** 2      # (d sh / d op_a) / op_a
    out = []
    for a in range(3):
        dC = p.lambda_ * p.delta_tau * op[a] * sh
        dS = (1j * op[1] - op[0]) * dsh * op[a] + ((1j if a == 1 else 0) - (1 if a == 0 else 0)) * sh
        dR = -op[2] * dsh * op[a] - (sh if a == 2 else 0.0)
        e = np.zeros((4, 4), dtype=np.complex128)
        e[0, 0] = dC; e[0, 1] = dS; e[1, 0] = np.conj(dS); e[1, 1] = dC
        e[0, 3] = dR; e[1, 2] = -dR; e[2, 1] = -dR; e[2, 2] = dC; e[2, 3] = np.conj(dS)
        e[3, 0] = dR; e[3, 2] = dS; e[3, 3] = dC
        out.append(e)
    return out


def force_logdetM(mc: "DQMCRef"):
    """d log|det M| / d phi[a, i, l] = -Re tr(G_l[ii] E_i^-1 dE_i/dphi_a), with
    M = 1 + B_M ... B_1 and G_l the equal-time G of slice l (computed from
    scratch, src/fermion_measurements.jl:1061)."""
    p, N, M = mc.p, mc.N, mc.M
    grad = np.zeros((3, N, M))
    for l in range(1, M + 1):
        G = mc.calc_greens(l)
        for i in range(N):
            op = mc.phi[:, i, l - 1]
            Einv = interaction_op(p, op, -1.0)
            dE = interaction_op_derivs(p, op)
            Gii = G[i::N, i::N]
            for a in range(3):
                grad[a, i, l - 1] = -np.real(np.trace(Gii @ Einv @ dE[a]))
    return grad


def force_boson(p: Params, phi):
    """d S_boson / d phi (src/action.jl:1-52)."""
    L, M = p.L, phi.shape[2]
    h = phi.reshape((3, L, L, M), order="F")
    g = (2 * h - np.roll(h, -1, axis=3) - np.roll(h, 1, axis=3)) / (p.delta_tau * p.c ** 2)
    if not p.edrun:
        nb = np.roll(h, -1, axis=1) + np.roll(h, 1, axis=1) + np.roll(h, -1, axis=2) + np.roll(h, 1, axis=2)
        g = g + p.delta_tau * (4 * h - nb)
    else:
        g = np.zeros_like(h)
    sq = np.sum(h * h, axis=0)[None]
    g = g + p.delta_tau * (p.r * h + (0.0 if p.edrun else p.u) * sq * h)
    return g.reshape((3, L * L, M), order="F")


def log_weight_parts(mc: "DQMCRef"):
    """(log|det M|, S_boson) of the current field; log|det M| = -log|det G|."""
    _, ld = mc.calc_greens_and_logdet(1)
    return -ld, boson_action(mc.p, mc.phi)


def hmc_update(mc: "DQMCRef", momenta, n_steps, eps, u):
    """Hybrid Monte Carlo move on S_eff = S_boson - log|det M| (the
    log-weight whose ratio src/global_updates.jl:18-58 accepts on):
    H = |pi|^2/2 + S_eff, n_steps leapfrog steps of size eps with the force
    -dS_eff/dphi = force_logdetM - force_boson, then accept if p > 1 or
    u < p with p = exp(-dH); a rejection restores the field.  The state is
    rebuilt with init() afterwards.  Returns (accepted, dH)."""
    p = mc.p
    phi0 = mc.phi.copy()
    pi = np.array(momenta, dtype=np.float64).reshape(phi0.shape)

    def H(phi, pi):
        mc.phi = phi
        ldm, sb = log_weight_parts(mc)
        return 0.5 * float(np.sum(pi * pi)) + sb - ldm

    def force(phi):
        mc.phi = phi
        return force_logdetM(mc) - force_boson(p, phi)

    H0 = H(phi0.copy(), pi)
    phi = phi0.copy()
    F = force(phi.copy())
    for _ in range(n_steps):
        pi = pi + 0.5 * eps * F
        phi = phi + eps * pi
        F = force(phi.copy())
        pi = pi + 0.5 * eps * F
    dH = H(phi.copy(), pi) - H0
    pacc = math.exp(-dH)
    acc = pacc > 1.0 or u < pacc
    mc.phi = phi if acc else phi0
    mc.init()
    return acc, dH


# ---------------------------------------------------------------------------
# boson measurements  (src/boson_measurements.jl:6-56)
# ---------------------------------------------------------------------------
def measure_chi_dynamic(conf, delta_tau=0.1):
    opdim, N, M = conf.shape
    L = int(round(math.sqrt(N)))
    h = conf.reshape((opdim, L, L, M), order="F")
    ft = np.fft.rfftn(h, axes=(2, 3, 1))       # halves axis 1 (y), as Julia rfft on dims [2,3,4]
    c = np.sum(np.real(ft * np.conj(ft)), axis=0)
    n = L // 2 + 1
    nt = M // 2 + 1
    return delta_tau / (N * M) * c[:, :n, :nt]


def measure_chi_static(conf, delta_tau=0.1):
    return float(measure_chi_dynamic(conf, delta_tau)[0, 0, 0])


def measure_op(conf):
    """measure_op (src/boson_measurements.jl:41-45): mean |phi| over all
    components, sites and slices, and the mean of each component."""
    conf = np.asarray(conf)
    return float(np.mean(np.abs(conf))), conf.mean(axis=(1, 2))


def measure_binder_factors(conf):
    m = conf.mean(axis=(1, 2))
    m2 = float(m @ m)
    return m2, m2 * m2


# ---------------------------------------------------------------------------
# synthetic inputs (seeded; no dataset is involved)
# ---------------------------------------------------------------------------
def synthetic_field(N, M, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(-1.0, 1.0, size=(3, N, M))


def synthetic_streams(N, n_calls, box, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    delta = rng.uniform(-box, box, size=(n_calls, 3, N))
    u = rng.uniform(0.0, 1.0, size=(n_calls, N))
    return delta, u
