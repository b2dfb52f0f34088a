"""Verified solution of Emden's equation on the unit square, on the GPU.

-Laplace(u) = u^2 in (0, 1)^2, u = 0 on the boundary, in the Legendre basis
of VCP's Legendre_Bases_Generator (vcp/ldbase.hpp), following the driver
test_PDE/test_Emden.cpp step by step:

1. Newton's method for the Galerkin system (test_Emden.cpp:100-145):
   DF = DL - 2 (uh phi_i, phi_j),  F = DL uh - (uh^2, phi_j),
   uh <- uh - DF^-1 F, from uh = 200 (1, ..., 1) with uh(0) = 600, on the
   even list (setting_evenlist: functions symmetric about 1/2, dimension
   ceil(M/2)^2).  The reference runs it in kv::dd; here in FP64 with the
   products on the GPU (an approximation, as there).
2. The inverse-norm bound K >= ||F'[uh]^-1|| (:173-252): the interval matrix
   (uh phi_i, phi_j) = Phi diag(w uh) Phi^T -- the reference's O(n^2 P)
   element loop (ldbase.hpp:994-1001) as one interval product on the GPU --,
   the stiffness matrix DL (exact rationals, dphidphi :1151-1223), the
   verified generalized eigenvalues of (2 (uh phi, phi), DL) (imats::eigsymge
   on the GPU), and K = max |E / (1 - E)| with
   E = lambda / (1 + CN^2 ||f'(uh)||_inf lambda) (upper end kept at lambda's).
3. The residual bound ||Laplace(uh) + uh^2||_L2 (:254-293), as
   sqrt(sum_q w_q r_q^2) with r_q = Laplace(uh)(x_q) + uh(x_q)^2 at Gauss
   points exact for the degree of r^2: the same quantity as the reference's
   sqrt(|(Luh, Luh) + 2 (Luh, uh^2) + (uh^2, uh^2)|), summed pointwise so
   that the cancellation happens in r_q, not between three large integrals.
4. G = 2 Cs3^3 and the Kantorovich check alpha omega <= 1/2 with
   alpha = K Cp ||r||, omega = K G; the H^1_0 error bound
   (1 - sqrt(1 - 2 alpha omega)) / omega (:295-365).

Every interval quantity is rigorous: the tables (vcp_gb300.legendre) enclose
the exact Gauss nodes, weights and basis values; products run in interval
arithmetic with directed rounding (pidcuda, the tensor-basis kernel,
vcp_gb300.ivnp); the constants use mpmath's interval arithmetic.  A
``Products`` object supplies the arithmetic: ``GpuProducts(form)`` runs on
the GPU in the plain FP64 or the tensor-core form; a host implementation
with the same methods gives the CPU pipeline.
"""
from __future__ import annotations

import time
import os
from dataclasses import dataclass, field
from fractions import Fraction

import numpy as np

from . import ivnp as V
from . import legendre

P_EXP = 2  # -Laplace(u) = u^p


# ---------------------------------------------------------------- lists, sizes

def even_list(M: int) -> tuple[np.ndarray, np.ndarray]:
    """Basis index pairs (a, b) of setting_evenlist (ldbase.hpp:279-312):
    row r = i0 * mn + i1 holds (2 i0, 2 i1), mn = ceil(M / 2)."""
    mn = (M + 1) // 2
    r = np.arange(mn * mn)
    return (2 * (r // mn)).astype(np.int32), (2 * (r % mn)).astype(np.int32)


def npts_inverse(M: int, p: int = P_EXP) -> int:
    """Gauss points per dimension of the inverse-norm generator
    (setting(M, p, 2, 1, 1, M), ldbase.hpp:712-728)."""
    nn1 = ((p - 1) * (M + 2) + 2 * (M + 2) + 2) // 2 + 2
    nn2 = (p * (M + 2) + (M + 2) + 2) // 2 + 2
    n = max(nn1, nn2)
    return n + (n % 2)


def npts_residual(M: int, p: int = P_EXP) -> int:
    """Gauss points per dimension of the residual generator (mode 2,
    ldbase.hpp:741-753)."""
    n = (2 * (M + 2) * p + 1) // 2 + 2
    return n + (n % 2)


# ---------------------------------------------------------------- DL (exact)

def _one_dim(M: int):
    """OneDimL and OneDimDL of dphidphi (ldbase.hpp:1165-1186), exact."""
    L1 = [[Fraction(0)] * M for _ in range(M)]
    for i in range(M):
        L1[i][i] = Fraction(1, 2 * (2 * i + 1) * (2 * i + 5) * (2 * i + 3))
        if i + 2 < M:
            v = Fraction(-1, 4 * (2 * i + 5) * (2 * i + 7) * (2 * i + 3))
            L1[i][i + 2] = v
            L1[i + 2][i] = v
    D1 = [Fraction(1, 2 * i + 3) for i in range(M)]
    return L1, D1


def _frac_down(fr: Fraction) -> float:
    f = float(fr)
    return float(np.nextafter(f, -np.inf)) if Fraction(f) > fr else f


def _frac_up(fr: Fraction) -> float:
    f = float(fr)
    return float(np.nextafter(f, np.inf)) if Fraction(f) < fr else f


def _stiffness_entries(M: int, ia: np.ndarray, ib: np.ndarray):
    """The non-zero entries of DL: (rows, cols, lo, hi, mid)."""
    L1, D1 = _one_dim(M)
    where = {(int(a), int(b)): r for r, (a, b) in enumerate(zip(ia, ib))}
    rows, cols, lo, hi, mid = [], [], [], [], []
    for r in range(ia.size):
        a, b = int(ia[r]), int(ib[r])
        for c in (a - 2, a, a + 2):
            for d in (b - 2, b, b + 2):
                s = where.get((c, d))
                if s is None:
                    continue
                v = (D1[a] if a == c else 0) * L1[b][d] + L1[a][c] * (D1[b] if b == d else 0)
                if v != 0:
                    rows.append(r)
                    cols.append(s)
                    lo.append(_frac_down(v))
                    hi.append(_frac_up(v))
                    mid.append(float(v))
    return (np.array(rows, dtype=np.int64), np.array(cols, dtype=np.int64), np.array(lo),
            np.array(hi), np.array(mid))


def stiffness(M: int, ia: np.ndarray, ib: np.ndarray, use_cache: bool = True):
    """DL = ((grad phi_r, grad phi_s))_{r,s} for the basis list (ia, ib):
    D1 (x) L1 + L1 (x) D1 evaluated exactly, rounded outward.  Returns
    (lo, hi, mid) n x n arrays (mid = nearest double).  Only |a - c| and
    |b - d| in {0, 2} give non-zero entries (L1 is pentadiagonal with a zero
    first off-diagonal, D1 diagonal), so each row visits nine neighbours.
    For the even list of M the non-zero entries are cached beside the
    Legendre tables (they depend on M alone)."""
    n = ia.size
    ea, eb = even_list(M)
    path = None
    if use_cache and np.array_equal(ia, ea) and np.array_equal(ib, eb):
        path = legendre._CACHE / f"stiffness_even_M{M}_v1.npz"
    ent = None
    if path is not None and path.exists():
        with np.load(path) as z:
            ent = tuple(z[k] for k in ("rows", "cols", "lo", "hi", "mid"))
    if ent is None:
        ent = _stiffness_entries(M, ia, ib)
        if path is not None:
            try:
                path.parent.mkdir(parents=True, exist_ok=True)
                tmp = path.with_suffix(".tmp.npz")
                np.savez(tmp, **dict(zip(("rows", "cols", "lo", "hi", "mid"), ent)))
                os.replace(tmp, path)
            except OSError:
                pass
    rows, cols, elo, ehi, emid = ent
    lo = np.zeros((n, n))
    hi = np.zeros((n, n))
    mid = np.zeros((n, n))
    lo[rows, cols] = elo
    hi[rows, cols] = ehi
    mid[rows, cols] = emid
    return lo, hi, mid


# ---------------------------------------------------------------- constants

def _iv():
    import mpmath
    mpmath.iv.dps = 40
    return mpmath.iv


def ritz_constant(N: int):
    """CN of Ritz_projection_error (ldbase.hpp:2025-2052): ||grad(u - R u)||
    <= CN ||Laplace u||."""
    iv = _iv()
    s3, s7, s11 = iv.sqrt(2 * N + 3), iv.sqrt(2 * N + 7), iv.sqrt(2 * N + 11)
    L1 = iv.mpf(1) / (2 * (2 * N + 1) * (2 * N + 5)) + 1 / ((4 * (2 * N + 5)) * s3 * s7)
    L2 = (1 / (4 * (2 * N + 5) * s3 * s7) + iv.mpf(1) / (2 * (2 * N + 5) * (2 * N + 9)) +
          1 / (4 * (2 * N + 9) * s7 * s11))
    return iv.sqrt(iv.mpf(max(L1.b, L2.b)))


def poincare_constant(dim: int = 2):
    """Cp = 1 / (sqrt(dim) pi) (ldbase.hpp:2073-2082)."""
    iv = _iv()
    return 1 / (iv.sqrt(dim) * iv.pi)


def sobolev_constant(p, dim: int = 2):
    """Cs_p of Sobolev_constant (ldbase.hpp:2102-2147) for dim = 2, p > 2:
    with q = n p / (n + p), pi^-1/2 n^-1/q ((q-1)/(n-q))^(1-1/q)
    (Gamma(1+n/2) Gamma(n) / (Gamma(n/q) Gamma(1+n-n/q)))^(1/n)."""
    iv = _iv()
    n = iv.mpf(dim)
    q = n * p / (n + p)
    g = (iv.gamma(1 + n / 2) * iv.gamma(n)) / (iv.gamma(n / q) * iv.gamma(1 + n - n / q))
    return (iv.pi ** iv.mpf(-0.5)) * n ** (-1 / q) * ((q - 1) / (n - q)) ** (1 - 1 / q) * \
        g ** (1 / n)


def _iv_of(lo: float, hi: float):
    return _iv().mpf([lo, hi])


# ---------------------------------------------------------------- products

def table_kv(lo: np.ndarray, hi: np.ndarray) -> np.ndarray:
    """(rows x cols) endpoint arrays -> flat kv buffer, column-major."""
    out = np.empty((lo.shape[1], lo.shape[0], 2))
    out[:, :, 0] = lo.T
    out[:, :, 1] = hi.T
    return out.reshape(-1)


class GpuProducts:
    """The Emden pipeline's arithmetic on the GPU: interval products in the
    given form (pidcuda.FORM_PLAIN or FORM_OZAKI), the tensor-basis kernel,
    the eigenvalue verification, and FP64 products for Newton."""

    def __init__(self, form: int, slices: int = 0, device: int = 0):
        import torch
        from . import pidcuda
        self.torch = torch
        self.pid = pidcuda
        self.form = form
        self.slices = slices
        self.dev = torch.device("cuda", device)
        self.name = {pidcuda.FORM_PLAIN: "plain", pidcuda.FORM_OZAKI: "ozaki"}.get(form, str(form))

    def to_dev(self, x: np.ndarray):
        return self.torch.from_numpy(np.ascontiguousarray(x)).to(self.dev)

    def to_host(self, x) -> np.ndarray:
        return x.cpu().numpy()

    def empty(self, ndoubles: int):
        return self.torch.empty(ndoubles, dtype=self.torch.float64, device=self.dev)

    def tensor(self, nb, ia, ib, nt, Ta, Tb, nqa, nqb, out, ld, s1=None, s2=None,
               transposed=False, accumulate=False, offset=0):
        from . import _lib
        torch = self.torch
        stream = torch.cuda.current_stream().cuda_stream
        _lib.call("vcpcu_tensor_basis_dev", nb, ia.data_ptr(), ib.data_ptr(), nt, Ta.data_ptr(),
                  Tb.data_ptr(), nqa, nqb, None if s1 is None else s1.data_ptr(),
                  None if s2 is None else s2.data_ptr(), out.data_ptr() + 8 * offset, ld,
                  int(transposed), int(accumulate), stream)

    def ints(self, x: np.ndarray):
        return self.torch.from_numpy(np.ascontiguousarray(x, dtype=np.int32)).to(self.dev)

    def igemm(self, m, n, k, A, lda, B, ldb, C, ldc, a_off=0, b_off=0, c_off=0):
        """C = A B (interval, kv layout, device buffers; offsets in doubles)."""
        self.pid.mulmm_dev(m, n, k, A[a_off:], lda, B[b_off:], ldb, C[c_off:], ldc, self.form,
                           self.slices)

    def sym_intersect(self, X, n: int):
        """In place: entries (i, j) and (j, i) of the n x n interval matrix X
        both enclose one value of a symmetric matrix; keep their
        intersection (symmetric, no wider than either)."""
        t = self.torch
        v = X.view(n, n, 2)
        lo = t.maximum(v[:, :, 0], v[:, :, 0].T)
        hi = t.minimum(v[:, :, 1], v[:, :, 1].T)
        v[:, :, 0] = lo
        v[:, :, 1] = hi

    def eig_enclose(self, A, B, n: int):
        """Verified eigenvalues of A x = lambda B x (device kv buffers):
        approximate eigenpairs of the midpoint problem by Cholesky reduction
        and a symmetric eigensolver on the GPU (the reference: LAPACK
        dsygv), then imats::eigsymge's verification on the device, Y the
        inverse of mid(B X), and the reference's overlap merge.  Returns
        (kv enclosures on the host, sup ||Y B X - I||, seconds of the
        approximation, seconds of the verification)."""
        t = self.torch
        from . import _lib
        t0 = time.perf_counter()
        Av, Bv = A.view(n, n, 2), B.view(n, n, 2)
        midA = 0.5 * (Av[:, :, 0] + Av[:, :, 1])   # symmetric: row- / column-major alike
        midB = 0.5 * (Bv[:, :, 0] + Bv[:, :, 1])
        Lc = t.linalg.cholesky(midB)
        Li = t.linalg.solve_triangular(Lc, t.eye(n, dtype=t.float64, device=self.dev),
                                       upper=False)
        lam, Vec = t.linalg.eigh(Li @ midA @ Li.T)
        Xr = Li.T @ Vec                                # columns: eigenvectors
        X = Xr.T.contiguous()                          # row-major (n, n) = column-major X
        lam = lam.contiguous()
        self.sync()
        t1 = time.perf_counter()
        s = t.cuda.current_stream().cuda_stream
        C = self.empty(2 * n * n)
        BX = self.empty(2 * n * n)
        midBX = self.empty(n * n)
        _lib.call("vcpcu_ieigsymge_stage1_dev", n, A.data_ptr(), n, B.data_ptr(), n,
                  X.data_ptr(), n, C.data_ptr(), BX.data_ptr(), midBX.data_ptr(), self.form,
                  self.slices, s)
        Y = t.linalg.inv(midBX.view(n, n).T).T.contiguous()   # column-major inverse
        enc = self.empty(2 * n)
        bound = self.empty(1)
        _lib.call("vcpcu_ieigsymge_stage2_dev", n, lam.data_ptr(), Y.data_ptr(), n,
                  C.data_ptr(), BX.data_ptr(), enc.data_ptr(), bound.data_ptr(), self.form,
                  self.slices, s)
        E = enc.cpu().numpy()
        g = float(bound.cpu().item())
        if not g < 1.0:
            from .errors import VerificationError
            raise VerificationError(f"eigenvalue verification failed: ||YBX - I|| <= {g}")
        _lib.call("vcpcu_eig_merge", n, E.ctypes.data)
        return E, g, t1 - t0, time.perf_counter() - t1

    def sync(self):
        self.torch.cuda.synchronize()

    # FP64 approximations (Newton)
    def newton_setup(self, Phi: np.ndarray, w2: np.ndarray, DL: np.ndarray):
        """Phi: n x P basis values at the points (row-major numpy), w2: the
        P weights, DL: the stiffness matrix (nearest doubles)."""
        t = self.torch
        self._Phi = t.from_numpy(Phi).to(self.dev)                # (n, P): col-major P x n
        self._PhiT = self._Phi.T.contiguous()                     # (P, n): col-major n x P
        self._w2 = t.from_numpy(w2).to(self.dev)
        self._DL = t.from_numpy(DL).to(self.dev)

    def newton_step(self, c: np.ndarray) -> np.ndarray:
        """delta = DF^-1 F at uh = c in FP64, the n x n x P product through
        this library's directed-rounding GEMM in round-to-nearest."""
        from . import vblas
        t = self.torch
        Phi, PhiT, w2, DL = self._Phi, self._PhiT, self._w2, self._DL
        n, P = Phi.shape
        cd = t.from_numpy(c).to(self.dev)
        u = cd @ Phi                                   # uh at the points
        A = (PhiT * (w2 * u)[:, None]).contiguous()    # col-major n x P: Phi diag(w u)
        G = t.empty((n, n), dtype=t.float64, device=self.dev)
        vblas.rmatmul_dev(n, P, n, A, n, Phi, P, G, n, 0)   # (Phi diag(w u)) Phi^T
        DF = DL - 2.0 * G.T
        F = DL @ cd - Phi @ (w2 * u * u)
        return t.linalg.solve(DF, F).cpu().numpy()


# ---------------------------------------------------------------- pipeline

@dataclass
class EmdenResult:
    M: int
    n: int
    form: str
    newton_iterations: int
    newton_last_step: float
    uh_max: float
    lambda_min: float
    lambda_max: float
    CN: float
    Cp: float
    Cs3: float
    K: float
    residual_L2: float
    residual_Hm1: float
    G: float
    kantorovich: float
    verified: bool
    error_bound_H10: float
    seconds: dict = field(default_factory=dict)
    sizes: dict = field(default_factory=dict)

    def as_dict(self) -> dict:
        return dict(self.__dict__)


def _pairs2(w_lo, w_hi):
    """2-D tensor weights w(qa) w(qb) as interval arrays (q = qa * N + qb)."""
    a = (np.repeat(w_lo, w_lo.size), np.repeat(w_hi, w_hi.size))
    b = (np.tile(w_lo, w_lo.size), np.tile(w_hi, w_hi.size))
    return V.mul(a, b)


def newton(M: int, prod, tol: float = 1e-13, max_iter: int = 40, tables=None):
    """Newton's method for the Galerkin system on the even list (FP64).
    Returns (coefficients, iterations, last |step|_inf)."""
    ia, ib = even_list(M)
    N = npts_inverse(M)
    T = tables or legendre.basis_tables(M, N)
    pm = T["phi_mid"]
    Phi = (pm[ia][:, :, None] * pm[ib][:, None, :]).reshape(ia.size, N * N)
    w2 = np.outer(T["w_mid"], T["w_mid"]).reshape(-1)
    _, _, DL = stiffness(M, ia, ib)
    prod.newton_setup(np.ascontiguousarray(Phi), w2, DL)
    c = np.full(ia.size, 200.0)
    c[0] = 600.0
    step = np.inf
    for it in range(1, max_iter + 1):
        d = prod.newton_step(c)
        c = c - d
        step = float(np.max(np.abs(d)))
        if step < tol * max(1.0, float(np.max(np.abs(c)))):
            return c, it, step
    return c, max_iter, step


def uh_max_bound(M: int, c: np.ndarray, prod, h_exp: int = 9) -> float:
    """Upper bound of max uh over [0, 1]^2 (uh is symmetric about 1/2 on the
    even list: [0, 1/2]^2 suffices, as test_Emden.cpp:154-161 takes): uh at
    the centres of cells of side h = 2^-h_exp enclosed by interval products,
    plus (h / 2)(Gx + Gy) with Gx = sum |c_ab| / (2 b + 3) >= sup |d uh / dx|
    (|phi_{a+2}'| <= 1, |phi_{b+2}| <= 1 / (2 b + 3) on [0, 1])."""
    ia, ib = even_list(M)
    mn = (M + 1) // 2
    h = 2.0 ** -h_exp
    g = 2 ** (h_exp - 1)
    centres = (np.arange(g) + 0.5) * h
    lo, hi = legendre.basis_at_points(M, centres, cache_key=f"grid_h{h_exp}")
    lo, hi = lo[0::2], hi[0::2]                      # the even basis functions, mn x g
    Cm = c.reshape(mn, mn)                           # C[i0, i1] = c[i0 * mn + i1]
    Ckv = table_kv(Cm, Cm)                           # mn x mn, column-major
    Vkv = table_kv(lo, hi)                           # mn x g
    Vt = table_kv(lo.T.copy(), hi.T.copy())          # g x mn
    dC, dV, dVt = prod.to_dev(Ckv), prod.to_dev(Vkv), prod.to_dev(Vt)
    # uh(x, y) = sum_{i0,i1} C[i0, i1] phi_{2 i0}(x) phi_{2 i1}(y) = (V^T C V)[x, y]
    T1 = prod.empty(2 * mn * g)
    prod.igemm(mn, g, mn, dC, mn, dV, mn, T1, mn)
    U = prod.empty(2 * g * g)
    prod.igemm(g, g, mn, dVt, g, T1, mn, U, g)
    Uh = prod.to_host(U)[1::2]
    absC = np.abs(Cm)
    wb = 1.0 / (2.0 * ib[: mn].astype(np.float64) + 3.0)   # 1 / (2 b + 3) for b = 0, 2, ...
    gx = V.sum_upper(V.up(absC * V.up(wb)[None, :]))
    gy = V.sum_upper(V.up(absC * V.up(wb)[:, None]))
    return float(V.up(float(np.max(Uh)) + V.up(V.up(h / 2) * V.up(gx + gy))))


def inverse_norm_matrices(M: int, c: np.ndarray, prod, tables=None):
    """(2 (uh phi_i, phi_j), DL) as kv buffers (n x n), the interval product
    Phi diag(w uh) Phi^T on the GPU.  Returns (A, B, seconds, sizes)."""
    ia, ib = even_list(M)
    nb = ia.size
    N = npts_inverse(M)
    P = N * N
    T = tables or legendre.basis_tables(M, N)
    t0 = time.perf_counter()
    Tphi = prod.to_dev(table_kv(T["phi_lo"], T["phi_hi"]))
    W2 = prod.to_dev(V.to_kv(_pairs2(T["w_lo"], T["w_hi"])))
    dia, dib = prod.ints(ia), prod.ints(ib)
    ckv = prod.to_dev(V.to_kv(V.point(c)))
    Phi = prod.empty(2 * nb * P)
    prod.tensor(nb, dia, dib, M, Tphi, Tphi, N, N, Phi, nb)
    uq = prod.empty(2 * P)
    prod.igemm(1, P, nb, ckv, 1, Phi, nb, uq, 1)                  # uh at the points
    prod.tensor(nb, dia, dib, M, Tphi, Tphi, N, N, Phi, nb, s1=W2, s2=uq)   # Phi diag(w uh)
    PhiT = prod.empty(2 * nb * P)
    prod.tensor(nb, dia, dib, M, Tphi, Tphi, N, N, PhiT, P, transposed=True)
    prod.sync()
    t1 = time.perf_counter()
    UPP = prod.empty(2 * nb * nb)
    prod.igemm(nb, nb, P, Phi, nb, PhiT, P, UPP, nb)              # the n x n x P product
    prod.sync()
    t2 = time.perf_counter()
    del Phi, PhiT
    prod.sym_intersect(UPP, nb)
    A = 2.0 * UPP                                                 # exact doubling
    lo, hi, _ = stiffness(M, ia, ib)
    B = prod.to_dev(table_kv(lo, hi))
    return A, B, {"basis_tables_to_factors": t1 - t0, "uhphiphi_product": t2 - t1}, \
        {"n": nb, "points": P, "uhphiphi_flops": 2.0 * nb * nb * P}


def residual_bound(M: int, c: np.ndarray, prod, tables=None) -> float:
    """Upper bound of ||Laplace(uh) + uh^2||_L2 (Gauss rule exact for the
    degree of the squared residual)."""
    ia, ib = even_list(M)
    nb = ia.size
    N = npts_residual(M)
    P = N * N
    T = tables or legendre.basis_tables(M, N)
    Tphi = prod.to_dev(table_kv(T["phi_lo"], T["phi_hi"]))
    Tdd = prod.to_dev(table_kv(T["dd_lo"], T["dd_hi"]))
    dia, dib = prod.ints(ia), prod.ints(ib)
    ckv = prod.to_dev(V.to_kv(V.point(c)))
    Bm = prod.empty(2 * nb * 2 * P)                  # [Phi | Laplace Phi], nb x 2P
    prod.tensor(nb, dia, dib, M, Tphi, Tphi, N, N, Bm, nb)
    off = 2 * nb * P
    prod.tensor(nb, dia, dib, M, Tdd, Tphi, N, N, Bm, nb, offset=off)
    prod.tensor(nb, dia, dib, M, Tphi, Tdd, N, N, Bm, nb, accumulate=True, offset=off)
    out = prod.empty(2 * 2 * P)
    prod.igemm(1, 2 * P, nb, ckv, 1, Bm, nb, out, 1)
    v = prod.to_host(out)
    u = (v[0:2 * P:2].copy(), v[1:2 * P:2].copy())
    lap = (v[2 * P::2].copy(), v[2 * P + 1::2].copy())
    r = V.add(lap, V.sqr(u))
    w2 = _pairs2(T["w_lo"], T["w_hi"])
    s = V.mul(w2, V.sqr(r))
    return float(V.up(np.sqrt(V.sum_upper(s[1]))))


def verify(M: int, prod, c: np.ndarray | None = None, newton_info=(0, 0.0)) -> EmdenResult:
    """The whole verification of test_Emden.cpp for order M (even list)."""
    iv = _iv()
    secs = {}
    t0 = time.perf_counter()
    if c is None:
        c, it, step = newton(M, prod)
    else:
        it, step = newton_info
    prod.sync()
    secs["newton"] = time.perf_counter() - t0
    N1, N2 = npts_inverse(M), npts_residual(M)
    t = time.perf_counter()
    T1 = legendre.basis_tables(M, N1)
    T2 = legendre.basis_tables(M, N2)
    secs["legendre_tables"] = time.perf_counter() - t
    t = time.perf_counter()
    umax = uh_max_bound(M, c, prod)
    secs["uh_max"] = time.perf_counter() - t
    t = time.perf_counter()
    A, B, s_inv, sizes = inverse_norm_matrices(M, c, prod, T1)
    secs.update(s_inv)
    n = sizes["n"]
    E, _, t_apx, t_ver = prod.eig_enclose(A, B, n)
    secs["eig_approximate"] = t_apx
    secs["eigsymge_verify"] = t_ver
    secs["inverse_norm_total"] = time.perf_counter() - t
    CN = ritz_constant(M)
    Cp = poincare_constant(2)
    Cs3 = sobolev_constant(3, 2)
    fduh = 2 * iv.mpf(umax)
    K = iv.mpf(0)
    for i in range(n):
        cc = _iv_of(E[2 * i], E[2 * i + 1])
        e = cc / (1 + CN ** 2 * fduh * cc)
        e = iv.mpf([e.a, cc.b])
        e = abs(e / (1 - e))
        if K.b < e.b:
            K = e
    if K.b < 1:
        K = iv.mpf(1)
    t = time.perf_counter()
    res = residual_bound(M, c, prod, T2)
    secs["residual"] = time.perf_counter() - t
    Res = Cp * iv.mpf(res)
    G = 2 * Cs3 ** 3
    alpha, omega = K * Res, K * G
    kc = alpha * omega
    ok = bool(kc.b <= 0.5)
    bound = (1 - iv.sqrt(1 - 2 * alpha * omega)) / omega if ok else iv.mpf([np.inf, np.inf])
    secs["total"] = time.perf_counter() - t0
    f = lambda x: float(x.b)  # noqa: E731  (upper ends)
    return EmdenResult(M=M, n=n, form=prod.name, newton_iterations=int(it),
                       newton_last_step=float(step), uh_max=umax,
                       lambda_min=float(np.min(E[0::2])), lambda_max=float(np.max(E[1::2])),
                       CN=f(CN), Cp=f(Cp), Cs3=f(Cs3), K=f(K), residual_L2=res,
                       residual_Hm1=f(Res), G=f(G), kantorovich=f(kc), verified=ok,
                       error_bound_H10=f(bound) if ok else float("inf"), seconds=secs,
                       sizes={**sizes, "points_residual": N2 * N2,
                              "points_per_dim": [N1, N2]})
