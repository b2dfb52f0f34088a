"""The Emden verification pipeline on the CPU (test infrastructure and the
timed CPU baseline of the Emden workload).

TEST INFRASTRUCTURE ONLY: the same pipeline as vcp_gb300.emden with every
product on the host -- the oracle's restatements of pidblas::mulmm
(vcp/pidblas.hpp:239-294), of imats::eigsymge's verification
(vcp/imats.hpp:419-522) and of the tensor-basis kernel -- and Newton's
method with numpy / LAPACK in FP64.  It is what test_Emden.cpp computes on
the CPU with its pidblas policy, with the products in the restated form.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O


class HostProducts:
    name = "cpu"

    def __init__(self, threads: int = 0):
        self.threads = threads

    def to_dev(self, x):
        return np.ascontiguousarray(x, dtype=np.float64).copy()

    def to_host(self, x):
        return x

    def empty(self, ndoubles):
        return np.empty(int(ndoubles))

    def ints(self, x):
        return np.ascontiguousarray(x, dtype=np.int32)

    def sync(self):
        pass

    def tensor(self, nb, ia, ib, nt, Ta, Tb, nqa, nqb, out, ld, s1=None, s2=None,
               transposed=False, accumulate=False, offset=0):
        O.tensor_basis(nb, ia, ib, nt, Ta, Tb, nqa, nqb, out, ld, s1, s2, transposed,
                       accumulate, offset, self.threads)

    def igemm(self, m, n, k, A, lda, B, ldb, C, ldc, a_off=0, b_off=0, c_off=0):
        assert lda == m and ldb == k and ldc == m
        Cm = O.pidblas_mulmm(m, n, k, np.ascontiguousarray(A[a_off:a_off + 2 * m * k]),
                             np.ascontiguousarray(B[b_off:b_off + 2 * k * n]), self.threads)
        C[c_off:c_off + 2 * m * n] = Cm

    def sym_intersect(self, X, n):
        v = X.reshape(n, n, 2)
        lo = np.maximum(v[:, :, 0], v[:, :, 0].T)
        hi = np.minimum(v[:, :, 1], v[:, :, 1].T)
        v[:, :, 0] = lo
        v[:, :, 1] = hi

    def eig_enclose(self, A, B, n):
        import time
        import scipy.linalg
        t0 = time.perf_counter()
        midA = (0.5 * (A[0::2] + A[1::2])).reshape(n, n, order="F")
        midB = (0.5 * (B[0::2] + B[1::2])).reshape(n, n, order="F")
        lam, Xm = scipy.linalg.eigh(midA, midB)
        Y = np.linalg.inv(midB @ Xm)
        t1 = time.perf_counter()
        st, out, g = O.ieigsymge(n, A, B, np.asfortranarray(Xm).ravel(order="F"), lam,
                                 np.asfortranarray(Y).ravel(order="F"), threads=self.threads)
        if st != 0:
            raise RuntimeError(f"eigenvalue verification failed (||YBX - I|| bound {g})")
        return out, g, t1 - t0, time.perf_counter() - t1

    def newton_setup(self, Phi, w2, DL):
        self._Phi, self._w2, self._DL = Phi, w2, DL

    def newton_step(self, c):
        Phi, w2, DL = self._Phi, self._w2, self._DL
        u = c @ Phi
        G = (Phi * (w2 * u)) @ Phi.T
        DF = DL - 2.0 * G
        F = DL @ c - Phi @ (w2 * u * u)
        return np.linalg.solve(DF, F)
