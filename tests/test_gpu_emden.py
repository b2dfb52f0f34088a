"""GPU tests of the Emden verification (test_PDE/test_Emden.cpp on the GPU).

* vcpcu_tensor_basis_dev (the two-dimensional Legendre basis at the Gauss
  points, phi_point_set / the uhphiphi element loop of vcp/ldbase.hpp) is
  bit-identical to the oracle's restatement for every flag combination, and
  a list index outside the table gives NaN entries instead of a read out of
  bounds;
* the interval matrix 2 (uh phi_i, phi_j) = 2 Phi diag(w uh) Phi^T of the
  M = 30 problem (entries (i, j) and (j, i) intersected): the plain form
  bit-identical to the CPU pipeline (oracle pidblas), the tensor-core form
  bit-identical to its host model;
* M = 30 end to end from one Newton solution: the plain and the tensor-core
  forms both close the Kantorovich check, the tensor-core bound is no
  looser than the plain one (tolerance 1e-9 relative: the two differ only
  in last bits of enclosures far below the residual) and both agree with the
  CPU pipeline's bound to 1e-6 relative.
"""
import numpy as np
import pytest

from vcp_gb300 import emden as E
from vcp_gb300 import ivnp

pytestmark = pytest.mark.gpu
pytest.importorskip("mpmath")


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


@pytest.mark.parametrize("flags", [dict(), dict(s1=True), dict(s1=True, s2=True),
                                   dict(transposed=True), dict(accumulate=True),
                                   dict(s1=True, transposed=True, accumulate=True)])
def test_tensor_basis_bitexact_oracle(cuda_lib, oracle, flags):
    import torch
    from vcp_gb300 import _lib
    rng = np.random.default_rng(len(flags) * 7 + 3 * int(flags.get("transposed", False)))
    nt, nqa, nqb, nb = 9, 13, 11, 37
    P = nqa * nqb
    def ivtab(r, c):
        m = rng.standard_normal((r, c))
        rad = np.abs(m) * 2.0 ** -45
        return E.table_kv(m - rad, m + rad)
    Ta, Tb = ivtab(nt, nqa), ivtab(nt, nqb)
    s1 = ivtab(1, P) if flags.get("s1") else None
    s2 = ivtab(1, P) if flags.get("s2") else None
    ia = rng.integers(0, nt, nb).astype(np.int32)
    ib = rng.integers(0, nt, nb).astype(np.int32)
    tr = bool(flags.get("transposed"))
    acc = bool(flags.get("accumulate"))
    ld = P + 3 if tr else nb + 5
    cols = nb if tr else P
    init = ivtab(ld, cols)
    ref = oracle.tensor_basis(nb, ia, ib, nt, Ta, Tb, nqa, nqb, init.copy(), ld, s1, s2, tr, acc)
    # keep every device copy alive until the kernel has run
    dev = {k: torch.from_numpy(v).cuda() for k, v in
           dict(ia=ia, ib=ib, Ta=Ta, Tb=Tb, s1=s1, s2=s2, out=init.copy()).items()
           if v is not None}
    ptr = lambda k: dev[k].data_ptr() if k in dev else None  # noqa: E731
    s = torch.cuda.current_stream().cuda_stream
    _lib.call("vcpcu_tensor_basis_dev", nb, ptr("ia"), ptr("ib"), nt, ptr("Ta"), ptr("Tb"), nqa,
              nqb, ptr("s1"), ptr("s2"), ptr("out"), ld, int(tr), int(acc), s)
    out = dev["out"]
    torch.cuda.synchronize()
    assert np.array_equal(bits(out.cpu().numpy()), bits(ref))


def test_tensor_basis_bad_index_gives_nan(cuda_lib):
    import torch
    from vcp_gb300 import _lib
    nt, nq = 3, 4
    T = torch.ones(2 * nt * nq, dtype=torch.float64, device="cuda")
    ia = torch.tensor([0, 3, -1], dtype=torch.int32, device="cuda")
    ib = torch.tensor([1, 1, 1], dtype=torch.int32, device="cuda")
    out = torch.zeros(2 * 3 * nq * nq, dtype=torch.float64, device="cuda")
    _lib.call("vcpcu_tensor_basis_dev", 3, ia.data_ptr(), ib.data_ptr(), nt, T.data_ptr(),
              T.data_ptr(), nq, nq, None, None, out.data_ptr(), 3, 0, 0,
              torch.cuda.current_stream().cuda_stream)
    o = out.cpu().numpy().reshape(nq * nq, 3, 2)
    assert np.all(o[:, 0, :] == 1.0)
    assert np.all(np.isnan(o[:, 1:, :]))


@pytest.fixture(scope="module")
def newton30():
    from oracle.emden_host import HostProducts
    c, it, step = E.newton(30, HostProducts())
    return c, it, step


def test_uhphiphi_plain_matches_cpu_and_ozaki_matches_model(cuda_lib, oracle, newton30):
    from oracle.emden_host import HostProducts
    from vcp_gb300 import pidcuda
    c = newton30[0]
    A_cpu, B_cpu, _, sz = E.inverse_norm_matrices(30, c, HostProducts())
    A_pl, B_pl, _, _ = E.inverse_norm_matrices(30, c, E.GpuProducts(pidcuda.FORM_PLAIN))
    A_pl, B_pl = A_pl.cpu().numpy(), B_pl.cpu().numpy()
    assert np.array_equal(bits(A_pl), bits(A_cpu))
    assert np.array_equal(bits(B_pl), bits(B_cpu))
    A_oz, _, _, _ = E.inverse_norm_matrices(30, c, E.GpuProducts(pidcuda.FORM_OZAKI))
    A_oz = A_oz.cpu().numpy()
    # the tensor-core product of the same factors, on the host model
    n, P = sz["n"], sz["points"]
    hp = HostProducts()
    from vcp_gb300 import legendre as L
    T = L.basis_tables(30, E.npts_inverse(30))
    ia, ib = E.even_list(30)
    Tphi = E.table_kv(T["phi_lo"], T["phi_hi"])
    W2 = ivnp.to_kv(E._pairs2(T["w_lo"], T["w_hi"]))
    Phi = np.empty(2 * n * P)
    N = E.npts_inverse(30)
    hp.tensor(n, ia, ib, 30, Tphi, Tphi, N, N, Phi, n)
    ckv = np.empty(2 * n)
    ckv[0::2] = c
    ckv[1::2] = c
    uq = np.empty(2 * P)
    g = E.GpuProducts(pidcuda.FORM_OZAKI)
    import torch
    duq = torch.empty(2 * P, dtype=torch.float64, device="cuda")
    g.igemm(1, P, n, torch.from_numpy(ckv).cuda(), 1, torch.from_numpy(Phi).cuda(), n, duq, 1)
    uq[:] = duq.cpu().numpy()
    hp.tensor(n, ia, ib, 30, Tphi, Tphi, N, N, Phi, n, s1=W2, s2=uq)
    PhiT = np.empty(2 * n * P)
    hp.tensor(n, ia, ib, 30, Tphi, Tphi, N, N, PhiT, P, transposed=True)
    ref, st = oracle.ozaki_igemm(n, n, P, Phi, PhiT, 8, 2, crt=True)
    assert st == 0
    hp.sym_intersect(ref, n)
    assert np.array_equal(bits(A_oz), bits(2.0 * ref))
    # both enclose the same matrix: the enclosures intersect
    assert np.all(A_oz[0::2] <= A_pl[1::2]) and np.all(A_pl[0::2] <= A_oz[1::2])


def test_emden_m30_end_to_end_plain_and_tensor_cores(cuda_lib, newton30):
    from oracle.emden_host import HostProducts
    from vcp_gb300 import pidcuda
    c, it, step = newton30
    r_cpu = E.verify(30, HostProducts(), c=c, newton_info=(it, step))
    r_pl = E.verify(30, E.GpuProducts(pidcuda.FORM_PLAIN), c=c, newton_info=(it, step))
    r_oz = E.verify(30, E.GpuProducts(pidcuda.FORM_OZAKI), c=c, newton_info=(it, step))
    for r in (r_cpu, r_pl, r_oz):
        assert r.verified and r.kantorovich <= 0.5
        assert r.error_bound_H10 < 1e-6
    assert r_oz.error_bound_H10 <= r_pl.error_bound_H10 * (1 + 1e-9)
    assert abs(r_pl.error_bound_H10 - r_cpu.error_bound_H10) <= 1e-6 * r_cpu.error_bound_H10
    # Newton on the GPU reaches the same solution
    g = E.GpuProducts(pidcuda.FORM_PLAIN)
    cg, _, _ = E.newton(30, g)
    assert np.max(np.abs(cg - c)) < 1e-9 * np.max(np.abs(c))
