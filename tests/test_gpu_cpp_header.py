"""The drop-in boundary from native code on the GPU.

* include/vcp_cuda/rmatmul_cuda.hpp -- the vblas drop-in, which needs no
  reference header -- compiled with g++ into a program that calls the
  unqualified vblas names (VCP_CUDA_VBLAS_NAMES): rmatmul in the three
  rounding modes and udmatmul are bit-identical to the oracle's sequential
  chains (vblas/rmatmul.hpp:102, vblas/udmatmul.hpp:758), and a rejected
  call (a null operand) throws std::runtime_error, the exception vblas
  throws when it cannot run (vblas/rmatmul.hpp:90-96);
* include/vcpcuda.h from a C program: vcpcu_igemm (host pointers) in the
  plain form is bit-identical to the pidblas::mulmm restatement
  (vcp/pidblas.hpp:239-294), in the tensor-core form to the host model, and
  a non-finite input makes the call return VCPCU_ERR_NONFINITE.

The policy classes of vcp_cuda/pidcuda.hpp and pddcuda.hpp sit on the
reference's own vcp::matrix headers, which exist only where the reference
tree does; they are compiled, linked and run there by test_policy_headers.py.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from vcp_gb300 import workloads as W

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent

CPP = r"""
#define VCP_CUDA_VBLAS_NAMES
#include <vcp_cuda/rmatmul_cuda.hpp>

#include <cstdio>
#include <stdexcept>
#include <vector>

int main(int argc, char** argv) {
  int m, n, k;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f || std::fread(&m, sizeof(int), 1, f) != 1 || std::fread(&n, sizeof(int), 1, f) != 1 ||
      std::fread(&k, sizeof(int), 1, f) != 1)
    return 2;
  std::vector<double> A((size_t)m * n), B((size_t)n * k);
  if (std::fread(A.data(), sizeof(double), A.size(), f) != A.size() ||
      std::fread(B.data(), sizeof(double), B.size(), f) != B.size())
    return 2;
  std::fclose(f);
  std::vector<double> out;
  for (int rnd : {1, -1, 0}) {
    std::vector<double> C((size_t)m * k);
    rmatmul(m, n, k, A.data(), B.data(), C.data(), rnd);
    out.insert(out.end(), C.begin(), C.end());
  }
  std::vector<double> CU((size_t)m * k), CD((size_t)m * k);
  udmatmul(m, n, k, A.data(), B.data(), CU.data(), CD.data());
  out.insert(out.end(), CU.begin(), CU.end());
  out.insert(out.end(), CD.begin(), CD.end());
  f = std::fopen(argv[2], "wb");
  if (!f || std::fwrite(out.data(), sizeof(double), out.size(), f) != out.size()) return 3;
  std::fclose(f);
  try {
    rmatmul(m, n, k, nullptr, B.data(), CU.data(), 1);  // rejected: null A
    std::printf("no exception\n");
  } catch (const std::runtime_error& e) {
    std::printf("runtime_error: %s\n", e.what());
  }
  return 0;
}
"""

C_SRC = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include "vcpcuda.h"

int main(int argc, char** argv) {
  int m, n, k;
  FILE* f = fopen(argv[1], "rb");
  if (!f || fread(&m, sizeof(int), 1, f) != 1 || fread(&n, sizeof(int), 1, f) != 1 ||
      fread(&k, sizeof(int), 1, f) != 1)
    return 2;
  size_t na = 2 * (size_t)m * k, nb = 2 * (size_t)k * n, nc = 2 * (size_t)m * n;
  double* A = malloc(na * sizeof(double));
  double* B = malloc(nb * sizeof(double));
  double* C = malloc(2 * nc * sizeof(double));
  if (fread(A, sizeof(double), na, f) != na || fread(B, sizeof(double), nb, f) != nb) return 2;
  fclose(f);
  int st = vcpcu_igemm(m, n, k, A, B, C, VCPCU_FORM_PLAIN, 0);
  if (st) { printf("plain: %d %s\n", st, vcpcu_last_error_string()); return 4; }
  st = vcpcu_igemm(m, n, k, A, B, C + nc, VCPCU_FORM_OZAKI, 0);
  if (st) { printf("ozaki: %d %s\n", st, vcpcu_last_error_string()); return 4; }
  f = fopen(argv[2], "wb");
  if (!f || fwrite(C, sizeof(double), 2 * nc, f) != 2 * nc) return 3;
  fclose(f);
  A[0] = NAN;  /* a NaN endpoint: the product reports it */
  st = vcpcu_igemm(m, n, k, A, B, C, VCPCU_FORM_OZAKI, 0);
  printf("nonfinite: %d %d\n", st, st == VCPCU_ERR_NONFINITE);
  free(A); free(B); free(C);
  return 0;
}
"""


def _compile(tmp_path, name, src, compiler, flags):
    exe = tmp_path / name
    srcf = tmp_path / (name + (".cpp" if compiler == "g++" else ".c"))
    srcf.write_text(src)
    lib = ROOT / "vcp_gb300"
    cmd = [compiler, *flags, "-O2", f"-I{ROOT / 'include'}", str(srcf), f"-L{lib}", "-lvcpcuda",
           f"-Wl,-rpath,{lib}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def _inputs(path, m, n, k, *arrays):
    with open(path, "wb") as f:
        np.array([m, n, k], dtype=np.int32).tofile(f)
        for a in arrays:
            np.ascontiguousarray(a, dtype=np.float64).tofile(f)


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
@pytest.mark.parametrize("shape", [(70, 90, 33), (129, 16, 200), (1, 300, 1)])
def test_rmatmul_header_from_cpp(cuda_lib, oracle, tmp_path, shape):
    m, n, k = shape
    exe = _compile(tmp_path, "vblas_dropin", CPP, "g++", ["-std=c++17"])
    rng = np.random.default_rng(m + n + k)
    A, B = W.ephi(rng, m * n, 8), W.ephi(rng, n * k, 8)
    _inputs(tmp_path / "in.bin", m, n, k, A, B)
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "runtime_error: vcpcu_rmatmul" in r.stdout
    out = np.fromfile(tmp_path / "out.bin", dtype=np.float64).reshape(5, m * k)
    for i, rnd in enumerate((1, -1, 0)):
        assert np.array_equal(bits(out[i]), bits(oracle.rmatmul(m, n, k, A, B, rnd))), rnd
    assert np.array_equal(bits(out[3]), bits(oracle.rmatmul(m, n, k, A, B, 1)))
    assert np.array_equal(bits(out[4]), bits(oracle.rmatmul(m, n, k, A, B, -1)))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no gcc")
def test_c_abi_from_c_program(cuda_lib, oracle, tmp_path):
    m, n, k = 150, 97, 333
    exe = _compile(tmp_path, "capi_user", C_SRC, "gcc", ["-std=c11"])
    rng = np.random.default_rng(5)
    A = W.interval_ephi(rng, m, k, 4, 2.0 ** -40)
    B = W.interval_ephi(rng, k, n, 4, 2.0 ** -40)
    _inputs(tmp_path / "in.bin", m, n, k, A, B)
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "nonfinite:" in r.stdout and r.stdout.strip().endswith(" 1"), r.stdout
    out = np.fromfile(tmp_path / "out.bin", dtype=np.float64).reshape(2, 2 * m * n)
    assert np.array_equal(bits(out[0]), bits(oracle.pidblas_mulmm(m, n, k, A, B)))
    ref, st = oracle.ozaki_igemm(m, n, k, A, B, 8, 2, crt=True)
    assert st == 0
    assert np.array_equal(bits(out[1]), bits(ref))
