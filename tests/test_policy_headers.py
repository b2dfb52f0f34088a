"""CPU tests of the C++ drop-in headers (include/vcp_cuda/): they compile
against the reference's own vcp/matrix.hpp (with the project's kv stand-in),
instantiate vcp::matrix<kv::interval<double>, vcp::pidcuda> with every hook
the imats algorithms use, link against libvcpcuda.so, and -- with no GPU in
this container -- report the library's "no device" status as vcp::state_error,
the exception pidblas raises for its failures.  (Running the headers on the
GPU needs the reference headers, which exist only here; the C ABI they call
is exercised on the GPU by the -m gpu tests.)"""
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
from oracle.build import reference_root

REF = reference_root()

PROGRAM = r'''
#include <cstdio>
#include <cstdlib>
#include <kv/interval.hpp>
#include <vcp/matrix.hpp>
#include <vcp_cuda/pidcuda.hpp>
#include <vcp_cuda/rmatmul_cuda.hpp>

// Fortran BLAS/LAPACK symbols pdblas references.  linearsolve forms R and
// mx on the host before its GPU call: these stubs give it some R and mx (an
// identity "inverse", a zero product); the rest are never reached.
extern "C" {
void dgemm_(char*, char*, int* m, int* n, int*, double*, const double*, int*, const double*,
            int*, double*, double* C, int*) {
  for (int i = 0; i < *m * *n; ++i) C[i] = 0.0;
}
double ddot_(int*, const double*, int*, const double*, int*) { std::abort(); }
void dgemv_(char*, int* m, int*, double*, const double*, int*, const double*, int*, double*,
            double* y, int*) {
  for (int i = 0; i < *m; ++i) y[i] = 0.0;
}
void dsyrk_(char*, char*, int*, int*, double*, const double*, int*, double*, double*, int*) {
  std::abort();
}
void dsymm_(char*, char*, int*, int*, double*, const double*, int*, const double*, int*,
            double*, double*, int*) { std::abort(); }
void dgetrf_(int*, int*, double*, int*, int*, int* info) { *info = 0; }
void dgetri_(int* n, double*, int*, int*, double* work, int* lwork, int* info) {
  if (*lwork == -1) work[0] = *n;
  *info = 0;
}
void dsyev_(char*, char*, int*, double*, int*, double*, double*, int*, int*) { std::abort(); }
void dgesv_(int*, int*, double*, int*, int*, double*, int*, int*) { std::abort(); }
void dsygv_(int*, char*, char*, int* n, double* A, int*, double*, int*, double* W, double* work,
            int* lwork, int* info) {  // W = diag(A), X = I
  *info = 0;
  if (*lwork == -1) {
    work[0] = 1;
    return;
  }
  for (int i = 0; i < *n; ++i)
    for (int j = 0; j < *n; ++j) {
      if (i == j) W[i] = A[i + *n * i];
      A[i + *n * j] = i == j ? 1.0 : 0.0;
    }
}
void dpotrf_(char*, int*, double*, int*, int*) { std::abort(); }
}

typedef kv::interval<double> I;
typedef vcp::matrix<I, vcp::pidcuda> M;
typedef vcp::matrix<I, vcp::pidcuda_fma> MF;

int main() {
  M A, B, C;
  A.zeros(4, 3);
  B.zeros(3, 5);
  for (int i = 0; i < 12; ++i) A.data()[i] = I(i - 1.0, i + 1.0);
  for (int i = 0; i < 15; ++i) B.data()[i] = I(2.0 * i, 2.0 * i + 0.5);
  int errors = 0;
  try {
    C = A * B;                            // pidcuda::mulmm -> vcpcu_igemm
    std::printf("NO_ERROR mulmm\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR mulmm: %s\n", e.what());
    ++errors;
  }
  try {
    C = ltransmul(A);                     // pidcuda::mulltmm -> vcpcu_isyrk
    std::printf("NO_ERROR mulltmm\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR mulltmm: %s\n", e.what());
    ++errors;
  }
  try {
    MF F, G, H;
    F.zeros(4, 3);
    G.zeros(3, 5);
    H = F * G;                            // pidcuda_fma::mulmm -> vcpcu_igemm_fma
    std::printf("NO_ERROR mulmm_fma\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR mulmm_fma: %s\n", e.what());
    ++errors;
  }
  try {
    M S, b1;
    S.zeros(3, 3);
    b1.zeros(3, 1);
    for (int i = 0; i < 3; ++i) S.data()[4 * i] = I(2.0, 2.5);
    M x = lss(S, b1);                     // pidcuda::linearsolve -> vcpcu_ilss_verify
    (void)x;
    std::printf("NO_ERROR lss\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR lss: %s\n", e.what());
    ++errors;
  }
  try {
    M S, T;
    S.zeros(3, 3);
    T.zeros(3, 3);
    for (int i = 0; i < 3; ++i) {
      S.data()[4 * i] = I(1.0 + i);
      T.data()[4 * i] = I(1.0);
    }
    M E;
    eigsymge(S, T, E);                    // pidcuda::eigsymge -> vcpcu_ieigsymge
    std::printf("NO_ERROR eigsymge\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR eigsymge: %s\n", e.what());
    ++errors;
  }
  std::fflush(stdout);
  double a[4] = {1, 2, 3, 4}, b[4] = {1, 0, 0, 1}, c[4];
  try {
    vcp_cuda::rmatmul(2, 2, 2, a, b, c, 1);
    std::printf("NO_ERROR rmatmul\n");
  } catch (std::runtime_error& e) {
    std::printf("RUNTIME_ERROR rmatmul: %s\n", e.what());
    ++errors;
  }
  return errors == 6 ? 0 : 1;
}
'''


def test_policy_headers_compile_link_and_map_errors(tmp_path, cuda_lib):
    if REF is None or not (REF / "vcp" / "matrix.hpp").exists():
        pytest.skip("reference headers not mounted")
    src = tmp_path / "use_pidcuda.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "use_pidcuda"
    cmd = ["g++", "-std=c++11", "-O1", f"-I{ROOT / 'oracle' / 'kvshim'}", f"-I{REF}",
           f"-I{ROOT / 'include'}", str(src), "-o", str(exe), f"-L{ROOT / 'vcp_gb300'}",
           "-lvcpcuda", f"-Wl,-rpath,{ROOT / 'vcp_gb300'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("compiled; the no-device error path is checked on CPU-only hosts")
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "STATE_ERROR mulmm" in run.stdout and "STATE_ERROR mulltmm" in run.stdout
    assert "STATE_ERROR mulmm_fma" in run.stdout
    assert "STATE_ERROR lss" in run.stdout
    assert "STATE_ERROR eigsymge" in run.stdout
    assert "RUNTIME_ERROR rmatmul" in run.stdout


PROGRAM_DD = r'''
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <kv/dd.hpp>
#include <vcp/matrix.hpp>
#include <vcp_cuda/pddcuda.hpp>

extern "C" {
void dgemm_(char*, char*, int*, int*, int*, double*, const double*, int*, const double*, int*,
            double*, double*, int*) { std::abort(); }
double ddot_(int*, const double*, int*, const double*, int*) { std::abort(); }
void dgemv_(char*, int*, int*, double*, const double*, int*, const double*, int*, double*,
            double*, int*) { std::abort(); }
void dsyrk_(char*, char*, int*, int*, double*, const double*, int*, double*, double*, int*) {
  std::abort();
}
void dsymm_(char*, char*, int*, int*, double*, const double*, int*, const double*, int*,
            double*, double*, int*) { std::abort(); }
// The LAPACK steps of the refinements run on the host before their first GPU
// product: these stubs let them through (identity factors).
void dgetrf_(int* m, int*, double*, int*, int* ipiv, int* info) {
  for (int i = 0; i < *m; ++i) ipiv[i] = i + 1;
  *info = 0;
}
void dgetrs_(char*, int*, int*, double*, int*, int*, double*, int*, int* info) { *info = 0; }
void dgetri_(int*, double*, int*, int*, double*, int*, int*) { std::abort(); }
void dsyev_(char*, char*, int* n, double* A, int*, double* W, double* work, int* lwork, int* info) {
  *info = 0;
  if (*lwork == -1) {
    work[0] = 1;
    return;
  }
  for (int i = 0; i < *n; ++i)
    for (int j = 0; j < *n; ++j) {
      if (i == j) W[i] = A[i + *n * i];
      A[i + *n * j] = i == j ? 1.0 : 0.0;
    }
}
void dgesv_(int*, int*, double*, int*, int*, double*, int*, int*) { std::abort(); }
void dsygv_(int*, char*, char*, int*, double*, int*, double*, int*, double*, double*, int*,
            int*) { std::abort(); }
void dpotrf_(char*, int*, double*, int*, int* info) { *info = 0; }
void dtrsm_(char*, char*, char*, char*, int*, int*, double*, double*, int*, double*, int*) {}
}

typedef vcp::matrix<kv::dd, vcp::pddcuda> M;

int main() {
  M A, B, C;
  A.zeros(4, 3);
  B.zeros(3, 5);
  for (int i = 0; i < 12; ++i) A.data()[i] = kv::dd(i - 1.0, std::ldexp(1.0, -60));
  for (int i = 0; i < 15; ++i) B.data()[i] = kv::dd(2.0 * i);
  int errors = 0;
  try {
    C = A * B;                            // pddcuda::mulmm -> vcpcu_ddgemm
    std::printf("NO_ERROR mulmm\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR mulmm: %s\n", e.what());
    ++errors;
  }
  try {
    C = ltransmul(A);                     // pddcuda::mulltmm -> vcpcu_ddgemm
    std::printf("NO_ERROR mulltmm\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR mulltmm: %s\n", e.what());
    ++errors;
  }
  M S, bv, x, E, V;
  S.zeros(3, 3);
  bv.zeros(3, 1);
  for (int i = 0; i < 3; ++i) S.data()[4 * i] = kv::dd(2.0 + i);
  bv.data()[0] = kv::dd(1.0);
  try {
    x = lss(S, bv);                       // pddcuda::linearsolve -> vcpcu_ddgemm residuals
    std::printf("NO_ERROR lss\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR lss: %s\n", e.what());
    ++errors;
  }
  try {
    M R = inv(S);                         // pddcuda::inv
    std::printf("NO_ERROR inv\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR inv: %s\n", e.what());
    ++errors;
  }
  try {
    E = Cholesky(S);                      // pddcuda::Cholesky
    std::printf("NO_ERROR Cholesky\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR Cholesky: %s\n", e.what());
    ++errors;
  }
  try {
    eigsym(S, E, V);                      // pddcuda::eigsym -> Ogita-Aishima on the GPU
    std::printf("NO_ERROR eigsym\n");
  } catch (vcp::state_error& e) {
    std::printf("STATE_ERROR eigsym: %s\n", e.what());
    ++errors;
  }
  M s, t;                                 // the scalar shortcut of pddblas stays on the host
  s.zeros(1, 1);
  s.data()[0] = kv::dd(3.0);
  t = s * A;
  if (t.data()[5].a1 != 12.0) ++errors;
  std::fflush(stdout);
  return errors == 6 ? 0 : 1;
}
'''


def test_pddcuda_header_compile_link_and_map_errors(tmp_path, cuda_lib):
    if REF is None or not (REF / "vcp" / "pddblas.hpp").exists():
        pytest.skip("reference headers not mounted")
    src = tmp_path / "use_pddcuda.cpp"
    src.write_text(PROGRAM_DD)
    exe = tmp_path / "use_pddcuda"
    cmd = ["g++", "-std=c++11", "-O1", f"-I{ROOT / 'oracle' / 'kvshim'}", f"-I{REF}",
           f"-I{ROOT / 'include'}", str(src), "-o", str(exe), f"-L{ROOT / 'vcp_gb300'}",
           "-lvcpcuda", f"-Wl,-rpath,{ROOT / 'vcp_gb300'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("compiled; the no-device error path is checked on CPU-only hosts")
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "STATE_ERROR mulmm" in run.stdout and "STATE_ERROR mulltmm" in run.stdout
    for what in ("lss", "inv", "Cholesky", "eigsym"):
        assert f"STATE_ERROR {what}" in run.stdout, run.stdout
