// emden.cu -- tensor-product basis matrices of the Legendre generator.
//
// The reference forms the two-dimensional basis at the Gauss-Legendre
// points element by element (phi_point_set, vcp/ldbase.hpp:355-374:
// phi_point(i, j) = prod_d Legendre_with_GLpoint(list(i, d), Pointlist(j, d)))
// and then multiplies weights, uh^p and two basis values inside the O(n^2 P)
// element loop of uhphiphi (:994-1001).  Here that loop is a GEMM
// Phi diag(w uh^p) Phi^T on the interval product of this library, and this
// kernel writes its factors: entry (i, q) of the n x P matrix is
//
//   Ta(ia[i], qa) * Tb(ib[i], qb) [* s1(q)] [* s2(q)],   q = qa * nqb + qb
//
// (the reference's Pointlist order: first coordinate slowest), an interval
// product per factor with directed rounding (the endpoint products of kv's
// interval multiplication, rounded down / up, min / max), optionally added
// to the entry already there (a sum of two tensor products: the Laplacian
// basis phi_a'' phi_b + phi_a phi_b'').
#include "common.cuh"

namespace vcpcu {

namespace {

struct Iv {
  double lo, hi;
};

__device__ __forceinline__ Iv imul(Iv a, Iv b) {
  const double l0 = __dmul_rd(a.lo, b.lo), l1 = __dmul_rd(a.lo, b.hi);
  const double l2 = __dmul_rd(a.hi, b.lo), l3 = __dmul_rd(a.hi, b.hi);
  const double u0 = __dmul_ru(a.lo, b.lo), u1 = __dmul_ru(a.lo, b.hi);
  const double u2 = __dmul_ru(a.hi, b.lo), u3 = __dmul_ru(a.hi, b.hi);
  return Iv{fmin(fmin(l0, l1), fmin(l2, l3)), fmax(fmax(u0, u1), fmax(u2, u3))};
}

__device__ __forceinline__ Iv ld_iv(const double* p, long idx) {
  const double2 v = *reinterpret_cast<const double2*>(p + 2 * idx);
  return Iv{v.x, v.y};
}

// One thread per entry (grid-stride); `transposed` writes entry (i, q) at
// q + i * ld (P x n, column-major) instead of i + q * ld (n x P).
__global__ void __launch_bounds__(256)
tensor_basis_kernel(int nb, const int* __restrict__ ia, const int* __restrict__ ib, int nt,
                    const double* __restrict__ Ta, const double* __restrict__ Tb, int nqa,
                    int nqb, const double* __restrict__ s1, const double* __restrict__ s2,
                    double* __restrict__ out, long ld, int transposed, int accumulate) {
  const long P = (long)nqa * nqb;
  const long total = P * nb;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long i, q;
    if (transposed) {  // consecutive threads walk q: coalesced stores
      i = idx / P;
      q = idx - i * P;
    } else {           // consecutive threads walk i
      q = idx / nb;
      i = idx - q * nb;
    }
    const int qa = (int)(q / nqb), qb = (int)(q - (long)qa * nqb);
    const int a = ia[i], b = ib[i];
    double* o = out + 2 * (transposed ? q + i * ld : i + q * ld);
    if ((unsigned)a >= (unsigned)nt || (unsigned)b >= (unsigned)nt) {  // bad list entry
      const double nan = __longlong_as_double(0x7ff8000000000000LL);
      *reinterpret_cast<double2*>(o) = make_double2(nan, nan);
      continue;
    }
    Iv v = imul(ld_iv(Ta, a + (long)qa * nt), ld_iv(Tb, b + (long)qb * nt));
    if (s1) v = imul(v, ld_iv(s1, q));
    if (s2) v = imul(v, ld_iv(s2, q));
    if (accumulate) {
      const double2 c = *reinterpret_cast<const double2*>(o);
      v.lo = __dadd_rd(v.lo, c.x);
      v.hi = __dadd_ru(v.hi, c.y);
    }
    *reinterpret_cast<double2*>(o) = make_double2(v.lo, v.hi);
  }
}

}  // namespace

}  // namespace vcpcu

using namespace vcpcu;

extern "C" int vcpcu_tensor_basis_dev(int nb, const int* ia, const int* ib, int nt,
                                      const double* Ta, const double* Tb, int nqa, int nqb,
                                      const double* s1, const double* s2, double* out, long ld,
                                      int transposed, int accumulate, void* stream) {
  clear_error();
  if (nb < 0 || nt < 0 || nqa < 0 || nqb < 0) {
    set_error("tensor_basis: negative size (nb %d, nt %d, nqa %d, nqb %d)", nb, nt, nqa, nqb);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (nb == 0 || nqa == 0 || nqb == 0) return VCPCU_OK;
  if (!ia || !ib || !Ta || !Tb || !out) {
    set_error("tensor_basis: null pointer");
    return VCPCU_ERR_INVALID_ARG;
  }
  const long P = (long)nqa * nqb;
  if (ld < (transposed ? P : (long)nb)) {
    set_error("tensor_basis: leading dimension %ld below %ld", ld, transposed ? P : (long)nb);
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((((uintptr_t)Ta | (uintptr_t)Tb | (uintptr_t)out | (uintptr_t)s1 | (uintptr_t)s2) & 15) !=
      0) {
    set_error("tensor_basis: interval arrays must be 16-byte aligned");
    return VCPCU_ERR_INVALID_ARG;
  }
  int st = check_device();
  if (st) return st;
  const long total = P * nb;
  const long blocks = (total + 255) / 256;
  const int grid = (int)(blocks < 152L * 16 ? blocks : 152L * 16);
  tensor_basis_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
      nb, ia, ib, nt, Ta, Tb, nqa, nqb, s1, s2, out, ld, transposed, accumulate);
  VCPCU_LAUNCH_CHECK("tensor_basis_kernel");
  return VCPCU_OK;
}
