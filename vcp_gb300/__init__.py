"""vcp_gb300 -- verified dense matrix products of VCP (koutasekine/vcp) on GB300.

The compute path is libvcpcuda.so (hand-written sm_103a CUDA behind the C ABI
of include/vcpcuda.h); this package is its Python host side:

* ``vblas``   -- rmatmul / udmatmul with the vblas signatures (directed-rounding
                 FP64 GEMM);
* ``pidcuda`` -- interval GEMM with pidblas semantics (plain FP64 form and the
                 Ozaki tensor-core form);
* ``vcpmat``  -- portable matrix files (.vcpmat) to and from host or device memory;
* ``build``   -- in-tree nvcc build of the library.
"""
from . import errors  # noqa: F401

__all__ = ["errors", "vblas", "pidcuda", "vcpmat", "build"]
