// kv/rdouble.hpp -- project-written stand-in for kv's directed-rounding
// double header (the kv library is absent here).  vcp/pidblas_fma.hpp
// includes it but uses none of its names; the directed operations the shim
// interval needs live in kv/interval.hpp and kv/hwround.hpp.  TEST
// INFRASTRUCTURE ONLY.
#ifndef RDOUBLE_HPP
#define RDOUBLE_HPP
#include <kv/hwround.hpp>
#endif  // RDOUBLE_HPP
