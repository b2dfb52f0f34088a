// kv/hwround.hpp -- project-written stand-in for the kv library's hwround
// (the kv library, github.com/mskashi/kv, is fetched unpinned from master by
// the reference's tools/download_vcp_kv.sh and is absent here).  Only the
// public names the VCP headers call are provided: the global rounding mode of
// the calling thread is switched with <cfenv>.  TEST INFRASTRUCTURE ONLY.
#ifndef KVSHIM_HWROUND_HPP
#define KVSHIM_HWROUND_HPP
#include <cfenv>

namespace kv {
struct hwround {
  static void roundup() { std::fesetround(FE_UPWARD); }
  static void rounddown() { std::fesetround(FE_DOWNWARD); }
  static void roundnear() { std::fesetround(FE_TONEAREST); }
  static void roundchop() { std::fesetround(FE_TOWARDZERO); }
};
}  // namespace kv
#endif
