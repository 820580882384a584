// ISA detection without the reference's ruapu dependency (absent here).
#include "AC/Core/SIMD.hpp"

namespace ac::core::simd
{
#if defined(__x86_64__) || defined(__i386__)
    bool supportSSE() noexcept { return __builtin_cpu_supports("sse"); }
    bool supportSSE2() noexcept { return __builtin_cpu_supports("sse2"); }
    bool supportAVX() noexcept { return __builtin_cpu_supports("avx"); }
    bool supportAVX2() noexcept { return __builtin_cpu_supports("avx2"); }
    bool supportAVX512() noexcept { return __builtin_cpu_supports("avx512f"); }
    bool supportFMA() noexcept { return __builtin_cpu_supports("fma"); }
    bool supportNEON() noexcept { return false; }
#else
    bool supportSSE() noexcept { return false; }
    bool supportSSE2() noexcept { return false; }
    bool supportAVX() noexcept { return false; }
    bool supportAVX2() noexcept { return false; }
    bool supportAVX512() noexcept { return false; }
    bool supportFMA() noexcept { return false; }
#   if defined(__aarch64__)
    bool supportNEON() noexcept { return true; }
#   else
    bool supportNEON() noexcept { return false; }
#   endif
#endif
    bool supportRVV() noexcept { return false; }
    bool supportLSX() noexcept { return false; }
    bool supportLASX() noexcept { return false; }
    bool supportMSA() noexcept { return false; }
    bool supportAltiVec() noexcept { return false; }
    bool supportVSX() noexcept { return false; }
}
