// Shim for the reference's optional half_float dependency (absent here).
// Float16 images are not reachable through the C ABI; the compiler's own
// _Float16 is enough for the reference's Float16 template instantiations to build.
#ifndef AC_HALF_SHIM_HPP
#define AC_HALF_SHIM_HPP
namespace half_float { using half = _Float16; }
#endif
