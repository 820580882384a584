// Shim for building the reference CPU processor outside its CMake build:
// CMake normally generates this export header; a static build needs no
// visibility attributes.
#ifndef AC_CORE_EXPORT_SHIM_HPP
#define AC_CORE_EXPORT_SHIM_HPP
#define AC_CORE_EXPORT
#endif
