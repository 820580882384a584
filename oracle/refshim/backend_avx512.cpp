// Translation unit for the reference's AVX-512 CPU backend (x86 only).
#include "AC/Core/Internal/Processor/CPU/X86/AVX512.hpp"
#define BACKEND_NAME X86SIMD512
#define LAYER_SUFFIX avx512
#include "AC/Core/Internal/Processor/CPU/Backend.hpp"
