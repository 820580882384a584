// Translation unit for the reference's NEON CPU backend (aarch64 only).
#include "AC/Core/Internal/Processor/CPU/ARM/NEON.hpp"
#define BACKEND_NAME NEON
#define LAYER_SUFFIX neon
#include "AC/Core/Internal/Processor/CPU/Backend.hpp"
