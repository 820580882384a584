// Translation unit for the reference's Generic CPU backend, written the way
// cmake/GenCPUProcessorBackend.cmake generates it.
#include "AC/Core/Internal/Processor/CPU/Generic.hpp"
#define BACKEND_NAME Generic
#define LAYER_SUFFIX generic
#include "AC/Core/Internal/Processor/CPU/Backend.hpp"
