// Internal view of the GB300 backend's processor: the public
// ac::core::Processor (reference interface core/include/AC/Core/
// Processor.hpp:15-48), the arithmetic forms, device-resident images and
// the output-shape rule of core/src/processor/Processor.cpp:199-276.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>

#include "AC/Core/Processor.hpp"
#include "image.hpp"
#include "kernels.hpp"
#include "models.hpp"

namespace acgb {

// Arithmetic form of the 8->8 convolutions.
enum class Precision : int
{
    FP32 = 0,  // plain FP32 on CUDA cores
    FP16 = 1,  // tcgen05 tensor cores, FP16 operands, FP32 accumulation
    BF16 = 2,  // tcgen05 tensor cores, BF16 operands, FP32 accumulation
};

// A device-resident image (pitched, interleaved channels).
struct DeviceImage
{
    void* ptr = nullptr;
    int w = 0, h = 0, c = 0, stride = 0, type = Image::UInt8;
};

// The backend's processor interface is the public ac::core::Processor
// (include/AC/Core/Processor.hpp).
using Processor = ac::core::Processor;
// Device list of a processor type (Processor::info<type>()).
const char* processor_info(int type);

// The GPU processor.  Exposed for the extension entry points.
class GB300Processor;

// Output size of process() with an empty dst (Processor.cpp:199-276).
void output_shape(int w, int h, int c, double factor, int& ow, int& oh);

}  // namespace acgb
