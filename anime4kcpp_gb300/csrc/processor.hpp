// Processor interface of the GB300 backend, mirroring the reference's
// ac::core::Processor (core/include/AC/Core/Processor.hpp:15-48): create()
// never returns null and reports failure through ok()/error(); process()
// follows core/src/processor/Processor.cpp:199-276; ok()/error() describe
// the calling thread's most recent call.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>

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

class Processor
{
public:
    static constexpr int CPU = 0;
    static constexpr int OpenCL = 1;
    static constexpr int CUDA = 2;

    virtual ~Processor() = default;

    Image process(const Image& src, double factor);
    // A non-empty dst is taken as preallocated with the shape the reference
    // would produce (Processor.hpp:27-29).
    void process(const Image& src, Image& dst, double factor);

    virtual bool ok() noexcept = 0;
    virtual const char* error() noexcept = 0;
    virtual const char* name() const noexcept = 0;
    virtual int type() const noexcept { return CUDA; }
    virtual const char* typeName() const noexcept { return "CUDA"; }

    static std::shared_ptr<Processor> create(const char* type, int device, const char* model);
    static const char* listInfo();
    static const char* info(int type);

protected:
    virtual void processHost(const Image& src, Image& dst, double factor) = 0;
};

// The GPU processor.  Exposed for the extension entry points.
class GB300Processor;

// Output size of process() with an empty dst (Processor.cpp:199-276).
void output_shape(int w, int h, int c, double factor, int& ow, int& oh);

}  // namespace acgb
