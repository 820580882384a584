/*
 * ac::core::Processor of the GB300 backend (libac_gb300.so), for C++
 * callers.
 *
 * The public interface is the reference's (core/include/AC/Core/
 * Processor.hpp:15-48): the factory create(type, device, model) never
 * returns null and reports failure through ok() / error(); process() has the
 * reference's factor semantics (core/src/processor/Processor.cpp:199-276)
 * and a non-empty dst is taken as preallocated with the output's shape (here
 * a dst of the wrong shape or type is an error, not an out-of-bounds write);
 * ok() / error() describe the calling thread's most recent call, and one
 * processor may be used from many threads at once.  The per-backend factory
 * hook create<type, Model>(device, model) is provided for type CUDA and
 * every model family of this backend.
 *
 * What differs by design: the whole path (RGB -> YUV split, the luma network
 * passes, chroma resize, YUV -> RGB merge) runs on one GPU inside the
 * processor, so the backend hook is processPath() for the whole call, where
 * the reference's backends implement one luma pass and leave the colour
 * work to the host.  There is no CPU fallback: type "cpu" or "opencl", or
 * "cuda" / "auto" without a usable GPU, gives a processor whose ok() is false
 * and whose error() says why.
 */
#ifndef AC_GB300_CXX_PROCESSOR_HPP
#define AC_GB300_CXX_PROCESSOR_HPP

#include <memory>

#include "AC/Core/Image.hpp"
#include "AC/Core/Model.hpp"

namespace ac::core
{
    class Processor;
}

class AC_GB300_CXX_API ac::core::Processor
{
public:
    static constexpr int CPU = 0;
    static constexpr int OpenCL = 1;
    static constexpr int CUDA = 2;

public:
    Processor() noexcept;
    virtual ~Processor();

    /* upscale src by factor into a new image */
    Image process(const Image& src, double factor);
    /* upscale into dst: an empty dst is allocated, a non-empty one must have
     * the output's size, channel count and element type */
    void process(const Image& src, Image& dst, double factor);

    /* the calling thread's most recent call succeeded / why it did not */
    virtual bool ok() noexcept;
    virtual const char* error() noexcept;
    virtual const char* name() const noexcept = 0;
    virtual int type() const noexcept = 0;
    virtual const char* typeName() const noexcept = 0;

public:
    /* type "cuda" / "auto" (any other string: a processor whose ok() is
     * false), device index (< 0: the GPU with the largest SM count x clock),
     * model string as the reference parses it (Processor.cpp:26-187) */
    static std::shared_ptr<Processor> create(const char* type, int device, const char* model);
    static const char* listInfo();

    template<int type, typename Model>
    static std::shared_ptr<Processor> create(int idx, const Model& model);
    template<int type>
    static const char* info();

protected:
    /* one whole process() call: shape checks, allocation of an empty dst,
     * the path on the GPU, per-thread error state */
    virtual void processPath(const Image& src, Image& dst, double factor) = 0;

protected:
    int idx = -1;
};

/* The factory hook of this backend: type CUDA, every model family. */
namespace ac::core
{
    template<> AC_GB300_CXX_API std::shared_ptr<Processor>
    Processor::create<Processor::CUDA, model::ACNetLegacy>(int idx, const model::ACNetLegacy& model);
    template<> AC_GB300_CXX_API std::shared_ptr<Processor>
    Processor::create<Processor::CUDA, model::ACNet<8>>(int idx, const model::ACNet<8>& model);
    template<> AC_GB300_CXX_API std::shared_ptr<Processor>
    Processor::create<Processor::CUDA, model::ARNet<8>>(int idx, const model::ARNet<8>& model);
    template<> AC_GB300_CXX_API std::shared_ptr<Processor>
    Processor::create<Processor::CUDA, model::ArtCNN<16>>(int idx, const model::ArtCNN<16>& model);
    template<> AC_GB300_CXX_API std::shared_ptr<Processor>
    Processor::create<Processor::CUDA, model::ArtCNN<32>>(int idx, const model::ArtCNN<32>& model);
    template<> AC_GB300_CXX_API std::shared_ptr<Processor>
    Processor::create<Processor::CUDA, model::FSRCNNX<8>>(int idx, const model::FSRCNNX<8>& model);
    template<> AC_GB300_CXX_API std::shared_ptr<Processor>
    Processor::create<Processor::CUDA, model::FSRCNNX<16>>(int idx, const model::FSRCNNX<16>& model);

    /* device list of a processor type ("not provided" for CPU / OpenCL) */
    template<> AC_GB300_CXX_API const char* Processor::info<Processor::CPU>();
    template<> AC_GB300_CXX_API const char* Processor::info<Processor::OpenCL>();
    template<> AC_GB300_CXX_API const char* Processor::info<Processor::CUDA>();
}

#endif
