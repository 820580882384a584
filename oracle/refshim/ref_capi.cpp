// Flat C entry points over the reference's own ac::core::Processor, used only
// by the tests (golden-vector generation and oracle validation) and by the
// CPU-baseline leg of the benchmark.
#include <cstring>
#include <memory>

#include "AC/Core.hpp"

extern "C" {

// arch: 0 = reference auto-selection, 1 = Generic, other = reference ISA index.
// dst is preallocated by the caller with the output shape the reference produces.
int acref_process(const char* model, int arch,
                  const void* src, int w, int h, int c, int sstride, int type,
                  void* dst, int dw, int dh, int dstride, double factor)
{
    auto proc = ac::core::Processor::create("cpu", arch, model);
    if (!proc || !proc->ok()) return -256;
    ac::core::Image in{};
    in.map(w, h, c, type, const_cast<void*>(src), sstride);
    ac::core::Image out{};
    out.map(dw, dh, c, type, dst, dstride);
    proc->process(in, out, factor);
    return proc->ok() ? 0 : -256;
}

const char* acref_name(const char* model, int arch)
{
    static thread_local char buf[128];
    auto proc = ac::core::Processor::create("cpu", arch, model);
    std::strncpy(buf, proc->name(), sizeof(buf) - 1);
    buf[sizeof(buf) - 1] = 0;
    return buf;
}

int acref_rgb2yuv(const void* rgb, int w, int h, int c, int sstride, int type,
                  void* y, int ystride, void* uv, int uvstride)
{
    ac::core::Image in{}, yi{}, uvi{};
    in.map(w, h, c, type, const_cast<void*>(rgb), sstride);
    yi.map(w, h, 1, type, y, ystride);
    uvi.map(w, h, c == 4 ? 3 : 2, type, uv, uvstride);
    if (c == 4) ac::core::rgba2yuva(in, yi, uvi);
    else ac::core::rgb2yuv(in, yi, uvi);
    return 0;
}

int acref_yuv2rgb(const void* y, int ystride, const void* uv, int uvstride, int w, int h, int c, int type,
                  void* rgb, int dstride)
{
    ac::core::Image yi{}, uvi{}, out{};
    yi.map(w, h, 1, type, const_cast<void*>(y), ystride);
    uvi.map(w, h, c == 4 ? 3 : 2, type, const_cast<void*>(uv), uvstride);
    out.map(w, h, c, type, rgb, dstride);
    if (c == 4) ac::core::yuva2rgba(yi, uvi, out);
    else ac::core::yuv2rgb(yi, uvi, out);
    return 0;
}

}
