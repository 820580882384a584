// Replacement for the reference's stb_image_resize2-backed ac::core::resize
// (core/src/ImageResize.cpp:136-273; stb is not vendored).  Size and aliasing
// rules follow ImageResize.cpp:138-170 and :275-293; the sampling is this
// project's restatement (orc_resize in oracle/acoracle.c).
#include <thread>

#include "AC/Core/Image.hpp"

extern "C" int orc_resize_mt(const void* src, int w, int h, int c, int sstride, int type,
                             void* dst, int dw, int dh, int dstride, int mode, int threads);

namespace
{
    void resizeImpl(const ac::core::Image& src, ac::core::Image& dst, const double fx, const double fy, const int mode) noexcept
    {
        if (src.empty()) return;
        if (fx > 0.0 && fy > 0.0)
        {
            if (fx == 1.0 && fy == 1.0) { dst = src; return; }
            auto dstW = static_cast<int>(src.width() * fx);
            auto dstH = static_cast<int>(src.height() * fy);
            if ((dst.width() != dstW) || (dst.height() != dstH) || (dst.channels() != src.channels()) || (dst.type() != src.type()))
                dst.create(dstW, dstH, src.channels(), src.type());
        }
        else
        {
            if (dst.empty()) return;
            if (dst.width() == src.width() && dst.height() == src.height()) { dst = src; return; }
            if ((dst.channels() != src.channels()) || (dst.type() != src.type()))
                dst.create(dst.width(), dst.height(), src.channels(), src.type());
        }
        int m = (mode == ac::core::RESIZE_POINT) ? 0 : ((mode == ac::core::RESIZE_BILINEAR) ? 16 : 1);
        orc_resize_mt(src.ptr(), src.width(), src.height(), src.channels(), src.stride(), src.type(),
                      dst.ptr(), dst.width(), dst.height(), dst.stride(), m, static_cast<int>(std::thread::hardware_concurrency()));
    }
}

void ac::core::resize(const Image& src, Image& dst, const double fx, const double fy, const int mode) noexcept
{
    if (src == dst)
    {
        Image tmp{};
        resizeImpl(src, tmp, fx, fy, mode);
        if (!tmp.empty()) dst = tmp;
    }
    else resizeImpl(src, dst, fx, fy, mode);
}
ac::core::Image ac::core::resize(const Image& src, const double fx, const double fy, const int mode) noexcept
{
    if (fx <= 0.0 || fy <= 0.0) return src;
    Image dst{};
    resizeImpl(src, dst, fx, fy, mode);
    return dst;
}
