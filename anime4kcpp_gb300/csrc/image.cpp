#include "image.hpp"

#include <algorithm>
#include <cstdlib>
#include <cstring>

namespace acgb {

struct Image::Buffer
{
    void* data = nullptr;
    explicit Buffer(size_t size)
    {
        // 64-byte aligned rows start for vector loads/stores on the host side.
        size_t aligned = (size + 63) & ~static_cast<size_t>(63);
        data = std::aligned_alloc(64, aligned ? aligned : 64);
    }
    ~Buffer() { std::free(data); }
    Buffer(const Buffer&) = delete;
    Buffer& operator=(const Buffer&) = delete;
};

void Image::create(int w, int h, int c, ElementType type, int stride)
{
    int lineSize = w * c * (type & 0xff);
    if (!(h > 0 && lineSize > 0)) return;
    int pitch = (stride >= lineSize) ? stride : ((lineSize + 3) & ~3);
    auto buf = std::make_shared<Buffer>(static_cast<size_t>(h) * pitch);
    if (!buf->data) throw std::bad_alloc();
    w_ = w;
    h_ = h;
    c_ = c;
    type_ = type;
    pitch_ = pitch;
    buf_ = std::move(buf);
    pixels_ = buf_->data;
}

void Image::map(int w, int h, int c, ElementType type, void* data, int stride) noexcept
{
    int lineSize = w * c * (type & 0xff);
    if (!(h > 0 && lineSize > 0) || !data) return;
    w_ = w;
    h_ = h;
    c_ = c;
    type_ = type;
    pitch_ = (stride >= lineSize) ? stride : lineSize;
    buf_.reset();
    pixels_ = data;
}

void Image::from(int w, int h, int c, ElementType type, const void* data, int stride)
{
    int lineSize = w * c * (type & 0xff);
    if (!(h > 0 && lineSize > 0) || !data) return;
    int pitch = (stride >= lineSize) ? stride : lineSize;
    create(w, h, c, type);
    auto src = static_cast<const uint8_t*>(data);
    for (int i = 0; i < h; i++) std::memcpy(line(i), src + static_cast<size_t>(i) * pitch, lineSize);
}

void Image::to(void* data, int stride) const noexcept
{
    int lineSize = w_ * pixelSize();
    if (!(h_ > 0 && lineSize > 0) || !data) return;
    int pitch = (stride >= lineSize) ? stride : lineSize;
    auto dst = static_cast<uint8_t*>(data);
    for (int i = 0; i < h_; i++) std::memcpy(dst + static_cast<size_t>(i) * pitch, line(i), lineSize);
}

Image Image::view(int x, int y, int w, int h) const noexcept
{
    Image dst{};
    int ix = std::max(x, 0);
    int iy = std::max(y, 0);
    int iw = std::min(w_, x + w) - ix;
    int ih = std::min(h_, y + h) - iy;
    if (iw > 0 && ih > 0)
    {
        dst.w_ = iw;
        dst.h_ = ih;
        dst.c_ = c_;
        dst.type_ = type_;
        dst.pitch_ = pitch_;
        dst.pixels_ = line(iy) + static_cast<size_t>(ix) * pixelSize();
        dst.buf_ = buf_;
    }
    return dst;
}

Image Image::clone() const
{
    Image dst{};
    dst.from(w_, h_, c_, type_, pixels_, pitch_);
    return dst;
}

}  // namespace acgb
