// Host image container with the semantics of the reference's ac::core::Image
// (core/include/AC/Core/Image.hpp:359-419, core/src/Image.cpp):
// width/height/channels/element type/row stride in bytes, pixels either owned
// through a shared buffer (copies share it) or mapped from caller memory.
#pragma once

#include <cstdint>
#include <memory>

namespace acgb {

class Image
{
public:
    using ElementType = int;
    static constexpr ElementType UInt8 = 0 << 8 | 1;
    static constexpr ElementType UInt16 = 0 << 8 | 2;
    static constexpr ElementType Float16 = 2 << 8 | 2;
    static constexpr ElementType Float32 = 2 << 8 | 4;

    Image() noexcept = default;
    Image(int w, int h, int c, ElementType type, int stride = 0) { create(w, h, c, type, stride); }

    // Image.cpp:40-53: stride = max(stride, line size rounded up to 4 bytes).
    void create(int w, int h, int c, ElementType type, int stride = 0);
    // Image.cpp:54-66: wrap caller memory, no ownership.
    void map(int w, int h, int c, ElementType type, void* data, int stride = 0) noexcept;
    // Image.cpp:67-76: allocate and copy rows from data (rows `stride` apart).
    void from(int w, int h, int c, ElementType type, const void* data, int stride = 0);
    // Image.cpp:77-84: copy rows out.
    void to(void* data, int stride = 0) const noexcept;
    // Image.cpp:85-106: intersection with the image, sharing pixels.
    Image view(int x, int y, int w, int h) const noexcept;
    Image clone() const;

    int width() const noexcept { return w_; }
    int height() const noexcept { return h_; }
    int channels() const noexcept { return c_; }
    int stride() const noexcept { return pitch_; }
    int size() const noexcept { return h_ * pitch_; }
    int elementSize() const noexcept { return type_ & 0xff; }
    int pixelSize() const noexcept { return c_ * elementSize(); }
    ElementType type() const noexcept { return type_; }
    uint8_t* data() const noexcept { return static_cast<uint8_t*>(pixels_); }
    uint8_t* line(int y) const noexcept { return data() + static_cast<size_t>(y) * pitch_; }
    void* ptr() const noexcept { return pixels_; }
    bool empty() const noexcept { return pixels_ == nullptr; }
    bool ownership() const noexcept { return buf_ != nullptr; }
    bool operator==(const Image& o) const noexcept
    {
        return (ownership() && o.ownership()) ? (buf_ == o.buf_) : (pixels_ == o.pixels_);
    }
    bool operator!=(const Image& o) const noexcept { return !operator==(o); }

private:
    struct Buffer;
    int w_ = 0, h_ = 0, c_ = 0;
    ElementType type_ = UInt8;
    int pitch_ = 0;
    void* pixels_ = nullptr;
    std::shared_ptr<Buffer> buf_;
};

}  // namespace acgb
