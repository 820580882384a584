// ac::core::Image (include/AC/Core/Image.hpp), implemented from its contract
// (reference interface core/include/AC/Core/Image.hpp:359-419):
//
//   * an owned image keeps its pixels in one Storage block shared by every
//     copy and view of it; a mapped image points at caller memory and owns
//     nothing;
//   * the row stride of an allocation is the requested stride when that
//     holds a row, else the row size rounded up to a multiple of 4 bytes;
//     a mapping or a copy-in / copy-out uses the caller's stride when it
//     holds a row, else packed rows;
//   * requests with a non-positive size (or a null pointer where one is
//     needed) leave the image as it was.
#include "AC/Core/Image.hpp"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <new>

namespace ac::core {

// One heap block of pixels, 64-byte aligned (vector loads on the host, and
// copies to the device start on a cache line).
struct Image::Storage
{
    void* block;
    explicit Storage(std::size_t bytes)
    {
        const std::size_t rounded = std::max<std::size_t>(64, (bytes + 63) / 64 * 64);
        block = std::aligned_alloc(64, rounded);
        if (!block) throw std::bad_alloc();
    }
    ~Storage() { std::free(block); }
    Storage(const Storage&) = delete;
    Storage& operator=(const Storage&) = delete;
};

namespace {

// Bytes of one row, or 0 when the shape is not a positive size.
std::size_t row_bytes(int w, int c, Image::ElementType type)
{
    if (w <= 0 || c <= 0 || (type & 0xff) == 0) return 0;
    return static_cast<std::size_t>(w) * static_cast<std::size_t>(c) * static_cast<std::size_t>(type & 0xff);
}

// The caller's stride when it holds a row, else packed rows.
std::size_t caller_pitch(int stride, std::size_t row)
{
    return stride > 0 && static_cast<std::size_t>(stride) >= row ? static_cast<std::size_t>(stride) : row;
}

void copy_rows(std::uint8_t* dst, std::size_t dpitch, const std::uint8_t* src, std::size_t spitch, std::size_t row, int rows)
{
    if (dpitch == row && spitch == row)
    {
        std::memcpy(dst, src, row * static_cast<std::size_t>(rows));
        return;
    }
    for (int y = 0; y < rows; y++) std::memcpy(dst + y * dpitch, src + y * spitch, row);
}

}  // namespace

Image::Image() noexcept = default;
Image::Image(int w, int h, int c, ElementType elementType, int stride) { create(w, h, c, elementType, stride); }
Image::Image(int w, int h, int c, ElementType elementType, void* data, int stride)
{
    map(w, h, c, elementType, data, stride);
}
Image::Image(const Image&) noexcept = default;
Image::Image(Image&&) noexcept = default;
Image::~Image() noexcept = default;
Image& Image::operator=(const Image&) noexcept = default;
Image& Image::operator=(Image&&) noexcept = default;

void Image::create(int w, int h, int c, ElementType elementType, int stride)
{
    const std::size_t row = row_bytes(w, c, elementType);
    if (row == 0 || h <= 0) return;
    const std::size_t pitch = stride > 0 && static_cast<std::size_t>(stride) >= row ? static_cast<std::size_t>(stride)
                                                                                      : (row + 3) / 4 * 4;
    auto storage = std::make_shared<Storage>(pitch * static_cast<std::size_t>(h));
    w_ = w;
    h_ = h;
    c_ = c;
    type_ = elementType;
    stride_ = static_cast<int>(pitch);
    pixels_ = storage->block;
    storage_ = std::move(storage);
}

void Image::map(int w, int h, int c, ElementType elementType, void* data, int stride) noexcept
{
    const std::size_t row = row_bytes(w, c, elementType);
    if (row == 0 || h <= 0 || !data) return;
    w_ = w;
    h_ = h;
    c_ = c;
    type_ = elementType;
    stride_ = static_cast<int>(caller_pitch(stride, row));
    pixels_ = data;
    storage_.reset();
}

void Image::from(int w, int h, int c, ElementType elementType, const void* data, int stride)
{
    const std::size_t row = row_bytes(w, c, elementType);
    if (row == 0 || h <= 0 || !data) return;
    create(w, h, c, elementType);
    copy_rows(this->data(), static_cast<std::size_t>(stride_), static_cast<const std::uint8_t*>(data),
              caller_pitch(stride, row), row, h);
}

void Image::to(void* data, int stride) const noexcept
{
    const std::size_t row = row_bytes(w_, c_, type_);
    if (row == 0 || h_ <= 0 || !data || empty()) return;
    copy_rows(static_cast<std::uint8_t*>(data), caller_pitch(stride, row), this->data(), static_cast<std::size_t>(stride_),
              row, h_);
}

Image Image::view(int x, int y, int w, int h) const noexcept
{
    Image part;
    const int x0 = std::max(0, x), y0 = std::max(0, y);
    const int x1 = std::min(w_, x + w), y1 = std::min(h_, y + h);
    if (empty() || x1 <= x0 || y1 <= y0) return part;
    part.w_ = x1 - x0;
    part.h_ = y1 - y0;
    part.c_ = c_;
    part.type_ = type_;
    part.stride_ = stride_;
    part.pixels_ = pixel(x0, y0);
    part.storage_ = storage_;
    return part;
}

Image Image::clone() const
{
    Image copy;
    if (!empty()) copy.from(w_, h_, c_, type_, pixels_, stride_);
    return copy;
}

}  // namespace ac::core
