/*
 * ac::core::Image and the image operations of the upscaling path, for C++
 * callers of the GB300 backend (libac_gb300.so).
 *
 * The public interface is the reference's (core/include/AC/Core/Image.hpp:
 * Image at :359-419, the colour conversions at :21-137, resize at :271-319):
 * the same names, element-type encoding ((kind << 8) | bytes), row-stride
 * rule and sharing semantics, so C++ code written against the reference's
 * core compiles against this header and links with this library.  The
 * member layout is this library's own: code must be recompiled against this
 * header, not mixed with objects built against the reference's.
 *
 * Semantics (core/src/Image.cpp): create() allocates an owned buffer whose
 * row stride is the requested stride when it holds a row, else the row size
 * rounded up to 4 bytes; map() wraps caller memory without ownership;
 * copies of an Image share its pixels; view() is a rectangle sharing the
 * pixels; clone() is a deep copy.  Image file I/O (imread / imwrite) is not
 * part of this backend (the reference's AC_CORE_DISABLE_IMAGE_IO build).
 */
#ifndef AC_GB300_CXX_IMAGE_HPP
#define AC_GB300_CXX_IMAGE_HPP

#include <cstdint>
#include <memory>

#ifndef AC_GB300_CXX_API
#define AC_GB300_CXX_API __attribute__((visibility("default")))
#endif

namespace ac::core
{
    class Image;

    /* Colour conversions (core/src/ImageProcess.cpp:39-61, :114-138,
     * :192-215, :276-308) between packed images of one element type, run on
     * the GPU: 3-channel RGB <-> YUV, 4-channel RGBA <-> YUVA (alpha
     * premultiplied into the chroma).  An empty dst is allocated. */
    AC_GB300_CXX_API void rgb2yuv(const Image& rgb, Image& yuv);
    AC_GB300_CXX_API void rgba2yuva(const Image& rgba, Image& yuva);
    AC_GB300_CXX_API void yuv2rgb(const Image& yuv, Image& rgb);
    AC_GB300_CXX_API void yuva2rgba(const Image& yuva, Image& rgba);

    /* Interpolation modes; the enumerator values are the reference's
     * (Image.hpp:271-289).  This backend implements RESIZE_POINT,
     * RESIZE_CATMULL_ROM and RESIZE_BILINEAR; other modes leave dst
     * unchanged. */
    enum ResizeModes
    {
        RESIZE_POINT = 0,
        RESIZE_CATMULL_ROM,
        RESIZE_MITCHELL_NETRAVALI,
        RESIZE_BICUBIC_0_60,
        RESIZE_BICUBIC_0_75,
        RESIZE_BICUBIC_0_100,
        RESIZE_BICUBIC_20_50,
        RESIZE_SOFTCUBIC50,
        RESIZE_SOFTCUBIC75,
        RESIZE_SOFTCUBIC100,
        RESIZE_LANCZOS2,
        RESIZE_LANCZOS3,
        RESIZE_LANCZOS4,
        RESIZE_SPLINE16,
        RESIZE_SPLINE36,
        RESIZE_SPLINE64,
        RESIZE_BILINEAR,
    };

    /* resize (core/src/ImageResize.cpp:136-170, :275-293): with fx and fy
     * > 0 the output is (w * fx) x (h * fy), else dst's own size; a size
     * equal to src's makes dst share src.  src and dst may be one image. */
    AC_GB300_CXX_API void resize(const Image& src, Image& dst, double fx, double fy, int mode = RESIZE_CATMULL_ROM) noexcept;
    AC_GB300_CXX_API Image resize(const Image& src, double fx, double fy, int mode = RESIZE_CATMULL_ROM) noexcept;
}

class ac::core::Image
{
public:
    /* (kind << 8) | bytes per element, kind 0 unsigned, 1 signed, 2 float. */
    using ElementType = int;
    static constexpr ElementType UInt8 = 0 << 8 | 1;
    static constexpr ElementType UInt16 = 0 << 8 | 2;
    static constexpr ElementType Float16 = 2 << 8 | 2;
    static constexpr ElementType Float32 = 2 << 8 | 4;

public:
    AC_GB300_CXX_API Image() noexcept;
    AC_GB300_CXX_API Image(int w, int h, int c, ElementType elementType, int stride = 0);
    AC_GB300_CXX_API Image(int w, int h, int c, ElementType elementType, void* data, int stride = 0);
    AC_GB300_CXX_API Image(const Image&) noexcept;
    AC_GB300_CXX_API Image(Image&&) noexcept;
    AC_GB300_CXX_API ~Image() noexcept;
    AC_GB300_CXX_API Image& operator=(const Image&) noexcept;
    AC_GB300_CXX_API Image& operator=(Image&&) noexcept;

    /* Each of these leaves the image unchanged when w, h or c is not
     * positive (and map / from when data is null). */
    AC_GB300_CXX_API void create(int w, int h, int c, ElementType elementType, int stride = 0);
    AC_GB300_CXX_API void map(int w, int h, int c, ElementType elementType, void* data, int stride = 0) noexcept;
    /* create() with the default stride, then copy the rows of `data`
     * (`stride` bytes apart, or packed when stride is smaller than a row). */
    AC_GB300_CXX_API void from(int w, int h, int c, ElementType elementType, const void* data, int stride = 0);
    /* copy the rows out to `data` (`stride` bytes apart, or packed). */
    AC_GB300_CXX_API void to(void* data, int stride = 0) const noexcept;
    /* the part of the rectangle inside the image, sharing the pixels; empty
     * when they do not intersect. */
    AC_GB300_CXX_API Image view(int x, int y, int w, int h) const noexcept;
    AC_GB300_CXX_API Image clone() const;

public:
    int width() const noexcept { return w_; }
    int height() const noexcept { return h_; }
    int channels() const noexcept { return c_; }
    int stride() const noexcept { return stride_; }
    int size() const noexcept { return h_ * stride_; }
    int elementSize() const noexcept { return type_ & 0xff; }
    int pixelSize() const noexcept { return c_ * elementSize(); }
    ElementType type() const noexcept { return type_; }
    std::uint8_t* data() const noexcept { return static_cast<std::uint8_t*>(pixels_); }
    std::uint8_t* line(const int y) const noexcept { return data() + static_cast<std::ptrdiff_t>(y) * stride_; }
    std::uint8_t* pixel(const int x, const int y) const noexcept { return line(y) + static_cast<std::ptrdiff_t>(x) * pixelSize(); }
    void* ptr() const noexcept { return pixels_; }
    void* ptr(const int y) const noexcept { return line(y); }
    void* ptr(const int x, const int y) const noexcept { return pixel(x, y); }
    bool empty() const noexcept { return pixels_ == nullptr; }
    bool isUint() const noexcept { return (type_ >> 8) == 0; }
    bool isInt() const noexcept { return (type_ >> 8) == 1; }
    bool isFloat() const noexcept { return (type_ >> 8) == 2; }
    bool ownership() const noexcept { return storage_ != nullptr; }
    /* true when both images show the same pixels: the same owned buffer, or
     * (for mapped images) the same first pixel. */
    bool operator==(const Image& other) const noexcept
    {
        return (ownership() && other.ownership()) ? storage_ == other.storage_ : pixels_ == other.pixels_;
    }
    bool operator!=(const Image& other) const noexcept { return !operator==(other); }

private:
    struct Storage;
    int w_ = 0, h_ = 0, c_ = 0;
    ElementType type_ = UInt8;
    int stride_ = 0;
    void* pixels_ = nullptr;
    std::shared_ptr<Storage> storage_;
};

#endif
