/*
 * Host image handles and image operations of the C ABI.
 *
 * Drop-in replacement for the reference binding's image API
 * (binding/c/include/AC/Core/Image.h:52-126, implemented in
 * binding/c/src/Binding.cpp:32-189).  Struct layout, enum values, function
 * names, argument meaning and return codes are kept identical so that code
 * compiled against the reference header links against this library.
 *
 * Images live in host memory.  The colour and resize operations below run on
 * the GPU (copy in, kernel, copy out); there is no CPU implementation.
 */
#ifndef AC_GB300_IMAGE_H
#define AC_GB300_IMAGE_H

#include <stdint.h>
#include <stddef.h>

#if defined(_WIN32)
#   define AC_GB300_EXPORT __declspec(dllexport)
#else
#   define AC_GB300_EXPORT __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
#   define AC_C_API extern "C" AC_GB300_EXPORT
#else
#   define AC_C_API AC_GB300_EXPORT
#endif

/* Image.h:15-20: (kind << 8) | bytes; kind 0 = unsigned, 2 = float. */
enum ACImageElementType
{
    AC_IMAGE_UINT8   = 0 << 8 | 1,
    AC_IMAGE_UINT16  = 0 << 8 | 2,
    AC_IMAGE_FLOAT32 = 2 << 8 | 4
};

/* Image.h:22-29 (image file I/O itself is not provided by this backend). */
enum ACImreadModes
{
    AC_IMREAD_UNCHANGED = 0,
    AC_IMREAD_GRAYSCALE = 1,
    AC_IMREAD_COLOR     = 3,
    AC_IMREAD_RGB       = 3,
    AC_IMREAD_RGBA      = 4,
};

/* Image.h:31-50.  This backend implements POINT, CATMULL_ROM and BILINEAR;
 * the other filter modes return AC_ERROR(AC_EINVAL) from ac_resize. */
enum ACResizeModes
{
    AC_RESIZE_POINT,
    AC_RESIZE_CATMULL_ROM,
    AC_RESIZE_MITCHELL_NETRAVALI,
    AC_RESIZE_BICUBIC_0_60,
    AC_RESIZE_BICUBIC_0_75,
    AC_RESIZE_BICUBIC_0_100,
    AC_RESIZE_BICUBIC_20_50,
    AC_RESIZE_SOFTCUBIC50,
    AC_RESIZE_SOFTCUBIC75,
    AC_RESIZE_SOFTCUBIC100,
    AC_RESIZE_LANCZOS2,
    AC_RESIZE_LANCZOS3,
    AC_RESIZE_LANCZOS4,
    AC_RESIZE_SPLINE16,
    AC_RESIZE_SPLINE36,
    AC_RESIZE_SPLINE64,
    AC_RESIZE_BILINEAR,
};

/* Image.h:52-61: same field order and types. */
typedef struct ACImage
{
    int width;
    int height;
    int channels;
    int stride;
    int element_type;
    void* ptr;
    struct ACImageHandle* hptr;
} ACImage;

/* Replaces Image.h:63 / Binding.cpp:32-38: zeroed heap struct. */
AC_C_API ACImage* ac_image_alloc(void);
/* Replaces Image.h:64 / Binding.cpp:39-45: unref, free, null the pointer. */
AC_C_API void ac_image_free(ACImage** image);
/* Replaces Image.h:65 / Binding.cpp:46-53: dst shares src's pixels. */
AC_C_API int ac_image_ref(const ACImage* src, ACImage* dst);
/* Replaces Image.h:66 / Binding.cpp:54-59: drop the handle, zero the struct. */
AC_C_API void ac_image_unref(ACImage* image);
/* Replaces Image.h:67 / Binding.cpp:60-67: allocate width x height x channels
 * of element_type with row stride max(stride, aligned line size). */
AC_C_API int ac_image_create(ACImage* image);
/* Replaces Image.h:68 / Binding.cpp:68-75: wrap image->ptr without ownership. */
AC_C_API int ac_image_map(ACImage* image);
/* Replaces Image.h:69 / Binding.cpp:76-83: allocate and copy from data. */
AC_C_API int ac_image_from(ACImage* image, const void* data);
/* Replaces Image.h:70 / Binding.cpp:84-91: sub-rectangle sharing pixels. */
AC_C_API int ac_image_view(const ACImage* src, ACImage* dst, int x, int y, int w, int h);
/* Replaces Image.h:71 / Binding.cpp:92-99: deep copy. */
AC_C_API int ac_image_clone(const ACImage* src, ACImage* dst);
/* Replaces Image.h:72 / Binding.cpp:100-105: copy pixels out to data. */
AC_C_API int ac_image_to(const ACImage* image, void* data, int stride);

/* Replaces Image.h:79 / Binding.cpp:127-133 (resize, GPU). */
AC_C_API int ac_resize(const ACImage* src, ACImage* dst, double fx, double fy, int mode);
/* Replaces Image.h:80 / Binding.cpp:134-140 (rgb -> interleaved yuv, GPU). */
AC_C_API int ac_rgb2yuv(const ACImage* rgb, ACImage* yuv);
/* Replaces Image.h:81 / Binding.cpp:141-147 (rgba -> yuva, GPU). */
AC_C_API int ac_rgba2yuva(const ACImage* rgba, ACImage* yuva);
/* Replaces Image.h:82 / Binding.cpp:148-154 (yuv -> rgb, GPU). */
AC_C_API int ac_yuv2rgb(const ACImage* yuv, ACImage* rgb);
/* Replaces Image.h:83 / Binding.cpp:155-161 (yuva -> rgba, GPU). */
AC_C_API int ac_yuva2rgba(const ACImage* yuva, ACImage* rgba);

/* Image.h:85-126: inline accessors, same definitions. */
static inline int ac_image_size(const ACImage* image) { return image->height * image->stride; }
static inline int ac_image_element_size(const ACImage* image) { return image->element_type & 0xff; }
static inline int ac_image_pixel_size(const ACImage* image) { return image->channels * ac_image_element_size(image); }
static inline uint8_t* ac_image_data(const ACImage* image) { return (uint8_t*)image->ptr; }
static inline uint8_t* ac_image_line(const ACImage* image, int y) { return ac_image_data(image) + image->stride * y; }
static inline uint8_t* ac_image_pixel(const ACImage* image, int x, int y) { return ac_image_line(image, y) + x * ac_image_pixel_size(image); }
static inline int ac_image_empty(const ACImage* image) { return image->ptr == NULL; }
static inline int ac_image_is_uint(const ACImage* image) { return (image->element_type >> 8) == 0; }
static inline int ac_image_is_int(const ACImage* image) { return (image->element_type >> 8) == 1; }
static inline int ac_image_is_float(const ACImage* image) { return (image->element_type >> 8) == 2; }

#endif
