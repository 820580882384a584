// Host-image operations of the C ABI (ac_resize, ac_rgb2yuv, ac_rgba2yuva,
// ac_yuv2rgb, ac_yuva2rgba) executed on the GPU: copy in, one kernel, copy
// out.  Shape rules follow core/src/ImageResize.cpp:136-170,275-293 and
// core/src/ImageProcess.cpp:436-577.
#include <mutex>

#include "ac_error.h"
#include "processor_impl.hpp"

namespace acgb {
namespace {

struct OpsContext
{
    std::mutex m;
    bool init = false;
    int device = 0;
    cudaStream_t stream = nullptr;
    DeviceBuffer a, b, ta, tb;
};

OpsContext& ops()
{
    static OpsContext* ctx = new OpsContext();  // intentionally leaked: no teardown ordering at exit
    return *ctx;
}

inline int align256(int v) { return (v + 255) & ~255; }

}  // namespace
}  // namespace acgb

// op: 0 resize, 1 rgb2yuv, 2 rgba2yuva, 3 yuv2rgb, 4 yuva2rgba
int acgb_image_op(int op, const acgb::Image& src, acgb::Image& dst, double fx, double fy, int mode)
{
    using namespace acgb;
    if (src.empty()) return AC_SUCCESS;
    int type = src.type();
    if (type != Image::UInt8 && type != Image::UInt16 && type != Image::Float32) return AC_ERROR(AC_EINVAL);
    int ow = src.width(), oh = src.height(), oc = src.channels();
    Image out = dst;
    if (op == 0)
    {
        if (mode != 0 && mode != 1 && mode != 16) return AC_ERROR(AC_EINVAL);
        if (fx > 0.0 && fy > 0.0)
        {
            if (fx == 1.0 && fy == 1.0)
            {
                dst = src;
                return AC_SUCCESS;
            }
            ow = static_cast<int>(src.width() * fx);
            oh = static_cast<int>(src.height() * fy);
        }
        else
        {
            if (dst.empty()) return AC_SUCCESS;
            if (dst.width() == src.width() && dst.height() == src.height())
            {
                dst = src;
                return AC_SUCCESS;
            }
            ow = dst.width();
            oh = dst.height();
        }
        if (ow <= 0 || oh <= 0) return AC_ERROR(AC_EINVAL);
        if (src == dst || out.width() != ow || out.height() != oh || out.channels() != oc || out.type() != type)
        {
            out = Image{};
            out.create(ow, oh, oc, type);
        }
    }
    else
    {
        if ((op == 1 && oc != 3) || ((op == 2 || op == 4) && oc != 4) || (op == 3 && oc != 3)) return AC_ERROR(AC_EINVAL);
        if (out.empty()) out.create(ow, oh, oc, type);
        if (out.width() != ow || out.height() != oh || out.channels() != oc || out.type() != type) return AC_ERROR(AC_EINVAL);
    }

    OpsContext& c = ops();
    std::lock_guard<std::mutex> lock(c.m);
    cudaError_t err;
    if (!c.init)
    {
        if ((err = cudaGetDevice(&c.device)) != cudaSuccess) return AC_ERROR(AC_EPROCESSOR);
        if ((err = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking)) != cudaSuccess) return AC_ERROR(AC_EPROCESSOR);
        c.init = true;
    }
    cudaSetDevice(c.device);
    const int es = type & 0xff;
    Plane ps{nullptr, src.width(), src.height(), align256(src.width() * oc * es), oc, type};
    Plane pd{nullptr, ow, oh, align256(ow * oc * es), oc, type};
    if (c.a.ensure(static_cast<size_t>(ps.pitch) * ps.h) != cudaSuccess) return AC_ERROR(AC_EPROCESSOR);
    if (c.b.ensure(static_cast<size_t>(pd.pitch) * pd.h) != cudaSuccess) return AC_ERROR(AC_EPROCESSOR);
    ps.ptr = c.a.ptr;
    pd.ptr = c.b.ptr;
    err = cudaMemcpy2DAsync(ps.ptr, ps.pitch, src.ptr(), src.stride(), static_cast<size_t>(src.width()) * src.pixelSize(),
                            src.height(), cudaMemcpyHostToDevice, c.stream);
    if (err != cudaSuccess) return AC_ERROR(AC_EPROCESSOR);
    std::vector<int> fxv, fyv;
    std::vector<float> wxv, wyv;
    switch (op)
    {
    case 0:
    {
        int tx, ty;
        make_axis_table(src.width(), ow, mode, fxv, wxv, tx);
        make_axis_table(src.height(), oh, mode, fyv, wyv, ty);
        size_t o1 = align256(static_cast<int>(fxv.size() * sizeof(int)));
        size_t o2 = o1 + align256(static_cast<int>(wxv.size() * sizeof(float)));
        size_t o3 = o2 + align256(static_cast<int>(fyv.size() * sizeof(int)));
        size_t total = o3 + wyv.size() * sizeof(float);
        if (c.ta.ensure(total) != cudaSuccess) return AC_ERROR(AC_EPROCESSOR);
        char* base = static_cast<char*>(c.ta.ptr);
        cudaMemcpyAsync(base, fxv.data(), fxv.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream);
        cudaMemcpyAsync(base + o1, wxv.data(), wxv.size() * sizeof(float), cudaMemcpyHostToDevice, c.stream);
        cudaMemcpyAsync(base + o2, fyv.data(), fyv.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream);
        cudaMemcpyAsync(base + o3, wyv.data(), wyv.size() * sizeof(float), cudaMemcpyHostToDevice, c.stream);
        ResizeAxis ax{reinterpret_cast<const int*>(base), reinterpret_cast<const float*>(base + o1), tx};
        ResizeAxis ay{reinterpret_cast<const int*>(base + o2), reinterpret_cast<const float*>(base + o3), ty};
        err = launch_resize(ps, pd, ax, ay, c.stream);
        break;
    }
    case 1:
    case 2: err = launch_rgb2yuv_packed(ps, pd, c.stream); break;
    default: err = launch_yuv2rgb_packed(ps, pd, c.stream); break;
    }
    if (err != cudaSuccess) return AC_ERROR(AC_EPROCESSOR);
    err = cudaMemcpy2DAsync(out.ptr(), out.stride(), pd.ptr, pd.pitch, static_cast<size_t>(ow) * out.pixelSize(), oh,
                            cudaMemcpyDeviceToHost, c.stream);
    if (err != cudaSuccess) return AC_ERROR(AC_EPROCESSOR);
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) return AC_ERROR(AC_EPROCESSOR);
    dst = out;
    return AC_SUCCESS;
}

// ------------------------------------------- ac::core image operations

namespace ac::core {

void rgb2yuv(const Image& rgb, Image& yuv) { acgb_image_op(1, rgb, yuv, 0.0, 0.0, 0); }
void rgba2yuva(const Image& rgba, Image& yuva) { acgb_image_op(2, rgba, yuva, 0.0, 0.0, 0); }
void yuv2rgb(const Image& yuv, Image& rgb) { acgb_image_op(3, yuv, rgb, 0.0, 0.0, 0); }
void yuva2rgba(const Image& yuva, Image& rgba) { acgb_image_op(4, yuva, rgba, 0.0, 0.0, 0); }

void resize(const Image& src, Image& dst, double fx, double fy, int mode) noexcept
{
    try
    {
        acgb_image_op(0, src, dst, fx, fy, mode);
    }
    catch (...)
    {
    }
}

Image resize(const Image& src, double fx, double fy, int mode) noexcept
{
    if (!(fx > 0.0) || !(fy > 0.0)) return src;
    Image dst;
    resize(src, dst, fx, fy, mode);
    return dst;
}

}  // namespace ac::core
