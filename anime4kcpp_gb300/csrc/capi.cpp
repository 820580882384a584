// The C ABI: the reference binding's entry points (binding/c/src/Binding.cpp)
// over this backend's Image and Processor, plus the GB300 extensions.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "ac_core.h"
#include "ac_gb300.h"
#include "processor_impl.hpp"
#include "server.hpp"

struct ACImageHandle
{
    acgb::Image object{};
};
struct ACProcessorHandle
{
    std::shared_ptr<acgb::Processor> object{};
};

namespace {

void copy_prop(const acgb::Image& src, ACImage* dst)
{
    dst->width = src.width();
    dst->height = src.height();
    dst->channels = src.channels();
    dst->stride = src.stride();
    dst->element_type = src.type();
    dst->ptr = src.ptr();
}

ACImageHandle* new_image_handle()
{
    return new (std::nothrow) ACImageHandle{};
}

}  // namespace

// ------------------------------------------------------------------ images

ACImage* ac_image_alloc(void)
{
    void* p = std::malloc(sizeof(ACImage));
    if (p) std::memset(p, 0, sizeof(ACImage));
    return static_cast<ACImage*>(p);
}

void ac_image_free(ACImage** image)
{
    if (!(image && *image)) return;
    ac_image_unref(*image);
    std::free(*image);
    *image = nullptr;
}

int ac_image_ref(const ACImage* src, ACImage* dst)
{
    if (!(src && dst && src->hptr)) return AC_ERROR(AC_EINVAL);
    if (!dst->hptr && !(dst->hptr = new_image_handle())) return AC_ERROR(AC_EINVAL);
    dst->hptr->object = src->hptr->object;
    copy_prop(dst->hptr->object, dst);
    return AC_SUCCESS;
}

void ac_image_unref(ACImage* image)
{
    if (!(image && image->hptr)) return;
    delete image->hptr;
    std::memset(image, 0, sizeof(ACImage));
}

int ac_image_create(ACImage* image)
{
    if (!image) return AC_ERROR(AC_EINVAL);
    if (!image->hptr && !(image->hptr = new_image_handle())) return AC_ERROR(AC_EINVAL);
    try
    {
        image->hptr->object.create(image->width, image->height, image->channels, image->element_type, image->stride);
    }
    catch (...)
    {
        return AC_ERROR(AC_EINVAL);
    }
    copy_prop(image->hptr->object, image);
    return AC_SUCCESS;
}

int ac_image_map(ACImage* image)
{
    if (!image) return AC_ERROR(AC_EINVAL);
    if (!image->hptr && !(image->hptr = new_image_handle())) return AC_ERROR(AC_EINVAL);
    image->hptr->object.map(image->width, image->height, image->channels, image->element_type, image->ptr, image->stride);
    copy_prop(image->hptr->object, image);
    return AC_SUCCESS;
}

int ac_image_from(ACImage* image, const void* data)
{
    if (!image) return AC_ERROR(AC_EINVAL);
    if (!image->hptr && !(image->hptr = new_image_handle())) return AC_ERROR(AC_EINVAL);
    try
    {
        image->hptr->object.from(image->width, image->height, image->channels, image->element_type, data, image->stride);
    }
    catch (...)
    {
        return AC_ERROR(AC_EINVAL);
    }
    copy_prop(image->hptr->object, image);
    return AC_SUCCESS;
}

int ac_image_view(const ACImage* src, ACImage* dst, int x, int y, int w, int h)
{
    if (!(src && dst && src->hptr)) return AC_ERROR(AC_EINVAL);
    if (!dst->hptr && !(dst->hptr = new_image_handle())) return AC_ERROR(AC_EINVAL);
    dst->hptr->object = src->hptr->object.view(x, y, w, h);
    copy_prop(dst->hptr->object, dst);
    return AC_SUCCESS;
}

int ac_image_clone(const ACImage* src, ACImage* dst)
{
    if (!(src && dst && src->hptr)) return AC_ERROR(AC_EINVAL);
    if (!dst->hptr && !(dst->hptr = new_image_handle())) return AC_ERROR(AC_EINVAL);
    try
    {
        dst->hptr->object = src->hptr->object.clone();
    }
    catch (...)
    {
        return AC_ERROR(AC_EINVAL);
    }
    copy_prop(dst->hptr->object, dst);
    return AC_SUCCESS;
}

int ac_image_to(const ACImage* image, void* data, int stride)
{
    if (!(image && image->hptr && data)) return AC_ERROR(AC_EINVAL);
    image->hptr->object.to(data, stride);
    return AC_SUCCESS;
}

// ------------------------------------------------ image operations (GPU)

int acgb_image_op(int op, const acgb::Image& src, acgb::Image& dst, double fx, double fy, int mode);

int ac_resize(const ACImage* src, ACImage* dst, double fx, double fy, int mode)
{
    if (!(src && src->hptr && dst && dst->hptr)) return AC_ERROR(AC_EINVAL);
    int rc = acgb_image_op(0, src->hptr->object, dst->hptr->object, fx, fy, mode);
    copy_prop(dst->hptr->object, dst);
    return rc;
}

int ac_rgb2yuv(const ACImage* rgb, ACImage* yuv)
{
    if (!(rgb && rgb->hptr && yuv && yuv->hptr)) return AC_ERROR(AC_EINVAL);
    int rc = acgb_image_op(1, rgb->hptr->object, yuv->hptr->object, 0, 0, 0);
    copy_prop(yuv->hptr->object, yuv);
    return rc;
}

int ac_rgba2yuva(const ACImage* rgba, ACImage* yuva)
{
    if (!(rgba && rgba->hptr && yuva && yuva->hptr)) return AC_ERROR(AC_EINVAL);
    int rc = acgb_image_op(2, rgba->hptr->object, yuva->hptr->object, 0, 0, 0);
    copy_prop(yuva->hptr->object, yuva);
    return rc;
}

int ac_yuv2rgb(const ACImage* yuv, ACImage* rgb)
{
    if (!(yuv && yuv->hptr && rgb && rgb->hptr)) return AC_ERROR(AC_EINVAL);
    int rc = acgb_image_op(3, yuv->hptr->object, rgb->hptr->object, 0, 0, 0);
    copy_prop(rgb->hptr->object, rgb);
    return rc;
}

int ac_yuva2rgba(const ACImage* yuva, ACImage* rgba)
{
    if (!(yuva && yuva->hptr && rgba && rgba->hptr)) return AC_ERROR(AC_EINVAL);
    int rc = acgb_image_op(4, yuva->hptr->object, rgba->hptr->object, 0, 0, 0);
    copy_prop(rgba->hptr->object, rgba);
    return rc;
}

// -------------------------------------------------------------- processors

ACProcessor* ac_processor_alloc(void)
{
    void* p = std::malloc(sizeof(ACProcessor));
    if (p) std::memset(p, 0, sizeof(ACProcessor));
    return static_cast<ACProcessor*>(p);
}

void ac_processor_free(ACProcessor** processor)
{
    if (!(processor && *processor)) return;
    ac_processor_unref(*processor);
    std::free(*processor);
    *processor = nullptr;
}

int ac_processor_ref(const ACProcessor* src, ACProcessor* dst)
{
    if (!(src && dst && src->hptr)) return AC_ERROR(AC_EINVAL);
    if (!dst->hptr && !(dst->hptr = new (std::nothrow) ACProcessorHandle{})) return AC_ERROR(AC_EINVAL);
    dst->hptr->object = src->hptr->object;
    dst->type = src->type;
    dst->device = src->device;
    dst->model = src->model;
    return AC_SUCCESS;
}

void ac_processor_unref(ACProcessor* processor)
{
    if (!(processor && processor->hptr)) return;
    delete processor->hptr;
    std::memset(processor, 0, sizeof(ACProcessor));
}

int ac_processor_create(ACProcessor* processor)
{
    if (!processor) return AC_ERROR(AC_EINVAL);
    if (!processor->hptr && !(processor->hptr = new (std::nothrow) ACProcessorHandle{})) return AC_ERROR(AC_EINVAL);
    try
    {
        processor->hptr->object = acgb::Processor::create(processor->type, processor->device, processor->model);
    }
    catch (...)
    {
        return AC_ERROR(AC_EPROCESSOR);
    }
    return ac_processor_ok(processor);
}

int ac_processor_process(ACProcessor* processor, const ACImage* src, ACImage* dst, double factor)
{
    if (!(processor && processor->hptr && processor->hptr->object && src && src->hptr && dst && dst->hptr))
        return AC_ERROR(AC_EINVAL);
    processor->hptr->object->process(src->hptr->object, dst->hptr->object, factor);
    copy_prop(dst->hptr->object, dst);
    return ac_processor_ok(processor);
}

int ac_processor_ok(const ACProcessor* processor)
{
    if (!(processor && processor->hptr && processor->hptr->object)) return AC_ERROR(AC_EINVAL);
    return processor->hptr->object->ok() ? AC_SUCCESS : AC_ERROR(AC_EPROCESSOR);
}

const char* ac_processor_error(const ACProcessor* processor)
{
    if (!(processor && processor->hptr && processor->hptr->object)) return nullptr;
    return processor->hptr->object->error();
}

const char* ac_processor_name(const ACProcessor* processor)
{
    if (!(processor && processor->hptr && processor->hptr->object)) return nullptr;
    return processor->hptr->object->name();
}

int ac_processor_type(const ACProcessor* processor)
{
    if (!(processor && processor->hptr && processor->hptr->object)) return AC_ERROR(AC_EINVAL);
    return processor->hptr->object->type();
}

const char* ac_processor_type_name(const ACProcessor* processor)
{
    if (!(processor && processor->hptr && processor->hptr->object)) return nullptr;
    return processor->hptr->object->typeName();
}

const char* ac_processor_info(int processor_type)
{
    switch (processor_type)
    {
    case AC_PROCESSOR_CPU:
    case AC_PROCESSOR_OPENCL:
    case AC_PROCESSOR_CUDA: return acgb::processor_info(processor_type);
    default: return "unsupported processor";
    }
}

const char* ac_processor_list_info(void) { return acgb::Processor::listInfo(); }

// -------------------------------------------------------------- extensions

namespace {

acgb::GB300Processor* gpu_of(const ACProcessor* p)
{
    if (!(p && p->hptr && p->hptr->object)) return nullptr;
    return dynamic_cast<acgb::GB300Processor*>(p->hptr->object.get());
}

}  // namespace

int ac_gb300_set_precision(ACProcessor* processor, int precision)
{
    auto* g = gpu_of(processor);
    if (!g || precision < 0 || precision > 2) return AC_ERROR(AC_EINVAL);
    g->setPrecision(static_cast<acgb::Precision>(precision));
    return AC_SUCCESS;
}

int ac_gb300_get_precision(const ACProcessor* processor)
{
    auto* g = gpu_of(processor);
    if (!g) return AC_ERROR(AC_EINVAL);
    return static_cast<int>(g->precision());
}

int ac_gb300_output_shape(int width, int height, int channels, double factor, int* out_width, int* out_height)
{
    if (!out_width || !out_height || width <= 0 || height <= 0 || !(factor > 0.0)) return AC_ERROR(AC_EINVAL);
    acgb::output_shape(width, height, channels, factor, *out_width, *out_height);
    return AC_SUCCESS;
}

int ac_gb300_process_device(ACProcessor* processor, const ACGB300DeviceImage* src, const ACGB300DeviceImage* dst,
                            double factor, void* stream, int sync)
{
    auto* g = gpu_of(processor);
    if (!g || !src || !dst) return AC_ERROR(AC_EINVAL);
    acgb::DeviceImage s{src->ptr, src->width, src->height, src->channels, src->stride, src->element_type};
    acgb::DeviceImage d{dst->ptr, dst->width, dst->height, dst->channels, dst->stride, dst->element_type};
    int rc = g->processDevice(s, d, factor, static_cast<cudaStream_t>(stream), sync != 0);
    return rc == 0 ? AC_SUCCESS : AC_ERROR(AC_EPROCESSOR);
}

int ac_gb300_process_batch_device(ACProcessor* processor, int count, const ACGB300DeviceImage* src,
                                  const ACGB300DeviceImage* dst, double factor, void* stream, int sync)
{
    auto* g = gpu_of(processor);
    if (!g || count < 0 || (count > 0 && (!src || !dst))) return AC_ERROR(AC_EINVAL);
    std::vector<acgb::DeviceImage> s(count), d(count);
    for (int i = 0; i < count; i++)
    {
        s[i] = acgb::DeviceImage{src[i].ptr, src[i].width, src[i].height, src[i].channels, src[i].stride, src[i].element_type};
        d[i] = acgb::DeviceImage{dst[i].ptr, dst[i].width, dst[i].height, dst[i].channels, dst[i].stride, dst[i].element_type};
    }
    const int rc = g->processBatchDevice(count, s.data(), d.data(), factor, static_cast<cudaStream_t>(stream), sync != 0);
    return rc == 0 ? AC_SUCCESS : AC_ERROR(AC_EPROCESSOR);
}

uint64_t ac_gb300_graph_replays(void) { return acgb::graph_replays(); }

void ac_gb300_debug_fail_alloc(int nth) { acgb::arm_alloc_failure(nth); }

int ac_gb300_last_plan(ACProcessor* processor, int* kernel, int* tile_w, int* tile_h, int* ctas_per_sm,
                       int* fusion_depth)
{
    acgb::GB300Processor* g = gpu_of(processor);
    if (!g || !kernel || !tile_w || !tile_h || !ctas_per_sm) return AC_ERROR(AC_EINVAL);
    const acgb::GB300Processor::LastPlan p = g->lastPlan();
    int tw = 0, th = 0;
    if (p.kernel == 4 && p.depth == 5) acgb::acnet_tc4_split_tail_shape(&tw, &th);
    else if (p.kernel == 4) acgb::acnet_tc4_shape(p.shape, &tw, &th);
    else if (p.kernel == 3) acgb::acnet_tc3_shape(p.shape, &tw, &th);
    else if (p.kernel == 5 && p.depth == 5) acgb::acnet8_tc4_split_tail_shape(&tw, &th);
    else if (p.kernel == 5) acgb::acnet8_tc4_shape(g->spec().blocks, &tw, &th);
    *kernel = p.kernel;
    *tile_w = tw;
    *tile_h = th;
    *ctas_per_sm = p.perSm;
    if (fusion_depth) *fusion_depth = p.kernel ? p.depth : 0;
    return AC_SUCCESS;
}

int ac_gb300_process_yuv_device(ACProcessor* processor, int frames, int planes, const ACGB300DeviceImage* src,
                                const ACGB300DeviceImage* dst, double factor, int shift, void* stream, int sync)
{
    auto* g = gpu_of(processor);
    if (!g || frames < 1 || planes < 1 || planes > 4 || !src || !dst) return AC_ERROR(AC_EINVAL);
    const int n = frames * planes;
    std::vector<acgb::DeviceImage> s(n), d(n);
    for (int i = 0; i < n; i++)
    {
        s[i] = acgb::DeviceImage{src[i].ptr, src[i].width, src[i].height, src[i].channels, src[i].stride, src[i].element_type};
        d[i] = acgb::DeviceImage{dst[i].ptr, dst[i].width, dst[i].height, dst[i].channels, dst[i].stride, dst[i].element_type};
    }
    const int rc = g->processYuvDevice(frames, planes, s.data(), d.data(), factor, shift, static_cast<cudaStream_t>(stream),
                                       sync != 0);
    return rc == 0 ? AC_SUCCESS : AC_ERROR(AC_EPROCESSOR);
}

int ac_gb300_process_device_noalloc(ACProcessor* processor, int count, const ACGB300DeviceImage* src,
                                    const ACGB300DeviceImage* dst, void* stream, int sync)
{
    auto* g = gpu_of(processor);
    if (!g || !src || !dst) return AC_ERROR(AC_EINVAL);
    if (count < 1 || count > 64)  // rejected with a message by the processor
        return g->processDeviceNoAlloc(count, nullptr, nullptr, static_cast<cudaStream_t>(stream), false), AC_ERROR(AC_EINVAL);
    acgb::DeviceImage s[64], d[64];
    for (int i = 0; i < count; i++)
    {
        s[i] = acgb::DeviceImage{src[i].ptr, src[i].width, src[i].height, src[i].channels, src[i].stride, src[i].element_type};
        d[i] = acgb::DeviceImage{dst[i].ptr, dst[i].width, dst[i].height, dst[i].channels, dst[i].stride, dst[i].element_type};
    }
    const int rc = g->processDeviceNoAlloc(count, s, d, static_cast<cudaStream_t>(stream), sync != 0);
    return rc == 0 ? AC_SUCCESS : (rc == -2 ? AC_ERROR(AC_EINVAL) : AC_ERROR(AC_EPROCESSOR));
}

uint64_t ac_gb300_launch_count(void) { return acgb::launch_count(); }

int ac_gb300_profile_enable(ACProcessor* processor, int enable)
{
    auto* g = gpu_of(processor);
    if (!g) return AC_ERROR(AC_EINVAL);
    g->setProfiling(enable != 0);
    return AC_SUCCESS;
}

int ac_gb300_profile_collect(ACProcessor* processor, double* ms, int* launches, double* out_pixels)
{
    auto* g = gpu_of(processor);
    if (!g || !ms || !launches || !out_pixels) return AC_ERROR(AC_EINVAL);
    return g->collectProfile(*ms, *launches, *out_pixels) == 0 ? AC_SUCCESS : AC_ERROR(AC_EPROCESSOR);
}

int ac_gb300_model_params(const char* model, float* kernels, int kernels_len, float* biases, int biases_len, float* alphas,
                          int alphas_len, int* counts)
{
    acgb::ModelSpec spec;
    std::string err;
    if (!acgb::parse_model(model, spec, err)) return AC_ERROR(AC_EINVAL);
    const acgb::ModelParams& p = acgb::model_params(spec);
    if (counts)
    {
        counts[0] = static_cast<int>(p.kernels.size());
        counts[1] = static_cast<int>(p.biases.size());
        counts[2] = static_cast<int>(p.alphas.size());
    }
    if (kernels)
    {
        if (kernels_len < static_cast<int>(p.kernels.size())) return AC_ERROR(AC_EINVAL);
        std::memcpy(kernels, p.kernels.data(), p.kernels.size() * sizeof(float));
    }
    if (biases)
    {
        if (biases_len < static_cast<int>(p.biases.size())) return AC_ERROR(AC_EINVAL);
        std::memcpy(biases, p.biases.data(), p.biases.size() * sizeof(float));
    }
    if (alphas && !p.alphas.empty())
    {
        if (alphas_len < static_cast<int>(p.alphas.size())) return AC_ERROR(AC_EINVAL);
        std::memcpy(alphas, p.alphas.data(), p.alphas.size() * sizeof(float));
    }
    return AC_SUCCESS;
}

// ---- serving loop ----

struct ACGB300Server
{
    std::unique_ptr<acgb::Server> server;
};

static acgb::HostPlane host_plane(const ACGB300HostPlane& p)
{
    return acgb::HostPlane{p.ptr, p.width, p.height, p.channels, p.stride, p.element_type};
}

ACGB300Server* ac_gb300_server_create(int device, int precision, double hbm_budget_bytes, int workers, int max_batch)
{
    auto* s = new (std::nothrow) ACGB300Server;
    if (!s) return nullptr;
    const acgb::Precision p = precision == AC_GB300_BF16 ? acgb::Precision::BF16
                              : precision == AC_GB300_FP16 ? acgb::Precision::FP16
                                                           : acgb::Precision::FP32;
    const size_t budget = hbm_budget_bytes > 0.0 ? static_cast<size_t>(hbm_budget_bytes) : 0;
    s->server.reset(new (std::nothrow) acgb::Server(device, p, budget, workers, max_batch));
    return s;
}

const char* ac_gb300_server_error(const ACGB300Server* server)
{
    if (!server || !server->server) return "no server";
    return server->server->initError().empty() ? nullptr : server->server->initError().c_str();
}

int ac_gb300_server_submit(ACGB300Server* server, const ACGB300ServeJob* job, uint64_t* ticket)
{
    if (!server || !server->server || !job || !job->model || !ticket) return AC_ERROR(AC_EINVAL);
    acgb::ServeJob j;
    j.model = job->model;
    j.factor = job->factor;
    j.planes = job->planes;
    j.shift = job->shift;
    for (int i = 0; i < 3; i++)
    {
        j.src[i] = host_plane(job->src[i]);
        j.dst[i] = host_plane(job->dst[i]);
    }
    *ticket = server->server->submit(j);
    return AC_SUCCESS;
}

int ac_gb300_server_wait(ACGB300Server* server, uint64_t ticket, double timeout_s, ACGB300ServeResult* result)
{
    if (!server || !server->server || !result) return AC_ERROR(AC_EINVAL);
    acgb::ServeResult r;
    if (!server->server->wait(ticket, timeout_s, r)) return 1;
    result->status = r.status;
    result->queue_ms = r.queueMs;
    result->device_ms = r.deviceMs;
    result->latency_ms = r.latencyMs;
    result->h2d_ms = r.h2dMs;
    result->compute_ms = r.computeMs;
    result->d2h_ms = r.d2hMs;
    result->batch = r.batch;
    std::snprintf(result->error, sizeof(result->error), "%s", r.error.c_str());
    return AC_SUCCESS;
}

int ac_gb300_server_stats(ACGB300Server* server, ACGB300ServeStats* stats)
{
    if (!server || !server->server || !stats) return AC_ERROR(AC_EINVAL);
    const acgb::ServeStats s = server->server->stats();
    stats->submitted = s.submitted;
    stats->completed = s.completed;
    stats->failed = s.failed;
    stats->batches = s.batches;
    stats->batched_jobs = s.batchedJobs;
    stats->budget_bytes = s.budgetBytes;
    stats->in_use_bytes = s.inUseBytes;
    stats->peak_bytes = s.peakBytes;
    stats->pool_bytes = s.poolBytes;
    stats->device_allocs = s.deviceAllocs;
    return AC_SUCCESS;
}

void ac_gb300_server_destroy(ACGB300Server* server) { delete server; }
