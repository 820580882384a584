// GB300 processor: the whole Processor::process path on one GPU.
//
// Pipeline of one call (core/src/processor/Processor.cpp:199-276):
//   power = factor > 2 ? ceilLog2(factor) : 1, fxy = factor / 2^power
//   RGB(A): split into Y and UV(A) (quantised to the source type)
//   `power` luma passes of the CNN, each x2
//   luma resize by fxy when fxy != 1 (Catmull-Rom)
//   RGB(A): chroma resampled by `factor` on the fly and merged back
// Host images are copied to device buffers once per call; intermediates stay
// in HBM.  Per calling thread the processor keeps a CUDA stream, grow-only
// device workspaces, cached resampling tables and the error state (the
// reference keeps per-thread scratch and error state the same way,
// core/src/processor/cuda/CUDAProcessor.cpp:284,374-377).
#include "processor_impl.hpp"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstring>
#include <sstream>

namespace acgb {

// ---------------------------------------------------------------- helpers

int ceil_log2(double v)
{
    // core/internal/AC/Core/Internal/Util.hpp:80-89.
    uint64_t bits;
    std::memcpy(&bits, &v, sizeof(bits));
    return static_cast<int>(static_cast<int64_t>((bits >> 52) & 0x7ff) - 1023 + ((bits << 12) != 0 ? 1 : 0));
}

void output_shape(int w, int h, int c, double factor, int& ow, int& oh)
{
    int power = factor > 2.0 ? ceil_log2(factor) : 1;
    double fxy = factor / static_cast<double>(1 << power);
    int lw = w << power, lh = h << power;
    if (fxy != 1.0)
    {
        lw = static_cast<int>(lw * fxy);
        lh = static_cast<int>(lh * fxy);
    }
    ow = lw;
    oh = lh;
    (void)c;
}

namespace {

// Resampling coefficients: the same arithmetic as the project's CPU
// restatement of the reference filters (ImageResize.cpp:62-83, 127-134).
float filter_eval(int mode, float x)
{
    float ax = std::fabs(x);
    if (mode == 16) return ax < 1.0f ? 1.0f - ax : 0.0f;
    if (mode == 0) return ax <= 0.5f ? 1.0f : 0.0f;
    if (ax < 1.0f) return 1.0f + ax * (0.0f + ax * (-2.5f + ax * 1.5f));
    if (ax < 2.0f) return 2.0f + ax * (-4.0f + ax * (2.5f + ax * -0.5f));
    return 0.0f;
}
float filter_support(int mode) { return mode == 16 ? 1.0f : (mode == 0 ? 0.5f : 2.0f); }

}  // namespace

void make_axis_table(int n_in, int n_out, int mode, std::vector<int>& first, std::vector<float>& weights, int& taps)
{
    constexpr int MT = 64;
    double scale = static_cast<double>(n_out) / static_cast<double>(n_in);
    float sup = filter_support(mode);
    float fscale = scale < 1.0 ? static_cast<float>(scale) : 1.0f;
    float radius = sup / fscale;
    std::vector<float> full(static_cast<size_t>(n_out) * MT, 0.0f);
    first.assign(n_out, 0);
    int maxUsed = 1;
    for (int o = 0; o < n_out; o++)
    {
        float center = static_cast<float>((static_cast<double>(o) + 0.5) / scale - 0.5);
        int lo = static_cast<int>(std::ceil(center - radius));
        int hi = static_cast<int>(std::floor(center + radius));
        if (mode == 0)
        {
            lo = static_cast<int>(std::floor(center + 0.5f));
            hi = lo;
        }
        if (hi - lo + 1 > MT) hi = lo + MT - 1;
        int cnt = hi - lo + 1;
        float wv[MT];
        float sum = 0.0f;
        for (int t = 0; t < cnt; t++)
        {
            float d = (static_cast<float>(lo + t) - center) * fscale;
            wv[t] = mode == 0 ? 1.0f : filter_eval(mode, d);
            sum += wv[t];
        }
        first[o] = lo;
        for (int t = 0; t < cnt; t++)
        {
            float v = sum != 0.0f ? wv[t] / sum : 0.0f;
            full[static_cast<size_t>(o) * MT + t] = v;
            if (v != 0.0f) maxUsed = std::max(maxUsed, t + 1);
        }
    }
    taps = maxUsed;
    weights.assign(static_cast<size_t>(n_out) * taps, 0.0f);
    for (int o = 0; o < n_out; o++)
        for (int t = 0; t < taps; t++) weights[static_cast<size_t>(o) * taps + t] = full[static_cast<size_t>(o) * MT + t];
}

// Catmull-Rom weights of an exact integer upscale, per output phase: output
// o = F*i + k uses source taps i + merge_int_phase_offset(F, k) + 0..3.  The
// weights do not depend on i (centres are exact binary fractions), which is
// verified here on a table of 64 outputs; returns false if the table has any
// other structure.
bool phase_weights(int F, float* w)
{
    std::vector<int> first;
    std::vector<float> wt;
    int taps = 0;
    make_axis_table(16, 16 * F, 1, first, wt, taps);
    if (taps > 4) return false;
    for (int o = 0; o < 16 * F; o++)
    {
        const int k = o % F;
        if (first[o] - o / F != merge_int_phase_offset(F, k)) return false;
        for (int t = 0; t < 4; t++)
        {
            const float v = t < taps ? wt[static_cast<size_t>(o) * taps + t] : 0.0f;
            if (o < F) w[k * 4 + t] = v;
            else if (v != w[k * 4 + t]) return false;
        }
    }
    return true;
}

// ----------------------------------------------------------- DeviceBuffer

cudaError_t DeviceBuffer::ensure(size_t bytes)
{
    if (bytes <= cap) return cudaSuccess;
    // Grow by at least half the current capacity (few growth events), in
    // 2 MB steps.  The outgrown block is not freed here: cudaFree waits for
    // the whole device, which would stall every other stream's work (the
    // serving loop's latency); it is kept until release().
    const size_t step = 2u << 20;
    const size_t grown = cap + cap / 2;
    const size_t want = (std::max(bytes, grown) + step - 1) & ~(step - 1);
    if (injected_alloc_failure()) return cudaErrorMemoryAllocation;
    void* fresh = nullptr;
    cudaError_t err = cudaMalloc(&fresh, want);
    if (err != cudaSuccess)
    {
        cudaGetLastError();  // the failed allocation is reported here, not left for a later check
        return err;
    }
    device_alloc_count().fetch_add(1, std::memory_order_relaxed);
    if (ptr)
    {
        try
        {
            retired.push_back(ptr);
        }
        catch (...)
        {
            cudaFree(ptr);
        }
    }
    ptr = fresh;
    cap = want;
    return cudaSuccess;
}

std::atomic<uint64_t>& device_alloc_count()
{
    static std::atomic<uint64_t> n{0};
    return n;
}

// Host-side fault injection: while armed with n > 0, the n-th next device
// allocation of DeviceBuffer::ensure or the serving pool fails as if the
// device were out of memory (no cudaMalloc is made for it).
namespace {
std::atomic<int> g_fail_alloc_countdown{0};
}

void arm_alloc_failure(int nth) { g_fail_alloc_countdown.store(nth > 0 ? nth : 0); }

bool injected_alloc_failure()
{
    int v = g_fail_alloc_countdown.load();
    while (v > 0)
        if (g_fail_alloc_countdown.compare_exchange_weak(v, v - 1)) return v == 1;
    return false;
}

void DeviceBuffer::release()
{
    if (ptr) cudaFree(ptr);
    for (void* r : retired) cudaFree(r);
    retired.clear();
    ptr = nullptr;
    cap = 0;
}

// ------------------------------------------------------------ Processor

}  // namespace acgb

// ---------------------------------------------------- ac::core::Processor

namespace ac::core {

Processor::Processor() noexcept = default;
Processor::~Processor() = default;

Image Processor::process(const Image& src, double factor)
{
    Image dst{};
    processPath(src, dst, factor);
    return dst;
}

void Processor::process(const Image& src, Image& dst, double factor) { processPath(src, dst, factor); }

bool Processor::ok() noexcept { return true; }
const char* Processor::error() noexcept { return "NO ERROR"; }

}  // namespace ac::core

namespace acgb {
namespace {

class UnavailableProcessor final : public Processor
{
public:
    UnavailableProcessor(int type, std::string why) : type_(type), why_(std::move(why)) {}
    bool ok() noexcept override { return false; }
    const char* error() noexcept override { return why_.c_str(); }
    const char* name() const noexcept override { return "unavailable"; }
    int type() const noexcept override { return type_; }
    const char* typeName() const noexcept override
    {
        return type_ == CPU ? "CPU" : (type_ == OpenCL ? "OpenCL" : "CUDA");
    }

protected:
    void processPath(const Image&, Image&, double) override {}

private:
    int type_;
    std::string why_;
};

int find_processor_type(const char* type)
{
    // Processor.cpp:12-25: "auto" -> -1, "opencl", "cuda", anything else CPU.
    if (!type) return Processor::CPU;
    std::string s = type;
    for (char& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
    if (s == "auto") return -1;
    if (s == "opencl") return Processor::OpenCL;
    if (s == "cuda") return Processor::CUDA;
    return Processor::CPU;
}

}  // namespace

const char* processor_info(int type)
{
    if (type != Processor::CUDA) return "not provided by the GB300 backend\n";
    static std::string text = []() {
        std::ostringstream os;
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
        os << "GB300 CUDA backend (sm_103a):\n";
        if (n == 0) os << "  no CUDA device\n";
        for (int i = 0; i < n; i++)
        {
            cudaDeviceProp p{};
            if (cudaGetDeviceProperties(&p, i) != cudaSuccess) continue;
            os << "  [" << i << "] " << p.name << ", compute capability " << p.major << "." << p.minor << ", "
               << p.multiProcessorCount << " SMs, " << (p.totalGlobalMem >> 20) << " MiB\n";
        }
        return os.str();
    }();
    return text.c_str();
}

}  // namespace acgb

namespace ac::core {

std::shared_ptr<Processor> Processor::create(const char* type, int device, const char* model)
{
    using acgb::UnavailableProcessor;
    const int t = acgb::find_processor_type(type);
    if (t == CPU)
        return std::make_shared<UnavailableProcessor>(CPU, "the GB300 backend provides no CPU processor; use type \"cuda\"");
    if (t == OpenCL)
        return std::make_shared<UnavailableProcessor>(OpenCL, "the GB300 backend provides no OpenCL processor; use type \"cuda\"");
    acgb::ModelSpec spec;
    std::string err;
    if (!acgb::parse_model(model, spec, err)) return std::make_shared<UnavailableProcessor>(CUDA, err);
    return std::make_shared<acgb::GB300Processor>(t == -1 ? -1 : device, spec);
}

const char* Processor::listInfo() { return acgb::processor_info(CUDA); }

// The per-model factory hook: each model descriptor names the model string
// the reference's parser maps to the same network (Processor.cpp:26-187).
namespace {
std::shared_ptr<Processor> create_cuda(int idx, const std::string& model)
{
    return Processor::create("cuda", idx, model.c_str());
}
const char* const kKinds[4] = {"", "-hdn", "-box", "-box-hdn"};
}  // namespace

template<>
std::shared_ptr<Processor> Processor::create<Processor::CUDA, model::ACNetLegacy>(int idx, const model::ACNetLegacy& m)
{
    const int v = static_cast<int>(m.variant());
    return create_cuda(idx, v == 0 ? std::string("acnet-legacy-gan") : "acnet-legacy-hdn" + std::to_string(v - 1));
}
template<>
std::shared_ptr<Processor> Processor::create<Processor::CUDA, model::ACNet<8>>(int idx, const model::ACNet<8>& m)
{
    return create_cuda(idx, "acnet-f8b" + std::to_string(m.blocks()) + kKinds[static_cast<int>(m.variant()) % 4]);
}
template<>
std::shared_ptr<Processor> Processor::create<Processor::CUDA, model::ARNet<8>>(int idx, const model::ARNet<8>& m)
{
    const int k = static_cast<int>(m.variant()) % 4;
    return create_cuda(idx, std::string("arnet") + (k & 1 ? "-hdn" : "") + (k & 2 ? "-box" : "") + "-b" +
                                std::to_string(m.blocks()));
}
template<>
std::shared_ptr<Processor> Processor::create<Processor::CUDA, model::ArtCNN<16>>(int idx, const model::ArtCNN<16>& m)
{
    const char* tail[3] = {"", "-dn", "-ds"};
    return create_cuda(idx, std::string("artcnn-c4f16") + tail[static_cast<int>(m.variant())]);
}
template<>
std::shared_ptr<Processor> Processor::create<Processor::CUDA, model::ArtCNN<32>>(int idx, const model::ArtCNN<32>& m)
{
    const char* tail[3] = {"", "-dn", "-ds"};
    return create_cuda(idx, std::string("artcnn-c4f32") + tail[static_cast<int>(m.variant())]);
}
template<>
std::shared_ptr<Processor> Processor::create<Processor::CUDA, model::FSRCNNX<8>>(int idx, const model::FSRCNNX<8>& m)
{
    return create_cuda(idx, m.variant() == model::FSRCNNX<8>::Variant::B4_DISTORT_PLUS ? "fsrcnnx-f8-dp" : "fsrcnnx-f8");
}
template<>
std::shared_ptr<Processor> Processor::create<Processor::CUDA, model::FSRCNNX<16>>(int idx, const model::FSRCNNX<16>& m)
{
    return create_cuda(idx, m.variant() == model::FSRCNNX<16>::Variant::B4_DISTORT_PLUS ? "fsrcnnx-f16-dp" : "fsrcnnx-f16");
}

template<> const char* Processor::info<Processor::CPU>() { return acgb::processor_info(CPU); }
template<> const char* Processor::info<Processor::OpenCL>() { return acgb::processor_info(OpenCL); }
template<> const char* Processor::info<Processor::CUDA>() { return acgb::processor_info(CUDA); }

}  // namespace ac::core

namespace acgb {

// --------------------------------------------------------- GB300Processor

GB300Processor::GB300Processor(int device, const ModelSpec& spec) : spec_(spec)
{
    precision_ = default_precision();
    if (const char* k = std::getenv("AC_GB300_TC_KERNEL"))
    {
        const int v = std::atoi(k);
        tcKernel_ = v == 3 ? 3 : 4;
    }
    if (const char* f = std::getenv("AC_GB300_FUSED")) fused_ = std::atoi(f) != 0;
    if (const char* n = std::getenv("AC_GB300_TC3_CTAS")) tc3Ctas_ = std::atoi(n);
    if (const char* v = std::getenv("AC_GB300_TC3_SHAPE")) tc3Shape_ = std::atoi(v);
    if (tc3Shape_ >= kTc3Shapes) tc3Shape_ = -1;
    if (const char* v = std::getenv("AC_GB300_TC3_PER_SM")) tc3PerSm_ = std::atoi(v);
    if (const char* v = std::getenv("AC_GB300_AUTOTUNE")) autotune_ = std::atoi(v) != 0;
    if (const char* v = std::getenv("AC_GB300_FUSION_DEPTH")) fusionDepth_ = std::atoi(v) == 5 ? 5 : (std::atoi(v) == 9 ? 9 : 0);
    if (const char* v = std::getenv("AC_GB300_ARNET_TC")) arnetTc_ = std::atoi(v) != 0;
    phase2Ok_ = phase_weights(2, &phase2_.w[0][0]);
    int n = 0;
    cudaError_t err = cudaGetDeviceCount(&n);
    if (err != cudaSuccess || n == 0)
    {
        initError_ = std::string("no CUDA device: ") + cudaGetErrorString(err == cudaSuccess ? cudaErrorNoDevice : err);
        return;
    }
    if (device >= 0 && device < n) device_ = device;
    else
    {
        // Like the reference (CUDAProcessor.cpp:233-251), pick the device with
        // the largest SM-count x clock score.
        long best = -1;
        for (int i = 0; i < n; i++)
        {
            int clk = 0, sms = 0;
            cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, i);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, i);
            if (static_cast<long>(clk) * sms > best)
            {
                best = static_cast<long>(clk) * sms;
                device_ = i;
            }
        }
    }
    cudaDeviceProp prop{};
    err = cudaGetDeviceProperties(&prop, device_);
    if (err != cudaSuccess)
    {
        initError_ = cudaGetErrorString(err);
        return;
    }
    if (!(prop.major == 10 && prop.minor == 3))
    {
        initError_ = std::string("device ") + prop.name + " is not sm_103 (GB300); the library carries only sm_103a code";
        return;
    }
    name_ = prop.name;
    smCount_ = prop.multiProcessorCount;
    const ModelParams& mp = model_params(spec_);
    if (spec_.family == Family::ACNetLegacy)
    {
        acnet_ = std::make_unique<AcnetLegacyWeights>();
        std::memcpy(acnet_->k, mp.kernels.data(), sizeof(acnet_->k));
        std::memcpy(acnet_->b, mp.biases.data(), sizeof(acnet_->b));
    }
}

GB300Processor::~GB300Processor()
{
    std::lock_guard<std::mutex> lock(mutex_);
    if (device_ >= 0) cudaSetDevice(device_);
    for (auto& kv : states_)
    {
        ThreadState& ts = *kv.second;
        if (ts.stream) cudaStreamSynchronize(ts.stream);
        ts.src.release();
        ts.y.release();
        ts.uv.release();
        ts.la.release();
        ts.lb.release();
        ts.out.release();
        for (auto& m : ts.maps) m.release();
        ts.counter.release();
        ts.batchTmp.release();
        ts.yuvTmp.release();
        for (auto& m : ts.splitMaps) m.second.release();
        for (auto& t : ts.tables) t.second.dev.release();
        for (auto& e : ts.events) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
        for (auto& e : ts.pool) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
        for (auto& g : ts.graphs)
        {
            if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
            if (g.second.graph) cudaGraphDestroy(g.second.graph);
            if (g.second.counters) cudaFree(g.second.counters);
        }
        if (ts.stream) cudaStreamDestroy(ts.stream);
    }
    states_.clear();
    for (auto& d : deviceWeights_) d.release();
    for (auto& d : arnetPacked_) d.release();
}

Precision GB300Processor::default_precision()
{
    const char* env = std::getenv("AC_GB300_PRECISION");
    if (env)
    {
        std::string s = env;
        for (char& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
        if (s == "fp32") return Precision::FP32;
        if (s == "fp16") return Precision::FP16;
        if (s == "bf16") return Precision::BF16;
    }
    return Precision::FP32;
}

GB300Processor::ThreadState& GB300Processor::state()
{
    std::lock_guard<std::mutex> lock(mutex_);
    auto& slot = states_[std::this_thread::get_id()];
    if (!slot) slot = std::make_unique<ThreadState>();
    return *slot;
}

bool GB300Processor::ok() noexcept
{
    if (!initError_.empty()) return false;
    return state().ok;
}

const char* GB300Processor::error() noexcept
{
    if (!initError_.empty()) return initError_.c_str();
    return state().err.c_str();
}

const char* GB300Processor::name() const noexcept { return name_.empty() ? "unavailable" : name_.c_str(); }

bool GB300Processor::fail(ThreadState& ts, const std::string& what, cudaError_t err)
{
    ts.ok = false;
    ts.err = what;
    if (err != cudaSuccess)
    {
        ts.err += ": ";
        ts.err += cudaGetErrorString(err);
        cudaGetLastError();  // clear a non-sticky error for the next call
    }
    return false;
}

bool GB300Processor::begin(ThreadState& ts)
{
    ts.ok = true;
    ts.err = "NO ERROR";
    if (!initError_.empty()) return fail(ts, initError_);
    cudaError_t err = cudaSetDevice(device_);
    if (err != cudaSuccess) return fail(ts, "cudaSetDevice", err);
    if (!ts.stream)
    {
        err = cudaStreamCreateWithFlags(&ts.stream, cudaStreamNonBlocking);
        if (err != cudaSuccess) return fail(ts, "cudaStreamCreate", err);
    }
    return true;
}

const ResizeAxis* GB300Processor::axis(ThreadState& ts, int n_in, int n_out, int mode, cudaStream_t stream, cudaError_t& err)
{
    auto key = std::make_tuple(n_in, n_out, mode);
    auto it = ts.tables.find(key);
    if (it != ts.tables.end()) return &it->second.axis;
    AxisTable t;
    make_axis_table(n_in, n_out, mode, t.first, t.w, t.taps);
    size_t fb = sizeof(int) * t.first.size();
    size_t wb = sizeof(float) * t.w.size();
    size_t off = (fb + 255) & ~static_cast<size_t>(255);
    err = t.dev.ensure(off + wb);
    if (err != cudaSuccess) return nullptr;
    err = cudaMemcpyAsync(t.dev.ptr, t.first.data(), fb, cudaMemcpyHostToDevice, stream);
    if (err != cudaSuccess) return nullptr;
    err = cudaMemcpyAsync(static_cast<char*>(t.dev.ptr) + off, t.w.data(), wb, cudaMemcpyHostToDevice, stream);
    if (err != cudaSuccess) return nullptr;
    // The host vectors must outlive the asynchronous copies: they live in the cache.
    t.axis.first = static_cast<const int*>(t.dev.ptr);
    t.axis.w = reinterpret_cast<const float*>(static_cast<char*>(t.dev.ptr) + off);
    t.axis.taps = t.taps;
    auto res = ts.tables.emplace(key, std::move(t));
    return &res.first->second.axis;
}

std::pair<cudaEvent_t, cudaEvent_t> GB300Processor::profileBegin(ThreadState& ts, cudaStream_t stream)
{
    std::pair<cudaEvent_t, cudaEvent_t> ev{nullptr, nullptr};
    if (!profiling_) return ev;
    if (ts.pool.empty())
    {
        cudaEventCreate(&ev.first);
        cudaEventCreate(&ev.second);
    }
    else
    {
        ev = ts.pool.back();
        ts.pool.pop_back();
    }
    cudaEventRecord(ev.first, stream);
    return ev;
}

void GB300Processor::profileEnd(ThreadState& ts, std::pair<cudaEvent_t, cudaEvent_t> ev, cudaStream_t stream, double outPixels)
{
    if (!ev.first) return;
    cudaEventRecord(ev.second, stream);
    ts.events.push_back(ev);
    ts.eventPixels.push_back(outPixels);
}

cudaError_t GB300Processor::luma_pass(ThreadState& ts, const Plane& in, const Plane& out, const Phase2* ph, cudaStream_t stream)
{
    const std::pair<cudaEvent_t, cudaEvent_t> ev = profileBegin(ts, stream);
    cudaError_t err = cudaErrorNotSupported;
    if (spec_.family == Family::ARNet && precision_ != Precision::FP32 && arnetTc_)
    {
        // tensor-core form: 8->8 layers on tcgen05, 16-bit maps between layers
        const bool bf16 = precision_ == Precision::BF16;
        const void* w = arnetWeights(bf16);
        const size_t bytes = static_cast<size_t>(in.w) * in.h * 16;
        void* maps[3];
        err = w ? cudaSuccess : cudaErrorMemoryAllocation;
        for (int i = 0; i < 3 && err == cudaSuccess; i++)
        {
            err = ts.maps[i].ensure(bytes);
            maps[i] = ts.maps[i].ptr;
        }
        int* status = tc_status_buffer();
        if (err == cudaSuccess && !status) err = cudaErrorMemoryAllocation;
        if (err == cudaSuccess)
        {
            const ModelParams& mp = model_params(spec_);
            err = launch_arnet_tc(mp.kernels.data(), mp.biases.data(), mp.alphas.data(), spec_.blocks, w, bf16, in, out, maps,
                                  status, stream);
        }
    }
    else if (spec_.family == Family::ARNet)
    {
        // the plain FP32 layer pipeline
        const size_t bytes = static_cast<size_t>(in.w) * in.h * 8 * sizeof(float);
        float* maps[4];
        for (int i = 0; i < 4; i++)
        {
            if ((err = ts.maps[i].ensure(bytes)) != cudaSuccess) return err;
            maps[i] = static_cast<float*>(ts.maps[i].ptr);
        }
        const ModelParams& mp = model_params(spec_);
        err = launch_arnet_fp32(mp.kernels.data(), mp.biases.data(), mp.alphas.data(), spec_.blocks, in, out, maps, stream);
    }
    else if (spec_.family == Family::FSRCNNX && spec_.channels == 8 && spec_.blocks == 4 && precision_ != Precision::FP32 &&
             arnetTc_)
    {
        // FSRCNNX<8>: the 8->8 layers on the two-layer tcgen05 conv, 16-bit maps
        const bool bf16 = precision_ == Precision::BF16;
        const void* w = arnetWeights(bf16);
        const size_t bytes = static_cast<size_t>(in.w) * in.h * 16;
        void* maps[3];
        err = w ? cudaSuccess : cudaErrorMemoryAllocation;
        for (int i = 0; i < 3 && err == cudaSuccess; i++)
        {
            err = ts.maps[i].ensure(bytes);
            maps[i] = ts.maps[i].ptr;
        }
        int* status = tc_status_buffer();
        if (err == cudaSuccess && !status) err = cudaErrorMemoryAllocation;
        if (err == cudaSuccess)
        {
            const ModelParams& mp = model_params(spec_);
            err = launch_fsrcnnx8_tc(mp.kernels.data(), mp.biases.data(), mp.alphas.data(), w, bf16, in, out, maps, status, stream);
        }
    }
    else if ((spec_.family == Family::ArtCNN || (spec_.family == Family::FSRCNNX && spec_.channels == 16)) &&
             precision_ != Precision::FP32 && arnetTc_)
    {
        // tensor-core form: the 3x3 F->F layers on tcgen05, F-channel 16-bit maps
        const bool bf16 = precision_ == Precision::BF16;
        const void* w = arnetWeights(bf16);
        const size_t bytes = static_cast<size_t>(in.w) * in.h * spec_.channels * 2;
        void* maps[3];
        err = w ? cudaSuccess : cudaErrorMemoryAllocation;
        for (int i = 0; i < 3 && err == cudaSuccess; i++)
        {
            err = ts.maps[i].ensure(bytes);
            maps[i] = ts.maps[i].ptr;
        }
        int* status = tc_status_buffer();
        if (err == cudaSuccess && !status) err = cudaErrorMemoryAllocation;
        if (err == cudaSuccess)
        {
            const ModelParams& mp = model_params(spec_);
            err = launch_f3_tc(mp.kernels.data(), mp.biases.data(), mp.alphas.empty() ? nullptr : mp.alphas.data(),
                               spec_.family == Family::ArtCNN, spec_.channels, spec_.blocks, w, bf16, in, out, maps, status,
                               stream);
        }
    }
    else if (spec_.family == Family::ArtCNN || spec_.family == Family::FSRCNNX)
    {
        // the plain FP32 layer pipeline (FP32 form)
        const size_t bytes = static_cast<size_t>(in.w) * in.h * spec_.channels * sizeof(float);
        float* maps[3];
        for (int i = 0; i < 3; i++)
        {
            if ((err = ts.maps[i].ensure(bytes)) != cudaSuccess) return err;
            maps[i] = static_cast<float*>(ts.maps[i].ptr);
        }
        const ModelParams& mp = model_params(spec_);
        err = spec_.family == Family::ArtCNN
                  ? launch_artcnn_fp32(mp.kernels.data(), mp.biases.data(), spec_.channels, spec_.blocks, in, out, maps, stream)
                  : launch_fsrcnnx_fp32(mp.kernels.data(), mp.biases.data(), mp.alphas.data(), spec_.channels, spec_.blocks, in,
                                        out, maps, stream);
    }
    else if (spec_.family == Family::ACNet8)
    {
        const ModelParams& mp = model_params(spec_);
        if (acnet8Quad())
        {
            // B4 / B8: every layer in the persistent quad kernel (with the fused colour path)
            const bool bf16 = precision_ == Precision::BF16;
            const void* w = tcWeights(precision_, 3);
            if (!w) err = cudaErrorMemoryAllocation;
            else if ((err = ts.counter.ensure(256)) == cudaSuccess)
            {
                int* counter = static_cast<int*>(ts.counter.ptr) + (ts.counterSlot & 62);
                ts.counterSlot += 2;
                const int perSm = tc3PerSm_ > 0 ? tc3PerSm_ : 2;
                ts.lastPlan = LastPlan{5, 0, perSm, acn8Depth()};
                err = launchAcn8(ts, acn8Depth(), 1, &in, &out, ph, w, bf16, counter, stream, perSm);
            }
        }
        else if (precision_ != Precision::FP32 && arnetTc_)
        {
            // tensor-core form: the 8->8 layers on tcgen05, 16-bit maps between layers
            const bool bf16 = precision_ == Precision::BF16;
            const void* w = arnetWeights(bf16);
            const size_t bytes = static_cast<size_t>(in.w) * in.h * 16;
            void* maps[2];
            err = w ? cudaSuccess : cudaErrorMemoryAllocation;
            for (int i = 0; i < 2 && err == cudaSuccess; i++)
            {
                err = ts.maps[i].ensure(bytes);
                maps[i] = ts.maps[i].ptr;
            }
            int* status = tc_status_buffer();
            if (err == cudaSuccess && !status) err = cudaErrorMemoryAllocation;
            if (err == cudaSuccess)
                err = launch_acnet8_tc(mp.kernels.data(), mp.biases.data(), mp.alphas.data(), spec_.blocks, w, bf16, in, out,
                                       maps, status, stream);
        }
        else
        {
            const size_t bytes = static_cast<size_t>(in.w) * in.h * 8 * sizeof(float);
            float* maps[2];
            for (int i = 0; i < 2; i++)
            {
                if ((err = ts.maps[i].ensure(bytes)) != cudaSuccess) return err;
                maps[i] = static_cast<float*>(ts.maps[i].ptr);
            }
            err = launch_acnet8_fp32(mp.kernels.data(), mp.biases.data(), mp.alphas.data(), spec_.blocks, in, out, maps,
                                     stream);
        }
    }
    else if (spec_.family == Family::ACNetLegacy)
    {
        if (precision_ == Precision::FP32) err = launch_acnet_legacy_fp32(*acnet_, in, out, ph, stream);
        else
        {
            const bool bf16 = precision_ == Precision::BF16;
            if (tcKernel_ == 4)
            {
                // persistent quad form: tile shape, CTAs per SM and fusion depth autotuned
                const void* w = tcWeights(precision_, 3);
                if (!w) err = cudaErrorMemoryAllocation;
                else if ((err = ts.counter.ensure(256)) == cudaSuccess)
                {
                    // two counters (the split network's two launches)
                    int* counter = static_cast<int*>(ts.counter.ptr) + (ts.counterSlot & 62);
                    ts.counterSlot += 2;
                    bool ran = false;
                    const Tc3Plan plan =
                        tc3Plan(1, &in, &out, ph, w, bf16, counter, stream, ran, err, true, splitMapFor(ts, stream));
                    ts.lastPlan = LastPlan{4, plan.shape, plan.perSm, plan.depth};
                    if (err == cudaSuccess && !ran) err = launchQuad(ts, plan, 1, &in, &out, ph, w, bf16, counter, stream);
                }
            }
            else
            {
                // persistent pair form (AC_GB300_TC_KERNEL=3), autotuned tile shapes
                const void* w = tcWeights(precision_, 2);
                if (!w) err = cudaErrorMemoryAllocation;
                else if ((err = ts.counter.ensure(256)) == cudaSuccess)
                {
                    // 64 counter slots used in turn: launches in flight on
                    // different streams of one thread get different counters
                    int* counter = static_cast<int*>(ts.counter.ptr) + (ts.counterSlot++ & 63);
                    bool ran = false;
                    const Tc3Plan plan = tc3Plan(1, &in, &out, ph, w, bf16, counter, stream, ran, err);
                    ts.lastPlan = LastPlan{3, plan.shape, plan.perSm, 9};
                    if (err == cudaSuccess && !ran)
                        err = launch_acnet_legacy_tc3(*acnet_, w, bf16, 1, &in, &out, ph, counter,
                                                      tc3Ctas_ > 0 ? tc3Ctas_ : smCount_, stream, plan.shape, plan.perSm);
                }
            }
        }
    }
    profileEnd(ts, ev, stream, static_cast<double>(out.w) * out.h);
    return err;
}

void GB300Processor::setProfiling(bool on) { profiling_ = on; }

GB300Processor::LastPlan GB300Processor::lastPlan() { return state().lastPlan; }

int GB300Processor::collectProfile(double& ms, int& launches, double& outPixels)
{
    ThreadState& ts = state();
    ms = 0.0;
    outPixels = 0.0;
    launches = static_cast<int>(ts.events.size());
    for (size_t i = 0; i < ts.events.size(); i++)
    {
        auto& e = ts.events[i];
        if (cudaEventSynchronize(e.second) != cudaSuccess) return -1;
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, e.first, e.second) != cudaSuccess) return -1;
        ms += t;
        outPixels += ts.eventPixels[i];
        ts.pool.push_back(e);
    }
    ts.events.clear();
    ts.eventPixels.clear();
    return 0;
}

const void* GB300Processor::arnetWeights(bool bf16)
{
    std::lock_guard<std::mutex> lock(mutex_);
    DeviceBuffer& d = arnetPacked_[bf16 ? 1 : 0];
    if (!d.ptr)
    {
        const ModelParams& mp = model_params(spec_);
        if (spec_.family == Family::FSRCNNX && spec_.channels == 8)
        {
            // FSRCNNX<8>: its four 3x3 8->8 layers (after the 5x5 head's 200 weights)
            std::vector<uint16_t> packed(static_cast<size_t>(spec_.blocks) * 1536);
            for (int l = 0; l < spec_.blocks; l++)
                pack_pair_conv8(mp.kernels.data() + 200 + 576 * l, bf16, packed.data() + static_cast<size_t>(l) * 1536);
            if (d.ensure(packed.size() * sizeof(uint16_t)) != cudaSuccess) return nullptr;
            if (cudaMemcpy(d.ptr, packed.data(), packed.size() * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess)
            {
                d.release();
                return nullptr;
            }
            return d.ptr;
        }
        if (spec_.family == Family::ArtCNN || spec_.family == Family::FSRCNNX)
        {
            // the 3x3 F->F layers of the wide families
            std::vector<uint16_t> packed;
            pack_f3_tc_weights(mp.kernels.data(), spec_.channels, spec_.family == Family::ArtCNN, spec_.blocks, bf16, packed);
            if (d.ensure(packed.size() * sizeof(uint16_t)) != cudaSuccess) return nullptr;
            if (cudaMemcpy(d.ptr, packed.data(), packed.size() * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess)
            {
                d.release();
                return nullptr;
            }
            return d.ptr;
        }
        // the 3x3 8->8 layers: two per ARNet block, one per ACNet<8> block
        const int layers = spec_.family == Family::ARNet ? 2 * spec_.blocks : spec_.blocks;
        std::vector<uint16_t> packed(static_cast<size_t>(layers) * 1536);
        for (int l = 1; l <= layers; l++)
            pack_pair_conv8(mp.kernels.data() + 72 + 576 * (l - 1), bf16, packed.data() + static_cast<size_t>(l - 1) * 1536);
        if (d.ensure(packed.size() * sizeof(uint16_t)) != cudaSuccess) return nullptr;
        if (cudaMemcpy(d.ptr, packed.data(), packed.size() * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess)
        {
            d.release();
            return nullptr;
        }
    }
    return d.ptr;
}

const void* GB300Processor::tcWeights(Precision p, int form)
{
    const bool bf16 = p == Precision::BF16;
    const int idx = 2 * form + (bf16 ? 1 : 0);
    std::lock_guard<std::mutex> lock(mutex_);
    if (!deviceWeights_[idx].ptr)
    {
        std::vector<uint16_t> packed;
        if (form == 3 && spec_.family == Family::ACNet8)
            pack_acnet8_tc4_weights(model_params(spec_).kernels.data(), spec_.blocks, bf16, packed);
        else if (form == 3) pack_acnet_tc4_weights(*acnet_, bf16, packed);
        else if (form == 2) pack_acnet_tc3_weights(*acnet_, bf16, packed);
        else return nullptr;
        if (deviceWeights_[idx].ensure(packed.size() * sizeof(uint16_t)) != cudaSuccess) return nullptr;
        if (cudaMemcpy(deviceWeights_[idx].ptr, packed.data(), packed.size() * sizeof(uint16_t), cudaMemcpyHostToDevice) !=
            cudaSuccess)
        {
            deviceWeights_[idx].release();
            return nullptr;
        }
    }
    return deviceWeights_[idx].ptr;
}

static std::atomic<uint64_t> g_graph_replays{0};
uint64_t graph_replays() { return g_graph_replays.load(); }

static int ilog2(double v)
{
    int k = 0;
    while (v >= 2.0 && k < 62) v *= 0.5, k++;
    return k;
}

size_t GB300Processor::splitMapBytes(int n, const Plane* in)
{
    size_t b = 0;
    for (int i = 0; i < n; i++) b += acnet_tc4_split_map_bytes(in[i].w, in[i].h);
    return b;
}

// ACNet<8> B8 runs split at layer 5 unless AC_GB300_FUSION_DEPTH=9: the
// split was faster for one 1080p RGB frame (0.199 against 0.220 ms) and for
// eight (1.338 against 1.586 ms), with the same bytes.
int GB300Processor::acn8Depth() const { return spec_.blocks == 8 && fusionDepth_ != 9 ? 5 : 9; }

cudaError_t GB300Processor::launchAcn8(ThreadState& ts, int depth, int n, const Plane* in, const Plane* out, const Phase2* ph,
                                       const void* w, bool bf16, int* counter, cudaStream_t stream, int perSm)
{
    const ModelParams& mp = model_params(spec_);
    const int ctas = tc3Ctas_ > 0 ? tc3Ctas_ : smCount_;
    DeviceBuffer* maps = depth != 9 ? splitMapFor(ts, stream) : nullptr;
    if (maps)
    {
        cudaError_t err = maps->ensure(splitMapBytes(n, in));
        if (err != cudaSuccess) return err;
        return launch_acnet8_tc4_split(mp.biases.data(), mp.alphas.data(), spec_.blocks, w, bf16, n, in, out, ph, maps->ptr,
                                       counter, ctas, stream, perSm);
    }
    return launch_acnet8_tc4(mp.biases.data(), mp.alphas.data(), spec_.blocks, w, bf16, n, in, out, ph, counter, ctas, stream,
                             perSm);
}

DeviceBuffer* GB300Processor::splitMapFor(ThreadState& ts, cudaStream_t stream)
{
    auto it = ts.splitMaps.find(stream);
    if (it != ts.splitMaps.end()) return &it->second;
    if (ts.splitMaps.size() >= 16) return nullptr;
    return &ts.splitMaps[stream];
}

cudaError_t GB300Processor::launchQuad(ThreadState& ts, const Tc3Plan& plan, int n, const Plane* in, const Plane* out,
                                       const Phase2* ph, const void* w, bool bf16, int* counter, cudaStream_t stream)
{
    const int ctas = tc3Ctas_ > 0 ? tc3Ctas_ : smCount_;
    DeviceBuffer* maps = plan.depth == 5 ? splitMapFor(ts, stream) : nullptr;
    if (maps)
    {
        cudaError_t err = maps->ensure(splitMapBytes(n, in));
        if (err != cudaSuccess) return err;
        return launch_acnet_legacy_tc4_split(*acnet_, w, bf16, n, in, out, ph, maps->ptr, counter, ctas, stream, plan.perSm);
    }
    // the whole network (also when this thread has no map buffer left for the stream)
    return launch_acnet_legacy_tc4(*acnet_, w, bf16, n, in, out, ph, counter, ctas, stream, plan.perSm,
                                   plan.depth == 5 ? 0 : plan.shape);
}

GB300Processor::Tc3Plan GB300Processor::tc3Plan(int n, const Plane* in, const Plane* out, const Phase2* ph, const void* w,
                                                bool bf16, int* counter, cudaStream_t stream, bool& ran, cudaError_t& err,
                                                bool quad, DeviceBuffer* mapBuffer)
{
    ran = false;
    err = cudaSuccess;
    Tc3Plan plan;
    if (tc3Shape_ >= 0) plan.shape = tc3Shape_;
    if (tc3PerSm_ > 0) plan.perSm = tc3PerSm_;
    if (quad && fusionDepth_ != 0) plan.depth = fusionDepth_;
    if (quad && plan.depth == 5) plan.shape = 0;  // the split network has its own tile shapes
    if (!autotune_ || tc3Shape_ >= 0 || tc3PerSm_ > 0 || (quad && fusionDepth_ != 0)) return plan;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) return plan;
    double total = 0.0, sw = 0.0, sh = 0.0;
    for (int i = 0; i < n; i++)
    {
        total += static_cast<double>(in[i].w) * in[i].h;
        sw += in[i].w;
        sh += in[i].h;
    }
    const auto key = std::make_tuple(in[0].type, in[0].channels, (bf16 ? 1 : 0) + (quad ? 2 : 0), ilog2(total), ilog2(sw / n),
                                     ilog2(sh / n));
    {
        std::lock_guard<std::mutex> lock(mutex_);
        auto it = plans_.find(key);
        if (it != plans_.end()) return it->second;
    }
    // Measure every shape x {2, 1} CTAs per SM (quad kernel: and the split
    // network x {2, 1}) with events on the launching stream.  Each candidate
    // writes the same bytes, so the output is valid afterwards.
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if ((err = cudaEventCreate(&e0)) != cudaSuccess) return plan;
    if ((err = cudaEventCreate(&e1)) != cudaSuccess)
    {
        cudaEventDestroy(e0);
        return plan;
    }
    // the split network's activation maps, only while it is a candidate
    // (an allocation failure drops the candidate)
    void* maps = nullptr;
    if (quad && mapBuffer && mapBuffer->ensure(splitMapBytes(n, in)) == cudaSuccess) maps = mapBuffer->ptr;
    const int ctas = tc3Ctas_ > 0 ? tc3Ctas_ : smCount_;
    float best = 1e30f;
    Tc3Plan bestPlan = plan;
    auto launch = [&](int shape, int perSm) {
        if (quad && shape == kTc4Shapes)
            return launch_acnet_legacy_tc4_split(*acnet_, w, bf16, n, in, out, ph, maps, counter, ctas, stream, perSm);
        return quad ? launch_acnet_legacy_tc4(*acnet_, w, bf16, n, in, out, ph, counter, ctas, stream, perSm, shape)
                    : launch_acnet_legacy_tc3(*acnet_, w, bf16, n, in, out, ph, counter, ctas, stream, shape, perSm);
    };
    // quad kernel: "shape" kTc4Shapes stands for the split network
    const int shapes = quad ? kTc4Shapes + (maps ? 1 : 0) : kTc3Shapes;
    for (int shape = 0; shape < shapes && err == cudaSuccess; shape++)
        for (int perSm = 2; perSm >= 1 && err == cudaSuccess; perSm--)
        {
            // a warm launch, then the faster of two timings of two launches
            // (candidates a few percent apart are told apart more reliably)
            err = launch(shape, perSm);
            float ms = 1e30f;
            for (int rep = 0; rep < 2 && err == cudaSuccess; rep++)
            {
                err = cudaEventRecord(e0, stream);
                for (int r = 0; r < 2 && err == cudaSuccess; r++) err = launch(shape, perSm);
                if (err == cudaSuccess) err = cudaEventRecord(e1, stream);
                if (err == cudaSuccess) err = cudaEventSynchronize(e1);
                float t = 0.0f;
                if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
                if (err == cudaSuccess && t < ms) ms = t;
            }
            if (err == cudaSuccess && ms < best)
            {
                best = ms;
                const bool split = quad && shape == kTc4Shapes;
                bestPlan.shape = split ? 0 : shape;
                bestPlan.depth = split ? 5 : 9;
                bestPlan.perSm = perSm;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return plan;
    ran = true;
    std::lock_guard<std::mutex> lock(mutex_);
    plans_[key] = bestPlan;
    return bestPlan;
}

static inline int align_pitch(int bytes) { return (bytes + 255) & ~255; }

static inline Plane plane_of(const DeviceImage& d)
{
    Plane p;
    p.ptr = d.ptr;
    p.w = d.w;
    p.h = d.h;
    p.pitch = d.stride;
    p.channels = d.c;
    p.type = d.type;
    return p;
}

bool GB300Processor::validate(ThreadState& ts, int w, int h, int c, int type, double factor)
{
    if (w <= 0 || h <= 0) return fail(ts, "empty source image");
    if (c != 1 && c != 3 && c != 4) return fail(ts, "unsupported channel count (1, 3 or 4)");
    if (type != Image::UInt8 && type != Image::UInt16 && type != Image::Float32)
        return fail(ts, "unsupported element type (u8, u16 or f32)");
    if (!(factor > 0.0) || !std::isfinite(factor) || factor > 64.0) return fail(ts, "factor must be in (0, 64]");
    int power = factor > 2.0 ? ceil_log2(factor) : 1;
    double lw = static_cast<double>(w) * (1 << power), lh = static_cast<double>(h) * (1 << power);
    if (lw * lh * c * (type & 0xff) > 2147483647.0) return fail(ts, "output image too large");
    return true;
}

bool GB300Processor::validStride(ThreadState& ts, const DeviceImage& d, const char* which)
{
    const int64_t row = static_cast<int64_t>(d.w) * d.c * (d.type & 0xff);
    if (d.stride <= 0 || static_cast<int64_t>(d.stride) < row)
        return fail(ts, std::string(which) + ": row stride must be positive and at least one row of pixels");
    if (static_cast<int64_t>(d.stride) * d.h > 2147483647) return fail(ts, std::string(which) + ": image too large");
    return true;
}

// Runs the pipeline between device images.  `dst` has the final shape.
bool GB300Processor::run(ThreadState& ts, const DeviceImage& src, const DeviceImage& dst, double factor, cudaStream_t stream)
{
    const int c = src.c, type = src.type, es = type & 0xff;
    const int power = factor > 2.0 ? ceil_log2(factor) : 1;
    const double fxy = factor / static_cast<double>(1 << power);
    const int lw = src.w << power, lh = src.h << power;
    const bool lumaResize = (dst.w != lw) || (dst.h != lh);
    cudaError_t err;

    // Fused path: RGB(A) x2 in one kernel (split, CNN, chroma resample and
    // merge), when the chroma resample is the exact x2 Catmull-Rom.
    if (c > 1 && power == 1 && fxy == 1.0 && dst.w == 2 * src.w && dst.h == 2 * src.h && fused_ &&
        (spec_.family == Family::ACNetLegacy || acnet8Quad()))
    {
        const Phase2& ph = phase2_;
        if (phase2Ok_)
        {
            bool nonzero = true;
            for (int k = 0; k < 2; k++)
                for (int t = 0; t < 4; t++) nonzero = nonzero && ph.w[k][t] != 0.0f;
            if (nonzero)
            {
                if ((err = luma_pass(ts, plane_of(src), plane_of(dst), &ph, stream)) != cudaSuccess)
                    return fail(ts, "fused upscale", err);
                return true;
            }
        }
    }

    Plane cur;
    Plane uv;
    if (c == 1) cur = plane_of(src);
    else
    {
        int yp = align_pitch(src.w * es), up = align_pitch(src.w * (c - 1) * es);
        if ((err = ts.y.ensure(static_cast<size_t>(yp) * src.h)) != cudaSuccess) return fail(ts, "device allocation", err);
        if ((err = ts.uv.ensure(static_cast<size_t>(up) * src.h)) != cudaSuccess) return fail(ts, "device allocation", err);
        Plane rgb = plane_of(src);
        cur = Plane{ts.y.ptr, src.w, src.h, yp, 1, type};
        uv = Plane{ts.uv.ptr, src.w, src.h, up, c - 1, type};
        if ((err = launch_rgb2yuv_split(rgb, cur, uv, stream)) != cudaSuccess) return fail(ts, "rgb2yuv", err);
    }
    const int lp = align_pitch(lw * es);
    DeviceBuffer* pp[2] = {&ts.la, &ts.lb};
    int which = 0;
    for (int k = 0; k < power; k++)
    {
        Plane next;
        const bool last = k == power - 1;
        if (last && !lumaResize && c == 1) next = plane_of(dst);
        else
        {
            if ((err = pp[which]->ensure(static_cast<size_t>(lp) * lh)) != cudaSuccess) return fail(ts, "device allocation", err);
            next = Plane{pp[which]->ptr, cur.w * 2, cur.h * 2, align_pitch(cur.w * 2 * es), 1, type};
            which ^= 1;
        }
        if ((err = luma_pass(ts, cur, next, nullptr, stream)) != cudaSuccess) return fail(ts, "luma pass", err);
        cur = next;
    }
    if (lumaResize)
    {
        Plane r;
        if (c == 1) r = plane_of(dst);
        else
        {
            if ((err = pp[which]->ensure(static_cast<size_t>(lp) * lh)) != cudaSuccess) return fail(ts, "device allocation", err);
            r = Plane{pp[which]->ptr, dst.w, dst.h, align_pitch(dst.w * es), 1, type};
        }
        const ResizeAxis* ax = axis(ts, cur.w, r.w, 1, stream, err);
        if (!ax) return fail(ts, "resize table", err);
        const ResizeAxis* ay = axis(ts, cur.h, r.h, 1, stream, err);
        if (!ay) return fail(ts, "resize table", err);
        if ((err = launch_resize(cur, r, *ax, *ay, stream)) != cudaSuccess) return fail(ts, "luma resize", err);
        cur = r;
    }
    if (c > 1)
    {
        const int F = (dst.w == 2 * src.w && dst.h == 2 * src.h) ? 2 : ((dst.w == 4 * src.w && dst.h == 4 * src.h) ? 4 : 0);
        float pw[16];
        if (F && phase_weights(F, pw))
        {
            if ((err = launch_merge_int(cur, uv, F, pw, plane_of(dst), stream)) != cudaSuccess) return fail(ts, "yuv2rgb", err);
            return true;
        }
        const ResizeAxis* ax = axis(ts, src.w, dst.w, 1, stream, err);
        if (!ax) return fail(ts, "resize table", err);
        const ResizeAxis* ay = axis(ts, src.h, dst.h, 1, stream, err);
        if (!ay) return fail(ts, "resize table", err);
        if ((err = launch_merge_resize(cur, uv, *ax, *ay, plane_of(dst), stream)) != cudaSuccess)
            return fail(ts, "yuv2rgb", err);
    }
    (void)fxy;
    return true;
}

void GB300Processor::processPath(const Image& src, Image& dst, double factor)
{
    ThreadState& ts = state();
    if (!begin(ts)) return;
    if (src.empty())
    {
        fail(ts, "empty source image");
        return;
    }
    if (!validate(ts, src.width(), src.height(), src.channels(), src.type(), factor)) return;
    int ow, oh;
    output_shape(src.width(), src.height(), src.channels(), factor, ow, oh);
    if (!dst.empty())
    {
        // Processor.cpp:215-229: a preallocated gray dst whose size differs
        // from the power-of-two result is reached by a final resize.
        if (src.channels() == 1 && factor / static_cast<double>(1 << (factor > 2.0 ? ceil_log2(factor) : 1)) != 1.0)
        {
            ow = dst.width();
            oh = dst.height();
        }
        if (dst.width() != ow || dst.height() != oh || dst.channels() != src.channels() || dst.type() != src.type())
        {
            fail(ts, "preallocated dst has the wrong shape or type");
            return;
        }
    }
    else
    {
        try
        {
            dst.create(ow, oh, src.channels(), src.type());
        }
        catch (...)
        {
            fail(ts, "host allocation failed");
            return;
        }
    }
    cudaStream_t stream = ts.stream;
    cudaError_t err;
    const int es = src.elementSize();
    // The device copy of the source keeps the caller's row stride when it is
    // 16-byte aligned, so the upload is one contiguous copy.
    const int srcRow = src.width() * src.pixelSize();
    const int devPitch = (src.stride() % 16 == 0 && src.stride() >= srcRow) ? src.stride() : align_pitch(srcRow);
    DeviceImage dsrc{nullptr, src.width(), src.height(), src.channels(), devPitch, src.type()};
    DeviceImage ddst{nullptr, ow, oh, src.channels(), align_pitch(ow * src.channels() * es), src.type()};
    if ((err = ts.src.ensure(static_cast<size_t>(dsrc.stride) * dsrc.h)) != cudaSuccess) { fail(ts, "device allocation", err); return; }
    if ((err = ts.out.ensure(static_cast<size_t>(ddst.stride) * ddst.h)) != cudaSuccess) { fail(ts, "device allocation", err); return; }
    dsrc.ptr = ts.src.ptr;
    ddst.ptr = ts.out.ptr;
    err = cudaMemcpy2DAsync(dsrc.ptr, dsrc.stride, src.ptr(), src.stride(), static_cast<size_t>(src.width()) * src.pixelSize(),
                            src.height(), cudaMemcpyHostToDevice, stream);
    if (err != cudaSuccess) { fail(ts, "host to device copy", err); return; }
    if (!run(ts, dsrc, ddst, factor, stream)) return;
    err = cudaMemcpy2DAsync(dst.ptr(), dst.stride(), ddst.ptr, ddst.stride, static_cast<size_t>(ow) * dst.pixelSize(), oh,
                            cudaMemcpyDeviceToHost, stream);
    if (err != cudaSuccess) { fail(ts, "device to host copy", err); return; }
    const bool tc = precision_ != Precision::FP32;
    if (tc && (err = tc_status_enqueue(stream)) != cudaSuccess) { fail(ts, "status read", err); return; }
    err = cudaStreamSynchronize(stream);
    if (err != cudaSuccess)
    {
        fail(ts, "kernel execution", err);
        return;
    }
    if (tc && tc_status_take() != 0) fail(ts, "tensor-core wait timed out");
}

int GB300Processor::processDevice(const DeviceImage& src, const DeviceImage& dst, double factor, cudaStream_t stream, bool sync)
{
    ThreadState& ts = state();
    if (!begin(ts)) return -1;
    if (!src.ptr || !dst.ptr) return fail(ts, "null device pointer"), -1;
    if (!validate(ts, src.w, src.h, src.c, src.type, factor)) return -1;
    if (!validStride(ts, src, "src") || !validStride(ts, dst, "dst")) return -1;
    int ow, oh;
    output_shape(src.w, src.h, src.c, factor, ow, oh);
    if (src.c == 1 && factor / static_cast<double>(1 << (factor > 2.0 ? ceil_log2(factor) : 1)) != 1.0)
    {
        ow = dst.w;
        oh = dst.h;
    }
    if (dst.w != ow || dst.h != oh || dst.c != src.c || dst.type != src.type) return fail(ts, "dst has the wrong shape or type"), -1;
    cudaStream_t s = stream ? stream : ts.stream;
    if (!run(ts, src, dst, factor, s)) return -1;
    if (sync)
    {
        const bool tc = precision_ != Precision::FP32;
        cudaError_t err = tc ? tc_status_enqueue(s) : cudaSuccess;
        if (err != cudaSuccess) return fail(ts, "status read", err), -1;
        if ((err = cudaStreamSynchronize(s)) != cudaSuccess) return fail(ts, "kernel execution", err), -1;
        if (tc && tc_status_take() != 0) return fail(ts, "tensor-core wait timed out"), -1;
    }
    return 0;
}

// Validated images: the batched persistent launches (ACNetLegacy x2, or x4
// of 1-channel planes as two chained batched x2 passes, in a tensor-core
// form), else image by image.
bool GB300Processor::batchRun(ThreadState& ts, int n, const DeviceImage* src, const DeviceImage* dst, double factor,
                              cudaStream_t s)
{
    const bool acn8 = acnet8Quad();
    const bool tcBatch =
        ((spec_.family == Family::ACNetLegacy && precision_ != Precision::FP32 && tcKernel_ >= 3) || acn8) && fused_;
    // ARNet, ACNet<8> B18, ArtCNN and FSRCNNX in a tensor-core form:
    // single-channel images of one element type run every layer as one launch
    // over all images
    bool layered = (((spec_.family == Family::ARNet || spec_.family == Family::ACNet8) && !acn8 &&
                     precision_ != Precision::FP32 && arnetTc_) ||
                    f3Tc()) &&
                   n > 1 && (factor == 2.0 || factor == 4.0);
    for (int i = 0; i < n && layered; i++)
        layered = src[i].c == 1 && src[i].type == src[0].type && dst[i].w == static_cast<int>(factor) * src[i].w &&
                  dst[i].h == static_cast<int>(factor) * src[i].h;
    if (layered) return layeredBatch(ts, n, src, dst, factor, s);
    bool gray4 = tcBatch && factor == 4.0 && n > 0;
    for (int i = 0; i < n && gray4; i++)
        gray4 = src[i].c == 1 && dst[i].w == 4 * src[i].w && dst[i].h == 4 * src[i].h;
    if (gray4)
    {
        // x4 of 1-channel planes: two chained batched x2 passes through
        // 2x temporaries (the reference's power-of-two pass loop)
        std::vector<DeviceImage> mid(n);
        std::vector<size_t> off(n);
        size_t total = 0;
        for (int i = 0; i < n; i++)
        {
            const int es = src[i].type & 0xff, pitch = align_pitch(2 * src[i].w * es);
            off[i] = total;
            total += (static_cast<size_t>(pitch) * 2 * src[i].h + 255) & ~static_cast<size_t>(255);
            mid[i] = DeviceImage{nullptr, 2 * src[i].w, 2 * src[i].h, 1, pitch, src[i].type};
        }
        cudaError_t err = ts.batchTmp.ensure(total);
        if (err != cudaSuccess) return fail(ts, "device allocation", err), false;
        for (int i = 0; i < n; i++) mid[i].ptr = static_cast<char*>(ts.batchTmp.ptr) + off[i];
        return batchRun(ts, n, src, mid.data(), 2.0, s) && batchRun(ts, n, mid.data(), dst, 2.0, s);
    }
    const bool batched = tcBatch && factor == 2.0;
    if (!batched)
    {
        for (int i = 0; i < n; i++)
            if (!run(ts, src[i], dst[i], factor, s)) return false;
    }
    else
    {
        const bool bf16 = precision_ == Precision::BF16;
        const bool quad = tcKernel_ == 4;
        const void* w = tcWeights(precision_, quad ? 3 : 2);
        if (!w) return fail(ts, "tensor-core weights", cudaErrorMemoryAllocation), false;
        cudaError_t err = ts.counter.ensure(256);
        if (err != cudaSuccess) return fail(ts, "device allocation", err), false;
        // two counters per launch (the split network's two launches)
        int* counter = static_cast<int*>(ts.counter.ptr) + (ts.counterSlot & 62);
        ts.counterSlot += 2;
        if (!phase2Ok_) return fail(ts, "chroma resample weights"), false;
        const Phase2& ph = phase2_;
        const int maxImages = std::min(quad ? acnet_tc4_max_images() : acnet_tc3_max_images(), 64);
        std::vector<int> order(n);
        for (int i = 0; i < n; i++) order[i] = i;
        // groups of one channel count and element type, in chunks of at most 64 images
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            return std::make_pair(src[a].c, src[a].type) < std::make_pair(src[b].c, src[b].type);
        });
        Plane in[64], out[64];
        for (int g0 = 0; g0 < n;)
        {
            int g1 = g0;
            while (g1 < n && g1 - g0 < maxImages && src[order[g1]].c == src[order[g0]].c &&
                   src[order[g1]].type == src[order[g0]].type)
                g1++;
            const int m = g1 - g0;
            uint64_t sig = 1469598103934665603ull;  // FNV-1a over the launch's arguments
            auto mix = [&sig](uint64_t v) {
                for (int b = 0; b < 8; b++) sig = (sig ^ ((v >> (8 * b)) & 0xff)) * 1099511628211ull;
            };
            mix(static_cast<uint64_t>(m));
            mix(static_cast<uint64_t>(bf16));
            mix(reinterpret_cast<uint64_t>(w));
            for (int j = 0; j < m; j++)
            {
                const DeviceImage& a = src[order[g0 + j]];
                const DeviceImage& b = dst[order[g0 + j]];
                in[j] = plane_of(a);
                out[j] = plane_of(b);
                mix(reinterpret_cast<uint64_t>(a.ptr));
                mix(reinterpret_cast<uint64_t>(b.ptr));
                mix((static_cast<uint64_t>(a.w) << 32) | static_cast<uint32_t>(a.h));
                mix((static_cast<uint64_t>(a.stride) << 32) | static_cast<uint32_t>(b.stride));
                mix((static_cast<uint64_t>(a.c) << 32) | static_cast<uint32_t>(a.type));
            }
            const Phase2* php = in[0].channels > 1 ? &ph : nullptr;
            bool ran = false;
            Tc3Plan plan;
            if (acn8)
            {
                plan.perSm = tc3PerSm_ > 0 ? tc3PerSm_ : 2;  // one tile shape per ACNet<8> depth
                plan.depth = acn8Depth();
                if (plan.depth != 9 && (err = splitMapFor(ts, s) ? splitMapFor(ts, s)->ensure(splitMapBytes(m, in))
                                                                 : cudaErrorMemoryAllocation) != cudaSuccess)
                    return fail(ts, "device allocation", err), false;
            }
            else plan = tc3Plan(m, in, out, php, w, bf16, counter, s, ran, err, quad, splitMapFor(ts, s));
            if (err != cudaSuccess) return fail(ts, "batched upscale", err), false;
            // the split network's maps exist before a capture begins
            DeviceBuffer* maps = quad && plan.depth == 5 ? splitMapFor(ts, s) : nullptr;
            if (maps && (err = maps->ensure(splitMapBytes(m, in))) != cudaSuccess)
                return fail(ts, "device allocation", err), false;
            if (quad && plan.depth == 5 && !maps)
            {
                plan.depth = 9;  // no map buffer for this stream: the whole network
                plan.shape = 0;
            }
            ts.lastPlan = LastPlan{acn8 ? 5 : (quad ? 4 : 3), plan.shape, plan.perSm, plan.depth};
            mix(static_cast<uint64_t>(plan.shape * 4 + plan.perSm));
            mix(static_cast<uint64_t>(plan.depth));
            mix(reinterpret_cast<uint64_t>(maps && plan.depth == 5 ? maps->ptr : nullptr));
            mix(static_cast<uint64_t>(quad));
            const int ctas = tc3Ctas_ > 0 ? tc3Ctas_ : smCount_;
            auto launchGroup = [&]() {
                if (acn8) return launchAcn8(ts, plan.depth, m, in, out, php, w, bf16, counter, s, plan.perSm);
                return quad ? launchQuad(ts, plan, m, in, out, php, w, bf16, counter, s)
                            : launch_acnet_legacy_tc3(*acnet_, w, bf16, m, in, out, php, counter, ctas, s, plan.shape,
                                                      plan.perSm);
            };
            cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
            if ((err = cudaStreamIsCapturing(s, &cap)) != cudaSuccess) return fail(ts, "stream state", err), false;
            auto git = ts.graphs.find(sig);
            // kernel timing of this group's launch (the measuring launches of
            // a first-seen batch class are not timed)
            double groupPixels = 0.0;
            for (int j = 0; j < m; j++) groupPixels += static_cast<double>(out[j].w) * out[j].h;
            const std::pair<cudaEvent_t, cudaEvent_t> ev =
                ran ? std::pair<cudaEvent_t, cudaEvent_t>{nullptr, nullptr} : profileBegin(ts, s);
            if (ran)
            {
            }
            else if (cap == cudaStreamCaptureStatusNone && git != ts.graphs.end())
            {
                // the same batch again: replay its graph (memset + persistent kernel)
                if ((err = cudaGraphLaunch(git->second.exec, s)) != cudaSuccess) return fail(ts, "graph launch", err), false;
                count_launch(git->second.kernels);
                g_graph_replays++;
            }
            else if (cap == cudaStreamCaptureStatusNone && ts.seen.count(sig) && ts.graphs.size() < 64)
            {
                // second sighting: capture the launch into a graph, then replay it
                GraphEntry ge;
                if ((err = cudaMalloc(&ge.counters, 2 * sizeof(int))) != cudaSuccess)
                    return fail(ts, "device allocation", err), false;
                if ((err = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
                {
                    cudaFree(ge.counters);
                    return fail(ts, "stream capture", err), false;
                }
                int* const ringCounter = counter;
                counter = ge.counters;  // launchGroup reads `counter`
                const cudaError_t lerr = launchGroup();
                counter = ringCounter;
                ge.kernels = plan.depth != 9 && (quad || acn8) ? 2 : 1;  // the split network: two kernels
                err = cudaStreamEndCapture(s, &ge.graph);
                if (lerr != cudaSuccess || err != cudaSuccess)
                {
                    if (ge.graph) cudaGraphDestroy(ge.graph);
                    cudaFree(ge.counters);
                    return fail(ts, "stream capture", lerr != cudaSuccess ? lerr : err), false;
                }
                if ((err = cudaGraphInstantiate(&ge.exec, ge.graph, 0)) != cudaSuccess)
                {
                    cudaGraphDestroy(ge.graph);
                    cudaFree(ge.counters);
                    return fail(ts, "graph instantiation", err), false;
                }
                ts.graphs[sig] = ge;
                if ((err = cudaGraphLaunch(ge.exec, s)) != cudaSuccess) return fail(ts, "graph launch", err), false;
                g_graph_replays++;
            }
            else
            {
                if (ts.seen.size() >= 4096) ts.seen.clear();
                ts.seen[sig] = 1;
                if ((err = launchGroup()) != cudaSuccess) return fail(ts, "batched upscale", err), false;
            }
            profileEnd(ts, ev, s, groupPixels);
            g0 = g1;
        }
    }
    return true;
}

bool GB300Processor::layeredBatch(ThreadState& ts, int n, const DeviceImage* src, const DeviceImage* dst, double factor,
                                  cudaStream_t s)
{
    const int per = spec_.family == Family::ACNet8 ? 2 : 3;  // work maps per image
    // bytes per map pixel: 8 16-bit channels, or F for ArtCNN / FSRCNNX<16>
    const bool wide = (spec_.family == Family::ArtCNN || spec_.family == Family::FSRCNNX) && spec_.channels > 8;
    const size_t bpp = wide ? static_cast<size_t>(spec_.channels) * 2 : 16;
    const bool bf16 = precision_ == Precision::BF16;
    const void* w = arnetWeights(bf16);
    int* status = tc_status_buffer();
    if (!w || !status) return fail(ts, "tensor-core weights", cudaErrorMemoryAllocation), false;
    const ModelParams& mp = model_params(spec_);
    // x4: x2 into temporaries, then x2 into dst (the reference's power-of-two pass loop)
    std::vector<DeviceImage> mid;
    if (factor == 4.0)
    {
        mid.resize(n);
        std::vector<size_t> off(n);
        size_t total = 0;
        for (int i = 0; i < n; i++)
        {
            const int es = src[i].type & 0xff, pitch = align_pitch(2 * src[i].w * es);
            off[i] = total;
            total += (static_cast<size_t>(pitch) * 2 * src[i].h + 255) & ~static_cast<size_t>(255);
            mid[i] = DeviceImage{nullptr, 2 * src[i].w, 2 * src[i].h, 1, pitch, src[i].type};
        }
        cudaError_t err = ts.batchTmp.ensure(total);
        if (err != cudaSuccess) return fail(ts, "device allocation", err), false;
        for (int i = 0; i < n; i++) mid[i].ptr = static_cast<char*>(ts.batchTmp.ptr) + off[i];
    }
    for (int pass = 0; pass < (factor == 4.0 ? 2 : 1); pass++)
    {
        const DeviceImage* a = pass == 0 ? src : mid.data();
        const DeviceImage* b = (factor == 4.0 && pass == 0) ? mid.data() : dst;
        for (int g0 = 0; g0 < n; g0 += kArnetTcMaxImages)
        {
            const int m = std::min(n - g0, kArnetTcMaxImages);
            std::vector<Plane> in(m), out(m);
            std::vector<size_t> moff(m);
            size_t mapBytes = 0;
            for (int j = 0; j < m; j++)
            {
                in[j] = plane_of(a[g0 + j]);
                out[j] = plane_of(b[g0 + j]);
                moff[j] = mapBytes;
                mapBytes += (static_cast<size_t>(in[j].w) * in[j].h * bpp + 255) & ~static_cast<size_t>(255);
            }
            std::vector<void*> maps(static_cast<size_t>(per) * m);
            for (int k = 0; k < per; k++)
            {
                cudaError_t err = ts.maps[k].ensure(mapBytes);
                if (err != cudaSuccess) return fail(ts, "device allocation", err), false;
                for (int j = 0; j < m; j++) maps[static_cast<size_t>(per) * j + k] = static_cast<char*>(ts.maps[k].ptr) + moff[j];
            }
            double px = 0.0;
            for (int j = 0; j < m; j++) px += static_cast<double>(out[j].w) * out[j].h;
            const std::pair<cudaEvent_t, cudaEvent_t> ev = profileBegin(ts, s);
            const float* al = mp.alphas.empty() ? nullptr : mp.alphas.data();
            cudaError_t err;
            if (spec_.family == Family::ARNet)
                err = launch_arnet_tc_batch(mp.kernels.data(), mp.biases.data(), al, spec_.blocks, w, bf16, m, in.data(),
                                            out.data(), maps.data(), status, s);
            else if (spec_.family == Family::ACNet8)
                err = launch_acnet8_tc_batch(mp.kernels.data(), mp.biases.data(), al, spec_.blocks, w, bf16, m, in.data(),
                                             out.data(), maps.data(), status, s);
            else if (!wide)
                err = launch_fsrcnnx8_tc_batch(mp.kernels.data(), mp.biases.data(), al, w, bf16, m, in.data(), out.data(),
                                               maps.data(), status, s);
            else
                err = launch_f3_tc_batch(mp.kernels.data(), mp.biases.data(), al, spec_.family == Family::ArtCNN,
                                         spec_.channels, spec_.blocks, w, bf16, m, in.data(), out.data(), maps.data(), status,
                                         s);
            profileEnd(ts, ev, s, px);
            if (err != cudaSuccess) return fail(ts, "batched upscale", err), false;
        }
    }
    return true;
}

int GB300Processor::processBatchDevice(int n, const DeviceImage* src, const DeviceImage* dst, double factor, cudaStream_t stream,
                                       bool sync)
{
    ThreadState& ts = state();
    if (!begin(ts)) return -1;
    if (n < 0 || (n > 0 && (!src || !dst))) return fail(ts, "batch: bad image arrays"), -1;
    cudaStream_t s = stream ? stream : ts.stream;
    for (int i = 0; i < n; i++)
    {
        if (!src[i].ptr || !dst[i].ptr) return fail(ts, "null device pointer"), -1;
        if (!validate(ts, src[i].w, src[i].h, src[i].c, src[i].type, factor)) return -1;
        if (!validStride(ts, src[i], "src") || !validStride(ts, dst[i], "dst")) return -1;
        int ow, oh;
        output_shape(src[i].w, src[i].h, src[i].c, factor, ow, oh);
        if (src[i].c == 1 && factor / static_cast<double>(1 << (factor > 2.0 ? ceil_log2(factor) : 1)) != 1.0)
        {
            ow = dst[i].w;
            oh = dst[i].h;
        }
        if (dst[i].w != ow || dst[i].h != oh || dst[i].c != src[i].c || dst[i].type != src[i].type)
            return fail(ts, "dst has the wrong shape or type"), -1;
    }
    if (!batchRun(ts, n, src, dst, factor, s)) return -1;
    if (sync)
    {
        const bool tc = precision_ != Precision::FP32;
        cudaError_t err = tc ? tc_status_enqueue(s) : cudaSuccess;
        if (err != cudaSuccess) return fail(ts, "status read", err), -1;
        if ((err = cudaStreamSynchronize(s)) != cudaSuccess) return fail(ts, "kernel execution", err), -1;
        if (tc && tc_status_take() != 0) return fail(ts, "tensor-core wait timed out"), -1;
    }
    return 0;
}

int GB300Processor::processYuvDevice(int frames, int planes, const DeviceImage* src, const DeviceImage* dst, double factor,
                                     int shift, cudaStream_t stream, bool sync)
{
    ThreadState& ts = state();
    if (!begin(ts)) return -1;
    if (frames < 1 || planes < 1 || planes > 4 || !src || !dst) return fail(ts, "yuv: bad frame arrays"), -1;
    if (shift < 0 || shift > 15) return fail(ts, "yuv: shift must be in [0, 15]"), -1;
    cudaStream_t s = stream ? stream : ts.stream;
    std::vector<DeviceImage> ys(frames), yd(frames);
    size_t tmpBytes = 0;
    std::vector<size_t> tmpOff(frames);
    for (int f = 0; f < frames; f++)
    {
        const DeviceImage& y = src[f * planes];
        const DeviceImage& oy = dst[f * planes];
        if (!y.ptr || !oy.ptr) return fail(ts, "null device pointer"), -1;
        if (y.c != 1 || oy.c != 1) return fail(ts, "yuv: plane 0 (Y) must have one channel"), -1;
        if (!validate(ts, y.w, y.h, 1, y.type, factor)) return -1;
        if (!validStride(ts, y, "src Y plane") || !validStride(ts, oy, "dst Y plane")) return -1;
        int ow, oh;
        output_shape(y.w, y.h, 1, factor, ow, oh);
        if (factor / static_cast<double>(1 << (factor > 2.0 ? ceil_log2(factor) : 1)) != 1.0)
        {
            ow = oy.w;
            oh = oy.h;
        }
        if (oy.w != ow || oy.h != oh || oy.type != y.type) return fail(ts, "dst Y plane has the wrong shape or type"), -1;
        if (shift && y.type != Image::UInt8 && y.type != Image::UInt16)
            return fail(ts, "yuv: a shift needs an integer element type"), -1;
        for (int p = 1; p < planes; p++)
        {
            const DeviceImage& a = src[f * planes + p];
            const DeviceImage& b = dst[f * planes + p];
            if (!a.ptr || !b.ptr) return fail(ts, "null device pointer"), -1;
            if (a.type != y.type || b.type != y.type || a.c != b.c || a.c < 1 || a.c > 4 || a.w <= 0 || a.h <= 0 ||
                b.w <= 0 || b.h <= 0)
                return fail(ts, "yuv: chroma planes need Y's element type, 1 to 4 channels and a size"), -1;
            if (!validStride(ts, a, "src chroma plane") || !validStride(ts, b, "dst chroma plane")) return -1;
        }
        ys[f] = y;
        yd[f] = oy;
        tmpOff[f] = tmpBytes;
        const int pitch = align_pitch(y.w * (y.type & 0xff));
        tmpBytes += (static_cast<size_t>(pitch) * y.h + 255) & ~static_cast<size_t>(255);
    }
    cudaError_t err;
    if (shift > 0)
    {
        // shl into temporaries (the caller's source planes stay untouched)
        if ((err = ts.yuvTmp.ensure(tmpBytes)) != cudaSuccess) return fail(ts, "device allocation", err), -1;
        for (int f = 0; f < frames; f++)
        {
            DeviceImage t = ys[f];
            t.ptr = static_cast<char*>(ts.yuvTmp.ptr) + tmpOff[f];
            t.stride = align_pitch(t.w * (t.type & 0xff));
            if ((err = launch_shift(plane_of(ys[f]), plane_of(t), shift, s)) != cudaSuccess) return fail(ts, "shl", err), -1;
            ys[f] = t;
        }
    }
    if (!batchRun(ts, frames, ys.data(), yd.data(), factor, s)) return -1;
    for (int f = 0; f < frames; f++)
    {
        if (shift > 0 && (err = launch_shift(plane_of(yd[f]), plane_of(yd[f]), -shift, s)) != cudaSuccess)
            return fail(ts, "shr", err), -1;
        for (int p = 1; p < planes; p++)
        {
            const DeviceImage& a = src[f * planes + p];
            const DeviceImage& b = dst[f * planes + p];
            // exactly x2 / x4 (4:2:0 chroma of a x2 / x4 frame): the phase-table kernel
            const int F = (b.w == 2 * a.w && b.h == 2 * a.h) ? 2 : ((b.w == 4 * a.w && b.h == 4 * a.h) ? 4 : 0);
            float pw[16];
            if (F && phase_weights(F, pw))
            {
                if ((err = launch_resize_int(plane_of(a), plane_of(b), F, pw, s)) != cudaSuccess)
                    return fail(ts, "chroma resize", err), -1;
                continue;
            }
            const ResizeAxis* ax = axis(ts, a.w, b.w, 1, s, err);
            if (!ax) return fail(ts, "resize table", err), -1;
            const ResizeAxis* ay = axis(ts, a.h, b.h, 1, s, err);
            if (!ay) return fail(ts, "resize table", err), -1;
            if ((err = launch_resize(plane_of(a), plane_of(b), *ax, *ay, s)) != cudaSuccess)
                return fail(ts, "chroma resize", err), -1;
        }
    }
    if (sync)
    {
        const bool tc = precision_ != Precision::FP32;
        if (tc && (err = tc_status_enqueue(s)) != cudaSuccess) return fail(ts, "status read", err), -1;
        if ((err = cudaStreamSynchronize(s)) != cudaSuccess) return fail(ts, "kernel execution", err), -1;
        if (tc && tc_status_take() != 0) return fail(ts, "tensor-core wait timed out"), -1;
    }
    return 0;
}

// The allocation-free batch entry.  Its success path allocates no device or
// host memory: the tile queue lives in the persistent kernel's static
// scratch, the weights must already be resident (an ordinary call in the
// same precision uploaded them), and the per-thread error record is only
// touched when it exists already or a call fails.
int GB300Processor::processDeviceNoAlloc(int n, const DeviceImage* src, const DeviceImage* dst, cudaStream_t stream, bool sync)
{
    auto failed = [&](const std::string& what, cudaError_t err = cudaSuccess) {
        fail(state(), what, err);
        return -1;
    };
    auto rejected = [&](const std::string& what) {
        fail(state(), what);
        return -2;
    };
    if (!initError_.empty()) return failed(initError_);
    if (spec_.family != Family::ACNetLegacy || precision_ == Precision::FP32)
        return rejected("allocation-free call: needs an ACNetLegacy model in the FP16 or BF16 form");
    const int maxImages = std::min(acnet_tc3_max_images(), 64);  // the Plane tables below
    if (n < 1 || n > maxImages || !src || !dst)
        return rejected("allocation-free call: " + std::to_string(n) + " images in one call; 1 to " + std::to_string(maxImages) +
                      " are allowed");
    const int c = src[0].c, type = src[0].type, es = type & 0xff;
    if (c != 1 && c != 3 && c != 4) return rejected("unsupported channel count (1, 3 or 4)");
    if (type != Image::UInt8 && type != Image::UInt16 && type != Image::Float32)
        return rejected("unsupported element type (u8, u16 or f32)");
    Plane in[64], out[64];
    for (int i = 0; i < n; i++)
    {
        const DeviceImage& a = src[i];
        const DeviceImage& b = dst[i];
        if (!a.ptr || !b.ptr) return rejected("null device pointer");
        if (a.c != c || a.type != type || b.c != c || b.type != type)
            return rejected("allocation-free call: every image needs the first image's channel count and element type");
        if (a.w <= 0 || a.h <= 0 || b.w != 2 * a.w || b.h != 2 * a.h)
            return rejected("allocation-free call: every dst must be exactly 2x its src");
        if (a.stride <= 0 || b.stride <= 0 || static_cast<int64_t>(a.stride) < static_cast<int64_t>(a.w) * c * es ||
            static_cast<int64_t>(b.stride) < static_cast<int64_t>(b.w) * c * es)
            return rejected("stride smaller than a row");
        if (static_cast<int64_t>(b.stride) * b.h > 2147483647 || static_cast<int64_t>(a.stride) * a.h > 2147483647)
            return rejected("image too large");
        in[i] = plane_of(a);
        out[i] = plane_of(b);
    }
    if (c > 1 && !phase2Ok_) return failed("chroma resample weights");
    const Phase2& ph = phase2_;
    const bool bf16 = precision_ == Precision::BF16;
    const void* w = nullptr;
    {
        std::lock_guard<std::mutex> lock(mutex_);
        w = deviceWeights_[(tcKernel_ == 4 ? 6 : 4) + (bf16 ? 1 : 0)].ptr;
    }
    if (!w)
        return rejected("allocation-free call: the tensor-core weights of this precision are not on the device yet; make one "
                      "ordinary process call in this precision first");
    cudaError_t err = cudaSetDevice(device_);
    if (err != cudaSuccess) return failed("cudaSetDevice", err);
    // the persistent kernel the ordinary entry runs (quad or pair form)
    err = tcKernel_ == 4 ? launch_acnet_legacy_tc4_noalloc(*acnet_, w, bf16, n, in, out, c > 1 ? &ph : nullptr,
                                                           tc3Ctas_ > 0 ? tc3Ctas_ : smCount_, stream)
                         : launch_acnet_legacy_tc3_noalloc(*acnet_, w, bf16, n, in, out, c > 1 ? &ph : nullptr,
                                                           tc3Ctas_ > 0 ? tc3Ctas_ : smCount_, stream);
    if (err != cudaSuccess) return failed("allocation-free upscale", err);
    if (sync)
    {
        if ((err = cudaStreamSynchronize(stream)) != cudaSuccess) return failed("kernel execution", err);
        int status = 0;
        if ((err = acnet_tc3_noalloc_status(&status)) != cudaSuccess) return failed("status read", err);
        if (status != 0) return failed("tensor-core wait timed out");
    }
    {
        std::lock_guard<std::mutex> lock(mutex_);
        auto it = states_.find(std::this_thread::get_id());
        if (it != states_.end() && it->second)
        {
            it->second->ok = true;
            it->second->err = "NO ERROR";
        }
    }
    return 0;
}

}  // namespace acgb
