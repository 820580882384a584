// Internal definition of the GPU processor (shared by processor.cpp and the
// C ABI translation unit).
#pragma once

#include <atomic>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "processor.hpp"

namespace acgb {

int ceil_log2(double v);
void make_axis_table(int n_in, int n_out, int mode, std::vector<int>& first, std::vector<float>& weights, int& taps);
bool phase_weights(int F, float* w);
// CUDA graphs of batched launches replayed in this process so far.
uint64_t graph_replays();

// Grow-only device allocation.  Outgrown blocks are kept (not freed while
// work may run) until release().
struct DeviceBuffer
{
    void* ptr = nullptr;
    size_t cap = 0;
    std::vector<void*> retired;
    cudaError_t ensure(size_t bytes);
    void release();
};
// Device allocations made by DeviceBuffer::ensure and the serving pool in
// this process (diagnostics of the serving loop).
std::atomic<uint64_t>& device_alloc_count();
// Fault injection: make the nth next device allocation fail (0 disarms);
// injected_alloc_failure() is asked before every such allocation.
void arm_alloc_failure(int nth);
bool injected_alloc_failure();

class GB300Processor final : public Processor
{
public:
    GB300Processor(int device, const ModelSpec& spec);
    ~GB300Processor() override;

    bool ok() noexcept override;
    const char* error() noexcept override;
    const char* name() const noexcept override;
    int type() const noexcept override { return CUDA; }
    const char* typeName() const noexcept override { return "CUDA"; }

    // Device-pointer entry: src/dst already in HBM; work is queued on
    // `stream` (the calling thread's own stream when null).  Returns 0 or -1
    // (details through ok()/error()).
    int processDevice(const DeviceImage& src, const DeviceImage& dst, double factor, cudaStream_t stream, bool sync);

    // Processor::process over n device images.  ACNetLegacy x2 in a
    // tensor-core form runs each group of images with one channel count and
    // element type as ONE persistent launch (tile shape and CTAs per SM from
    // the autotuner; a repeated identical batch replays a captured CUDA
    // graph); anything else runs image by image.  Returns 0 or -1.
    int processBatchDevice(int n, const DeviceImage* src, const DeviceImage* dst, double factor, cudaStream_t stream, bool sync);

    // The reference CLI's video recipe over `frames` planar frames of
    // `planes` planes (src[f * planes + p]): Y shifted left by `shift`,
    // upscaled (batched over the frames) and shifted back; the other planes
    // resized to their dst sizes with Catmull-Rom.  Returns 0 or -1.
    int processYuvDevice(int frames, int planes, const DeviceImage* src, const DeviceImage* dst, double factor, int shift,
                         cudaStream_t stream, bool sync);

    // Allocation-free x2 of n device images in one persistent tensor-core
    // launch on `stream` (ACNetLegacy, FP16/BF16 form).  Returns 0, -1 when
    // the work failed, -2 when the request was rejected.
    int processDeviceNoAlloc(int n, const DeviceImage* src, const DeviceImage* dst, cudaStream_t stream, bool sync);

    // Kernel timing of the luma passes with CUDA events recorded on the
    // launching stream around each launch (for roofline figures).
    void setProfiling(bool on);
    int collectProfile(double& ms, int& launches, double& outPixels);

    void setPrecision(Precision p) { precision_ = p; }
    // Off: the persistent kernel runs its default plan instead of measuring
    // one the first time a batch class is seen (no measurement launches in a
    // latency-sensitive request path).
    void setAutotune(bool on) { autotune_ = on; }
    // Caps the CTAs per SM of this processor's persistent launches (0: the
    // plan's own); the serving loop runs large jobs at one per SM, so a
    // small job's blocks always find room on every SM.
    void setCtasPerSm(int n) { tc3PerSm_ = n > 0 ? n : 0; }
    Precision precision() const { return precision_; }
    int device() const { return device_; }
    const ModelSpec& spec() const { return spec_; }

protected:
    void processPath(const Image& src, Image& dst, double factor) override;

private:
    struct AxisTable
    {
        std::vector<int> first;
        std::vector<float> w;
        int taps = 0;
        DeviceBuffer dev;
        ResizeAxis axis;
    };
    struct Tc3Plan
    {
        int shape = 0;  // tile geometry of the persistent kernel
        int perSm = 2;  // CTAs per SM (cap)
        int depth = 9;  // quad kernel: layers fused per launch, 9 (one launch) or 5 (split 5 + 4)
    };
    struct GraphEntry
    {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        int kernels = 1;  // kernel launches a replay runs
        // the graph's own two tile counters: a replay may run beside the
        // thread's direct launches on other streams, which take counters
        // from the ring
        int* counters = nullptr;
    };
public:
    // The persistent launch plan of the calling thread's most recent
    // tensor-core call: kernel 4 quad (ACNetLegacy), 3 pair, 5 quad
    // (ACNet<8>), 0 none; tile shape index; CTAs per SM.
    struct LastPlan
    {
        int kernel = 0, shape = 0, perSm = 0, depth = 9;
    };
    LastPlan lastPlan();

private:
    struct ThreadState
    {
        LastPlan lastPlan;
        cudaStream_t stream = nullptr;
        DeviceBuffer src, y, uv, la, lb, out;
        DeviceBuffer maps[4];  // ARNet feature maps
        DeviceBuffer counter;  // 64 tile-queue counters of the persistent kernel, used in turn
        unsigned counterSlot = 0;
        DeviceBuffer batchTmp; // x2 intermediates of batched x4 passes
        DeviceBuffer yuvTmp;   // shifted Y planes of the YUV path
        // 16-bit activation maps of the split quad network, one buffer per
        // stream: calls on different streams may run at once, as the whole
        // network's launches may
        std::map<cudaStream_t, DeviceBuffer> splitMaps;
        std::map<std::tuple<int, int, int>, AxisTable> tables;
        bool ok = true;
        std::string err = "NO ERROR";
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> events;  // recorded pairs
        std::vector<double> eventPixels;                           // output pixels per pair
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pool;     // free pairs
        std::unordered_map<uint64_t, GraphEntry> graphs;           // captured batches by signature
        std::unordered_map<uint64_t, int> seen;                    // batch signatures launched directly so far
    };

    static Precision default_precision();
    ThreadState& state();
    bool begin(ThreadState& ts);
    bool fail(ThreadState& ts, const std::string& what, cudaError_t err = cudaSuccess);
    bool validate(ThreadState& ts, int w, int h, int c, int type, double factor);
    // A caller's device image: row stride positive and at least one row of
    // w * c elements (computed in 64 bits), the last row's end addressable
    // in the int byte offsets the kernels use.
    bool validStride(ThreadState& ts, const DeviceImage& d, const char* which);
    bool run(ThreadState& ts, const DeviceImage& src, const DeviceImage& dst, double factor, cudaStream_t stream);
    const ResizeAxis* axis(ThreadState& ts, int n_in, int n_out, int mode, cudaStream_t stream, cudaError_t& err);
    cudaError_t luma_pass(ThreadState& ts, const Plane& in, const Plane& out, const Phase2* ph, cudaStream_t stream);
    // Kernel timing (setProfiling): an event pair recorded around one launch
    // on its stream, with the output pixels it produced.
    std::pair<cudaEvent_t, cudaEvent_t> profileBegin(ThreadState& ts, cudaStream_t stream);
    void profileEnd(ThreadState& ts, std::pair<cudaEvent_t, cudaEvent_t> ev, cudaStream_t stream, double outPixels);
    // Packed tensor-core weights on the device: form 0 one pixel per row, 1
    // pair-interleaved (per-tile kernel), 2 persistent kernel, 3 persistent
    // quad kernel.
    const void* tcWeights(Precision p, int form);
    const void* arnetWeights(bool bf16);  // packed 8->8 layers of the ARNet / ACNet<8> tensor-core forms
    // ArtCNN / FSRCNNX in a tensor-core form (FSRCNNX<8>: B4, the 8-channel path)
    bool f3Tc() const
    {
        return (spec_.family == Family::ArtCNN ||
                (spec_.family == Family::FSRCNNX && (spec_.channels == 16 || (spec_.channels == 8 && spec_.blocks == 4)))) &&
               precision_ != Precision::FP32 && arnetTc_;
    }
    // ACNet<8> B4 / B8 in a tensor-core form run the quad kernel (fused colour path, batching)
    bool acnet8Quad() const
    {
        return spec_.family == Family::ACNet8 && precision_ != Precision::FP32 && arnetTc_ && tcKernel_ == 4 &&
               acnet8_tc4_supported(spec_.blocks);
    }
    bool batchRun(ThreadState& ts, int n, const DeviceImage* src, const DeviceImage* dst, double factor, cudaStream_t s);
    // ARNet / ACNet<8> tensor-core forms over n single-channel images, x2 or
    // x4: each layer one launch over every image (up to kArnetTcMaxImages).
    bool layeredBatch(ThreadState& ts, int n, const DeviceImage* src, const DeviceImage* dst, double factor, cudaStream_t s);
    // Tile shape and CTAs per SM for a persistent launch of the pair kernel
    // or (quad) the quad kernel over these images: forced by
    // AC_GB300_TC3_SHAPE / AC_GB300_TC3_PER_SM, else measured once per batch
    // class (kernel, element type, channels, form, log2 of the total and mean
    // image sizes) over every tile shape x {2, 1} CTAs per SM.  When it
    // measured, the launches already produced the output (`ran`).
    Tc3Plan tc3Plan(int n, const Plane* in, const Plane* out, const Phase2* ph, const void* w, bool bf16, int* counter,
                    cudaStream_t stream, bool& ran, cudaError_t& err, bool quad = false, DeviceBuffer* maps = nullptr);
    // The quad kernel's launch under `plan` (whole network, or split in two
    // launches over the stream's map buffer); `counter` points at two device
    // ints.
    cudaError_t launchQuad(ThreadState& ts, const Tc3Plan& plan, int n, const Plane* in, const Plane* out,
                           const Phase2* ph, const void* w, bool bf16, int* counter, cudaStream_t stream);
    static size_t splitMapBytes(int n, const Plane* in);
    // ACNet<8> in the quad kernel: the whole network (depth 9) or, for B8,
    // split in two launches at layer 5 (depth 5, AC_GB300_FUSION_DEPTH=5)
    int acn8Depth() const;
    cudaError_t launchAcn8(ThreadState& ts, int depth, int n, const Plane* in, const Plane* out, const Phase2* ph,
                           const void* w, bool bf16, int* counter, cudaStream_t stream, int perSm);
    // The split network's map buffer of `stream` (null when the thread
    // already holds buffers for 16 other streams: the split is then not used).
    static DeviceBuffer* splitMapFor(ThreadState& ts, cudaStream_t stream);

    int device_ = -1;
    int smCount_ = 0;
    ModelSpec spec_;
    std::string name_;
    std::string initError_;
    Precision precision_ = Precision::FP32;
    bool profiling_ = false;
    std::unique_ptr<AcnetLegacyWeights> acnet_;
    DeviceBuffer deviceWeights_[8];  // TC weights: {one-pixel, pair, persistent, quad} x {FP16, BF16}
    DeviceBuffer arnetPacked_[2];    // ARNet / ACNet<8> 8->8 layers, pair form: FP16, BF16
    bool arnetTc_ = true;            // ARNet / ACNet<8> tensor-core form in FP16/BF16 (AC_GB300_ARNET_TC=0: FP32 pipeline)
    int tc3Ctas_ = 0;                // CTAs of the persistent kernel (0: one per SM; AC_GB300_TC3_CTAS)
    bool fused_ = true;              // RGB(A) x2 in one fused kernel (AC_GB300_FUSED=0 disables)
    int tcKernel_ = 4;               // tensor-core kernel: 4 persistent quad (default), 3 persistent pair, 2 pair-interleaved per tile, 1 one-pixel-per-row (AC_GB300_TC_KERNEL)
    int tc3Shape_ = -1;              // forced tile shape (AC_GB300_TC3_SHAPE), -1: autotuned
    int tc3PerSm_ = 0;               // forced CTAs per SM (AC_GB300_TC3_PER_SM), 0: autotuned
    int fusionDepth_ = 0;            // forced quad-kernel fusion depth (AC_GB300_FUSION_DEPTH: 9 or 5), 0: autotuned
    bool autotune_ = true;           // AC_GB300_AUTOTUNE=0: default shape, two CTAs per SM
    std::map<std::tuple<int, int, int, int, int, int>, Tc3Plan> plans_;
    // x2 Catmull-Rom phase weights of the fused chroma resample, computed
    // once at construction (the allocation-free entry must not build them)
    Phase2 phase2_{};
    bool phase2Ok_ = false;
    std::mutex mutex_;
    std::unordered_map<std::thread::id, std::unique_ptr<ThreadState>> states_;
};

}  // namespace acgb
