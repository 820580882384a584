// Host-side launch interface of the CUDA kernels (no torch types, plain
// pointers and sizes).  All planes live in device memory.
#pragma once

#include <atomic>
#include <cstdint>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

namespace acgb {

// A device image plane: `channels` interleaved elements per pixel.
struct Plane
{
    void* ptr = nullptr;
    int w = 0, h = 0;
    int pitch = 0;     // bytes between rows
    int channels = 1;
    int type = 0x001;  // ElemType
};

// ACNetLegacy parameters in the reference's NHWC layout
// (core/include/AC/Core/Model/ACNet.hpp:34-60): 8*9 + 8*8*9*8 + 8*4 kernel
// floats, 8 + 8*8 bias floats.
constexpr int kAcnetKernels = 8 * 9 + 8 * 8 * 9 * 8 + 8 * 4;
constexpr int kAcnetBiases = 8 + 8 * 8;
// One-time launch set-up of a kernel (function attributes, CTAs per SM, SM
// count), computed once per device by device_once.
struct LaunchSetup
{
    cudaError_t err;
    int per_sm;
    int sms;
};

// Runs f for each device it is called on (the current device) until it
// succeeds once, and returns that device's successful result afterwards.
// Function attributes such as the dynamic shared-memory limit are per device,
// so a process that launches on several GPUs sets them on each.  A failed
// set-up is not cached: the next call on that device runs f again, so a
// transient error does not disable the kernel for the life of the process.
// Thread-safe (one lock per device; f runs under it); F is the call site's
// lambda, so every call site and template instance has its own table.
constexpr int kMaxDevices = 64;
inline bool setup_succeeded(cudaError_t e) { return e == cudaSuccess; }
inline bool setup_succeeded(const LaunchSetup& s) { return s.err == cudaSuccess; }
template <typename F>
auto device_once(F f) -> decltype(f())
{
    using R = decltype(f());
    static std::mutex locks[kMaxDevices];
    static std::atomic<bool> done[kMaxDevices];
    static R values[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return f();
    if (done[dev].load(std::memory_order_acquire)) return values[dev];
    std::lock_guard<std::mutex> lock(locks[dev]);
    if (done[dev].load(std::memory_order_relaxed)) return values[dev];
    const R r = f();
    if (setup_succeeded(r))
    {
        values[dev] = r;
        done[dev].store(true, std::memory_order_release);
    }
    return r;
}

struct AcnetLegacyWeights
{
    float k[kAcnetKernels];
    float b[kAcnetBiases];
};

// Separable resampling table for one axis: for output index o, taps
// first[o] .. first[o] + taps - 1 (clamped to the source) with weights
// w[o * taps + t]; zero weights are skipped.
struct ResizeAxis
{
    const int* first = nullptr;
    const float* w = nullptr;
    int taps = 0;
};

// Catmull-Rom weights of an exact x2 upscale by output phase (even, odd):
// even outputs take source taps i-2 .. i+1, odd outputs i-1 .. i+2.
struct Phase2
{
    float w[2][4];
};

// Plain FP32 layer-fused ACNetLegacy x2 pass: in (1 ch) -> out (1 ch, 2w x 2h),
// same element type; or, for a 3/4-channel RGB(A) input, the fused
// split/CNN/chroma/merge pass writing RGB(A) (phase2 required).
cudaError_t launch_acnet_legacy_fp32(const AcnetLegacyWeights& wts, const Plane& in, const Plane& out, const Phase2* phase2,
                                     cudaStream_t stream);

// Timeout status word of the tensor-core kernels (tc_status.cpp): the
// calling thread's word on the current device, 0 or 1 after a bounded wait
// gave up.  tc_status_enqueue(s) queues its copy to a pinned host slot and
// its reset on stream s; after s synchronised, tc_status_take() returns the
// copied value (-1 when nothing was queued).  tc_status_reset() reads and
// clears it synchronously.
int* tc_status_buffer();
cudaError_t tc_status_enqueue(cudaStream_t stream);
int tc_status_take();
int tc_status_reset();

// Persistent warp-specialised tensor-core form over a tile queue of n images
// (same type and channel count, every output 2x its input); packed2 is the
// device copy of pack_acnet_tc3_weights() (nine layers, layer 0 included).  `counter` is a device int (zeroed by the call
// on `stream`); `ctas` = SMs' worth of CTAs to launch.
// `shape` picks the tile geometry (0: 48x44, 1: 64x31, 2: 32x63; the same
// bytes come out of each) and `per_sm_cap` caps the CTAs per SM (1 or 2).
constexpr int kTc3Shapes = 3;
void pack_acnet_tc3_weights(const AcnetLegacyWeights& wts, bool bf16, std::vector<uint16_t>& packed);
int acnet_tc3_max_images();
void acnet_tc3_shape(int shape, int* tw, int* th);
cudaError_t launch_acnet_legacy_tc3(const AcnetLegacyWeights& wts, const void* packed2, bool bf16, int n, const Plane* in,
                                    const Plane* out, const Phase2* phase2, int* counter, int ctas, cudaStream_t stream,
                                    int shape = 0, int per_sm_cap = 2);
// The same launch with its tile counter and status word in a static device
// array of that file (256 bytes): no allocation; concurrent calls on one
// device race.  acnet_tc3_noalloc_status reads its status word (0, or 1
// after a timed-out wait) once the stream has synchronised.
cudaError_t launch_acnet_legacy_tc3_noalloc(const AcnetLegacyWeights& wts, const void* packed2, bool bf16, int n,
                                            const Plane* in, const Plane* out, const Phase2* phase2, int ctas,
                                            cudaStream_t stream);
cudaError_t acnet_tc3_noalloc_status(int* value);

// Quad form of the persistent kernel: four pixels per GEMM row (N = 32),
// B matrices streamed per layer; `packed4` is the device copy of
// pack_acnet_tc4_weights().  Three tile shapes (`shape` 0: 46x46 in a 64x64
// window, the default; 1: 62x33 in 80x51; 2: 30x67 in 48x85), every one
// computing each output pixel from the same window with the same arithmetic
// (identical bytes).  Same arguments and output contract as
// launch_acnet_legacy_tc3 (results agree within the FP16/BF16 tolerance; the
// MMA accumulation order differs).
constexpr int kTc4Shapes = 3;
int acnet_tc4_max_images();
void acnet_tc4_shape(int shape, int* tw, int* th);
void pack_acnet_tc4_weights(const AcnetLegacyWeights& wts, bool bf16, std::vector<uint16_t>& packed);
cudaError_t launch_acnet_legacy_tc4(const AcnetLegacyWeights& wts, const void* packed4, bool bf16, int n, const Plane* in,
                                    const Plane* out, const Phase2* phase2, int* counter, int ctas, cudaStream_t stream,
                                    int per_sm_cap = 2, int shape = 0);
// The network in two launches, split at layer 5 (fusion depth 5 + 4): the
// head writes layer 4's 16-bit activations to one map per image in `maps`
// (acnet_tc4_split_map_bytes(w, h) each, in image order, 256-byte aligned),
// the tail reads them and runs layers 5 .. 8 and the colour merge; the same
// bytes as the whole-network launch.  counters: two device ints.
size_t acnet_tc4_split_map_bytes(int w, int h);
void acnet_tc4_split_tail_shape(int* tw, int* th);
cudaError_t launch_acnet_legacy_tc4_split(const AcnetLegacyWeights& wts, const void* packed4, bool bf16, int n,
                                          const Plane* in, const Plane* out, const Phase2* phase2, void* maps,
                                          int* counters, int ctas, cudaStream_t stream, int per_sm_cap);
// The same with the caller's status word (`status`, 0 or 1 after a timed-out wait).
cudaError_t launch_acnet_legacy_tc4_core(const AcnetLegacyWeights& wts, const void* packed4, bool bf16, int n, const Plane* in,
                                         const Plane* out, const Phase2* phase2, int* counter, int* status, int ctas,
                                         cudaStream_t stream, int per_sm_cap, int shape = 0);
// ACNet<8> with 4 or 8 blocks in the quad kernel (PReLU layers, conv3x3
// 8 -> 4 pixel-shuffle tail with the nearest-source add; fused colour path as
// for ACNetLegacy).  `packed4` is the device copy of pack_acnet8_tc4_weights();
// biases / alphas in the reference layout (8 + 8 blocks + 4 / 8 (blocks + 1)).
bool acnet8_tc4_supported(int blocks);
void acnet8_tc4_shape(int blocks, int* tw, int* th);
void acnet8_tc4_split_tail_shape(int* tw, int* th);
void pack_acnet8_tc4_weights(const float* kernels, int blocks, bool bf16, std::vector<uint16_t>& packed);
cudaError_t launch_acnet8_tc4(const float* biases, const float* alphas, int blocks, const void* packed4, bool bf16, int n,
                              const Plane* in, const Plane* out, const Phase2* phase2, int* counter, int ctas,
                              cudaStream_t stream, int per_sm_cap = 2);
// ACNet<8> B8 split in two launches at layer 5 (the head writes block 4's
// activations to one 16-bit map per image in `maps`, acnet_tc4_split_map_bytes
// each); the same bytes as launch_acnet8_tc4.  counters: two device ints.
cudaError_t launch_acnet8_tc4_split(const float* biases, const float* alphas, int blocks, const void* packed4, bool bf16, int n,
                                    const Plane* in, const Plane* out, const Phase2* phase2, void* maps, int* counters, int ctas,
                                    cudaStream_t stream, int per_sm_cap);
// The quad launch with its tile counter and status word in the static
// scratch of the allocation-free entry (see launch_acnet_legacy_tc3_noalloc).
cudaError_t launch_acnet_legacy_tc4_noalloc(const AcnetLegacyWeights& wts, const void* packed4, bool bf16, int n,
                                            const Plane* in, const Plane* out, const Phase2* phase2, int ctas,
                                            cudaStream_t stream);

// RGB(A) -> Y + UV(A) (rgb2yuv / rgba2yuva of core/src/ImageProcess.cpp).
cudaError_t launch_rgb2yuv_split(const Plane& rgb, const Plane& y, const Plane& uv, cudaStream_t stream);
// Interleaved 3/4-channel RGB(A) -> interleaved YUV(A) in place or not.
cudaError_t launch_rgb2yuv_packed(const Plane& rgb, const Plane& yuv, cudaStream_t stream);
cudaError_t launch_yuv2rgb_packed(const Plane& yuv, const Plane& rgb, cudaStream_t stream);

// Y (full size) + UV(A) at any size, resampled on the fly to Y's size with
// the given tables, then yuv2rgb / yuva2rgba into rgb.
cudaError_t launch_merge_resize(const Plane& y, const Plane& uv, ResizeAxis ax, ResizeAxis ay, const Plane& rgb,
                                cudaStream_t stream);

// ARNet<8> x2 pass in plain FP32 (one kernel per layer): parameters in the
// reference blob layout (ARNet.hpp:26-70), `blocks` residual blocks, four
// [h][w][8] float work maps of the input size.
cudaError_t launch_arnet_fp32(const float* kernels, const float* biases, const float* alphas, int blocks, const Plane& in,
                              const Plane& out, float* const maps[4], cudaStream_t stream);

// ARNet<8> x2 pass in the tensor-core form: the 2*blocks 3x3 8->8 layers on
// tcgen05 (FP16 or BF16 operands, FP32 accumulation, 16-bit maps between
// layers), the head and the upscale layer in FP32.  `packed`: device copy of
// 2*blocks pack_pair_conv8 layers (3 KB each); maps: three [h][w] arrays of
// 16-byte pixels; `status` as tc_status_buffer().
void pack_pair_conv8(const float* k576, bool bf16, uint16_t* out /* 1536 values */);
cudaError_t launch_arnet_tc(const float* kernels, const float* biases, const float* alphas, int blocks, const void* packed,
                            bool bf16, const Plane& in, const Plane& out, void* const maps[3], int* status,
                            cudaStream_t stream);
// The same for n single-channel images at once (1 to kArnetTcMaxImages, one
// element type, each output 2x its input): every layer is one launch over all
// images' tiles; maps[3 i + j] are image i's three work maps.
constexpr int kArnetTcMaxImages = 16;
cudaError_t launch_arnet_tc_batch(const float* kernels, const float* biases, const float* alphas, int blocks, const void* packed,
                                  bool bf16, int n, const Plane* in, const Plane* out, void* const* maps, int* status,
                                  cudaStream_t stream);

// ACNet<8> x2 pass (head conv 1->8 + PReLU, `blocks` conv 8->8 + PReLU, conv
// 8->4 + pixel shuffle + nearest input; ACNet.hpp:63-116).  Plain FP32 with
// two [h][w][8] float maps, or the tensor-core form with `blocks` packed 8->8
// layers and two [h][w] arrays of 16-byte pixels.
cudaError_t launch_acnet8_fp32(const float* kernels, const float* biases, const float* alphas, int blocks, const Plane& in,
                               const Plane& out, float* const maps[2], cudaStream_t stream);
cudaError_t launch_acnet8_tc(const float* kernels, const float* biases, const float* alphas, int blocks, const void* packed,
                             bool bf16, const Plane& in, const Plane& out, void* const maps[2], int* status,
                             cudaStream_t stream);
// n images at once (as launch_arnet_tc_batch); maps[2 i + j].
cudaError_t launch_acnet8_tc_batch(const float* kernels, const float* biases, const float* alphas, int blocks,
                                   const void* packed, bool bf16, int n, const Plane* in, const Plane* out,
                                   void* const* maps, int* status, cudaStream_t stream);

// FSRCNNX<8> in a tensor-core form (k_arnet_tc.cu): FP32 5x5 head
// (launch_f3_head8), the 3x3 8->8 layers as two two-layer tcgen05 launches,
// FP32 upscale.  packed: 4 x pack_pair_conv8; maps: three w*h*16-byte arrays.
cudaError_t launch_f3_head8(const float* kernels, const float* biases, bool bf16, int n, const Plane* in, void* const* feat,
                            cudaStream_t stream);
cudaError_t launch_fsrcnnx8_tc(const float* kernels, const float* biases, const float* alphas, const void* packed, bool bf16,
                               const Plane& in, const Plane& out, void* const maps[3], int* status, cudaStream_t stream);
// The same over n <= 16 single-channel images (maps[3 i + j]), every layer one launch.
cudaError_t launch_fsrcnnx8_tc_batch(const float* kernels, const float* biases, const float* alphas, const void* packed, bool bf16,
                                     int n, const Plane* in, const Plane* out, void* const* maps, int* status, cudaStream_t stream);
// ArtCNN<F> (F = 16, 32) and FSRCNNX<F> (F = 8, 16) x2 passes in plain FP32
// (one kernel per layer; parameters in the reference blob layout,
// ArtCNN.hpp:44-56, FSRCNNX.hpp:46-66); maps: three [h][w][F] float arrays.
cudaError_t launch_artcnn_fp32(const float* kernels, const float* biases, int F, int blocks, const Plane& in, const Plane& out,
                               float* const maps[3], cudaStream_t stream);
cudaError_t launch_fsrcnnx_fp32(const float* kernels, const float* biases, const float* alphas, int F, int blocks,
                                const Plane& in, const Plane& out, float* const maps[3], cudaStream_t stream);
// Their tensor-core form for F = 16 or 32 (ArtCNN<16/32>, FSRCNNX<16>): the
// 3x3 F->F layers on tcgen05 (one pixel per GEMM row, N = F), head and
// upscale FP32, F-channel 16-bit maps.  `packed`: device copy of
// pack_f3_tc_weights(); maps: three [h][w][F] 16-bit arrays.
void pack_f3_tc_weights(const float* kernels, int F, bool artcnn, int blocks, bool bf16, std::vector<uint16_t>& packed);
cudaError_t launch_f3_tc(const float* kernels, const float* biases, const float* alphas, bool artcnn, int F, int blocks,
                         const void* packed, bool bf16, const Plane& in, const Plane& out, void* const maps[3], int* status,
                         cudaStream_t stream);
// The same over n <= 16 single-channel images of one element type, every
// layer one launch over all of them; maps[3 i + j] holds image i's maps.
cudaError_t launch_f3_tc_batch(const float* kernels, const float* biases, const float* alphas, bool artcnn, int F, int blocks,
                               const void* packed, bool bf16, int n, const Plane* in, const Plane* out, void* const* maps,
                               int* status, cudaStream_t stream);

// Merge for chroma resampled by exactly `factor` (2 or 4) on both axes:
// phase_weights[k*4 + t] is the Catmull-Rom weight of tap t of output phase k,
// whose first tap is source index + merge_int_phase_offset(factor, k).
cudaError_t launch_merge_int(const Plane& y, const Plane& uv, int factor, const float* phase_weights, const Plane& rgb,
                             cudaStream_t stream);
int merge_int_phase_offset(int factor, int k);

// Element-wise shl (n > 0) / shr (n < 0) of a u8 or u16 plane; src == dst
// allowed (core/src/ImageProcess.cpp:601-616).
cudaError_t launch_shift(const Plane& src, const Plane& dst, int n, cudaStream_t stream);

// General separable resize of an interleaved plane (any channel count).
cudaError_t launch_resize(const Plane& src, const Plane& dst, ResizeAxis ax, ResizeAxis ay, cudaStream_t stream);
// Catmull-Rom resize by exactly 2 or 4 on both axes (phase weights of
// phase_weights(factor)), the same values as launch_resize with the axis tables.
cudaError_t launch_resize_int(const Plane& src, const Plane& dst, int factor, const float* phase_weights,
                              cudaStream_t stream);

// Number of kernel launches issued by this library in the process so far.
uint64_t launch_count();
void count_launch(int n = 1);

}  // namespace acgb
