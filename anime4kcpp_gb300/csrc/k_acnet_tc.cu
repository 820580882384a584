// Tensor-core (tcgen05) layer-fused ACNetLegacy x2 pass.
//
// Same network and clamp-to-edge semantics as the plain FP32 kernel
// (core/internal/AC/Core/Internal/Processor/CPU/Common.hpp:116-197,344-393;
// core/src/processor/cpu/CPUProcessor.cpp:1371-1390).  Layer 0 (1->8) and
// the 2x2 transposed convolution run in FP32 on CUDA cores; the eight
// 3x3 8->8 convolutions run on the 5th-generation tensor cores as implicit
// GEMMs with FP16 (or BF16) operands and FP32 accumulation in tensor memory.
//
// Per CTA: a 46x46 tile of input pixels with a 9-pixel halo, i.e. a 64x64
// window = 4096 pixels = 32 GEMM row blocks of 128.  Activations live in
// shared memory as 16 bytes per pixel (8 channels, 16-bit), row-major over
// the flattened window, which is exactly the K-major "core matrix" row layout
// of the MMA operand: row block b of tap (dy, dx) is the buffer shifted by
// (dy-1)*64 + (dx-1) pixels, so a 3x3 convolution is nine shifted-view
// GEMM chunks of K = 8 with no im2col copy.  Two taps form one K = 16 MMA
// (the leading-byte offset of the descriptor is the distance between the two
// shifted views); the ninth tap is paired with a constant "ones" chunk whose
// B rows carry the bias (split into FP16 high and low parts), so the bias add
// is free.  D is M=128 x N=16 (eight real output channels, eight zero
// columns) FP32 in tensor memory: 32 row blocks x 16 columns = all 512
// columns, so a whole layer is computed before its outputs overwrite the
// activations in place.  The epilogue (16 warps) reads D with tcgen05.ld,
// applies ReLU while converting to 16-bit (cvt.rn.relu.f16x2) and stores
// back; positions of the window outside the image then take the value of
// their clamped in-image position (the reference's clamp-to-edge read of the
// intermediate map).  The last layer's epilogue keeps FP32, applies the
// transposed convolution and writes the 2x2 output pixels.
//
// One thread issues all MMAs and commits them to an mbarrier; every wait is
// bounded by %globaltimer and reports through a status word instead of
// hanging.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "kernels.hpp"
#include "tc_ptx.cuh"

namespace acgb {
namespace tcv1 {

constexpr int TILE = 46, HALO = 9, WIN = TILE + 2 * HALO;  // 64
constexpr int NPIX = WIN * WIN;                            // 4096
constexpr int NBLK = NPIX / 128;                           // 32
constexpr int PAD = 72;                                    // >= WIN + 1 pixels of slack before/after
constexpr int THREADS = 512;
constexpr int KCHUNKS = 10;                  // 9 taps + bias chunk
constexpr int BLAYER_BYTES = KCHUNKS * 256;  // 16 rows x 80 K x 2 bytes, canonical layout
constexpr int NLAYERS = 8;                   // tensor-core layers (1..8)
constexpr uint32_t TMEM_COLS = 512;
static_assert(NPIX % 128 == 0 && NBLK * 16 <= static_cast<int>(TMEM_COLS), "window accumulators must fit tensor memory");

constexpr int ACT_OFF = 0;
constexpr int ACT_BYTES = (PAD + NPIX + PAD) * 16;
constexpr int ONES_OFF = ACT_OFF + ACT_BYTES;
constexpr int ONES_BYTES = 128 * 16;
constexpr int B_OFF = ONES_OFF + ONES_BYTES;
constexpr int B_BYTES = NLAYERS * BLAYER_BYTES;
constexpr int INP_OFF = B_OFF + B_BYTES;
constexpr int INP_BYTES = NPIX * 4;
constexpr int MISC_OFF = INP_OFF + INP_BYTES;
constexpr int SMEM_BYTES = MISC_OFF + 64;

struct Params
{
    const uint4* bw;  // packed B matrices, NLAYERS * BLAYER_BYTES
    float k0[72];
    float b0[8];
    float k2[32];
    Plane in, out;
    int* status;
};

// Pixel shift of tap t (row-major 3x3) in the flattened window.
__device__ __forceinline__ int tap_shift(int t) { return (t / 3 - 1) * WIN + (t % 3 - 1); }

template <bool BF16>
__device__ __forceinline__ uint32_t pack_relu(float lo, float hi)
{
    if constexpr (BF16) return tc::pack_relu_bf16x2(lo, hi);
    else return tc::pack_relu_f16x2(lo, hi);
}

template <typename T, bool BF16>
__global__ void __launch_bounds__(THREADS, 1) acnet_tc_kernel(const __grid_constant__ Params P)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    uint4* act4 = reinterpret_cast<uint4*>(smem + ACT_OFF);   // index PAD + q
    uint4* ones4 = reinterpret_cast<uint4*>(smem + ONES_OFF);
    uint4* bsm4 = reinterpret_cast<uint4*>(smem + B_OFF);
    float* inp = reinterpret_cast<float*>(smem + INP_OFF);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + MISC_OFF);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + MISC_OFF + 8);
    int* abort_flag = reinterpret_cast<int*>(smem + MISC_OFF + 16);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int gx0 = blockIdx.x * TILE - HALO, gy0 = blockIdx.y * TILE - HALO;
    const int W = P.in.w, H = P.in.h;
    // in-image part of the window (inclusive, window coordinates)
    const int ix0 = max(0, -gx0), ix1 = min(WIN - 1, W - 1 - gx0);
    const int iy0 = max(0, -gy0), iy1 = min(WIN - 1, H - 1 - gy0);
    const bool border = ix0 > 0 || ix1 < WIN - 1 || iy0 > 0 || iy1 < WIN - 1;

    // ---- stage: zero activations, ones chunk, B matrices, input window ----
    for (int i = tid; i < ACT_BYTES / 16; i += THREADS) act4[i] = make_uint4(0, 0, 0, 0);
    if (tid < 128)
    {
        // rows of [1, 1, 0, ...]: the bias chunk multiplies B's high and low bias parts by one
        const uint32_t one = BF16 ? 0x3F80u : 0x3C00u;
        ones4[tid] = make_uint4(one | (one << 16), 0, 0, 0);
    }
    for (int i = tid; i < B_BYTES / 16; i += THREADS) bsm4[i] = P.bw[i];
    for (int i = tid; i < NPIX; i += THREADS)
    {
        const int wy = i / WIN, wx = i % WIN;
        const int gx = clampi(gx0 + wx, 0, W - 1), gy = clampi(gy0 + wy, 0, H - 1);
        inp[i] = to_float<T>(row_ptr<T>(P.in.ptr, P.in.pitch, gy)[gx]);
    }
    if (tid == 0)
    {
        tc::mbar_init(mbar, 1);
        tc::fence_mbar_init();
        *abort_flag = 0;
    }
    __syncthreads();

    // ---- layer 0 (FP32, CUDA cores) over the window inset by 1, evaluated
    // at clamped positions so out-of-image entries replicate the edge ----
    for (int i = tid; i < (WIN - 2) * (WIN - 2); i += THREADS)
    {
        const int y = 1 + i / (WIN - 2), x = 1 + i % (WIN - 2);
        const int cy = clampi(y, iy0, iy1), cx = clampi(x, ix0, ix1);
        float r[9];
#pragma unroll
        for (int t = 0; t < 9; t++) r[t] = inp[(cy + t / 3 - 1) * WIN + cx + t % 3 - 1];
        float a[8];
#pragma unroll
        for (int n = 0; n < 8; n++)
        {
            float s = r[0] * P.k0[n * 9];
#pragma unroll
            for (int t = 1; t < 9; t++) s = fmaf(r[t], P.k0[n * 9 + t], s);
            a[n] = s + P.b0[n];
        }
        act4[PAD + y * WIN + x] = make_uint4(pack_relu<BF16>(a[0], a[1]), pack_relu<BF16>(a[2], a[3]),
                                             pack_relu<BF16>(a[4], a[5]), pack_relu<BF16>(a[6], a[7]));
    }

    // Tensor memory for the whole window's accumulators.
    if (warp == 0)
    {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t act_base = tc::smem_u32(smem + ACT_OFF);
    const uint32_t ones_base = tc::smem_u32(smem + ONES_OFF);
    const uint32_t b_base = tc::smem_u32(smem + B_OFF);
    constexpr uint32_t IDESC = tc::idesc_f16(128, 16, BF16);
    const int quarter = warp & 3, group = warp >> 2;

    uint32_t phase = 0;
    for (int l = 1; l <= NLAYERS; l++)
    {
        // output region of layer l: the window inset by l+1, inside the image
        const int ry0 = max(l + 1, iy0), ry1 = min(WIN - 2 - l, iy1);
        const int rx0 = max(l + 1, ix0), rx1 = min(WIN - 2 - l, ix1);
        const int b0 = (ry0 * WIN + rx0) >> 7, b1 = (ry1 * WIN + rx1) >> 7;
        if (tid == 0)
        {
            const uint32_t bl = b_base + static_cast<uint32_t>((l - 1) * BLAYER_BYTES);
            for (int b = b0; b <= b1; b++)
            {
#pragma unroll
                for (int kk = 0; kk < 5; kk++)
                {
                    const uint32_t a0 = act_base + static_cast<uint32_t>((PAD + b * 128 + tap_shift(2 * kk)) * 16);
                    const uint32_t lbo = kk < 4 ? static_cast<uint32_t>((tap_shift(2 * kk + 1) - tap_shift(2 * kk)) * 16)
                                                : ones_base - a0;
                    tc::mma_f16(tmem + static_cast<uint32_t>(b * 16), tc::smem_desc(a0, lbo, 128),
                                tc::smem_desc(bl + static_cast<uint32_t>(kk * 512), 256, 128), IDESC, kk > 0 ? 1u : 0u);
                }
            }
            tc::mma_commit(mbar);
        }
        // bounded wait for this layer's MMAs, made CTA-uniform (tcgen05.ld is warp-collective)
        const bool done = __syncthreads_and(tc::mbar_wait_ns(mbar, phase, 2000000000ull) ? 1 : 0) != 0;
        phase ^= 1;
        if (!done && tid == 0) *abort_flag = 1;
        tc::fence_after_sync();
        if (done)
        {
            for (int b = b0 + group; b <= b1; b += 4)
            {
                float v[8];
                tc::tmem_ld8(tmem + (static_cast<uint32_t>(quarter * 32) << 16) + static_cast<uint32_t>(b * 16), v);
                tc::tmem_wait_ld();
                const int q = b * 128 + quarter * 32 + lane;
                const int y = q >> 6, x = q & (WIN - 1);
                const bool valid = y >= ry0 && y <= ry1 && x >= rx0 && x <= rx1;
                if (!valid) continue;
                if (l < NLAYERS)
                {
                    act4[PAD + q] = make_uint4(pack_relu<BF16>(v[0], v[1]), pack_relu<BF16>(v[2], v[3]),
                                               pack_relu<BF16>(v[4], v[5]), pack_relu<BF16>(v[6], v[7]));
                }
                else
                {
#pragma unroll
                    for (int c = 0; c < 8; c++) v[c] = fmaxf(v[c], 0.0f);
                    const int ox = 2 * (gx0 + x), oy = 2 * (gy0 + y);
#pragma unroll
                    for (int dy = 0; dy < 2; dy++)
                    {
                        T o[2];
#pragma unroll
                        for (int dx = 0; dx < 2; dx++)
                        {
                            const int ko = 8 * (dy * 2 + dx);
                            float d = v[0] * P.k2[ko];
#pragma unroll
                            for (int c = 1; c < 8; c++) d = fmaf(v[c], P.k2[ko + c], d);
                            o[dx] = from_float<T>(d);
                        }
                        T* row = row_ptr_w<T>(P.out.ptr, P.out.pitch, oy + dy) + ox;
                        row[0] = o[0];
                        row[1] = o[1];
                    }
                }
            }
        }
        if (border && l < NLAYERS)
        {
            __syncthreads();
            // out-of-image positions of this layer's region take their clamped value
            const int lo = l + 1, hi = WIN - 2 - l, n = hi - lo + 1;
            for (int i = tid; i < n * n; i += THREADS)
            {
                const int y = lo + i / n, x = lo + i % n;
                const int cy = clampi(y, iy0, iy1), cx = clampi(x, ix0, ix1);
                if (cy != y || cx != x) act4[PAD + y * WIN + x] = act4[PAD + cy * WIN + cx];
            }
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (*abort_flag) break;
    }
    if (tid == 0 && *abort_flag) atomicExch(P.status, 1);
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

template <typename T, bool BF16>
cudaError_t launch_typed(const Params& p, dim3 grid, cudaStream_t stream)
{
    // one-time set-up per device, thread-safe
    const cudaError_t setup = device_once([] {
        return cudaFuncSetAttribute(acnet_tc_kernel<T, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    });
    if (setup != cudaSuccess) return setup;
    acnet_tc_kernel<T, BF16><<<grid, THREADS, SMEM_BYTES, stream>>>(p);
    return cudaGetLastError();
}

uint16_t to_bits(float v, bool bf16)
{
    if (bf16)
    {
        __nv_bfloat16 h = __float2bfloat16_rn(v);
        return *reinterpret_cast<uint16_t*>(&h);
    }
    __half h = __float2half_rn(v);
    return *reinterpret_cast<uint16_t*>(&h);
}
float from_bits(uint16_t b, bool bf16)
{
    if (bf16)
    {
        __nv_bfloat16 h;
        *reinterpret_cast<uint16_t*>(&h) = b;
        return __bfloat162float(h);
    }
    __half h;
    *reinterpret_cast<uint16_t*>(&h) = b;
    return __half2float(h);
}

}  // namespace tcv1

// B operand of layer l (1..8), K-major canonical layout: for K chunk kc
// (taps 0..8, then the bias chunk), 8-row group g of the 16 output columns and
// row r: 8 16-bit values at byte kc*256 + g*128 + r*16.  Output columns 8..15
// are zero.  The bias chunk holds (bias_hi, bias_lo, 0...) so that the MMA
// against ones rows (1, 1, 0, ...) adds bias_hi + bias_lo.
void pack_acnet_tc_weights(const AcnetLegacyWeights& w, bool bf16, std::vector<uint16_t>& packed)
{
    using namespace tcv1;
    packed.assign(static_cast<size_t>(NLAYERS) * BLAYER_BYTES / 2, 0);
    for (int l = 1; l <= NLAYERS; l++)
    {
        uint16_t* base = packed.data() + static_cast<size_t>(l - 1) * BLAYER_BYTES / 2;
        for (int n = 0; n < 8; n++)
        {
            for (int kc = 0; kc < 9; kc++)
                for (int c = 0; c < 8; c++)
                {
                    float v = w.k[72 + 576 * (l - 1) + n * 72 + kc * 8 + c];
                    base[(kc * 256 + (n / 8) * 128 + (n % 8) * 16) / 2 + c] = to_bits(v, bf16);
                }
            float bias = w.b[8 * l + n];
            uint16_t hi = to_bits(bias, bf16);
            uint16_t lo = to_bits(bias - from_bits(hi, bf16), bf16);
            base[(9 * 256 + (n / 8) * 128 + (n % 8) * 16) / 2 + 0] = hi;
            base[(9 * 256 + (n / 8) * 128 + (n % 8) * 16) / 2 + 1] = lo;
        }
    }
}

// Device word that a tensor-core kernel sets when a bounded wait gave up.
// The calling host thread's status word of the tensor-core kernels (0, or 1
// after a timed-out wait): one per thread, as the reference keeps error state
// per calling thread (CUDAProcessor.cpp:284), so one thread's reset never
// clears or reports another thread's timeout; and one per device, so a thread
// that serves processors on several GPUs hands each kernel a word in its own
// device's memory.
namespace {
struct StatusWords
{
    int* p[kMaxDevices] = {};
    ~StatusWords()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        for (int d = 0; d < kMaxDevices; d++)
            if (p[d] && cudaSetDevice(d) == cudaSuccess) cudaFree(p[d]);
        if (cur >= 0) cudaSetDevice(cur);
    }
};
}  // namespace

int* tc_status_buffer()
{
    static thread_local StatusWords w;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    if (!w.p[dev] && cudaMalloc(&w.p[dev], sizeof(int)) == cudaSuccess) cudaMemset(w.p[dev], 0, sizeof(int));
    return w.p[dev];
}

cudaError_t launch_acnet_legacy_tc(const AcnetLegacyWeights& wts, const void* packed, bool bf16, const Plane& in,
                                   const Plane& out, cudaStream_t stream)
{
    using namespace tcv1;
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    if (!packed) return cudaErrorInvalidValue;
    Params p;
    p.bw = static_cast<const uint4*>(packed);
    for (int i = 0; i < 72; i++) p.k0[i] = wts.k[i];
    for (int i = 0; i < 8; i++) p.b0[i] = wts.b[i];
    for (int i = 0; i < 32; i++) p.k2[i] = wts.k[72 + 576 * 8 + i];
    p.in = in;
    p.out = out;
    p.status = tc_status_buffer();
    if (!p.status) return cudaErrorMemoryAllocation;
    dim3 grid((in.w + TILE - 1) / TILE, (in.h + TILE - 1) / TILE);
    cudaError_t err;
    switch (in.type)
    {
    case kU8: err = bf16 ? launch_typed<uint8_t, true>(p, grid, stream) : launch_typed<uint8_t, false>(p, grid, stream); break;
    case kU16: err = bf16 ? launch_typed<uint16_t, true>(p, grid, stream) : launch_typed<uint16_t, false>(p, grid, stream); break;
    case kF32: err = bf16 ? launch_typed<float, true>(p, grid, stream) : launch_typed<float, false>(p, grid, stream); break;
    default: return cudaErrorInvalidValue;
    }
    if (err == cudaSuccess) count_launch();
    return err;
}

// Reads and clears the tensor-core timeout flag (1 if any MMA wait gave up).
int tc_status_reset()
{
    int* p = tc_status_buffer();
    if (!p) return -1;
    int v = 0;
    cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemset(p, 0, sizeof(int));
    return v;
}

}  // namespace acgb
