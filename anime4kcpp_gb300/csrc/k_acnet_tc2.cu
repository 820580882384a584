// Tensor-core (tcgen05) layer-fused ACNetLegacy x2 pass, pair-interleaved form.
//
// Network and clamp semantics as in k_acnet_fp32.cu (reference:
// core/internal/AC/Core/Internal/Processor/CPU/Common.hpp:116-197,344-393).
//
// Tile: 48x44 input pixels plus a 9-pixel halo = a 66x62 window (4092
// pixels).  Activations are 8 channels x 16 bit = 16 bytes per pixel, split
// into two planes by column parity: plane E holds the even columns, plane O
// the odd ones, each indexed by the pixel-pair number r = (y*66 + x) / 2.
// One GEMM row is one horizontal pixel pair, and one MMA computes both
// pixels of 128 pairs: N = 16 output columns = 8 channels of pixel 2r then 8
// of pixel 2r+1.  For kernel row dy the pair needs input pixels 2r-1 .. 2r+2
// of that row, i.e. four 8-channel chunks
//   O[r-1+s], E[r+s], O[r+s], E[r+1+s]        (s = (dy-1) * 33 pairs)
// each a contiguous run of 16-byte rows in one plane -- a valid K-major core
// matrix view.  Two chunks form one K=16 MMA (E first, O second, so the
// descriptor's leading-byte offset is the plane distance minus 16 bytes);
// three kernel rows give six MMAs and a seventh multiplies a constant "ones"
// chunk by the bias (split into 16-bit high and low parts).  Seven MMAs per
// 256 output pixels instead of ten with one pixel per row, and every output
// column is useful.  D = 16 blocks x 16 columns fits 256 tensor-memory
// columns, so two CTAs share an SM and one's epilogue overlaps the other's
// MMAs.
//
// Data movement: one TMA 2-D tiled load brings the raw input window (its
// x origin rounded down to a 16-byte boundary), one bulk copy brings the
// packed weights of all eight layers, both completing on one mbarrier.  The
// epilogue converts D with cvt.rn.relu to 16 bit and writes the next layer's
// activations in place (all MMAs of a layer complete before any write); an
// output pixel on the image edge also writes its value to the out-of-image
// neighbour the next layer reads (clamp-to-edge of the intermediate map).
// The last layer keeps FP32, applies the 2x2 transposed convolution and
// stores the outputs.
//
// RGB(A) inputs (C = 3 or 4) take the fused path: the prologue loads the
// RGB(A) window with coalesced loads and derives the quantised Y window and
// the UV(A) region (tile + 2 pixels) exactly as rgb2yuv does; the last
// layer's epilogue resamples UV(A) x2 with Catmull-Rom and merges it with the
// new luma (yuv2rgb), writing RGB(A) output directly.  No intermediate plane
// touches HBM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstring>

#include "colour.cuh"
#include "device_common.cuh"
#include "kernels.hpp"
#include "tc_ptx.cuh"
#include "tma_host.hpp"

namespace acgb {
namespace tcv2 {

constexpr int TW = 48, TH = 44, HALO = 9;
constexpr int WW = TW + 2 * HALO, WH = TH + 2 * HALO;  // 66 x 62
constexpr int PPR = WW / 2;                             // pairs per window row
constexpr int NPAIR = WW * WH / 2;                      // 2046
constexpr int NBLK = 16;                                // 16 x 128 pairs
constexpr int PADP = 40;                                // >= PPR + 1 pairs of slack
constexpr int PLANE_PAIRS = PADP + NBLK * 128 + PADP;
constexpr int PLANE_BYTES = PLANE_PAIRS * 16;
constexpr int KCH = 14;                 // 12 tap chunks + bias chunk + zero chunk
constexpr int BL_BYTES = KCH * 256;     // per layer
constexpr int NL = 8;
constexpr int B_BYTES = NL * BL_BYTES;  // 28672
constexpr uint32_t TMEM_COLS = 256;
constexpr int THREADS = 512;
static_assert(WW % 2 == 0 && NPAIR <= NBLK * 128, "window must fit the pair blocks");
static_assert(NBLK * 16 <= static_cast<int>(TMEM_COLS), "accumulators must fit tensor memory");

template <typename T>
struct InBox
{
    static constexpr int align = 16 / static_cast<int>(sizeof(T));  // x alignment in elements
    static constexpr int w = ((WW + align - 1 + align - 1) / align) * align;
    static constexpr int bytes = w * WH * static_cast<int>(sizeof(T));
};

constexpr int E_OFF = 0;
constexpr int O_OFF = PLANE_BYTES;
constexpr int ONES_OFF = 2 * PLANE_BYTES;
constexpr int ONES_BYTES = 129 * 16 + 112;  // 129 rows, rounded up to a 128-byte multiple
constexpr int B_OFF = ONES_OFF + ONES_BYTES;
constexpr int IN_OFF = B_OFF + B_BYTES;
static_assert(IN_OFF % 128 == 0, "TMA destination must be 128-byte aligned");

constexpr int UVW = TW + 4, UVH = TH + 4;  // chroma region: the tile plus 2 pixels each side
constexpr int UVX0 = HALO - 2, UVY0 = HALO - 2;  // its origin in window coordinates
static_assert(UVH * 2 * TW * 3 * 4 <= 2 * PLANE_BYTES, "horizontal chroma sums must fit the activation planes");

template <typename T, int C>
struct Layout
{
    static constexpr int in_bytes = (InBox<T>::bytes + 127) / 128 * 128;
    static constexpr int lut_off = IN_OFF + in_bytes;
    static constexpr int lut_bytes = sizeof(T) == 1 ? 1024 : 0;
    static constexpr int uv_off = lut_off + lut_bytes;
    static constexpr int uv_bytes = C == 1 ? 0 : (UVW * UVH * (C - 1) * static_cast<int>(sizeof(T)) + 15) / 16 * 16;
    static constexpr int misc_off = uv_off + uv_bytes;
    static constexpr int smem = misc_off + 64;
};

struct Params
{
    const uint4* bw;  // packed weights, B_BYTES
    float k0[72];
    float b0[8];
    float k2[32];
    int w, h;         // input size
    Plane in;         // RGB(A) input for C = 3, 4
    Plane out;        // luma (C = 1) or RGB(A) output
    Phase2 ph;        // x2 Catmull-Rom weights for the fused chroma
    int* status;
};

template <bool BF16>
__device__ __forceinline__ uint32_t pack_relu(float lo, float hi)
{
    if constexpr (BF16) return tc::pack_relu_bf16x2(lo, hi);
    else return tc::pack_relu_f16x2(lo, hi);
}

template <bool BF16>
__device__ __forceinline__ uint4 pack8(const float* v)
{
    return make_uint4(pack_relu<BF16>(v[0], v[1]), pack_relu<BF16>(v[2], v[3]), pack_relu<BF16>(v[4], v[5]),
                      pack_relu<BF16>(v[6], v[7]));
}

// Activation slot of window pixel p (flattened y*WW + x).
__device__ __forceinline__ uint4* slot(unsigned char* smem, int p)
{
    return reinterpret_cast<uint4*>(smem + ((p & 1) ? O_OFF : E_OFF)) + PADP + (p >> 1);
}

template <typename T, int C, bool BF16>
__global__ void __launch_bounds__(THREADS, 2)
acnet_tc2_kernel(const __grid_constant__ CUtensorMap in_map, const __grid_constant__ Params P)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    using L = Layout<T, C>;
    T* raw = reinterpret_cast<T*>(smem + IN_OFF);
    T* uvs = reinterpret_cast<T*>(smem + L::uv_off);
    float* lut = reinterpret_cast<float*>(smem + L::lut_off);
    uint64_t* mbar_in = reinterpret_cast<uint64_t*>(smem + L::misc_off);
    uint64_t* mbar_mma = reinterpret_cast<uint64_t*>(smem + L::misc_off + 8);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L::misc_off + 16);
    int* abort_flag = reinterpret_cast<int*>(smem + L::misc_off + 20);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int gx0 = blockIdx.x * TW - HALO, gy0 = blockIdx.y * TH - HALO;
    const int ix0 = max(0, -gx0), ix1 = min(WW - 1, P.w - 1 - gx0);
    const int iy0 = max(0, -gy0), iy1 = min(WH - 1, P.h - 1 - gy0);
    // TMA origin: x rounded down to a 16-byte boundary (may be negative; zero fill)
    const int xal = gx0 >= 0 ? (gx0 / InBox<T>::align) * InBox<T>::align : -(((-gx0) + InBox<T>::align - 1) / InBox<T>::align) * InBox<T>::align;
    const int xoff = C == 1 ? gx0 - xal : 0;

    if (tid == 0)
    {
        tc::mbar_init(mbar_in, 1);
        tc::mbar_init(mbar_mma, 1);
        tc::fence_mbar_init();
        *abort_flag = 0;
    }
    if constexpr (sizeof(T) == 1)
        if (tid < 256) lut[tid] = __fdiv_rn(static_cast<float>(tid), 255.0f);
    __syncthreads();
    if (tid == 0)
    {
        if constexpr (C == 1)
        {
            tc::mbar_arrive_expect_tx(mbar_in, static_cast<uint32_t>(InBox<T>::bytes + B_BYTES));
            tc::tma_load_2d(smem + IN_OFF, &in_map, xal, gy0, mbar_in);
        }
        else tc::mbar_arrive_expect_tx(mbar_in, static_cast<uint32_t>(B_BYTES));
        tc::bulk_load(smem + B_OFF, P.bw, B_BYTES, mbar_in);
    }
    if constexpr (C > 1)
    {
        // fused split: quantised Y for the whole window, UV(A) for the chroma
        // region; out-of-image positions take the clamped (edge) pixel
        for (int i = tid; i < WW * WH; i += THREADS)
        {
            const int wy = i / WW, wx = i - (i / WW) * WW;
            const int gx = clampi(gx0 + wx, 0, P.w - 1), gy = clampi(gy0 + wy, 0, P.h - 1);
            T px[C];
            const T* src = row_ptr<T>(P.in.ptr, P.in.pitch, gy) + gx * C;
#pragma unroll
            for (int c = 0; c < C; c++) px[c] = src[c];
            T yq, uvq[C - 1];
            rgb_to_yuv_q_lut<T, C>(px, yq, uvq, lut);
            raw[wy * InBox<T>::w + wx] = yq;
            const int ux = wx - UVX0, uy = wy - UVY0;
            if (ux >= 0 && ux < UVW && uy >= 0 && uy < UVH)
            {
#pragma unroll
                for (int c = 0; c < C - 1; c++) uvs[(uy * UVW + ux) * (C - 1) + c] = uvq[c];
            }
        }
    }
    if (tid < 129)
    {
        const uint32_t one = BF16 ? 0x3F80u : 0x3C00u;
        reinterpret_cast<uint4*>(smem + ONES_OFF)[tid] = make_uint4(one | (one << 16), 0, 0, 0);
    }
    __syncthreads();
    // CTA-uniform outcome of the bounded wait for the input tile and weights
    if (!__syncthreads_and(tc::mbar_wait_ns(mbar_in, 0, 2000000000ull) ? 1 : 0))
    {
        if (tid == 0) atomicExch(P.status, 2);
        return;
    }

    // ---- layer 0 (FP32, CUDA cores): window inset by 1, evaluated at the
    // clamped in-image position so out-of-image entries replicate the edge ----
    for (int i = tid; i < (WW - 2) * (WH - 2); i += THREADS)
    {
        const int y = 1 + i / (WW - 2), x = 1 + i % (WW - 2);
        const int cy = clampi(y, iy0, iy1), cx = clampi(x, ix0, ix1);
        // the TMA tile holds zeros outside the image: clamp every tap
        const int ty[3] = {max(cy - 1, iy0), cy, min(cy + 1, iy1)};
        const int tx[3] = {xoff + max(cx - 1, ix0), xoff + cx, xoff + min(cx + 1, ix1)};
        float r[9];
#pragma unroll
        for (int t = 0; t < 9; t++)
        {
            const T v = raw[ty[t / 3] * InBox<T>::w + tx[t % 3]];
            if constexpr (sizeof(T) == 1) r[t] = lut[v];
            else r[t] = to_float<T>(v);
        }
        float a[8];
#pragma unroll
        for (int n = 0; n < 8; n++)
        {
            float s = r[0] * P.k0[n * 9];
#pragma unroll
            for (int t = 1; t < 9; t++) s = fmaf(r[t], P.k0[n * 9 + t], s);
            a[n] = s + P.b0[n];
        }
        *slot(smem, y * WW + x) = pack8<BF16>(a);
    }

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
    const uint32_t e_base = tc::smem_u32(smem + E_OFF);
    const uint32_t ones_base = tc::smem_u32(smem + ONES_OFF);
    const uint32_t b_base = tc::smem_u32(smem + B_OFF);
    constexpr uint32_t IDESC = tc::idesc_f16(128, 16, BF16);
    const int quarter = warp & 3, group = warp >> 2;

    uint32_t phase = 0;
    for (int l = 1; l <= NL; l++)
    {
        const int ry0 = max(l + 1, iy0), ry1 = min(WH - 2 - l, iy1);
        const int rx0 = max(l + 1, ix0), rx1 = min(WW - 2 - l, ix1);
        const int b0 = ((ry0 * WW + rx0) >> 1) >> 7, b1 = ((ry1 * WW + rx1) >> 1) >> 7;
        if (tid == 0)
        {
            const uint32_t bl = b_base + static_cast<uint32_t>((l - 1) * BL_BYTES);
            for (int b = b0; b <= b1; b++)
            {
                const uint32_t d = tmem + static_cast<uint32_t>(b * 16);
#pragma unroll
                for (int dy = 0; dy < 3; dy++)
                {
                    const int s = (dy - 1) * PPR;
                    const uint32_t a0 = e_base + static_cast<uint32_t>((PADP + b * 128 + s) * 16);
                    tc::mma_f16(d, tc::smem_desc(a0, PLANE_BYTES - 16, 128), tc::smem_desc(bl + (2 * dy) * 512, 256, 128),
                                IDESC, dy > 0 ? 1u : 0u);
                    tc::mma_f16(d, tc::smem_desc(a0 + 16, PLANE_BYTES - 16, 128),
                                tc::smem_desc(bl + (2 * dy + 1) * 512, 256, 128), IDESC, 1u);
                }
                tc::mma_f16(d, tc::smem_desc(ones_base, 16, 128), tc::smem_desc(bl + 6 * 512, 256, 128), IDESC, 1u);
            }
            tc::mma_commit(mbar_mma);
        }
        // CTA-uniform outcome of the bounded wait (tcgen05.ld is warp-collective)
        const bool done = __syncthreads_and(tc::mbar_wait_ns(mbar_mma, phase, 2000000000ull) ? 1 : 0) != 0;
        phase ^= 1;
        if (!done && tid == 0) *abort_flag = 1;
        tc::fence_after_sync();
        float* H = reinterpret_cast<float*>(smem + E_OFF);  // last layer: the activations are dead
        if constexpr (C > 1)
        {
            if (done && l == NL)
            {
                // horizontal pass of the x2 chroma resample for the whole tile,
                // shared by the vertical passes of the epilogue below
                for (int e = tid; e < UVH * 2 * TW; e += THREADS)
                {
                    const int r = e / (2 * TW), ox = e - r * (2 * TW);
                    chroma_hpass<T, C - 1>(uvs + r * UVW * (C - 1), ox >> 1, ox & 1, P.ph, H + e * (C - 1));
                }
                __syncthreads();
            }
        }
        if (done)
        {
            for (int b = b0 + group; b <= b1; b += 4)
            {
                float v[16];
                tc::tmem_ld16(tmem + (static_cast<uint32_t>(quarter * 32) << 16) + static_cast<uint32_t>(b * 16), v);
                tc::tmem_wait_ld();
                const int r = b * 128 + quarter * 32 + lane;
#pragma unroll
                for (int k = 0; k < 2; k++)
                {
                    const int p = 2 * r + k;
                    const int y = p / WW, x = p - y * WW;
                    if (y < ry0 || y > ry1 || x < rx0 || x > rx1) continue;
                    if (l < NL)
                    {
                        const uint4 val = pack8<BF16>(v + 8 * k);
                        *slot(smem, p) = val;
                        // clamp-to-edge for the next layer: the out-of-image
                        // neighbours it reads get this edge value
                        const bool xl = x == ix0 && x > 0, xr = x == ix1 && x < WW - 1;
                        const bool yt = y == iy0 && y > 0, yb = y == iy1 && y < WH - 1;
                        if (xl) *slot(smem, p - 1) = val;
                        if (xr) *slot(smem, p + 1) = val;
                        if (yt)
                        {
                            *slot(smem, p - WW) = val;
                            if (xl) *slot(smem, p - WW - 1) = val;
                            if (xr) *slot(smem, p - WW + 1) = val;
                        }
                        if (yb)
                        {
                            *slot(smem, p + WW) = val;
                            if (xl) *slot(smem, p + WW - 1) = val;
                            if (xr) *slot(smem, p + WW + 1) = val;
                        }
                    }
                    else
                    {
                        float s[8];
#pragma unroll
                        for (int c = 0; c < 8; c++) s[c] = fmaxf(v[8 * k + c], 0.0f);
                        const int ox = 2 * (gx0 + x), oy = 2 * (gy0 + y);
                        T o[2][2];
#pragma unroll
                        for (int dy = 0; dy < 2; dy++)
#pragma unroll
                            for (int dx = 0; dx < 2; dx++)
                            {
                                const int ko = 8 * (dy * 2 + dx);
                                float d = s[0] * P.k2[ko];
#pragma unroll
                                for (int c = 1; c < 8; c++) d = fmaf(s[c], P.k2[ko + c], d);
                                o[dy][dx] = from_float<T>(d);
                            }
                        T* row0 = row_ptr_w<T>(P.out.ptr, P.out.pitch, oy) + ox * C;
                        T* row1 = row_ptr_w<T>(P.out.ptr, P.out.pitch, oy + 1) + ox * C;
                        if constexpr (C == 1)
                        {
                            row0[0] = o[0][0];
                            row0[1] = o[0][1];
                            row1[0] = o[1][0];
                            row1[1] = o[1][1];
                        }
                        else merge_block2_h<T, C>(H, 2 * TW, x - HALO, y - HALO, P.ph, o, row0, row1, lut);
                    }
                }
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

template <typename T, int C, bool BF16>
cudaError_t launch_typed(const CUtensorMap& map, const Params& p, dim3 grid, cudaStream_t stream)
{
    // one-time set-up per device, thread-safe
    const cudaError_t setup = device_once([] {
        return cudaFuncSetAttribute(acnet_tc2_kernel<T, C, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize, Layout<T, C>::smem);
    });
    if (setup != cudaSuccess) return setup;
    acnet_tc2_kernel<T, C, BF16><<<grid, THREADS, Layout<T, C>::smem, stream>>>(map, p);
    return cudaGetLastError();
}

template <typename T, bool BF16>
cudaError_t launch_channels(int c, const CUtensorMap& map, const Params& p, dim3 grid, cudaStream_t stream)
{
    switch (c)
    {
    case 1: return launch_typed<T, 1, BF16>(map, p, grid, stream);
    case 3: return launch_typed<T, 3, BF16>(map, p, grid, stream);
    case 4: return launch_typed<T, 4, BF16>(map, p, grid, stream);
    default: return cudaErrorInvalidValue;
    }
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

}  // namespace tcv2

// Weights of the pair-interleaved form.  Layer l (1..8), chunk j (0..13),
// output column n (0..15; n < 8 is pixel 2r, n >= 8 pixel 2r+1, channel n % 8),
// input channel c: 16-bit value at element (j*256 + (n/8)*128 + (n%8)*16)/2 + c.
// MMA m = 2*dy multiplies chunks 4*dy (E[r+s]) and 4*dy+1 (O[r-1+s]);
// MMA m = 2*dy+1 multiplies chunks 4*dy+2 (E[r+1+s]) and 4*dy+3 (O[r+s]):
//   E[r+s]   : pixel 2r tap dx=1, pixel 2r+1 tap dx=0
//   O[r-1+s] : pixel 2r tap dx=0, pixel 2r+1 none
//   E[r+1+s] : pixel 2r none,     pixel 2r+1 tap dx=2
//   O[r+s]   : pixel 2r tap dx=2, pixel 2r+1 tap dx=1
// Chunk 12 is the ones chunk (bias high, bias low), chunk 13 is zero.
void pack_acnet_tc2_weights(const AcnetLegacyWeights& w, bool bf16, std::vector<uint16_t>& packed)
{
    using namespace tcv2;
    packed.assign(static_cast<size_t>(B_BYTES) / 2, 0);
    for (int l = 1; l <= NL; l++)
    {
        uint16_t* base = packed.data() + static_cast<size_t>(l - 1) * BL_BYTES / 2;
        auto put = [&](int chunk, int n, int tap, int dy) {
            // n: output column 0..15; tap dx of output pixel (n / 8) in kernel row dy
            for (int c = 0; c < 8; c++)
            {
                float v = w.k[72 + 576 * (l - 1) + (n % 8) * 72 + (dy * 3 + tap) * 8 + c];
                base[(chunk * 256 + (n / 8) * 128 + (n % 8) * 16) / 2 + c] = to_bits(v, bf16);
            }
        };
        for (int dy = 0; dy < 3; dy++)
        {
            const int m0 = 2 * dy, m1 = 2 * dy + 1;
            for (int n = 0; n < 16; n++)
            {
                const bool second = n >= 8;
                // MMA m0: chunk (first) = E[r+s], chunk (second) = O[r-1+s]
                put(2 * m0 + 0, n, second ? 0 : 1, dy);
                if (!second) put(2 * m0 + 1, n, 0, dy);
                // MMA m1: chunk (first) = E[r+1+s], chunk (second) = O[r+s]
                if (second) put(2 * m1 + 0, n, 2, dy);
                put(2 * m1 + 1, n, second ? 1 : 2, dy);
            }
        }
        for (int n = 0; n < 16; n++)
        {
            float bias = w.b[8 * l + (n % 8)];
            uint16_t hi = to_bits(bias, bf16);
            uint16_t lo = to_bits(bias - from_bits(hi, bf16), bf16);
            base[(12 * 256 + (n / 8) * 128 + (n % 8) * 16) / 2 + 0] = hi;
            base[(12 * 256 + (n / 8) * 128 + (n % 8) * 16) / 2 + 1] = lo;
        }
    }
}

int* tc_status_buffer();

bool acnet_tc2_supported(const Plane& in) { return in.channels > 1 || tma_plane_ok(in.ptr, in.pitch); }

cudaError_t launch_acnet_legacy_tc2(const AcnetLegacyWeights& wts, const void* packed2, bool bf16, const Plane& in,
                                    const Plane& out, const Phase2* phase2, cudaStream_t stream)
{
    using namespace tcv2;
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    if (!packed2) return cudaErrorInvalidValue;
    const int es = in.type & 0xff;
    const int boxw = es == 1 ? InBox<uint8_t>::w : (es == 2 ? InBox<uint16_t>::w : InBox<float>::w);
    CUtensorMap map;
    std::memset(&map, 0, sizeof(map));
    if (in.channels == 1 && !encode_tmap_2d(&map, in.ptr, es, in.w, in.h, in.pitch, boxw, WH)) return cudaErrorInvalidValue;
    if (in.channels > 1 && !phase2)
        return cudaErrorInvalidValue;
    Params p;
    if (phase2) p.ph = *phase2;
    p.in = in;
    p.bw = static_cast<const uint4*>(packed2);
    for (int i = 0; i < 72; i++) p.k0[i] = wts.k[i];
    for (int i = 0; i < 8; i++) p.b0[i] = wts.b[i];
    for (int i = 0; i < 32; i++) p.k2[i] = wts.k[72 + 576 * 8 + i];
    p.w = in.w;
    p.h = in.h;
    p.out = out;
    p.status = tc_status_buffer();
    if (!p.status) return cudaErrorMemoryAllocation;
    dim3 grid((in.w + TW - 1) / TW, (in.h + TH - 1) / TH);
    cudaError_t err;
    const int c = in.channels;
    switch (in.type)
    {
    case kU8: err = bf16 ? launch_channels<uint8_t, true>(c, map, p, grid, stream) : launch_channels<uint8_t, false>(c, map, p, grid, stream); break;
    case kU16: err = bf16 ? launch_channels<uint16_t, true>(c, map, p, grid, stream) : launch_channels<uint16_t, false>(c, map, p, grid, stream); break;
    case kF32: err = bf16 ? launch_channels<float, true>(c, map, p, grid, stream) : launch_channels<float, false>(c, map, p, grid, stream); break;
    default: return cudaErrorInvalidValue;
    }
    if (err == cudaSuccess) count_launch();
    return err;
}

}  // namespace acgb
