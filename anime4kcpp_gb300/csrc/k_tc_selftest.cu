// Self-test of the tcgen05 building blocks used by the tensor-core kernels:
// shared-memory descriptors (SWIZZLE_NONE, K-major), the kind::f16
// instruction descriptor, tensor-memory allocation, MMA completion through an
// mbarrier, and the 32x32b tensor-memory load layout.
//
// One CTA computes D[128][16] = A * B^T with A(m, k) = X[m + (k / 8) * shift][k % 8]
// -- the shifted-row view the convolution kernels use for their taps -- and
// B[16][K] K-major.  All operand addresses stay inside the allocated shared
// memory for any reading of the descriptor stride fields.
#include <cuda_runtime.h>

#include "ac_gb300.h"
#include "tc_ptx.cuh"

namespace acgb {
namespace {

constexpr int kSelfTestXBytes = 48 * 1024;
constexpr int kSelfTestBBytes = 4 * 1024;

__device__ __forceinline__ uint64_t global_timer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

__global__ void __launch_bounds__(128, 1)
tc_selftest_kernel(const uint4* __restrict__ x, int px, const uint16_t* __restrict__ b, int k, int shift, int bf16,
                   float* __restrict__ d, int* __restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* xs = smem;
    unsigned char* bs = smem + kSelfTestXBytes;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kSelfTestXBytes + kSelfTestBBytes);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kSelfTestXBytes + kSelfTestBBytes + 8);

    const int tid = threadIdx.x, warp = tid >> 5;
    // X rows: 16 bytes per pixel, contiguous.
    for (int i = tid; i < kSelfTestXBytes / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(xs)[i] = i < px ? x[i] : make_uint4(0, 0, 0, 0);
    // B in canonical K-major layout: chunk kc, 8-row group g, row r at kc*256 + g*128 + r*16.
    for (int i = tid; i < kSelfTestBBytes / 16; i += blockDim.x) reinterpret_cast<uint4*>(bs)[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    for (int i = tid; i < 16 * (k / 8); i += blockDim.x)
    {
        int n = i / (k / 8), kc = i % (k / 8);
        const uint16_t* src = b + n * k + kc * 8;
        uint16_t* dst = reinterpret_cast<uint16_t*>(bs + kc * 256 + (n / 8) * 128 + (n % 8) * 16);
        for (int e = 0; e < 8; e++) dst[e] = src[e];
    }
    if (warp == 0)
    {
        tc::tmem_alloc(tmem_slot, 32);
        tc::tmem_relinquish();
    }
    if (tid == 0)
    {
        tc::mbar_init(mbar, 1);
        tc::fence_mbar_init();
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    if (tid == 0)
    {
        const uint32_t idesc = tc::idesc_f16(128, 16, bf16 != 0);
        const uint32_t xa = tc::smem_u32(xs), ba = tc::smem_u32(bs);
        for (int i = 0; i < k / 16; i++)
        {
            uint64_t ad = tc::smem_desc(xa + static_cast<uint32_t>(2 * i * shift * 16), static_cast<uint32_t>(shift * 16), 128);
            uint64_t bd = tc::smem_desc(ba + static_cast<uint32_t>(2 * i * 256), 256, 128);
            tc::mma_f16(tmem, ad, bd, idesc, i > 0 ? 1u : 0u);
        }
        tc::mma_commit(mbar);
    }
    bool ok = false;
    const uint64_t t0 = global_timer_ns();
    while (!(ok = tc::mbar_try_wait(mbar, 0)))
        if (global_timer_ns() - t0 > 2000000000ull) break;
    if (!ok)
    {
        if (tid == 0) atomicExch(status, 1);
    }
    else
    {
        tc::fence_after_sync();
        float v[16];
        tc::tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16), v);
        tc::tmem_wait_ld();
        const int row = warp * 32 + (tid & 31);
        for (int j = 0; j < 16; j++) d[row * 16 + j] = v[j];
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 32);
}

}  // namespace
}  // namespace acgb

// Runs the self-test with host arrays: x[px][8] and b[16][k] 16-bit values
// (FP16 or BF16 bit patterns), k a multiple of 16 (at most 64), d[128][16].
// Returns 0, 1 when the MMA did not complete within 2 s, or -1 on a CUDA error.
int ac_gb300_tc_selftest(const uint16_t* x, int px, const uint16_t* b, int k, int shift, int bf16, float* d)
{
    using namespace acgb;
    if (!x || !b || !d || k % 16 != 0 || k <= 0 || k > 64 || px <= 0 || px * 16 > kSelfTestXBytes || shift < 0) return -1;
    if (128 + (k / 8 - 1) * shift > px) return -1;
    uint4* dx = nullptr;
    uint16_t* db = nullptr;
    float* dd = nullptr;
    int* ds = nullptr;
    int rc = -1;
    const size_t smem = kSelfTestXBytes + kSelfTestBBytes + 64;
    if (cudaMalloc(&dx, px * 16) != cudaSuccess) goto done;
    if (cudaMalloc(&db, 16 * k * 2) != cudaSuccess) goto done;
    if (cudaMalloc(&dd, 128 * 16 * 4) != cudaSuccess) goto done;
    if (cudaMalloc(&ds, 4) != cudaSuccess) goto done;
    cudaMemcpy(dx, x, px * 16, cudaMemcpyHostToDevice);
    cudaMemcpy(db, b, 16 * k * 2, cudaMemcpyHostToDevice);
    cudaMemset(dd, 0, 128 * 16 * 4);
    cudaMemset(ds, 0, 4);
    if (cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
        goto done;
    tc_selftest_kernel<<<1, 128, smem>>>(dx, px, db, k, shift, bf16, dd, ds);
    if (cudaDeviceSynchronize() != cudaSuccess) goto done;
    {
        int status = 0;
        cudaMemcpy(&status, ds, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(d, dd, 128 * 16 * 4, cudaMemcpyDeviceToHost);
        rc = status ? 1 : 0;
    }
done:
    if (dx) cudaFree(dx);
    if (db) cudaFree(db);
    if (dd) cudaFree(dd);
    if (ds) cudaFree(ds);
    return rc;
}

namespace acgb {
namespace {

// One thread waits, with the tensor-core kernels' bounded wait
// (tc::mbar_wait_ns), on an mbarrier phase that nothing completes: the wait
// must give up after `ns` and the kernel must end with status 1 (2 would mean
// the phase completed).  No asynchronous operation is in flight, so the kernel
// exits cleanly and the context stays usable.
__global__ void wait_selftest_kernel(uint64_t ns, int* status, unsigned long long* elapsed)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0)
    {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        const uint64_t t0 = global_timer_ns();
        const bool done = tc::mbar_wait_ns(&bar, 0, ns);
        *elapsed = global_timer_ns() - t0;
        *status = done ? 2 : 1;
    }
}

}  // namespace
}  // namespace acgb

int ac_gb300_wait_selftest(int limit_ms, int* status, double* elapsed_ms)
{
    using namespace acgb;
    if (!status || !elapsed_ms || limit_ms <= 0 || limit_ms > 2000) return -1;
    int* ds = nullptr;
    unsigned long long* de = nullptr;
    int rc = -1;
    if (cudaMalloc(&ds, sizeof(int)) != cudaSuccess) goto done;
    if (cudaMalloc(&de, sizeof(unsigned long long)) != cudaSuccess) goto done;
    cudaMemset(ds, 0, sizeof(int));
    wait_selftest_kernel<<<1, 32>>>(static_cast<uint64_t>(limit_ms) * 1000000ull, ds, de);
    if (cudaDeviceSynchronize() != cudaSuccess) goto done;
    {
        unsigned long long ns = 0;
        if (cudaMemcpy(status, ds, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) goto done;
        if (cudaMemcpy(&ns, de, sizeof(ns), cudaMemcpyDeviceToHost) != cudaSuccess) goto done;
        *elapsed_ms = static_cast<double>(ns) / 1e6;
        rc = 0;
    }
done:
    if (ds) cudaFree(ds);
    if (de) cudaFree(de);
    return rc;
}
