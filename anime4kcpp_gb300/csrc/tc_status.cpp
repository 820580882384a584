// Timeout status word of the tensor-core kernels.
//
// Every bounded wait in a tcgen05 kernel that gives up sets a device word to
// 1 (the kernel then releases its tensor memory and returns).  The word
// belongs to the calling host thread -- one per thread, as the reference
// keeps error state per calling thread (CUDAProcessor.cpp:284), so one
// thread's reset never clears or reports another thread's timeout -- and to
// the current device, so a thread that serves processors on several GPUs
// hands each kernel a word in its own device's memory.
//
// Reading it: tc_status_enqueue(s) queues, on the caller's stream behind the
// call's kernels, a copy of the word into a pinned host slot of the thread
// and the word's reset; after the caller synchronised s, tc_status_take()
// returns the copied value.  No extra synchronisation, no legacy-stream work.
#include <cuda_runtime.h>

#include "kernels.hpp"

namespace acgb {

namespace {
struct StatusWords
{
    int* dev[kMaxDevices] = {};
    int* host[kMaxDevices] = {};  // pinned landing slots
    int last = -1;                // device of the last enqueue
    ~StatusWords()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        for (int d = 0; d < kMaxDevices; d++)
        {
            if (dev[d] && cudaSetDevice(d) == cudaSuccess) cudaFree(dev[d]);
            if (host[d]) cudaFreeHost(host[d]);
        }
        if (cur >= 0) cudaSetDevice(cur);
    }
};
thread_local StatusWords g_words;

int current_device()
{
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) return -1;
    return d;
}
}  // namespace

int* tc_status_buffer()
{
    const int d = current_device();
    if (d < 0) return nullptr;
    StatusWords& w = g_words;
    if (!w.dev[d])
    {
        int* p = nullptr;
        if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
        if (cudaMemsetAsync(p, 0, sizeof(int), cudaStreamLegacy) != cudaSuccess ||
            cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess)
        {
            cudaFree(p);
            return nullptr;
        }
        w.dev[d] = p;
    }
    return w.dev[d];
}

cudaError_t tc_status_enqueue(cudaStream_t stream)
{
    const int d = current_device();
    int* word = tc_status_buffer();
    if (d < 0 || !word) return cudaErrorMemoryAllocation;
    StatusWords& w = g_words;
    if (!w.host[d])
    {
        void* h = nullptr;
        if (cudaHostAlloc(&h, sizeof(int), cudaHostAllocDefault) != cudaSuccess) return cudaErrorMemoryAllocation;
        w.host[d] = static_cast<int*>(h);
    }
    *w.host[d] = 0;
    cudaError_t err = cudaMemcpyAsync(w.host[d], word, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(word, 0, sizeof(int), stream);
    w.last = err == cudaSuccess ? d : -1;
    return err;
}

int tc_status_take()
{
    StatusWords& w = g_words;
    if (w.last < 0 || !w.host[w.last]) return -1;
    const int v = *static_cast<volatile int*>(w.host[w.last]);
    *w.host[w.last] = 0;
    w.last = -1;
    return v;
}

int tc_status_reset()
{
    int* p = tc_status_buffer();
    if (!p) return -1;
    int v = 0;
    if (cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    if (cudaMemset(p, 0, sizeof(int)) != cudaSuccess) return -1;
    return v;
}

}  // namespace acgb
