// Serving loop: a request queue in front of the GB300 processors that admits
// upscale jobs of mixed resolutions, factors, models and formats by an HBM
// budget, keeps weights and frame buffers resident on the device, batches
// compatible jobs as they arrive (continuous batching) and overlaps the work
// of different jobs on the device through several worker streams.
//
// The reference has no serving loop (its callers are the CLI, the GUI and the
// host filters, all one image at a time through Processor::process); the jobs
// run through the same processors and kernels as ac_processor_process, so a
// job's result is the same alone and in any mix.
#pragma once

#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "processor_impl.hpp"

namespace acgb {

// A host image plane (pinned host memory lets the copies run asynchronously).
struct HostPlane
{
    void* ptr = nullptr;
    int w = 0, h = 0, c = 0, stride = 0, type = Image::UInt8;
};

struct ServeJob
{
    std::string model;
    double factor = 2.0;
    int planes = 1;  // 1: one interleaved image (1, 3 or 4 channels); 2 or 3: planar YUV, Y first
    int shift = 0;   // planar YUV: shl / shr bits of Y (the reference CLI's recipe)
    HostPlane src[3], dst[3];
};

struct ServeResult
{
    int status = 0;  // 0 done, -1 failed, -2 rejected (can never fit the budget, bad job)
    std::string error;
    double queueMs = 0.0;    // submit -> admitted
    double deviceMs = 0.0;   // first copy issued -> result in the dst planes
    double latencyMs = 0.0;  // submit -> result in the dst planes
    // GPU time on the worker's stream (CUDA events): the input copies, the
    // processing, the output copies; 0 when the job failed before them
    double h2dMs = 0.0, computeMs = 0.0, d2hMs = 0.0;
    int batch = 0;           // jobs that shared this job's launch
};

struct ServeStats
{
    uint64_t submitted = 0, completed = 0, failed = 0, batches = 0, batchedJobs = 0;
    double budgetBytes = 0.0, inUseBytes = 0.0, peakBytes = 0.0, poolBytes = 0.0;
    uint64_t deviceAllocs = 0;  // device allocations of this process so far (pool and work buffers)
};

class Server
{
public:
    // `budget` caps the device bytes of admitted jobs (their frame buffers and
    // a conservative estimate of the processors' work buffers) and of the
    // buffer pool; `workers` streams; at most `maxBatch` jobs per launch.
    Server(int device, Precision precision, size_t budget, int workers, int maxBatch);
    ~Server();

    const std::string& initError() const { return initError_; }
    uint64_t submit(const ServeJob& job);
    // Waits up to `timeoutS` seconds for a job; false on timeout or unknown ticket.
    bool wait(uint64_t ticket, double timeoutS, ServeResult& out);
    ServeStats stats();

private:
    struct Block
    {
        void* ptr = nullptr;
        size_t bytes = 0;
    };
    struct Job
    {
        uint64_t id = 0;
        ServeJob job;
        size_t bytes = 0;  // admission charge
        bool batchable = false;
        bool express = false;  // small job: served by the high-priority workers
        std::string batchKey;
        double tSubmit = 0.0, tAdmit = 0.0, tStart = 0.0;
        Block blocks[6];  // src planes then dst planes
        DeviceImage dsrc[3], ddst[3];
        ServeResult result;
    };

    void admitLoop();
    void workerLoop(int w);
    // The processor of a model for small (express) or large jobs; large
    // jobs' persistent launches run one CTA per SM.
    GB300Processor* processorFor(const std::string& model, bool express, std::string& err);
    bool check(Job& j, std::string& err);
    bool allocate(Job& j, std::string& err);
    void release(Job& j);
    Block poolGet(size_t bytes, cudaError_t& err);
    void poolPut(const Block& b);
    void complete(std::unique_ptr<Job> j, int status, const std::string& err, double tDone);

    int device_ = 0;
    Precision precision_ = Precision::FP16;
    size_t budget_ = 0;
    int maxBatch_ = 64;
    std::string initError_;

    std::mutex m_;  // queues, accounting, results
    std::condition_variable cvAdmit_, cvWork_, cvDone_;
    std::deque<std::unique_ptr<Job>> pending_;  // submitted, not admitted
    std::deque<std::unique_ptr<Job>> ready_;    // admitted, device buffers assigned
    std::unordered_map<uint64_t, ServeResult> done_;
    bool admitDirty_ = false;
    size_t inUse_ = 0, peak_ = 0;
    uint64_t next_ = 1;
    ServeStats counters_;
    bool stop_ = false;

    std::mutex procMutex_;
    std::map<std::string, std::shared_ptr<Processor>> procs_;

    std::mutex poolMutex_;
    std::multimap<size_t, void*> free_;  // cached device blocks by size
    size_t poolBytes_ = 0;               // cached + handed out

    std::vector<cudaStream_t> streams_;  // one per worker
    std::vector<cudaEvent_t> events_;    // four per worker: the job's copy / processing boundaries
    int express_ = 0;                    // workers 0 .. express_-1 serve small jobs on high-priority streams
    std::thread admitter_;
    std::vector<std::thread> workers_;
};

}  // namespace acgb
