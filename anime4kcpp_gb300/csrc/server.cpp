// Serving loop (see server.hpp).
//
// Threads: callers submit jobs; one admission thread moves jobs from the
// pending queue to the ready queue as the HBM budget allows (in arrival
// order, letting smaller later jobs past a job that does not fit yet unless
// that job has waited 50 ms) and gives them device frame buffers from a
// resident pool; each worker thread owns a CUDA stream and takes the next
// ready job it serves together with every other ready job it can batch with
// (ACNetLegacy x2 of interleaved images in a tensor-core form, same model,
// channel count and element type), copies the inputs in, runs one launch for
// the batch, copies the results out and synchronises its stream.  Several
// workers keep several jobs' copies and kernels in flight at once.  All but
// one in eight of the workers ("express") serve only small jobs (an input of
// at most 1920x1080) on high-priority streams, so a small job's blocks are
// scheduled ahead of the pending blocks of large jobs; the others take large
// jobs first (one or two large jobs on the device at a time) and small ones
// when no large job waits.  Copies go out in pieces
// of at most 16 MB, so a small job's copy is not queued behind a large one.
#include "server.hpp"

#include <algorithm>
#include <chrono>

namespace acgb {

namespace {

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int pitch_of(int w, int c, int type) { return (w * c * (type & 0xff) + 255) & ~255; }

size_t plane_bytes(int w, int h, int c, int type) { return static_cast<size_t>(pitch_of(w, c, type)) * h; }

size_t round_block(size_t bytes)
{
    const size_t mb = size_t(1) << 20, g = bytes <= (size_t(64) << 20) ? mb : (size_t(16) << 20);
    return std::max(mb, (bytes + g - 1) / g * g);
}

// A pitched copy issued as pieces of at most 16 MB: a copy engine serves
// the streams' copies piece by piece, so a small job's copy is not queued
// behind all of a large job's (a 7680x4320 x4 RGB result is 400 MB).
cudaError_t copy_rows(void* dst, size_t dpitch, const void* src, size_t spitch, size_t row, int rows, cudaMemcpyKind kind,
                      cudaStream_t st)
{
    const size_t piece = 16u << 20;
    const int step = static_cast<int>(std::max<size_t>(1, piece / std::max<size_t>(row, 1)));
    for (int y = 0; y < rows; y += step)
    {
        const int n = std::min(step, rows - y);
        const cudaError_t e = cudaMemcpy2DAsync(static_cast<char*>(dst) + static_cast<size_t>(y) * dpitch, dpitch,
                                                static_cast<const char*>(src) + static_cast<size_t>(y) * spitch, spitch, row, n,
                                                kind, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace

Server::Server(int device, Precision precision, size_t budget, int workers, int maxBatch)
    : device_(device), precision_(precision), budget_(budget), maxBatch_(std::max(1, std::min(maxBatch, 64)))
{
    cudaError_t err = cudaSetDevice(device_);
    if (err != cudaSuccess)
    {
        initError_ = std::string("cudaSetDevice: ") + cudaGetErrorString(err);
        return;
    }
    workers = std::max(1, std::min(workers, 16));
    // One large-job worker per eight workers (at least one): large jobs run
    // one or two at a time, so at most that much of the device is theirs
    // when a small job arrives; the rest serve small jobs.
    express_ = workers - std::max(1, workers / 8);
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) least = greatest = 0;
    for (int w = 0; w < workers; w++)
    {
        cudaStream_t s = nullptr;
        if ((err = cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, w < express_ ? greatest : least)) != cudaSuccess)
        {
            initError_ = std::string("cudaStreamCreate: ") + cudaGetErrorString(err);
            break;
        }
        streams_.push_back(s);
        for (int k = 0; k < 4; k++)
        {
            cudaEvent_t e = nullptr;
            if ((err = cudaEventCreate(&e)) != cudaSuccess)
            {
                initError_ = std::string("cudaEventCreate: ") + cudaGetErrorString(err);
                break;
            }
            events_.push_back(e);
        }
        if (!initError_.empty()) break;
    }
    if (!initError_.empty()) return;
    counters_.budgetBytes = static_cast<double>(budget_);
    admitter_ = std::thread(&Server::admitLoop, this);
    for (int w = 0; w < workers; w++) workers_.emplace_back(&Server::workerLoop, this, w);
}

Server::~Server()
{
    {
        std::lock_guard<std::mutex> lock(m_);
        stop_ = true;
    }
    cvAdmit_.notify_all();
    cvWork_.notify_all();
    if (admitter_.joinable()) admitter_.join();
    for (auto& t : workers_)
        if (t.joinable()) t.join();
    for (auto& j : ready_) release(*j);
    ready_.clear();
    pending_.clear();
    cudaSetDevice(device_);
    for (auto& kv : free_) cudaFree(kv.second);
    free_.clear();
    procs_.clear();
    for (cudaStream_t s : streams_) cudaStreamDestroy(s);
    for (cudaEvent_t e : events_) cudaEventDestroy(e);
}

GB300Processor* Server::processorFor(const std::string& model, bool express, std::string& err)
{
    std::lock_guard<std::mutex> lock(procMutex_);
    const std::string key = (express ? "s/" : "l/") + model;
    auto it = procs_.find(key);
    if (it == procs_.end())
    {
        std::shared_ptr<Processor> p = Processor::create("cuda", device_, model.c_str());
        auto* g = dynamic_cast<GB300Processor*>(p.get());
        if (!g || !g->ok())
        {
            err = p->error();
            return nullptr;
        }
        g->setPrecision(precision_);
        g->setAutotune(false);  // the default tile plan: no measurement launches in the request path
        // A large job's persistent launch would hold both CTA slots of every
        // SM until its tile queue drains; at one per SM a small job's blocks
        // start at once beside it.
        if (!express) g->setCtasPerSm(1);
        it = procs_.emplace(key, p).first;
    }
    return static_cast<GB300Processor*>(it->second.get());
}

// Validates a job and sets its admission charge: its frame buffers plus the
// work buffers its pipeline may use (the processors' per-thread buffers,
// charged per job as an upper bound).
bool Server::check(Job& j, std::string& err)
{
    const ServeJob& s = j.job;
    if (s.planes < 1 || s.planes > 3)
    {
        err = "planes must be 1 (an interleaved image) or 2..3 (planar YUV)";
        return false;
    }
    ModelSpec spec;
    if (!parse_model(s.model.c_str(), spec, err)) return false;
    if (!(s.factor > 0.0) || s.factor > 64.0)
    {
        err = "factor must be in (0, 64]";
        return false;
    }
    size_t io = 0;
    for (int p = 0; p < s.planes; p++)
    {
        const HostPlane& a = s.src[p];
        const HostPlane& b = s.dst[p];
        if (!a.ptr || !b.ptr || a.w <= 0 || a.h <= 0 || b.w <= 0 || b.h <= 0 || a.c < 1 || a.c > 4)
        {
            err = "empty or malformed plane";
            return false;
        }
        if (a.type != b.type || a.c != b.c)
        {
            err = "src and dst planes differ in element type or channels";
            return false;
        }
        if (a.stride < a.w * a.c * (a.type & 0xff) || b.stride < b.w * b.c * (b.type & 0xff))
        {
            err = "stride smaller than a row";
            return false;
        }
        io += plane_bytes(a.w, a.h, a.c, a.type) + plane_bytes(b.w, b.h, b.c, b.type);
    }
    const HostPlane& y = s.src[0];
    const int es = y.type & 0xff, c = s.planes == 1 ? y.c : 1;
    const int power = s.factor > 2.0 ? ceil_log2(s.factor) : 1;
    const double lw = static_cast<double>(y.w) * (1 << power), lh = static_cast<double>(y.h) * (1 << power);
    const bool x2 = s.factor == 2.0 && s.dst[0].w == 2 * y.w && s.dst[0].h == 2 * y.h;
    const bool fused = s.planes == 1 && spec.family == Family::ACNetLegacy && x2;
    double ws = 1 << 20;  // resize tables, counters
    if (!fused)
    {
        if (c > 1) ws += static_cast<double>(y.w) * y.h * c * es;  // Y + UV(A) split
        ws += 2.0 * lw * lh * es;                                     // the luma ping-pong planes
        if (spec.family != Family::ACNetLegacy)  // work maps of the last pass
            ws += 4.0 * (lw / 2) * (lh / 2) * 4.0 * (spec.channels > 8 ? spec.channels : 8);
        if (s.planes > 1) ws += static_cast<double>(y.w) * y.h * es;  // shifted Y
    }
    j.bytes = io + static_cast<size_t>(ws);
    j.batchable = fused && precision_ != Precision::FP32;
    // Small jobs -- an input of at most 1920x1080 (any model, factor and
    // format) -- are served by the express workers on high-priority streams,
    // so their kernels are scheduled ahead of pending blocks of large jobs.
    const double inPx = static_cast<double>(y.w) * y.h;
    j.express = inPx <= 1920.0 * 1080.0;
    // jobs batch with jobs of their own class (a large job would slow an
    // express batch down)
    j.batchKey = std::string(j.express ? "s/" : "l/") + s.model + "/" + std::to_string(y.c) + "/" + std::to_string(y.type);
    return true;
}

Server::Block Server::poolGet(size_t bytes, cudaError_t& err)
{
    err = cudaSuccess;
    const size_t r = round_block(bytes);
    std::lock_guard<std::mutex> lock(poolMutex_);
    auto it = free_.lower_bound(r);
    if (it != free_.end() && it->first <= 2 * r)
    {
        Block b{it->second, it->first};
        free_.erase(it);
        return b;
    }
    // keep the pool under the budget: drop cached blocks, largest first
    while (poolBytes_ + r > budget_ && !free_.empty())
    {
        auto big = std::prev(free_.end());
        cudaFree(big->second);
        poolBytes_ -= big->first;
        free_.erase(big);
    }
    void* p = nullptr;
    if (injected_alloc_failure())
    {
        err = cudaErrorMemoryAllocation;
        return Block{};
    }
    if ((err = cudaMalloc(&p, r)) != cudaSuccess) return Block{};
    device_alloc_count().fetch_add(1, std::memory_order_relaxed);
    poolBytes_ += r;
    return Block{p, r};
}

void Server::poolPut(const Block& b)
{
    if (!b.ptr) return;
    std::lock_guard<std::mutex> lock(poolMutex_);
    free_.emplace(b.bytes, b.ptr);
}

bool Server::allocate(Job& j, std::string& err)
{
    const ServeJob& s = j.job;
    for (int p = 0; p < s.planes; p++)
    {
        const HostPlane* pl[2] = {&s.src[p], &s.dst[p]};
        for (int k = 0; k < 2; k++)
        {
            const HostPlane& h = *pl[k];
            cudaError_t e;
            Block b = poolGet(plane_bytes(h.w, h.h, h.c, h.type), e);
            if (!b.ptr)
            {
                err = std::string("device allocation: ") + cudaGetErrorString(e);
                release(j);
                return false;
            }
            j.blocks[k * 3 + p] = b;
            DeviceImage d{b.ptr, h.w, h.h, h.c, pitch_of(h.w, h.c, h.type), h.type};
            (k == 0 ? j.dsrc : j.ddst)[p] = d;
        }
    }
    return true;
}

void Server::release(Job& j)
{
    for (Block& b : j.blocks)
    {
        poolPut(b);
        b = Block{};
    }
}

uint64_t Server::submit(const ServeJob& job)
{
    auto j = std::make_unique<Job>();
    j->job = job;
    j->tSubmit = now_s();
    std::string err = initError_;
    const bool good = err.empty() && check(*j, err);
    std::lock_guard<std::mutex> lock(m_);
    j->id = next_++;
    const uint64_t id = j->id;
    counters_.submitted++;
    if (!good)
    {
        ServeResult r;
        r.status = -2;
        r.error = err;
        done_[id] = r;
        counters_.failed++;
        cvDone_.notify_all();
        return id;
    }
    pending_.push_back(std::move(j));
    admitDirty_ = true;
    cvAdmit_.notify_one();
    return id;
}

bool Server::wait(uint64_t ticket, double timeoutS, ServeResult& out)
{
    std::unique_lock<std::mutex> lock(m_);
    auto ready = [&] { return done_.count(ticket) != 0; };
    if (!cvDone_.wait_for(lock, std::chrono::duration<double>(std::max(0.0, timeoutS)), ready)) return false;
    auto it = done_.find(ticket);
    out = std::move(it->second);
    done_.erase(it);
    return true;
}

ServeStats Server::stats()
{
    ServeStats s;
    {
        std::lock_guard<std::mutex> lock(m_);
        s = counters_;
        s.inUseBytes = static_cast<double>(inUse_);
        s.peakBytes = static_cast<double>(peak_);
    }
    std::lock_guard<std::mutex> lock(poolMutex_);
    s.poolBytes = static_cast<double>(poolBytes_);
    s.deviceAllocs = device_alloc_count().load(std::memory_order_relaxed);
    return s;
}

void Server::complete(std::unique_ptr<Job> j, int status, const std::string& err, double tDone)
{
    ServeResult r = j->result;
    r.status = status;
    r.error = err;
    if (j->tAdmit > 0.0) r.queueMs = (j->tAdmit - j->tSubmit) * 1e3;
    if (j->tStart > 0.0) r.deviceMs = (tDone - j->tStart) * 1e3;
    r.latencyMs = (tDone - j->tSubmit) * 1e3;
    std::lock_guard<std::mutex> lock(m_);
    if (j->tAdmit > 0.0)
    {
        inUse_ -= j->bytes;
        admitDirty_ = true;
        cvAdmit_.notify_one();
    }
    if (status == 0) counters_.completed++;
    else counters_.failed++;
    done_[j->id] = std::move(r);
    cvDone_.notify_all();
}

void Server::admitLoop()
{
    cudaSetDevice(device_);
    for (;;)
    {
        std::vector<std::unique_ptr<Job>> admitted, rejected;
        double t = 0.0;
        {
            std::unique_lock<std::mutex> lock(m_);
            cvAdmit_.wait(lock, [&] { return stop_ || admitDirty_; });
            if (stop_) return;
            admitDirty_ = false;
            t = now_s();
            for (auto it = pending_.begin(); it != pending_.end();)
            {
                Job& j = **it;
                if (j.bytes > budget_)
                {
                    rejected.push_back(std::move(*it));
                    it = pending_.erase(it);
                }
                else if (inUse_ + j.bytes <= budget_)
                {
                    inUse_ += j.bytes;
                    peak_ = std::max(peak_, inUse_);
                    j.tAdmit = t;
                    admitted.push_back(std::move(*it));
                    it = pending_.erase(it);
                }
                else if (t - j.tSubmit > 0.05)
                    break;  // a job waiting 50 ms holds the later ones back until it fits
                else
                    ++it;
            }
        }
        for (auto& j : rejected)
        {
            const std::string msg = "job needs " + std::to_string(j->bytes) + " device bytes, more than the HBM budget of " +
                                    std::to_string(budget_);
            complete(std::move(j), -2, msg, t);
        }
        for (auto& j : admitted)
        {
            std::string err;
            if (!allocate(*j, err))
            {
                complete(std::move(j), -1, err, now_s());
                continue;
            }
            std::lock_guard<std::mutex> lock(m_);
            ready_.push_back(std::move(j));
            cvWork_.notify_all();  // the workers differ in which jobs they take
        }
    }
}

void Server::workerLoop(int w)
{
    cudaSetDevice(device_);
    cudaStream_t st = streams_[w];
    for (;;)
    {
        std::vector<std::unique_ptr<Job>> batch;
        {
            std::unique_lock<std::mutex> lock(m_);
            // express workers take small jobs only; the others large jobs first
            const bool express = w < express_;
            auto pick = [&]() {
                auto it = ready_.begin();
                if (express)
                {
                    while (it != ready_.end() && !(*it)->express) ++it;
                    return it;
                }
                auto big = std::find_if(ready_.begin(), ready_.end(), [](const std::unique_ptr<Job>& j) { return !j->express; });
                return big != ready_.end() ? big : ready_.begin();
            };
            cvWork_.wait(lock, [&] { return stop_ || pick() != ready_.end(); });
            if (stop_) return;
            auto first = pick();
            batch.push_back(std::move(*first));
            ready_.erase(first);
            if (batch[0]->batchable)
                for (auto it = ready_.begin(); it != ready_.end() && static_cast<int>(batch.size()) < maxBatch_;)
                {
                    if ((*it)->batchable && (*it)->batchKey == batch[0]->batchKey)
                    {
                        batch.push_back(std::move(*it));
                        it = ready_.erase(it);
                    }
                    else
                        ++it;
                }
            if (batch.size() > 1)
            {
                counters_.batches++;
                counters_.batchedJobs += batch.size();
            }
        }
        const double t0 = now_s();
        const int n = static_cast<int>(batch.size());
        for (auto& j : batch)
        {
            j->tStart = t0;
            j->result.batch = n;
        }
        std::string err;
        cudaError_t e = cudaSuccess;
        GB300Processor* proc = processorFor(batch[0]->job.model, batch[0]->express, err);
        cudaEvent_t* ev = events_.data() + 4 * w;
        bool timed = cudaEventRecord(ev[0], st) == cudaSuccess;
        for (auto& j : batch)
            for (int p = 0; p < j->job.planes && e == cudaSuccess; p++)
            {
                const HostPlane& h = j->job.src[p];
                e = copy_rows(j->dsrc[p].ptr, j->dsrc[p].stride, h.ptr, h.stride,
                              static_cast<size_t>(h.w) * h.c * (h.type & 0xff), h.h, cudaMemcpyHostToDevice, st);
            }
        int rc = proc ? 0 : -1;
        timed = timed && cudaEventRecord(ev[1], st) == cudaSuccess;
        if (proc && e == cudaSuccess)
        {
            const ServeJob& s0 = batch[0]->job;
            if (batch[0]->batchable)
            {
                std::vector<DeviceImage> src(n), dst(n);
                for (int i = 0; i < n; i++)
                {
                    src[i] = batch[i]->dsrc[0];
                    dst[i] = batch[i]->ddst[0];
                }
                rc = proc->processBatchDevice(n, src.data(), dst.data(), 2.0, st, false);
            }
            else if (s0.planes == 1)
                rc = proc->processDevice(batch[0]->dsrc[0], batch[0]->ddst[0], s0.factor, st, false);
            else
                rc = proc->processYuvDevice(1, s0.planes, batch[0]->dsrc, batch[0]->ddst, s0.factor, s0.shift, st, false);
            if (rc != 0) err = proc->error();
        }
        timed = timed && cudaEventRecord(ev[2], st) == cudaSuccess;
        if (rc == 0)
            for (auto& j : batch)
                for (int p = 0; p < j->job.planes && e == cudaSuccess; p++)
                {
                    const HostPlane& h = j->job.dst[p];
                    e = copy_rows(h.ptr, h.stride, j->ddst[p].ptr, j->ddst[p].stride,
                                  static_cast<size_t>(h.w) * h.c * (h.type & 0xff), h.h, cudaMemcpyDeviceToHost, st);
                }
        timed = timed && cudaEventRecord(ev[3], st) == cudaSuccess;
        const bool tc = precision_ != Precision::FP32;
        if (tc && e == cudaSuccess) e = tc_status_enqueue(st);
        const cudaError_t se = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = se;
        if (e != cudaSuccess && err.empty()) err = std::string("CUDA: ") + cudaGetErrorString(e);
        if (e == cudaSuccess && rc == 0 && tc && tc_status_take() != 0)
        {
            rc = -1;
            err = "tensor-core wait timed out";
        }
        const double t1 = now_s();
        float part[3] = {0.0f, 0.0f, 0.0f};
        if (timed && e == cudaSuccess && rc == 0)
            for (int k = 0; k < 3; k++)
                if (cudaEventElapsedTime(&part[k], ev[k], ev[k + 1]) != cudaSuccess) part[k] = 0.0f;
        for (auto& j : batch)
        {
            j->result.h2dMs = part[0];
            j->result.computeMs = part[1];
            j->result.d2hMs = part[2];
            release(*j);
            complete(std::move(j), (e == cudaSuccess && rc == 0) ? 0 : -1, err, t1);
        }
    }
}

}  // namespace acgb
