// Host side of the sample streaming: a process-wide set of pinned staging
// buffers and a pool of host threads that copy between the caller's
// (pageable) arrays and those buffers.  Pageable cudaMemcpy rates depend on
// how the caller's pages are backed (transparent huge pages copy an order of
// magnitude slower on the first and sometimes every transfer); pinned
// buffers filled by all host cores keep both directions near the link rate
// and let the DMA run asynchronously beside the sampling kernels.
#include "gcv_staging.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace gcv {

namespace {

class CopyPool {
public:
    CopyPool()
    {
        unsigned n = std::thread::hardware_concurrency();
        n = std::max(1u, std::min(n, 32u));
        for (unsigned i = 1; i < n; ++i) workers_.emplace_back([this, i] { loop(i); });
        nthreads_ = n;
    }
    ~CopyPool()
    {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }

    void copy(void* dst, const void* src, size_t n)
    {
        if (n < (8u << 20) || nthreads_ == 1) {
            std::memcpy(dst, src, n);
            return;
        }
        std::unique_lock<std::mutex> call(call_m_);  // one job at a time
        {
            std::lock_guard<std::mutex> g(m_);
            dst_ = (char*)dst;
            src_ = (const char*)src;
            n_ = n;
            pending_ = nthreads_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        part(0);
        std::unique_lock<std::mutex> g(m_);
        done_cv_.wait(g, [this] { return pending_ == 0; });
    }

private:
    void part(unsigned i)
    {
        // 64-byte aligned pieces
        const size_t per = ((n_ + nthreads_ - 1) / nthreads_ + 63) & ~size_t(63);
        const size_t a = std::min(n_, per * i), b = std::min(n_, a + per);
        if (b > a) std::memcpy(dst_ + a, src_ + a, b - a);
    }
    void loop(unsigned i)
    {
        unsigned long long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(m_);
                cv_.wait(g, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
            }
            part(i);
            {
                std::lock_guard<std::mutex> g(m_);
                if (--pending_ == 0) done_cv_.notify_one();
            }
        }
    }

    std::vector<std::thread> workers_;
    unsigned nthreads_ = 1;
    std::mutex m_, call_m_;
    std::condition_variable cv_, done_cv_;
    unsigned long long gen_ = 0;
    bool stop_ = false;
    unsigned pending_ = 0;
    char* dst_ = nullptr;
    const char* src_ = nullptr;
    size_t n_ = 0;
};

CopyPool& pool()
{
    static CopyPool p;
    return p;
}

std::mutex g_stage_m;
void* g_slot[STAGE_SLOTS] = {};
size_t g_slot_bytes[STAGE_SLOTS] = {};

}  // namespace

void host_copy(void* dst, const void* src, size_t n) { pool().copy(dst, src, n); }

std::unique_lock<std::mutex> staging_lock() { return std::unique_lock<std::mutex>(g_stage_m); }

cudaError_t staging_slot(int i, size_t bytes, void** out)
{
    if (i < 0 || i >= STAGE_SLOTS) return cudaErrorInvalidValue;
    if (g_slot_bytes[i] < bytes) {
        if (g_slot[i]) cudaFreeHost(g_slot[i]);
        g_slot[i] = nullptr;
        g_slot_bytes[i] = 0;
        cudaError_t e = cudaMallocHost(&g_slot[i], bytes);
        if (e != cudaSuccess) {
            g_slot[i] = nullptr;
            return e;
        }
        g_slot_bytes[i] = bytes;
    }
    *out = g_slot[i];
    return cudaSuccess;
}

}  // namespace gcv
