// Pre-faulting of freshly malloc'd host output buffers.
//
// The reference API returns its outputs in malloc'd memory
// (szx/src/szx_float.cc:1413, szx/src/szxd_float.cc:442), so every call's
// device->host copy lands in pages that do not exist yet.  The kernel then
// faults them in one page at a time from the copying thread, which on a Grace
// host runs at ~15 GB/s -- several times slower than the copy itself
// (~190 GB/s over NVLink-C2C).  Faulting the pages in from a few host threads
// while the GPU is still busy with the call takes that cost off the critical
// path: the copy then writes resident pages.
//
// Pages are handed out in ascending chunks from an atomic cursor, so when the
// caller learns that it needs fewer bytes than it asked for (a compressed
// stream is shorter than its bound) the work beyond that point is skipped.
// Each chunk is flagged when its pages are in, so the caller can copy the
// front of the buffer while the workers are still faulting in the back.
//
// Measured on a Grace host (64 KiB pages, 512 MiB buffer): touching one byte
// per page from 8 threads faults ~125 GB/s (16 threads are no faster);
// madvise(MADV_POPULATE_WRITE) is slower (35-85 GB/s) and leaves pages that
// the copy engine then writes at ~30 GB/s instead of ~140 GB/s.
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "kernels.h"

namespace szxg {

namespace {

constexpr size_t kTouchChunk = size_t(4) << 20;   // bytes a worker claims at a time

class Toucher {
   public:
    static Toucher& get() {
        static Toucher* t = new Toucher();   // never destroyed: workers outlive static destruction
        return *t;
    }

    void start(void* p, size_t n) {
        job_mu_.lock();   // one job at a time; released by finish()
        const size_t nc = (n + kTouchChunk - 1) / kTouchChunk;
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (nc > ready_cap_) {
                ready_.reset(new std::atomic<unsigned char>[nc]);
                ready_cap_ = nc;
            }
            for (size_t i = 0; i < nc; i++) ready_[i].store(0, std::memory_order_relaxed);
            base_ = (volatile char*)p;
            limit_.store(n);
            cursor_.store(0);
            busy_ = (int)workers_.size();
            gen_++;
        }
        cv_.notify_all();
    }

    // Lower the job's extent to n bytes (never raises it).
    void limit(size_t n) {
        size_t cur = limit_.load();
        while (n < cur && !limit_.compare_exchange_weak(cur, n)) {
        }
    }

    // Wait until every page below byte hi (within the job's extent) is resident.
    void wait(size_t hi) {
        const size_t lim = limit_.load();
        if (hi > lim) hi = lim;
        const size_t nc = (hi + kTouchChunk - 1) / kTouchChunk;
        std::unique_lock<std::mutex> lk(mu_);
        ready_cv_.wait(lk, [&] {
            while (waited_ < nc && ready_[waited_].load(std::memory_order_acquire)) waited_++;
            return waited_ >= nc || busy_ == 0;
        });
    }

    // Lower the job's extent to n bytes, wait until every page below it is resident.
    void finish(size_t n) {
        limit(n);
        {
            std::unique_lock<std::mutex> lk(mu_);
            done_cv_.wait(lk, [&] { return busy_ == 0; });
            waited_ = 0;
        }
        job_mu_.unlock();
    }

   private:
    Toucher() {
        page_ = (size_t)sysconf(_SC_PAGESIZE);
        if (page_ == 0 || page_ > kTouchChunk) page_ = 4096;
        unsigned hw = std::thread::hardware_concurrency();
        const unsigned nw = std::max(1u, std::min(8u, hw ? hw : 1u));
        for (unsigned i = 0; i < nw; i++) workers_.emplace_back([this] { run(); });
        for (auto& w : workers_) w.detach();
    }

    void run() {
        unsigned long long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
            }
            for (;;) {
                const size_t lo = cursor_.fetch_add(kTouchChunk);
                const size_t lim = limit_.load();
                if (lo >= lim) break;
                const size_t hi = std::min(lo + kTouchChunk, lim);
                for (size_t i = lo; i < hi; i += page_) base_[i] = 0;
                base_[hi - 1] = 0;
                {
                    std::lock_guard<std::mutex> lk(mu_);
                    ready_[lo / kTouchChunk].store(1, std::memory_order_release);
                }
                ready_cv_.notify_all();
            }
            {
                std::lock_guard<std::mutex> lk(mu_);
                if (--busy_ == 0) done_cv_.notify_all();
            }
            ready_cv_.notify_all();
        }
    }

    std::mutex job_mu_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_, ready_cv_;
    std::unique_ptr<std::atomic<unsigned char>[]> ready_;   // per chunk: pages resident
    size_t ready_cap_ = 0;
    size_t waited_ = 0;                                      // chunks the caller has seen ready
    std::vector<std::thread> workers_;
    volatile char* base_ = nullptr;
    std::atomic<size_t> limit_{0}, cursor_{0};
    size_t page_ = 4096;
    int busy_ = 0;
    unsigned long long gen_ = 0;
};

}  // namespace

void host_prefault_start(void* p, size_t n) { Toucher::get().start(p, n); }
void host_prefault_limit(size_t n) { Toucher::get().limit(n); }
void host_prefault_wait(size_t hi) { Toucher::get().wait(hi); }
void host_prefault_finish(size_t n) { Toucher::get().finish(n); }

}  // namespace szxg
