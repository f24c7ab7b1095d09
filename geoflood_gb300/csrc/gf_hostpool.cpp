/*
 * A small persistent pool of host threads for the gathers and scatters at
 * the host-buffer boundary (patches in the caller's own storage copied into
 * and out of one pinned staging block). One core's memcpy moves about
 * 10 GB/s, well below the host-device link, so large batches split the
 * copy over the host's cores; the calling thread takes a share too.
 */
#include <algorithm>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "gf_internal.h"

namespace gf {
namespace {

class Pool {
public:
    Pool()
    {
        unsigned hc = std::thread::hardware_concurrency();
        const int n = (int)std::min<unsigned>(hc > 1 ? hc - 1 : 0, 15);
        for (int k = 0; k < n; ++k) workers_.emplace_back([this, k] { loop(k); });
    }
    ~Pool()
    {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }
    int size() const { return (int)workers_.size() + 1; }

    /* Run fn(lo, hi) over `parts` contiguous shares of [0, n); returns when
     * every share is done. Calls are serialised. */
    void run(long n, int parts, const std::function<void(long, long)>& fn)
    {
        std::lock_guard<std::mutex> one(call_);
        {
            std::lock_guard<std::mutex> g(m_);
            fn_ = &fn;
            n_ = n;
            parts_ = parts;
            next_ = 0;
            done_ = 0;
            ++gen_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> g(m_);
        done_cv_.wait(g, [this] { return done_ == parts_; });
        fn_ = nullptr;
    }

private:
    void work()
    {
        for (;;) {
            int p;
            {
                std::lock_guard<std::mutex> g(m_);
                if (!fn_ || next_ >= parts_) return;
                p = next_++;
            }
            const long lo = n_ * p / parts_, hi = n_ * (p + 1) / parts_;
            (*fn_)(lo, hi);
            std::lock_guard<std::mutex> g(m_);
            if (++done_ == parts_) done_cv_.notify_all();
        }
    }
    void loop(int)
    {
        unsigned long long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(m_);
                cv_.wait(g, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
            }
            work();
        }
    }

    std::vector<std::thread> workers_;
    std::mutex m_, call_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(long, long)>* fn_ = nullptr;
    long n_ = 0;
    int parts_ = 0, next_ = 0, done_ = 0;
    unsigned long long gen_ = 0;
    bool stop_ = false;
};

Pool& pool()
{
    static Pool p;
    return p;
}

} // namespace

void host_parallel_for(long n, long bytes, const std::function<void(long, long)>& fn)
{
    constexpr long kSerialBytes = 4L << 20; /* below this one thread is quicker */
    if (n <= 1 || bytes < kSerialBytes) {
        fn(0, n);
        return;
    }
    Pool& p = pool();
    const long by_bytes = bytes / kSerialBytes + 1;
    const int parts = (int)std::min<long>({n, (long)p.size(), by_bytes});
    if (parts <= 1) {
        fn(0, n);
        return;
    }
    p.run(n, parts, fn);
}

} // namespace gf
