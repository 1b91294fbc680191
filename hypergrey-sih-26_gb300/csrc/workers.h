// Host worker pool of the submission path: the input scan of every submitted problem and the
// CSR builder run their pieces on it.  hardware_concurrency - 1 threads start on first use and
// live for the process.  run(pieces, fn) hands pieces out through an atomic counter and the
// calling thread takes pieces too, so a thread that shares its core with another busy thread
// (the engine thread waiting on a launch, another caller) takes fewer pieces instead of holding
// up the others, and no threads are started per call.  Several callers may run at once; their
// tasks queue and the workers help them in turn.  In a child process after fork() the workers
// do not exist, and run() works through every piece on the calling thread.
#pragma once

#include <pthread.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <functional>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

namespace bqp {

class WorkerPool {
public:
    static WorkerPool& get() {
        static WorkerPool* pool = new WorkerPool;  // never destroyed: the workers outlive main()
        return *pool;
    }

    // threads that may work on one task, the caller included
    int threads() const { return workers_ + 1; }

    // fn(p) for p in [0, pieces), each piece once, on the workers and the calling thread
    void run(int64_t pieces, const std::function<void(int64_t)>& fn) {
        if (pieces <= 0) return;
        if (pieces == 1 || workers_ == 0 || forked_child().load(std::memory_order_relaxed)) {
            for (int64_t p = 0; p < pieces; ++p) fn(p);
            return;
        }
        Task t;
        t.fn = &fn;
        t.pieces = pieces;
        {
            std::lock_guard<std::mutex> g(mu_);
            tasks_.push_back(&t);
            t.users = 1;
        }
        cv_.notify_all();
        work(t);
        std::unique_lock<std::mutex> lk(mu_);
        auto it = std::find(tasks_.begin(), tasks_.end(), &t);
        if (it != tasks_.end()) tasks_.erase(it);
        --t.users;
        // no new user can take the task now; the ones that took it finish their pieces
        done_.wait(lk, [&] { return t.users == 0; });
        if (t.failed) throw std::bad_alloc();
    }

private:
    struct Task {
        const std::function<void(int64_t)>* fn = nullptr;
        int64_t pieces = 0;
        std::atomic<int64_t> next{0};
        int users = 0;  // threads working on the task (under mu_)
        bool failed = false;
    };

    WorkerPool() {
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        workers_ = static_cast<int>(std::min(hw, 64u)) - 1;
        pthread_atfork(nullptr, nullptr, [] { forked_child().store(true); });
        for (int w = 0; w < workers_; ++w) std::thread([this] { loop(); }).detach();
    }

    static std::atomic<bool>& forked_child() {
        static std::atomic<bool> flag{false};
        return flag;
    }

    void work(Task& t) {
        bool failed = false;
        for (;;) {
            const int64_t p = t.next.fetch_add(1, std::memory_order_relaxed);
            if (p >= t.pieces) break;
            try {
                (*t.fn)(p);
            } catch (...) {
                failed = true;
            }
        }
        if (failed) {
            std::lock_guard<std::mutex> g(mu_);
            t.failed = true;
        }
    }

    void loop() {
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_.wait(lk, [&] { return !tasks_.empty(); });
            Task* t = tasks_.front();
            ++t->users;
            lk.unlock();
            work(*t);
            lk.lock();
            // every piece of t is taken: later workers go to the next task
            if (!tasks_.empty() && tasks_.front() == t) tasks_.pop_front();
            if (--t->users == 0) done_.notify_all();
        }
    }

    int workers_ = 0;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    std::deque<Task*> tasks_;
};

}  // namespace bqp
