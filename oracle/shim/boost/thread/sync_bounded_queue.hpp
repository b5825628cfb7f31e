// Mutex + condition-variable bounded queue with the push_back / pull_front
// calls the reference's swap pipeline makes. Oracle build only.
#pragma once
#include <condition_variable>
#include <cstddef>
#include <deque>
#include <mutex>

namespace boost {
template <class T>
class sync_bounded_queue {
public:
    explicit sync_bounded_queue(std::size_t cap) : cap_(cap) {}
    void push_back(const T& v) {
        std::unique_lock<std::mutex> lk(m_);
        not_full_.wait(lk, [&] { return q_.size() < cap_; });
        q_.push_back(v);
        not_empty_.notify_one();
    }
    T pull_front() {
        std::unique_lock<std::mutex> lk(m_);
        not_empty_.wait(lk, [&] { return !q_.empty(); });
        T v = q_.front();
        q_.pop_front();
        not_full_.notify_one();
        return v;
    }
    void pull_front(T& out) { out = pull_front(); }

private:
    std::size_t cap_;
    std::deque<T> q_;
    std::mutex m_;
    std::condition_variable not_empty_, not_full_;
};
}  // namespace boost
