// Stand-in for tbb::spin_mutex (oracle-only test infrastructure).
#pragma once
#include <mutex>
namespace tbb {
class spin_mutex {
public:
    void lock() { m_.lock(); }
    void unlock() { m_.unlock(); }
    class scoped_lock {
    public:
        scoped_lock() : m_(nullptr) {}
        explicit scoped_lock(spin_mutex& m) : m_(&m) { m_->lock(); }
        ~scoped_lock() { if (m_) m_->unlock(); }
        void acquire(spin_mutex& m) { m_ = &m; m_->lock(); }
        void release() { if (m_) { m_->unlock(); m_ = nullptr; } }
    private:
        spin_mutex* m_;
    };
private:
    std::mutex m_;
};
}  // namespace tbb
