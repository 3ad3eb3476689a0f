// attr_cache.h -- kernel attributes raised once per (device, size).
//
// cudaFuncSetAttribute(cudaFuncAttributeMaxDynamicSharedMemorySize) sets the
// attribute on the CURRENT device only: a process that drives several GPUs
// must raise it on each one before the kernel's first launch there with that
// much dynamic shared memory.  AttrCache remembers, per device, the largest
// size raised so far.  The raise itself runs under a lock, so host threads
// that launch at the same time (a request server's scheduler thread and
// direct callers, or threads driving different GPUs) neither race on the
// record nor skip a raise another thread has not finished.  A raise that
// fails is not recorded, so the next launch tries again.
//
// Header-only and free of CUDA types: the host tests compile it with g++
// and drive it with a fake setter.
#pragma once
#include <atomic>
#include <cstddef>
#include <mutex>

namespace vg {

constexpr int kMaxDevices = 64;

class AttrCache {
 public:
  // Make sure the attribute is at least `bytes` on device `dev`: calls
  // set(bytes) (0 = success) unless a size >= bytes was raised there
  // already.  Returns 0 or set()'s error.  Devices outside [0, kMaxDevices)
  // are raised on every call.
  template <class Set>
  int ensure(int dev, size_t bytes, Set&& set) {
    if (dev < 0 || dev >= kMaxDevices) return set(bytes);
    if (raised_[dev].load(std::memory_order_acquire) >= bytes) return 0;   // fast path
    std::lock_guard<std::mutex> g(mu_);
    if (raised_[dev].load(std::memory_order_relaxed) >= bytes) return 0;
    const int rc = set(bytes);
    if (rc == 0) raised_[dev].store(bytes, std::memory_order_release);
    return rc;
  }
  size_t raised(int dev) const {
    return dev >= 0 && dev < kMaxDevices ? raised_[dev].load(std::memory_order_acquire) : 0;
  }

 private:
  std::mutex mu_;
  std::atomic<size_t> raised_[kMaxDevices] = {};
};

}  // namespace vg
