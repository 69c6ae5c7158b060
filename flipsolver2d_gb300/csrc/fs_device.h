// fs_device.h -- facts about the current CUDA device that the launchers need
// on every call (SM count, resident blocks per SM), cached per device.
//
// A process may drive several devices, and handles on different devices may
// run from different host threads.  So each fact is kept in one slot per
// device ordinal, computed with that device current on the first call there.
// Two threads that race on a first call both compute the same value; the
// slots are atomics, so the race is benign.
#ifndef FS_DEVICE_H
#define FS_DEVICE_H

#include <atomic>
#include <cuda_runtime.h>

namespace fsg {

constexpr int kMaxDevices = 64;

inline int current_device()
{
    int dev = 0;
    return cudaGetDevice(&dev) == cudaSuccess ? dev : -1;
}

// value of f() on the current device, computed once per device (f must
// return a positive value; devices beyond kMaxDevices are not cached)
template <typename F> inline int device_cached(std::atomic<int> *slots, F f)
{
    const int dev = current_device();
    if (dev < 0 || dev >= kMaxDevices) return f();
    int v = slots[dev].load(std::memory_order_relaxed);
    if (v <= 0) {
        v = f();
        slots[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

inline int device_sm_count()
{
    static std::atomic<int> slots[kMaxDevices];
    return device_cached(slots, [] {
        int sms = 0;
        const int dev = current_device();
        if (dev < 0 || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            sms < 1) {
            cudaGetLastError();
            return 1;
        }
        return sms;
    });
}

// SMs x resident blocks per SM of `fn` at `threads` threads and `smem` bytes
// of dynamic shared memory, capped at max_per_sm blocks per SM
inline int occupancy_grid(const void *fn, int threads, int max_per_sm, size_t smem = 0)
{
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        per = 1;
    }
    if (per < 1) per = 1;
    if (per > max_per_sm) per = max_per_sm;
    return device_sm_count() * per;
}

} // namespace fsg

#endif // FS_DEVICE_H
