// Host emulation of one CUDA warp (test infrastructure only).
//
// Runs a device function on 32 host threads, one per lane, and provides the
// warp intrinsics the device code uses -- __shfl_sync, __activemask and a
// per-lane threadIdx -- so that a kernel's warp form can be compared on the
// CPU with the sequential form it replaces.  Every intrinsic is a rendezvous
// of all 32 lanes: a lane that does not arrive (the lanes took different
// paths, which on the GPU would leave a full-mask shuffle waiting) makes the
// rendezvous time out and the run report the divergence instead of hanging.
#pragma once

#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

struct HostDim3 {
    unsigned x, y, z;
};

namespace warp_emu {

constexpr int kLanes = 32;

class Warp {
  public:
    // Waits until all 32 lanes have arrived; false when they do not within
    // `limit` (divergent lanes) or an earlier rendezvous already failed.
    // Lanes wait by yielding, which on a host with fewer cores than lanes
    // hands the core to the lanes still on their way.
    bool rendezvous(std::chrono::milliseconds limit = std::chrono::milliseconds(20000)) {
        if (failed_.load(std::memory_order_acquire)) return false;
        const unsigned generation = generation_.load(std::memory_order_acquire);
        if (arrived_.fetch_add(1, std::memory_order_acq_rel) + 1 == kLanes) {
            arrived_.store(0, std::memory_order_relaxed);
            generation_.store(generation + 1, std::memory_order_release);
            return true;
        }
        const auto deadline = std::chrono::steady_clock::now() + limit;
        for (unsigned spin = 1;; ++spin) {
            if (generation_.load(std::memory_order_acquire) != generation) return true;
            if (failed_.load(std::memory_order_acquire)) return false;
            if ((spin & 1023u) == 0 && std::chrono::steady_clock::now() > deadline) {
                failed_.store(true, std::memory_order_release);
                return false;
            }
            std::this_thread::yield();
        }
    }
    bool failed() const { return failed_.load(std::memory_order_acquire); }
    uint64_t slot[kLanes] = {};
    long exchanges = 0;  // shuffles completed (counted by lane 0)

  private:
    std::atomic<int> arrived_{0};
    std::atomic<unsigned> generation_{0};
    std::atomic<bool> failed_{false};
};

inline thread_local Warp* t_warp = nullptr;
inline thread_local int t_lane = 0;

// Lane `src`'s value of v, read by every lane.
template <class T>
T shuffle(T v, int src) {
    static_assert(sizeof(T) <= sizeof(uint64_t), "shuffle of a value wider than 64 bits");
    Warp& w = *t_warp;
    uint64_t bits = 0;
    std::memcpy(&bits, &v, sizeof(T));
    w.slot[t_lane] = bits;
    if (!w.rendezvous()) return v;
    T out;
    const uint64_t got = w.slot[src & (kLanes - 1)];
    std::memcpy(&out, &got, sizeof(T));
    if (t_lane == 0) ++w.exchanges;
    w.rendezvous();  // no lane writes its slot again before every lane has read
    return out;
}

// Runs body(lane) on 32 threads sharing one warp; returns false if the lanes
// diverged at an intrinsic.  `exchanges` receives the number of shuffles.
template <class Body>
bool run(Body&& body, long* exchanges = nullptr);

}  // namespace warp_emu

inline thread_local HostDim3 threadIdx{0, 0, 0};
inline HostDim3 blockDim{warp_emu::kLanes, 1, 1};
inline void __syncthreads() {}
inline unsigned __activemask() { return 0xffffffffu; }
template <class T>
inline T __shfl_sync(unsigned, T v, int src) {
    return warp_emu::shuffle(v, src);
}

template <class Body>
bool warp_emu::run(Body&& body, long* exchanges) {
    Warp w;
    std::vector<std::thread> lanes;
    lanes.reserve(kLanes);
    for (int lane = 0; lane < kLanes; ++lane)
        lanes.emplace_back([&, lane] {
            t_warp = &w;
            t_lane = lane;
            threadIdx = HostDim3{static_cast<unsigned>(lane), 0, 0};
            body(lane);
        });
    for (auto& t : lanes) t.join();
    if (exchanges) *exchanges = w.exchanges;
    return !w.failed();
}
