// Host emulation of one CUDA lane group (test infrastructure only).
//
// Runs a device function on `width` host threads (a warp, or the S-lane group
// of a lane-group kernel: width 4, 8, 16 or 32), one per lane, and provides
// the warp intrinsics the device code uses -- __shfl_sync, __shfl_xor_sync,
// __ballot_sync, __any_sync, __all_sync, __syncwarp, __activemask and a
// per-lane threadIdx -- so that a kernel's lane form can be compared on the
// CPU with the sequential form it replaces.  Every intrinsic is a rendezvous
// of all the lanes: a lane that does not arrive (the lanes took different
// paths, which on the GPU would leave a shuffle waiting) makes the rendezvous
// time out, and the run reports the divergence instead of hanging.  So does
// an intrinsic whose mask is not the whole group.
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
    explicit Warp(int width) : width_(width) {}
    int width() const { return width_; }
    unsigned mask() const { return width_ == 32 ? 0xffffffffu : (1u << width_) - 1u; }
    // Waits until every lane has arrived; false when they do not within
    // `limit` (divergent lanes) or an earlier rendezvous already failed.
    // Lanes wait by yielding, which on a host with fewer cores than lanes
    // hands the core to the lanes still on their way.
    bool rendezvous(std::chrono::milliseconds limit = std::chrono::milliseconds(20000)) {
        if (failed_.load(std::memory_order_acquire)) return false;
        const unsigned generation = generation_.load(std::memory_order_acquire);
        if (arrived_.fetch_add(1, std::memory_order_acq_rel) + 1 == width_) {
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
    void fail() { failed_.store(true, std::memory_order_release); }
    bool failed() const { return failed_.load(std::memory_order_acquire); }
    uint64_t slot[kLanes] = {};
    long exchanges = 0;  // intrinsics completed (counted by lane 0)

  private:
    int width_;
    std::atomic<int> arrived_{0};
    std::atomic<unsigned> generation_{0};
    std::atomic<bool> failed_{false};
};

inline thread_local Warp* t_warp = nullptr;
inline thread_local int t_lane = 0;

// Every lane publishes `bits`, then reads all lanes' words through `read`.
template <class Read>
auto exchange(unsigned mask, uint64_t bits, Read&& read) -> decltype(read(static_cast<const uint64_t*>(nullptr))) {
    Warp& w = *t_warp;
    if (mask != w.mask()) w.fail();  // a mask other than the whole group is not emulated
    w.slot[t_lane] = bits;
    if (!w.rendezvous()) return read(w.slot);
    auto out = read(w.slot);
    if (t_lane == 0) ++w.exchanges;
    w.rendezvous();  // no lane writes its slot again before every lane has read
    return out;
}

template <class T>
T shuffle_from(unsigned mask, T v, int src_of_lane) {
    static_assert(sizeof(T) <= sizeof(uint64_t), "shuffle of a value wider than 64 bits");
    uint64_t bits = 0;
    std::memcpy(&bits, &v, sizeof(T));
    const int src = src_of_lane & (t_warp->width() - 1);
    return exchange(mask, bits, [&](const uint64_t* slots) {
        T out;
        std::memcpy(&out, &slots[src], sizeof(T));
        return out;
    });
}

inline unsigned ballot(unsigned mask, bool p) {
    return exchange(mask, p ? 1u : 0u, [&](const uint64_t* slots) {
        unsigned b = 0;
        for (int l = 0; l < t_warp->width(); ++l)
            if (slots[l]) b |= 1u << l;
        return b;
    });
}

// Runs body(lane) on `width` threads sharing one lane group; returns false if
// the lanes diverged at an intrinsic.  `exchanges` receives the number of
// intrinsics the group completed.
template <class Body>
bool run(int width, Body&& body, long* exchanges = nullptr);

}  // namespace warp_emu

inline thread_local HostDim3 threadIdx{0, 0, 0};
inline thread_local HostDim3 blockDim{warp_emu::kLanes, 1, 1};
inline void __syncthreads() {}
inline unsigned __activemask() { return warp_emu::t_warp ? warp_emu::t_warp->mask() : 1u; }
template <class T>
inline T __shfl_sync(unsigned mask, T v, int src, int width = 32) {
    (void)width;
    return warp_emu::shuffle_from(mask, v, src);
}
template <class T>
inline T __shfl_xor_sync(unsigned mask, T v, int lane_mask, int width = 32) {
    (void)width;
    return warp_emu::shuffle_from(mask, v, warp_emu::t_lane ^ lane_mask);
}
inline unsigned __ballot_sync(unsigned mask, bool p) { return warp_emu::ballot(mask, p); }
inline bool __any_sync(unsigned mask, bool p) { return warp_emu::ballot(mask, p) != 0; }
inline bool __all_sync(unsigned mask, bool p) { return warp_emu::ballot(mask, p) == warp_emu::t_warp->mask(); }
inline void __syncwarp(unsigned mask = 0xffffffffu) {
    if (mask == 0xffffffffu) mask = warp_emu::t_warp->mask();  // the whole (emulated) group
    warp_emu::ballot(mask, true);
}

template <class Body>
bool warp_emu::run(int width, Body&& body, long* exchanges) {
    Warp w(width);
    std::vector<std::thread> lanes;
    lanes.reserve(width);
    for (int lane = 0; lane < width; ++lane)
        lanes.emplace_back([&, lane] {
            t_warp = &w;
            t_lane = lane;
            threadIdx = HostDim3{static_cast<unsigned>(lane), 0, 0};
            blockDim = HostDim3{static_cast<unsigned>(width), 1, 1};
            body(lane);
        });
    for (auto& t : lanes) t.join();
    if (exchanges) *exchanges = w.exchanges;
    return !w.failed();
}
