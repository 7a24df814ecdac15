// Host emulation of CUDA kernel launches (test infrastructure only).
//
// Runs a kernel's blocks one after another on the host, each block as
// blockDim.x threads with their own threadIdx / blockIdx, and provides the
// device intrinsics the batched flash pipeline uses: __syncthreads (a block
// barrier), the warp shuffles, votes and reductions (a rendezvous of the lanes
// named by the mask, grouped per warp), atomicAdd, and the few bit and cast
// builtins.  __activemask() returns the calling lane alone: the pipeline asks
// it only to aggregate statistics, which then add lane by lane.  A rendezvous
// that a lane never reaches times out and marks the run failed instead of
// hanging.  The CUDA runtime calls of the orchestration are stubs that act on
// host memory (memsets) or do nothing (events, stream waits): every launch
// runs to completion in program order.
//
// Include it before any CUDA header of the code under test (g++ -include).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <thread>
#include <vector>

using std::isfinite;

#undef __shared__
#define __shared__ static  // one block runs at a time
#define __launch_bounds__(...)
#ifndef __noinline__
#define __noinline__ __attribute__((noinline))
#endif

// the integer min / max device code calls unqualified
template <class T>
inline T min(T a, T b) {
    return b < a ? b : a;
}
template <class T>
inline T max(T a, T b) {
    return a < b ? b : a;
}

struct EmuDim3 {
    unsigned x = 1, y = 1, z = 1;
};

inline thread_local EmuDim3 threadIdx, blockIdx, blockDim, gridDim;

namespace cuda_emu {

inline std::atomic<bool> g_failed{false};
inline std::atomic<long> g_rendezvous{0};

class Barrier {
  public:
    void reset(int count) {
        count_ = count;
        arrived_.store(0);
        generation_.store(0);
    }
    bool wait() {
        if (g_failed.load(std::memory_order_acquire)) return false;
        const unsigned generation = generation_.load(std::memory_order_acquire);
        if (arrived_.fetch_add(1, std::memory_order_acq_rel) + 1 == count_) {
            arrived_.store(0, std::memory_order_relaxed);
            generation_.store(generation + 1, std::memory_order_release);
            return true;
        }
        const auto deadline = std::chrono::steady_clock::now() + std::chrono::seconds(30);
        for (unsigned spin = 1;; ++spin) {
            if (generation_.load(std::memory_order_acquire) != generation) return true;
            if (g_failed.load(std::memory_order_acquire)) return false;
            if ((spin & 1023u) == 0 && std::chrono::steady_clock::now() > deadline) {
                g_failed.store(true, std::memory_order_release);
                return false;
            }
            std::this_thread::yield();
        }
    }

  private:
    int count_ = 1;
    std::atomic<int> arrived_{0};
    std::atomic<unsigned> generation_{0};
};

// The rendezvous of one mask's lanes within a warp: the mask's lowest lane and
// its lane count identify it.
struct Group {
    Barrier bar;
    uint64_t slot[32] = {};
};

struct Block {
    explicit Block(int threads) : warps((threads + 31) / 32), groups(static_cast<size_t>(warps) * 32 * 6) {
        block_bar.reset(threads);
        for (int w = 0; w < warps; ++w)
            for (int base = 0; base < 32; ++base)
                for (int k = 0; k < 6; ++k) groups[(static_cast<size_t>(w) * 32 + base) * 6 + k].bar.reset(1 << k);
    }
    int warps;
    Barrier block_bar;
    std::vector<Group> groups;
};

inline thread_local Block* t_block = nullptr;

inline int lane() { return static_cast<int>(threadIdx.x & 31u); }

inline Group* group_of(unsigned mask) {
    const int count = __builtin_popcount(mask);
    if (count <= 1) return nullptr;  // the lane alone: no rendezvous
    int k = 0;
    while ((1 << k) < count) ++k;
    if ((1 << k) != count) {  // masks of the pipeline are whole power-of-two groups
        g_failed.store(true);
        return nullptr;
    }
    const int base = __builtin_ctz(mask);
    const int warp = static_cast<int>(threadIdx.x / 32);
    return &t_block->groups[(static_cast<size_t>(warp) * 32 + base) * 6 + k];
}

// Every lane of `mask` publishes `bits`; `read` sees all lanes' words.
template <class Read>
auto exchange(unsigned mask, uint64_t bits, Read&& read) -> decltype(read(static_cast<const uint64_t*>(nullptr), 0)) {
    Group* g = group_of(mask);
    const int me = lane();
    if (!g) {
        uint64_t alone[32] = {};
        alone[me] = bits;
        return read(alone, me);
    }
    g->slot[me] = bits;
    g->bar.wait();
    auto out = read(g->slot, me);
    g_rendezvous.fetch_add(1, std::memory_order_relaxed);
    g->bar.wait();
    return out;
}

template <class T>
T shuffle(unsigned mask, T v, int src_lane) {
    static_assert(sizeof(T) <= sizeof(uint64_t), "shuffle wider than 64 bits");
    uint64_t bits = 0;
    std::memcpy(&bits, &v, sizeof(T));
    return exchange(mask, bits, [&](const uint64_t* s, int me) {
        T out;
        const uint64_t w = ((mask >> (src_lane & 31)) & 1u) ? s[src_lane & 31] : s[me];
        std::memcpy(&out, &w, sizeof(T));
        return out;
    });
}

inline unsigned ballot(unsigned mask, bool p) {
    return exchange(mask, p ? 1u : 0u, [&](const uint64_t* s, int me) {
        if (__builtin_popcount(mask) <= 1) return p ? (1u << me) : 0u;
        unsigned b = 0;
        for (int l = 0; l < 32; ++l)
            if (((mask >> l) & 1u) && s[l]) b |= 1u << l;
        return b;
    });
}

inline unsigned reduce_add(unsigned mask, unsigned v) {
    return exchange(mask, v, [&](const uint64_t* s, int me) {
        if (__builtin_popcount(mask) <= 1) return v;
        unsigned sum = 0;
        for (int l = 0; l < 32; ++l)
            if ((mask >> l) & 1u) sum += static_cast<unsigned>(s[l]);
        (void)me;
        return sum;
    });
}

// Runs kernel(args...) over `grid` blocks of `block` threads, block by block.
struct Launcher {
    unsigned grid, block;
    template <class Kernel, class... Args>
    void run(Kernel kernel, Args... args) const {
        for (unsigned b = 0; b < grid && !g_failed.load(); ++b) {
            Block blk(static_cast<int>(block));
            std::vector<std::thread> threads;
            threads.reserve(block);
            for (unsigned tid = 0; tid < block; ++tid)
                threads.emplace_back([&, tid] {
                    t_block = &blk;
                    threadIdx = EmuDim3{tid, 0, 0};
                    blockIdx = EmuDim3{b, 0, 0};
                    blockDim = EmuDim3{block, 1, 1};
                    gridDim = EmuDim3{grid, 1, 1};
                    kernel(args...);
                });
            for (auto& th : threads) th.join();
        }
    }
};

template <class Kernel>
struct Bound {
    Launcher l;
    Kernel k;
    template <class... Args>
    void operator()(Args&&... args) const {
        l.run(k, std::forward<Args>(args)...);
    }
};

template <class Kernel>
Bound<Kernel> launch(unsigned grid, unsigned block, Kernel kernel) {
    return Bound<Kernel>{Launcher{grid, block}, kernel};
}

}  // namespace cuda_emu

// ---- device intrinsics -------------------------------------------------
inline void __syncthreads() { cuda_emu::t_block->block_bar.wait(); }
inline unsigned __activemask() { return 1u << cuda_emu::lane(); }
inline void __syncwarp(unsigned mask = 0xffffffffu) { cuda_emu::ballot(mask, true); }
template <class T>
inline T __shfl_sync(unsigned mask, T v, int src, int width = 32) {
    const int base = cuda_emu::lane() & ~(width - 1);
    return cuda_emu::shuffle(mask, v, base + (src & (width - 1)));
}
template <class T>
inline T __shfl_xor_sync(unsigned mask, T v, int lane_mask, int width = 32) {
    const int me = cuda_emu::lane();
    const int base = me & ~(width - 1);
    return cuda_emu::shuffle(mask, v, base + ((me ^ lane_mask) & (width - 1)));
}
inline unsigned __ballot_sync(unsigned mask, bool p) { return cuda_emu::ballot(mask, p); }
inline bool __any_sync(unsigned mask, bool p) { return cuda_emu::ballot(mask, p) != 0; }
inline bool __all_sync(unsigned mask, bool p) {
    const unsigned b = cuda_emu::ballot(mask, p);
    return __builtin_popcount(mask) <= 1 ? p : b == mask;
}
inline unsigned __reduce_add_sync(unsigned mask, unsigned v) { return cuda_emu::reduce_add(mask, v); }
inline int __popc(unsigned v) { return __builtin_popcount(v); }
inline int __ffs(int v) { return __builtin_ffs(v); }
inline double __longlong_as_double(long long v) {
    double d;
    std::memcpy(&d, &v, sizeof d);
    return d;
}
template <class T>
inline T atomicAdd(T* p, T v) {
    return std::atomic_ref<T>(*p).fetch_add(v);
}

// ---- runtime calls of the orchestration ----------------------------------
// (defined once: the test harness that includes this header is one translation
// unit; it links with -Bsymbolic, so that a CUDA runtime already loaded into
// the process cannot take these calls over)
extern "C" {
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
cudaError_t cudaMemsetAsync(void* p, int v, size_t n, cudaStream_t) {
    std::memset(p, v, n);
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaStreamWaitEvent(cudaStream_t, cudaEvent_t, unsigned int) { return cudaSuccess; }
cudaError_t cudaOccupancyMaxActiveBlocksPerMultiprocessor(int* n, const void*, int, size_t) {
    *n = 1;
    return cudaSuccess;
}
cudaError_t cudaOccupancyMaxActiveBlocksPerMultiprocessorWithFlags(int* n, const void*, int, size_t, unsigned int) {
    *n = 1;
    return cudaSuccess;
}
cudaError_t cudaGetDevice(int* d) {
    *d = 0;
    return cudaSuccess;
}
cudaError_t cudaDeviceGetAttribute(int* v, cudaDeviceAttr, int) {
    *v = 1;  // one SM: the queue kernels run one block of workers
    return cudaSuccess;
}
}
