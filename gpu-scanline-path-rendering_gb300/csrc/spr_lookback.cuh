// spr_lookback.cuh -- single-pass scans by decoupled look-back.
//
// Blocks take tiles in launch order from an atomic counter.  A tile
// publishes its own aggregate as soon as it has it, then walks back over its
// predecessors' words, 32 at a time (one warp), adding aggregates until it
// meets an inclusive prefix, and publishes its own inclusive prefix.  Since
// every predecessor of a tile was handed to a block that started earlier,
// the walk always ends; it is nevertheless bounded: after `spin_cap` polls
// of a window that still holds an empty word the tile records a timeout in
// the frame's status word and stops waiting (the frame is then reported as
// failed).
//
// A tile word is 64 bits: the state in bits 62-63 (0 empty, 1 aggregate,
// 2 inclusive) and a 62-bit payload written in the same store.  Payloads
// are combined by addition; with a segment bit (the winding scan of a batch
// restarts at every scene) an aggregate whose segment bit is set ends the
// walk like an inclusive prefix.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "spr_internal.h"

namespace spr {

constexpr uint64_t kLbAggregate = 1ull << 62;
constexpr uint64_t kLbInclusive = 2ull << 62;
constexpr uint64_t kLbPayload = (1ull << 62) - 1ull;

__device__ __forceinline__ uint64_t lb_load(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void lb_store(uint64_t *p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Exclusive prefix of tile t (t > 0), called by all lanes of one warp.
// seg_bit: payload bit that starts a new segment (0: none).  The sum is
// returned whole; callers keep the bits of their fields (no field of a
// payload overflows into the next).
__device__ __forceinline__ uint64_t lb_walk(const uint64_t *status, int64_t t, uint64_t seg_bit, uint32_t spin_cap,
                                            uint32_t *frame_status) {
    const int lane = threadIdx.x & 31;
    uint64_t prefix = 0;
    int64_t end = t;  // predecessors [end - 32, end) in this window, lane 0 nearest
    uint32_t spins = 0;
    while (end > 0) {
        const int64_t p = end - 1 - lane;
        const uint64_t w = p >= 0 ? lb_load(status + p) : kLbInclusive;
        const uint32_t state = (uint32_t)(w >> 62);
        const bool stop = state == 2u || (state == 1u && (w & seg_bit) != 0ull);
        const uint32_t stops = __ballot_sync(0xffffffffu, stop);
        const uint32_t upto = stops ? (((stops & (0u - stops)) << 1) - 1u) : 0xFFFFFFFFu;
        const uint32_t empty = __ballot_sync(0xffffffffu, state == 0u) & upto;
        if (empty) {
            if (++spins > spin_cap) {
                if (lane == 0) atomicOr(frame_status, kStatusTimeout);
                return prefix;  // gives up: the frame is reported as failed
            }
            __nanosleep(64);
            continue;
        }
        uint64_t v = ((upto >> lane) & 1u) ? (w & kLbPayload & ~seg_bit) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        prefix += v;
        if (stops) return prefix;
        end -= 32;
    }
    return prefix;
}

}  // namespace spr
