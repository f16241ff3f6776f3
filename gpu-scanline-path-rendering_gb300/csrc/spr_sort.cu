// spr_sort.cu -- device-wide exclusive scans and stable LSD radix sort.
//
// The frame's scans of sizes (entry offsets, resolve-pair offsets) are
// single-pass decoupled look-back scans (spr_lookback.cuh) whose sizes may
// come from device memory.  The radix sort's digit scans, which run over
// sizes known on the host, and the allocation-free scan are reduce-then-scan
// designs in which no block waits on another.  The radix scatter ranks keys
// stably inside a tile with warp-level __match_any_sync and per-warp digit
// counters, so equal keys keep their input order across the whole array
// (the segmented sort of the reference is stable).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/spr.h"
#include "spr_internal.h"
#include "spr_lookback.cuh"

namespace spr {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

constexpr int kRadixThreads = 256;
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kRadixItems = 16;  // per lane
constexpr int kRadixTile = kRadixThreads * kRadixItems;
constexpr int kRadixWarpSpan = 32 * kRadixItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// Exclusive block scan of one value per thread; returns the prefix and the
// block total through *total.
template <int THREADS>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *smem_warp, uint32_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int W = THREADS / 32;
    uint32_t inc = warp_incl_scan(v);
    if (lane == 31) smem_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < W ? smem_warp[lane] : 0u;
        uint32_t ti = warp_incl_scan(t);
        if (lane < W) smem_warp[lane] = ti - t;
        if (lane == W - 1) smem_warp[W] = ti;
    }
    __syncthreads();
    uint32_t r = smem_warp[warp] + inc - v;
    *total = smem_warp[W];
    __syncthreads();
    return r;
}

__global__ void k_scan_reduce(const uint32_t *__restrict__ in, int64_t n, uint32_t *__restrict__ tile_sums) {
    __shared__ uint32_t sw[kScanThreads / 32 + 1];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        if (i < n) s += in[i];
    }
    uint32_t total;
    block_excl_scan<kScanThreads>(s, sw, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// Exclusive scan of tile sums in place by one block; tile_sums[n] = total.
__global__ void k_scan_tiles(uint32_t *tile_sums, int64_t n) {
    __shared__ uint32_t sw[1024 / 32 + 1];
    uint32_t carry = 0;
    for (int64_t b = 0; b < n; b += 1024) {
        int64_t i = b + threadIdx.x;
        uint32_t v = i < n ? tile_sums[i] : 0u;
        uint32_t total;
        uint32_t p = block_excl_scan<1024>(v, sw, &total);
        if (i < n) tile_sums[i] = carry + p;
        carry += total;
    }
    if (threadIdx.x == 0) tile_sums[n] = carry;
}

__global__ void k_scan_down(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, int64_t n,
                            const uint32_t *__restrict__ tile_sums, int64_t ntiles) {
    __shared__ uint32_t sw[kScanThreads / 32 + 1];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        v[k] = i < n ? in[i] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t p = block_excl_scan<kScanThreads>(s, sw, &total) + tile_sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        if (i < n) out[i] = p;
        p += v[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = tile_sums[ntiles];
}

template <class K>
__global__ void k_radix_hist(const K *__restrict__ keys, int64_t n_cap, const uint32_t *__restrict__ n_dev, int shift,
                             uint32_t *__restrict__ counts, int64_t ntiles) {
    const int64_t n = n_dev ? min((int64_t)*n_dev, n_cap) : n_cap;
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kRadixTile;
#pragma unroll 4
    for (int k = 0; k < kRadixItems; ++k) {
        int64_t i = base + (int64_t)k * kRadixThreads + threadIdx.x;
        if (i < n) atomicAdd(&hist[(uint32_t)(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    counts[(int64_t)threadIdx.x * ntiles + blockIdx.x] = hist[threadIdx.x];
}

// Shared memory of the scatter: the tile reordered by digit, then written
// out in digit runs (consecutive elements of a digit go to consecutive
// global positions, so the writes coalesce).
template <class K>
struct ScatterSmem {
    K key[kRadixTile];
    uint32_t val[kRadixTile];
    uint32_t whist[kRadixWarps][256];
    uint32_t lstart[256];  // first local position of each digit
    uint32_t gstart[256];  // the tile's first global position of each digit
};

template <class K>
__global__ void __launch_bounds__(kRadixThreads) k_radix_scatter(const K *__restrict__ keys,
                                                                  const uint32_t *__restrict__ vals, int64_t n_cap,
                                                                  const uint32_t *__restrict__ n_dev, int shift,
                                                                  const uint32_t *__restrict__ offsets,
                                                                  int64_t ntiles, K *__restrict__ keys_out,
                                                                  uint32_t *__restrict__ vals_out) {
    const int64_t n = n_dev ? min((int64_t)*n_dev, n_cap) : n_cap;
    if ((int64_t)blockIdx.x * kRadixTile >= n) return;  // a tile past the end (nothing to move)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ScatterSmem<K> &sm = *reinterpret_cast<ScatterSmem<K> *>(smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kRadixWarps * 256; i += kRadixThreads) (&sm.whist[0][0])[i] = 0;
    __syncthreads();
    const int64_t tile0 = (int64_t)blockIdx.x * kRadixTile;
    const int64_t base = tile0 + (int64_t)warp * kRadixWarpSpan;
    const int cnt = (int)min((int64_t)kRadixTile, n - tile0);
    K kk[kRadixItems];
    uint32_t vv[kRadixItems];
    uint32_t rank[kRadixItems];
#pragma unroll
    for (int r = 0; r < kRadixItems; ++r) {
        int64_t i = base + r * 32 + lane;
        bool valid = i < n;
        kk[r] = valid ? keys[i] : (K)0;
        vv[r] = valid ? vals[i] : 0u;
        uint32_t d = valid ? ((uint32_t)(kk[r] >> shift) & 0xFFu) : (256u + lane);
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = __popc(peers & ((1u << lane) - 1u));
        uint32_t cur = valid ? sm.whist[warp][d] : 0u;
        __syncwarp();
        if (valid && before == 0) sm.whist[warp][d] = cur + __popc(peers);
        __syncwarp();
        rank[r] = cur + before;
    }
    __syncthreads();
    {
        const int d = threadIdx.x;  // one digit per thread: the tile's count of d, per-warp local offsets
        uint32_t tot = 0;
#pragma unroll
        for (int w = 0; w < kRadixWarps; ++w) {
            const uint32_t c = sm.whist[w][d];
            sm.whist[w][d] = tot;
            tot += c;
        }
        // exclusive scan of the digit totals over the block
        __shared__ uint32_t wsum[kRadixWarps + 1];
        uint32_t inc = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            uint32_t t = lane < kRadixWarps ? wsum[lane] : 0u, ti = t;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, ti, o);
                if (lane >= o) ti += v;
            }
            if (lane < kRadixWarps) wsum[lane] = ti - t;
        }
        __syncthreads();
        const uint32_t ls = wsum[warp] + inc - tot;
        sm.lstart[d] = ls;
        sm.gstart[d] = offsets[(int64_t)d * ntiles + blockIdx.x];
#pragma unroll
        for (int w = 0; w < kRadixWarps; ++w) sm.whist[w][d] += ls;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRadixItems; ++r) {
        int64_t i = base + r * 32 + lane;
        if (i < n) {
            const uint32_t d = (uint32_t)(kk[r] >> shift) & 0xFFu;
            const uint32_t lp = sm.whist[warp][d] + rank[r];
            sm.key[lp] = kk[r];
            sm.val[lp] = vv[r];
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += kRadixThreads) {
        const K k = sm.key[i];
        const uint32_t d = (uint32_t)(k >> shift) & 0xFFu;
        const uint32_t pos = sm.gstart[d] + (uint32_t)i - sm.lstart[d];
        keys_out[pos] = k;
        vals_out[pos] = sm.val[i];
    }
}

// ---- per-path segment sort ---------------------------------------------------
// The fragment entries arrive grouped by path (curves are in path order and
// each curve's entries are contiguous), so the stable sort by (path, cell
// key) is a stable sort of every path's segment by its 24-bit cell key.  One
// block per path: segments of up to kSegTile entries are sorted in shared
// memory (three 8-bit passes, a pass skipped when its digit is constant) and
// written once; longer ones make the same passes over the segment in global
// memory, chunk by chunk, ping-ponging through the input keys' own range.
// Ranking inside a chunk is the scatter's (per-warp digit counters, lanes in
// input order), so equal keys keep their input order.  Inside a segment the
// keys' path bits are the path's own, so only the 24-bit cell keys move.

constexpr int kSegThreads = 256;
constexpr int kSegWarps = kSegThreads / 32;
constexpr int kSegItems = 8;
constexpr int kSegTile = kSegThreads * kSegItems;
constexpr int kSegWarpSpan = 32 * kSegItems;

struct SegSmem {
    uint32_t key[kSegTile];
    uint32_t val[kSegTile];
    uint32_t whist[kSegWarps][256];
    uint32_t lstart[256];  // first position of each digit in the staged chunk
    uint32_t dstart[256];  // next output position of each digit in the segment (long segments)
    uint32_t wsum[kSegWarps + 1];
};

// Shared-memory form of a sort key within its path: the 24-bit cell key
// and, in bits 24-27, key bits 60-63 (the digit passes read bits 0-23).
__device__ __forceinline__ uint32_t sk_pack(uint64_t k) {
    return ((uint32_t)k & 0xFFFFFFu) | ((uint32_t)(k >> kFwShift) << 24);
}
__device__ __forceinline__ uint64_t sk_unpack(uint64_t hi, uint32_t k) {
    return hi | (uint64_t)(k & 0xFFFFFFu) | ((uint64_t)(k >> 24) << kFwShift);
}

// First curve of every path (curves ascending by path); start[P] = C.
__global__ void k_path_starts(const CurveDesc *__restrict__ curves, uint32_t C, uint32_t P, uint32_t *__restrict__ start) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c > (int64_t)C) return;
    const uint32_t lo = c == 0 ? 0u : curves[c - 1].pid + 1u;
    const uint32_t hi = c == (int64_t)C ? P : curves[c].pid;
    for (uint32_t q = lo; q <= hi && q <= P; ++q) start[q] = (uint32_t)c;
}

// Ranks one chunk (kk[], count cnt, input order = warp-major, then item,
// then lane) by digit `shift` and stages it in shared memory ordered by
// digit; sm.lstart gets each digit's first staged position, the return value
// through `tot` the per-digit counts of thread d (d = threadIdx.x).
__device__ __forceinline__ void seg_stage_chunk(SegSmem &sm, const uint32_t (&kk)[kSegItems],
                                                const uint32_t (&vv)[kSegItems], int cnt, int shift, uint32_t *tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kSegWarps * 256; i += kSegThreads) (&sm.whist[0][0])[i] = 0;
    __syncthreads();
    uint32_t rank[kSegItems];
#pragma unroll
    for (int r = 0; r < kSegItems; ++r) {
        if (warp * kSegWarpSpan + r * 32 >= cnt) break;  // the warp's remaining items are past the end
        const int li = warp * kSegWarpSpan + r * 32 + lane;
        const bool valid = li < cnt;
        const uint32_t d = valid ? ((kk[r] >> shift) & 0xFFu) : (256u + lane);
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t before = __popc(peers & ((1u << lane) - 1u));
        const uint32_t cur = valid ? sm.whist[warp][d] : 0u;
        __syncwarp();
        if (valid && before == 0) sm.whist[warp][d] = cur + __popc(peers);
        __syncwarp();
        rank[r] = cur + before;
    }
    __syncthreads();
    {
        // one digit per thread of the first 256: its count and per-warp offsets
        const int d = threadIdx.x;
        const bool dig = d < 256;
        uint32_t t = 0;
        if (dig) {
#pragma unroll
            for (int w = 0; w < kSegWarps; ++w) {
                const uint32_t c = sm.whist[w][d];
                sm.whist[w][d] = t;
                t += c;
            }
        }
        uint32_t inc = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31 && dig) sm.wsum[warp] = inc;
        __syncthreads();
        if (warp == 0) {  // the 8 digit warps' totals
            const uint32_t x = lane < 8 ? sm.wsum[lane] : 0u;
            uint32_t xi = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, xi, o);
                if (lane >= o) xi += v;
            }
            if (lane < 8) sm.wsum[lane] = xi - x;
        }
        __syncthreads();
        if (dig) {
            const uint32_t ls = sm.wsum[warp] + inc - t;
            sm.lstart[d] = ls;
#pragma unroll
            for (int w = 0; w < kSegWarps; ++w) sm.whist[w][d] += ls;
        }
        *tot = t;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSegItems; ++r) {
        if (warp * kSegWarpSpan + r * 32 >= cnt) break;
        const int li = warp * kSegWarpSpan + r * 32 + lane;
        if (li < cnt) {
            const uint32_t d = (kk[r] >> shift) & 0xFFu;
            const uint32_t lp = sm.whist[warp][d] + rank[r];
            sm.key[lp] = kk[r];
            sm.val[lp] = vv[r];
        }
    }
    __syncthreads();
}

// Segments of up to kWarpSeg entries: one warp each, three 8-bit passes in
// the warp's own shared memory (no block barriers).  Lane l ranks entry
// 32c + l of every chunk c; the warp's digit counters make the ranks stable.
constexpr int kWarpSeg = 512;
constexpr int kSmallWarps = 4;

__global__ void __launch_bounds__(kSmallWarps * 32) k_segment_sort_small(const uint64_t *__restrict__ keys_in,
                                                                        const uint32_t *__restrict__ start,
                                                                        const uint32_t *__restrict__ offsets,
                                                                        uint32_t P, uint64_t *__restrict__ keys_out,
                                                                        uint32_t *__restrict__ vals_out,
                                                                        const FrameCounters *__restrict__ ctr) {
    __shared__ uint32_t skey[kSmallWarps][2][kWarpSeg], sval[kSmallWarps][2][kWarpSeg], shist[kSmallWarps][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t p = blockIdx.x * kSmallWarps + w;
    if (p >= P || ctr->status != 0u || ctr->nf != ctr->need_nf) return;  // (entries not admitted: nothing to sort)
    const uint32_t b = offsets[start[p]], e = offsets[start[p + 1]];
    if (e <= b || e - b > (uint32_t)kWarpSeg) return;
    const int n = (int)(e - b);
    const uint64_t hi = (uint64_t)p << 24;
    for (int i = lane; i < n; i += 32) {
        skey[w][0][i] = sk_pack(keys_in[b + i]);
        sval[w][0][i] = b + (uint32_t)i;
    }
    __syncwarp();
    int cur = 0;
    const int nch = (n + 31) >> 5;
    for (int shift = 0; shift < 24; shift += 8) {
        const uint32_t d0 = (skey[w][cur][0] >> shift) & 0xFFu;
        bool diff = false;
        for (int i = lane; i < n; i += 32) diff |= ((skey[w][cur][i] >> shift) & 0xFFu) != d0;
        if (!__any_sync(0xffffffffu, diff)) continue;  // one digit throughout
        for (int i = lane; i < 256; i += 32) shist[w][i] = 0u;
        __syncwarp();
        uint32_t rk[kWarpSeg / 32];
#pragma unroll
        for (int c = 0; c < kWarpSeg / 32; ++c) {
            if (c >= nch) break;
            const int i = c * 32 + lane;
            const bool valid = i < n;
            const uint32_t d = valid ? (skey[w][cur][i] >> shift) & 0xFFu : 256u + lane;
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            const uint32_t before = __popc(peers & ((1u << lane) - 1u));
            const uint32_t old = valid ? shist[w][d] : 0u;
            __syncwarp();
            if (valid && before == 0) shist[w][d] = old + __popc(peers);
            __syncwarp();
            rk[c] = old + before;
        }
        // exclusive scan of the 256 digit counts: lane owns digits 8l .. 8l + 7
        uint32_t loc[8], sum = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            loc[q] = sum;
            sum += shist[w][lane * 8 + q];
        }
        uint32_t inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 8; ++q) shist[w][lane * 8 + q] = inc - sum + loc[q];
        __syncwarp();
#pragma unroll
        for (int c = 0; c < kWarpSeg / 32; ++c) {
            if (c >= nch) break;
            const int i = c * 32 + lane;
            if (i < n) {
                const uint32_t k = skey[w][cur][i];
                const uint32_t pos = shist[w][(k >> shift) & 0xFFu] + rk[c];
                skey[w][cur ^ 1][pos] = k;
                sval[w][cur ^ 1][pos] = sval[w][cur][i];
            }
        }
        __syncwarp();
        cur ^= 1;
    }
    for (int i = lane; i < n; i += 32) {
        keys_out[b + i] = sk_unpack(hi, skey[w][cur][i]);
        vals_out[b + i] = sval[w][cur][i];
    }
}

__global__ void __launch_bounds__(kSegThreads, 5) k_segment_sort(const uint64_t *__restrict__ keys_in,
                                                               const uint32_t *__restrict__ start,
                                                               const uint32_t *__restrict__ offsets,
                                                               uint64_t *__restrict__ keys_out,
                                                               uint32_t *__restrict__ vals_out, uint64_t *keys_tmp,
                                                               uint32_t *vals_tmp, const FrameCounters *__restrict__ ctr) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SegSmem &sm = *reinterpret_cast<SegSmem *>(smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t p = blockIdx.x;
    if (ctr->status != 0u || ctr->nf != ctr->need_nf) return;  // entries not admitted: nothing to sort
    const uint32_t b = offsets[start[p]], e = offsets[start[p + 1]];
    if (e - b <= (uint32_t)kWarpSeg) return;  // empty, or a warp's (k_segment_sort_small)
    const uint32_t n = e - b;
    const uint64_t hi = (uint64_t)p << 24;  // the segment's path bits
    if (n <= (uint32_t)kSegTile) {
        uint32_t kk[kSegItems];
        uint32_t vv[kSegItems];
#pragma unroll
        for (int r = 0; r < kSegItems; ++r) {
            const uint32_t li = (uint32_t)(warp * kSegWarpSpan + r * 32 + lane);
            kk[r] = li < n ? sk_pack(keys_in[b + li]) : 0u;
            vv[r] = b + li;
        }
        bool staged = false;  // the current order is in shared memory
        for (int shift = 0; shift < 24; shift += 8) {
            const uint32_t d0 = (__shfl_sync(0xffffffffu, kk[0], 0) >> shift) & 0xFFu;
            bool diff = false;
#pragma unroll
            for (int r = 0; r < kSegItems; ++r) {
                const uint32_t li = (uint32_t)(warp * kSegWarpSpan + r * 32 + lane);
                diff |= li < n && ((kk[r] >> shift) & 0xFFu) != d0;
            }
            // warp 0's first key stands for the block: compare across warps too
            if (warp == 0 && lane == 0) sm.wsum[kSegWarps] = d0;
            __syncthreads();
            const uint32_t dblock = sm.wsum[kSegWarps];
            diff = diff || (n > 0 && ((kk[0] >> shift) & 0xFFu) != dblock &&
                            (uint32_t)(warp * kSegWarpSpan + lane) < n);
            if (!__syncthreads_or(diff)) continue;  // one digit throughout: order unchanged
            uint32_t tot;
            seg_stage_chunk(sm, kk, vv, (int)n, shift, &tot);
            staged = true;
#pragma unroll
            for (int r = 0; r < kSegItems; ++r) {
                const uint32_t li = (uint32_t)(warp * kSegWarpSpan + r * 32 + lane);
                if (li < n) {
                    kk[r] = sm.key[li];
                    vv[r] = sm.val[li];
                }
            }
            __syncthreads();
        }
        if (!staged) {  // already in order
#pragma unroll
            for (int r = 0; r < kSegItems; ++r) {
                const uint32_t li = (uint32_t)(warp * kSegWarpSpan + r * 32 + lane);
                if (li < n) {
                    keys_out[b + li] = sk_unpack(hi, kk[r]);
                    vals_out[b + li] = vv[r];
                }
            }
            return;
        }
        for (uint32_t i = threadIdx.x; i < n; i += kSegThreads) {
            keys_out[b + i] = sk_unpack(hi, sm.key[i]);
            vals_out[b + i] = sm.val[i];
        }
        return;
    }
    // long segment: chunked passes through global memory
    int cur = 0;  // data in: 0 keys_in (values = positions), 1 *_out, 2 *_tmp
    for (int shift = 0; shift < 24; shift += 8) {
        const uint64_t *ksrc = cur == 0 ? keys_in : (cur == 1 ? keys_out : keys_tmp);
        const uint32_t *vsrc = cur == 1 ? vals_out : vals_tmp;
        uint64_t *kdst = cur == 1 ? keys_tmp : keys_out;
        uint32_t *vdst = cur == 1 ? vals_tmp : vals_out;
        // digit histogram of the segment
        const bool dig = threadIdx.x < 256;
        if (dig) sm.dstart[threadIdx.x] = 0;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < n; i += kSegThreads)
            atomicAdd(&sm.dstart[(uint32_t)(ksrc[b + i] >> shift) & 0xFFu], 1u);
        __syncthreads();
        const uint32_t cnt_d = dig ? sm.dstart[threadIdx.x] : 0u;
        if (__syncthreads_or(cnt_d == n)) continue;  // one digit throughout
        {
            uint32_t inc = cnt_d;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            if (lane == 31 && dig) sm.wsum[warp] = inc;
            __syncthreads();
            if (warp == 0) {
                const uint32_t x = lane < 8 ? sm.wsum[lane] : 0u;
                uint32_t xi = x;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t v = __shfl_up_sync(0xffffffffu, xi, o);
                    if (lane >= o) xi += v;
                }
                if (lane < 8) sm.wsum[lane] = xi - x;
            }
            __syncthreads();
            if (dig) sm.dstart[threadIdx.x] = b + sm.wsum[warp] + inc - cnt_d;
            __syncthreads();
        }
        for (uint32_t c0 = 0; c0 < n; c0 += kSegTile) {
            const int cnt = (int)min((uint32_t)kSegTile, n - c0);
            uint32_t kk[kSegItems];
            uint32_t vv[kSegItems];
#pragma unroll
            for (int r = 0; r < kSegItems; ++r) {
                const int li = warp * kSegWarpSpan + r * 32 + lane;
                const bool valid = li < cnt;
                kk[r] = valid ? sk_pack(ksrc[b + c0 + li]) : 0u;
                vv[r] = valid ? (cur == 0 ? b + c0 + (uint32_t)li : vsrc[b + c0 + li]) : 0u;
            }
            uint32_t tot;
            seg_stage_chunk(sm, kk, vv, cnt, shift, &tot);
            for (int i = threadIdx.x; i < cnt; i += kSegThreads) {
                const uint32_t k = sm.key[i];
                const uint32_t d = (k >> shift) & 0xFFu;
                const uint32_t pos = sm.dstart[d] + (uint32_t)i - sm.lstart[d];
                kdst[pos] = sk_unpack(hi, k);
                vdst[pos] = sm.val[i];
            }
            __syncthreads();
            if (threadIdx.x < 256) sm.dstart[threadIdx.x] += tot;
            __syncthreads();
        }
        cur = cur == 1 ? 2 : 1;
    }
    if (cur == 1) return;
    for (uint32_t i = threadIdx.x; i < n; i += kSegThreads) {  // into the output arrays
        keys_out[b + i] = cur == 0 ? keys_in[b + i] : keys_tmp[b + i];
        vals_out[b + i] = cur == 0 ? b + i : vals_tmp[b + i];
    }
}

}  // namespace

int launch_segment_sort(const CurveDesc *curves, uint32_t C, uint32_t P, const uint32_t *offsets, uint64_t *keys,
                        uint32_t *vals, uint64_t *keys_out, uint32_t *vals_out, uint32_t *path_start,
                        const FrameCounters *ctr, cudaStream_t s) {
    if (P == 0) return 0;
    k_path_starts<<<(unsigned)(((int64_t)C + 1 + 255) / 256), 256, 0, s>>>(curves, C, P, path_start);
    cudaFuncSetAttribute(k_segment_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SegSmem));
    k_segment_sort_small<<<(P + kSmallWarps - 1) / kSmallWarps, kSmallWarps * 32, 0, s>>>(keys, path_start, offsets, P,
                                                                                      keys_out, vals_out, ctr);
    k_segment_sort<<<P, kSegThreads, sizeof(SegSmem), s>>>(keys, path_start, offsets, keys_out, vals_out, keys, vals,
                                                           ctr);
    return 3;
}

// ---- single-pass scans of frame sizes ------------------------------------------
// One tile of kScanTile counts per block; tiles are taken in launch order.
__global__ void __launch_bounds__(kScanThreads) k_scan_lb(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                                                           const uint32_t *__restrict__ n_dev, int64_t n_cap,
                                                           uint64_t *__restrict__ status, uint32_t *__restrict__ tile_ctr,
                                                           uint32_t spin_cap, uint32_t *__restrict__ frame_status,
                                                           uint32_t *__restrict__ total_out, int64_t hold_tile) {
    __shared__ uint32_t sw[kScanThreads / 32 + 1];
    __shared__ uint32_t s_tile, s_prefix;
    const int64_t n = n_dev ? min((int64_t)*n_dev, n_cap) : n_cap;
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1u);
    __syncthreads();
    const int64_t t = s_tile;
    if (t >= ntiles) {
        if (t == 0 && threadIdx.x == 0) {  // nothing to scan
            out[0] = 0u;
            if (total_out) *total_out = 0u;
        }
        return;
    }
    const int64_t base = t * kScanTile + (int64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    if (base + kScanItems <= n) {  // two 128-bit loads
        const uint4 a = reinterpret_cast<const uint4 *>(in + base)[0], b = reinterpret_cast<const uint4 *>(in + base)[1];
        v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) v[k] = base + k < n ? in[base + k] : 0u;
    }
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += v[k];
    uint32_t total;
    const uint32_t ex = block_excl_scan<kScanThreads>(sum, sw, &total);
    if (threadIdx.x < 32) {
        const bool publish = t != hold_tile;  // (a held tile's successors wait until they give up)
        uint64_t pre = 0;
        if (t > 0) {
            if (threadIdx.x == 0 && publish) lb_store(status + t, kLbAggregate | total);
            pre = lb_walk(status, t, 0ull, spin_cap, frame_status);
        }
        if (threadIdx.x == 0) {
            if (publish) lb_store(status + t, kLbInclusive | (uint32_t)(pre + total));
            s_prefix = (uint32_t)pre;
        }
    }
    __syncthreads();
    uint32_t p = s_prefix + ex;
    uint32_t o[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        o[k] = p;
        p += v[k];
    }
    if (base + kScanItems <= n) {
        reinterpret_cast<uint4 *>(out + base)[0] = make_uint4(o[0], o[1], o[2], o[3]);
        reinterpret_cast<uint4 *>(out + base)[1] = make_uint4(o[4], o[5], o[6], o[7]);
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
            if (base + k < n) out[base + k] = o[k];
    }
    if (t == ntiles - 1 && threadIdx.x == 0) {
        out[n] = s_prefix + total;
        if (total_out) *total_out = s_prefix + total;
    }
}

__global__ void k_admit(const uint32_t *__restrict__ need, uint32_t *__restrict__ admitted, uint32_t cap,
                        uint32_t *__restrict__ status) {
    const uint32_t v = *need;
    if (v <= cap && !(*status & kStatusTimeout)) {  // (after a timeout the size itself may be wrong)
        *admitted = v;
    } else {
        *admitted = 0u;
        atomicOr(status, kStatusOverflow);
    }
}

int64_t scan_tmp_words(int64_t n) { return (n + kScanTile - 1) / kScanTile + 2; }

int64_t lookback_words(int64_t n) { return std::max<int64_t>(1, (n + kScanTile - 1) / kScanTile); }

int scan_lookback_u32(const uint32_t *in, uint32_t *out, const uint32_t *n_dev, int64_t n_cap, uint64_t *tile_status,
                      uint32_t *tile_ctr, uint32_t spin_cap, uint32_t *frame_status, uint32_t *total_out,
                      cudaStream_t s, int64_t hold_tile) {
    k_scan_lb<<<(unsigned)lookback_words(n_cap), kScanThreads, 0, s>>>(in, out, n_dev, n_cap, tile_status, tile_ctr,
                                                                     spin_cap, frame_status, total_out, hold_tile);
    return 1;
}

int launch_admit(const uint32_t *need, uint32_t *admitted, uint32_t cap, uint32_t *status, cudaStream_t s) {
    k_admit<<<1, 1, 0, s>>>(need, admitted, cap, status);
    return 1;
}

int scan_exclusive_u32(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp, cudaStream_t s) {
    int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles == 0) {
        cudaMemsetAsync(out, 0, sizeof(uint32_t), s);
        return 0;
    }
    k_scan_reduce<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, tmp);
    k_scan_tiles<<<1, 1024, 0, s>>>(tmp, ntiles);
    k_scan_down<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, out, n, tmp, ntiles);
    return 3;
}

int scan_tiles_inplace(uint32_t *a, int64_t n, cudaStream_t s) {
    k_scan_tiles<<<1, 1024, 0, s>>>(a, n);
    return 1;
}

int64_t radix_tiles(int64_t n) { return (n + kRadixTile - 1) / kRadixTile; }

int64_t radix_tmp_words(int64_t n) {
    int64_t c = 256 * radix_tiles(n);
    return 2 * (c + 1) + scan_tmp_words(c) + 64;
}

template <class K>
bool radix_sort(K *keys, uint32_t *vals, K *keys_alt, uint32_t *vals_alt, int64_t n, int key_bits, uint32_t *tmp,
                cudaStream_t s, int *launches, const uint32_t *n_dev) {
    *launches = 0;
    if (n <= 1 && !n_dev) return false;
    if (n <= 0) n = 1;
    const int64_t ntiles = radix_tiles(n);
    const int64_t c = 256 * ntiles;
    uint32_t *counts = tmp;
    uint32_t *offsets = tmp + (c + 1);
    uint32_t *scan_tmp = tmp + 2 * (c + 1);
    bool alt = false;
    cudaFuncSetAttribute(k_radix_scatter<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ScatterSmem<K>));
    for (int shift = 0; shift < key_bits; shift += 8) {
        const K *ki = alt ? keys_alt : keys;
        const uint32_t *vi = alt ? vals_alt : vals;
        K *ko = alt ? keys : keys_alt;
        uint32_t *vo = alt ? vals : vals_alt;
        k_radix_hist<K><<<(unsigned)ntiles, kRadixThreads, 0, s>>>(ki, n, n_dev, shift, counts, ntiles);
        *launches += 2 + scan_exclusive_u32(counts, offsets, c, scan_tmp, s);
        k_radix_scatter<K><<<(unsigned)ntiles, kRadixThreads, sizeof(ScatterSmem<K>), s>>>(ki, vi, n, n_dev, shift,
                                                                                       offsets, ntiles, ko, vo);
        alt = !alt;
    }
    return alt;
}

template bool radix_sort<uint64_t>(uint64_t *, uint32_t *, uint64_t *, uint32_t *, int64_t, int, uint32_t *,
                                   cudaStream_t, int *, const uint32_t *);
template bool radix_sort<uint32_t>(uint32_t *, uint32_t *, uint32_t *, uint32_t *, int64_t, int, uint32_t *,
                                   cudaStream_t, int *, const uint32_t *);

// ---- allocation-free exclusive scan ------------------------------------------
// Scratch of spr_scan_offsets_noalloc: the per-tile partial sums of one scan
// (kNoAllocMaxTiles + 2 words = 64 KB).  Being a file-scope __device__ array,
// it exists on every GPU that loads this library until the process exits,
// and all calls on a device share it.
namespace {
constexpr int64_t kNoAllocMaxTiles = 16384;
static __device__ __align__(256) uint32_t g_noalloc_tile_sums[kNoAllocMaxTiles + 2];
}  // namespace

}  // namespace spr

extern "C" int spr_scan_offsets_noalloc(const uint32_t *d_counts, uint32_t *d_offsets, int64_t n, void *stream) {
    using namespace spr;
    if (n < 0 || !d_offsets || (n > 0 && !d_counts)) return SPR_ERR_INVALID_ARG;
    if (n > kNoAllocMaxTiles * (int64_t)kScanTile) return SPR_ERR_CAPACITY_EXCEEDED;
    // An error left pending by the caller's own earlier work is not this
    // call's: report it without clearing it and launch nothing.
    if (cudaPeekAtLastError() != cudaSuccess) return SPR_ERR_CUDA;
    // The device address of the scratch array in the current context.  In
    // host code the array's name is only a host-side stand-in, so kernels are
    // always given this address.  It is looked up on every call (a cheap
    // lookup once the module is loaded; the first call on a device loads it),
    // so a device reset or a switch of context between calls is followed.
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_tile_sums) != cudaSuccess || !p) {
        cudaGetLastError();
        return SPR_ERR_CUDA;
    }
    // Every tile sum is written before it is read, so nothing needs clearing.
    scan_exclusive_u32(d_counts, d_offsets, n, static_cast<uint32_t *>(p), static_cast<cudaStream_t>(stream));
    return cudaGetLastError() == cudaSuccess ? SPR_OK : SPR_ERR_CUDA;
}
