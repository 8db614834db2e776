// Tiled scatter kernels of the exchange: G[d, c, b, t] += coef * src_row[t - delay]
// over the source groups of a plan (exchange_plan.cuh).
#pragma once
#include "exchange_plan.cuh"

namespace {

// --------------------------------------------------------- PTX helpers
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// An mbarrier's shared memory may serve another purpose (the next work item
// of a persistent block) only after the barrier is invalidated.
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after kWaitLimit polls (each poll may suspend
// briefly) or as soon as another CTA has reported a failure.
constexpr unsigned kWaitLimit = 1u << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, const volatile int* err) {
    for (unsigned it = 0; it < kWaitLimit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 255u && *err) return false;
    }
    return false;
}
// Wait for a CTA's own bulk copies still in flight before it leaves after a
// failure: bounded, but not cut short by the error flag (the CTA must not
// exit while a copy can still write into its shared memory).
__device__ __forceinline__ bool mbar_drain(uint64_t* bar, unsigned parity) {
    for (unsigned it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// Values of the error flag: which bounded wait gave up first.
constexpr int kErrConsumerWait = 1;  // a consumer warp waiting for a stage's copies
constexpr int kErrProducerWait = 2;  // the producer waiting for a stage to be released
constexpr int kErrDrain = 3;         // the drain of a failed CTA's copies in flight
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// ------------------------------------------------------- scatter (FP32, FP64)
// Warp-specialised pipeline.  One producer warp streams the groups of a
// segment through kStages shared-memory stages of kGps groups each, with
// bulk copies (per group the source window; per stage the groups' packed
// per-warp words and their 16 coefficients of this band).  kConsumers consumer
// warps, warp w owning receiver slots 2w and 2w + 1 of the tile, accumulate
// those slots' windows in registers (lane l owns bins t0 + l + 32 r).
// Stage hand-off: `full` (producer arrival + transaction bytes) and `empty`
// (one arrival per consumer warp); every wait is bounded.
//
// FP32 windows are 1024 bins (32 per lane): the kernel is bound by
// shared-memory bandwidth, one window value per FMA.  FP64 windows are 256
// bins (8 per lane, 16 accumulator registers per slot): the kernel is bound
// by the FP64 pipe, and shorter windows keep registers low and the grid large.
constexpr int kSlotsPerWarp = 2;
constexpr int kConsumers = kTile / kSlotsPerWarp;    // 8 consumer warps
constexpr int kWsThreads = (kConsumers + 1) * 32;    // + one producer warp
constexpr int kGps = 4;                              // groups per stage
constexpr int kStages = 6;
constexpr int kBarBytes = 128;                       // full[kStages], empty[kStages]
static_assert(2 * kStages * 8 <= kBarBytes, "barrier area too small");
static_assert(kPackWarps == kConsumers, "one packed word per consumer warp");

template <typename T, int kBinsPerLane = (sizeof(T) == 4 ? 32 : 8)>
struct WsLayout {
    static constexpr int kBins = kBinsPerLane;               // bins per lane, strided by 32
    static constexpr int kTW = 32 * kBins;                   // bins per window
    static constexpr int kAlign = 16 / (int)sizeof(T);       // elements per 16 bytes
    static constexpr int kStageF = kTW + kMaxSpan + kAlign - 1;  // staged elements per group
    static constexpr int kWinBytes = kStageF * (int)sizeof(T);
    static constexpr int kPackOff = kGps * kWinBytes;        // kGps x kPackWarps packed words
    static constexpr int kCoefOff = kPackOff + kGps * kPackWarps * 4;  // kGps x 16 coefficients
    static constexpr int kStageBytes = kCoefOff + kGps * kTile * (int)sizeof(T);
    static constexpr size_t kSmem = (size_t)kBarBytes + (size_t)kStages * kStageBytes;
    static_assert(kStageF % kAlign == 0, "staged window must be a whole number of 16-byte chunks");
    static_assert(kWinBytes % 16 == 0 && kPackOff % 16 == 0 && kCoefOff % 16 == 0 && kStageBytes % 16 == 0,
                  "stage parts must stay 16-byte aligned");
};
// FP32 names used by the callers
constexpr int kBins = WsLayout<float>::kBins;
constexpr int kTW = WsLayout<float>::kTW;
constexpr int kStageF = WsLayout<float>::kStageF;    // also bounds the FP64 window (the row tail)
constexpr size_t kScatterSmem = WsLayout<float>::kSmem;
static_assert(WsLayout<double>::kStageF <= kStageF, "the row tail is sized for the longer window");

template <typename T>
struct Vec2;
template <>
struct Vec2<float> {
    using type = float2;
};
template <>
struct Vec2<double> {
    using type = double2;
};

// One Kahan step: s += x with the running compensation c (the exchange's
// late-bin E_total sums).  y = x - c; t = s + y; c = (t - s) - y; s = t.
template <typename T>
__device__ __forceinline__ void kahan_add(T& s, T& c, T x) {
    const T y = x - c;
    const T t = s + y;
    c = (t - s) - y;
    s = t;
}
// The compensation terms are kept between orders as bfloat16 (the top 16
// bits of the FP32 term, rounded to nearest even): c is the rounding error
// of s, at most half an FP32 ulp of s, so its 8-bit mantissa still carries
// the sum to about 2^-33 of s, at half the memory traffic of FP32 terms.
__device__ __forceinline__ float comp_get(uint16_t bits) { return __uint_as_float((uint32_t)bits << 16); }
__device__ __forceinline__ uint16_t comp_put(float c) {
    const uint32_t u = __float_as_uint(c);
    return (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);  // finite values: round to nearest even
}

__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }

// acc[r] += cf * staged[lane + 32 r + base - off] for one member slot, with
// base = kMaxSpan + mu (mu: elements the staged start was rounded down by).
template <typename T, int kN>
__device__ __forceinline__ void slot_window(T (&acc)[kN], const T* win, T cf, int off, int base, int lane) {
    const T* p = win + lane + base - off;
#pragma unroll
    for (int r = 0; r < kN; ++r) acc[r] = fma_t(cf, p[32 * r], acc[r]);
}

// One order, one window, bands b_lo .. b_hi - 1: G[j, c, b, window] for the
// 16 receivers of a segment.  Histogram rows of eprev are padded: row r
// starts at r * rs with bin 0 at offset `lead` (>= nt + kMaxSpan + 4 zeros
// before it), so a staged window reaching before bin 0 reads zeros and needs
// no masking, and no window starts before the buffer.  Every shared-memory
// read of a consumer warp covers 32 consecutive elements (no bank conflict
// at any offset).  The bands run through one pipeline: the producer streams
// band after band (the groups are the same, their rows and coefficients
// differ), and a consumer warp writes a band's rows out as soon as it has
// consumed that band's last stage.
//
// The work item is (seg_i: index into seg_order, win: window, bands); the
// kernels below take one band from the block index (kBands false: the band
// loop and the write-out compile to the single-band form), the batched
// exchange every band from its work queue (kBands true).
template <typename T, int kB = WsLayout<T>::kBins, bool kBands = false>
__device__ __forceinline__ void scatter_ws(int n_class, int nb, int nt, long long rs, int lead, long long cap,
                                           const int32_t* __restrict__ tile_recv,
                                           const int32_t* __restrict__ seg_order,
                                           const int64_t* __restrict__ seg_off, const Group* __restrict__ groups,
                                           const uint32_t* __restrict__ wpack, const T* __restrict__ coef,
                                           const T* __restrict__ eprev, T* __restrict__ gout,
                                           int* __restrict__ err, int seg_i, int win, int b_lo, int b_hi) {
    using L = WsLayout<T, kB>;
    using T2 = typename Vec2<T>::type;
    extern __shared__ __align__(128) unsigned char s_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(s_raw);
    uint64_t* empty = full + kStages;
    unsigned char* stages = s_raw + kBarBytes;
    __shared__ volatile int s_abort;
    __shared__ volatile int s_issued;  // stages issued

    const long long seg = seg_order[seg_i];
    const int t0 = win * L::kTW;
    const long long g_beg = seg_off[seg], g_end = seg_off[seg + 1];
    const int n_grp = (int)(g_end - g_beg);  // groups of one segment (< 2^31)
    if (n_grp == 0 || b_hi <= b_lo) return;   // the same for every thread of the block
    const int n_stage = (n_grp + kGps - 1) / kGps;  // stages per band
    const int n_band = kBands ? b_hi - b_lo : 1;
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumers);
        }
        s_abort = *(volatile int*)err ? 1 : 0;  // one reading of the flag for the whole block
        s_issued = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (s_abort) return;

    T acc0[L::kBins], acc1[L::kBins];
#pragma unroll
    for (int r = 0; r < L::kBins; ++r) {
        acc0[r] = T(0);
        acc1[r] = T(0);
    }

    if (warp == kConsumers) {
        // producer: lane q computes the window address of group base + q and,
        // once lane 0 has claimed the stage, issues that group's copy itself
        bool stop = false;
        for (int bi = 0; bi < n_band && !stop; ++bi) {
            const int b = b_lo + bi;
            for (int base = 0; base < n_grp && !stop; base += 32) {
                long long a0 = 0;
                if (base + lane < n_grp) {
                    const int2 h = __ldg(reinterpret_cast<const int2*>(groups + g_beg + base + lane));
                    const long long row = ((long long)h.x * nb + b) * rs + lead;
                    a0 = (row + t0 - h.y - kMaxSpan) & ~(long long)(L::kAlign - 1);  // 16-byte aligned start
                }
                const int cnt = min(32, n_grp - base);
                for (int k0 = 0; k0 < cnt; k0 += kGps) {
                    // stage index over all bands (base is a multiple of kGps)
                    const int si = bi * n_stage + (base + k0) / kGps;
                    const int st = si % kStages;
                    const int ng = min(kGps, cnt - k0);
                    int halt = 0;
                    if (lane == 0) {
                        if (s_abort) {
                            halt = 1;
                        } else if (si >= kStages && !mbar_wait(&empty[st], (unsigned)((si / kStages - 1) & 1), err)) {
                            atomicCAS(err, 0, kErrProducerWait);
                            s_abort = 1;
                            halt = 1;
                        } else {
                            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                            mbar_expect_tx(&full[st], (unsigned)(ng * (L::kWinBytes + kPackWarps * 4 +
                                                                       kTile * (int)sizeof(T))));
                        }
                    }
                    halt = __shfl_sync(0xffffffffu, halt, 0);
                    if (halt) {
                        stop = true;
                        break;
                    }
                    unsigned char* sp = stages + (size_t)st * L::kStageBytes;
                    const int q = lane - k0;  // this lane's group within the stage
                    if (q >= 0 && q < ng) bulk_copy_g2s(sp + q * L::kWinBytes, eprev + a0, L::kWinBytes, &full[st]);
                    if (lane == 0) {
                        const long long g0 = g_beg + base + k0;
                        bulk_copy_g2s(sp + L::kPackOff, wpack + g0 * kPackWarps, (unsigned)(ng * kPackWarps * 4),
                                      &full[st]);
                        bulk_copy_g2s(sp + L::kCoefOff, coef + ((size_t)b * cap + g0) * kTile,
                                      (unsigned)(ng * kTile * (int)sizeof(T)), &full[st]);
                        s_issued = si + 1;
                    }
                }
            }
        }
    } else {
        // consumer: receiver slots 2 warp and 2 warp + 1 of the tile
        const int sh = kSlotsPerWarp * warp;
        const int tile = (int)(seg / n_class), c = (int)(seg % n_class);
        bool failed = false;
        for (int bi = 0; bi < n_band && !failed; ++bi) {
            if (kBands && bi > 0) {
#pragma unroll
                for (int r = 0; r < L::kBins; ++r) {
                    acc0[r] = T(0);
                    acc1[r] = T(0);
                }
            }
            for (int sb = 0; sb < n_stage; ++sb) {
                const int si = bi * n_stage + sb;
                const int st = si % kStages;
                const bool ok = mbar_wait(&full[st], (unsigned)((si / kStages) & 1), err);
                if (!__all_sync(0xffffffffu, ok)) {  // the whole warp leaves together
                    if (lane == 0) {
                        atomicCAS(err, 0, kErrConsumerWait);
                        s_abort = 1;
                    }
                    failed = true;
                    break;
                }
                const unsigned char* sp = stages + (size_t)st * L::kStageBytes;
                const int ng = min(kGps, n_grp - sb * kGps);
                const uint32_t* packs = reinterpret_cast<const uint32_t*>(sp + L::kPackOff) + warp;
                const T* coefs = reinterpret_cast<const T*>(sp + L::kCoefOff) + sh;
                // the stage's words first (independent loads), then the windows
                uint32_t pk[kGps];
                T2 cf[kGps];
#pragma unroll
                for (int q = 0; q < kGps; ++q) {
                    pk[q] = q < ng ? packs[q * kPackWarps] : 0u;  // 0: no member of this warp
                    cf[q] = *reinterpret_cast<const T2*>(coefs + q * kTile);
                }
#pragma unroll
                for (int q = 0; q < kGps; ++q) {
                    const unsigned bits = (pk[q] >> 12) & 3u;
                    // the word's alignment field holds (-n_base - kMaxSpan) mod 4
                    const int base_off = kMaxSpan + (int)((pk[q] >> 14) & (unsigned)(L::kAlign - 1));
                    const T* w = reinterpret_cast<const T*>(sp + q * L::kWinBytes);
                    if (bits & 1u) slot_window(acc0, w, cf[q].x, (int)(pk[q] & 63u), base_off, lane);
                    if (bits & 2u) slot_window(acc1, w, cf[q].y, (int)((pk[q] >> 6) & 63u), base_off, lane);
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&empty[st]);
            }
            if (failed) break;
            if constexpr (kBands) {
                // this band's rows of the warp's two slots
                const int b = b_lo + bi;
#pragma unroll
                for (int h = 0; h < kSlotsPerWarp; ++h) {
                    const int j = tile_recv[tile * kTile + sh + h];
                    if (j < 0) continue;
                    T* out = gout + (((size_t)j * n_class + c) * nb + b) * nt + t0 + lane;
#pragma unroll
                    for (int r = 0; r < L::kBins; ++r)
                        if (t0 + lane + 32 * r < nt) out[32 * r] = h == 0 ? acc0[r] : acc1[r];
                }
            }
        }
    }
    __syncthreads();
    if (s_abort) {
        // drain: wait (bounded) until every issued copy has landed; only the
        // last kStages stages can still have copies in flight
        if (threadIdx.x == 0) {
            const int issued = s_issued;
            bool landed = true;
            for (int si = issued - 1; si >= 0 && si >= issued - kStages; --si)
                if (!mbar_drain(&full[si % kStages], (unsigned)((si / kStages) & 1))) {
                    atomicCAS(err, 0, kErrDrain);
                    landed = false;
                }
            if (landed)
                for (int s = 0; s < kStages; ++s) {
                    mbar_inval(&full[s]);
                    mbar_inval(&empty[s]);
                }
        }
        return;
    }
    if (threadIdx.x == 0)  // every stage is consumed: the barriers are done with
        for (int s = 0; s < kStages; ++s) {
            mbar_inval(&full[s]);
            mbar_inval(&empty[s]);
        }
    if constexpr (!kBands) {
        if (warp < kConsumers) {
            const int tile = (int)(seg / n_class), c = (int)(seg % n_class);
#pragma unroll
            for (int h = 0; h < kSlotsPerWarp; ++h) {
                const int j = tile_recv[tile * kTile + kSlotsPerWarp * warp + h];
                if (j < 0) continue;
                T* out = gout + (((size_t)j * n_class + c) * nb + b_lo) * nt + t0 + lane;
#pragma unroll
                for (int r = 0; r < L::kBins; ++r)
                    if (t0 + lane + 32 * r < nt) out[32 * r] = h == 0 ? acc0[r] : acc1[r];
            }
        }
    }
}

#define SP_SCATTER_ARGS(T)                                                                                 \
    int n_class, int nb, int nt, long long rs, int lead, long long cap, const int32_t *__restrict__ tile_recv, \
        const int32_t *__restrict__ seg_order, const int64_t *__restrict__ seg_off,                           \
        const Group *__restrict__ groups, const uint32_t *__restrict__ wpack, const T *__restrict__ coef,      \
        const T *__restrict__ eprev, T *__restrict__ gout, int *__restrict__ err
__global__ void __launch_bounds__(kWsThreads, 2) k_scatter_f32(SP_SCATTER_ARGS(float)) {
    scatter_ws<float>(n_class, nb, nt, rs, lead, cap, tile_recv, seg_order, seg_off, groups, wpack, coef, eprev, gout,
                      err, blockIdx.x, blockIdx.y, blockIdx.z, blockIdx.z + 1);
}
__global__ void __launch_bounds__(kWsThreads, 2) k_scatter_f64(SP_SCATTER_ARGS(double)) {
    scatter_ws<double>(n_class, nb, nt, rs, lead, cap, tile_recv, seg_order, seg_off, groups, wpack, coef, eprev, gout,
                       err, blockIdx.x, blockIdx.y, blockIdx.z, blockIdx.z + 1);
}
#undef SP_SCATTER_ARGS

}  // namespace
