// Tiled structured energy exchange (RadiosityFast.py:1073-1145) for BRDF
// tables whose rows are  diff + spec * [o == m]  up to a per-slot scale:
//   BRDF[slot, s, o, b] = scale[slot, b] * (diff[c, b] + spec[c, b] * [o == m_c]),
// c = (material group of the slot, s) is the pair's class.  This is the form
// brdf.py:100-120 (`create_from_scattering`) produces, stored times pi.
//
// For receiver j and order k:
//   G_k[j, c, b, t] = sum_{pairs p -> j of class c} w_pb * E_{k-1}[src_p, p2o_p, b, t - n_p]
//   E_k[j, o, b, t] = sum_c (diff[c, b] + spec[c, b] [o == m_c]) * G_k[j, c, b, t]
//   E_total += E_k
// with w_pb = F'_p * exp(-att_b |u_p|) * scale[slot(src_p), b].
//
// Plan (once per exchange call): receivers are cut into tiles of 16 (a given
// receiver order, normally spatial); a segment is (tile, class).  The
// segment's pairs are merged by source patch and cut into source groups:
// one source row (src * D + p2o), up to 16 member receivers, delays within
// n_base .. n_base + 45.  Everything is built in parallel and
// deterministically (row-wise class sort, merge by binary search, scans).
//
// Scatter (per order, FP32): one CTA per (segment, 1024-bin window, band),
// 128 threads; thread tid owns bins t0 + tid + 128 r (r < 8) of all 16
// receivers in registers.  Each group's source window (1072 values) is
// staged in shared memory by a bulk asynchronous copy (cp.async.bulk +
// mbarrier, 12 stages, refilled by the last warp to finish a stage); every
// member reads the staged window at its own delay offset, each warp read
// covering 32 consecutive floats, so one staged window feeds every member
// of the group.  FP64 uses the same plan with direct loads.  Mix: streams G
// into E_k and E_total.
#include "common.cuh"
#include <algorithm>
#include <vector>

#include "exchange_common.cuh"

namespace {

constexpr int kTile = 16;         // receivers per tile
constexpr int kMaxSpan = 45;      // max delay spread inside a source group
constexpr int kMaxClasses = 256;

struct Group {
    int32_t srcrow;      // src * D + p2o
    int32_t n_base;      // smallest delay of the members
    uint32_t mask;       // bit w set: receiver slot w of the tile is a member
    int32_t pad;
    uint8_t off[kTile];  // per slot: delay - n_base (0 .. kMaxSpan)
};
static_assert(sizeof(Group) == 32, "Group is copied in 16-byte units");

// ------------------------------------------------------------------ plan
__global__ void k_delays_t(long long n_dir, const double* __restrict__ dist, double c, double dt,
                           int32_t* __restrict__ delay) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_dir) return;
    delay[e] = (int32_t)(long long)xdiv(xdiv(dist[e], c), dt);
}

__global__ void k_pair_class_t(long long n_dir, const int32_t* __restrict__ src, const int32_t* __restrict__ in_dir,
                               const int32_t* __restrict__ wall_of, const int32_t* __restrict__ brdf_index,
                               const int32_t* __restrict__ slot_group, int n_in, int32_t* __restrict__ cls) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_dir) return;
    int slot = brdf_index[wall_of[src[e]]];
    cls[e] = slot_group[slot] * n_in + in_dir[e];
}

// Stable counting sort of each destination row by class (one warp per row);
// writes the class boundaries rco[j * (C + 1) + c] and the row of each position.
__global__ void k_row_sort_by_class_t(int n, const int64_t* __restrict__ off, const int32_t* __restrict__ cls,
                                      int n_class, int64_t* __restrict__ perm, int64_t* __restrict__ rco,
                                      int32_t* __restrict__ row_of) {
    extern __shared__ int s_hist[];
    int j = blockIdx.x;
    int lane = threadIdx.x;
    long long b = off[j], e = off[j + 1];
    for (int c = lane; c < n_class; c += 32) s_hist[c] = 0;
    __syncwarp();
    for (long long k = b + lane; k < e; k += 32) {
        atomicAdd(&s_hist[cls[k]], 1);
        row_of[k] = j;
    }
    __syncwarp();
    if (lane == 0) {
        int run = 0;
        for (int c = 0; c < n_class; ++c) {
            int h = s_hist[c];
            s_hist[c] = run;
            rco[(size_t)j * (n_class + 1) + c] = b + run;
            run += h;
        }
        rco[(size_t)j * (n_class + 1) + n_class] = b + run;
    }
    __syncwarp();
    for (long long k0 = b; k0 < e; k0 += 32) {
        long long k = k0 + lane;
        bool on = k < e;
        unsigned active = __ballot_sync(0xffffffffu, on);
        if (on) {
            int c = cls[k];
            unsigned peers = __match_any_sync(active, c);
            int rank = __popc(peers & ((1u << lane) - 1u));
            int pos = s_hist[c] + rank;
            perm[b + pos] = k;
            __syncwarp(active);
            if (rank == 0) s_hist[c] += __popc(peers);
        }
        __syncwarp();
    }
}

__global__ void k_default_tiles(int n, int n_tiles, const int32_t* __restrict__ order, int32_t* __restrict__ tile_recv,
                                int32_t* __restrict__ tile_of, int32_t* __restrict__ slot_of) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_tiles * kTile) return;
    int j = (k < n) ? (order ? order[k] : k) : -1;
    tile_recv[k] = j;
    if (j >= 0) {
        tile_of[j] = k / kTile;
        slot_of[j] = k % kTile;
    }
}

__global__ void k_seg_size(long long n_seg, int n_class, const int32_t* __restrict__ tile_recv,
                           const int64_t* __restrict__ rco, int64_t* __restrict__ seg_size) {
    long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_seg) return;
    int tile = (int)(s / n_class), c = (int)(s % n_class);
    long long tot = 0;
    for (int w = 0; w < kTile; ++w) {
        int j = tile_recv[tile * kTile + w];
        if (j >= 0) tot += rco[(size_t)j * (n_class + 1) + c + 1] - rco[(size_t)j * (n_class + 1) + c];
    }
    seg_size[s] = tot;
}

// Multi-block exclusive scan of int64 values: block sums, scan of the sums,
// add-back.  out[n] = total.
constexpr int kScanBlock = 1024;
__global__ void k_scan_blocks(long long n, const int64_t* __restrict__ in, int64_t* __restrict__ out,
                              int64_t* __restrict__ block_sums) {
    __shared__ int64_t s[kScanBlock];
    long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
    int64_t v = (i < n) ? in[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        int64_t x = (threadIdx.x >= (unsigned)off) ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += x;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = s[kScanBlock - 1];
}
__global__ void k_scan_sums(long long nblocks, int64_t* __restrict__ sums, int64_t* __restrict__ total) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int64_t run = 0;
    for (long long k = 0; k < nblocks; ++k) {
        int64_t v = sums[k];
        sums[k] = run;
        run += v;
    }
    *total = run;
}
__global__ void k_scan_add(long long n, int64_t* __restrict__ out, const int64_t* __restrict__ sums) {
    long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
}

// Position of one entry inside its segment's (src, slot)-ordered merge.
__device__ __forceinline__ long long count_before(const int64_t* __restrict__ perm, const int32_t* __restrict__ src,
                                                  long long lo, long long hi, int key, bool inclusive) {
    // number of list elements (sorted by src) with src < key (or <= key)
    while (lo < hi) {
        long long mid = (lo + hi) >> 1;
        int v = src[perm[mid]];
        if (v < key || (inclusive && v == key))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__global__ void k_merge_positions(long long n_dir, int n_class, const int64_t* __restrict__ perm,
                                  const int32_t* __restrict__ row_of, const int32_t* __restrict__ cls,
                                  const int32_t* __restrict__ src, const int64_t* __restrict__ rco,
                                  const int32_t* __restrict__ tile_of, const int32_t* __restrict__ slot_of,
                                  const int32_t* __restrict__ tile_recv, const int64_t* __restrict__ seg_base,
                                  int64_t* __restrict__ merged) {
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_dir) return;
    long long e = perm[q];
    int j = row_of[q];
    int c = cls[e];
    int key = src[e];
    int tile = tile_of[j], w = slot_of[j];
    long long pos = q - rco[(size_t)j * (n_class + 1) + c];
    for (int w2 = 0; w2 < kTile; ++w2) {
        if (w2 == w) continue;
        int j2 = tile_recv[tile * kTile + w2];
        if (j2 < 0) continue;
        long long lo = rco[(size_t)j2 * (n_class + 1) + c], hi = rco[(size_t)j2 * (n_class + 1) + c + 1];
        pos += count_before(perm, src, lo, hi, key, w2 < w) - lo;
    }
    merged[seg_base[(long long)tile * n_class + c] + pos] = e;
}

// Cells: runs of equal (segment, src) in merged order (<= 8 entries, one per
// receiver).  For each cell start: sort members by (p2o, delay), cut into
// groups; write == 0 counts, write == 1 emits.
template <typename T>
__global__ void k_cells(long long n_dir, int nd, int nb, int nt, const int64_t* __restrict__ merged,
                        const int32_t* __restrict__ src, const int32_t* __restrict__ dst, const int32_t* __restrict__ out_dir,
                        const int32_t* __restrict__ delay, const int32_t* __restrict__ cls,
                        const int32_t* __restrict__ tile_of, const int32_t* __restrict__ slot_of,
                        const double* __restrict__ fprime, const double* __restrict__ unit_len,
                        const double* __restrict__ att, const int32_t* __restrict__ wall_of,
                        const int32_t* __restrict__ brdf_index, const double* __restrict__ slot_scale, int write,
                        int64_t* __restrict__ cell_count, const int64_t* __restrict__ cell_base,
                        long long cap, Group* __restrict__ groups, T* __restrict__ coef) {
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_dir) return;
    long long e = merged[q];
    int s_src = src[e];
    int s_tile = tile_of[dst[e]];
    int s_cls = cls[e];
    if (q > 0) {
        long long ep = merged[q - 1];
        if (src[ep] == s_src && tile_of[dst[ep]] == s_tile && cls[ep] == s_cls) {
            if (!write) cell_count[q] = 0;
            return;
        }
    }
    int mo[kTile], md[kTile], mw[kTile];
    long long me[kTile];
    int m = 0;
    for (long long k = q; k < n_dir && m < kTile; ++k) {
        long long ek = merged[k];
        if (src[ek] != s_src || tile_of[dst[ek]] != s_tile || cls[ek] != s_cls) break;
        int dl = delay[ek];
        if (dl >= nt) continue;  // contributes nothing inside the histogram
        mo[m] = out_dir[ek];
        md[m] = dl;
        mw[m] = slot_of[dst[ek]];
        me[m] = ek;
        ++m;
    }
    for (int a = 1; a < m; ++a) {
        int to = mo[a], td = md[a], tw = mw[a];
        long long te = me[a];
        int r = a - 1;
        while (r >= 0 && (mo[r] > to || (mo[r] == to && md[r] > td))) {
            mo[r + 1] = mo[r];
            md[r + 1] = md[r];
            mw[r + 1] = mw[r];
            me[r + 1] = me[r];
            --r;
        }
        mo[r + 1] = to;
        md[r + 1] = td;
        mw[r + 1] = tw;
        me[r + 1] = te;
    }
    long long g_out = write ? cell_base[q] : 0;
    long long n_groups = 0;
    int slot = brdf_index[wall_of[s_src]];
    int a = 0;
    while (a < m) {
        int r = a;
        while (r + 1 < m && mo[r + 1] == mo[a] && md[r + 1] - md[a] <= kMaxSpan) ++r;
        if (write) {
            Group g;
            g.srcrow = s_src * nd + mo[a];
            g.n_base = md[a];
            g.mask = 0;
            g.pad = 0;
            for (int k = 0; k < kTile; ++k) g.off[k] = 0;
            for (int b = 0; b < nb; ++b)
                for (int k = 0; k < kTile; ++k) coef[((size_t)b * cap + g_out) * kTile + k] = T(0);
            for (int x = a; x <= r; ++x) {
                const int w = mw[x];
                g.mask |= 1u << w;
                g.off[w] = (uint8_t)(md[x] - md[a]);
                long long ex = me[x];
                for (int b = 0; b < nb; ++b) {
                    double f = fprime[ex];
                    if (att) f = f * exp(-att[b] * unit_len[ex]);
                    coef[((size_t)b * cap + g_out) * kTile + w] = (T)(f * slot_scale[(size_t)slot * nb + b]);
                }
            }
            groups[g_out] = g;
            ++g_out;
        }
        ++n_groups;
        a = r + 1;
    }
    if (!write) cell_count[q] = n_groups;
}

// seg_off[s] = group index of the first cell of segment s.
__global__ void k_seg_offsets(long long n_seg, long long n_dir, const int64_t* __restrict__ seg_base,
                              const int64_t* __restrict__ cell_base, int64_t* __restrict__ seg_off) {
    long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s > n_seg) return;
    long long q = seg_base[s];
    seg_off[s] = (q < n_dir) ? cell_base[q] : cell_base[n_dir];
}

// --------------------------------------------------------- PTX helpers
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
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
constexpr unsigned kWaitLimit = 1u << 16;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, const volatile int* err) {
    for (unsigned it = 0; it < kWaitLimit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 255u && *err) return false;
    }
    return false;
}
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

// --------------------------------------------------------- FP32 scatter
// Warp-specialised pipeline.  One producer warp streams the groups of a
// segment through kStages shared-memory stages of kGps groups each, with
// bulk copies (per group the source window; per stage the kGps 32-byte group
// records and their 16 coefficients of this band).  kConsumers consumer
// warps, warp w owning receiver slots 2w and 2w + 1 of the tile, accumulate
// those slots' 1024-bin windows in registers (lane l owns bins t0 + l + 32 r).
// Stage hand-off: `full` (producer arrival + transaction bytes) and `empty`
// (one arrival per consumer warp); every wait is bounded.
constexpr int kThreads = 128;                        // FP64 scatter block
constexpr int kSlotsPerWarp = 2;
constexpr int kConsumers = kTile / kSlotsPerWarp;    // 8 consumer warps
constexpr int kWsThreads = (kConsumers + 1) * 32;    // + one producer warp
constexpr int kBins = 32;                            // bins per lane, strided by 32
constexpr int kTW = 32 * kBins;                      // 1024 bins per window
constexpr int kStageF = kTW + kMaxSpan + 3;          // staged floats per group (multiple of 4)
static_assert(kStageF % 4 == 0, "staged window must be a whole number of 16-byte chunks");
constexpr int kGps = 4;                              // groups per stage
constexpr int kWinBytes = kStageF * 4;
constexpr int kHdrOff = kGps * kWinBytes;            // kGps group records
constexpr int kCoefOff = kHdrOff + kGps * (int)sizeof(Group);  // kGps x 16 coefficients
constexpr int kStageBytes = kCoefOff + kGps * kTile * 4;
static_assert(kWinBytes % 16 == 0 && kHdrOff % 16 == 0 && kCoefOff % 16 == 0 && kStageBytes % 16 == 0,
              "stage parts must stay 16-byte aligned");
constexpr int kStages = 6;
constexpr int kBarBytes = 128;                       // full[kStages], empty[kStages]
static_assert(2 * kStages * 8 <= kBarBytes, "barrier area too small");
constexpr size_t kScatterSmem = (size_t)kBarBytes + (size_t)kStages * kStageBytes;

// acc[r] += cf * staged[lane + 32 r + base - off] for one member slot, with
// base = kMaxSpan + mu (mu: floats the staged start was rounded down by).
__device__ __forceinline__ void slot_window(float (&acc)[kBins], const float* win, float cf, int off, int base,
                                            int lane) {
    const float* p = win + lane + base - off;
#pragma unroll
    for (int r = 0; r < kBins; ++r) acc[r] = fmaf(cf, p[32 * r], acc[r]);
}

// One order, one band, one 1024-bin window: G[j, c, b, window] for the 16
// receivers of a segment.  Histogram rows of eprev are padded: row r starts
// at r * rs with bin 0 at offset `lead` (>= nt + kMaxSpan + 4 zeros before
// it), so a staged window reaching before bin 0 reads zeros and needs no
// masking, and no window starts before the buffer.  Every shared-memory read
// of a consumer warp covers 32 consecutive floats (no bank conflict at any
// offset).
__global__ void __launch_bounds__(kWsThreads, 2) k_scatter_f32(int n_class, int nb, int nt, long long rs, int lead,
                                                               long long cap, const int32_t* __restrict__ tile_recv,
                                                               const int32_t* __restrict__ seg_order,
                                                               const int64_t* __restrict__ seg_off,
                                                               const Group* __restrict__ groups,
                                                               const float* __restrict__ coef,
                                                               const float* __restrict__ eprev,
                                                               float* __restrict__ gout, int* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char s_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(s_raw);
    uint64_t* empty = full + kStages;
    unsigned char* stages = s_raw + kBarBytes;
    __shared__ volatile int s_abort;
    __shared__ volatile int s_issued;  // stages issued

    const long long seg = seg_order[blockIdx.x];
    const int b = blockIdx.z;
    const int t0 = blockIdx.y * kTW;
    const long long g_beg = seg_off[seg], g_end = seg_off[seg + 1];
    const int n_grp = (int)(g_end - g_beg);  // groups of one segment (< 2^31)
    if (n_grp == 0) return;                   // the same for every thread of the block
    const int n_stage = (n_grp + kGps - 1) / kGps;
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

    float acc0[kBins], acc1[kBins];
#pragma unroll
    for (int r = 0; r < kBins; ++r) {
        acc0[r] = 0.0f;
        acc1[r] = 0.0f;
    }

    if (warp == kConsumers) {
        // producer: lane q computes the window address of group base + q and,
        // once lane 0 has claimed the stage, issues that group's copy itself
        bool stop = false;
        for (int base = 0; base < n_grp && !stop; base += 32) {
            long long a0 = 0;
            if (base + lane < n_grp) {
                const int2 h = __ldg(reinterpret_cast<const int2*>(groups + g_beg + base + lane));
                const long long row = ((long long)h.x * nb + b) * rs + lead;
                a0 = (row + t0 - h.y - kMaxSpan) & ~3LL;  // 16-byte aligned start of the window
            }
            const int cnt = min(32, n_grp - base);
            for (int k0 = 0; k0 < cnt; k0 += kGps) {
                const int si = (base + k0) / kGps;  // stage index (base is a multiple of kGps)
                const int st = si % kStages;
                const int ng = min(kGps, cnt - k0);
                int halt = 0;
                if (lane == 0) {
                    if (s_abort) {
                        halt = 1;
                    } else if (si >= kStages && !mbar_wait(&empty[st], (unsigned)((si / kStages - 1) & 1), err)) {
                        atomicExch(err, 1);
                        s_abort = 1;
                        halt = 1;
                    } else {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        mbar_expect_tx(&full[st], (unsigned)(ng * (kWinBytes + (int)sizeof(Group) + kTile * 4)));
                    }
                }
                halt = __shfl_sync(0xffffffffu, halt, 0);
                if (halt) {
                    stop = true;
                    break;
                }
                unsigned char* sp = stages + (size_t)st * kStageBytes;
                const int q = lane - k0;  // this lane's group within the stage
                if (q >= 0 && q < ng) bulk_copy_g2s(sp + q * kWinBytes, eprev + a0, kWinBytes, &full[st]);
                if (lane == 0) {
                    const long long g0 = g_beg + base + k0;
                    bulk_copy_g2s(sp + kHdrOff, groups + g0, (unsigned)(ng * sizeof(Group)), &full[st]);
                    bulk_copy_g2s(sp + kCoefOff, coef + ((size_t)b * cap + g0) * kTile, (unsigned)(ng * kTile * 4),
                                  &full[st]);
                    s_issued = si + 1;
                }
            }
        }
    } else {
        // consumer: receiver slots 2 warp and 2 warp + 1 of the tile
        const int sh = kSlotsPerWarp * warp;
        for (int si = 0; si < n_stage; ++si) {
            const int st = si % kStages;
            const bool ok = mbar_wait(&full[st], (unsigned)((si / kStages) & 1), err);
            if (!__all_sync(0xffffffffu, ok)) {  // the whole warp leaves together
                if (lane == 0) {
                    atomicExch(err, 1);
                    s_abort = 1;
                }
                break;
            }
            const unsigned char* sp = stages + (size_t)st * kStageBytes;
            const int ng = min(kGps, n_grp - si * kGps);
            // the stage's records first (independent loads), then the windows
            unsigned bits[kGps];
            int base_off[kGps];  // kMaxSpan + mu, per group
            float2 cf[kGps];
            unsigned offs[kGps];  // off of slot sh (low byte) and sh + 1 (second byte)
#pragma unroll
            for (int q = 0; q < kGps; ++q) {
                const Group* g = reinterpret_cast<const Group*>(sp + kHdrOff) + q;
                // record at a 16-byte boundary: srcrow, n_base, mask, pad
                const int4 hdr = q < ng ? *reinterpret_cast<const int4*>(g) : make_int4(0, 0, 0, 0);
                bits[q] = ((unsigned)hdr.z >> sh) & 3u;
                base_off[q] = kMaxSpan + ((-hdr.y - kMaxSpan) & 3);  // staged start was rounded down by mu floats
                cf[q] = *reinterpret_cast<const float2*>(reinterpret_cast<const float*>(sp + kCoefOff) + q * kTile + sh);
                offs[q] = *reinterpret_cast<const uint16_t*>(&g->off[sh]);
            }
#pragma unroll
            for (int q = 0; q < kGps; ++q) {
                const float* win = reinterpret_cast<const float*>(sp + q * kWinBytes);
                if (bits[q] & 1u) slot_window(acc0, win, cf[q].x, (int)(offs[q] & 0xffu), base_off[q], lane);
                if (bits[q] & 2u) slot_window(acc1, win, cf[q].y, (int)(offs[q] >> 8), base_off[q], lane);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
        }
    }
    __syncthreads();
    if (s_abort) {
        // drain: wait (bounded) until every issued copy has landed
        if (threadIdx.x == 0) {
            const int issued = s_issued;
            for (int si = issued - 1; si >= 0 && si >= issued - kStages; --si)
                mbar_wait(&full[si % kStages], (unsigned)((si / kStages) & 1), err);
        }
        return;
    }
    if (warp < kConsumers) {
        const int tile = (int)(seg / n_class), c = (int)(seg % n_class);
#pragma unroll
        for (int h = 0; h < kSlotsPerWarp; ++h) {
            const int j = tile_recv[tile * kTile + kSlotsPerWarp * warp + h];
            if (j < 0) continue;
            float* out = gout + (((size_t)j * n_class + c) * nb + b) * nt + t0 + lane;
#pragma unroll
            for (int r = 0; r < kBins; ++r)
                if (t0 + lane + 32 * r < nt) out[32 * r] = h == 0 ? acc0[r] : acc1[r];
        }
    }
}

// --------------------------------------------------------- FP64 scatter
constexpr int kR64 = 4;
constexpr int kTW64 = kThreads * kR64;

template <int W>
__device__ __forceinline__ void slot_f64(double (&acc)[kTile][kR64], const Group& g, const double* sp, const double* cf) {
    if (g.mask & (1u << W)) {
        const double cfw = cf[W];
        const double* p = sp - g.off[W];
#pragma unroll
        for (int r = 0; r < kR64; ++r) acc[W][r] = fma(cfw, __ldg(p + kThreads * r), acc[W][r]);
    }
}
__device__ __forceinline__ void group_f64(double (&acc)[kTile][kR64], const Group& g, const double* sp, const double* cf) {
    slot_f64<0>(acc, g, sp, cf);
    slot_f64<1>(acc, g, sp, cf);
    slot_f64<2>(acc, g, sp, cf);
    slot_f64<3>(acc, g, sp, cf);
    slot_f64<4>(acc, g, sp, cf);
    slot_f64<5>(acc, g, sp, cf);
    slot_f64<6>(acc, g, sp, cf);
    slot_f64<7>(acc, g, sp, cf);
    slot_f64<8>(acc, g, sp, cf);
    slot_f64<9>(acc, g, sp, cf);
    slot_f64<10>(acc, g, sp, cf);
    slot_f64<11>(acc, g, sp, cf);
    slot_f64<12>(acc, g, sp, cf);
    slot_f64<13>(acc, g, sp, cf);
    slot_f64<14>(acc, g, sp, cf);
    slot_f64<15>(acc, g, sp, cf);
}

// FP64: same plan, direct (L1-cached) loads, thread owns bins t0 + tid + 128 r.
__global__ void __launch_bounds__(kThreads) k_scatter_f64(int n_class, int nb, int nt, long long rs, int lead,
                                                          long long cap, const int32_t* __restrict__ tile_recv,
                                                          const int32_t* __restrict__ seg_order,
                                                          const int64_t* __restrict__ seg_off,
                                                          const Group* __restrict__ groups,
                                                          const double* __restrict__ coef,
                                                          const double* __restrict__ eprev,
                                                          double* __restrict__ gout) {
    const long long seg = seg_order[blockIdx.x];
    const int b = blockIdx.z;
    const int t0 = blockIdx.y * kTW64;
    const long long g_beg = seg_off[seg], g_end = seg_off[seg + 1];
    if (g_beg == g_end) return;
    const int tid = threadIdx.x;
    const int tile = (int)(seg / n_class), c = (int)(seg % n_class);
    double acc[kTile][kR64];
#pragma unroll
    for (int w = 0; w < kTile; ++w)
#pragma unroll
        for (int r = 0; r < kR64; ++r) acc[w][r] = 0.0;
    for (long long gidx = g_beg; gidx < g_end; ++gidx) {
        const Group& g = groups[gidx];  // read in place (no local copy)
        const double* cf = coef + ((size_t)b * cap + gidx) * kTile;
        // padded rows: the zero lead covers source indices below 0
        const double* sp = eprev + ((long long)g.srcrow * nb + b) * rs + lead + t0 + tid - g.n_base;
        group_f64(acc, g, sp, cf);
    }
#pragma unroll
    for (int w = 0; w < kTile; ++w) {
        int j = tile_recv[tile * kTile + w];
        if (j < 0) continue;
        double* out = gout + (((size_t)j * n_class + c) * nb + b) * nt + t0 + tid;
#pragma unroll
        for (int r = 0; r < kR64; ++r)
            if (t0 + tid + kThreads * r < nt) out[kThreads * r] = acc[w][r];
    }
}

// --------------------------------------------------------------- mix
// E_k[j, o, b, t] = sum_c (diff_c + spec_c [o == m_c]) G[j, c, b, t];  E_total += E_k.
// Per tile: the classes present (segments with groups) and, per outgoing
// direction o, the present classes whose mirror direction is o.  Layout of a
// row of kTab(n_class, nd) ints: [np, cls[n_class], inv_off[nd + 1], inv[n_class]].
__host__ __device__ inline int tile_tab_stride(int n_class, int nd) { return 2 + 2 * n_class + nd; }

__global__ void k_tile_table(int n_tiles, int n_class, int nd, const int64_t* __restrict__ seg_off,
                             const int32_t* __restrict__ ctarget, int32_t* __restrict__ tab) {
    const int tile = blockIdx.x * blockDim.x + threadIdx.x;
    if (tile >= n_tiles) return;
    int32_t* row = tab + (size_t)tile * tile_tab_stride(n_class, nd);
    int32_t* cls = row + 1;
    int32_t* inv_off = cls + n_class;
    int32_t* inv = inv_off + nd + 1;
    int np = 0;
    for (int c = 0; c < n_class; ++c) {
        const long long sg = (long long)tile * n_class + c;
        if (seg_off[sg + 1] > seg_off[sg]) cls[np++] = c;
    }
    row[0] = np;
    int k = 0;
    for (int o = 0; o < nd; ++o) {
        inv_off[o] = k;
        for (int q = 0; q < np; ++q)
            if (ctarget[cls[q]] == o) inv[k++] = cls[q];
    }
    inv_off[nd] = k;
}

// E_k[j, o, b, t] = sum_c diff[c, b] G[j, c, b, t] + sum_{c: m_c = o} spec[c, b] G[j, c, b, t]
// (the slot scale is folded into the scatter coefficients), written to the
// padded row of ecur, and E_total += E_k.  One block per (band, receiver),
// all bins; only the classes present in the receiver's tile are read.
template <typename T>
__global__ void __launch_bounds__(256) k_mix(int n_class, int nd, int nb, int nt, long long rs, int lead,
                                             const int32_t* __restrict__ tile_of, const int32_t* __restrict__ tab,
                                             const T* __restrict__ cdiff, const T* __restrict__ cspec,
                                             const T* __restrict__ g, T* __restrict__ ecur, T* __restrict__ etot) {
    extern __shared__ __align__(16) unsigned char s_mix[];
    const int stride = tile_tab_stride(n_class, nd);
    T* s_cd = reinterpret_cast<T*>(s_mix);  // [n_class] diffuse weight of band b
    T* s_cs = s_cd + n_class;               // [n_class] specular weight of band b
    int* s_tab = reinterpret_cast<int*>(s_cs + n_class);
    const int b = blockIdx.x, j = blockIdx.y;
    const int tile = tile_of[j];
    for (int k = threadIdx.x; k < stride; k += blockDim.x) s_tab[k] = tab[(size_t)tile * stride + k];
    for (int c = threadIdx.x; c < n_class; c += blockDim.x) {
        s_cd[c] = cdiff[(size_t)c * nb + b];
        s_cs[c] = cspec[(size_t)c * nb + b];
    }
    __syncthreads();
    const int np = s_tab[0];
    const int* cls = s_tab + 1;
    const int* inv_off = cls + n_class;
    const int* inv = inv_off + nd + 1;
    const size_t cstride = (size_t)nb * nt;
    const T* gj = g + ((size_t)j * n_class * nb + b) * nt;
    T* ek = ecur + ((size_t)j * nd * nb + b) * rs + lead;  // padded rows, stride rs
    T* et = etot + ((size_t)j * nd * nb + b) * nt;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        T diffuse = T(0);
        for (int q = 0; q < np; ++q) {
            const int c = cls[q];
            diffuse = fma(s_cd[c], gj[c * cstride + t], diffuse);
        }
        for (int o = 0; o < nd; ++o) {
            T v = diffuse;
            for (int q = inv_off[o]; q < inv_off[o + 1]; ++q) {
                const int c = inv[q];
                v = fma(s_cs[c], gj[c * cstride + t], v);
            }
            ek[(size_t)o * nb * rs + t] = v;
            et[o * cstride + t] += v;
        }
    }
}

// k_mix for FP32 with nt % 4 == 0: four bins per thread (16-byte accesses),
// and the E_total values of up to 8 directions loaded before any is stored.
__device__ __forceinline__ float4 fma4(float a, float4 x, float4 y) {
    return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}
__device__ __forceinline__ float4 add4(float4 x, float4 y) {
    return make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
}

__global__ void __launch_bounds__(128) k_mix4(int n_class, int nd, int nb, int nt, long long rs, int lead,
                                              const int32_t* __restrict__ tile_of, const int32_t* __restrict__ tab,
                                              const float* __restrict__ cdiff, const float* __restrict__ cspec,
                                              const float* __restrict__ g, float* __restrict__ ecur,
                                              float* __restrict__ etot) {
    extern __shared__ __align__(16) unsigned char s_mix[];
    const int stride = tile_tab_stride(n_class, nd);
    float* s_cd = reinterpret_cast<float*>(s_mix);
    float* s_cs = s_cd + n_class;
    int* s_tab = reinterpret_cast<int*>(s_cs + n_class);
    const int b = blockIdx.x, j = blockIdx.y;
    const int tile = tile_of[j];
    for (int k = threadIdx.x; k < stride; k += blockDim.x) s_tab[k] = tab[(size_t)tile * stride + k];
    for (int c = threadIdx.x; c < n_class; c += blockDim.x) {
        s_cd[c] = cdiff[(size_t)c * nb + b];
        s_cs[c] = cspec[(size_t)c * nb + b];
    }
    __syncthreads();
    const int np = s_tab[0];
    const int* cls = s_tab + 1;
    const int* inv_off = cls + n_class;
    const int* inv = inv_off + nd + 1;
    const int nt4 = nt >> 2;
    const size_t cs4 = (size_t)nb * nt4;  // class (G) and direction (E_total) stride, in float4
    const size_t ers4 = (size_t)nb * (size_t)(rs >> 2);  // direction stride of the padded ecur rows
    const float4* gj = reinterpret_cast<const float4*>(g + ((size_t)j * n_class * nb + b) * nt);
    float4* ek = reinterpret_cast<float4*>(ecur + ((size_t)j * nd * nb + b) * rs + lead);
    float4* et = reinterpret_cast<float4*>(etot + ((size_t)j * nd * nb + b) * nt);
    for (int t = threadIdx.x; t < nt4; t += blockDim.x) {
        float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int q = 0; q < np; ++q) {
            const int c = cls[q];
            d = fma4(s_cd[c], __ldg(gj + c * cs4 + t), d);
        }
        for (int o0 = 0; o0 < nd; o0 += 8) {
            const int no = min(8, nd - o0);
            float4 e[8];
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < no) e[k] = et[(o0 + k) * cs4 + t];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (k < no) {
                    const int o = o0 + k;
                    float4 v = d;
                    for (int q = inv_off[o]; q < inv_off[o + 1]; ++q) {
                        const int c = inv[q];
                        v = fma4(s_cs[c], __ldg(gj + c * cs4 + t), v);
                    }
                    ek[o * ers4 + t] = v;
                    et[o * cs4 + t] = add4(e[k], v);
                }
            }
        }
    }
}

template <typename T>
__global__ void k_init_energy_t(int n, int nd, int nb, int nt, long long rs, int lead, const double* __restrict__ e0dir,
                                const double* __restrict__ d0, double c, double dt, T* __restrict__ etot,
                                T* __restrict__ eprev, int* __restrict__ err) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)n * nd * nb;
    if (e >= total) return;
    int i = (int)(e / ((long long)nd * nb));
    long long dly = (long long)xdiv(xdiv(d0[i], c), dt);
    if (dly < 0 || dly >= nt) {
        atomicExch(err, 1);
        return;
    }
    T v = (T)e0dir[e];
    etot[(size_t)e * nt + dly] = v;
    eprev[(size_t)e * rs + lead + dly] = v;
}

template <typename T>
__global__ void k_convert_t(long long count, const double* __restrict__ in, T* __restrict__ out) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) out[e] = (T)in[e];
}

// ------------------------------------------------------------ layout
struct Plan {
    size_t bytes;
    int lead;          // zero elements before bin 0 of every padded histogram row
    size_t rs;         // padded row stride (elements)
    size_t rows;       // N * D * B
    void* eprev;
    void* ecur;
    void* g;
    int32_t* delay;
    int32_t* cls;
    int64_t* perm;
    int32_t* row_of;
    int64_t* merged;
    int64_t* rco;
    int32_t* tile_recv;
    int32_t* tile_of;
    int32_t* slot_of;
    int64_t* seg_size;
    int64_t* seg_base;
    int64_t* seg_off;
    int32_t* tile_tab;
    int32_t* seg_order;
    int64_t* cell_count;
    int64_t* cell_base;
    int64_t* scan_tmp;
    Group* groups;
    void* coef;
    void* cdiff;
    void* cspec;
    int* err;
};

Plan plan_layout(void* base, int esz, int n, int nd, int nb, int nt, long long p, int n_class) {
    Plan L;
    char* q = (char*)base;
    auto take = [&](size_t bytes) {
        char* r = q;
        q += sp_align(bytes);
        return (void*)r;
    };
    int n_tiles = (n + kTile - 1) / kTile;
    // padded histogram rows: `lead` zeros, then nt bins; stride rs (multiple
    // of 4 elements so rows stay 16-byte aligned); a tail after the last row
    // keeps the staged windows of the last rows inside the allocation
    L.lead = (int)((((size_t)nt + kMaxSpan + 4) + 3) & ~(size_t)3);
    L.rs = (((size_t)nt + L.lead) + 3) & ~(size_t)3;
    L.rows = (size_t)n * nd * nb;
    size_t tail = (size_t)kStageF + 64;
    L.eprev = take((L.rows * L.rs + tail) * esz);
    L.ecur = take((L.rows * L.rs + tail) * esz);
    L.g = take((size_t)n * n_class * nb * nt * esz);
    L.delay = (int32_t*)take((size_t)p * 4);
    L.cls = (int32_t*)take((size_t)p * 4);
    L.perm = (int64_t*)take((size_t)p * 8);
    L.row_of = (int32_t*)take((size_t)p * 4);
    L.merged = (int64_t*)take((size_t)p * 8);
    L.rco = (int64_t*)take((size_t)n * (n_class + 1) * 8);
    L.tile_recv = (int32_t*)take((size_t)n_tiles * kTile * 4);
    L.tile_of = (int32_t*)take((size_t)n * 4);
    L.slot_of = (int32_t*)take((size_t)n * 4);
    long long n_seg = (long long)n_tiles * n_class;
    L.seg_size = (int64_t*)take(((size_t)n_seg + 1) * 8);
    L.seg_base = (int64_t*)take(((size_t)n_seg + 1) * 8);
    L.seg_off = (int64_t*)take(((size_t)n_seg + 1) * 8);
    L.tile_tab = (int32_t*)take((size_t)n_tiles * tile_tab_stride(n_class, nd) * 4);
    L.seg_order = (int32_t*)take((size_t)n_seg * 4);
    L.cell_count = (int64_t*)take(((size_t)p + 1) * 8);
    L.cell_base = (int64_t*)take(((size_t)p + 1) * 8);
    long long big = p > n_seg ? p : n_seg;
    L.scan_tmp = (int64_t*)take(((size_t)(big / kScanBlock) + 2) * 8);
    L.groups = (Group*)take((size_t)(p + 1) * sizeof(Group));
    L.coef = take((size_t)(p + 1) * nb * kTile * esz);
    L.cdiff = take((size_t)n_class * nb * esz);
    L.cspec = take((size_t)n_class * nb * esz);
    L.err = (int*)take(16);
    L.bytes = (size_t)(q - (char*)base);
    return L;
}

void scan64(long long n, const int64_t* in, int64_t* out, int64_t* tmp, cudaStream_t st) {
    // out[0..n] exclusive scan, out[n] = total
    long long nblocks = (n + kScanBlock - 1) / kScanBlock;
    if (nblocks < 1) nblocks = 1;
    k_scan_blocks<<<(unsigned)nblocks, kScanBlock, 0, sp_counted(st)>>>(n, in, out, tmp);
    k_scan_sums<<<1, 32, 0, sp_counted(st)>>>(nblocks, tmp, out + n);
    k_scan_add<<<(unsigned)nblocks, kScanBlock, 0, sp_counted(st)>>>(n, out, tmp);
}

template <typename T>
int run_tiled(const sp_exchange_args* a, void* ws, size_t ws_bytes, cudaStream_t st) {
    const int n = a->n_patches, nd = a->n_dirs, nb = a->n_bins, nt = a->n_samples;
    const long long p = a->n_dir_pairs;
    if (!a->slot_group || !a->slot_scale || !a->class_diff || !a->class_spec || !a->class_target || a->n_groups < 1)
        return SP_ERR_ARG;
    const int n_class = a->n_groups * a->n_in_dirs;
    if (n_class > kMaxClasses) return SP_ERR_UNSUPPORTED;
    Plan L = plan_layout(nullptr, sizeof(T), n, nd, nb, nt, p, n_class);
    if (ws_bytes < L.bytes) return SP_ERR_WORKSPACE;
    L = plan_layout(ws, sizeof(T), n, nd, nb, nt, p, n_class);
    const int n_tiles = (n + kTile - 1) / kTile;
    const long long n_seg = (long long)n_tiles * n_class;
    const size_t e = (size_t)n * nd * nb * nt;
    T* etot = (T*)a->etc_total;
    T* eprev = (T*)L.eprev;
    T* ecur = (T*)L.ecur;
    const long long rs = (long long)L.rs;
    const int lead = L.lead;
    cudaMemsetAsync(L.err, 0, sizeof(int), st);
    cudaMemsetAsync(etot, 0, e * sizeof(T), st);
    // eprev: all zero before the initial energies are placed; ecur: only the
    // leads need zeros (every bin is written each order)
    cudaMemsetAsync(eprev, 0, (L.rows * L.rs + kStageF + 64) * sizeof(T), st);
    cudaMemset2DAsync(ecur, L.rs * sizeof(T), 0, (size_t)lead * sizeof(T), L.rows, st);
    long long ne = (long long)n * nd * nb;
    k_init_energy_t<T><<<sp_blocks(ne, 256), 256, 0, sp_counted(st)>>>(n, nd, nb, nt, rs, lead, a->energy_0_dir, a->distance_0,
                                                           a->speed_of_sound, a->time_resolution, etot, eprev, L.err);
    int herr = 0;
    cudaMemcpyAsync(&herr, L.err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    if (herr) return SP_ERR_RANGE;
    if (a->max_order < 1 || p == 0) return sp_check_launch();

    // ---- plan
    k_delays_t<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, a->pair_distance, a->speed_of_sound, a->time_resolution, L.delay);
    k_pair_class_t<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, a->pair_src, a->pair_in_dir, a->wall_of, a->brdf_index,
                                                      a->slot_group, a->n_in_dirs, L.cls);
    k_row_sort_by_class_t<<<n, 32, n_class * sizeof(int), sp_counted(st)>>>(n, a->dst_offset, L.cls, n_class, L.perm, L.rco,
                                                                L.row_of);
    k_default_tiles<<<sp_blocks((long long)n_tiles * kTile, 256), 256, 0, sp_counted(st)>>>(n, n_tiles, a->receiver_order,
                                                                               L.tile_recv, L.tile_of, L.slot_of);
    k_seg_size<<<sp_blocks(n_seg, 256), 256, 0, sp_counted(st)>>>(n_seg, n_class, L.tile_recv, L.rco, L.seg_size);
    scan64(n_seg, L.seg_size, L.seg_base, L.scan_tmp, st);
    k_merge_positions<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, n_class, L.perm, L.row_of, L.cls, a->pair_src, L.rco,
                                                         L.tile_of, L.slot_of, L.tile_recv, L.seg_base, L.merged);
    k_cells<T><<<sp_blocks(p, 128), 128, 0, sp_counted(st)>>>(p, nd, nb, nt, L.merged, a->pair_src, a->pair_dst, a->pair_out_dir,
                                                  L.delay, L.cls, L.tile_of, L.slot_of, a->pair_fprime,
                                                  a->pair_unit_len, a->air_attenuation, a->wall_of, a->brdf_index,
                                                  a->slot_scale, 0, L.cell_count, nullptr, p, nullptr, nullptr);
    scan64(p, L.cell_count, L.cell_base, L.scan_tmp, st);
    k_cells<T><<<sp_blocks(p, 128), 128, 0, sp_counted(st)>>>(p, nd, nb, nt, L.merged, a->pair_src, a->pair_dst, a->pair_out_dir,
                                                  L.delay, L.cls, L.tile_of, L.slot_of, a->pair_fprime,
                                                  a->pair_unit_len, a->air_attenuation, a->wall_of, a->brdf_index,
                                                  a->slot_scale, 1, nullptr, L.cell_base, p, L.groups, (T*)L.coef);
    k_seg_offsets<<<sp_blocks(n_seg + 1, 256), 256, 0, sp_counted(st)>>>(n_seg, p, L.seg_base, L.cell_base, L.seg_off);
    long long nc = (long long)n_class * nb;
    k_convert_t<T><<<sp_blocks(nc, 256), 256, 0, sp_counted(st)>>>(nc, a->class_diff, (T*)L.cdiff);
    k_convert_t<T><<<sp_blocks(nc, 256), 256, 0, sp_counted(st)>>>(nc, a->class_spec, (T*)L.cspec);
    k_tile_table<<<sp_blocks(n_tiles, 128), 128, 0, sp_counted(st)>>>(n_tiles, n_class, nd, L.seg_off, a->class_target,
                                                                         L.tile_tab);
    // scatter blocks visit the non-empty segments longest first, so the
    // longest blocks do not end up in the tail of the grid
    std::vector<int64_t> h_off((size_t)n_seg + 1);
    cudaMemcpyAsync(h_off.data(), L.seg_off, h_off.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    std::vector<int32_t> order;
    order.reserve((size_t)n_seg);
    for (long long sg = 0; sg < n_seg; ++sg)
        if (h_off[sg + 1] > h_off[sg]) order.push_back((int32_t)sg);
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        return h_off[x + 1] - h_off[x] > h_off[y + 1] - h_off[y];
    });
    const unsigned n_active = (unsigned)order.size();
    if (n_active > 0) {
        cudaMemcpyAsync(L.seg_order, order.data(), order.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    }
    if (a->plan_stats) {
        a->plan_stats[0] = h_off[n_seg];
        a->plan_stats[1] = n_seg;
        a->plan_stats[2] = p;
        a->plan_stats[3] = n_tiles;
    }

    // ---- orders
    dim3 mgrid(nb, n);
    size_t msmem = (size_t)2 * n_class * sizeof(T) + (size_t)tile_tab_stride(n_class, nd) * sizeof(int);
    SpEventTimer timer(a->order_ms != nullptr, st);
    for (int k = 0; k < a->max_order; ++k) {
        if constexpr (sizeof(T) == 4) {
            if (k == 0)
                cudaFuncSetAttribute(k_scatter_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kScatterSmem);
            dim3 sgrid(n_active, (nt + kTW - 1) / kTW, nb);
            if (n_active > 0)
                k_scatter_f32<<<sgrid, kWsThreads, kScatterSmem, sp_counted(st)>>>(
                    n_class, nb, nt, rs, lead, p, L.tile_recv, L.seg_order, L.seg_off, L.groups, (const float*)L.coef,
                    (const float*)eprev, (float*)L.g, L.err);
        } else {
            dim3 sgrid(n_active, (nt + kTW64 - 1) / kTW64, nb);
            if (n_active > 0)
                k_scatter_f64<<<sgrid, kThreads, 0, sp_counted(st)>>>(n_class, nb, nt, rs, lead, p, L.tile_recv,
                                                                      L.seg_order, L.seg_off, L.groups,
                                                                      (const double*)L.coef, (const double*)eprev,
                                                                      (double*)L.g);
        }
        if (sizeof(T) == 4 && nt % 4 == 0)
            k_mix4<<<mgrid, 128, msmem, sp_counted(st)>>>(n_class, nd, nb, nt, rs, lead, L.tile_of, L.tile_tab,
                                                          (const float*)L.cdiff, (const float*)L.cspec,
                                                          (const float*)L.g, (float*)ecur, (float*)etot);
        else
            k_mix<T><<<mgrid, 256, msmem, sp_counted(st)>>>(n_class, nd, nb, nt, rs, lead, L.tile_of, L.tile_tab,
                                                            (const T*)L.cdiff, (const T*)L.cspec, (const T*)L.g, ecur,
                                                            etot);
        T* tmp = eprev;
        eprev = ecur;
        ecur = tmp;
    }
    timer.stop(st);
    int rc = sp_check_launch();
    if (rc != SP_OK) return rc;
    cudaMemcpyAsync(&herr, L.err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    if (a->order_ms) *a->order_ms = timer.elapsed_ms();
    return herr ? SP_ERR_TIMEOUT : SP_OK;
}

}  // namespace

size_t sp_structured_workspace(int precision, int n_patches, int n_dirs, int n_bins, int n_samples,
                               long long n_dir_pairs, int n_class) {
    int esz = precision == SP_F64 ? 8 : 4;
    return plan_layout(nullptr, esz, n_patches, n_dirs, n_bins, n_samples, n_dir_pairs, n_class).bytes;
}

int sp_run_structured(const sp_exchange_args* a, void* ws, size_t ws_bytes, cudaStream_t st) {
    if (!a->pair_dst) return SP_ERR_ARG;
    if (a->precision == SP_F64) return run_tiled<double>(a, ws, ws_bytes, st);
    return run_tiled<float>(a, ws, ws_bytes, st);
}
