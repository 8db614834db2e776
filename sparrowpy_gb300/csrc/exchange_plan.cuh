// Exchange planner: groups the (destination, source row, class) pairs of a
// delayed scatter into source groups for the tiled scatter kernels.
//
// Destinations are cut into tiles of kTile (a given order); a segment is one
// (tile, class); a group is one source histogram row feeding up to kTile
// destinations of a tile, with a base delay and per-destination offsets up
// to kMaxSpan.  Used for the forward exchange (pairs i -> j, class = incoming
// direction class) and for its adjoint (the transposed pairs).
#pragma once
#include <algorithm>
#include <vector>

#include "common.cuh"
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

// What consumer warp w of the FP32 scatter needs of a group, in one word:
// offsets of slots 2w and 2w + 1 (6 bits each), their membership (2 bits),
// the window alignment mu (2 bits) and the base delay (16 bits).
constexpr int kPackWarps = kTile / 2;
__host__ __device__ inline uint32_t warp_pack(int off0, int off1, unsigned bits, int mu, int n_base) {
    return (uint32_t)off0 | ((uint32_t)off1 << 6) | (bits << 12) | ((uint32_t)mu << 14) | ((uint32_t)n_base << 16);
}

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
// Exclusive scan of the block sums in one block of kScanBlock threads: each
// thread takes a contiguous chunk, the chunk totals are scanned in shared
// memory, then each chunk is written from its prefix (integers: exact).
__global__ void k_scan_sums(long long nblocks, int64_t* __restrict__ sums, int64_t* __restrict__ total) {
    __shared__ int64_t s[kScanBlock];
    const int t = threadIdx.x;
    const long long per = (nblocks + kScanBlock - 1) / kScanBlock;
    const long long b0 = (long long)t * per;
    const long long b1 = b0 + per < nblocks ? b0 + per : nblocks;
    int64_t local = 0;
    for (long long k = b0; k < b1; ++k) local += sums[k];
    s[t] = local;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        const int64_t x = (t >= off) ? s[t - off] : 0;
        __syncthreads();
        s[t] += x;
        __syncthreads();
    }
    int64_t run = s[t] - local;
    for (long long k = b0; k < b1; ++k) {
        const int64_t v = sums[k];
        sums[k] = run;
        run += v;
    }
    if (t == kScanBlock - 1) *total = s[kScanBlock - 1];
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

// Per pair and band, the coefficient a source group carries for it (Coef:
// F', air attenuation, material), one pair per thread so that every lane of
// a warp runs the FP64 arithmetic together.
template <typename T, typename Coef>
__global__ void k_pair_coef(long long n_dir, int nb, Coef pair_coef, T* __restrict__ out) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_dir) return;
    for (int b = 0; b < nb; ++b) {
        if constexpr (sizeof(T) == 4)
            out[e * nb + b] = pair_coef.f32(e, b);  // GB300's FP64 pipe is a small fraction of FP32
        else
            out[e * nb + b] = pair_coef(e, b);
    }
}

// 1 where merged position q starts a cell (a new (src, tile, class) run), else 0.
__global__ void k_cell_flags(long long n_dir, const int64_t* __restrict__ merged, const int32_t* __restrict__ src,
                             const int32_t* __restrict__ dst, const int32_t* __restrict__ tile_of,
                             const int32_t* __restrict__ cls, int64_t* __restrict__ flag) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_dir) return;
    int start = 1;
    if (q > 0) {
        const long long e = merged[q], ep = merged[q - 1];
        start = !(src[ep] == src[e] && tile_of[dst[ep]] == tile_of[dst[e]] && cls[ep] == cls[e]);
    }
    flag[q] = start;
}

// starts[c] = merged position of cell c (fscan: exclusive scan of the flags).
__global__ void k_cell_compact(long long n_dir, const int64_t* __restrict__ flag, const int64_t* __restrict__ fscan,
                               int64_t* __restrict__ starts) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n_dir && flag[q]) starts[fscan[q]] = q;
}

// Cells: runs of equal (segment, src) in merged order (<= kTile entries, one
// per destination), one thread per cell (the compacted cell starts, so that
// every lane works).  Per cell: sort members by (p2o, delay), cut into
// groups; write == 0 counts (cell_count[c]), write == 1 emits at
// cell_base[c] with the coefficients of k_pair_coef.
// n_cells is read on the device (the flag scan's total), so the launch covers
// all n_dir slots; slots past it count zero groups.
template <typename T>
__global__ void k_cells(const int64_t* __restrict__ n_cells_p, const int64_t* __restrict__ starts, long long n_dir,
                        int nd, int nb, int nt, const int64_t* __restrict__ merged, const int32_t* __restrict__ src,
                        const int32_t* __restrict__ dst, const int32_t* __restrict__ out_dir,
                        const int32_t* __restrict__ delay, const int32_t* __restrict__ cls,
                        const int32_t* __restrict__ tile_of, const int32_t* __restrict__ slot_of,
                        const T* __restrict__ pair_coef,
                        int write, int64_t* __restrict__ cell_count, const int64_t* __restrict__ cell_base,
                        long long cap, Group* __restrict__ groups, T* __restrict__ coef,
                        uint32_t* __restrict__ wpack) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_dir) return;
    if (c >= *n_cells_p) {
        if (!write) cell_count[c] = 0;
        return;
    }
    const long long q = starts[c];
    long long e = merged[q];
    int s_src = src[e];
    int s_tile = tile_of[dst[e]];
    int s_cls = cls[e];
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
    long long g_out = write ? cell_base[c] : 0;
    long long n_groups = 0;
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
                for (int b = 0; b < nb; ++b) coef[((size_t)b * cap + g_out) * kTile + w] = pair_coef[ex * nb + b];
            }
            groups[g_out] = g;
            const int mu = (-g.n_base - kMaxSpan) & 3;
            for (int w = 0; w < kPackWarps; ++w)
                wpack[(size_t)g_out * kPackWarps + w] =
                    warp_pack(g.off[2 * w], g.off[2 * w + 1], (g.mask >> (2 * w)) & 3u, mu, g.n_base);
            ++g_out;
        }
        ++n_groups;
        a = r + 1;
    }
    if (!write) cell_count[c] = n_groups;
}

// seg_off[s] = group index of the first cell of segment s: its first merged
// position starts a cell (or, for an empty segment, the next one does), and
// fscan turns positions into cell numbers (fscan[n_dir] = number of cells).
__global__ void k_seg_offsets(long long n_seg, const int64_t* __restrict__ seg_base, const int64_t* __restrict__ fscan,
                              const int64_t* __restrict__ cell_base, int64_t* __restrict__ seg_off) {
    long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s > n_seg) return;
    seg_off[s] = cell_base[fscan[seg_base[s]]];
}

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

void scan64(long long n, const int64_t* in, int64_t* out, int64_t* tmp, cudaStream_t st) {
    // out[0..n] exclusive scan, out[n] = total
    long long nblocks = (n + kScanBlock - 1) / kScanBlock;
    if (nblocks < 1) nblocks = 1;
    k_scan_blocks<<<(unsigned)nblocks, kScanBlock, 0, sp_counted(st)>>>(n, in, out, tmp);
    k_scan_sums<<<1, kScanBlock, 0, sp_counted(st)>>>(nblocks, tmp, out + n);
    k_scan_add<<<(unsigned)nblocks, kScanBlock, 0, sp_counted(st)>>>(n, out, tmp);
}

// Forward coefficient of pair e (i -> j) in band b:
// F'_ij exp(-att_b |u_ij|) scale[slot of i, b] (the class part is applied by the mix).
struct FwdCoef {
    const double* fprime;
    const double* unit_len;
    const double* att;
    const int32_t* wall_of;
    const int32_t* brdf_index;
    const double* slot_scale;
    const int32_t* src;
    int nb;
    __device__ double operator()(long long e, int b) const {
        double f = fprime[e];
        if (att) f = f * exp(-att[b] * unit_len[e]);
        return f * slot_scale[(size_t)brdf_index[wall_of[src[e]]] * nb + b];
    }
    // the same in FP32 (inputs truncated to 2^-23) for the FP32 plan
    __device__ float f32(long long e, int b) const {
        float f = f64_trunc_f32(fprime[e]);
        if (att) f = f * expf(-f64_trunc_f32(att[b]) * f64_trunc_f32(unit_len[e]));
        return f * f64_trunc_f32(slot_scale[(size_t)brdf_index[wall_of[src[e]]] * nb + b]);
    }
};

// The pairs a plan groups: destination-major CSR; the source row of pair e is
// src[e] * rows_per_src + row[e].
struct PairSet {
    long long p;
    const int64_t* dst_off;  // (n + 1)
    const int32_t* src;
    const int32_t* dst;
    const int32_t* row;
    const int32_t* cls;
    const int32_t* delay;
    int rows_per_src;
    int n_class;
};

// Device arrays of a plan (sized for p pairs, n destinations, n_class classes).
struct PlanCore {
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
    int32_t* seg_order;
    int64_t* cell_count;
    int64_t* cell_base;
    int64_t* cell_flag;   // [pairs + 1] start flags, then their exclusive scan in cell_fscan
    int64_t* cell_fscan;  // [pairs + 1]
    int64_t* cell_start;  // [pairs] merged position of each cell
    int64_t* scan_tmp;
    Group* groups;
    uint32_t* wpack;  // [cap][kPackWarps]
    void* coef;       // [nb][cap][kTile]
    void* pcoef;      // [pairs][nb] per-pair coefficients (k_pair_coef)
};

// Carve PlanCore arrays from q (advanced); esz = coefficient element size.
template <typename Take>
PlanCore plan_core_layout(Take& take, int esz, int n, int nb, long long p, int n_class) {
    PlanCore C;
    const int n_tiles = (n + kTile - 1) / kTile;
    const long long n_seg = (long long)n_tiles * n_class;
    C.perm = (int64_t*)take((size_t)p * 8);
    C.row_of = (int32_t*)take((size_t)p * 4);
    C.merged = (int64_t*)take((size_t)p * 8);
    C.rco = (int64_t*)take((size_t)n * (n_class + 1) * 8);
    C.tile_recv = (int32_t*)take((size_t)n_tiles * kTile * 4);
    C.tile_of = (int32_t*)take((size_t)n * 4);
    C.slot_of = (int32_t*)take((size_t)n * 4);
    C.seg_size = (int64_t*)take(((size_t)n_seg + 1) * 8);
    C.seg_base = (int64_t*)take(((size_t)n_seg + 1) * 8);
    C.seg_off = (int64_t*)take(((size_t)n_seg + 1) * 8);
    C.seg_order = (int32_t*)take((size_t)n_seg * 4);
    C.cell_count = (int64_t*)take(((size_t)p + 1) * 8);
    C.cell_base = (int64_t*)take(((size_t)p + 1) * 8);
    C.cell_flag = (int64_t*)take(((size_t)p + 1) * 8);
    C.cell_fscan = (int64_t*)take(((size_t)p + 1) * 8);
    C.cell_start = (int64_t*)take(((size_t)p + 1) * 8);
    long long big = p > n_seg ? p : n_seg;
    C.scan_tmp = (int64_t*)take(((size_t)(big / kScanBlock) + 2) * 8);
    C.groups = (Group*)take((size_t)(p + 1) * sizeof(Group));
    C.wpack = (uint32_t*)take((size_t)(p + 1) * kPackWarps * 4);
    C.coef = take((size_t)(p + 1) * nb * kTile * esz);
    C.pcoef = take((size_t)(p + 1) * nb * esz);
    return C;
}

// Group the pairs into segments and source groups, fill the coefficients and
// order the non-empty segments longest first (host sort).  n = destinations,
// order = destination order cut into tiles (nullptr: identity).  Returns the
// number of non-empty segments in *n_active and of groups in *n_groups.
template <typename T, typename Coef>
int build_groups(int n, int nb, int nt, const PairSet& ps, const int32_t* order, Coef coef, PlanCore& C,
                 unsigned* n_active, long long* n_groups, cudaStream_t st) {
    const long long p = ps.p;
    const int n_class = ps.n_class;
    const int n_tiles = (n + kTile - 1) / kTile;
    const long long n_seg = (long long)n_tiles * n_class;
    k_row_sort_by_class_t<<<n, 32, n_class * sizeof(int), sp_counted(st)>>>(n, ps.dst_off, ps.cls, n_class, C.perm,
                                                                             C.rco, C.row_of);
    k_default_tiles<<<sp_blocks((long long)n_tiles * kTile, 256), 256, 0, sp_counted(st)>>>(n, n_tiles, order,
                                                                                           C.tile_recv, C.tile_of,
                                                                                           C.slot_of);
    k_seg_size<<<sp_blocks(n_seg, 256), 256, 0, sp_counted(st)>>>(n_seg, n_class, C.tile_recv, C.rco, C.seg_size);
    scan64(n_seg, C.seg_size, C.seg_base, C.scan_tmp, st);
    k_merge_positions<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, n_class, C.perm, C.row_of, ps.cls, ps.src,
                                                                     C.rco, C.tile_of, C.slot_of, C.tile_recv,
                                                                     C.seg_base, C.merged);
    k_pair_coef<T, Coef><<<sp_blocks(p, 128), 128, 0, sp_counted(st)>>>(p, nb, coef, (T*)C.pcoef);
    // cell starts, compacted so that one thread per cell builds its groups
    k_cell_flags<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, C.merged, ps.src, ps.dst, C.tile_of, ps.cls,
                                                                C.cell_flag);
    scan64(p, C.cell_flag, C.cell_fscan, C.scan_tmp, st);
    k_cell_compact<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, C.cell_flag, C.cell_fscan, C.cell_start);
    const int64_t* n_cells = C.cell_fscan + p;
    k_cells<T><<<sp_blocks(p, 128), 128, 0, sp_counted(st)>>>(
        n_cells, C.cell_start, p, ps.rows_per_src, nb, nt, C.merged, ps.src, ps.dst, ps.row, ps.delay, ps.cls,
        C.tile_of, C.slot_of, (const T*)C.pcoef, 0, C.cell_count, nullptr, p, nullptr, nullptr, nullptr);
    scan64(p, C.cell_count, C.cell_base, C.scan_tmp, st);
    k_cells<T><<<sp_blocks(p, 128), 128, 0, sp_counted(st)>>>(
        n_cells, C.cell_start, p, ps.rows_per_src, nb, nt, C.merged, ps.src, ps.dst, ps.row, ps.delay, ps.cls,
        C.tile_of, C.slot_of, (const T*)C.pcoef, 1, nullptr, C.cell_base, p, C.groups, (T*)C.coef, C.wpack);
    k_seg_offsets<<<sp_blocks(n_seg + 1, 256), 256, 0, sp_counted(st)>>>(n_seg, C.seg_base, C.cell_fscan,
                                                                         C.cell_base, C.seg_off);
    // scatter blocks visit the non-empty segments longest first, so the
    // longest blocks do not end up in the tail of the grid
    std::vector<int64_t> h_off((size_t)n_seg + 1);
    cudaMemcpyAsync(h_off.data(), C.seg_off, h_off.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    std::vector<int32_t> seg_order;
    seg_order.reserve((size_t)n_seg);
    for (long long sg = 0; sg < n_seg; ++sg)
        if (h_off[sg + 1] > h_off[sg]) seg_order.push_back((int32_t)sg);
    std::stable_sort(seg_order.begin(), seg_order.end(), [&](int32_t x, int32_t y) {
        return h_off[x + 1] - h_off[x] > h_off[y + 1] - h_off[y];
    });
    *n_active = (unsigned)seg_order.size();
    *n_groups = h_off[n_seg];
    if (!seg_order.empty()) {
        cudaMemcpyAsync(C.seg_order, seg_order.data(), seg_order.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                        st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    }
    return sp_check_launch();
}

}  // namespace
