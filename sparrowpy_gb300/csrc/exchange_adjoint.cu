// Adjoint (reverse mode) of the structured energy exchange, FP32 or FP64.
//
// Forward, order k (RadiosityFast.py:1121-1143, pair e: i -> j, sender slot
// s(i), incoming direction c(e), outgoing index p(e) of i toward j):
//   E_k[j, o, b, t] = sum_e w_e,b BRDF_s(i)[c(e), o, b] E_{k-1}[i, p(e), b, t - n_e]
// with w = F' exp(-att_b |u|) and, for the tables of create_from_scattering
// (sparrowpy/brdf.py:8-130) stored x pi,
//   BRDF_s[c, o, b] = (1 - a_s,b) (s_s,b + (1 - s_s,b) K_c [o == m_c]).
// E_total = sum_k E_k and the receiver histograms are linear in E_total.
//
// Reverse sweep with mu_k = dL/dE_k: mu_K = g = dL/dE_total, and
//   mu_{k-1} = g + (1 - a)(s lamU + (1 - s) lamV),
//   lamU[i, p, b, t] = sum_{e: i->j, p(e) = p} w_e U_k[j, b, t + n_e],  U_k = sum_o mu_k[j, o],
//   lamV[i, p, b, t] = sum_{e: i->j, p(e) = p} w_e K_c(e) mu_k[j, m_c(e), b, t + n_e],
//   dL/da_s,b += -sum_{i in s} sum_{p,t} E_{k-1}[i, p, b, t] (s lamU + (1 - s) lamV),
//   dL/ds_s,b +=  sum_{i in s} (1 - a) sum_{p,t} E_{k-1}[i, p, b, t] (lamU - lamV).
// In reversed time (tau = T - 1 - t) the advances t + n_e become delays, so
// lamU and lamV are one delayed scatter of the forward kind over the
// transposed pairs: destination i, class p (lamU) or D + p (lamV), source row
// U_j (row D of patch j) or mu[j, m_c] - the same planner and scatter kernel
// as the forward exchange.  The combine kernel forms mu_{k-1} (with its U
// row) and the two gradient dot products in one pass.
#include "exchange_scatter.cuh"

namespace {

// rev[e] = index of the pair (dst_e -> src_e) in the destination-major list
// (sources ascend within each destination row).
__global__ void k_reverse_index(long long p, const int64_t* __restrict__ off, const int32_t* __restrict__ src,
                                const int32_t* __restrict__ dst, int32_t* __restrict__ rev) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p) return;
    const int i = src[e], j = dst[e];
    const long long end = off[i + 1];
    long long lo = off[i], hi = end;  // pairs into i, ascending source
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (src[mid] < j) lo = mid + 1;
        else hi = mid;
    }
    rev[e] = (lo < end && src[lo] == j) ? (int32_t)lo : -1;  // -1: no reverse pair (not a symmetric list)
}

// Every transposed row i first holds placeholders (destination i, delay nt:
// dropped by the planner), so rows stay well formed for any pair list.
__global__ void k_transposed_defaults(int n, int nt, const int64_t* __restrict__ off, int32_t* __restrict__ t_src,
                                      int32_t* __restrict__ t_dst, int32_t* __restrict__ t_row,
                                      int32_t* __restrict__ t_cls, int32_t* __restrict__ t_delay,
                                      int32_t* __restrict__ t_fwd) {
    const int i = blockIdx.x;
    for (long long t = 2 * off[i] + threadIdx.x; t < 2 * off[i + 1]; t += blockDim.x) {
        t_src[t] = 0;
        t_dst[t] = i;
        t_row[t] = 0;
        t_cls[t] = 0;
        t_delay[t] = nt;
        t_fwd[t] = 0;
    }
}

// Transposed pairs, destination-major over i: row i holds 2 deg(i) entries,
// first the diffuse (U) kind, then the mirror (V) kind, each with ascending
// source j (the position of e in i's row is rev[e] - off[i]).
__global__ void k_transpose_pairs(long long p, int nd, int nt, const int64_t* __restrict__ off,
                                  const int32_t* __restrict__ rev, const int32_t* __restrict__ src,
                                  const int32_t* __restrict__ dst, const int32_t* __restrict__ out_dir,
                                  const int32_t* __restrict__ in_dir, const int32_t* __restrict__ delay,
                                  const int32_t* __restrict__ mirror_of_in, int32_t* __restrict__ t_src,
                                  int32_t* __restrict__ t_dst, int32_t* __restrict__ t_row, int32_t* __restrict__ t_cls,
                                  int32_t* __restrict__ t_delay, int32_t* __restrict__ t_fwd) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p) return;
    if (rev[e] < 0) return;  // stays a placeholder
    const int i = src[e];
    const long long deg = off[i + 1] - off[i];
    const long long t0 = 2 * off[i] + (rev[e] - off[i]);
    const long long t1 = t0 + deg;
    const int m = mirror_of_in[in_dir[e]];
    t_src[t0] = dst[e];
    t_src[t1] = dst[e];
    t_dst[t0] = i;
    t_dst[t1] = i;
    t_row[t0] = nd;  // U row
    t_row[t1] = m >= 0 ? m : 0;
    t_cls[t0] = out_dir[e];
    t_cls[t1] = nd + out_dir[e];
    t_delay[t0] = delay[e];
    t_delay[t1] = m >= 0 ? delay[e] : nt;  // no mirror term: dropped by the planner
    t_fwd[t0] = (int32_t)e;
    t_fwd[t1] = (int32_t)e;
}

__global__ void k_double_offsets(int n, const int64_t* __restrict__ off, int64_t* __restrict__ t_off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= n) t_off[i] = 2 * off[i];
}

// Coefficient of transposed pair t in band b: w_e,b (U kind) or w_e,b K_c(e)
// (V kind), in FP64 (the FP64 adjoint) or from inputs truncated to FP32.
struct AdjCoef {
    const int32_t* fwd;
    const int32_t* cls;
    const int32_t* in_dir;
    const double* gain;
    const double* fprime;
    const double* unit_len;
    const double* att;
    int nd;
    __device__ double operator()(long long t, int b) const {
        const long long e = fwd[t];
        double f = fprime[e];
        if (att) f = f * exp(-att[b] * unit_len[e]);
        return cls[t] >= nd ? f * gain[in_dir[e]] : f;
    }
    __device__ float f32(long long t, int b) const {
        const long long e = fwd[t];
        float f = f64_trunc_f32(fprime[e]);
        if (att) f = f * expf(-f64_trunc_f32(att[b]) * f64_trunc_f32(unit_len[e]));
        return cls[t] >= nd ? f * f64_trunc_f32(gain[in_dir[e]]) : f;
    }
};

// g = dL/dE_total is nonzero only in the row (k, ridx_rk) of each receiver r:
// mono[r, b, t] = sum_k E[k, ridx_rk, b, (t - s_rk) mod T] f_rk a_rkb (k_collect_mono),
// so that row of g, reversed, is g_r[k, b, tau] = f_rk a_rkb gm[r, b, (T - 1 - tau + s_rk) mod T].
// One block per (band, patch); g_rev is (R, N, B, T).
template <typename T>
__global__ void k_adjoint_g(int n, int nb, int nt, int n_rcv, const double* __restrict__ rfac,
                            const double* __restrict__ rdist, double c, double dt, const double* __restrict__ att,
                            const double* __restrict__ gm, T* __restrict__ g_rev) {
    const int b = blockIdx.x, k = blockIdx.y;
    for (int r = 0; r < n_rcv; ++r) {
        const size_t rk = (size_t)r * n + k;
        const double q = ceil(xdiv(xdiv(rdist[rk], c), dt));
        long long s = (long long)q;
        s %= nt;
        if (s < 0) s += nt;
        const double f = rfac[rk] * (att ? exp(-att[b] * rdist[rk]) : 1.0);
        T* out = g_rev + (rk * nb + b) * nt;
        const double* src = gm + ((size_t)r * nb + b) * nt;
        for (int tau = threadIdx.x; tau < nt; tau += blockDim.x) {
            long long t = nt - 1 - tau + s;
            if (t >= nt) t -= nt;
            out[tau] = (T)(f * src[t]);
        }
    }
}

// mu_{k-1} = g + (1 - a)(s lamU + (1 - s) lamV) into the padded source buffer
// (rows 0..D-1 of each patch, reversed time) with U = sum over rows in row D;
// gradient dot products with E_{k-1} (normal time).  lam == nullptr: mu = g
// (the first step, no gradient).  One block per (band, patch).
constexpr int kMaxReceivers = 64;  // receivers one adjoint pass can take (dL/dmono rows)
constexpr int kCombineBins = 16;   // bins per thread in k_adjoint_combine: nt <= 256 * 16

// Rows of dL/dE_total beyond the first two that fall on direction p of patch i
// (three or more receivers seen along one direction): added to `out` (a mu
// row, or the U row) at the bins this thread owns.
template <typename T>
__device__ __noinline__ void add_extra_rows(int p, int n_rcv, const int* s_ridx, const T* __restrict__ g_rev,
                                            int n, int i, int nb, int b, int nt, T* out) {
    for (int r = 0, h = 0; r < n_rcv; ++r) {
        if (s_ridx[r] != p || h++ < 2) continue;
        const T* row = g_rev + (((size_t)r * n + i) * nb + b) * nt;
        for (int tau = threadIdx.x; tau < nt; tau += 256) out[tau] += row[tau];
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_adjoint_combine(
    int n, int nd, int nb, int nt, long long rs, int lead, int n_rcv, const int32_t* __restrict__ ridx,
    const T* __restrict__ g_rev, const T* __restrict__ lam, const uint32_t* __restrict__ present, int words,
    const int32_t* __restrict__ tile_of, const T* __restrict__ e_prev, const int32_t* __restrict__ wall_of,
    const int32_t* __restrict__ brdf_index, const double* __restrict__ alpha, const double* __restrict__ scat,
    T* __restrict__ mu_out, double* __restrict__ grad_a, double* __restrict__ grad_s) {
    const int b = blockIdx.x, i = blockIdx.y;
    __shared__ int s_ridx[kMaxReceivers];
    for (int r = threadIdx.x; r < n_rcv; r += blockDim.x) s_ridx[r] = ridx[(size_t)r * n + i];
    __syncthreads();
    const int slot = brdf_index[wall_of[i]];
    const T a = (T)alpha[(size_t)slot * nb + b];
    const T sc = (T)scat[(size_t)slot * nb + b];
    const T keep = T(1) - a;
    const uint32_t* pres = lam ? present + (size_t)tile_of[i] * words : nullptr;
    constexpr int kMaxPerThread = kCombineBins;
    T usum[kMaxPerThread];
#pragma unroll
    for (int q = 0; q < kMaxPerThread; ++q) usum[q] = T(0);
    T dot_mix = T(0), dot_diff = T(0);
    for (int p = 0; p < nd; ++p) {
        // rows of dL/dE_total in direction p of this patch (one per receiver seeing it along p)
        const T* g0 = nullptr;
        const T* g1 = nullptr;
        int n_hit = 0;
        for (int r = 0; r < n_rcv; ++r)
            if (s_ridx[r] == p) {
                const T* row = g_rev + (((size_t)r * n + i) * nb + b) * nt;
                if (n_hit == 0) g0 = row;
                else if (n_hit == 1) g1 = row;
                ++n_hit;
            }
        const bool has_u = pres && ((pres[p >> 5] >> (p & 31)) & 1u);
        const bool has_v = pres && ((pres[(nd + p) >> 5] >> ((nd + p) & 31)) & 1u);
        const T* lu = has_u ? lam + (((size_t)i * 2 * nd + p) * nb + b) * nt : nullptr;
        const T* lv = has_v ? lam + (((size_t)i * 2 * nd + nd + p) * nb + b) * nt : nullptr;
        const T* ep = e_prev ? e_prev + (((size_t)i * nd + p) * nb + b) * nt : nullptr;
        T* mo = mu_out + (((size_t)i * (nd + 1) + p) * nb + b) * rs + lead;
#pragma unroll
        for (int q = 0; q < kMaxPerThread; ++q) {
            const int tau = threadIdx.x + 256 * q;
            if (tau < nt) {
                const T u = lu ? lu[tau] : T(0);
                const T v = lv ? lv[tau] : T(0);
                const T mixed = sc * u + (T(1) - sc) * v;
                T m = keep * mixed;
                if (g0) m += g0[tau];
                if (g1) m += g1[tau];
                mo[tau] = m;
                usum[q] += m;
                if (ep) {
                    const T e = ep[nt - 1 - tau];
                    dot_mix = fma(e, mixed, dot_mix);
                    dot_diff = fma(e, u - v, dot_diff);
                }
            }
        }
        if (n_hit > 2) add_extra_rows(p, n_rcv, s_ridx, g_rev, n, i, nb, b, nt, mo);
    }
    T* mu_u = mu_out + (((size_t)i * (nd + 1) + nd) * nb + b) * rs + lead;
#pragma unroll
    for (int q = 0; q < kMaxPerThread; ++q) {
        const int tau = threadIdx.x + 256 * q;
        if (tau < nt) mu_u[tau] = usum[q];
    }
    for (int p = 0; p < nd; ++p) {  // the extra rows' share of U (rare)
        int hits = 0;
        for (int r = 0; r < n_rcv; ++r) hits += s_ridx[r] == p;
        if (hits > 2) add_extra_rows(p, n_rcv, s_ridx, g_rev, n, i, nb, b, nt, mu_u);
    }
    if (!e_prev) return;
    // block reduction of the two dot products
    __shared__ T s_red[2][8];
    for (int off = 16; off > 0; off >>= 1) {
        dot_mix += __shfl_xor_sync(0xffffffffu, dot_mix, off);
        dot_diff += __shfl_xor_sync(0xffffffffu, dot_diff, off);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_red[0][w] = dot_mix;
        s_red[1][w] = dot_diff;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double dm = 0.0, dd = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            dm += s_red[0][k];
            dd += s_red[1][k];
        }
        atomicAdd(&grad_a[(size_t)slot * nb + b], -dm);
        atomicAdd(&grad_s[(size_t)slot * nb + b], (double)keep * dd);
    }
}

// k_adjoint_combine for nt % 4 == 0: four bins per thread (16-byte accesses;
// the reversed-time E_{k-1} row is read as float4 and taken back to front).
__device__ __forceinline__ float4 c4_add(float4 x, float4 y) {
    return make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
}
__device__ __noinline__ void add_extra_rows4(int p, int n_rcv, const int* s_ridx, const float* __restrict__ g_rev,
                                             int n, int i, int nb, int b, int nt, float4* out) {
    const int nt4 = nt >> 2;
    for (int r = 0, h = 0; r < n_rcv; ++r) {
        if (s_ridx[r] != p || h++ < 2) continue;
        const float4* row = reinterpret_cast<const float4*>(g_rev + (((size_t)r * n + i) * nb + b) * nt);
        for (int t = threadIdx.x; t < nt4; t += 256) out[t] = c4_add(out[t], row[t]);
    }
}

constexpr int kCombine4 = kCombineBins / 4;  // float4 per thread

__global__ void __launch_bounds__(256) k_adjoint_combine4(
    int n, int nd, int nb, int nt, long long rs, int lead, int n_rcv, const int32_t* __restrict__ ridx,
    const float* __restrict__ g_rev, const float* __restrict__ lam, const uint32_t* __restrict__ present, int words,
    const int32_t* __restrict__ tile_of, const float* __restrict__ e_prev, const int32_t* __restrict__ wall_of,
    const int32_t* __restrict__ brdf_index, const double* __restrict__ alpha, const double* __restrict__ scat,
    float* __restrict__ mu_out, double* __restrict__ grad_a, double* __restrict__ grad_s) {
    const int b = blockIdx.x, i = blockIdx.y;
    __shared__ int s_ridx[kMaxReceivers];
    for (int r = threadIdx.x; r < n_rcv; r += blockDim.x) s_ridx[r] = ridx[(size_t)r * n + i];
    __syncthreads();
    const int slot = brdf_index[wall_of[i]];
    const float a = (float)alpha[(size_t)slot * nb + b];
    const float sc = (float)scat[(size_t)slot * nb + b];
    const float keep = 1.0f - a;
    const uint32_t* pres = lam ? present + (size_t)tile_of[i] * words : nullptr;
    const int nt4 = nt >> 2;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 usum[kCombine4];
#pragma unroll
    for (int q = 0; q < kCombine4; ++q) usum[q] = zero;
    float dot_mix = 0.0f, dot_diff = 0.0f;
    for (int p = 0; p < nd; ++p) {
        const float4* g0 = nullptr;
        const float4* g1 = nullptr;
        int n_hit = 0;
        for (int r = 0; r < n_rcv; ++r)
            if (s_ridx[r] == p) {
                const float4* row = reinterpret_cast<const float4*>(g_rev + (((size_t)r * n + i) * nb + b) * nt);
                if (n_hit == 0) g0 = row;
                else if (n_hit == 1) g1 = row;
                ++n_hit;
            }
        const bool has_u = pres && ((pres[p >> 5] >> (p & 31)) & 1u);
        const bool has_v = pres && ((pres[(nd + p) >> 5] >> ((nd + p) & 31)) & 1u);
        const float4* lu = has_u ? reinterpret_cast<const float4*>(lam + (((size_t)i * 2 * nd + p) * nb + b) * nt)
                                 : nullptr;
        const float4* lv = has_v ? reinterpret_cast<const float4*>(lam + (((size_t)i * 2 * nd + nd + p) * nb + b) * nt)
                                 : nullptr;
        const float4* ep = e_prev ? reinterpret_cast<const float4*>(e_prev + (((size_t)i * nd + p) * nb + b) * nt)
                                  : nullptr;
        float4* mo = reinterpret_cast<float4*>(mu_out + (((size_t)i * (nd + 1) + p) * nb + b) * rs + lead);
#pragma unroll
        for (int q = 0; q < kCombine4; ++q) {
            const int t = threadIdx.x + 256 * q;
            if (t < nt4) {
                const float4 u = lu ? __ldg(lu + t) : zero;
                const float4 v = lv ? __ldg(lv + t) : zero;
                const float4 mixed = make_float4(sc * u.x + (1.0f - sc) * v.x, sc * u.y + (1.0f - sc) * v.y,
                                                 sc * u.z + (1.0f - sc) * v.z, sc * u.w + (1.0f - sc) * v.w);
                float4 m = make_float4(keep * mixed.x, keep * mixed.y, keep * mixed.z, keep * mixed.w);
                if (g0) m = c4_add(m, __ldg(g0 + t));
                if (g1) m = c4_add(m, __ldg(g1 + t));
                mo[t] = m;
                usum[q] = c4_add(usum[q], m);
                if (ep) {
                    const float4 e = __ldg(ep + (nt4 - 1 - t));  // bins 4t .. 4t + 3 read E at nt - 1 - 4t .. nt - 4 - 4t
                    dot_mix = fmaf(e.w, mixed.x, dot_mix);
                    dot_mix = fmaf(e.z, mixed.y, dot_mix);
                    dot_mix = fmaf(e.y, mixed.z, dot_mix);
                    dot_mix = fmaf(e.x, mixed.w, dot_mix);
                    dot_diff = fmaf(e.w, u.x - v.x, dot_diff);
                    dot_diff = fmaf(e.z, u.y - v.y, dot_diff);
                    dot_diff = fmaf(e.y, u.z - v.z, dot_diff);
                    dot_diff = fmaf(e.x, u.w - v.w, dot_diff);
                }
            }
        }
        if (n_hit > 2) add_extra_rows4(p, n_rcv, s_ridx, g_rev, n, i, nb, b, nt, mo);
    }
    float4* mu_u = reinterpret_cast<float4*>(mu_out + (((size_t)i * (nd + 1) + nd) * nb + b) * rs + lead);
#pragma unroll
    for (int q = 0; q < kCombine4; ++q) {
        const int t = threadIdx.x + 256 * q;
        if (t < nt4) mu_u[t] = usum[q];
    }
    for (int p = 0; p < nd; ++p) {  // the extra rows' share of U (rare)
        int hits = 0;
        for (int r = 0; r < n_rcv; ++r) hits += s_ridx[r] == p;
        if (hits > 2) add_extra_rows4(p, n_rcv, s_ridx, g_rev, n, i, nb, b, nt, mu_u);
    }
    if (!e_prev) return;
    __shared__ float s_red[2][8];
    for (int off = 16; off > 0; off >>= 1) {
        dot_mix += __shfl_xor_sync(0xffffffffu, dot_mix, off);
        dot_diff += __shfl_xor_sync(0xffffffffu, dot_diff, off);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_red[0][w] = dot_mix;
        s_red[1][w] = dot_diff;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double dm = 0.0, dd = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            dm += s_red[0][k];
            dd += s_red[1][k];
        }
        atomicAdd(&grad_a[(size_t)slot * nb + b], -dm);
        atomicAdd(&grad_s[(size_t)slot * nb + b], (double)keep * dd);
    }
}

// Present classes of each tile as bit masks (absent segments have no output rows).
__global__ void k_present_bits(int n_tiles, int n_class, int words, const int64_t* __restrict__ seg_off,
                               uint32_t* __restrict__ bits) {
    const int tile = blockIdx.x * blockDim.x + threadIdx.x;
    if (tile >= n_tiles) return;
    for (int w = 0; w < words; ++w) {
        uint32_t v = 0;
        for (int c = 32 * w; c < min(n_class, 32 * w + 32); ++c) {
            const long long sg = (long long)tile * n_class + c;
            if (seg_off[sg + 1] > seg_off[sg]) v |= 1u << (c - 32 * w);
        }
        bits[(size_t)tile * words + w] = v;
    }
}

// dL/dE0dir[i, o, b] = mu_0[i, o, b, n0_i] (E_0 sits at bin n0 = int(d0 / c / dt)).
template <typename T>
__global__ void k_adjoint_e0(int n, int nd, int nb, int nt, long long rs, int lead, const T* __restrict__ mu,
                             const double* __restrict__ d0, double c, double dt, double* __restrict__ out) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)n * nd * nb) return;
    const int i = (int)(e / ((long long)nd * nb));
    const int o = (int)((e / nb) % nd);
    const int b = (int)(e % nb);
    const long long dly = (long long)xdiv(xdiv(d0[i], c), dt);
    const long long tau = nt - 1 - dly;
    out[e] = (tau >= 0 && tau < nt) ? (double)mu[(((size_t)i * (nd + 1) + o) * nb + b) * rs + lead + tau] : 0.0;
}

// ------------------------------------------------------------ layout
struct AdjLayout {
    size_t bytes;
    int lead;
    size_t rs;
    size_t rows;  // N * (D + 1) * B
    void* mu[2];
    void* lam;    // (N, 2D, B, T)
    void* g_rev;  // (R, N, B, T): the receivers' rows of dL/dE_total, reversed
    int32_t* rev;
    int32_t* delay;
    int64_t* t_off;
    int32_t *t_src, *t_dst, *t_row, *t_cls, *t_delay, *t_fwd;
    uint32_t* present;
    PlanCore C;
    int* err;
};

// esz: element size of the histograms and of the arithmetic (4: FP32, 8: FP64)
AdjLayout adj_layout(void* base, int esz, int n, int nd, int nb, int nt, long long p, int n_rcv) {
    AdjLayout L;
    char* q = (char*)base;
    auto take = [&](size_t bytes) {
        char* r = q;
        q += sp_align(bytes);
        return (void*)r;
    };
    const int n_class = 2 * nd;
    const int n_tiles = (n + kTile - 1) / kTile;
    L.lead = (int)((((size_t)nt + kMaxSpan + 4) + 3) & ~(size_t)3);
    L.rs = (((size_t)nt + L.lead) + 3) & ~(size_t)3;
    L.rows = (size_t)n * (nd + 1) * nb;
    const size_t tail = (size_t)kStageF + 64;
    for (int k = 0; k < 2; ++k) L.mu[k] = take((L.rows * L.rs + tail) * esz);
    L.lam = take((size_t)n * n_class * nb * nt * esz);
    L.g_rev = take((size_t)(n_rcv > 0 ? n_rcv : 1) * n * nb * nt * esz);
    L.rev = (int32_t*)take((size_t)p * 4);
    L.delay = (int32_t*)take((size_t)p * 4);
    L.t_off = (int64_t*)take(((size_t)n + 1) * 8);
    const long long tp = 2 * p;
    L.t_src = (int32_t*)take((size_t)tp * 4);
    L.t_dst = (int32_t*)take((size_t)tp * 4);
    L.t_row = (int32_t*)take((size_t)tp * 4);
    L.t_cls = (int32_t*)take((size_t)tp * 4);
    L.t_delay = (int32_t*)take((size_t)tp * 4);
    L.t_fwd = (int32_t*)take((size_t)tp * 4);
    L.present = (uint32_t*)take((size_t)n_tiles * ((n_class + 31) / 32) * 4);
    L.C = plan_core_layout(take, esz, n, nb, tp, n_class);
    L.err = (int*)take(16);
    L.bytes = (size_t)(q - (char*)base);
    return L;
}

inline int adj_esz(int precision) { return precision == SP_F64 ? 8 : 4; }

bool adj_args_ok(const sp_adjoint_args* a) {
    if (!a || !a->fwd) return false;
    const sp_exchange_args* f = a->fwd;
    return (f->precision == SP_F32 || f->precision == SP_F64) && f->n_patches > 0 && f->n_dirs > 0 &&
           f->n_bins > 0 && f->n_samples > 0 &&
           f->n_samples <= 256 * 16 && f->n_dir_pairs >= 0 && 2 * f->n_dir_pairs < (1LL << 31) && f->dst_offset &&
           f->pair_src && f->pair_dst && f->pair_out_dir && f->pair_in_dir && f->pair_distance && f->pair_fprime &&
           f->pair_unit_len && f->wall_of && f->brdf_index && a->mirror_of_in && a->mirror_gain && a->alpha &&
           a->scattering && a->grad_alpha && a->grad_scattering && a->state && a->n_receivers >= 0 &&
           a->n_receivers <= kMaxReceivers && (a->n_receivers == 0 || a->recv_dir);
}

template <typename T>
int adjoint_begin(const sp_adjoint_args* a, void* ws, size_t ws_bytes, cudaStream_t st) {
    const sp_exchange_args* f = a->fwd;
    const int n = f->n_patches, nd = f->n_dirs, nb = f->n_bins, nt = f->n_samples;
    const long long p = f->n_dir_pairs;
    AdjLayout L = adj_layout(nullptr, sizeof(T), n, nd, nb, nt, p, a->n_receivers);
    if (ws_bytes < L.bytes) return SP_ERR_WORKSPACE;
    L = adj_layout(ws, sizeof(T), n, nd, nb, nt, p, a->n_receivers);
    sp_adjoint_state* S = a->state;
    S->ready = 0;
    S->cur = 0;
    S->n_active = 0;
    S->n_groups = 0;
    cudaMemsetAsync(L.err, 0, sizeof(int), st);
    // transposed plan
    if (p > 0) {
        k_reverse_index<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, f->dst_offset, f->pair_src, f->pair_dst,
                                                                       L.rev);
        k_delays_t<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, f->pair_distance, f->speed_of_sound,
                                                                  f->time_resolution, L.delay);
        k_transposed_defaults<<<n, 256, 0, sp_counted(st)>>>(n, nt, f->dst_offset, L.t_src, L.t_dst, L.t_row,
                                                             L.t_cls, L.t_delay, L.t_fwd);
        k_transpose_pairs<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(
            p, nd, nt, f->dst_offset, L.rev, f->pair_src, f->pair_dst, f->pair_out_dir, f->pair_in_dir, L.delay,
            a->mirror_of_in, L.t_src, L.t_dst, L.t_row, L.t_cls, L.t_delay, L.t_fwd);
        k_double_offsets<<<sp_blocks(n + 1, 256), 256, 0, sp_counted(st)>>>(n, f->dst_offset, L.t_off);
        PairSet ps{2 * p, L.t_off, L.t_src, L.t_dst, L.t_row, L.t_cls, L.t_delay, nd + 1, 2 * nd};
        AdjCoef coef{L.t_fwd, L.t_cls, f->pair_in_dir, a->mirror_gain, f->pair_fprime, f->pair_unit_len,
                     f->air_attenuation, nd};
        unsigned n_active = 0;
        long long n_groups = 0;
        int rc = build_groups<T>(n, nb, nt, ps, f->receiver_order, coef, L.C, &n_active, &n_groups, st);
        if (rc != SP_OK) return rc;
        const int n_tiles = (n + kTile - 1) / kTile;
        const int words = (2 * nd + 31) / 32;
        k_present_bits<<<sp_blocks(n_tiles, 128), 128, 0, sp_counted(st)>>>(n_tiles, 2 * nd, words, L.C.seg_off,
                                                                            L.present);
        S->n_active = n_active;
        S->n_groups = n_groups;
    }
    // g and mu_K = g
    if (a->n_receivers > 0) {
        dim3 gg(nb, n);
        k_adjoint_g<T><<<gg, 256, 0, sp_counted(st)>>>(n, nb, nt, a->n_receivers, a->recv_factor, a->recv_dist,
                                                       f->speed_of_sound, f->time_resolution, f->air_attenuation,
                                                       a->grad_mono, (T*)L.g_rev);
    }
    for (int k = 0; k < 2; ++k) cudaMemsetAsync(L.mu[k], 0, (L.rows * L.rs + kStageF + 64) * sizeof(T), st);
    dim3 cg(nb, n);
    k_adjoint_combine<T><<<cg, 256, 0, sp_counted(st)>>>(n, nd, nb, nt, (long long)L.rs, L.lead, a->n_receivers,
                                                         a->recv_dir, (const T*)L.g_rev, nullptr, nullptr, 0,
                                                         L.C.tile_of, nullptr, f->wall_of, f->brdf_index, a->alpha,
                                                         a->scattering, (T*)L.mu[0], a->grad_alpha,
                                                         a->grad_scattering);
    S->ready = 1;
    return sp_check_launch();
}

template <typename T>
int adjoint_order(const sp_adjoint_args* a, const void* e_prev, void* ws, size_t ws_bytes, cudaStream_t st) {
    using WL = WsLayout<T>;
    const sp_exchange_args* f = a->fwd;
    const int n = f->n_patches, nd = f->n_dirs, nb = f->n_bins, nt = f->n_samples;
    const long long p = f->n_dir_pairs;
    AdjLayout L = adj_layout(nullptr, sizeof(T), n, nd, nb, nt, p, a->n_receivers);
    if (ws_bytes < L.bytes) return SP_ERR_WORKSPACE;
    L = adj_layout(ws, sizeof(T), n, nd, nb, nt, p, a->n_receivers);
    sp_adjoint_state* S = a->state;
    const int words = (2 * nd + 31) / 32;
    T* mu_in = (T*)L.mu[S->cur];
    T* mu_out = (T*)L.mu[1 - S->cur];
    if (S->n_active > 0) {
        auto kern = [] {
            if constexpr (sizeof(T) == 4)
                return k_scatter_f32;
            else
                return k_scatter_f64;
        }();
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WL::kSmem);
        dim3 sgrid(S->n_active, (nt + WL::kTW - 1) / WL::kTW, nb);
        kern<<<sgrid, kWsThreads, WL::kSmem, sp_counted(st)>>>(2 * nd, nb, nt, (long long)L.rs, L.lead, 2 * p,
                                                               L.C.tile_recv, L.C.seg_order, L.C.seg_off, L.C.groups,
                                                               L.C.wpack, (const T*)L.C.coef, mu_in, (T*)L.lam, L.err);
    }
    dim3 cg(nb, n);
    const T* lam = S->n_active > 0 ? (const T*)L.lam : nullptr;
    bool vec4 = false;  // FP32 with nt % 4 == 0: the float4 combine
    if constexpr (sizeof(T) == 4) {
        if (nt % 4 == 0) {
            k_adjoint_combine4<<<cg, 256, 0, sp_counted(st)>>>(
                n, nd, nb, nt, (long long)L.rs, L.lead, a->n_receivers, a->recv_dir, (const float*)L.g_rev, lam,
                L.present, words, L.C.tile_of, (const float*)e_prev, f->wall_of, f->brdf_index, a->alpha,
                a->scattering, mu_out, a->grad_alpha, a->grad_scattering);
            vec4 = true;
        }
    }
    if (!vec4)
        k_adjoint_combine<T><<<cg, 256, 0, sp_counted(st)>>>(
            n, nd, nb, nt, (long long)L.rs, L.lead, a->n_receivers, a->recv_dir, (const T*)L.g_rev, lam, L.present,
            words, L.C.tile_of, (const T*)e_prev, f->wall_of, f->brdf_index, a->alpha, a->scattering, mu_out,
            a->grad_alpha, a->grad_scattering);
    S->cur = 1 - S->cur;
    int rc = sp_check_launch();
    if (rc != SP_OK) return rc;
    int herr = 0;
    cudaMemcpyAsync(&herr, L.err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    return herr ? SP_ERR_TIMEOUT : SP_OK;
}

}  // namespace

extern "C" {

size_t sp_adjoint_workspace(int precision, int n_patches, int n_dirs, int n_bins, int n_samples,
                            long long n_dir_pairs, int n_receivers) {
    return adj_layout(nullptr, adj_esz(precision), n_patches, n_dirs, n_bins, n_samples, n_dir_pairs, n_receivers)
        .bytes;
}

int sp_adjoint_begin(const sp_adjoint_args* a, void* ws, size_t ws_bytes, void* stream) {
    if (!adj_args_ok(a) || !ws || a->n_receivers < 0 || (a->n_receivers > 0 && (!a->recv_dir || !a->recv_factor ||
                                                                               !a->recv_dist || !a->grad_mono)))
        return SP_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (a->fwd->precision == SP_F64) return adjoint_begin<double>(a, ws, ws_bytes, st);
    return adjoint_begin<float>(a, ws, ws_bytes, st);
}

int sp_adjoint_order(const sp_adjoint_args* a, const void* e_prev, void* ws, size_t ws_bytes, void* stream) {
    if (!adj_args_ok(a) || !ws || !e_prev || !a->state->ready) return SP_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (a->fwd->precision == SP_F64) return adjoint_order<double>(a, e_prev, ws, ws_bytes, st);
    return adjoint_order<float>(a, e_prev, ws, ws_bytes, st);
}

int sp_adjoint_finish(const sp_adjoint_args* a, double* grad_e0dir, void* ws, size_t ws_bytes, void* stream) {
    if (!adj_args_ok(a) || !ws || !grad_e0dir || !a->state->ready || !a->fwd->distance_0) return SP_ERR_ARG;
    const sp_exchange_args* f = a->fwd;
    const int n = f->n_patches, nd = f->n_dirs, nb = f->n_bins, nt = f->n_samples;
    const int esz = adj_esz(f->precision);
    AdjLayout L = adj_layout(nullptr, esz, n, nd, nb, nt, f->n_dir_pairs, a->n_receivers);
    if (ws_bytes < L.bytes) return SP_ERR_WORKSPACE;
    L = adj_layout(ws, esz, n, nd, nb, nt, f->n_dir_pairs, a->n_receivers);
    cudaStream_t st = (cudaStream_t)stream;
    const long long ne = (long long)n * nd * nb;
    if (esz == 8)
        k_adjoint_e0<double><<<sp_blocks(ne, 256), 256, 0, sp_counted(st)>>>(
            n, nd, nb, nt, (long long)L.rs, L.lead, (const double*)L.mu[a->state->cur], f->distance_0,
            f->speed_of_sound, f->time_resolution, grad_e0dir);
    else
        k_adjoint_e0<float><<<sp_blocks(ne, 256), 256, 0, sp_counted(st)>>>(
            n, nd, nb, nt, (long long)L.rs, L.lead, (const float*)L.mu[a->state->cur], f->distance_0,
            f->speed_of_sound, f->time_resolution, grad_e0dir);
    return sp_check_launch();
}

}  // extern "C"
