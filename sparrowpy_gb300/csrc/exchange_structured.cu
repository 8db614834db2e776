// Tiled structured energy exchange (RadiosityFast.py:1073-1145) for BRDF
// tables whose rows are  diff + spec * [o == m]  up to a per-slot scale:
//   BRDF[slot, s, o, b] = scale[slot, b] * (diff[c, b] + spec[c, b] * [o == m_c]),
// c = (material group of the slot, s) is the pair's class.  This is the form
// brdf.py:100-120 (`create_from_scattering`) produces, stored times pi.
//
// For receiver j and order k:
//   G_k[j, c, b, t] = sum_{pairs p -> j of class c} w_pb * E_{k-1}[src_p, p2o_p, b, t - n_p]
//   E_k[j, o, b, t] = sum_c (diff[c, b] + spec[c, b] [o == m_c]) * G_k[j, c, b, t]
//   E_total += E_k  (two orders at a time: see the order loop)
// with w_pb = F'_p * exp(-att_b |u_p|) * scale[slot(src_p), b].
//
// Plan (once per exchange call): receivers are cut into tiles of 16 (a given
// receiver order, normally spatial); a segment is (tile, class).  The
// segment's pairs are merged by source patch and cut into source groups:
// one source row (src * D + p2o), up to 16 member receivers, delays within
// n_base .. n_base + 45.  Everything is built in parallel and
// deterministically (row-wise class sort, merge by binary search, scans).
//
// Scatter (per order, FP32; exchange_scatter.cuh): one CTA per (segment,
// 1024-bin window, band).  A producer warp stages each group's source window
// (1072 values), packed member words and coefficients in shared memory with
// bulk asynchronous copies (cp.async.bulk + mbarrier, 6 stages of 4
// groups); 8 consumer warps, each owning 2 receiver slots x 1024 bins in
// registers, read the staged window at each member's delay offset, every
// warp read covering 32 consecutive floats.  FP64 uses the same plan with
// direct loads.  Mix: streams G into E_k and E_total.
#include "exchange_scatter.cuh"
#include "exchange_tc.cuh"

namespace {

// --------------------------------------------------------------- mix
// E_k[j, o, b, t] = sum_c diff[c, b] G[j, c, b, t] + sum_{c: m_c = o} spec[c, b] G[j, c, b, t]
// (the slot scale is folded into the scatter coefficients), written to the
// padded row of ecur, and E_total += E_k, or E_total += E_{k-1} + E_k when
// eadd holds the deferred previous order (padded rows), or nothing when
// etot is null.  One block per (band, receiver),
// all bins; only the classes present in the receiver's tile are read.
//
// Late bins (t >= t_late) of an FP32 E_total are added with Kahan
// compensation when comp is given: comp holds, per row, the compensation of
// bins t_late .. nt - 1 (rows of nt - t_late bfloat16 values), zero before
// the first order.  With x the order's addend (E_{k-1} + E_k, or E_k):
//   y = x - c;  s' = s + y;  c' = (s' - s) - y
// and the last update of a solve (fold) stores s' - c', the compensated sum.
template <typename T>
__global__ void __launch_bounds__(256) k_mix(int n_class, int nd, int nb, int nt, long long rs, int lead,
                                             const int32_t* __restrict__ tile_of, const int32_t* __restrict__ tab,
                                             const T* __restrict__ cdiff, const T* __restrict__ cspec,
                                             const T* __restrict__ g, T* __restrict__ ecur, T* __restrict__ etot,
                                             const T* __restrict__ eadd, uint16_t* __restrict__ comp, int t_late,
                                             int fold) {
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
    const int nl = nt - t_late;  // compensated bins per row
    const T* gj = g + ((size_t)j * n_class * nb + b) * nt;
    T* ek = ecur + ((size_t)j * nd * nb + b) * rs + lead;  // padded rows, stride rs
    T* et = etot ? etot + ((size_t)j * nd * nb + b) * nt : nullptr;  // nullptr: E_total not accumulated
    const T* ea = eadd ? eadd + ((size_t)j * nd * nb + b) * rs + lead : nullptr;  // deferred E_{k-1}, padded
    uint16_t* cj = (comp && et) ? comp + ((size_t)j * nd * nb + b) * nl : nullptr;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        T diffuse = T(0);
        for (int q = 0; q < np; ++q) {
            const int c = cls[q];
            if (s_cd[c] != T(0)) diffuse = fma(s_cd[c], gj[c * cstride + t], diffuse);  // skip pure mirror classes
        }
        for (int o = 0; o < nd; ++o) {
            T v = diffuse;
            for (int q = inv_off[o]; q < inv_off[o + 1]; ++q) {
                const int c = inv[q];
                v = fma(s_cs[c], gj[c * cstride + t], v);
            }
            ek[(size_t)o * nb * rs + t] = v;
            if (et) {
                T acc = et[o * cstride + t];
                if (cj && t >= t_late) {
                    uint16_t* cp = cj + (size_t)o * nb * nl + (t - t_late);
                    T cc = (T)comp_get(*cp);
                    kahan_add(acc, cc, ea ? ea[(size_t)o * nb * rs + t] + v : v);
                    if (fold) {
                        et[o * cstride + t] = acc - cc;
                    } else {
                        et[o * cstride + t] = acc;
                        *cp = comp_put((float)cc);
                    }
                } else {
                    if (ea) acc += ea[(size_t)o * nb * rs + t];
                    et[o * cstride + t] = acc + v;
                }
            }
        }
    }
}

// SP_EXCHANGE_GENERAL: E_k[j, o, b, t] = sum_c tab[c, o, b] G[j, c, b, t] over
// the classes present in j's tile (any BRDF table rows; the slot scale is in
// the scatter coefficients), on CUDA cores: one block per (band, receiver),
// one bin per thread, the D outputs of a bin in registers, each class value
// read once and broadcast weights from shared memory.  E_total as in k_mix.
constexpr int kGeneralMaxDirs = 64;
template <typename T>
__global__ void __launch_bounds__(128) k_mix_general(int n_class, int nd, int nb, int nt, long long rs, int lead,
                                                     const int32_t* __restrict__ tile_of,
                                                     const int32_t* __restrict__ tab, const T* __restrict__ ctab,
                                                     const T* __restrict__ g, T* __restrict__ ecur,
                                                     T* __restrict__ etot, const T* __restrict__ eadd,
                                                     uint16_t* __restrict__ comp, int t_late, int fold) {
    extern __shared__ __align__(16) unsigned char s_mix[];
    const int stride = tile_tab_stride(n_class, nd);
    int* s_tab = reinterpret_cast<int*>(s_mix);
    T* s_w = reinterpret_cast<T*>(s_mix + (((size_t)stride * sizeof(int) + 15) & ~(size_t)15));  // [np][nd]
    const int b = blockIdx.x, j = blockIdx.y;
    const int tile = tile_of[j];
    for (int k = threadIdx.x; k < stride; k += blockDim.x) s_tab[k] = tab[(size_t)tile * stride + k];
    __syncthreads();
    const int np = s_tab[0];
    const int* cls = s_tab + 1;
    for (int k = threadIdx.x; k < np * nd; k += blockDim.x) {
        const int q = k / nd, o = k % nd;
        s_w[k] = ctab[((size_t)cls[q] * nd + o) * nb + b];
    }
    __syncthreads();
    const size_t cstride = (size_t)nb * nt;
    const int nl = nt - t_late;
    const T* gj = g + ((size_t)j * n_class * nb + b) * nt;
    T* ek = ecur + ((size_t)j * nd * nb + b) * rs + lead;
    T* et = etot ? etot + ((size_t)j * nd * nb + b) * nt : nullptr;
    const T* ea = eadd ? eadd + ((size_t)j * nd * nb + b) * rs + lead : nullptr;
    uint16_t* cj = (comp && et) ? comp + ((size_t)j * nd * nb + b) * nl : nullptr;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        T v[kGeneralMaxDirs];
#pragma unroll
        for (int o = 0; o < kGeneralMaxDirs; ++o) v[o] = T(0);
        for (int q = 0; q < np; ++q) {
            const T x = gj[(size_t)cls[q] * cstride + t];
            const T* w = s_w + (size_t)q * nd;
#pragma unroll
            for (int o = 0; o < kGeneralMaxDirs; ++o)
                if (o < nd) v[o] = fma(w[o], x, v[o]);
        }
        const bool late = cj != nullptr && t >= t_late;
#pragma unroll
        for (int o0 = 0; o0 < kGeneralMaxDirs; o0 += 8) {
            if (o0 >= nd) break;
            // eight directions' loads before their stores
            T e8[8], a8[8];
            uint16_t c8[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int o = o0 + q;
                e8[q] = (o < nd && et) ? et[o * cstride + t] : T(0);
                a8[q] = (o < nd && ea) ? ea[(size_t)o * nb * rs + t] : T(0);
                c8[q] = (o < nd && late) ? cj[(size_t)o * nb * nl + (t - t_late)] : (uint16_t)0;
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int o = o0 + q;
                if (o >= nd) break;
                const T vo = v[o];  // o is a compile-time index (both loops unrolled)
                ek[(size_t)o * nb * rs + t] = vo;
                if (!et) continue;
                if (late) {
                    T acc = e8[q], cc = (T)comp_get(c8[q]);
                    kahan_add(acc, cc, ea ? a8[q] + vo : vo);
                    if (fold) {
                        et[o * cstride + t] = acc - cc;
                    } else {
                        et[o * cstride + t] = acc;
                        cj[(size_t)o * nb * nl + (t - t_late)] = comp_put((float)cc);
                    }
                } else {
                    et[o * cstride + t] = (ea ? e8[q] + a8[q] : e8[q]) + vo;
                }
            }
        }
    }
}

constexpr size_t kMixGeneralMaxSmem = 200 * 1024;
inline size_t mix_general_smem(int n_class, int nd, int esz) {
    return (((size_t)tile_tab_stride(n_class, nd) * sizeof(int) + 15) & ~(size_t)15) + (size_t)n_class * nd * esz;
}

// k_mix for FP32 with nt % 4 == 0: four bins per thread (16-byte accesses),
// and the E_total values of up to 8 directions loaded before any is stored.
__device__ __forceinline__ float4 fma4(float a, float4 x, float4 y) {
    return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}
__device__ __forceinline__ float4 add4(float4 x, float4 y) {
    return make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
}

__device__ __forceinline__ float4 sub4(float4 x, float4 y) {
    return make_float4(x.x - y.x, x.y - y.y, x.z - y.z, x.w - y.w);
}
// Kahan step on four lanes: s += x with compensation c (see k_mix)
__device__ __forceinline__ void kahan_add4(float4& s, float4& c, float4 x) {
    const float4 y = sub4(x, c);
    const float4 t = add4(s, y);
    c = sub4(sub4(t, s), y);
    s = t;
}

// The mix of one (band b, receiver j) by the whole block (any block size);
// s_mix: 2 n_class floats + the tile table row.  kOG directions' loads are
// issued together (8 in k_mix4; fewer where registers are short).
// One float4 of bins (index t) of one (band, receiver) row of the mix: the
// class sums, E_k and the E_total update (see k_mix).  s_cd / s_cs: the
// band's class weights; the row pointers are those of the (band, receiver).
// The mix of float4 bins t, t + step, ..., t + (kU - 1) step (those below
// nt4) without an E_total update: the class sums and E_k only.  The kU bins'
// loads of one class are issued together, so that a thread keeps kU loads in
// flight (the persistent batch runs few threads per SM).
template <int kU>
__device__ __forceinline__ void mix4_store_bins(int t, int step, int nt4, int np, const int* cls, const int* inv_off,
                                                const int* inv, const float* s_cd, const float* s_cs, int nd,
                                                size_t cs4, size_t ers4, const float4* __restrict__ gj,
                                                float4* __restrict__ ek) {
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 d[kU];
    bool on[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
        on[u] = t + u * step < nt4;
        d[u] = zero;
    }
    for (int q = 0; q < np; ++q) {
        const int c = cls[q];
        const float w = s_cd[c];
        if (w == 0.0f) continue;  // pure mirror classes
        float4 g[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) g[u] = on[u] ? __ldg(gj + c * cs4 + t + u * step) : zero;
#pragma unroll
        for (int u = 0; u < kU; ++u) d[u] = fma4(w, g[u], d[u]);
    }
    for (int o = 0; o < nd; ++o) {
        float4 v[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) v[u] = d[u];
        for (int q = inv_off[o]; q < inv_off[o + 1]; ++q) {
            const int cl = inv[q];
            const float w = s_cs[cl];
            float4 g[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) g[u] = on[u] ? __ldg(gj + cl * cs4 + t + u * step) : zero;
#pragma unroll
            for (int u = 0; u < kU; ++u) v[u] = fma4(w, g[u], v[u]);
        }
#pragma unroll
        for (int u = 0; u < kU; ++u)
            if (on[u]) ek[o * ers4 + t + u * step] = v[u];
    }
}

template <int kOG>
__device__ __forceinline__ void mix4_bin(int t, int np, const int* cls, const int* inv_off, const int* inv,
                                         const float* s_cd, const float* s_cs, int nd, size_t cs4, size_t ers4,
                                         size_t cc4, int tl4, const float4* __restrict__ gj, float4* __restrict__ ek,
                                         float4* __restrict__ et, const float4* __restrict__ ea,
                                         ushort4* __restrict__ cj, int fold) {
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 d = zero;
    for (int q = 0; q < np; ++q) {
        const int c = cls[q];
        if (s_cd[c] != 0.0f) d = fma4(s_cd[c], __ldg(gj + c * cs4 + t), d);  // skip pure mirror classes
    }
    const bool late = cj != nullptr && t >= tl4;
    for (int o0 = 0; o0 < nd; o0 += kOG) {
        const int no = min(kOG, nd - o0);
        // every load of the kOG directions (E_total, deferred E_{k-1}, compensation) before any store
        float4 e[kOG], x[kOG];
        ushort4 c[kOG];
#pragma unroll
        for (int k = 0; k < kOG; ++k) {
            e[k] = (k < no && et) ? et[(o0 + k) * cs4 + t] : zero;
            x[k] = (k < no && ea) ? __ldg(ea + (o0 + k) * ers4 + t) : zero;
            c[k] = (k < no && late) ? cj[(o0 + k) * cc4 + (t - tl4)] : make_ushort4(0, 0, 0, 0);
        }
#pragma unroll
        for (int k = 0; k < kOG; ++k) {
            if (k < no) {
                const int o = o0 + k;
                float4 v = d;
                for (int q = inv_off[o]; q < inv_off[o + 1]; ++q) {
                    const int cl = inv[q];
                    v = fma4(s_cs[cl], __ldg(gj + cl * cs4 + t), v);
                }
                ek[o * ers4 + t] = v;
                if (!et) continue;
                if (late) {
                    float4 s_ = e[k];
                    float4 cc = make_float4(comp_get(c[k].x), comp_get(c[k].y), comp_get(c[k].z), comp_get(c[k].w));
                    kahan_add4(s_, cc, ea ? add4(x[k], v) : v);
                    if (fold) {
                        et[o * cs4 + t] = sub4(s_, cc);
                    } else {
                        et[o * cs4 + t] = s_;
                        cj[o * cc4 + (t - tl4)] =
                            make_ushort4(comp_put(cc.x), comp_put(cc.y), comp_put(cc.z), comp_put(cc.w));
                    }
                } else {
                    et[o * cs4 + t] = add4(ea ? add4(e[k], x[k]) : e[k], v);
                }
            }
        }
    }
}

// The mix of receiver j for the bands [b0, b0 + n_bands) by the whole block
// (any block size): the tile table and the bands' class weights in s_mix
// (n_bands x 2 n_class floats, then the tile table row), then the threads
// split evenly over the bands, each walking its band's bins (float4).
template <int kOG = 8, bool kSplitBands = false, bool kTotal = true>
__device__ __forceinline__ void mix4_item(int n_class, int nd, int nb, int nt, long long rs, int lead,
                                          const int32_t* __restrict__ tile_of, const int32_t* __restrict__ tab,
                                          const float* __restrict__ cdiff, const float* __restrict__ cspec,
                                          const float* __restrict__ g, float* __restrict__ ecur,
                                          float* __restrict__ etot, const float* __restrict__ eadd,
                                          uint16_t* __restrict__ comp, int t_late, int fold, int b0, int j,
                                          unsigned char* s_mix, int n_bands = 1) {
    const int stride = tile_tab_stride(n_class, nd);
    float* s_w = reinterpret_cast<float*>(s_mix);  // [n_bands][2][n_class]
    int* s_tab = reinterpret_cast<int*>(s_w + (size_t)2 * n_bands * n_class);
    const int tile = tile_of[j];
    for (int k = threadIdx.x; k < stride; k += blockDim.x) s_tab[k] = tab[(size_t)tile * stride + k];
    for (int q = threadIdx.x; q < n_bands * n_class; q += blockDim.x) {
        const int bb = q / n_class, c = q % n_class;
        s_w[(size_t)2 * bb * n_class + c] = cdiff[(size_t)c * nb + b0 + bb];
        s_w[(size_t)(2 * bb + 1) * n_class + c] = cspec[(size_t)c * nb + b0 + bb];
    }
    __syncthreads();
    const int per = kSplitBands ? (int)blockDim.x / n_bands : (int)blockDim.x;  // threads per band
    const int bb = kSplitBands ? (int)threadIdx.x / per : 0;
    const int lt = kSplitBands ? (int)threadIdx.x % per : (int)threadIdx.x;
    if (kSplitBands && bb >= n_bands) return;  // the remainder threads have no band
    const int b = b0 + bb;
    const float* s_cd = s_w + (size_t)2 * bb * n_class;
    const float* s_cs = s_cd + n_class;
    const int np = s_tab[0];
    const int* cls = s_tab + 1;
    const int* inv_off = cls + n_class;
    const int* inv = inv_off + nd + 1;
    const int nt4 = nt >> 2;
    const int tl4 = t_late >> 2;  // t_late is a multiple of 4
    const size_t cs4 = (size_t)nb * nt4;  // class (G) and direction (E_total) stride, in float4
    const size_t ers4 = (size_t)nb * (size_t)(rs >> 2);  // direction stride of the padded ecur rows
    const size_t cc4 = (size_t)nb * (nt4 - tl4);        // direction stride of the compensation rows
    const float4* gj = reinterpret_cast<const float4*>(g + ((size_t)j * n_class * nb + b) * nt);
    float4* ek = reinterpret_cast<float4*>(ecur + ((size_t)j * nd * nb + b) * rs + lead);
    float4* et = etot ? reinterpret_cast<float4*>(etot + ((size_t)j * nd * nb + b) * nt) : nullptr;
    const float4* ea = eadd ? reinterpret_cast<const float4*>(eadd + ((size_t)j * nd * nb + b) * rs + lead) : nullptr;
    ushort4* cj = (comp && et) ? reinterpret_cast<ushort4*>(comp + ((size_t)j * nd * nb + b) * (nt - t_late)) : nullptr;
    if constexpr (kTotal) {
        for (int t = lt; t < nt4; t += per)
            mix4_bin<kOG>(t, np, cls, inv_off, inv, s_cd, s_cs, nd, cs4, ers4, cc4, tl4, gj, ek, et, ea, cj, fold);
    } else {
        // one bin a thread at a time: four (measured on the canyon) read 30 % more DRAM bytes for the same time
        constexpr int kU = 1;
        for (int t = lt; t < nt4; t += per * kU)
            mix4_store_bins<kU>(t, per, nt4, np, cls, inv_off, inv, s_cd, s_cs, nd, cs4, ers4, gj, ek);
    }
}

// kTotal: with the E_total update (etot non-null); without it (the first
// order of a pair, and every order of the partial sums) only E_k is written.
template <bool kTotal>
__global__ void __launch_bounds__(128, kTotal ? 4 : 8) k_mix4(int n_class, int nd, int nb, int nt, long long rs, int lead,
                                              const int32_t* __restrict__ tile_of, const int32_t* __restrict__ tab,
                                              const float* __restrict__ cdiff, const float* __restrict__ cspec,
                                              const float* __restrict__ g, float* __restrict__ ecur,
                                              float* __restrict__ etot, const float* __restrict__ eadd,
                                              uint16_t* __restrict__ comp, int t_late, int fold) {
    extern __shared__ __align__(16) unsigned char s_mix[];
    mix4_item<8, false, kTotal>(n_class, nd, nb, nt, rs, lead, tile_of, tab, cdiff, cspec, g, ecur, etot, eadd,
                                comp, t_late, fold, blockIdx.x, blockIdx.y, s_mix);
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
    if (etot) etot[(size_t)e * nt + dly] = v;
    eprev[(size_t)e * rs + lead + dly] = v;
}

// Partial sums (sp_exchange_args.partial_sums): S_k = E_0 + M(S_{k-1}).
// After the mix has written M(S_{k-1}) into `dst` (rows of pitch rs, bin 0
// at lead), add the source energies at the bins k_init_energy_t placed them
// in (one bin per row; the delays were range-checked there).
template <typename T>
__global__ void k_add_e0_t(int n, int nd, int nb, int nt, long long rs, int lead, const double* __restrict__ e0dir,
                           const double* __restrict__ d0, double c, double dt, T* __restrict__ dst) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)n * nd * nb) return;
    int i = (int)(e / ((long long)nd * nb));
    long long dly = (long long)xdiv(xdiv(d0[i], c), dt);
    if (dly < 0 || dly >= nt) return;
    dst[(size_t)e * rs + lead + dly] += (T)e0dir[e];
}

template <typename T>
__global__ void k_convert_t(long long count, const double* __restrict__ in, T* __restrict__ out) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) out[e] = (T)in[e];
}

// ----------------------------------------------------------- materials
// SP_EXCHANGE_MATERIAL: BRDF_s[c, o, b] = (1 - a_s,b)(s_s,b + (1 - s_s,b) K_c [o == m_c])
// (create_from_scattering tables x pi).  Each pair e: i -> j enters twice:
// the diffuse part (class 0, coefficient w (1 - a) s, shared by all incoming
// directions) and the mirror part (class 1 + c(e), coefficient
// w (1 - a)(1 - s) K_c); the mix then adds class 0 to every outgoing row and
// class 1 + c to row m_c.  Rows of j: diffuse entries, then mirror entries,
// each in the source order of the pair list.
__global__ void k_expand_material_pairs(long long p, int nt, const int64_t* __restrict__ off,
                                        const int32_t* __restrict__ src, const int32_t* __restrict__ dst,
                                        const int32_t* __restrict__ out_dir, const int32_t* __restrict__ in_dir,
                                        const int32_t* __restrict__ delay, const int32_t* __restrict__ mirror,
                                        int32_t* __restrict__ x_src, int32_t* __restrict__ x_dst,
                                        int32_t* __restrict__ x_row, int32_t* __restrict__ x_cls,
                                        int32_t* __restrict__ x_delay, int32_t* __restrict__ x_fwd) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p) return;
    const int j = dst[e];
    const long long deg = off[j + 1] - off[j];
    const long long t0 = 2 * off[j] + (e - off[j]);
    const long long t1 = t0 + deg;
    const int c = in_dir[e];
    x_src[t0] = src[e];
    x_src[t1] = src[e];
    x_dst[t0] = j;
    x_dst[t1] = j;
    x_row[t0] = out_dir[e];
    x_row[t1] = out_dir[e];
    x_cls[t0] = 0;
    x_cls[t1] = 1 + c;
    x_delay[t0] = delay[e];
    x_delay[t1] = mirror[c] >= 0 ? delay[e] : nt;  // no mirror term: dropped by the planner
    x_fwd[t0] = (int32_t)e;
    x_fwd[t1] = (int32_t)e;
}

__global__ void k_double_offsets_fwd(int n, const int64_t* __restrict__ off, int64_t* __restrict__ x_off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= n) x_off[i] = 2 * off[i];
}

// Class tables of the material mode: class 0 diffuse (to every row), class 1 + c mirror (to row m_c).
template <typename T>
__global__ void k_material_classes(int n_in, int nb, const int32_t* __restrict__ mirror, T* __restrict__ cdiff,
                                   T* __restrict__ cspec, int32_t* __restrict__ ctarget) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > n_in) return;
    for (int b = 0; b < nb; ++b) {
        cdiff[(size_t)c * nb + b] = c == 0 ? T(1) : T(0);
        cspec[(size_t)c * nb + b] = c == 0 ? T(0) : T(1);
    }
    ctarget[c] = c == 0 ? -1 : mirror[c - 1];
}

// SP_EXCHANGE_SLOTWISE: tables of the diffuse-plus-mirror form with any
// number of material groups (e.g. per-patch scattering, where every slot's
// normalised rows differ):
//   BRDF[slot, s, o, b] = scale[slot, b] (diff[c, b] + spec[c, b] [o == m_c]),
// c = group(slot) n_in + s.  Each pair e enters twice: the diffuse part
// (class 0, coefficient w scale diff_c) and the mirror part (class 1 + m_c,
// coefficient w scale spec_c; none when m_c < 0).  The mix adds class 0 to
// every outgoing row and class 1 + o to row o, so the class count is 1 + D
// whatever the number of groups.
__global__ void k_expand_slotwise_pairs(long long p, int nt, const int64_t* __restrict__ off,
                                        const int32_t* __restrict__ src, const int32_t* __restrict__ dst,
                                        const int32_t* __restrict__ out_dir, const int32_t* __restrict__ pcls,
                                        const int32_t* __restrict__ delay, const int32_t* __restrict__ ctarget,
                                        int32_t* __restrict__ x_src, int32_t* __restrict__ x_dst,
                                        int32_t* __restrict__ x_row, int32_t* __restrict__ x_cls,
                                        int32_t* __restrict__ x_delay, int32_t* __restrict__ x_fwd) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p) return;
    const int j = dst[e];
    const long long deg = off[j + 1] - off[j];
    const long long t0 = 2 * off[j] + (e - off[j]);
    const long long t1 = t0 + deg;
    const int m = ctarget[pcls[e]];
    x_src[t0] = src[e];
    x_src[t1] = src[e];
    x_dst[t0] = j;
    x_dst[t1] = j;
    x_row[t0] = out_dir[e];
    x_row[t1] = out_dir[e];
    x_cls[t0] = 0;
    x_cls[t1] = m >= 0 ? 1 + m : 0;
    x_delay[t0] = delay[e];
    x_delay[t1] = m >= 0 ? delay[e] : nt;  // no mirror term: dropped by the planner
    x_fwd[t0] = (int32_t)e;
    x_fwd[t1] = (int32_t)e;
}

// Class tables of the slot-wise mode: class 0 diffuse (to every row), class 1 + o mirror (to row o).
template <typename T>
__global__ void k_slotwise_classes(int nd, int nb, T* __restrict__ cdiff, T* __restrict__ cspec,
                                   int32_t* __restrict__ ctarget) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > nd) return;
    for (int b = 0; b < nb; ++b) {
        cdiff[(size_t)c * nb + b] = c == 0 ? T(1) : T(0);
        cspec[(size_t)c * nb + b] = c == 0 ? T(0) : T(1);
    }
    ctarget[c] = c - 1;
}

struct SlotCoef {
    const int32_t* fwd;
    const int32_t* xcls;
    const int32_t* pcls;  // structured class of each pair
    const int32_t* src;
    const int32_t* wall_of;
    const int32_t* brdf_index;
    const double* slot_scale;
    const double* cdiff;
    const double* cspec;
    const double* fprime;
    const double* unit_len;
    const double* att;
    int nb;
    __device__ double operator()(long long t, int b) const {
        const long long e = fwd[t];
        const int slot = brdf_index[wall_of[src[e]]];
        const size_t cb = (size_t)pcls[e] * nb + b;
        double f = fprime[e];
        if (att) f = f * exp(-att[b] * unit_len[e]);
        f = f * slot_scale[(size_t)slot * nb + b];
        return xcls[t] == 0 ? f * cdiff[cb] : f * cspec[cb];
    }
    __device__ float f32(long long t, int b) const {
        const long long e = fwd[t];
        const int slot = brdf_index[wall_of[src[e]]];
        const size_t cb = (size_t)pcls[e] * nb + b;
        float f = f64_trunc_f32(fprime[e]);
        if (att) f = f * expf(-f64_trunc_f32(att[b]) * f64_trunc_f32(unit_len[e]));
        f = f * f64_trunc_f32(slot_scale[(size_t)slot * nb + b]);
        return xcls[t] == 0 ? f * f64_trunc_f32(cdiff[cb]) : f * f64_trunc_f32(cspec[cb]);
    }
};

struct MatCoef {
    const int32_t* fwd;
    const int32_t* cls;
    const int32_t* src;
    const int32_t* in_dir;
    const int32_t* wall_of;
    const int32_t* brdf_index;
    const double* alpha;
    const double* scat;
    const double* gain;
    const double* fprime;
    const double* unit_len;
    const double* att;
    int nb;
    __device__ double operator()(long long t, int b) const {
        const long long e = fwd[t];
        const int slot = brdf_index[wall_of[src[e]]];
        double f = fprime[e];
        if (att) f = f * exp(-att[b] * unit_len[e]);
        const double a = alpha[(size_t)slot * nb + b], s = scat[(size_t)slot * nb + b];
        return cls[t] == 0 ? f * ((1.0 - a) * s) : f * ((1.0 - a) * (1.0 - s) * gain[in_dir[e]]);
    }
    __device__ float f32(long long t, int b) const {
        const long long e = fwd[t];
        const int slot = brdf_index[wall_of[src[e]]];
        float f = f64_trunc_f32(fprime[e]);
        if (att) f = f * expf(-f64_trunc_f32(att[b]) * f64_trunc_f32(unit_len[e]));
        const float a = f64_trunc_f32(alpha[(size_t)slot * nb + b]), s = f64_trunc_f32(scat[(size_t)slot * nb + b]);
        return cls[t] == 0 ? f * ((1.0f - a) * s)
                           : f * ((1.0f - a) * (1.0f - s) * f64_trunc_f32(gain[in_dir[e]]));
    }
};

// ------------------------------------------------------------ layout
// Padded histogram rows: `lead` zeros, then nt bins; stride rs (a multiple of
// 4 elements, so rows stay 16-byte aligned); `lead` >= nt + kMaxSpan + 4 so
// that no staged window starts before its buffer, and a tail after the last
// row keeps the last rows' windows inside the allocation.
struct Rows {
    int lead;
    size_t rs;
    size_t tail;
};
inline Rows padded_rows(int nt) {
    Rows R;
    R.lead = (int)((((size_t)nt + kMaxSpan + 4) + 3) & ~(size_t)3);
    R.rs = (((size_t)nt + R.lead) + 3) & ~(size_t)3;
    R.tail = (size_t)kStageF + 64;
    return R;
}

struct Plan {
    size_t bytes;
    Rows R;
    size_t rows;  // N * D * B
    void* eprev;
    void* ecur;
    void* g;
    int32_t* delay;
    int32_t* cls;
    PlanCore C;
    int32_t* tile_tab;
    void* cdiff;
    void* cspec;
    int32_t* ctarget;
    void* ctab;  // SP_EXCHANGE_GENERAL: (n_class, D, B) class table rows in T
    // material mode: the expanded pair list
    int64_t* x_off;
    int32_t *x_src, *x_dst, *x_row, *x_cls, *x_delay, *x_fwd;
    int64_t* info;  // [signature, n_active, n_groups, 0]
    int* err;
    int t_late;     // first compensated E_total bin (FP32): nt / 2, rounded down to a multiple of 4
    uint16_t* comp;  // FP32: (N * D * B, nt - t_late) Kahan compensation of E_total's late bins (bfloat16)
};

// First late bin of E_total: half the histogram, on a float4 boundary.
inline int late_bin(int nt) { return (nt / 2) & ~3; }

Plan plan_layout(void* base, int esz, int n, int nd, int nb, int nt, long long p, int n_class, bool material,
                 bool general) {
    Plan L;
    char* q = (char*)base;
    auto take = [&](size_t bytes) {
        char* r = q;
        q += sp_align(bytes);
        return (void*)r;
    };
    const int n_tiles = (n + kTile - 1) / kTile;
    L.R = padded_rows(nt);
    L.rows = (size_t)n * nd * nb;
    L.eprev = take((L.rows * L.R.rs + L.R.tail) * esz);
    L.ecur = take((L.rows * L.R.rs + L.R.tail) * esz);
    L.g = take((size_t)n * n_class * nb * nt * esz);
    L.delay = (int32_t*)take((size_t)p * 4);
    L.cls = (int32_t*)take((size_t)p * 4);
    const long long pp = material ? 2 * p : p;  // pairs the plan groups
    L.C = plan_core_layout(take, esz, n, nb, pp, n_class);
    L.tile_tab = (int32_t*)take((size_t)n_tiles * tile_tab_stride(n_class, nd) * 4);
    L.cdiff = take((size_t)n_class * nb * esz);
    L.cspec = take((size_t)n_class * nb * esz);
    L.ctarget = (int32_t*)take((size_t)n_class * 4);
    L.ctab = general ? take((size_t)n_class * nd * nb * esz) : nullptr;
    L.x_off = nullptr;
    L.x_src = L.x_dst = L.x_row = L.x_cls = L.x_delay = L.x_fwd = nullptr;
    if (material) {
        L.x_off = (int64_t*)take(((size_t)n + 1) * 8);
        L.x_src = (int32_t*)take((size_t)pp * 4);
        L.x_dst = (int32_t*)take((size_t)pp * 4);
        L.x_row = (int32_t*)take((size_t)pp * 4);
        L.x_cls = (int32_t*)take((size_t)pp * 4);
        L.x_delay = (int32_t*)take((size_t)pp * 4);
        L.x_fwd = (int32_t*)take((size_t)pp * 4);
    }
    L.info = (int64_t*)take(32);
    L.err = (int*)take(16);
    L.t_late = late_bin(nt);
    L.comp = esz == 4 ? (uint16_t*)take(L.rows * (size_t)(nt - L.t_late) * 2) : nullptr;
    L.bytes = (size_t)(q - (char*)base);
    return L;
}

// Identifies a plan for reuse: the caller's tag and every size it depends on.
inline int64_t plan_signature(const sp_exchange_args* a, int n_class) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        h ^= v;
        h *= 1099511628211ull;
    };
    mix((uint64_t)a->plan_tag);
    mix((uint64_t)a->algorithm);
    mix((uint64_t)a->n_patches);
    mix((uint64_t)a->n_dirs);
    mix((uint64_t)a->n_bins);
    mix((uint64_t)a->n_samples);
    mix((uint64_t)a->n_dir_pairs);
    mix((uint64_t)n_class);
    mix((uint64_t)(uintptr_t)a->pair_src);
    mix((uint64_t)(uintptr_t)a->dst_offset);
    return (int64_t)(h | 1ull);  // never 0
}

// Copy between unpadded (N*D*B, nt) histograms and padded rows (stride rs, bin 0 at lead).
template <typename T>
void copy_rows(T* dst, size_t dst_pitch, const T* src, size_t src_pitch, int nt, size_t rows, cudaStream_t st) {
    cudaMemcpy2DAsync(dst, dst_pitch * sizeof(T), src, src_pitch * sizeof(T), (size_t)nt * sizeof(T), rows,
                      cudaMemcpyDeviceToDevice, st);
}

template <typename T>
int run_tiled(const sp_exchange_args* a, void* ws, size_t ws_bytes, cudaStream_t st) {
    const int n = a->n_patches, nd = a->n_dirs, nb = a->n_bins, nt = a->n_samples;
    const long long p = a->n_dir_pairs;
    const bool slotwise = a->algorithm == SP_EXCHANGE_SLOTWISE;
    const bool general = a->algorithm == SP_EXCHANGE_GENERAL;
    const bool material = a->algorithm == SP_EXCHANGE_MATERIAL || slotwise;  // pairs enter twice
    if (a->algorithm == SP_EXCHANGE_MATERIAL) {
        if (!a->mat_alpha || !a->mat_scattering || !a->mat_mirror || !a->mat_gain || a->n_in_dirs < 1)
            return SP_ERR_ARG;
    } else if (general) {
        if (!a->slot_group || !a->slot_scale || !a->class_table || a->n_groups < 1) return SP_ERR_ARG;
        if (nd > kGeneralMaxDirs) return SP_ERR_UNSUPPORTED;
    } else if (!a->slot_group || !a->slot_scale || !a->class_diff || !a->class_spec || !a->class_target ||
               a->n_groups < 1) {
        return SP_ERR_ARG;
    }
    const int n_class = slotwise ? 1 + nd : material ? 1 + a->n_in_dirs : a->n_groups * a->n_in_dirs;
    if (n_class > kMaxClasses) return SP_ERR_UNSUPPORTED;
    const int k0 = a->state_in ? a->state_order : 0;
    if (k0 < 0 || (a->states_out && a->states_every < 1)) return SP_ERR_ARG;
    if (nt > 65535) return SP_ERR_UNSUPPORTED;  // base delays are packed in 16 bits
    if (general && mix_general_smem(n_class, nd, sizeof(T)) > kMixGeneralMaxSmem) return SP_ERR_UNSUPPORTED;
    // the receiver-side contraction on tensor cores: FP32, 32 <= D <= 64 (a multiple of 16, the MMA's N)
    const bool tensor_mix = general && sizeof(T) == 4 && !a->no_tensor_cores && nd >= 32 && nd <= 64 &&
                            nd % 16 == 0 && tc_smem_bytes(n_class, nd) <= kTcSmemMax;
    Plan L = plan_layout(nullptr, sizeof(T), n, nd, nb, nt, p, n_class, material, general);
    if (ws_bytes < L.bytes) return SP_ERR_WORKSPACE;
    L = plan_layout(ws, sizeof(T), n, nd, nb, nt, p, n_class, material, general);
    const int n_tiles = (n + kTile - 1) / kTile;
    const size_t e = (size_t)n * nd * nb * nt;
    T* etot = a->skip_total ? nullptr : (T*)a->etc_total;
    T* eprev = (T*)L.eprev;
    T* ecur = (T*)L.ecur;
    const long long rs = (long long)L.R.rs;
    const int lead = L.R.lead;
    T* states = (T*)a->states_out;
    // partial sums S_k = E_0 + M(S_{k-1}): E_total is S_K, no per-order E_total update
    const bool partial = a->partial_sums != 0;
    if (partial && (!etot || states || a->state_in)) return SP_ERR_ARG;
    // Kahan compensation of E_total's late bins (FP32, unless switched off)
    uint16_t* comp = (sizeof(T) == 4 && etot && !a->plain_total && !partial) ? L.comp : nullptr;
    cudaMemsetAsync(L.err, 0, sizeof(int), st);
    if (comp) cudaMemsetAsync(comp, 0, L.rows * (size_t)(nt - L.t_late) * sizeof(uint16_t), st);
    // ecur: only the leads need zeros (every bin is written each order);
    // eprev: the same when a starting state fills its bins, else all zero
    // before the starting energies are placed
    cudaMemset2DAsync(ecur, L.R.rs * sizeof(T), 0, (size_t)lead * sizeof(T), L.rows, st);
    if (a->state_in) {
        cudaMemset2DAsync(eprev, L.R.rs * sizeof(T), 0, (size_t)lead * sizeof(T), L.rows, st);
        cudaMemsetAsync(eprev + L.rows * L.R.rs, 0, L.R.tail * sizeof(T), st);
        copy_rows(eprev + lead, L.R.rs, (const T*)a->state_in, (size_t)nt, nt, L.rows, st);
        if (etot) cudaMemcpyAsync(etot, a->state_in, e * sizeof(T), cudaMemcpyDeviceToDevice, st);
    } else {
        cudaMemsetAsync(eprev, 0, (L.rows * L.R.rs + L.R.tail) * sizeof(T), st);
        if (etot) cudaMemsetAsync(etot, 0, e * sizeof(T), st);
        long long ne = (long long)n * nd * nb;
        k_init_energy_t<T><<<sp_blocks(ne, 256), 256, 0, sp_counted(st)>>>(
            n, nd, nb, nt, rs, lead, a->energy_0_dir, a->distance_0, a->speed_of_sound, a->time_resolution, etot,
            eprev, L.err);
        int herr = 0;
        cudaMemcpyAsync(&herr, L.err, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
        if (herr) return SP_ERR_RANGE;
    }
    if (states && !a->state_in) copy_rows(states, (size_t)nt, eprev + lead, L.R.rs, nt, L.rows, st);
    if (a->max_order <= k0 || p == 0) return sp_check_launch();

    // ---- plan (or the one a previous call with the same tag left in ws)
    unsigned n_active = 0;
    long long n_groups = 0;
    int rc;
    const long long pp = material ? 2 * p : p;  // entries in the plan's pair list
    const int64_t sig = a->plan_tag ? plan_signature(a, n_class) : 0;
    bool reuse = false;
    if (sig) {
        int64_t info[4] = {0, 0, 0, 0};
        cudaMemcpyAsync(info, L.info, sizeof(info), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
        if (info[0] == sig) {
            reuse = true;
            n_active = (unsigned)info[1];
            n_groups = info[2];
        }
    }
    if (!reuse) {
    k_delays_t<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, a->pair_distance, a->speed_of_sound,
                                                              a->time_resolution, L.delay);
    if (slotwise) {
        k_pair_class_t<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, a->pair_src, a->pair_in_dir, a->wall_of,
                                                                      a->brdf_index, a->slot_group, a->n_in_dirs,
                                                                      L.cls);
        k_expand_slotwise_pairs<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(
            p, nt, a->dst_offset, a->pair_src, a->pair_dst, a->pair_out_dir, L.cls, L.delay, a->class_target,
            L.x_src, L.x_dst, L.x_row, L.x_cls, L.x_delay, L.x_fwd);
        k_double_offsets_fwd<<<sp_blocks(n + 1, 256), 256, 0, sp_counted(st)>>>(n, a->dst_offset, L.x_off);
        PairSet ps{pp, L.x_off, L.x_src, L.x_dst, L.x_row, L.x_cls, L.x_delay, nd, n_class};
        SlotCoef coef{L.x_fwd, L.x_cls, L.cls, a->pair_src, a->wall_of, a->brdf_index, a->slot_scale, a->class_diff,
                      a->class_spec, a->pair_fprime, a->pair_unit_len, a->air_attenuation, nb};
        rc = build_groups<T>(n, nb, nt, ps, a->receiver_order, coef, L.C, &n_active, &n_groups, st);
        if (rc != SP_OK) return rc;
        k_slotwise_classes<T><<<sp_blocks(n_class, 128), 128, 0, sp_counted(st)>>>(nd, nb, (T*)L.cdiff,
                                                                                  (T*)L.cspec, L.ctarget);
    } else if (material) {
        k_expand_material_pairs<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(
            p, nt, a->dst_offset, a->pair_src, a->pair_dst, a->pair_out_dir, a->pair_in_dir, L.delay, a->mat_mirror,
            L.x_src, L.x_dst, L.x_row, L.x_cls, L.x_delay, L.x_fwd);
        k_double_offsets_fwd<<<sp_blocks(n + 1, 256), 256, 0, sp_counted(st)>>>(n, a->dst_offset, L.x_off);
        PairSet ps{pp, L.x_off, L.x_src, L.x_dst, L.x_row, L.x_cls, L.x_delay, nd, n_class};
        MatCoef coef{L.x_fwd, L.x_cls, a->pair_src, a->pair_in_dir, a->wall_of, a->brdf_index, a->mat_alpha,
                     a->mat_scattering, a->mat_gain, a->pair_fprime, a->pair_unit_len, a->air_attenuation, nb};
        rc = build_groups<T>(n, nb, nt, ps, a->receiver_order, coef, L.C, &n_active, &n_groups, st);
        if (rc != SP_OK) return rc;
        k_material_classes<T><<<sp_blocks(n_class, 128), 128, 0, sp_counted(st)>>>(
            a->n_in_dirs, nb, a->mat_mirror, (T*)L.cdiff, (T*)L.cspec, L.ctarget);
    } else {
        k_pair_class_t<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, a->pair_src, a->pair_in_dir, a->wall_of,
                                                                      a->brdf_index, a->slot_group, a->n_in_dirs,
                                                                      L.cls);
        PairSet ps{p, a->dst_offset, a->pair_src, a->pair_dst, a->pair_out_dir, L.cls, L.delay, nd, n_class};
        FwdCoef coef{a->pair_fprime, a->pair_unit_len, a->air_attenuation, a->wall_of, a->brdf_index,
                     a->slot_scale, a->pair_src, nb};
        rc = build_groups<T>(n, nb, nt, ps, a->receiver_order, coef, L.C, &n_active, &n_groups, st);
        if (rc != SP_OK) return rc;
        if (general) {
            long long nc = (long long)n_class * nd * nb;
            k_convert_t<T><<<sp_blocks(nc, 256), 256, 0, sp_counted(st)>>>(nc, a->class_table, (T*)L.ctab);
            cudaMemsetAsync(L.ctarget, 0xff, (size_t)n_class * sizeof(int32_t), st);  // -1: no mirror lists
        } else {
            long long nc = (long long)n_class * nb;
            k_convert_t<T><<<sp_blocks(nc, 256), 256, 0, sp_counted(st)>>>(nc, a->class_diff, (T*)L.cdiff);
            k_convert_t<T><<<sp_blocks(nc, 256), 256, 0, sp_counted(st)>>>(nc, a->class_spec, (T*)L.cspec);
            cudaMemcpyAsync(L.ctarget, a->class_target, (size_t)n_class * sizeof(int32_t), cudaMemcpyDeviceToDevice,
                            st);
        }
    }
    k_tile_table<<<sp_blocks(n_tiles, 128), 128, 0, sp_counted(st)>>>(n_tiles, n_class, nd, L.C.seg_off,
                                                                      L.ctarget, L.tile_tab);
    const int64_t info[4] = {sig, (int64_t)n_active, (int64_t)n_groups, 0};
    cudaMemcpyAsync(L.info, info, sizeof(info), cudaMemcpyHostToDevice, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;  // `info` is a host local
    }
    if (a->prepare_only) {
        // the batched exchange runs the orders: leave E_0, E_total and the plan (with n_active in info) in ws
        if (reuse) {
            const int64_t info[4] = {sig, (int64_t)n_active, (int64_t)n_groups, 0};
            cudaMemcpyAsync(L.info, info, sizeof(info), cudaMemcpyHostToDevice, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
        }
    }
    if (a->plan_stats) {
        a->plan_stats[0] = n_groups;
        a->plan_stats[1] = (long long)n_tiles * n_class;
        a->plan_stats[2] = pp;
        a->plan_stats[3] = n_tiles;
    }

    if (a->prepare_only) return sp_check_launch();

    // ---- orders
    dim3 mgrid(nb, n);
    size_t msmem = (size_t)2 * n_class * sizeof(T) + (size_t)tile_tab_stride(n_class, nd) * sizeof(int);
    SpEventTimer timer(a->order_ms != nullptr, st);
    SpIntervalTimer scatter_timer(a->scatter_ms != nullptr, a->max_order - k0);
    for (int k = k0 + 1; k <= a->max_order; ++k) {
        scatter_timer.start(st);
        {
            using WL = WsLayout<T>;
            auto kern = [] {
                if constexpr (sizeof(T) == 4)
                    return k_scatter_f32;
                else
                    return k_scatter_f64;
            }();
            if (k == k0 + 1) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WL::kSmem);
            dim3 sgrid(n_active, (nt + WL::kTW - 1) / WL::kTW, nb);
            if (n_active > 0)
                kern<<<sgrid, kWsThreads, WL::kSmem, sp_counted(st)>>>(
                    n_class, nb, nt, rs, lead, pp, L.C.tile_recv, L.C.seg_order, L.C.seg_off, L.C.groups, L.C.wpack,
                    (const T*)L.C.coef, (const T*)eprev, (T*)L.g, L.err);
        }
        // E_total takes the orders in pairs: the first of a pair is deferred
        // and added by the second from the scatter's input rows (E_{k-1},
        // intact until the next mix overwrites them), which saves one read
        // and one write of E_total per pair; a last unpaired order adds alone.
        const bool first_of_pair = (k - k0) % 2 == 1;
        T* et_k = (first_of_pair && k < a->max_order) ? nullptr : etot;
        const T* ea_k = (etot && !first_of_pair) ? eprev : nullptr;
        const int fold = k == a->max_order;  // the last E_total update folds the compensation in
        // the mix's destination rows: the padded ecur, or (partial sums, last order) E_total itself
        T* ek_k = ecur;
        long long rs_k = rs;
        int lead_k = lead;
        if (partial) {
            et_k = nullptr;
            ea_k = nullptr;
            if (k == a->max_order) {
                ek_k = etot;
                rs_k = nt;
                lead_k = 0;
            }
        }
        scatter_timer.stop(st);
        if (general && tensor_mix) {
            const size_t tsmem = tc_smem_bytes(n_class, nd);
            if (k == k0 + 1)
                cudaFuncSetAttribute(k_mix_general_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem);
            k_mix_general_tc<<<mgrid, kTcThreads, tsmem, sp_counted(st)>>>(
                n_class, nd, nb, nt, rs_k, lead_k, L.C.tile_of, L.tile_tab, (const float*)L.ctab, (const float*)L.g,
                (float*)ek_k, (float*)et_k, (const float*)ea_k, comp, L.t_late, fold, L.err);
        } else if (general) {
            const size_t gsmem = mix_general_smem(n_class, nd, sizeof(T));
            if (k == k0 + 1)
                cudaFuncSetAttribute(k_mix_general<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsmem);
            k_mix_general<T><<<mgrid, 128, gsmem, sp_counted(st)>>>(n_class, nd, nb, nt, rs_k, lead_k, L.C.tile_of,
                                                                    L.tile_tab, (const T*)L.ctab, (const T*)L.g, ek_k,
                                                                    et_k, ea_k, comp, L.t_late, fold);
        } else if (sizeof(T) == 4 && nt % 4 == 0)
            (et_k ? k_mix4<true> : k_mix4<false>)<<<mgrid, 128, msmem, sp_counted(st)>>>(
                n_class, nd, nb, nt, rs_k, lead_k, L.C.tile_of, L.tile_tab, (const float*)L.cdiff,
                (const float*)L.cspec, (const float*)L.g, (float*)ek_k, (float*)et_k, (const float*)ea_k, comp,
                L.t_late, fold);
        else
            k_mix<T><<<mgrid, 256, msmem, sp_counted(st)>>>(n_class, nd, nb, nt, rs_k, lead_k, L.C.tile_of,
                                                            L.tile_tab, (const T*)L.cdiff, (const T*)L.cspec,
                                                            (const T*)L.g, ek_k, et_k, ea_k, comp, L.t_late, fold);
        if (partial) {
            const long long ne = (long long)n * nd * nb;
            k_add_e0_t<T><<<sp_blocks(ne, 256), 256, 0, sp_counted(st)>>>(
                n, nd, nb, nt, rs_k, lead_k, a->energy_0_dir, a->distance_0, a->speed_of_sound, a->time_resolution,
                ek_k);
        }
        if (states && (k - k0) % a->states_every == 0)
            copy_rows(states + (size_t)((k - k0) / a->states_every) * e, (size_t)nt, ecur + lead, L.R.rs, nt, L.rows,
                      st);
        T* tmp = eprev;
        eprev = ecur;
        ecur = tmp;
    }
    timer.stop(st);
    rc = sp_check_launch();
    if (rc != SP_OK) return rc;
    int herr = 0;
    cudaMemcpyAsync(&herr, L.err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    if (a->order_ms) *a->order_ms = timer.elapsed_ms();
    if (a->scatter_ms) *a->scatter_ms = scatter_timer.total_ms();
    return herr ? SP_ERR_TIMEOUT : SP_OK;
}

// ------------------------------------------------------------ batched rooms
// Many rooms' exchanges in one persistent launch.  Each room was prepared by
// sp_energy_exchange with prepare_only (E_0, E_total, plan in its own
// workspace); all rooms share D, B, T and the order count K.  The work items
// of order k are every room's scatter items (segment, window; all bands) and
// then every room's mix items (receiver; all bands); a block takes the next item from a
// ticket counter, waits until the item's inputs are complete (a scatter item
// of room r and order k: all mix items of (r, k - 1); a mix item: all scatter
// items of (r, k) and all mix items of (r, k - 1)), runs it and counts it
// done.  With partial sums (every room's partial_sums) a mix item writes
// S_k = M(S_{k-1}) + E_0 (the last order straight into E_total) instead of
// E_k and an E_total update.  Tickets are taken in item order, so every item a block waits for
// was taken earlier by a running block: the launch always progresses.  Waits
// are bounded; a wait that gives up sets the error flag, after which blocks
// only count the remaining items.
struct BatchRoom {
    int n, n_class, n_active, comp_on;
    double c, dt;          // speed of sound, bin width (the source delays of the partial sums)
    const double* e0dir;   // (N, D, B) source energies
    const double* d0;      // (N) source distances
    long long cap, n_scatter, n_mix;  // scatter / mix items per order
    long long s_off, m_off;           // offsets of the room's items in an order's scatter / mix part
    const int32_t* tile_recv;
    const int32_t* seg_order;
    const int64_t* seg_off;
    const Group* groups;
    const uint32_t* wpack;
    const float* coef;
    float* buf0;  // E_0 and the odd orders' inputs (padded rows)
    float* buf1;
    float* g;
    const int32_t* tile_of;
    const int32_t* tile_tab;
    const float* cdiff;
    const float* cspec;
    float* etot;
    uint16_t* comp;
    unsigned long long* done;  // [0]: scatter items done, [1]: mix items done (over all orders)
};

struct BatchShape {
    int nd, nb, nt, K, lead, t_late, windows, n_rooms;
    long long rs, s_total, m_total, per_order, total;
    unsigned wait_limit;
    int force_timeout;
};

constexpr int kErrBatchWait = 5;  // error flag: a batched item's dependency wait gave up

// Bounded wait until *ctr >= target (acquire); false when the limit is reached or another block failed.
// *polls counts the polls that found the count short.
__device__ __forceinline__ bool batch_wait(const unsigned long long* ctr, unsigned long long target, unsigned limit,
                                           const volatile int* err, unsigned long long* polls) {
    for (unsigned it = 0;; ++it) {
        unsigned long long v;
        asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(ctr) : "memory");
        if (v >= target) return true;
        ++*polls;
        if (it >= limit || *err) return false;
        __nanosleep(128);
    }
}

template <int kB, bool kPartial, int kMinBlocks = 2>
__global__ void __launch_bounds__(kWsThreads, kMinBlocks) k_batch_exchange(const BatchRoom* __restrict__ rooms, BatchShape S,
                                                                  unsigned long long* __restrict__ ticket,
                                                                  int* __restrict__ err,
                                                                  unsigned long long* __restrict__ wait_polls) {
    extern __shared__ __align__(128) unsigned char s_dyn[];
    __shared__ long long s_item;
    __shared__ int s_go, s_room;
    int room_hint = 0;  // thread 0: the last item's room (consecutive items mostly share it)
    for (;;) {
        if (threadIdx.x == 0) s_item = (long long)atomicAdd(ticket, 1ull);
        __syncthreads();
        const long long t = s_item;
        if (t >= S.total) break;
        const int k = (int)(t / S.per_order) + 1;
        const long long rem = t % S.per_order;
        const bool scatter = rem < S.s_total;
        const long long pos = scatter ? rem : rem - S.s_total;
        if (threadIdx.x == 0) {
            // the room whose part holds pos: the last one if it still does, else a binary search
            const BatchRoom& H = rooms[room_hint];
            const long long h0 = scatter ? H.s_off : H.m_off, hn = scatter ? H.n_scatter : H.n_mix;
            int lo = room_hint;
            if (pos < h0 || pos >= h0 + hn) {
                lo = 0;
                int hi = S.n_rooms - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if ((scatter ? rooms[mid].s_off : rooms[mid].m_off) <= pos)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
            }
            room_hint = lo;
            s_room = lo;
            const BatchRoom& R = rooms[lo];
            bool ok = *(volatile int*)err == 0;
            const unsigned long long prev_mix = (unsigned long long)(k - 1) * (unsigned long long)R.n_mix;
            unsigned long long polls = 0;
            if (ok && S.force_timeout && t == 0)
                ok = batch_wait(&R.done[1], ~0ull, S.wait_limit, err, &polls);  // test hook
            if (ok) ok = batch_wait(&R.done[1], prev_mix, S.wait_limit, err, &polls);
            if (ok && !scatter)
                ok = batch_wait(&R.done[0], (unsigned long long)k * (unsigned long long)R.n_scatter, S.wait_limit,
                                err, &polls);
            if (polls) atomicAdd(wait_polls, polls);
            if (!ok) atomicCAS(err, 0, kErrBatchWait);
            __threadfence();
            s_go = ok && *(volatile int*)err == 0;
        }
        __syncthreads();
        const BatchRoom& R = rooms[s_room];
        const long long local = pos - (scatter ? R.s_off : R.m_off);
        if (s_go) {
            float* eprev = (k & 1) ? R.buf0 : R.buf1;  // E_{k-1}
            if (scatter) {
                // one (segment, window) item covers every band, in one pipeline
                asm volatile("fence.proxy.async.global;" ::: "memory");  // E_{k-1} was written by generic stores
                scatter_ws<float, kB, true>(R.n_class, S.nb, S.nt, S.rs, S.lead, R.cap, R.tile_recv, R.seg_order,
                                      R.seg_off, R.groups, R.wpack, R.coef, eprev, R.g, err,
                                      (int)(local / S.windows), (int)(local % S.windows), 0, S.nb);
            } else if constexpr (kPartial) {
                // S_k of one receiver, every band: the mix, then E_0 at the source delay of each row
                const bool last = k == S.K;
                float* dst = last ? R.etot : ((k & 1) ? R.buf1 : R.buf0);
                const long long rs = last ? (long long)S.nt : S.rs;
                const int lead = last ? 0 : S.lead;
                mix4_item<8, true, false>(R.n_class, S.nd, S.nb, S.nt, rs, lead, R.tile_of, R.tile_tab, R.cdiff,
                                          R.cspec, R.g, dst, nullptr, nullptr, nullptr, S.t_late, 0, 0, (int)local,
                                          s_dyn, S.nb);
                __syncthreads();  // the rows are written before the source energies are added to them
                const long long dly = (long long)xdiv(xdiv(R.d0[local], R.c), R.dt);
                if (dly >= 0 && dly < S.nt)
                    for (int q = threadIdx.x; q < S.nd * S.nb; q += blockDim.x) {
                        const size_t e = (size_t)local * S.nd * S.nb + q;
                        dst[e * rs + lead + dly] += (float)R.e0dir[e];
                    }
            } else {
                // one receiver item covers every band, the block's threads split over the bands
                float* ecur = (k & 1) ? R.buf1 : R.buf0;
                const bool first_of_pair = (k & 1) == 1;
                float* et = (first_of_pair && k < S.K) ? nullptr : R.etot;
                const float* ea = (R.etot && !first_of_pair) ? eprev : nullptr;
                mix4_item<2, true>(R.n_class, S.nd, S.nb, S.nt, S.rs, S.lead, R.tile_of, R.tile_tab, R.cdiff, R.cspec,
                             R.g, ecur, et, ea, R.comp_on ? R.comp : nullptr, S.t_late, k == S.K, 0, (int)local,
                             s_dyn, S.nb);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();  // the item's results before its count
            atomicAdd(&R.done[scatter ? 0 : 1], 1ull);
        }
    }
}

}  // namespace

extern "C" size_t sp_exchange_batch_workspace(int n_rooms) {
    return sp_align((size_t)(n_rooms > 0 ? n_rooms : 1) * sizeof(BatchRoom)) +
           sp_align((size_t)(n_rooms > 0 ? n_rooms : 1) * 2 * sizeof(unsigned long long)) + 256;
}

extern "C" int sp_exchange_batch(const sp_batch_args* b, void* ws, size_t ws_bytes, void* stream) {
    if (!b || !b->rooms || b->n_rooms < 1 || !ws) return SP_ERR_ARG;
    if (b->window_bins != 1024 && b->window_bins != 512) return SP_ERR_ARG;
    if (ws_bytes < sp_exchange_batch_workspace(b->n_rooms)) return SP_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    const sp_exchange_args* a0 = b->rooms[0].args;
    if (!a0) return SP_ERR_ARG;
    BatchShape S{};
    S.nd = a0->n_dirs;
    S.nb = a0->n_bins;
    S.nt = a0->n_samples;
    S.K = a0->max_order;
    S.n_rooms = b->n_rooms;
    S.wait_limit = b->wait_limit ? b->wait_limit : (1u << 24);
    S.force_timeout = b->force_timeout;
    if (S.nt % 4 != 0 || S.K < 1 || S.nt > 65535) return SP_ERR_UNSUPPORTED;
    const Rows R0 = padded_rows(S.nt);
    S.lead = R0.lead;
    S.rs = (long long)R0.rs;
    S.t_late = late_bin(S.nt);
    const int kTWb = b->window_bins;
    S.windows = (S.nt + kTWb - 1) / kTWb;
    std::vector<BatchRoom> host((size_t)b->n_rooms);
    size_t smem = b->window_bins == 1024 ? WsLayout<float, 32>::kSmem : WsLayout<float, 16>::kSmem;
    long long s_tot = 0, m_tot = 0;
    for (int r = 0; r < b->n_rooms; ++r) {
        const sp_exchange_args* a = b->rooms[r].args;
        if (!a || a->precision != SP_F32 || a->n_dirs != S.nd || a->n_bins != S.nb || a->n_samples != S.nt ||
            a->max_order != S.K || a->state_in || a->states_out || !a->etc_total || a->skip_total ||
            a->n_dir_pairs < 1 || (a->algorithm != SP_EXCHANGE_STRUCTURED && a->algorithm != SP_EXCHANGE_SLOTWISE &&
                                   a->algorithm != SP_EXCHANGE_MATERIAL))
            return SP_ERR_ARG;
        const bool slotwise = a->algorithm == SP_EXCHANGE_SLOTWISE;
        const bool material = a->algorithm == SP_EXCHANGE_MATERIAL || slotwise;
        const int n_class = slotwise ? 1 + S.nd : material ? 1 + a->n_in_dirs : a->n_groups * a->n_in_dirs;
        const Plan L = plan_layout(b->rooms[r].ws, 4, a->n_patches, S.nd, S.nb, S.nt, a->n_dir_pairs, n_class, material,
                                   false);
        if (b->rooms[r].ws_bytes < L.bytes) return SP_ERR_WORKSPACE;
        int64_t info[4] = {0, 0, 0, 0};
        cudaMemcpyAsync(info, L.info, sizeof(info), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
        BatchRoom& R = host[(size_t)r];
        R.n = a->n_patches;
        R.n_class = n_class;
        R.n_active = (int)info[1];
        R.comp_on = a->plain_total ? 0 : 1;
        R.c = a->speed_of_sound;
        R.dt = a->time_resolution;
        R.e0dir = a->energy_0_dir;
        R.d0 = a->distance_0;
        if ((a->partial_sums != 0) != (a0->partial_sums != 0)) return SP_ERR_ARG;  // one form for the launch
        R.cap = material ? 2 * a->n_dir_pairs : a->n_dir_pairs;
        R.n_scatter = (long long)R.n_active * S.windows;  // (segment, window) items, all bands each
        R.n_mix = (long long)R.n;                          // receiver items, all bands each
        if (R.n_scatter < 1) return SP_ERR_ARG;  // a room without pairs inside the histogram: solve it alone
        R.s_off = s_tot;
        R.m_off = m_tot;
        s_tot += R.n_scatter;
        m_tot += R.n_mix;
        R.tile_recv = L.C.tile_recv;
        R.seg_order = L.C.seg_order;
        R.seg_off = L.C.seg_off;
        R.groups = L.C.groups;
        R.wpack = L.C.wpack;
        R.coef = (const float*)L.C.coef;
        R.buf0 = (float*)L.eprev;
        R.buf1 = (float*)L.ecur;
        R.g = (float*)L.g;
        R.tile_of = L.C.tile_of;
        R.tile_tab = L.tile_tab;
        R.cdiff = (const float*)L.cdiff;
        R.cspec = (const float*)L.cspec;
        R.etot = (float*)a->etc_total;
        R.comp = L.comp;
        const size_t msmem =
            (size_t)2 * S.nb * n_class * sizeof(float) + (size_t)tile_tab_stride(n_class, S.nd) * sizeof(int);
        if (msmem > smem) smem = msmem;
    }
    S.s_total = s_tot;
    S.m_total = m_tot;
    S.per_order = s_tot + m_tot;
    S.total = S.per_order * S.K;
    char* q = (char*)ws;
    BatchRoom* d_rooms = (BatchRoom*)q;
    q += sp_align((size_t)b->n_rooms * sizeof(BatchRoom));
    unsigned long long* done = (unsigned long long*)q;
    q += sp_align((size_t)b->n_rooms * 2 * sizeof(unsigned long long));
    unsigned long long* ticket = (unsigned long long*)q;
    int* err = (int*)(q + 64);
    unsigned long long* wait_polls = (unsigned long long*)(q + 128);
    for (int r = 0; r < b->n_rooms; ++r) host[(size_t)r].done = done + 2 * r;
    cudaMemcpyAsync(d_rooms, host.data(), host.size() * sizeof(BatchRoom), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(done, 0, (size_t)b->n_rooms * 2 * sizeof(unsigned long long), st);
    cudaMemsetAsync(q, 0, 256, st);
    int dev = 0, n_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = b->ctas_per_sm > 0 ? b->ctas_per_sm : 1;
    SpEventTimer timer(b->exchange_ms != nullptr, st);
    const bool partial = a0->partial_sums != 0;
    // three blocks per SM (512-bin windows only): an instantiation compiled for that register budget
    auto kern = b->window_bins == 1024 ? (partial ? k_batch_exchange<32, true> : k_batch_exchange<32, false>)
                : per_sm >= 3 ? (partial ? k_batch_exchange<16, true, 3> : k_batch_exchange<16, false, 3>)
                              : (partial ? k_batch_exchange<16, true> : k_batch_exchange<16, false>);
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<n_sm * per_sm, kWsThreads, smem, sp_counted(st)>>>(d_rooms, S, ticket, err, wait_polls);
    timer.stop(st);
    int rc = sp_check_launch();
    if (rc != SP_OK) return rc;
    int herr = 0;
    unsigned long long polls = 0;
    cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&polls, wait_polls, sizeof(polls), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    if (b->exchange_ms) *b->exchange_ms = timer.elapsed_ms();
    if (b->items) *b->items = S.total;
    if (b->wait_polls) *b->wait_polls = (long long)polls;
    return herr ? SP_ERR_TIMEOUT : SP_OK;
}

size_t sp_structured_workspace(int precision, int algorithm, int n_patches, int n_dirs, int n_bins, int n_samples,
                               long long n_dir_pairs, int n_class) {
    int esz = precision == SP_F64 ? 8 : 4;
    return plan_layout(nullptr, esz, n_patches, n_dirs, n_bins, n_samples, n_dir_pairs, n_class,
                       algorithm == SP_EXCHANGE_MATERIAL || algorithm == SP_EXCHANGE_SLOTWISE,
                       algorithm == SP_EXCHANGE_GENERAL)
        .bytes;
}

int sp_run_structured(const sp_exchange_args* a, void* ws, size_t ws_bytes, cudaStream_t st) {
    if (!a->pair_dst) return SP_ERR_ARG;
    if (a->precision == SP_F64) return run_tiled<double>(a, ws, ws_bytes, st);
    return run_tiled<float>(a, ws, ws_bytes, st);
}
