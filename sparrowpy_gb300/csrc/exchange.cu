// Energy exchange over time histograms and receiver collection.
//
// RadiosityFast.py:1073-1145 `_energy_exchange`: for every order k and every
// directed visible pair (i -> j)
//   E_k[j, :, :, n_ij:] += ff_tilde[i, j][:, :, None] * E_{k-1}[i, p2o[i, j], :, :T-n_ij]
// with n_ij = int(d_ij / c / dt), and E_total = E_0 + sum_k E_k.
// ff_tilde is never materialised: per directed pair we keep F'_ij, the
// incoming-direction index s_ij and the sender's BRDF slot, and form
//   ff_tilde[i, j, o, b] = (F'_ij * exp(-att_b |u_ij|)) * BRDF[slot_i, s_ij, o, b]
// (RadiosityFast.py:1255-1270) when it is needed.
//
// Two exchange kernels share this entry point:
//  * dense      - one CTA per (receiver j, band b, 256-bin time chunk), one
//                 thread per bin, all D outgoing directions accumulated in
//                 shared memory.  Any BRDF table.  D FMAs per pair and bin.
//  * structured - for BRDF rows of the form  diff + spec * [o == m]  (the
//                 diffuse-plus-mirror tables of brdf.py:100-120): the pairs of
//                 a receiver are grouped by class (material group, s_ij) and a
//                 class run costs one FMA per pair and bin; the run total is
//                 then spread as diff_c (all o) and spec_c (o = m_c).
//                 Implemented in exchange_structured.cu.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "exchange_common.cuh"

namespace {

constexpr int kChunk = 256;

template <typename T>
__global__ void k_init_energy(int n, int nd, int nb, int nt, const double* __restrict__ e0dir,
                              const double* __restrict__ d0, double c, double dt, T* __restrict__ etot,
                              T* __restrict__ eprev, int* __restrict__ err) {
    // RadiosityFast.py:1037-1070: E[i, :, :, int(d0/c/dt)] += E0dir[i]
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)n * nd * nb;
    if (e >= total) return;
    int i = (int)(e / ((long long)nd * nb));
    long long dly = (long long)xdiv(xdiv(d0[i], c), dt);
    if (dly < 0 || dly >= nt) {
        atomicExch(err, 1);
        return;
    }
    size_t off = (size_t)e * nt + dly;
    T v = (T)e0dir[e];
    etot[off] = v;
    if (eprev) eprev[off] = v;
}

__global__ void k_pair_delays(long long n_dir, const double* __restrict__ dist, double c, double dt,
                              int32_t* __restrict__ delay) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_dir) return;
    // RadiosityFast.py:1135-1136: int(distance / speed_of_sound / dt)
    double q = xdiv(xdiv(dist[e], c), dt);
    delay[e] = (int32_t)(long long)q;
}

// Per directed pair and band: F'_ij * exp(-att_b * |u_ij|)  (RadiosityFast.py:1259-1262)
template <typename T>
__global__ void k_pair_base(long long n_dir, int nb, const double* __restrict__ fprime,
                            const double* __restrict__ unit_len, const double* __restrict__ att, T* __restrict__ base) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_dir) return;
    for (int b = 0; b < nb; ++b) {
        double f = fprime[e];
        if (att) f = f * exp(-att[b] * unit_len[e]);
        base[e * nb + b] = (T)f;
    }
}

template <typename T>
__global__ void k_convert(long long count, const double* __restrict__ in, T* __restrict__ out) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) out[e] = (T)in[e];
}

// Dense exchange for one order.  grid (time chunks, bands, receivers).
template <typename T>
__global__ void __launch_bounds__(kChunk) k_exchange_dense(
    int n, int nd, int nb, int nt, const int64_t* __restrict__ dst_off, const int32_t* __restrict__ src,
    const int32_t* __restrict__ out_dir, const int32_t* __restrict__ in_dir, const int32_t* __restrict__ delay,
    const T* __restrict__ base, const int32_t* __restrict__ slot_of_src, int n_in, const T* __restrict__ brdf,
    const T* __restrict__ eprev, T* __restrict__ ecur, T* __restrict__ etot) {
    extern __shared__ unsigned char s_raw[];
    T* acc = reinterpret_cast<T*>(s_raw);  // [nd][kChunk]
    int j = blockIdx.z, b = blockIdx.y;
    int t = blockIdx.x * kChunk + threadIdx.x;
    for (int o = 0; o < nd; ++o) acc[o * kChunk + threadIdx.x] = T(0);
    const size_t row = (size_t)nd * nb * nt;
    for (long long e = dst_off[j]; e < dst_off[j + 1]; ++e) {
        int i = src[e];
        int nsh = delay[e];
        T x = T(0);
        if (t < nt && t >= nsh) x = eprev[(size_t)i * row + ((size_t)out_dir[e] * nb + b) * nt + (t - nsh)];
        T fb = base[e * nb + b];
        const T* brow = brdf + ((size_t)slot_of_src[i] * n_in + in_dir[e]) * nd * nb + b;
        for (int o = 0; o < nd; ++o) acc[o * kChunk + threadIdx.x] += (fb * brow[(size_t)o * nb]) * x;
    }
    if (t < nt) {
        for (int o = 0; o < nd; ++o) {
            size_t off = (size_t)j * row + ((size_t)o * nb + b) * nt + t;
            T v = acc[o * kChunk + threadIdx.x];
            ecur[off] = v;
            etot[off] += v;
        }
    }
}

template <typename T>
size_t exchange_dense_workspace(int n, int nd, int nb, int nt, long long n_dir, int n_slots, int n_in) {
    size_t e = (size_t)n * nd * nb * nt * sizeof(T);
    size_t w = 2 * sp_align(e);
    w += sp_align((size_t)n_dir * sizeof(int32_t));                     // delays
    w += sp_align((size_t)n_dir * nb * sizeof(T));                      // pair base factors
    w += sp_align((size_t)n_slots * n_in * nd * nb * sizeof(T));        // brdf in T
    w += sp_align((size_t)n * sizeof(int32_t));                         // slot per patch
    w += sp_align(sizeof(int) * 4);                                     // error flag
    return w;
}

__global__ void k_slot_of_patch(int n, const int32_t* __restrict__ wall_of, const int32_t* __restrict__ brdf_index,
                                int32_t* __restrict__ slot) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) slot[i] = brdf_index[wall_of[i]];
}

template <typename T>
int run_exchange_dense(const sp_exchange_args* a, void* ws, size_t ws_bytes, cudaStream_t st) {
    const int n = a->n_patches, nd = a->n_dirs, nb = a->n_bins, nt = a->n_samples;
    const long long n_dir = a->n_dir_pairs;
    if (ws_bytes < exchange_dense_workspace<T>(n, nd, nb, nt, n_dir, a->n_slots, a->n_in_dirs)) return SP_ERR_WORKSPACE;
    size_t e = (size_t)n * nd * nb * nt;
    char* p = (char*)ws;
    T* eprev = (T*)p;
    p += sp_align(e * sizeof(T));
    T* ecur = (T*)p;
    p += sp_align(e * sizeof(T));
    int32_t* delay = (int32_t*)p;
    p += sp_align((size_t)n_dir * sizeof(int32_t));
    T* base = (T*)p;
    p += sp_align((size_t)n_dir * nb * sizeof(T));
    T* brdf = (T*)p;
    p += sp_align((size_t)a->n_slots * a->n_in_dirs * nd * nb * sizeof(T));
    int32_t* slot = (int32_t*)p;
    p += sp_align((size_t)n * sizeof(int32_t));
    int* err = (int*)p;

    T* etot = (T*)a->etc_total;
    cudaMemsetAsync(err, 0, sizeof(int), st);
    cudaMemsetAsync(etot, 0, e * sizeof(T), st);
    cudaMemsetAsync(eprev, 0, e * sizeof(T), st);
    long long ne = (long long)n * nd * nb;
    if (ne > 0)
        k_init_energy<T><<<sp_blocks(ne, 256), 256, 0, sp_counted(st)>>>(n, nd, nb, nt, a->energy_0_dir, a->distance_0,
                                                             a->speed_of_sound, a->time_resolution, etot, eprev, err);
    int hrr = 0;
    cudaMemcpyAsync(&hrr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    if (hrr) return SP_ERR_RANGE;
    if (a->max_order < 1 || n_dir == 0) return sp_check_launch();

    k_pair_delays<<<sp_blocks(n_dir, 256), 256, 0, sp_counted(st)>>>(n_dir, a->pair_distance, a->speed_of_sound,
                                                          a->time_resolution, delay);
    k_pair_base<T><<<sp_blocks(n_dir, 256), 256, 0, sp_counted(st)>>>(n_dir, nb, a->pair_fprime, a->pair_unit_len,
                                                          a->air_attenuation, base);
    long long nbr = (long long)a->n_slots * a->n_in_dirs * nd * nb;
    k_convert<T><<<sp_blocks(nbr, 256), 256, 0, sp_counted(st)>>>(nbr, a->brdf, brdf);
    k_slot_of_patch<<<sp_blocks(n, 128), 128, 0, sp_counted(st)>>>(n, a->wall_of, a->brdf_index, slot);

    size_t smem = (size_t)nd * kChunk * sizeof(T);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_exchange_dense<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((nt + kChunk - 1) / kChunk, nb, n);
    SpEventTimer timer(a->order_ms != nullptr, st);
    for (int k = 0; k < a->max_order; ++k) {
        k_exchange_dense<T><<<grid, kChunk, smem, sp_counted(st)>>>(n, nd, nb, nt, a->dst_offset, a->pair_src, a->pair_out_dir,
                                                        a->pair_in_dir, delay, base, slot, a->n_in_dirs, brdf, eprev,
                                                        ecur, etot);
        T* tmp = eprev;
        eprev = ecur;
        ecur = tmp;
    }
    timer.stop(st);
    int rc = sp_check_launch();
    if (rc == SP_OK && a->order_ms) {
        if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
        *a->order_ms = timer.elapsed_ms();
    }
    return rc;
}

// RadiosityFast.py:686-752 + :1148-1185 for one receiver: per patch k the
// factor r_k * exp(-att_b d_k) and the circular shift ceil(d_k / c / dt).
__global__ void k_collect_coef(int n, int nb, int nt, const double* __restrict__ rfac, const double* __restrict__ dist,
                               double c, double dt, const double* __restrict__ att, double* __restrict__ coef,
                               int32_t* __restrict__ shift) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double q = ceil(xdiv(xdiv(dist[k], c), dt));
    long long s = (long long)q;
    s %= nt;
    if (s < 0) s += nt;
    shift[k] = (int32_t)s;
    for (int b = 0; b < nb; ++b) coef[(size_t)k * nb + b] = rfac[k];
    if (att)
        for (int b = 0; b < nb; ++b) coef[(size_t)k * nb + b + (size_t)n * nb] = exp(-att[b] * dist[k]);
    else
        for (int b = 0; b < nb; ++b) coef[(size_t)k * nb + b + (size_t)n * nb] = 1.0;
}

// Patchwise histogram: out[k, b, (t + s_k) % T] = (E[k, ridx_k, b, t] * r_k) * a_kb
template <typename T>
__global__ void k_collect_patchwise(int n, int nd, int nb, int nt, const T* __restrict__ etot,
                                    const int32_t* __restrict__ ridx, const double* __restrict__ coef,
                                    const int32_t* __restrict__ shift, double* __restrict__ out) {
    int k = blockIdx.z, b = blockIdx.y;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    double v = (double)etot[(((size_t)k * nd + ridx[k]) * nb + b) * nt + t];
    double r = coef[(size_t)k * nb + b], a = coef[(size_t)n * nb + (size_t)k * nb + b];
    int dst = t + shift[k];
    if (dst >= nt) dst -= nt;
    out[((size_t)k * nb + b) * nt + dst] = (v * r) * a;
}

// Mono histogram: sum over patches of the patchwise histogram (RadiosityFast.py:592).
// A block holds 32 bins of one band; its kMonoWarps warps split the patches
// (warp w takes k = w, w + kMonoWarps, ...) and their partial sums are added
// in warp order through shared memory, so the result does not depend on
// scheduling.  Each term is (E * r_k) * a_kb, added with one FP64 fma: the
// terms are non-negative, so the sum of N of them is within N * 2^-53 of
// exact (7e-13 relative at N = 6000).
constexpr int kMonoWarps = 8;
template <typename T>
__global__ void __launch_bounds__(kMonoWarps * 32) k_collect_mono(int n, int nd, int nb, int nt,
                                                                  const T* __restrict__ etot,
                                                                  const int32_t* __restrict__ ridx,
                                                                  const double* __restrict__ coef,
                                                                  const int32_t* __restrict__ shift,
                                                                  double* __restrict__ out) {
    __shared__ double part[kMonoWarps][32];
    const int b = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int t = blockIdx.x * 32 + lane;
    double s = 0.0;
    if (t < nt) {
#pragma unroll 4
        for (int k = warp; k < n; k += kMonoWarps) {
            int src_t = t - shift[k];
            if (src_t < 0) src_t += nt;
            const double v = (double)etot[(((size_t)k * nd + ridx[k]) * nb + b) * nt + src_t];
            s = fma(v * coef[(size_t)k * nb + b], coef[(size_t)n * nb + (size_t)k * nb + b], s);
        }
    }
    part[warp][lane] = s;
    __syncthreads();
    if (warp == 0 && t < nt) {
        double tot = part[0][lane];
        for (int w = 1; w < kMonoWarps; ++w) tot += part[w][lane];
        out[(size_t)b * nt + t] = tot;
    }
}

template <typename T>
int run_collect(int n, int nd, int nb, int nt, const void* etot, const int32_t* ridx, const double* rfac,
                const double* dist, double c, double dt, const double* att, double* patchwise, double* mono, void* ws,
                size_t ws_bytes, cudaStream_t st) {
    size_t need = sp_align((size_t)n * nb * 2 * sizeof(double)) + sp_align((size_t)n * sizeof(int32_t));
    if (ws_bytes < need) return SP_ERR_WORKSPACE;
    double* coef = (double*)ws;
    int32_t* shift = (int32_t*)((char*)ws + sp_align((size_t)n * nb * 2 * sizeof(double)));
    k_collect_coef<<<sp_blocks(n, 128), 128, 0, sp_counted(st)>>>(n, nb, nt, rfac, dist, c, dt, att, coef, shift);
    if (patchwise) {
        dim3 g((nt + 255) / 256, nb, n);
        k_collect_patchwise<T><<<g, 256, 0, sp_counted(st)>>>(n, nd, nb, nt, (const T*)etot, ridx, coef, shift, patchwise);
    }
    if (mono) {
        dim3 g((nt + 31) / 32, nb);
        k_collect_mono<T><<<g, kMonoWarps * 32, 0, sp_counted(st)>>>(n, nd, nb, nt, (const T*)etot, ridx, coef, shift,
                                                                    mono);
    }
    return sp_check_launch();
}

}  // namespace

extern "C" {

size_t sp_energy_exchange_workspace(int precision, int algorithm, int n_patches, int n_dirs, int n_bins,
                                    int n_samples, long long n_dir_pairs, int n_slots, int n_in_dirs,
                                    int n_classes) {
    if (algorithm == SP_EXCHANGE_STRUCTURED || algorithm == SP_EXCHANGE_MATERIAL || algorithm == SP_EXCHANGE_SLOTWISE ||
        algorithm == SP_EXCHANGE_GENERAL)
        return sp_structured_workspace(precision, algorithm, n_patches, n_dirs, n_bins, n_samples, n_dir_pairs,
                                       n_classes);
    if (precision == SP_F64)
        return exchange_dense_workspace<double>(n_patches, n_dirs, n_bins, n_samples, n_dir_pairs, n_slots, n_in_dirs);
    return exchange_dense_workspace<float>(n_patches, n_dirs, n_bins, n_samples, n_dir_pairs, n_slots, n_in_dirs);
}

int sp_energy_exchange(const sp_exchange_args* a, void* ws, size_t ws_bytes, void* stream) {
    if (!a) return SP_ERR_ARG;
    if (a->n_patches < 0 || a->n_dirs < 1 || a->n_bins < 1 || a->n_samples < 1 || a->n_dir_pairs < 0 ||
        a->n_slots < 1 || a->n_in_dirs < 1 || !(a->speed_of_sound > 0) || !(a->time_resolution > 0))
        return SP_ERR_ARG;
    if (a->precision != SP_F32 && a->precision != SP_F64) return SP_ERR_ARG;
    if (a->n_patches == 0) return SP_OK;
    if (!a->energy_0_dir || !a->distance_0 || !a->etc_total || !ws || !a->wall_of || !a->brdf_index || !a->brdf)
        return SP_ERR_ARG;
    if (a->n_dir_pairs > 0 && (!a->dst_offset || !a->pair_src || !a->pair_out_dir || !a->pair_in_dir ||
                               !a->pair_distance || !a->pair_fprime || !a->pair_unit_len))
        return SP_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (a->algorithm == SP_EXCHANGE_STRUCTURED || a->algorithm == SP_EXCHANGE_MATERIAL ||
        a->algorithm == SP_EXCHANGE_SLOTWISE || a->algorithm == SP_EXCHANGE_GENERAL)
        return sp_run_structured(a, ws, ws_bytes, st);
    if (a->precision == SP_F64) return run_exchange_dense<double>(a, ws, ws_bytes, st);
    return run_exchange_dense<float>(a, ws, ws_bytes, st);
}

size_t sp_collect_workspace(int n_patches, int n_bins) {
    return sp_align((size_t)n_patches * n_bins * 2 * sizeof(double)) + sp_align((size_t)n_patches * sizeof(int32_t));
}

int sp_collect_receiver(int precision, int n, int nd, int nb, int nt, const void* etot, const int32_t* ridx,
                        const double* rfac, const double* dist, double c, double dt, const double* att,
                        double* patchwise, double* mono, void* ws, size_t ws_bytes, void* stream) {
    if (n < 0 || nd < 1 || nb < 1 || nt < 1 || !(c > 0) || !(dt > 0)) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    if (!etot || !ridx || !rfac || !dist || !ws || (!patchwise && !mono)) return SP_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == SP_F64)
        return run_collect<double>(n, nd, nb, nt, etot, ridx, rfac, dist, c, dt, att, patchwise, mono, ws, ws_bytes, st);
    if (precision == SP_F32)
        return run_collect<float>(n, nd, nb, nt, etot, ridx, rfac, dist, c, dt, att, patchwise, mono, ws, ws_bytes, st);
    return SP_ERR_ARG;
}

}  // extern "C"
