// Structured energy exchange (RadiosityFast.py:1073-1145) for BRDF tables
// whose rows are  diff + spec * [o == m]  up to a per-slot, per-band scale:
//   BRDF[slot, s, o, b] = scale[slot, b] * (diff[g, s, b] + spec[g, s, b] * [o == m[g, s]])
// with g = material group of the slot.  This is the form produced by
// brdf.py:100-120 (`create_from_scattering`: s(1-a)/pi everywhere plus the
// mirror term on one outgoing direction), stored times pi.
//
// For a receiver j, pairs of equal class c = (g, s) share their BRDF row, so
//   E_k[j, o, b, t] = sum_c (diff_c + spec_c [o == m_c]) * G_c[t],
//   G_c[t] = sum_{pairs of class c} w_p * E_{k-1}[src_p, p2o_p, b, t - n_p],
//   w_p = F'_p * exp(-att_b |u_p|) * scale[slot(src_p), b].
// A class run costs one multiply-add per pair and bin; each run total is then
// spread once as diff_c (all directions) and spec_c (direction m_c).
#include "common.cuh"
#include "exchange_common.cuh"

namespace {

template <typename T>
struct Cfg;
template <>
struct Cfg<float> {
    static constexpr int R = 2;  // bins per thread
};
template <>
struct Cfg<double> {
    static constexpr int R = 1;
};
constexpr int kThreads = 256;

__global__ void k_delays_s(long long n_dir, const double* __restrict__ dist, double c, double dt,
                           int32_t* __restrict__ delay) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_dir) return;
    delay[e] = (int32_t)(long long)xdiv(xdiv(dist[e], c), dt);
}

__global__ void k_pair_class(long long n_dir, const int32_t* __restrict__ src, const int32_t* __restrict__ in_dir,
                             const int32_t* __restrict__ wall_of, const int32_t* __restrict__ brdf_index,
                             const int32_t* __restrict__ slot_group, int n_in, int32_t* __restrict__ cls) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_dir) return;
    int slot = brdf_index[wall_of[src[e]]];
    cls[e] = slot_group[slot] * n_in + in_dir[e];
}

// Stable counting sort of each destination row by class, one warp per row.
// perm[k] = original entry placed at position k.
__global__ void k_row_sort_by_class(int n, const int64_t* __restrict__ off, const int32_t* __restrict__ cls,
                                    int n_class, int64_t* __restrict__ perm) {
    extern __shared__ int s_hist[];
    int j = blockIdx.x;
    int lane = threadIdx.x;
    long long b = off[j], e = off[j + 1];
    for (int c = lane; c < n_class; c += 32) s_hist[c] = 0;
    __syncwarp();
    for (long long k = b + lane; k < e; k += 32) atomicAdd(&s_hist[cls[k]], 1);
    __syncwarp();
    if (lane == 0) {
        int run = 0;
        for (int c = 0; c < n_class; ++c) {
            int h = s_hist[c];
            s_hist[c] = run;
            run += h;
        }
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

template <typename T>
__global__ void k_gather_pairs(long long n_dir, int nb, const int64_t* __restrict__ perm, const int32_t* __restrict__ src,
                               const int32_t* __restrict__ out_dir, const int32_t* __restrict__ delay,
                               const int32_t* __restrict__ cls, const double* __restrict__ fprime,
                               const double* __restrict__ unit_len, const double* __restrict__ att,
                               const int32_t* __restrict__ wall_of, const int32_t* __restrict__ brdf_index,
                               const double* __restrict__ slot_scale, int32_t* __restrict__ s_src,
                               int32_t* __restrict__ s_odir, int32_t* __restrict__ s_delay,
                               int32_t* __restrict__ s_cls, T* __restrict__ s_w) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_dir) return;
    long long e = perm[k];
    int i = src[e];
    s_src[k] = i;
    s_odir[k] = out_dir[e];
    s_delay[k] = delay[e];
    s_cls[k] = cls[e];
    int slot = brdf_index[wall_of[i]];
    for (int b = 0; b < nb; ++b) {
        double f = fprime[e];
        if (att) f = f * exp(-att[b] * unit_len[e]);
        s_w[k * nb + b] = (T)(f * slot_scale[(size_t)slot * nb + b]);
    }
}

template <typename T>
__global__ void k_init_energy_s(int n, int nd, int nb, int nt, const double* __restrict__ e0dir,
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
    size_t off = (size_t)e * nt + dly;
    T v = (T)e0dir[e];
    etot[off] = v;
    eprev[off] = v;
}

template <typename T>
__global__ void k_convert_s(long long count, const double* __restrict__ in, T* __restrict__ out) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) out[e] = (T)in[e];
}

// One order of the structured exchange.  grid (receiver, time chunk, band).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_exchange_structured(
    int nd, int nb, int nt, const int64_t* __restrict__ off, const int32_t* __restrict__ s_src,
    const int32_t* __restrict__ s_odir, const int32_t* __restrict__ s_delay, const int32_t* __restrict__ s_cls,
    const T* __restrict__ s_w, const T* __restrict__ cdiff, const T* __restrict__ cspec,
    const int32_t* __restrict__ ctarget, const T* __restrict__ eprev, T* __restrict__ ecur, T* __restrict__ etot) {
    constexpr int R = Cfg<T>::R;
    constexpr int CH = kThreads * R;
    extern __shared__ unsigned char s_raw[];
    T* spec = reinterpret_cast<T*>(s_raw);  // [nd][CH]
    const int j = blockIdx.x, b = blockIdx.z;
    const int t0 = blockIdx.y * CH;
    for (int o = 0; o < nd; ++o)
#pragma unroll
        for (int r = 0; r < R; ++r) spec[o * CH + r * kThreads + threadIdx.x] = T(0);
    T diffuse[R], run[R];
#pragma unroll
    for (int r = 0; r < R; ++r) diffuse[r] = run[r] = T(0);
    const size_t row = (size_t)nd * nb * nt;
    int cur = -1;
    const long long e_beg = off[j], e_end = off[j + 1];
    for (long long e = e_beg; e < e_end; ++e) {
        int c = s_cls[e];
        if (c != cur) {
            if (cur >= 0) {
                T u = cdiff[(size_t)cur * nb + b], v = cspec[(size_t)cur * nb + b];
                int m = ctarget[cur];
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    diffuse[r] += u * run[r];
                    if (m >= 0) spec[m * CH + r * kThreads + threadIdx.x] += v * run[r];
                    run[r] = T(0);
                }
            }
            cur = c;
        }
        const int nsh = s_delay[e];
        const T w = s_w[e * nb + b];
        const T* in = eprev + (size_t)s_src[e] * row + ((size_t)s_odir[e] * nb + b) * nt;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            int t = t0 + r * kThreads + threadIdx.x;
            int ts = t - nsh;
            if (t < nt && ts >= 0) run[r] += w * in[ts];
        }
    }
    if (cur >= 0) {
        T u = cdiff[(size_t)cur * nb + b], v = cspec[(size_t)cur * nb + b];
        int m = ctarget[cur];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            diffuse[r] += u * run[r];
            if (m >= 0) spec[m * CH + r * kThreads + threadIdx.x] += v * run[r];
        }
    }
    for (int o = 0; o < nd; ++o) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            int t = t0 + r * kThreads + threadIdx.x;
            if (t < nt) {
                size_t idx = (size_t)j * row + ((size_t)o * nb + b) * nt + t;
                T val = diffuse[r] + spec[o * CH + r * kThreads + threadIdx.x];
                ecur[idx] = val;
                etot[idx] += val;
            }
        }
    }
}

template <typename T>
struct Layout {
    T* eprev;
    T* ecur;
    int32_t* delay;
    int32_t* cls;
    int64_t* perm;
    int32_t* s_src;
    int32_t* s_odir;
    int32_t* s_delay;
    int32_t* s_cls;
    T* s_w;
    T* cdiff;
    T* cspec;
    int* err;
    size_t bytes;
};

template <typename T>
Layout<T> layout(void* base, int n, int nd, int nb, int nt, long long p, int n_class) {
    Layout<T> L;
    char* q = (char*)base;
    size_t e = (size_t)n * nd * nb * nt;
    auto take = [&](size_t bytes) {
        char* r = q;
        q += sp_align(bytes);
        return r;
    };
    L.eprev = (T*)take(e * sizeof(T));
    L.ecur = (T*)take(e * sizeof(T));
    L.delay = (int32_t*)take((size_t)p * 4);
    L.cls = (int32_t*)take((size_t)p * 4);
    L.perm = (int64_t*)take((size_t)p * 8);
    L.s_src = (int32_t*)take((size_t)p * 4);
    L.s_odir = (int32_t*)take((size_t)p * 4);
    L.s_delay = (int32_t*)take((size_t)p * 4);
    L.s_cls = (int32_t*)take((size_t)p * 4);
    L.s_w = (T*)take((size_t)p * nb * sizeof(T));
    L.cdiff = (T*)take((size_t)n_class * nb * sizeof(T));
    L.cspec = (T*)take((size_t)n_class * nb * sizeof(T));
    L.err = (int*)take(16);
    L.bytes = (size_t)(q - (char*)base);
    return L;
}

constexpr int kMaxClasses = 8192;

template <typename T>
int run_structured(const sp_exchange_args* a, void* ws, size_t ws_bytes, cudaStream_t st) {
    const int n = a->n_patches, nd = a->n_dirs, nb = a->n_bins, nt = a->n_samples;
    const long long p = a->n_dir_pairs;
    if (!a->slot_group || !a->slot_scale || !a->class_diff || !a->class_spec || !a->class_target || a->n_groups < 1)
        return SP_ERR_ARG;
    const int n_class = a->n_groups * a->n_in_dirs;
    if (n_class > kMaxClasses) return SP_ERR_UNSUPPORTED;
    Layout<T> L = layout<T>(nullptr, n, nd, nb, nt, p, kMaxClasses);
    if (ws_bytes < L.bytes) return SP_ERR_WORKSPACE;
    L = layout<T>(ws, n, nd, nb, nt, p, kMaxClasses);
    const size_t e = (size_t)n * nd * nb * nt;
    T* etot = (T*)a->etc_total;
    cudaMemsetAsync(L.err, 0, sizeof(int), st);
    cudaMemsetAsync(etot, 0, e * sizeof(T), st);
    cudaMemsetAsync(L.eprev, 0, e * sizeof(T), st);
    long long ne = (long long)n * nd * nb;
    k_init_energy_s<T><<<sp_blocks(ne, 256), 256, 0, st>>>(n, nd, nb, nt, a->energy_0_dir, a->distance_0,
                                                           a->speed_of_sound, a->time_resolution, etot, L.eprev, L.err);
    int herr = 0;
    cudaMemcpyAsync(&herr, L.err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    if (herr) return SP_ERR_RANGE;
    if (a->max_order < 1 || p == 0) return sp_check_launch();

    k_delays_s<<<sp_blocks(p, 256), 256, 0, st>>>(p, a->pair_distance, a->speed_of_sound, a->time_resolution, L.delay);
    k_pair_class<<<sp_blocks(p, 256), 256, 0, st>>>(p, a->pair_src, a->pair_in_dir, a->wall_of, a->brdf_index,
                                                    a->slot_group, a->n_in_dirs, L.cls);
    k_row_sort_by_class<<<n, 32, n_class * sizeof(int), st>>>(n, a->dst_offset, L.cls, n_class, L.perm);
    k_gather_pairs<T><<<sp_blocks(p, 256), 256, 0, st>>>(p, nb, L.perm, a->pair_src, a->pair_out_dir, L.delay, L.cls,
                                                         a->pair_fprime, a->pair_unit_len, a->air_attenuation,
                                                         a->wall_of, a->brdf_index, a->slot_scale, L.s_src, L.s_odir,
                                                         L.s_delay, L.s_cls, L.s_w);
    long long nc = (long long)n_class * nb;
    k_convert_s<T><<<sp_blocks(nc, 256), 256, 0, st>>>(nc, a->class_diff, L.cdiff);
    k_convert_s<T><<<sp_blocks(nc, 256), 256, 0, st>>>(nc, a->class_spec, L.cspec);

    constexpr int CH = kThreads * Cfg<T>::R;
    size_t smem = (size_t)nd * CH * sizeof(T);
    if (smem > 227 * 1024) return SP_ERR_UNSUPPORTED;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_exchange_structured<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(n, (nt + CH - 1) / CH, nb);
    T* eprev = L.eprev;
    T* ecur = L.ecur;
    for (int k = 0; k < a->max_order; ++k) {
        k_exchange_structured<T><<<grid, kThreads, smem, st>>>(nd, nb, nt, a->dst_offset, L.s_src, L.s_odir, L.s_delay,
                                                               L.s_cls, L.s_w, L.cdiff, L.cspec, a->class_target, eprev,
                                                               ecur, etot);
        T* tmp = eprev;
        eprev = ecur;
        ecur = tmp;
    }
    return sp_check_launch();
}

}  // namespace

size_t sp_structured_workspace(int precision, int n_patches, int n_dirs, int n_bins, int n_samples,
                               long long n_dir_pairs, int n_slots, int n_in_dirs) {
    (void)n_slots;
    (void)n_in_dirs;
    if (precision == SP_F64)
        return layout<double>(nullptr, n_patches, n_dirs, n_bins, n_samples, n_dir_pairs, kMaxClasses).bytes;
    return layout<float>(nullptr, n_patches, n_dirs, n_bins, n_samples, n_dir_pairs, kMaxClasses).bytes;
}

int sp_run_structured(const sp_exchange_args* a, void* ws, size_t ws_bytes, cudaStream_t st) {
    if (a->precision == SP_F64) return run_structured<double>(a, ws, ws_bytes, st);
    return run_structured<float>(a, ws, ws_bytes, st);
}
