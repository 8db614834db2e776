// FP64 per-band energy check of the exchange.
//
// sp_energy_totals: per band, the sum over patches, outgoing directions and
// bins of E_total (N, D, B, T), FP32 or FP64, accumulated in FP64 in a fixed
// order (partial sums per block, then one block per band).
//
// sp_energy_budget: the same totals predicted without time.  Summing
// RadiosityFast.py:1121-1143 over t, every order maps the energies
// e_{k-1}[i, o, b] = sum_t E_{k-1}[i, o, b, t] linearly:
//   e_k[j, o, b] = sum_{pairs e: i -> j} F'_e exp(-att_b |u_e|) BRDF[slot(i), s_e, o, b] e_{k-1}[i, p2o_e, b]
// (the ff_tilde of RadiosityFast.py:1234-1272), e_0 = E0dir.  The budget is
// sum_k sum_{j,o} e_k[j, o, b].  It equals the histograms' totals exactly
// when no contribution is delayed past the last bin (the reference drops
// those, RadiosityFast.py:1137-1143), so the difference measures rounding
// in a closed room whose histogram outlasts the orders, and otherwise the
// energy beyond the histogram.
#include "common.cuh"
#include "exchange_common.cuh"

namespace {

constexpr int kTotChunks = 1024;  // partial sums per band
constexpr int kTotThreads = 256;

// partial[b * kTotChunks + q] = sum over rows q, q + kTotChunks, ... of row (r, b)'s bins
template <typename T>
__global__ void __launch_bounds__(kTotThreads) k_totals_partial(long long n_rows, int nb, int nt,
                                                                const T* __restrict__ e, double* __restrict__ partial) {
    const int q = blockIdx.x, b = blockIdx.y;
    double acc = 0.0;
    for (long long r = q; r < n_rows; r += kTotChunks) {
        const T* row = e + ((size_t)r * nb + b) * nt;
        for (int t = threadIdx.x; t < nt; t += kTotThreads) acc += (double)row[t];
    }
    __shared__ double s[kTotThreads];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kTotThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[(size_t)b * kTotChunks + q] = s[0];
}

__global__ void __launch_bounds__(kTotThreads) k_totals_final(const double* __restrict__ partial,
                                                              double* __restrict__ out) {
    const int b = blockIdx.x;
    __shared__ double s[kTotThreads];
    double acc = 0.0;
    for (int q = threadIdx.x; q < kTotChunks; q += kTotThreads) acc += partial[(size_t)b * kTotChunks + q];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kTotThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[b] = s[0];
}

// Per directed pair and band: F'_e exp(-att_b |u_e|) (RadiosityFast.py:1255-1262).
__global__ void k_budget_pair_base(long long p, int nb, const double* __restrict__ fprime,
                                   const double* __restrict__ unit_len, const double* __restrict__ att,
                                   double* __restrict__ base) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p) return;
    for (int b = 0; b < nb; ++b) {
        double f = fprime[e];
        if (att) f = f * exp(-att[b] * unit_len[e]);
        base[e * nb + b] = f;
    }
}

// One order of the time-free recursion: one block per destination j, thread
// q over the (o, b) entries of j, pairs in list order.
constexpr int kBudgetThreads = 128;
__global__ void __launch_bounds__(kBudgetThreads) k_budget_order(
    int nd, int nb, const int64_t* __restrict__ dst_off, const int32_t* __restrict__ src,
    const int32_t* __restrict__ out_dir, const int32_t* __restrict__ in_dir, const double* __restrict__ base,
    const int32_t* __restrict__ wall_of, const int32_t* __restrict__ brdf_index, int n_in,
    const double* __restrict__ brdf, const double* __restrict__ e_in, double* __restrict__ e_out) {
    const int j = blockIdx.x;
    const int nq = nd * nb;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};  // (o, b) entries threadIdx.x + 128 r, r < 4
    for (long long e = dst_off[j]; e < dst_off[j + 1]; ++e) {
        const int i = src[e];
        const double* brow = brdf + ((size_t)brdf_index[wall_of[i]] * n_in + in_dir[e]) * nq;
        const double* ein = e_in + ((size_t)i * nd + out_dir[e]) * nb;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int q = threadIdx.x + kBudgetThreads * r;
            if (q < nq) {
                const int b = q % nb;
                acc[r] = fma(base[e * nb + b] * brow[q], ein[b], acc[r]);
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int q = threadIdx.x + kBudgetThreads * r;
        if (q < nq) e_out[(size_t)j * nq + q] = acc[r];
    }
}

// total[b] += sum_{j, o} e[j, o, b] (one block per band, fixed order).
__global__ void __launch_bounds__(kTotThreads) k_budget_sum(int n_rows, int nb, const double* __restrict__ e,
                                                            double* __restrict__ total) {
    const int b = blockIdx.x;
    __shared__ double s[kTotThreads];
    double acc = 0.0;
    for (int r = threadIdx.x; r < n_rows; r += kTotThreads) acc += e[(size_t)r * nb + b];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kTotThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) total[b] += s[0];
}

struct BudgetLayout {
    size_t bytes;
    double* base;  // (P, B)
    double* e[2];  // (N, D, B)
};

BudgetLayout budget_layout(void* p0, int n, int nd, int nb, long long p) {
    BudgetLayout L;
    char* q = (char*)p0;
    auto take = [&](size_t bytes) {
        char* r = q;
        q += sp_align(bytes);
        return (void*)r;
    };
    L.base = (double*)take((size_t)(p > 0 ? p : 1) * nb * 8);
    for (int k = 0; k < 2; ++k) L.e[k] = (double*)take((size_t)n * nd * nb * 8);
    L.bytes = (size_t)(q - (char*)p0);
    return L;
}

}  // namespace

extern "C" {

size_t sp_energy_totals_workspace(int n_bins) { return (size_t)(n_bins > 0 ? n_bins : 1) * kTotChunks * 8; }

int sp_energy_totals(int precision, long long n_rows, int nb, int nt, const void* etot, double* out, void* ws,
                     size_t ws_bytes, void* stream) {
    if (n_rows < 0 || nb < 1 || nt < 1 || !etot || !out || !ws) return SP_ERR_ARG;
    if (precision != SP_F32 && precision != SP_F64) return SP_ERR_ARG;
    if (ws_bytes < sp_energy_totals_workspace(nb)) return SP_ERR_WORKSPACE;
    if (nb > 65535) return SP_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    double* partial = (double*)ws;
    dim3 grid(kTotChunks, nb);
    if (precision == SP_F32)
        k_totals_partial<float><<<grid, kTotThreads, 0, sp_counted(st)>>>(n_rows, nb, nt, (const float*)etot, partial);
    else
        k_totals_partial<double><<<grid, kTotThreads, 0, sp_counted(st)>>>(n_rows, nb, nt, (const double*)etot,
                                                                           partial);
    k_totals_final<<<nb, kTotThreads, 0, sp_counted(st)>>>(partial, out);
    return sp_check_launch();
}

size_t sp_energy_budget_workspace(int n_patches, int n_dirs, int n_bins, long long n_dir_pairs) {
    return budget_layout(nullptr, n_patches, n_dirs, n_bins, n_dir_pairs).bytes;
}

int sp_energy_budget(const sp_exchange_args* a, double* totals, void* ws, size_t ws_bytes, void* stream) {
    if (!a || !totals || !ws) return SP_ERR_ARG;
    const int n = a->n_patches, nd = a->n_dirs, nb = a->n_bins;
    const long long p = a->n_dir_pairs;
    if (n < 1 || nd < 1 || nb < 1 || p < 0 || a->max_order < 0 || !a->energy_0_dir || !a->brdf || !a->wall_of ||
        !a->brdf_index || a->n_in_dirs < 1)
        return SP_ERR_ARG;
    if (p > 0 && (!a->dst_offset || !a->pair_src || !a->pair_out_dir || !a->pair_in_dir || !a->pair_fprime ||
                  !a->pair_unit_len))
        return SP_ERR_ARG;
    if (nd * nb > 4 * kBudgetThreads) return SP_ERR_UNSUPPORTED;
    BudgetLayout L = budget_layout(nullptr, n, nd, nb, p);
    if (ws_bytes < L.bytes) return SP_ERR_WORKSPACE;
    L = budget_layout(ws, n, nd, nb, p);
    cudaStream_t st = (cudaStream_t)stream;
    cudaMemsetAsync(totals, 0, (size_t)nb * sizeof(double), st);
    k_budget_sum<<<nb, kTotThreads, 0, sp_counted(st)>>>(n * nd, nb, a->energy_0_dir, totals);  // order 0
    if (a->max_order < 1 || p == 0) return sp_check_launch();
    k_budget_pair_base<<<sp_blocks(p, 256), 256, 0, sp_counted(st)>>>(p, nb, a->pair_fprime, a->pair_unit_len,
                                                                      a->air_attenuation, L.base);
    const double* e_in = a->energy_0_dir;
    for (int k = 1; k <= a->max_order; ++k) {
        double* e_out = L.e[k & 1];
        k_budget_order<<<n, kBudgetThreads, 0, sp_counted(st)>>>(nd, nb, a->dst_offset, a->pair_src, a->pair_out_dir,
                                                                 a->pair_in_dir, L.base, a->wall_of, a->brdf_index,
                                                                 a->n_in_dirs, a->brdf, e_in, e_out);
        k_budget_sum<<<nb, kTotThreads, 0, sp_counted(st)>>>(n * nd, nb, e_out, totals);
        e_in = e_out;
    }
    return sp_check_launch();
}

}  // extern "C"
