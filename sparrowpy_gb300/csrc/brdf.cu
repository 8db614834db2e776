// Structure analysis of BRDF tables for the structured exchange.
//
// A table row brdf[s, i, :, b] (slot s, incoming direction i, band b) is
// "diffuse plus one mirror term" when every outgoing direction shares one
// value (diff) except at most one direction m, the same m for every band of
// the row.  create_from_scattering tables (sparrowpy/brdf.py:8-130) have
// this form; the exchange then needs one histogram per incoming-direction
// class instead of one per outgoing direction.  diff is the median over the
// outgoing directions (the common value when at most one deviates), and a
// value deviates when it differs from diff by more than rel_tol * max|brdf|.
#include "common.cuh"

namespace {

// max |v| over the table, as the bit pattern of a non-negative double
// (ordered like the value, so atomicMax on the bits is a max on the values)
__global__ void k_brdf_absmax(long long total, const double* __restrict__ brdf, unsigned long long* __restrict__ gmax) {
    double m = 0.0;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x)
        m = fmax(m, fabs(brdf[e]));
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) atomicMax(gmax, (unsigned long long)__double_as_longlong(m));
}

// k-th smallest (0-based) of v[0..n) by counting: the value x = v[a] with
// #{v < x} <= k < #{v <= x} (ties included, as a sort would place them).
__device__ double kth_smallest(const double* v, int stride, int n, int k) {
    for (int a = 0; a < n; ++a) {
        const double x = v[(size_t)a * stride];
        int lt = 0, le = 0;
        for (int c = 0; c < n; ++c) {
            const double y = v[(size_t)c * stride];
            lt += y < x;
            le += y <= x;
        }
        if (lt <= k && k < le) return x;
    }
    return v[0];  // not reached for finite values
}

// One thread per row (s, i): diff and spec per band, target, slot scale.
__global__ void k_brdf_rows(int n_slots, int n_in, int n_out, int nb, const double* __restrict__ brdf,
                            double rel_tol, const unsigned long long* __restrict__ gmax, double* __restrict__ diff,
                            double* __restrict__ spec, int32_t* __restrict__ target,
                            unsigned long long* __restrict__ scale_bits, int* __restrict__ n_irregular) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (long long)n_slots * n_in) return;
    const int s = (int)(r / n_in);
    const double tol = rel_tol * fmax(__longlong_as_double((long long)*gmax), 1e-300);
    const double* row = brdf + (size_t)r * n_out * nb;  // row[o * nb + b]
    double* d = diff + (size_t)r * nb;
    int m = -1;
    bool irregular = false;
    for (int b = 0; b < nb; ++b) {
        double db;
        if (n_out >= 3) db = kth_smallest(row + b, nb, n_out, n_out / 2);
        else db = row[b];
        d[b] = db;
        double mx = 0.0;
        for (int o = 0; o < n_out; ++o) {
            const double v = row[(size_t)o * nb + b];
            mx = fmax(mx, fabs(v));
            if (fabs(v - db) > tol) {
                if (m < 0) m = o;
                else if (m != o) irregular = true;
            }
        }
        atomicMax(&scale_bits[(size_t)s * nb + b], (unsigned long long)__double_as_longlong(mx));
    }
    target[r] = m;
    for (int b = 0; b < nb; ++b) spec[(size_t)r * nb + b] = m >= 0 ? row[(size_t)m * nb + b] - d[b] : 0.0;
    if (irregular) atomicAdd(n_irregular, 1);
}

}  // namespace

extern "C" {

size_t sp_brdf_structure_workspace(void) { return 256; }

int sp_brdf_structure(int n_slots, int n_in, int n_out, int nb, const double* brdf, double rel_tol, double* diff,
                      double* spec, int32_t* target, double* scale, int* n_irregular, void* ws, size_t ws_bytes,
                      void* stream) {
    if (n_slots < 0 || n_in < 0 || n_out < 1 || nb < 1 || !(rel_tol >= 0.0)) return SP_ERR_ARG;
    if (!n_irregular || !ws) return SP_ERR_ARG;
    if (ws_bytes < sp_brdf_structure_workspace()) return SP_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    cudaMemsetAsync(n_irregular, 0, sizeof(int), st);
    const long long rows = (long long)n_slots * n_in;
    if (rows == 0) return SP_OK;
    if (!brdf || !diff || !spec || !target || !scale) return SP_ERR_ARG;
    unsigned long long* gmax = (unsigned long long*)ws;
    cudaMemsetAsync(gmax, 0, sizeof(unsigned long long), st);
    cudaMemsetAsync(scale, 0, (size_t)n_slots * nb * sizeof(double), st);
    const long long total = rows * n_out * nb;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_brdf_absmax<<<(unsigned)blocks, 256, 0, sp_counted(st)>>>(total, brdf, gmax);
    k_brdf_rows<<<sp_blocks(rows, 128), 128, 0, sp_counted(st)>>>(n_slots, n_in, n_out, nb, brdf, rel_tol, gmax, diff,
                                                                  spec, target, (unsigned long long*)scale,
                                                                  n_irregular);
    return sp_check_launch();
}

}  // extern "C"
