// Tensor-core contraction of the general exchange (SP_EXCHANGE_GENERAL, FP32,
// 32 <= D <= 64, D % 16 == 0, T % 4 == 0):
//   E_k[j, o, b, t] = sum_c tab[c, o, b] G[j, c, b, t]      (c over the classes present in j's tile)
// the receiver-side BRDF contraction of RadiosityFast.py:1127-1143 (ff_tilde
// rows of :1234-1272, factored into the class histograms G by the scatter).
//
// One CTA (4 warps) per (band b, receiver j); it walks j's bins in chunks of
// 128.  Per chunk, one tcgen05 MMA chain computes the 128 x D block
//   D[t, o] = sum_k A[t, k] B[o, k],   A = G[j, cls[k], b, t0 + t],  B = tab[cls[k], o, b]
// with M = 128 (bins), N = D (outgoing directions), K = present classes in
// steps of 8, the accumulator in tensor memory (128 lanes x D columns).
// FP32 accuracy from TF32 operands by the split x = hi + lo, hi = x with its
// 13 low mantissa bits cleared: A B ~ Ahi Bhi + Ahi Blo + Alo Bhi (the
// dropped Alo Blo is about 2^-22 of the product).
//
// Shared-memory operands use the canonical no-swizzle K-major layout (the
// classes contiguous): core matrices of 8 rows x 16 B (4 classes); for A
// (rows = bins) class groups of 4 are 128 B apart (leading byte offset) and
// row groups of 8 are 1 KB apart (stride byte offset, a 32-class chunk); for
// B (rows = outgoing directions) class groups are 128 B apart and row groups
// Kp/4 x 128 B apart.  G is stored bins-contiguous, so staging A transposes
// it: lane l of a warp takes class 4 q + l % 4 and bin 8 r + l / 4, one core
// matrix per warp store.
//
// Thread 0 issues the MMAs; tcgen05.commit arrives on an mbarrier that every
// thread waits on (bounded: on a timeout the CTA records kErrTcWait, waits
// again for the MMAs in flight, frees its tensor memory and leaves).  The
// accumulator is read with tcgen05.ld (warp w: lanes 32w .. 32w + 31, one bin
// per thread, 16 columns per load).
#pragma once
#include "exchange_scatter.cuh"

namespace {

constexpr int kTcM = 128;           // bins per chunk (MMA M)
constexpr int kTcKc = 32;           // classes staged per A chunk (4 MMA k-steps)
constexpr int kTcThreads = 128;     // 4 warps: one per tensor-memory lane quarter
constexpr int kErrTcWait = 4;       // error flag: an MMA completion wait gave up
constexpr size_t kTcSmemMax = 200 * 1024;  // dynamic shared memory limit of a CTA
constexpr uint32_t kTcALbo = 128;                   // A: bytes between class groups of 4
constexpr uint32_t kTcASbo = (kTcKc / 4) * 128;     // A: bytes between bin groups of 8 (1 KB)
constexpr uint32_t kTcAPart = (kTcM / 8) * kTcASbo;  // one of A hi / A lo (16 KB)

__host__ __device__ inline int tc_kpad(int n) { return (n + 7) & ~7; }
// dynamic shared memory of k_mix_general_tc for up to n_class classes and N = nd columns
inline size_t tc_smem_bytes(int n_class, int nd) {
    const size_t b_part = (size_t)nd * tc_kpad(n_class) * 4;
    return 256 + 2 * (size_t)kTcAPart + 2 * b_part + ((size_t)tile_tab_stride(n_class, nd) * 4 + 15) / 16 * 16;
}

__device__ __forceinline__ uint64_t tc_smem_desc(const void* p, uint32_t lbo, uint32_t sbo) {
    const uint64_t a = (uint64_t)smem_addr(p);
    return ((a & 0x3FFFFull) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);  // version 1, no swizzle, base offset 0
}

// kind::tf32 instruction descriptor: D F32 (bits 4-5), A and B TF32 (7-9, 10-12), both K-major (15, 16),
// N >> 3 (17-22), M >> 4 (24-28)
__host__ __device__ constexpr uint32_t tc_idesc(int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | (0u << 15) | (0u << 16) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(kTcM >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xffffe000u); }

// Element offset (in floats) of (bin t, class k) inside one A part, and of (direction o, class k) inside one
// B part with kp classes.
__device__ __forceinline__ uint32_t tc_a_off(int t, int k) {
    return (uint32_t)((t >> 3) * (kTcASbo / 4) + (k >> 2) * (kTcALbo / 4) + (t & 7) * 4 + (k & 3));
}
__device__ __forceinline__ uint32_t tc_b_off(int o, int k, int kp) {
    return (uint32_t)((o >> 3) * (kp / 4) * 32 + (k >> 2) * 32 + (o & 7) * 4 + (k & 3));
}

__global__ void __launch_bounds__(kTcThreads) k_mix_general_tc(
    int n_class, int nd, int nb, int nt, long long rs, int lead, const int32_t* __restrict__ tile_of,
    const int32_t* __restrict__ tab, const float* __restrict__ ctab, const float* __restrict__ g,
    float* __restrict__ ecur, float* __restrict__ etot, const float* __restrict__ eadd, uint16_t* __restrict__ comp,
    int t_late, int fold, int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char s_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(s_raw);            // MMA completion
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(s_raw + 16);    // tensor-memory address
    const int kp_max = tc_kpad(n_class);
    float* a_hi = reinterpret_cast<float*>(s_raw + 256);
    float* a_lo = a_hi + kTcAPart / 4;
    float* b_hi = a_lo + kTcAPart / 4;
    float* b_lo = b_hi + (size_t)nd * kp_max;
    int* s_tab = reinterpret_cast<int*>(b_lo + (size_t)nd * kp_max);

    const int b = blockIdx.x, j = blockIdx.y;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int stride = tile_tab_stride(n_class, nd);
    const int tile = tile_of[j];
    for (int k = threadIdx.x; k < stride; k += kTcThreads) s_tab[k] = tab[(size_t)tile * stride + k];
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    const uint32_t n_cols = nd <= 32 ? 32u : 64u;  // power of two >= N
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(s_tmem)),
                     "r"(n_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *s_tmem;
    const int np = s_tab[0];
    const int* cls = s_tab + 1;
    const int kp = tc_kpad(np);
    // B = tab[cls[k], o, b] split into hi / lo, K-major; zero past np
    for (int q = threadIdx.x; q < nd * kp; q += kTcThreads) {
        const int o = q / kp, k = q % kp;
        const float w = k < np ? ctab[((size_t)cls[k] * nd + o) * nb + b] : 0.0f;
        const float h = tf32_hi(w);
        b_hi[tc_b_off(o, k, kp)] = h;
        b_lo[tc_b_off(o, k, kp)] = w - h;
    }
    const uint32_t idesc = tc_idesc(nd);
    const uint32_t b_sbo = (uint32_t)(kp / 4) * 128u;
    const size_t cstride = (size_t)nb * nt;
    const int nl = nt - t_late;
    const float* gj = g + ((size_t)j * n_class * nb + b) * nt;
    float* ek = ecur + ((size_t)j * nd * nb + b) * rs + lead;
    float* et = etot ? etot + ((size_t)j * nd * nb + b) * nt : nullptr;
    const float* ea = eadd ? eadd + ((size_t)j * nd * nb + b) * rs + lead : nullptr;
    uint16_t* cj = (comp && et) ? comp + ((size_t)j * nd * nb + b) * nl : nullptr;
    unsigned phase = 0;
    bool ok = true;
    for (int t0 = 0; t0 < nt && ok; t0 += kTcM) {
        for (int kc = 0; kc < kp && ok; kc += kTcKc) {
            // stage A = G[cls[kc + k], t0 + t] (hi / lo), transposed to classes-contiguous rows
            // (all of a thread's loads are issued before its stores: 32 loads in flight per thread)
            const int kcn = min(kTcKc, kp - kc);
            constexpr int kPer = kTcM * kTcKc / kTcThreads;
            float xs[kPer];
#pragma unroll
            for (int i = 0; i < kPer; ++i) {
                const int q = threadIdx.x + i * kTcThreads;
                const int k = (q & 3) | (((q >> 5) & 7) << 2);  // class within the chunk (bits 0-1, 5-7)
                const int t = ((q >> 2) & 7) | ((q >> 8) << 3);   // bin within the chunk (bits 2-4, 8-11)
                xs[i] = (k < kcn && kc + k < np && t0 + t < nt) ? __ldg(gj + (size_t)cls[kc + k] * cstride + t0 + t)
                                                                : 0.0f;
            }
#pragma unroll
            for (int i = 0; i < kPer; ++i) {
                const int q = threadIdx.x + i * kTcThreads;
                const int k = (q & 3) | (((q >> 5) & 7) << 2);
                const int t = ((q >> 2) & 7) | ((q >> 8) << 3);
                const float h = tf32_hi(xs[i]);
                const uint32_t off = tc_a_off(t, k);
                a_hi[off] = h;
                a_lo[off] = xs[i] - h;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (threadIdx.x == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                for (int ks = 0; ks < kcn / 8; ++ks) {
                    const uint64_t ah = tc_smem_desc(a_hi + ks * 2 * (kTcALbo / 4), kTcALbo, kTcASbo);
                    const uint64_t al = tc_smem_desc(a_lo + ks * 2 * (kTcALbo / 4), kTcALbo, kTcASbo);
                    const int kg = kc + 8 * ks;  // class index of this k-step within B
                    const uint64_t bh = tc_smem_desc(b_hi + (kg / 4) * 32, 128u, b_sbo);
                    const uint64_t bl = tc_smem_desc(b_lo + (kg / 4) * 32, 128u, b_sbo);
                    tc_mma(tmem, ah, bh, idesc, (kc > 0 || ks > 0) ? 1u : 0u);
                    tc_mma(tmem, ah, bl, idesc, 1u);
                    tc_mma(tmem, al, bh, idesc, 1u);
                }
                tc_commit(bar);
            }
            // every thread waits for the chain (the A buffers are reused by the next chunk); the block agrees
            // on the outcome, so that every thread leaves the loops together
            const bool waited = mbar_wait(bar, phase, err);
            phase ^= 1u;
            if (__syncthreads_or(waited ? 0 : 1)) ok = false;
        }
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // epilogue: thread (warp w, lane l) holds bin t0 + 32 w + l, columns o = 0 .. nd - 1
        const int t = t0 + 32 * warp + lane;
        for (int o0 = 0; o0 < nd; o0 += 16) {
            float v[16];
            tc_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)o0, v);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (t >= nt) continue;
            // the 16 columns' E_total, deferred E_{k-1} and compensation loads first, then the stores
            const bool late = cj != nullptr && t >= t_late;
            float e16[16], a16[16];
            uint16_t c16[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int o = o0 + q;
                e16[q] = et ? et[o * cstride + t] : 0.0f;
                a16[q] = ea ? __ldg(ea + (size_t)o * nb * rs + t) : 0.0f;
                c16[q] = late ? cj[(size_t)o * nb * nl + (t - t_late)] : (uint16_t)0;
            }
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int o = o0 + q;
                ek[(size_t)o * nb * rs + t] = v[q];
                if (!et) continue;
                if (late) {
                    float acc = e16[q], cc = comp_get(c16[q]);
                    kahan_add(acc, cc, ea ? a16[q] + v[q] : v[q]);
                    if (fold) {
                        et[o * cstride + t] = acc - cc;
                    } else {
                        et[o * cstride + t] = acc;
                        cj[(size_t)o * nb * nl + (t - t_late)] = comp_put(cc);
                    }
                } else {
                    et[o * cstride + t] = (ea ? e16[q] + a16[q] : e16[q]) + v[q];
                }
            }
        }
        // the next chunk's MMAs overwrite the accumulator only after every thread has read it
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
    }
    if (!ok) {
        if (threadIdx.x == 0) {
            atomicCAS(err, 0, kErrTcWait);
            // the MMAs of the chain still own the accumulator: wait for them (bounded) before freeing it
            if (!mbar_drain(bar, phase ^ 1u)) atomicCAS(err, 0, kErrDrain);
        }
        __syncthreads();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(n_cols) : "memory");
}

}  // namespace
