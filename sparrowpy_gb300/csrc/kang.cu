// Kang radiosity (sparrowpy/classes/RadiosityKang.py) in FP64: closed-form
// source energy and form factors for axis-aligned rectangular patches, the
// delayed energy exchange between walls per order, and the energy at a
// receiver.  Arithmetic follows the reference's evaluation order with
// unfused operations (x* helpers), so results agree with it up to the last
// bit of exp / atan / pow.  Histograms are E (n_bins, n_orders, n, nt) per
// wall, as the reference's E_matrix.
//
// The directional variant (RadiosityKang.py:500-810) keeps one histogram per
// outgoing direction: E (n_bins, n_orders, n, n_dirs, nt) on the device (the
// reference's E_matrix is (n_bins, n_orders, n, nt, n_dirs); the host
// transposes).  Every kernel is templated on kDir; with kDir false, n_dirs is
// 1 and the arithmetic is the plain solver's.  The directional factors come
// from the receiving wall's table scat (n_src_dirs, n_dirs, n_bins), indexed
// per patch (init) or per (receiver, source) pair (exchange) by the nearest
// source direction, which the host finds as the reference does.
#include "common.cuh"
#include "exchange_common.cuh"

namespace {

enum { kKangErrIndex = 1, kKangErrDelay = 2 };  // IndexError (init), ValueError (_add_delay)

__device__ __forceinline__ double sq(double a) { return xmul(a, a); }

// np.linalg.norm(a - b) for 3-vectors.
__device__ __forceinline__ double dist3(const double* a, const double* b) {
    const double d[3] = {xsub(a[0], b[0]), xsub(a[1], b[1]), xsub(a[2], b[2])};
    return xnorm3(d);
}

// RadiosityKang.py:812-849 `_init_energy_exchange` without the per-band
// constant: |sin_phi_delta - sin_phi| and beta.
__device__ void kang_init_geom(double dl, double dm, double dn, double dd_l, double dd_m, double sx, double sy,
                               double sz, double* dphi, double* beta_out) {
    const double half_l = xdiv(dd_l, 2.0), half_m = xdiv(dd_m, 2.0);
    const double a = xsub(xadd(dl, half_l), sx);
    const double sin_phi_delta = xdiv(a, __dsqrt_rn(xadd(xadd(sq(a), sq(xsub(dm, sy))), sq(xsub(dn, sz)))));
    const double k_phi = (xsub(dl, half_l) <= sx && sx <= xadd(dl, half_l)) ? -1.0 : 1.0;
    const double b = xsub(xsub(dl, half_l), sx);
    double sin_phi = xdiv(xmul(k_phi, b), __dsqrt_rn(xadd(xadd(sq(b), sq(xsub(dm, sy))), sq(xsub(dn, sz)))));
    if (xsub(sin_phi_delta, sin_phi) < 1e-11) sin_phi = -sin_phi;
    const double plus = atan(fabs(xdiv(xsub(xadd(dm, half_m), sy), fabs(sz))));
    const double minus = atan(fabs(xdiv(xsub(xsub(dm, half_m), sy), fabs(sz))));
    const double k_beta = (xsub(dm, half_m) <= sy && sy <= xadd(dm, half_m)) ? -1.0 : 1.0;
    *beta_out = fabs(xsub(plus, xmul(k_beta, minus)));
    *dphi = fabs(xsub(sin_phi_delta, sin_phi));
}

// RadiosityKang.py:141-207 `init_energy_exchange`, one patch per thread:
// E[b, 0, i, delay] += energy_b.
// Directional (RadiosityKang.py:629-671): E[b, 0, i, d, delay] = energy_b *
// |scat[idx_i, d, b]|, the tiled histogram times the directional factors.
template <bool kDir>
__global__ void k_kang_init(int n, const double* __restrict__ centers, const double* __restrict__ sizes,
                            const double* __restrict__ normal, const double* __restrict__ src, double power, int nb,
                            const double* __restrict__ absorption, const double* __restrict__ attenuation, double c,
                            double fs, int n_orders, int nt, int n_dirs, const double* __restrict__ scat,
                            const int32_t* __restrict__ scat_idx, double* __restrict__ E, int* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s[3] = {src[0], src[1], src[2]};
    double r[3] = {centers[3 * i], centers[3 * i + 1], centers[3 * i + 2]};
    const double distance = dist3(r, s);
    const long long delay = (long long)xmul(xdiv(distance, c), fs);
    int ax, idx[3];
    if (fabs(normal[2]) > 0.99) {
        ax = 2, idx[0] = 0, idx[1] = 1, idx[2] = 2;
    } else if (fabs(normal[1]) > 0.99) {
        ax = 1, idx[0] = 2, idx[1] = 0, idx[2] = 1;
    } else {  // |normal[0]| > 0.99, checked by the host
        ax = 0, idx[0] = 1, idx[1] = 2, idx[2] = 0;
    }
    const double off = r[ax];
    s[ax] = fabs(xsub(s[ax], off));
    r[ax] = fabs(xsub(r[ax], off));
    const double* sz = sizes + 3 * i;
    double dphi, beta;
    kang_init_geom(r[idx[0]], r[idx[1]], r[idx[2]], sz[idx[0]], sz[idx[1]], s[idx[0]], s[idx[1]], s[idx[2]], &dphi,
                   &beta);
    if (delay < 0 || delay >= nt) {
        atomicCAS(err, 0, kKangErrIndex);
        return;
    }
    for (int b = 0; b < nb; ++b) {
        const double cst = xmul(xmul(power, xsub(1.0, absorption[b])), exp(xmul(-attenuation[b], distance)));
        const double e = xdiv(xmul(xmul(cst, dphi), beta), 4 * SP_PI);
        if (!kDir) {
            double* p = E + (((size_t)b * n_orders) * n + i) * nt + delay;
            *p = xadd(*p, e);
        } else {
            for (int d = 0; d < n_dirs; ++d) {
                double* p = E + ((((size_t)b * n_orders) * n + i) * n_dirs + d) * nt + delay;
                *p = xmul(xadd(*p, e), fabs(scat[((size_t)scat_idx[i] * n_dirs + d) * nb + b]));
            }
        }
    }
}

// In-plane axes of a patch by its normal, in the reference's order of tests
// (RadiosityKang.py:301-322); returned as a bit set.
__device__ __forceinline__ int plane_axes(const double* nrm) {
    if (fabs(nrm[0]) > 1e-5) return (1 << 2) | (1 << 1);
    if (fabs(nrm[1]) > 1e-5) return (1 << 2) | (1 << 0);
    return (1 << 0) | (1 << 1);
}
__device__ __forceinline__ int only_axis(int bits) { return bits == 1 ? 0 : (bits == 2 ? 1 : 2); }

// RadiosityKang.py:269-408 `calculate_form_factor`: one (source patch,
// receiver column) per thread; ff is (n_src, n_rcv) row-major.
__global__ void k_kang_ff(int n_src, const double* __restrict__ src_c, const double* __restrict__ src_n,
                          const double* __restrict__ src_wc, int n_rcv, const double* __restrict__ rcv_c,
                          const double* __restrict__ rcv_n, const double* __restrict__ rcv_wc, double dd,
                          double* __restrict__ ff) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)n_src * n_rcv) return;
    const int i = (int)(q / n_rcv), j = (int)(q % n_rcv);
    const double* sc = src_c + 3 * i;
    const double* rc = rcv_c + 3 * j;
    const double* rn = rcv_n + 3 * j;
    const double dot = xadd(xadd(xmul(rn[0], src_n[0]), xmul(rn[1], src_n[1])), xmul(rn[2], src_n[2]));
    double out;
    if (dot == 0.0) {  // perpendicular
        const int s_ax = plane_axes(src_n), r_ax = plane_axes(rn);
        const int l = only_axis(s_ax & r_ax), sa = only_axis(s_ax & ~(s_ax & r_ax)),
                  ra = only_axis(r_ax & ~(s_ax & r_ax));
        const double dm = fabs(xsub(sc[sa], rc[sa]));
        const double dl = sc[l], dlp = rc[l];
        const double dnp = fabs(xsub(sc[ra], rc[ra]));
        const double h = xmul(0.5, dd);
        const double A = xdiv(xsub(dm, h), __dsqrt_rn(xadd(xadd(sq(xsub(dl, dlp)), sq(xsub(dm, h))), sq(dnp))));
        const double B = xdiv(xadd(dm, h), __dsqrt_rn(xadd(xadd(sq(xsub(dl, dlp)), sq(xadd(dm, h))), sq(dnp))));
        const double one = atan(fabs(xdiv(xsub(xsub(dl, h), dlp), dnp)));
        const double two = atan(fabs(xdiv(xsub(xadd(dl, h), dlp), dnp)));
        const double k = fabs(xsub(dl, dlp)) < 1e-12 ? -1.0 : 1.0;
        const double theta = fabs(xsub(one, xmul(k, two)));
        out = xmul(xmul(xdiv(1.0, 2 * SP_PI), fabs(xsub(sq(A), sq(B)))), theta);
    } else {  // parallel: axes by the walls' centre difference
        const double* rw = rcv_wc + 3 * j;
        double dif[3];
        for (int d = 0; d < 3; ++d) dif[d] = fabs(xsub(rw[d], src_wc[d]));
        int a, m, b;
        if (dif[0] > 1e-5)
            a = 1, m = 0, b = 2;
        else if (dif[1] > 1e-5)
            a = 0, m = 1, b = 2;
        else  // dif[2] > 1e-5, checked by the host
            a = 1, m = 2, b = 0;
        const double d = __dsqrt_rn(xadd(xadd(sq(xsub(rc[a], sc[a])), sq(xsub(rc[b], sc[b]))), sq(xsub(rc[m], sc[m]))));
        out = xdiv(xmul(xmul(dd, dd), sq(xsub(rc[m], sc[m]))), xmul(SP_PI, pow(d, 4.0)));
    }
    ff[q] = out;
}

// Per (receiver r, source s) of one wall pair: the delay and, per band, the
// factor exp(-m_b d) of RadiosityKang.py:240-262.
__global__ void k_kang_pair(int n_rcv, const double* __restrict__ rcv_c, int n_src, const double* __restrict__ src_c,
                            int nb, const double* __restrict__ attenuation, double c, double fs, int nt,
                            int32_t* __restrict__ delay, double* __restrict__ expo, int* __restrict__ err) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)n_rcv * n_src) return;
    const int r = (int)(q / n_src), s = (int)(q % n_src);
    const double d = dist3(rcv_c + 3 * r, src_c + 3 * s);
    const long long dl = (long long)xmul(xdiv(d, c), fs);
    if (dl > nt) atomicCAS(err, 0, kKangErrDelay);
    delay[q] = (int32_t)(dl % (nt > 0 ? nt : 1));  // np.roll by delay == nt is the identity
    for (int b = 0; b < nb; ++b) expo[(size_t)b * n_rcv * n_src + q] = exp(xmul(-attenuation[b], d));
}

// RadiosityKang.py:209-267 for one source wall: E_rcv[b, k, r, t] +=
// sum_s (((roll(E_src[b, k-1, s], delay)[t] * ff) * scattering_b) * (1 - alpha_b)) * expo,
// sources in order, one (band, receiver row, bin) per thread.  A row is a
// receiver patch r and an outgoing direction d (row = r * n_dirs + d).
// Directional (RadiosityKang.py:673-745): the source's direction-d row, the
// term times scat[idx(r, s), d, b]; the wall's scattering is 1 there, so
// ((v * ff) * 1) * (1 - alpha) equals the reference's (v * ff) * (1 - alpha).
template <bool kDir>
__global__ void k_kang_exchange(int k, int nb, int n_orders, int nt, int n_rcv, int n_dirs, long long row0,
                                double* __restrict__ E_rcv, const double* __restrict__ scattering,
                                const double* __restrict__ absorption, int n_src, const double* __restrict__ E_src,
                                const double* __restrict__ ff, long long ff_stride, long long ff_col0,
                                const int32_t* __restrict__ delay, const double* __restrict__ expo,
                                const double* __restrict__ scat, const int32_t* __restrict__ scat_idx) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const long long row = row0 + (long long)blockIdx.y;
    const int b = blockIdx.z;
    if (t >= nt || row >= (long long)n_rcv * n_dirs) return;
    const int r = (int)(row / n_dirs), d = (int)(row % n_dirs);
    const double sc = scattering[b], om = xsub(1.0, absorption[b]);
    const double* prev = E_src + (((size_t)b * n_orders + (k - 1)) * n_src) * n_dirs * nt;
    double* out = E_rcv + ((((size_t)b * n_orders + k) * n_rcv + r) * n_dirs + d) * nt + t;
    double acc = *out;
    for (int s = 0; s < n_src; ++s) {
        const long long q = (long long)r * n_src + s;
        int src_t = t - delay[q];
        if (src_t < 0) src_t += nt;
        const double v = prev[((size_t)s * n_dirs + d) * nt + src_t];
        const double f = ff[(size_t)s * ff_stride + ff_col0 + r];
        double e = xmul(xmul(xmul(xmul(v, f), sc), om), expo[(size_t)b * n_rcv * n_src + q]);
        if (kDir) e = xmul(e, scat[((size_t)scat_idx[q] * n_dirs + d) * nb + b]);
        acc = xadd(acc, e);
    }
    *out = acc;
}

// RadiosityKang.py:443-498 `energy_at_receiver` of one wall, added to out
// (n_bins, nt): out[b, t] += sum_s sum_k roll(E[b, k, s], delay_s)[t] * factor_sb,
// one (band, bin) per thread.
// Directional (RadiosityKang.py:747-810): patch s contributes its row of
// the outgoing direction dir_idx[s] nearest to the receiver.
template <bool kDir>
__global__ void k_kang_receiver(int n, const double* __restrict__ centers, const double* __restrict__ normal, int nb,
                                int n_orders, int nt, const double* __restrict__ E, int max_order,
                                const double* __restrict__ rcv, const double* __restrict__ attenuation, double c,
                                double fs, int n_dirs, const int32_t* __restrict__ dir_idx, double* __restrict__ out,
                                int* __restrict__ err) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (t >= nt) return;
    double resp = 0.0;
    for (int s = 0; s < n; ++s) {
        const double* sp = centers + 3 * s;
        const double dif[3] = {fabs(xsub(rcv[0], sp[0])), fabs(xsub(rcv[1], sp[1])), fabs(xsub(rcv[2], sp[2]))};
        const double R = dist3(sp, rcv);
        const long long dl = (long long)xmul(xdiv(R, c), fs);
        if (dl > nt) {
            if (t == 0 && b == 0) atomicCAS(err, 0, kKangErrDelay);
            continue;
        }
        const int delay = (int)(dl % nt);
        const double cos_xi =
            xdiv(fabs(xadd(xadd(xmul(normal[0], dif[0]), xmul(normal[1], dif[1])), xmul(normal[2], dif[2]))), R);
        const double factor = xdiv(xmul(cos_xi, exp(xmul(-attenuation[b], R))), xmul(SP_PI, xmul(R, R)));
        int src_t = t - delay;
        if (src_t < 0) src_t += nt;
        const int d = kDir ? dir_idx[s] : 0;
        for (int k = 0; k <= max_order; ++k)
            resp = xadd(resp, xmul(E[((((size_t)b * n_orders + k) * n + s) * n_dirs + d) * nt + src_t], factor));
    }
    double* o = out + (size_t)b * nt + t;
    *o = xadd(*o, resp);
}

// form_factor/kang.py:12-169 `patch2patch_ff_kang`: one listed (source,
// receiver) pair per thread over arbitrary axis-aligned patches; sizes is
// (n, size_cols), size_cols 2 or 3 as the reference's patches_size.
__global__ void k_ff_kang_pairs(long long n_pairs, const int32_t* __restrict__ pairs, const double* __restrict__ ctr,
                                const double* __restrict__ nrm, const double* __restrict__ size, int size_cols,
                                double* __restrict__ ff) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_pairs) return;
    const int i = pairs[2 * q], j = pairs[2 * q + 1];
    const double* sc = ctr + 3 * i;
    const double* sn = nrm + 3 * i;
    const double* rc = ctr + 3 * j;
    const double* rn = nrm + 3 * j;
    const double* sz = size + (size_t)size_cols * i;
    const double dot = xadd(xadd(xmul(rn[0], sn[0]), xmul(rn[1], sn[1])), xmul(rn[2], sn[2]));
    double out = 0.0;
    if (dot == 0.0) {  // orthogonal (kang.py:44-120)
        int s_lo, s_hi;  // the source's in-plane axes, as the set idx_source
        double dl, dd_l, dd_m;
        if (fabs(sn[0]) > 1e-5) {
            s_lo = 1, s_hi = 2, dl = sc[2], dd_l = sz[2], dd_m = sz[1];
        } else if (fabs(sn[1]) > 1e-5) {
            s_lo = 0, s_hi = 2, dl = sc[2], dd_l = sz[2], dd_m = sz[0];
        } else {  // |sn[2]| > 1e-5, checked by the host
            s_lo = 0, s_hi = 1, dl = sc[1], dd_l = sz[1], dd_m = sz[0];
        }
        const bool has0 = s_lo == 0, has1 = s_lo == 1 || s_hi == 1;
        int il, is, ir;
        if (fabs(rn[0]) > 1e-5)
            il = has1 ? 1 : 2, is = 0, ir = has1 ? 2 : 1;
        else if (fabs(rn[1]) > 1e-5)
            il = has0 ? 0 : 2, is = 1, ir = has0 ? 2 : 0;
        else
            il = has0 ? 0 : 1, is = 2, ir = has0 ? 1 : 0;
        const double dm = fabs(xsub(sc[is], rc[is]));
        dl = sc[il];
        const double dlp = rc[il];
        const double dnp = fabs(xsub(sc[ir], rc[ir]));
        const double hm = xmul(0.5, dd_m), hl = xmul(0.5, dd_l);
        const double A = xdiv(xsub(dm, hm), __dsqrt_rn(xadd(xadd(sq(xsub(dl, dlp)), sq(xsub(dm, hm))), sq(dnp))));
        const double B = xdiv(xadd(dm, hm), __dsqrt_rn(xadd(xadd(sq(xsub(dl, dlp)), sq(xadd(dm, hm))), sq(dnp))));
        const double one = atan(fabs(xdiv(xsub(xsub(dl, hl), dlp), dnp)));
        const double two = atan(fabs(xdiv(xsub(xadd(dl, hl), dlp), dnp)));
        const double k = fabs(xsub(dl, dlp)) < 1e-12 ? -1.0 : 1.0;
        const double theta = fabs(xsub(one, xmul(k, two)));
        out = xmul(xmul(xdiv(1.0, 2 * SP_PI), fabs(xsub(sq(A), sq(B)))), theta);
    } else {  // parallel (kang.py:122-166), axes by the receiver's normal
        int a, m, b, cl, cn;
        if (fabs(rn[0]) > 1e-5)
            a = 1, m = 0, b = 2, cl = 1, cn = size_cols > 2 ? 2 : 1;
        else if (fabs(rn[1]) > 1e-5)
            a = 0, m = 1, b = 2, cl = 0, cn = size_cols > 2 ? 2 : 1;
        else
            a = 1, m = 2, b = 0, cl = 1, cn = 0;
        const double d = __dsqrt_rn(xadd(xadd(sq(xsub(rc[a], sc[a])), sq(xsub(rc[b], sc[b]))), sq(xsub(rc[m], sc[m]))));
        out = xdiv(xmul(xmul(sz[cl], sz[cn]), sq(xsub(rc[m], sc[m]))), xmul(SP_PI, pow(d, 4.0)));
    }
    ff[q] = out;
}

// form_factor/kang.py:171-262 `_source2patch_energy_kang`: one patch per
// thread; energy (n, nb) = |sin_phi_delta - sin_phi| beta / (4 pi), times
// exp(-att_b d) when att is given; distance (n) in the patch's frame.
__global__ void k_kang_point_source(int n, const double* __restrict__ src, const double* __restrict__ ctr,
                                    const double* __restrict__ nrm, const double* __restrict__ size, int nb,
                                    const double* __restrict__ att, double* __restrict__ energy,
                                    double* __restrict__ distance, int* __restrict__ err) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s[3] = {src[0], src[1], src[2]};
    double r[3] = {ctr[3 * j], ctr[3 * j + 1], ctr[3 * j + 2]};
    const double* nj = nrm + 3 * j;
    int ax, idx[3];
    if (fabs(nj[2]) > 0.99) {
        ax = 2, idx[0] = 0, idx[1] = 1, idx[2] = 2;
    } else if (fabs(nj[1]) > 0.99) {
        ax = 1, idx[0] = 2, idx[1] = 0, idx[2] = 1;
    } else if (fabs(nj[0]) > 0.99) {
        ax = 0, idx[0] = 1, idx[1] = 2, idx[2] = 0;
    } else {
        atomicCAS(err, 0, 3);  // not aligned with an axis
        return;
    }
    const double off = r[ax];
    s[ax] = fabs(xsub(s[ax], off));
    r[ax] = fabs(xsub(r[ax], off));
    const double* sz = size + 3 * j;
    double dphi, beta;
    kang_init_geom(r[idx[0]], r[idx[1]], r[idx[2]], sz[idx[0]], sz[idx[1]], s[idx[0]], s[idx[1]], s[idx[2]], &dphi,
                   &beta);
    const double d = __dsqrt_rn(xadd(xadd(sq(xsub(r[idx[0]], s[idx[0]])), sq(xsub(r[idx[1]], s[idx[1]]))),
                                     sq(xsub(r[idx[2]], s[idx[2]]))));
    distance[j] = d;
    const double e = xdiv(xmul(dphi, beta), 4 * SP_PI);
    for (int b = 0; b < nb; ++b) energy[(size_t)j * nb + b] = att ? xmul(e, exp(xmul(-att[b], d))) : e;
}

// form_factor/kang.py:264-277 `_patch2receiver_energy_kang`: one patch per
// thread; factor = |n . |v|| / R / (pi R^2) for the patch-to-receiver vector v.
__global__ void k_kang_point_receiver(int n, const double* __restrict__ vec, const double* __restrict__ nrm,
                                      double* __restrict__ factor) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* v = vec + 3 * i;
    const double* ni = nrm + 3 * i;
    const double R = __dsqrt_rn(xadd(xadd(sq(v[0]), sq(v[1])), sq(v[2])));
    const double cos_xi =
        xdiv(fabs(xadd(xadd(xmul(ni[0], fabs(v[0])), xmul(ni[1], fabs(v[1]))), xmul(ni[2], fabs(v[2])))), R);
    factor[i] = xdiv(cos_xi, xmul(SP_PI, sq(R)));
}

// Launchers shared by the plain and the directional entry points.
template <bool kDir>
int kang_init(int n, const double* centers, const double* sizes, const double* normal, const double* src,
              double sound_power, int nb, const double* absorption, const double* attenuation,
              double speed_of_sound, double sampling_rate, int n_orders, int nt, int n_dirs, const double* scat,
              const int32_t* scat_idx, double* E, int* err, void* stream) {
    if (n < 0 || nb < 1 || n_orders < 1 || nt < 1 || n_dirs < 1 || !(speed_of_sound > 0) || !(sampling_rate > 0))
        return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    if (!centers || !sizes || !normal || !src || !absorption || !attenuation || !E || !err) return SP_ERR_ARG;
    if (kDir && (!scat || !scat_idx)) return SP_ERR_ARG;
    k_kang_init<kDir><<<sp_blocks(n, 128), 128, 0, sp_counted((cudaStream_t)stream)>>>(
        n, centers, sizes, normal, src, sound_power, nb, absorption, attenuation, speed_of_sound, sampling_rate,
        n_orders, nt, n_dirs, scat, scat_idx, E, err);
    return sp_check_launch();
}

template <bool kDir>
int kang_exchange(int order, int nb, int n_orders, int nt, int n_rcv, const double* rcv_centers, double* E_rcv,
                  const double* scattering, const double* absorption, const double* attenuation, int n_src,
                  const double* src_centers, const double* E_src, const double* ff_src, long long ff_stride,
                  long long ff_col0, double speed_of_sound, double sampling_rate, int n_dirs, const double* scat,
                  const int32_t* scat_idx, void* ws, size_t ws_bytes, int* err, void* stream) {
    if (order < 1 || order >= n_orders || nb < 1 || nt < 1 || n_rcv < 0 || n_src < 0 || n_dirs < 1 ||
        ff_stride < 0 || ff_col0 < 0 || !(speed_of_sound > 0) || !(sampling_rate > 0))
        return SP_ERR_ARG;
    if (n_rcv == 0 || n_src == 0) return SP_OK;
    if (ff_col0 + n_rcv > ff_stride) return SP_ERR_ARG;
    if (!rcv_centers || !E_rcv || !scattering || !absorption || !attenuation || !src_centers || !E_src || !ff_src ||
        !err)
        return SP_ERR_ARG;
    if (kDir && (!scat || !scat_idx)) return SP_ERR_ARG;
    if (!ws || ws_bytes < sp_kang_exchange_workspace(n_rcv, n_src, nb)) return SP_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t pairs = (size_t)n_rcv * n_src;
    int32_t* delay = (int32_t*)ws;
    double* expo = (double*)((char*)ws + sp_align(pairs * 4));
    k_kang_pair<<<sp_blocks((long long)pairs, 128), 128, 0, sp_counted(st)>>>(
        n_rcv, rcv_centers, n_src, src_centers, nb, attenuation, speed_of_sound, sampling_rate, nt, delay, expo, err);
    constexpr long long kMaxGridY = 65535;  // receiver rows per launch (grid y limit)
    const long long rows = (long long)n_rcv * n_dirs;
    for (long long r0 = 0; r0 < rows; r0 += kMaxGridY) {
        dim3 grid((nt + 127) / 128, (unsigned)(rows - r0 < kMaxGridY ? rows - r0 : kMaxGridY), nb);
        k_kang_exchange<kDir><<<grid, 128, 0, sp_counted(st)>>>(order, nb, n_orders, nt, n_rcv, n_dirs, r0, E_rcv,
                                                                scattering, absorption, n_src, E_src, ff_src,
                                                                ff_stride, ff_col0, delay, expo, scat, scat_idx);
    }
    return sp_check_launch();
}

template <bool kDir>
int kang_receiver(int n, const double* centers, const double* normal, int nb, int n_orders, int nt, const double* E,
                  int max_order, const double* receiver, const double* attenuation, double speed_of_sound,
                  double sampling_rate, int n_dirs, const int32_t* dir_idx, double* out, int* err, void* stream) {
    if (n < 0 || nb < 1 || n_orders < 1 || nt < 1 || n_dirs < 1 || max_order < 0 || max_order >= n_orders ||
        !(speed_of_sound > 0) || !(sampling_rate > 0))
        return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    if (!centers || !normal || !E || !receiver || !attenuation || !out || !err) return SP_ERR_ARG;
    if (kDir && !dir_idx) return SP_ERR_ARG;
    dim3 grid((nt + 127) / 128, nb);
    k_kang_receiver<kDir><<<grid, 128, 0, sp_counted((cudaStream_t)stream)>>>(
        n, centers, normal, nb, n_orders, nt, E, max_order, receiver, attenuation, speed_of_sound, sampling_rate,
        n_dirs, dir_idx, out, err);
    return sp_check_launch();
}

}  // namespace

extern "C" {

int sp_kang_init_energy(int n, const double* centers, const double* sizes, const double* normal, const double* src,
                        double sound_power, int nb, const double* absorption, const double* attenuation,
                        double speed_of_sound, double sampling_rate, int n_orders, int nt, double* E, int* err,
                        void* stream) {
    return kang_init<false>(n, centers, sizes, normal, src, sound_power, nb, absorption, attenuation, speed_of_sound,
                            sampling_rate, n_orders, nt, 1, nullptr, nullptr, E, err, stream);
}

int sp_kang_directional_init_energy(int n, const double* centers, const double* sizes, const double* normal,
                                    const double* src, double sound_power, int nb, const double* absorption,
                                    const double* attenuation, double speed_of_sound, double sampling_rate,
                                    int n_orders, int nt, int n_dirs, const double* scat, const int32_t* scat_idx,
                                    double* E, int* err, void* stream) {
    return kang_init<true>(n, centers, sizes, normal, src, sound_power, nb, absorption, attenuation, speed_of_sound,
                           sampling_rate, n_orders, nt, n_dirs, scat, scat_idx, E, err, stream);
}

int sp_kang_form_factors(int n_src, const double* src_centers, const double* src_normal, const double* src_wall_center,
                         int n_rcv, const double* rcv_centers, const double* rcv_normals,
                         const double* rcv_wall_centers, double max_size, double* ff, void* stream) {
    if (n_src < 0 || n_rcv < 0) return SP_ERR_ARG;
    if (n_src == 0 || n_rcv == 0) return SP_OK;
    if (!src_centers || !src_normal || !src_wall_center || !rcv_centers || !rcv_normals || !rcv_wall_centers || !ff)
        return SP_ERR_ARG;
    const long long total = (long long)n_src * n_rcv;
    k_kang_ff<<<sp_blocks(total, 128), 128, 0, sp_counted((cudaStream_t)stream)>>>(
        n_src, src_centers, src_normal, src_wall_center, n_rcv, rcv_centers, rcv_normals, rcv_wall_centers, max_size,
        ff);
    return sp_check_launch();
}

size_t sp_kang_exchange_workspace(int n_rcv, int n_src, int nb) {
    const size_t pairs = (size_t)(n_rcv > 0 ? n_rcv : 0) * (size_t)(n_src > 0 ? n_src : 0);
    return sp_align(pairs * 4) + sp_align(pairs * (size_t)(nb > 0 ? nb : 0) * 8) + 256;
}

int sp_kang_exchange(int order, int nb, int n_orders, int nt, int n_rcv, const double* rcv_centers, double* E_rcv,
                     const double* scattering, const double* absorption, const double* attenuation, int n_src,
                     const double* src_centers, const double* E_src, const double* ff_src, long long ff_stride,
                     long long ff_col0, double speed_of_sound, double sampling_rate, void* ws, size_t ws_bytes,
                     int* err, void* stream) {
    return kang_exchange<false>(order, nb, n_orders, nt, n_rcv, rcv_centers, E_rcv, scattering, absorption,
                                attenuation, n_src, src_centers, E_src, ff_src, ff_stride, ff_col0, speed_of_sound,
                                sampling_rate, 1, nullptr, nullptr, ws, ws_bytes, err, stream);
}

int sp_kang_directional_exchange(int order, int nb, int n_orders, int nt, int n_rcv, const double* rcv_centers,
                                 double* E_rcv, const double* scattering, const double* absorption,
                                 const double* attenuation, int n_src, const double* src_centers, const double* E_src,
                                 const double* ff_src, long long ff_stride, long long ff_col0, double speed_of_sound,
                                 double sampling_rate, int n_dirs, const double* scat, const int32_t* scat_idx,
                                 void* ws, size_t ws_bytes, int* err, void* stream) {
    return kang_exchange<true>(order, nb, n_orders, nt, n_rcv, rcv_centers, E_rcv, scattering, absorption,
                               attenuation, n_src, src_centers, E_src, ff_src, ff_stride, ff_col0, speed_of_sound,
                               sampling_rate, n_dirs, scat, scat_idx, ws, ws_bytes, err, stream);
}

int sp_kang_receiver(int n, const double* centers, const double* normal, int nb, int n_orders, int nt,
                     const double* E, int max_order, const double* receiver, const double* attenuation,
                     double speed_of_sound, double sampling_rate, double* out, int* err, void* stream) {
    return kang_receiver<false>(n, centers, normal, nb, n_orders, nt, E, max_order, receiver, attenuation,
                                speed_of_sound, sampling_rate, 1, nullptr, out, err, stream);
}

int sp_kang_directional_receiver(int n, const double* centers, const double* normal, int nb, int n_orders, int nt,
                                 const double* E, int max_order, const double* receiver, const double* attenuation,
                                 double speed_of_sound, double sampling_rate, int n_dirs, const int32_t* dir_idx,
                                 double* out, int* err, void* stream) {
    return kang_receiver<true>(n, centers, normal, nb, n_orders, nt, E, max_order, receiver, attenuation,
                               speed_of_sound, sampling_rate, n_dirs, dir_idx, out, err, stream);
}

int sp_kang_pair_form_factors(long long n_pairs, const int32_t* pairs, int n, const double* centers,
                              const double* normals, const double* sizes, int size_cols, double* ff, void* stream) {
    if (n_pairs < 0 || n < 0 || (size_cols != 2 && size_cols != 3)) return SP_ERR_ARG;
    if (n_pairs == 0) return SP_OK;
    if (!pairs || !centers || !normals || !sizes || !ff) return SP_ERR_ARG;
    k_ff_kang_pairs<<<sp_blocks(n_pairs, 128), 128, 0, sp_counted((cudaStream_t)stream)>>>(n_pairs, pairs, centers,
                                                                                             normals, sizes, size_cols, ff);
    return sp_check_launch();
}

int sp_kang_point_source(int n, const double* src, const double* centers, const double* normals, const double* sizes,
                         int nb, const double* attenuation, double* energy, double* distance, int* err,
                         void* stream) {
    if (n < 0 || nb < 1) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    if (!src || !centers || !normals || !sizes || !energy || !distance || !err) return SP_ERR_ARG;
    k_kang_point_source<<<sp_blocks(n, 128), 128, 0, sp_counted((cudaStream_t)stream)>>>(
        n, src, centers, normals, sizes, nb, attenuation, energy, distance, err);
    return sp_check_launch();
}

int sp_kang_point_receiver(int n, const double* vectors, const double* normals, double* factor, void* stream) {
    if (n < 0) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    if (!vectors || !normals || !factor) return SP_ERR_ARG;
    k_kang_point_receiver<<<sp_blocks(n, 128), 128, 0, sp_counted((cudaStream_t)stream)>>>(n, vectors, normals,
                                                                                              factor);
    return sp_check_launch();
}

}  // extern "C"
