// Patch-to-patch form factors (universal method) and point-to-patch factors.
//
// * Pairs with a shared vertex (distance < 1e-6, geometry.py:719-748) use the
//   Nusselt analogue in FP64 (integration.py:116-289), as the reference does.
// * All other pairs use the Stokes boundary integral (integration.py:38-114):
//   F = |sum_ab (u_a . v_b) ln|P_a - Q_b|| / (2 pi A_i), where P_a, Q_b are the
//   16 Boole sample points of each boundary and u_a, v_b their Boole weight
//   vectors (a segment whose |dx_dim| <= 1e-3 contributes nothing to dim).
//   - FP64 mode evaluates the logarithms directly.
//   - FP32 mode uses an exact re-centring: with D = c_i - c_j,
//     ln r_ab = ln|D| + (1/2)(L_ab + Q_ab) + (1/2) phi(delta_ab), where
//     delta = L + Q, L = 2 D.e/|D|^2, Q = |e|^2/|D|^2, e = (P_a - c_i) - (Q_b - c_j)
//     and phi(x) = ln(1 + x) - x.  The ln|D|, L and Q sums, and the
//     (D.e)^2 and (D.e)|e|^2 parts of -delta^2/2, reduce to per-patch moments
//     of the weights (FP64).  FP32 carries only the remainder
//     phi(delta) + delta^2/2 - |e|^4/(2|D|^4) = O(|e|^3/|D|^3), so its
//     rounding error is small beside the heavily cancelling sum.  Pairs
//     whose sample points come closer than 0.3 |D|, or whose FP32 error
//     indicator exceeds kFP32RelTol of the result, are recomputed in FP64.
#include "common.cuh"
#include "exchange_common.cuh"

namespace {

__device__ __forceinline__ double boole_coef(int k) {
    return (k == 0 || k == 4) ? 7.0 : ((k == 2) ? 12.0 : 32.0);
}

// geometry.py:498-559 (n_out = z); same operation order as the reference.
__device__ void rotation_matrix_ff(const double* n_in, double* m) {
    if (n_in[0] == 0.0 && n_in[1] == 0.0 && n_in[2] == 1.0) {
        for (int i = 0; i < 9; ++i) m[i] = (i % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    double nn = xnorm3(n_in);
    double a[3] = {xdiv(n_in[0], nn), xdiv(n_in[1], nn), xdiv(n_in[2], nn)};
    double c = a[2];
    if (c != -1.0) {
        double v[3] = {a[1], -a[0], 0.0};  // a x (0,0,1)
        double s = xnorm3(v);
        double k[9] = {0.0, -v[2], v[1], v[2], 0.0, -v[0], -v[1], v[0], 0.0};
        double f = xdiv(xsub(1.0, c), xmul(s, s));
        for (int r = 0; r < 3; ++r)
            for (int col = 0; col < 3; ++col) {
                double kk = k[r * 3 + 0] * k[col] + k[r * 3 + 1] * k[3 + col] + k[r * 3 + 2] * k[6 + col];
                m[r * 3 + col] = ((r == col) ? 1.0 : 0.0) + k[r * 3 + col] + kk * f;
            }
    } else {
        const double flip[9] = {-1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, -1.0};
        for (int i = 0; i < 9; ++i) m[i] = flip[i];
    }
}

// Boundary sample point `a` (0..15) of a quadrilateral: integration.py:639-649
// with npoints = 5 (segment a/4, position a%4).
__device__ __forceinline__ void boundary_point5(const double* el, int a, double* out) {
    int s = a >> 2, k = a & 3;
    const double* p = el + 3 * s;
    const double* q = el + 3 * ((s + 1) & 3);
    for (int d = 0; d < 3; ++d) out[d] = p[d] + (k * (q[d] - p[d])) / 4;
}

// Boole weight vector of boundary point a (0..15): the point is position
// a%4 of segment a/4 and, when a%4 == 0, also position 4 of segment a/4 - 1.
// Segment weight per dim: (2h/45) * c_k with h = x1 - x0, zero when
// |x4 - x0| <= 1e-3 (integration.py:96, :109).
__device__ void boole_weight(const double* el, int a, double* w) {
    int s = a >> 2, k = a & 3;
    for (int d = 0; d < 3; ++d) w[d] = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
        int seg, pos;
        if (pass == 0) {
            seg = s;
            pos = k;
        } else {
            if (k != 0) break;
            seg = (s + 3) & 3;
            pos = 4;
        }
        double x0[3], x1[3], x4[3];
        boundary_point5(el, 4 * seg, x0);
        boundary_point5(el, 4 * seg + 1, x1);
        boundary_point5(el, (4 * seg + 4) & 15, x4);
        for (int d = 0; d < 3; ++d) {
            if (fabs(x4[d] - x0[d]) > 1e-3) {
                double h = x1[d] - x0[d];
                w[d] += 2 * h / 45 * boole_coef(pos);
            }
        }
    }
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// phi3(x) = ln(1 + x) - x + x^2/2, accurate to a few ulp of its value in FP32
// for |x| < 0.2 (14 terms of the Taylor series x^3/3 - x^4/4 + ...).
__device__ __forceinline__ float phi3_f(float x) {
    if (fabsf(x) < 0.2f) {
        float p = -1.0f / 17.0f;
#pragma unroll
        for (int k = 16; k >= 3; --k) p = fmaf(p, x, ((k & 1) ? 1.0f : -1.0f) / (float)k);
        return ((p * x) * x) * x;
    }
    return (log1pf(x) - x) + 0.5f * x * x;
}

// FP32 error indicator of the remainder sum, per term |W| times
// * |rem|: the rounding of the term and of the sum;
// * |rem'(delta)| ~ delta^2 / (1 + delta) times delta's own rounding error,
//   about 2^-24 (2 |D| (|p_a| + |q_b|) + |e|^2) / |D|^2 (the sample points
//   are rounded to FP32 relative to their patch centres);
// * |delta| + delta^2 where log1p(delta) - delta + delta^2/2 cancels.
// The pair's indicator is 2^-24 / 2 times the sum over its 256 terms; the
// pair is recomputed in FP64 when that exceeds kFP32RelTol of |num|, the
// Stokes sum itself.  On the 24046 sampled pairs of a 5939-patch street
// canyon the measured error of the FP32 result never exceeded 1.8 times
// the indicator, so FP32 results keep a relative error below 1e-5 (measured
// at most 1.0e-6 there), and 1.4 % of the pairs are recomputed.
constexpr double kUnitRoundoff32 = 5.960464477539063e-08;  // 2^-24
constexpr double kFP32RelTol = 5e-6;
__device__ __forceinline__ float rem_term_err(float W, float rem, float delta, float ee, float invD2,
                                              float Dn, float la, float lb) {
    const float ad = fabsf(delta);
    return fabsf(W) * (fabsf(rem) + __fdividef(delta * delta, 1.0f + delta) * ((2.0f * Dn * (la + lb) + ee) * invD2) +
                       (ad >= 0.2f ? ad + delta * delta : 0.0f));
}

// integration.py:38-114 `stokes_integration` for one pair, one warp, FP64
// direct logarithms.  Lane l < 16 owns sample point a = l of patch i, lane
// l >= 16 owns point b = l - 16 of patch j; then lane l sums the terms
// (a = l & 15, b in (l >> 4) * 8 .. +8).  Returns the same value on all lanes.
__device__ double stokes_pair(const double* pi, const double* pj, double area_i) {
    int lane = threadIdx.x & 31;
    bool is_i = lane < 16;
    int a = lane & 15;
    const double* el = is_i ? pi : pj;
    double P[3], w[3];
    boundary_point5(el, a, P);
    boole_weight(el, a, w);
    double s = 0.0;
    int half = lane >> 4;
    double Pa[3], ua[3];
    for (int d = 0; d < 3; ++d) {
        Pa[d] = __shfl_sync(0xffffffffu, P[d], a);
        ua[d] = __shfl_sync(0xffffffffu, w[d], a);
    }
    for (int bb = 0; bb < 8; ++bb) {
        int b = half * 8 + bb;
        double Qb[3], vb[3];
        for (int d = 0; d < 3; ++d) {
            Qb[d] = __shfl_sync(0xffffffffu, P[d], 16 + b);
            vb[d] = __shfl_sync(0xffffffffu, w[d], 16 + b);
        }
        double dd[3] = {Pa[0] - Qb[0], Pa[1] - Qb[1], Pa[2] - Qb[2]};
        double r = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
        s += (ua[0] * vb[0] + ua[1] * vb[1] + ua[2] * vb[2]) * log(r);
    }
    s = warp_sum(s);
    return fabs(s / (2 * SP_PI * area_i));
}

__device__ __forceinline__ double dsign(double v) { return (v > 0) ? 1.0 : ((v < 0) ? -1.0 : 0.0); }

// 3x3 inverse with partial pivoting (np.linalg.inv in integration.py:380).
__device__ bool inv3(const double* a, double* out) {
    double m[3][6];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) m[r][c] = a[r * 3 + c];
        for (int c = 0; c < 3; ++c) m[r][3 + c] = (r == c) ? 1.0 : 0.0;
    }
    for (int col = 0; col < 3; ++col) {
        int piv = col;
        for (int r = col + 1; r < 3; ++r)
            if (fabs(m[r][col]) > fabs(m[piv][col])) piv = r;
        if (m[piv][col] == 0.0) return false;
        if (piv != col)
            for (int c = 0; c < 6; ++c) {
                double t = m[piv][c];
                m[piv][c] = m[col][c];
                m[col][c] = t;
            }
        double p = m[col][col];
        for (int c = 0; c < 6; ++c) m[col][c] /= p;
        for (int r = 0; r < 3; ++r) {
            if (r == col) continue;
            double f = m[r][col];
            for (int c = 0; c < 6; ++c) m[r][c] -= f * m[col][c];
        }
    }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[r * 3 + c] = m[r][3 + c];
    return true;
}

// integration.py:416-460 `_area_under_curve` (3 samples, order 2).
__device__ double area_under_curve(const double ps[3][2]) {
    double f[2] = {ps[2][0] - ps[0][0], ps[2][1] - ps[0][1]};
    double nf = sqrt(f[0] * f[0] + f[1] * f[1]);
    double rm[4] = {f[0] / nf, f[1] / nf, -f[1] / nf, f[0] / nf};
    double x[3] = {0, 0, 0}, y[3] = {0, 0, 0};
    for (int k = 1; k < 3; ++k) {
        double c[2] = {ps[k][0] - ps[0][0], ps[k][1] - ps[0][1]};
        x[k] = rm[0] * c[0] + rm[1] * c[1];
        y[k] = rm[2] * c[0] + rm[3] * c[1];
    }
    double b[3] = {0, 0, 0};
    if (!(fabs(x[2] - x[0]) < 1e-6)) {
        double xm[9];
        for (int i = 0; i < 3; ++i) {
            xm[i * 3 + 2] = 1.0;
            xm[i * 3 + 1] = x[i];
            xm[i * 3 + 0] = x[i] * x[i];
        }
        double iv[9];
        if (inv3(xm, iv))
            for (int r = 0; r < 3; ++r) b[r] = iv[r * 3] * y[0] + iv[r * 3 + 1] * y[1] + iv[r * 3 + 2] * y[2];
    }
    double out = 0.0;
    for (int i = 0; i < 3; ++i) {
        int p = 3 - i;
        double x2p = (p == 3) ? x[2] * x[2] * x[2] : ((p == 2) ? x[2] * x[2] : x[2]);
        double x0p = (p == 3) ? x[0] * x[0] * x[0] : ((p == 2) ? x[0] * x[0] : x[0]);
        out += b[i] * x2p / p;
        out -= b[i] * x0p / p;
    }
    return out;
}

// integration.py:116-230 `nusselt_analog` (quadrilateral receiver).
__device__ double nusselt_analog(const double* origin, const double* rot, const double* pp, double hand) {
    double sph[8][3], pln[8][2];
    for (int ii = 0; ii < 8; ++ii) {
        int s = ii >> 1, k = ii & 1;
        const double* p = pp + 3 * s;
        const double* q = pp + 3 * ((s + 1) & 3);
        double bp[3], d[3];
        for (int dd = 0; dd < 3; ++dd) {
            bp[dd] = p[dd] + (k * (q[dd] - p[dd])) / 2;
            d[dd] = bp[dd] - origin[dd];
        }
        double nd = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int dd = 0; dd < 3; ++dd) sph[ii][dd] = d[dd] / nd;
        pln[ii][0] = rot[0] * sph[ii][0] + rot[1] * sph[ii][1] + rot[2] * sph[ii][2];
        pln[ii][1] = rot[3] * sph[ii][0] + rot[4] * sph[ii][1] + rot[5] * sph[ii][2];
    }
    // _polygon_area of the 4 projected corners (z = 0)
    double big = 0.0;
    for (int t = 0; t < 2; ++t) {
        double a0 = pln[2 * (t + 1)][0] - pln[0][0], a1 = pln[2 * (t + 1)][1] - pln[0][1];
        double b0 = pln[2 * (t + 2)][0] - pln[0][0], b1 = pln[2 * (t + 2)][1] - pln[0][1];
        big += 0.5 * fabs(a0 * b1 - a1 * b0);
    }
    double curved = 0.0;
    for (int jj = 0; jj < 4; ++jj) {
        int s0 = 2 * jj, s1 = 2 * jj + 1, s2 = (2 * jj + 2) & 7;
        double crz = pln[s2][0] * pln[s0][1] - pln[s2][1] * pln[s0][0];
        if (fabs(crz) > 1e-6) {
            if (pln[s2][0] * pln[s0][0] + pln[s2][1] * pln[s0][1] >= 1e-6) {
                double seg[3][2] = {{pln[s0][0], pln[s0][1]}, {pln[s1][0], pln[s1][1]}, {pln[s2][0], pln[s2][1]}};
                curved += area_under_curve(seg);
            } else {
                double mp[3], marc[3], a[3], b[3];
                for (int k = 0; k < 3; ++k) mp[k] = sph[s0][k] + (sph[s2][k] - sph[s0][k]) / 2;
                double nm = sqrt(mp[0] * mp[0] + mp[1] * mp[1] + mp[2] * mp[2]);
                for (int k = 0; k < 3; ++k) marc[k] = mp[k] / nm;
                for (int k = 0; k < 3; ++k) a[k] = sph[s0][k] + (marc[k] - sph[s0][k]) / 2;
                for (int k = 0; k < 3; ++k) b[k] = marc[k] + (sph[s2][k] - marc[k]) / 2;
                double na = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
                double nb = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
                for (int k = 0; k < 3; ++k) {
                    a[k] /= na;
                    b[k] /= nb;
                }
                double mp2[2] = {rot[0] * mp[0] + rot[1] * mp[1] + rot[2] * mp[2],
                                 rot[3] * mp[0] + rot[4] * mp[1] + rot[5] * mp[2]};
                double marc2[2] = {rot[0] * marc[0] + rot[1] * marc[1] + rot[2] * marc[2],
                                   rot[3] * marc[0] + rot[4] * marc[1] + rot[5] * marc[2]};
                double a2[2] = {rot[0] * a[0] + rot[1] * a[1] + rot[2] * a[2],
                                rot[3] * a[0] + rot[4] * a[1] + rot[5] * a[2]};
                double b2[2] = {rot[0] * b[0] + rot[1] * b[1] + rot[2] * b[2],
                                rot[3] * b[0] + rot[4] * b[1] + rot[5] * b[2]};
                double d1[2] = {pln[s2][0] - pln[s0][0], pln[s2][1] - pln[s0][1]};
                double d2[2] = {mp2[0] - marc2[0], mp2[1] - marc2[1]};
                double lin = sqrt(d1[0] * d1[0] + d1[1] * d1[1]) * sqrt(d2[0] * d2[0] + d2[1] * d2[1]) / 2;
                double left_seg[3][2] = {{pln[s0][0], pln[s0][1]}, {a2[0], a2[1]}, {marc2[0], marc2[1]}};
                double right_seg[3][2] = {{marc2[0], marc2[1]}, {b2[0], b2[1]}, {pln[s2][0], pln[s2][1]}};
                double left = area_under_curve(left_seg);
                double right = area_under_curve(right_seg);
                curved += (lin * dsign(left) + left + right);
            }
        }
    }
    return big + hand * curved;
}

// integration.py:232-289 `nusselt_integration`, 64 regular-grid samples
// (integration.py:533-605), one warp per pair.
__device__ double nusselt_pair(const double* pi, const double* pj, const double* ni, const double* nj) {
    int lane = threadIdx.x & 31;
    double u[3] = {pi[3] - pi[0], pi[4] - pi[1], pi[5] - pi[2]};
    double v[3] = {pi[9] - pi[0], pi[10] - pi[1], pi[11] - pi[2]};
    double nu = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    double nvv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    long npx = (long)rint(nu / nvv * sqrt(64.0));
    long npz = (long)rint(nvv / nu * sqrt(64.0));
    if (npz == 0) npz = 1;
    if (npx == 0) npx = 1;
    double e1[3] = {pj[3] - pj[0], pj[4] - pj[1], pj[5] - pj[2]};
    double e2[3] = {pj[6] - pj[3], pj[7] - pj[4], pj[8] - pj[5]};
    double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    double hand = dsign(cr[0] * nj[0] + cr[1] * nj[1] + cr[2] * nj[2]);
    double rot[9];
    rotation_matrix_ff(ni, rot);
    long total = npx * npz;
    double s = 0.0;
    for (long idx = lane; idx < total; idx += 32) {
        long ix = idx / npz, iz = idx % npz;
        double stopx = 1 - 1.0 / npx, stopz = 1 - 1.0 / npz;
        double tx = (npx > 1) ? ((ix == npx - 1) ? stopx : ix * (stopx / (npx - 1))) : 0.0;
        double tz = (npz > 1) ? ((iz == npz - 1) ? stopz : iz * (stopz / (npz - 1))) : 0.0;
        tx += 1.0 / (npx * 2);
        tz += 1.0 / (npz * 2);
        double o[3];
        for (int d = 0; d < 3; ++d) o[d] = tx * u[d] + tz * v[d] + pi[d];
        s += nusselt_analog(o, rot, pj, hand);
    }
    s = warp_sum(s);
    return s * (1 / (SP_PI * total));
}

__device__ __forceinline__ bool coincident(const double* p0, const double* p1) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double d[3] = {p0[3 * i] - p1[3 * j], p0[3 * i + 1] - p1[3 * j + 1], p0[3 * i + 2] - p1[3 * j + 2]};
            if (sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) < 1e-6) return true;
        }
    return false;
}

// method codes written per pair
enum { kStokes32 = 0, kStokes64 = 1, kNusselt = 2 };

// universal.py:12-96 in FP64: one warp per visible pair (i < j, i = source).
__global__ void __launch_bounds__(256) k_form_factors(long long n_pairs, const int32_t* __restrict__ pairs,
                                                      const double* __restrict__ pts, const double* __restrict__ normals,
                                                      const double* __restrict__ areas, double* __restrict__ ff,
                                                      uint8_t* __restrict__ method) {
    long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (q >= n_pairs) return;
    int lane = threadIdx.x & 31;
    int i = pairs[2 * q], j = pairs[2 * q + 1];
    double pi[12], pj[12];
    for (int k = 0; k < 12; ++k) {
        pi[k] = pts[(size_t)i * 12 + k];
        pj[k] = pts[(size_t)j * 12 + k];
    }
    double result;
    int m;
    if (coincident(pj, pi)) {
        double ni[3] = {normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]};
        double nj[3] = {normals[3 * j], normals[3 * j + 1], normals[3 * j + 2]};
        result = nusselt_pair(pi, pj, ni, nj);
        m = kNusselt;
    } else {
        result = stokes_pair(pi, pj, areas[i]);
        m = kStokes64;
    }
    if (lane == 0) {
        ff[q] = result;
        if (method) method[q] = (uint8_t)m;
    }
}

// ---------------------------------------------------------------------------
// Patches of nv != 4 vertices (3 <= nv <= kMaxPolyVerts): the same universal
// form factor, FP64, one warp per pair, written for any convex polygon.
constexpr int kMaxPolyVerts = 8;

// Boundary sample point a of a polygon of nv vertices, n_div points per side
// (integration.py:639-649 with npoints = n_div + 1): side a / n_div,
// position a % n_div.
__device__ __forceinline__ void boundary_point_n(const double* el, int nv, int n_div, int a, double* out) {
    const int s = a / n_div, k = a % n_div;
    const double* p = el + 3 * s;
    const double* q = el + 3 * ((s + 1) % nv);
    for (int d = 0; d < 3; ++d) out[d] = p[d] + (k * (q[d] - p[d])) / n_div;
}

// Boole weight vector of boundary point a (0 .. 4 nv - 1); see boole_weight.
__device__ void boole_weight_n(const double* el, int nv, int a, double* w) {
    const int s = a >> 2, k = a & 3, nb = 4 * nv;
    for (int d = 0; d < 3; ++d) w[d] = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
        int seg, pos;
        if (pass == 0) {
            seg = s;
            pos = k;
        } else {
            if (k != 0) break;
            seg = (s + nv - 1) % nv;
            pos = 4;
        }
        double x0[3], x1[3], x4[3];
        boundary_point_n(el, nv, 4, 4 * seg, x0);
        boundary_point_n(el, nv, 4, 4 * seg + 1, x1);
        boundary_point_n(el, nv, 4, (4 * seg + 4) % nb, x4);
        for (int d = 0; d < 3; ++d) {
            if (fabs(x4[d] - x0[d]) > 1e-3) {
                double h = x1[d] - x0[d];
                w[d] += 2 * h / 45 * boole_coef(pos);
            }
        }
    }
}

// integration.py:38-114 `stokes_integration` for polygons of nvi and nvj
// vertices (4 nv <= 32 sample points each), one warp, FP64 logarithms: lane
// l owns point l of both boundaries, patch j's points reach every lane by
// shuffles.  Returns the same value on all lanes.
__device__ double stokes_pair_n(const double* pi, int nvi, const double* pj, int nvj, double area_i) {
    const int lane = threadIdx.x & 31;
    const int na = 4 * nvi, nb = 4 * nvj;
    double P[3] = {0, 0, 0}, u[3] = {0, 0, 0}, Q[3] = {0, 0, 0}, v[3] = {0, 0, 0};
    if (lane < na) {
        boundary_point_n(pi, nvi, 4, lane, P);
        boole_weight_n(pi, nvi, lane, u);
    }
    if (lane < nb) {
        boundary_point_n(pj, nvj, 4, lane, Q);
        boole_weight_n(pj, nvj, lane, v);
    }
    double s = 0.0;
    for (int b = 0; b < nb; ++b) {
        double Qb[3], vb[3];
        for (int d = 0; d < 3; ++d) {
            Qb[d] = __shfl_sync(0xffffffffu, Q[d], b);
            vb[d] = __shfl_sync(0xffffffffu, v[d], b);
        }
        if (lane < na) {
            double dd[3] = {P[0] - Qb[0], P[1] - Qb[1], P[2] - Qb[2]};
            double r = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
            s += (u[0] * vb[0] + u[1] * vb[1] + u[2] * vb[2]) * log(r);
        }
    }
    s = warp_sum(s);
    return fabs(s / (2 * SP_PI * area_i));
}

// integration.py:116-230 `nusselt_analog` for a receiver polygon of nvp
// vertices (2 nvp boundary points, nvp sides of 3 points).
__device__ double nusselt_analog_n(const double* origin, const double* rot, const double* pp, int nvp, double hand) {
    const int nbp = 2 * nvp;
    double sph[2 * kMaxPolyVerts][3], pln[2 * kMaxPolyVerts][2];
    for (int ii = 0; ii < nbp; ++ii) {
        double bp[3], d[3];
        boundary_point_n(pp, nvp, 2, ii, bp);
        for (int dd = 0; dd < 3; ++dd) d[dd] = bp[dd] - origin[dd];
        double nd = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int dd = 0; dd < 3; ++dd) sph[ii][dd] = d[dd] / nd;
        pln[ii][0] = rot[0] * sph[ii][0] + rot[1] * sph[ii][1] + rot[2] * sph[ii][2];
        pln[ii][1] = rot[3] * sph[ii][0] + rot[4] * sph[ii][1] + rot[5] * sph[ii][2];
    }
    // geometry.py:420-440 `_polygon_area` of the nvp projected corners (z = 0)
    double big = 0.0;
    for (int t = 0; t < nvp - 2; ++t) {
        double a0 = pln[2 * (t + 1)][0] - pln[0][0], a1 = pln[2 * (t + 1)][1] - pln[0][1];
        double b0 = pln[2 * (t + 2)][0] - pln[0][0], b1 = pln[2 * (t + 2)][1] - pln[0][1];
        big += 0.5 * fabs(a0 * b1 - a1 * b0);
    }
    double curved = 0.0;
    for (int jj = 0; jj < nvp; ++jj) {
        int s0 = 2 * jj, s1 = 2 * jj + 1, s2 = (2 * jj + 2) % nbp;
        double crz = pln[s2][0] * pln[s0][1] - pln[s2][1] * pln[s0][0];
        if (fabs(crz) > 1e-6) {
            if (pln[s2][0] * pln[s0][0] + pln[s2][1] * pln[s0][1] >= 1e-6) {
                double seg[3][2] = {{pln[s0][0], pln[s0][1]}, {pln[s1][0], pln[s1][1]}, {pln[s2][0], pln[s2][1]}};
                curved += area_under_curve(seg);
            } else {
                double mp[3], marc[3], a[3], b[3];
                for (int k = 0; k < 3; ++k) mp[k] = sph[s0][k] + (sph[s2][k] - sph[s0][k]) / 2;
                double nm = sqrt(mp[0] * mp[0] + mp[1] * mp[1] + mp[2] * mp[2]);
                for (int k = 0; k < 3; ++k) marc[k] = mp[k] / nm;
                for (int k = 0; k < 3; ++k) a[k] = sph[s0][k] + (marc[k] - sph[s0][k]) / 2;
                for (int k = 0; k < 3; ++k) b[k] = marc[k] + (sph[s2][k] - marc[k]) / 2;
                double na = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
                double nb = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
                for (int k = 0; k < 3; ++k) {
                    a[k] /= na;
                    b[k] /= nb;
                }
                double mp2[2] = {rot[0] * mp[0] + rot[1] * mp[1] + rot[2] * mp[2],
                                 rot[3] * mp[0] + rot[4] * mp[1] + rot[5] * mp[2]};
                double marc2[2] = {rot[0] * marc[0] + rot[1] * marc[1] + rot[2] * marc[2],
                                   rot[3] * marc[0] + rot[4] * marc[1] + rot[5] * marc[2]};
                double a2[2] = {rot[0] * a[0] + rot[1] * a[1] + rot[2] * a[2],
                                rot[3] * a[0] + rot[4] * a[1] + rot[5] * a[2]};
                double b2[2] = {rot[0] * b[0] + rot[1] * b[1] + rot[2] * b[2],
                                rot[3] * b[0] + rot[4] * b[1] + rot[5] * b[2]};
                double d1[2] = {pln[s2][0] - pln[s0][0], pln[s2][1] - pln[s0][1]};
                double d2[2] = {mp2[0] - marc2[0], mp2[1] - marc2[1]};
                double lin = sqrt(d1[0] * d1[0] + d1[1] * d1[1]) * sqrt(d2[0] * d2[0] + d2[1] * d2[1]) / 2;
                double left_seg[3][2] = {{pln[s0][0], pln[s0][1]}, {a2[0], a2[1]}, {marc2[0], marc2[1]}};
                double right_seg[3][2] = {{marc2[0], marc2[1]}, {b2[0], b2[1]}, {pln[s2][0], pln[s2][1]}};
                double left = area_under_curve(left_seg);
                double right = area_under_curve(right_seg);
                curved += (lin * dsign(left) + left + right);
            }
        }
    }
    return big + hand * curved;
}

// integration.py:232-289 `nusselt_integration` with the regular grid of
// integration.py:533-605 (64 requested samples): the parallelogram spanned
// by el[1] - el[0] and el[nv - 1] - el[0], or for a triangle (twice the
// requested density) the columns shortened along the first side and the
// points past the hypotenuse (s + t > 1 - thres) left out.  One warp.
__device__ double nusselt_pair_n(const double* pi, int nvi, const double* pj, int nvj, const double* ni,
                                 const double* nj) {
    const int lane = threadIdx.x & 31;
    const double* last = pi + 3 * (nvi - 1);
    double u[3] = {pi[3] - pi[0], pi[4] - pi[1], pi[5] - pi[2]};
    double v[3] = {last[0] - pi[0], last[1] - pi[1], last[2] - pi[2]};
    const bool tri = nvi == 3;
    const double dens = tri ? 2.0 * 64.0 : 64.0;
    double nu = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    double nvv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    long npx = (long)rint(nu / nvv * sqrt(dens));
    long npz = (long)rint(nvv / nu * sqrt(dens));
    if (npz == 0) npz = 1;
    if (npx == 0) npx = 1;
    const double sstep = 1.0 / (npx * 2), sstepz = 1.0 / (npz * 2);
    const double thres = sqrt(sstepz * sstepz + sstep * sstep) / 2;
    double e1[3] = {pj[3] - pj[0], pj[4] - pj[1], pj[5] - pj[2]};
    double e2[3] = {pj[6] - pj[3], pj[7] - pj[4], pj[8] - pj[5]};
    double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    double hand = dsign(cr[0] * nj[0] + cr[1] * nj[1] + cr[2] * nj[2]);
    double rot[9];
    rotation_matrix_ff(ni, rot);
    const long total = npx * npz;
    double s = 0.0;
    int cnt = 0;
    for (long idx = lane; idx < total; idx += 32) {
        long ix = idx / npz, iz = idx % npz;
        // tz[0 : npz - round(npz / npx * ix)] for a triangle (a stop below 0 counts from the end)
        long stop = tri ? npz - (long)rint((double)npz / (double)npx * (double)ix) : npz;
        if (stop < 0) stop = npz + stop > 0 ? npz + stop : 0;
        if (iz >= stop) continue;
        double stopx = 1 - 1.0 / npx, stopz = 1 - 1.0 / npz;
        double tx = (npx > 1) ? ((ix == npx - 1) ? stopx : ix * (stopx / (npx - 1))) : 0.0;
        double tz = (npz > 1) ? ((iz == npz - 1) ? stopz : iz * (stopz / (npz - 1))) : 0.0;
        tx += sstep;
        tz += sstepz;
        if (tri && !(tx + tz <= 1 - thres)) continue;
        double o[3];
        for (int d = 0; d < 3; ++d) o[d] = tx * u[d] + tz * v[d] + pi[d];
        s += nusselt_analog_n(o, rot, pj, nvj, hand);
        ++cnt;
    }
    s = warp_sum(s);
    cnt = warp_sum(cnt);
    return s * (1 / (SP_PI * cnt));
}

__device__ __forceinline__ bool coincident_n(const double* p0, int nv0, const double* p1, int nv1) {
    for (int i = 0; i < nv0; ++i)
        for (int j = 0; j < nv1; ++j) {
            double d[3] = {p0[3 * i] - p1[3 * j], p0[3 * i + 1] - p1[3 * j + 1], p0[3 * i + 2] - p1[3 * j + 2]};
            if (sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) < 1e-6) return true;
        }
    return false;
}

// universal.py:54-96 for patches of nv vertices, one warp per pair.
__global__ void __launch_bounds__(256) k_form_factors_poly(long long n_pairs, int nv, const int32_t* __restrict__ pairs,
                                                           const double* __restrict__ pts,
                                                           const double* __restrict__ normals,
                                                           const double* __restrict__ areas, double* __restrict__ ff,
                                                           uint8_t* __restrict__ method) {
    long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (q >= n_pairs) return;
    int lane = threadIdx.x & 31;
    int i = pairs[2 * q], j = pairs[2 * q + 1];
    double pi[3 * kMaxPolyVerts], pj[3 * kMaxPolyVerts];
    for (int k = 0; k < 3 * nv; ++k) {
        pi[k] = pts[(size_t)i * 3 * nv + k];
        pj[k] = pts[(size_t)j * 3 * nv + k];
    }
    double result;
    int m;
    if (coincident_n(pj, nv, pi, nv)) {
        double ni[3] = {normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]};
        double nj[3] = {normals[3 * j], normals[3 * j + 1], normals[3 * j + 2]};
        result = nusselt_pair_n(pi, nv, pj, nv, ni, nj);
        m = kNusselt;
    } else {
        result = stokes_pair_n(pi, nv, pj, nv, areas[i]);
        m = kStokes64;
    }
    if (lane == 0) {
        ff[q] = result;
        if (method) method[q] = (uint8_t)m;
    }
}

// ---------------------------------------------------------------------------
// FP32 Stokes in three passes (the FP64 pipe carries only per-patch sums and
// one short base term per pair):
//   k_ff_patch_data: per patch, the 16 boundary points relative to the centre
//     and their Boole weights (FP32 copies for the remainder sum) and the
//     FP64 sums over the samples a (loc = p_a):
//       W[d] = sum w[d],             M[d][e] = sum w[d] loc[e],
//       Q[d] = sum w[d] |loc|^2,     T[d][e][f] = sum w[d] loc[e] loc[f],
//       R[d][e] = sum w[d] loc[e] |loc|^2;
//   k_ff_base: one pair per thread: shared-vertex test (Nusselt pairs are
//     set aside) and, from the sums, base = 1/2 ln|D|^2 W_i.W_j + lin + quad
//     - (A + B) / |D|^4 with A = sum W_ab (D.e)^2, B = sum W_ab (D.e)|e|^2;
//   k_ff_phi: one pair per warp: the FP32 sum of (u_a.v_b) rem(delta_ab)
//     and its error indicator; pairs whose sample points come closer than
//     0.3 |D| are set aside;
//   k_ff_finish: ff = |base + sum / 2| / (2 pi A_i), or set aside;
//   k_ff_rework: set-aside pairs, one warp each, in FP64 (Stokes or Nusselt).
struct PatchStokes {
    double c[3];   // centre (vertex mean, geometry.py:412-413)
    double W[3];
    double Q[3];
    double M[9];   // M[3 d + e]
    double T[18];  // T[6 d + s], s over the symmetric (e, f) = 00 01 02 11 12 22
    double R[9];   // R[3 d + e]
    double rad;    // largest vertex distance from the centre
};
constexpr int kPatchF = 16 * 8;  // per patch: 16 x (loc.xyz, |loc|, w.xyz, 0) floats
// The (e, f) of slot s: 00 01 02 11 12 22.
__device__ __forceinline__ int sym_e(int s) { return s < 3 ? 0 : (s < 5 ? 1 : 2); }
__device__ __forceinline__ int sym_f(int s) { return s < 3 ? s : (s < 5 ? s - 2 : 2); }

// Index of the symmetric pair (e, f) in T's 6 slots.
__device__ __forceinline__ int sym_slot(int e, int f) {
    const int lo = e < f ? e : f, hi = e < f ? f : e;
    return lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
}

// Two patches per warp: lanes 0-15 patch 2w, lanes 16-31 patch 2w + 1 (the
// half-warp reduction order of stokes_pair).  nv = 4 (16 sample points) or
// 3 (12 sample points; the last four slots carry weight 0 at the centre).
__global__ void k_ff_patch_data(int n, int nv, const double* __restrict__ pts, PatchStokes* __restrict__ out,
                                float* __restrict__ outf) {
    const int warp = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    const int k = 2 * warp + (lane >> 4);
    const bool on = k < n;
    const int a = lane & 15;
    double el[12];
    for (int q = 0; q < 12; ++q) el[q] = (on && q < 3 * nv) ? pts[(size_t)k * 3 * nv + q] : 0.0;
    double P[3], w[3], c[3];
    if (nv == 4) {
        boundary_point5(el, a, P);
        boole_weight(el, a, w);
        for (int d = 0; d < 3; ++d) c[d] = (((el[d] + el[3 + d]) + el[6 + d]) + el[9 + d]) / 4;
    } else {
        for (int d = 0; d < 3; ++d) c[d] = ((el[d] + el[3 + d]) + el[6 + d]) / 3;
        if (a < 4 * nv) {
            boundary_point_n(el, nv, 4, a, P);
            boole_weight_n(el, nv, a, w);
        } else {
            for (int d = 0; d < 3; ++d) {
                P[d] = c[d];
                w[d] = 0.0;
            }
        }
    }
    double loc[3] = {P[0] - c[0], P[1] - c[1], P[2] - c[2]};
    double l2 = loc[0] * loc[0] + loc[1] * loc[1] + loc[2] * loc[2];
    constexpr int kMom = 42;  // W 3, Q 3, M 9, T 18, R 9
    double mom[kMom];
    for (int d = 0; d < 3; ++d) {
        mom[d] = w[d];
        mom[3 + d] = l2 * w[d];
        for (int e = 0; e < 3; ++e) {
            mom[6 + 3 * d + e] = w[d] * loc[e];
            mom[33 + 3 * d + e] = (w[d] * loc[e]) * l2;
        }
        for (int s = 0; s < 6; ++s) mom[15 + 6 * d + s] = (w[d] * loc[sym_e(s)]) * loc[sym_f(s)];
    }
    for (int q = 0; q < kMom; ++q) {
        double v = mom[q];
        for (int off = 8; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        mom[q] = v;
    }
    if (!on) return;
    float* f = outf + (size_t)k * kPatchF + 8 * a;
    f[0] = (float)loc[0];
    f[1] = (float)loc[1];
    f[2] = (float)loc[2];
    f[3] = (float)sqrt(l2);
    f[4] = (float)w[0];
    f[5] = (float)w[1];
    f[6] = (float)w[2];
    f[7] = 0.0f;
    if (a == 0) {
        PatchStokes r;
        for (int d = 0; d < 3; ++d) {
            r.c[d] = c[d];
            r.W[d] = mom[d];
            r.Q[d] = mom[3 + d];
        }
        for (int q = 0; q < 9; ++q) {
            r.M[q] = mom[6 + q];
            r.R[q] = mom[33 + q];
        }
        for (int q = 0; q < 18; ++q) r.T[q] = mom[15 + q];
        double rad2 = 0.0;
        for (int v = 0; v < nv; ++v) {
            const double dv[3] = {el[3 * v] - c[0], el[3 * v + 1] - c[1], el[3 * v + 2] - c[2]};
            rad2 = fmax(rad2, dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
        }
        r.rad = sqrt(rad2);
        out[k] = r;
    }
}

// A patch's moments contracted with D: m1[d] = sum w[d] (D.loc),
// t1[d][f] = sum w[d] (D.loc) loc[f], m2[d] = sum w[d] (D.loc)^2 and
// mq1[d] = sum w[d] (D.loc) |loc|^2.
struct DMoments {
    double m1[3], t1[9], m2[3], mq1[3];
};
__device__ __forceinline__ void d_moments(const PatchStokes& P, const double* D, DMoments& o) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        o.m1[d] = D[0] * P.M[3 * d] + D[1] * P.M[3 * d + 1] + D[2] * P.M[3 * d + 2];
        o.mq1[d] = D[0] * P.R[3 * d] + D[1] * P.R[3 * d + 1] + D[2] * P.R[3 * d + 2];
#pragma unroll
        for (int f = 0; f < 3; ++f)
            o.t1[3 * d + f] = D[0] * P.T[6 * d + sym_slot(0, f)] + D[1] * P.T[6 * d + sym_slot(1, f)] +
                              D[2] * P.T[6 * d + sym_slot(2, f)];
        o.m2[d] = D[0] * o.t1[3 * d] + D[1] * o.t1[3 * d + 1] + D[2] * o.t1[3 * d + 2];
    }
}

// One pair per thread.  method: kNusselt for shared-vertex pairs (handled in
// k_ff_rework), else kStokes32 with ff = base (completed by k_ff_finish).
__global__ void k_ff_base(long long n_pairs, int nv, const int32_t* __restrict__ pairs, const double* __restrict__ pts,
                          const PatchStokes* __restrict__ pd, double* __restrict__ ff, uint8_t* __restrict__ method,
                          float4* __restrict__ geo, unsigned long long* __restrict__ n_rework,
                          int64_t* __restrict__ rework) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_pairs) return;
    const int i = pairs[2 * q], j = pairs[2 * q + 1];
    const PatchStokes& A = pd[i];
    const PatchStokes& B = pd[j];
    const double D[3] = {A.c[0] - B.c[0], A.c[1] - B.c[1], A.c[2] - B.c[2]};
    const double D2 = D[0] * D[0] + D[1] * D[1] + D[2] * D[2];
    // Every vertex distance is at least |D| - rad_i - rad_j: beyond 1e-5 no
    // vertex pair can pass the shared-vertex test (distance < 1e-6), which
    // then runs only for the remaining pairs.
    const double reach = A.rad + B.rad + 1e-5;
    if (D2 <= reach * reach) {
        double pi[12], pj[12];
        for (int k = 0; k < 3 * nv; ++k) {
            pi[k] = pts[(size_t)i * 3 * nv + k];
            pj[k] = pts[(size_t)j * 3 * nv + k];
        }
        if (coincident_n(pj, nv, pi, nv)) {
            method[q] = kNusselt;
            rework[atomicAdd(n_rework, 1ull)] = q;
            return;
        }
    }
    DMoments a, b;
    d_moments(A, D, a);
    d_moments(B, D, b);
    // e = p_a - q_b; with W_ab = sum_d u_a[d] v_b[d] every sum below splits
    // into products of the two patches' moments.
    double UV = 0.0, lin = 0.0, pq = 0.0, qq = 0.0, sA = 0.0, sB = 0.0;
    for (int d = 0; d < 3; ++d) {
        UV += A.W[d] * B.W[d];
        lin += a.m1[d] * B.W[d] - A.W[d] * b.m1[d];                            // sum W D.e
        qq += A.Q[d] * B.W[d] + A.W[d] * B.Q[d];
        double cross = 0.0;
        for (int e = 0; e < 3; ++e) {
            pq += A.M[3 * d + e] * B.M[3 * d + e];
            cross += A.M[3 * d + e] * b.t1[3 * d + e] - a.t1[3 * d + e] * B.M[3 * d + e];
        }
        sA += a.m2[d] * B.W[d] - 2.0 * a.m1[d] * b.m1[d] + A.W[d] * b.m2[d];  // sum W (D.e)^2
        sB += (a.mq1[d] * B.W[d] - A.W[d] * b.mq1[d]) + (a.m1[d] * B.Q[d] - A.Q[d] * b.m1[d]) +
              2.0 * cross;                                                      // sum W (D.e)|e|^2
    }
    ff[q] = 0.5 * log(D2) * UV + lin / D2 + 0.5 * (qq - 2.0 * pq) / D2 - (sA + sB) / (D2 * D2);
    method[q] = kStokes32;
    // what the warp-per-pair phi sum needs, rounded once here (FP64 on every lane of a full warp)
    geo[q] = make_float4((float)D[0], (float)D[1], (float)D[2], (float)(1.0 / D2));
}

// One pair per warp, FP32 only: acc = sum_ab (u_a.v_b) rem_ab over the 256
// sample pairs, rem = phi3(delta) - |e|^4 / (2 |D|^4), with the sum of
// rem_term_err beside it; k_ff_finish forms ff = |base + acc / 2| / (2 pi A_i).
__global__ void __launch_bounds__(256) k_ff_phi(long long n_pairs, const int32_t* __restrict__ pairs,
                                                const float4* __restrict__ geo, const float* __restrict__ pf,
                                                float2* __restrict__ acc_out, uint8_t* __restrict__ method,
                                                unsigned long long* __restrict__ n_rework,
                                                int64_t* __restrict__ rework) {
    const long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (q >= n_pairs) return;
    if (method[q] != kStokes32) return;  // the same for the whole warp
    const int lane = threadIdx.x & 31;
    const int i = pairs[2 * q], j = pairs[2 * q + 1];
    const float4 g = geo[q];
    const float Df[3] = {g.x, g.y, g.z};
    const float invD2 = g.w;
    const float Dn = rsqrtf(invD2);
    const int a = lane & 15, half = lane >> 4;
    const float4* fi = reinterpret_cast<const float4*>(pf + (size_t)i * kPatchF) + 2 * a;
    const float4 pa = fi[0], ua = fi[1];
    const float4* fj = reinterpret_cast<const float4*>(pf + (size_t)j * kPatchF);
    float acc = 0.0f, aerr = 0.0f, min_ratio = 1e30f;
#pragma unroll
    for (int bb = 0; bb < 8; ++bb) {
        const int b = half * 8 + bb;
        const float4 qb = fj[2 * b], vb = fj[2 * b + 1];
        const float e[3] = {pa.x - qb.x, pa.y - qb.y, pa.z - qb.z};
        const float de = Df[0] * e[0] + Df[1] * e[1] + Df[2] * e[2];
        const float ee = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
        const float delta = (2.0f * de + ee) * invD2;
        min_ratio = fminf(min_ratio, 1.0f + delta);
        const float W = ua.x * vb.x + ua.y * vb.y + ua.z * vb.z;
        const float q2 = ee * invD2;
        const float rem = phi3_f(delta) - 0.5f * q2 * q2;
        acc = fmaf(W, rem, acc);
        aerr += rem_term_err(W, rem, delta, ee, invD2, Dn, pa.w, qb.w);
    }
    acc = warp_sum(acc);
    aerr = warp_sum(aerr);
    for (int off = 16; off > 0; off >>= 1) min_ratio = fminf(min_ratio, __shfl_xor_sync(0xffffffffu, min_ratio, off));
    if (lane != 0) return;
    if (min_ratio < 0.09f) {  // some r_ab < 0.3 |D|: FP64
        method[q] = kStokes64;
        rework[atomicAdd(n_rework, 1ull)] = q;
        return;
    }
    acc_out[q] = make_float2(acc, aerr);
}

// One pair per thread: the FP32 Stokes pairs' form factors from the base term
// and the remainder sum, or a place in the FP64 rework list when the sum's
// error indicator exceeds kFP32RelTol of the result.
__global__ void k_ff_finish(long long n_pairs, const int32_t* __restrict__ pairs, const float2* __restrict__ acc,
                            const double* __restrict__ areas, uint8_t* __restrict__ method, double* __restrict__ ff,
                            unsigned long long* __restrict__ n_rework, int64_t* __restrict__ rework) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_pairs || method[q] != kStokes32) return;
    const float2 s = acc[q];
    const double num = ff[q] + 0.5 * (double)s.x;
    if (0.5 * kUnitRoundoff32 * (double)s.y > kFP32RelTol * fabs(num)) {
        method[q] = kStokes64;
        rework[atomicAdd(n_rework, 1ull)] = q;
        return;
    }
    ff[q] = fabs(num / (2 * SP_PI * areas[pairs[2 * q]]));
}

// Set-aside pairs, one warp each: FP64 Stokes or the Nusselt analogue.
__global__ void __launch_bounds__(256) k_ff_rework(long long count, int nv, const int64_t* __restrict__ rework,
                                                   const int32_t* __restrict__ pairs, const double* __restrict__ pts,
                                                   const double* __restrict__ normals, const double* __restrict__ areas,
                                                   double* __restrict__ ff, const uint8_t* __restrict__ method) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= count) return;
    const int lane = threadIdx.x & 31;
    const long long q = rework[w];
    const int i = pairs[2 * q], j = pairs[2 * q + 1];
    double pi[12], pj[12];
    for (int k = 0; k < 3 * nv; ++k) {
        pi[k] = pts[(size_t)i * 3 * nv + k];
        pj[k] = pts[(size_t)j * 3 * nv + k];
    }
    double result;
    if (method[q] == kNusselt) {
        double ni[3] = {normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]};
        double nj[3] = {normals[3 * j], normals[3 * j + 1], normals[3 * j + 2]};
        result = nv == 4 ? nusselt_pair(pi, pj, ni, nj) : nusselt_pair_n(pi, nv, pj, nv, ni, nj);
    } else {
        result = nv == 4 ? stokes_pair(pi, pj, areas[i]) : stokes_pair_n(pi, nv, pj, nv, areas[i]);
    }
    if (lane == 0) ff[q] = result;
}

// geometry.py:688-715 `_sphere_tangent_vector`.
__device__ void sphere_tangent(const double* v0, const double* v1, double* out) {
    if (fabs(v0[0] * v1[0] + v0[1] * v1[1] + v0[2] * v1[2]) > 1e-10) {
        double d[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
        double f = (d[0] * v0[0] + d[1] * v0[1] + d[2] * v0[2]) / (v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
        for (int k = 0; k < 3; ++k) out[k] = d[k] - f * v0[k];
        double n = sqrt(out[0] * out[0] + out[1] * out[1] + out[2] * out[2]);
        for (int k = 0; k < 3; ++k) out[k] /= n;
    } else {
        double n = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
        for (int k = 0; k < 3; ++k) out[k] = v1[k] / n;
    }
}

}  // namespace

// integration.py:295-344 `pt_solution` (mode 0 = source, 1 = receiver).
static __device__ double sp_pt_solution(const double* point, const double* patch, int nv, int mode) {
    double area = 4.0;
    if (mode == 1) {
        area = 0.0;
        for (int t = 0; t < nv - 2; ++t) {
            const double* p1 = patch + 3 * (t + 1);
            const double* p2 = patch + 3 * (t + 2);
            double a[3] = {p1[0] - patch[0], p1[1] - patch[1], p1[2] - patch[2]};
            double b[3] = {p2[0] - patch[0], p2[1] - patch[1], p2[2] - patch[2]};
            double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            area += 0.5 * sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        }
    }
    double ons[8][3];
    for (int i = 0; i < nv; ++i) {
        double d[3] = {patch[3 * i] - point[0], patch[3 * i + 1] - point[1], patch[3 * i + 2] - point[2]};
        double n = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int k = 0; k < 3; ++k) ons[i][k] = d[k] / n;
    }
    double s = 0.0;
    for (int i = 0; i < nv; ++i) {
        double v0[3], v1[3];
        sphere_tangent(ons[i], ons[(i - 1 + nv) % nv], v0);
        sphere_tangent(ons[i], ons[(i + 1) % nv], v1);
        s += acos(v0[0] * v1[0] + v0[1] * v1[1] + v0[2] * v1[2]);
    }
    double factor = s - (nv - 2) * SP_PI;
    return factor / (SP_PI * area);
}

namespace {

// universal.py:98-147 `_source2patch_energy_universal` fused with
// RadiosityFast.py:988-1034 `_add_directional`.
__global__ void k_source_energy(const double* __restrict__ src, int n, const double* __restrict__ centers,
                                const double* __restrict__ pts, int nv, const uint8_t* __restrict__ vis, int nb,
                                const double* __restrict__ att, const int32_t* __restrict__ wall_of,
                                const int32_t* __restrict__ brdf_index, int n_in, const double* __restrict__ dirs_in,
                                int n_out, const double* __restrict__ brdf, double* __restrict__ e0,
                                double* __restrict__ d0, double* __restrict__ e0dir) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s[3] = {src[0], src[1], src[2]};
    double c[3] = {centers[3 * j], centers[3 * j + 1], centers[3 * j + 2]};
    double dist = 0.0, g = 0.0;
    bool v = vis[j] != 0;
    if (v) {
        double dv[3] = {xsub(s[0], c[0]), xsub(s[1], c[1]), xsub(s[2], c[2])};
        dist = xnorm3(dv);
        g = sp_pt_solution(s, pts + (size_t)j * 3 * nv, nv, 0);
    }
    d0[j] = dist;
    int w = wall_of[j];
    int slot = brdf_index[w];
    // get_scattering_data_source(pos_h = source, pos_i = c_j): unit(source - c_j)
    int sidx = sp_nearest_dir(c, s, dirs_in + (size_t)w * n_in * 3, n_in);
    const double* row = brdf + ((size_t)slot * n_in + sidx) * n_out * nb;
    for (int b = 0; b < nb; ++b) {
        double e = v ? exp(-att[b] * dist) * g : 0.0;
        e0[(size_t)j * nb + b] = e;
        for (int o = 0; o < n_out; ++o) e0dir[((size_t)j * n_out + o) * nb + b] = e * row[(size_t)o * nb + b];
    }
}

// Receiver side of RadiosityFast.py:711-738: per patch the point-to-patch
// factor (universal.py:149-160), the outgoing direction toward the receiver
// (get_scattering_data_receiver_index with pos_j = receiver) and the
// patch-receiver distance (:712, :745).
__global__ void k_receiver_factors(const double* __restrict__ rcv, int n, const double* __restrict__ centers,
                                   const double* __restrict__ pts, int nv, const uint8_t* __restrict__ vis,
                                   const int32_t* __restrict__ wall_of, int n_out, const double* __restrict__ dirs_out,
                                   double* __restrict__ rfac, int32_t* __restrict__ ridx, double* __restrict__ dist) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double r[3] = {rcv[0], rcv[1], rcv[2]};
    double c[3] = {centers[3 * k], centers[3 * k + 1], centers[3 * k + 2]};
    rfac[k] = vis[k] ? sp_pt_solution(r, pts + (size_t)k * 3 * nv, nv, 1) : 0.0;
    ridx[k] = sp_nearest_dir(c, r, dirs_out + (size_t)wall_of[k] * n_out * 3, n_out);
    double dv[3] = {xsub(c[0], r[0]), xsub(c[1], r[1]), xsub(c[2], r[2])};
    dist[k] = xnorm3(dv);
}

}  // namespace

extern "C" {

int sp_source_energy(const double* src, int n, const double* centers, const double* pts, int nv, const uint8_t* vis,
                     int nb, const double* att, const int32_t* wall_of, const int32_t* brdf_index, int n_in,
                     const double* dirs_in, int n_out, const double* brdf, double* e0, double* d0, double* e0dir,
                     void* stream) {
    if (n < 0 || nb < 1 || n_in < 1 || n_out < 1 || nv < 3 || nv > kMaxPolyVerts) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    if (!src || !centers || !pts || !vis || !att || !wall_of || !brdf_index || !dirs_in || !brdf || !e0 || !d0 || !e0dir)
        return SP_ERR_ARG;
    k_source_energy<<<sp_blocks(n, 128), 128, 0, sp_counted((cudaStream_t)stream)>>>(
        src, n, centers, pts, nv, vis, nb, att, wall_of, brdf_index, n_in, dirs_in, n_out, brdf, e0, d0, e0dir);
    return sp_check_launch();
}

int sp_receiver_factors(const double* rcv, int n, const double* centers, const double* pts, int nv,
                        const uint8_t* vis, const int32_t* wall_of, int n_out, const double* dirs_out, double* rfac,
                        int32_t* ridx, double* dist, void* stream) {
    if (n < 0 || n_out < 1 || nv < 3 || nv > kMaxPolyVerts) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    if (!rcv || !centers || !pts || !vis || !wall_of || !dirs_out || !rfac || !ridx || !dist) return SP_ERR_ARG;
    k_receiver_factors<<<sp_blocks(n, 128), 128, 0, sp_counted((cudaStream_t)stream)>>>(
        rcv, n, centers, pts, nv, vis, wall_of, n_out, dirs_out, rfac, ridx, dist);
    return sp_check_launch();
}

size_t sp_form_factors_workspace(int n_patches, long long n_pairs) {
    return sp_align((size_t)n_patches * sizeof(PatchStokes)) + sp_align((size_t)n_patches * kPatchF * 4) +
           sp_align(((size_t)n_pairs + 1) * 8) + sp_align((size_t)n_pairs * sizeof(float4)) +
           sp_align((size_t)n_pairs * sizeof(float2)) + 256;
}

int sp_form_factors(int precision, int n_patches, int nv, long long n_pairs, const int32_t* pairs, const double* pts,
                    const double* normals, const double* areas, double* ff, uint8_t* method, void* ws,
                    size_t ws_bytes, void* stream) {
    if (n_pairs < 0 || n_patches < 0 || (precision != SP_F32 && precision != SP_F64)) return SP_ERR_ARG;
    if (nv < 3 || nv > kMaxPolyVerts) return SP_ERR_ARG;
    if (n_pairs == 0) return SP_OK;
    if (!pairs || !pts || !normals || !areas || !ff) return SP_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (nv > 4 || (nv == 3 && (precision == SP_F64 || !method))) {  // FP64, one warp per pair
        k_form_factors_poly<<<sp_blocks(n_pairs * 32, 256), 256, 0, sp_counted(st)>>>(n_pairs, nv, pairs, pts,
                                                                                      normals, areas, ff, method);
        return sp_check_launch();
    }
    if (precision == SP_F64 || !method) {
        long long threads = n_pairs * 32;
        k_form_factors<<<sp_blocks(threads, 256), 256, 0, sp_counted(st)>>>(n_pairs, pairs, pts, normals, areas, ff,
                                                                           method);
        return sp_check_launch();
    }
    if (!ws || ws_bytes < sp_form_factors_workspace(n_patches, n_pairs)) return SP_ERR_WORKSPACE;
    char* q = (char*)ws;
    PatchStokes* pd = (PatchStokes*)q;
    q += sp_align((size_t)n_patches * sizeof(PatchStokes));
    float* pf = (float*)q;
    q += sp_align((size_t)n_patches * kPatchF * 4);
    int64_t* rework = (int64_t*)q;
    q += sp_align(((size_t)n_pairs + 1) * 8);
    float4* geo = (float4*)q;
    q += sp_align((size_t)n_pairs * sizeof(float4));
    float2* acc = (float2*)q;
    q += sp_align((size_t)n_pairs * sizeof(float2));
    unsigned long long* n_rework = (unsigned long long*)q;
    cudaMemsetAsync(n_rework, 0, sizeof(unsigned long long), st);
    const long long warps = ((long long)n_patches + 1) / 2;
    k_ff_patch_data<<<sp_blocks(warps * 32, 256), 256, 0, sp_counted(st)>>>(n_patches, nv, pts, pd, pf);
    k_ff_base<<<sp_blocks(n_pairs, 128), 128, 0, sp_counted(st)>>>(n_pairs, nv, pairs, pts, pd, ff, method, geo,
                                                                  n_rework, rework);
    k_ff_phi<<<sp_blocks(n_pairs * 32, 256), 256, 0, sp_counted(st)>>>(n_pairs, pairs, geo, pf, acc, method,
                                                                      n_rework, rework);
    k_ff_finish<<<sp_blocks(n_pairs, 256), 256, 0, sp_counted(st)>>>(n_pairs, pairs, acc, areas, method, ff,
                                                                    n_rework, rework);
    unsigned long long count = 0;
    cudaMemcpyAsync(&count, n_rework, sizeof(count), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
    if (count > (unsigned long long)n_pairs) return SP_ERR_CUDA;
    if (count > 0)
        k_ff_rework<<<sp_blocks((long long)count * 32, 256), 256, 0, sp_counted(st)>>>(
            (long long)count, nv, rework, pairs, pts, normals, areas, ff, method);
    return sp_check_launch();
}

}  // extern "C"
