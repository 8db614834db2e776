// Geometry kernels: patch centres/areas, patch<->patch and point<->patch
// visibility, visible-pair compaction and the destination-major pair list.
//
// The visibility predicate is evaluated in FP64 with the reference's exact
// operation order (no fused multiply-add) so that the boolean result equals
// the reference's on inputs in generic position.  A conservative FP32
// segment-vs-box test, over groups of 32 consecutive blockers and then over
// single blockers, decides which blockers need the exact test at all: a
// blocker whose (slightly enlarged) bounding box the segment misses can only
// return "visible" in the reference predicate (see exact_visibility below).
#include <atomic>
#include <vector>

#include "common.cuh"
#include "exchange_common.cuh"

namespace {

constexpr int kGroup = 32;       // blockers per culling group
constexpr int kMaxVerts = 8;     // polygon vertices supported by the predicate

// geometry.py:498-559 `_rotation_matrix(n_in)` with n_out = (0, 0, 1).
__device__ void rotation_matrix(const double* n_in, double* m) {
    if (n_in[0] == 0.0 && n_in[1] == 0.0 && n_in[2] == 1.0) {
        for (int i = 0; i < 9; ++i) m[i] = (i % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    double nn = xnorm3(n_in);
    double a[3] = {xdiv(n_in[0], nn), xdiv(n_in[1], nn), xdiv(n_in[2], nn)};
    double b[3] = {0.0, 0.0, 1.0};
    double c = xdot3(a, b);
    if (c != -1.0) {
        double v[3];
        xcross3(a, b, v);
        double s = xnorm3(v);
        double k[9] = {0.0, -v[2], v[1], v[2], 0.0, -v[0], -v[1], v[0], 0.0};
        double f = xdiv(xsub(1.0, c), xmul(s, s));
        for (int r = 0; r < 3; ++r)
            for (int col = 0; col < 3; ++col) {
                double kk = xadd(xadd(xmul(k[r * 3 + 0], k[0 * 3 + col]), xmul(k[r * 3 + 1], k[1 * 3 + col])),
                                 xmul(k[r * 3 + 2], k[2 * 3 + col]));
                double id = (r == col) ? 1.0 : 0.0;
                m[r * 3 + col] = xadd(xadd(id, k[r * 3 + col]), xmul(kk, f));
            }
    } else {
        const double flip[9] = {-1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, -1.0};
        for (int i = 0; i < 9; ++i) m[i] = flip[i];
    }
}

// geometry.py:614-686 `_point_in_polygon` (winding number, eta = 1e-6).
__device__ bool point_in_polygon(const double* p3, const double* poly3, int nv, const double* n) {
    const double eta = 1e-6;
    double d0[3] = {xsub(p3[0], poly3[0]), xsub(p3[1], poly3[1]), xsub(p3[2], poly3[2])};
    if (fabs(xdot3(d0, n)) > eta) return false;
    double rot[9];
    rotation_matrix(n, rot);
    double pt[2] = {xdot3(rot, p3), xdot3(rot + 3, p3)};
    double poly[kMaxVerts][2];
    for (int i = 0; i < nv; ++i) {
        poly[i][0] = xdot3(rot, poly3 + 3 * i);
        poly[i][1] = xdot3(rot + 3, poly3 + 3 * i);
    }
    int count = 0;
    for (int i = 0; i < nv; ++i) {
        const double* a1 = poly[(i + 1) % nv];
        const double* a0 = poly[i];
        double side[2] = {xsub(a1[0], a0[0]), xsub(a1[1], a0[1])};
        double ns = xnorm2(side);
        double nl[2] = {xdiv(-side[1], ns), xdiv(side[0], ns)};
        double point[2] = {xadd(pt[0], 1.0), xadd(pt[1], 0.0)};
        double v[2] = {xsub(point[0], pt[0]), xsub(point[1], pt[1])};
        double dp = xdot2(v, nl);
        if (!(fabs(dp) > 1e-6)) continue;
        double w[2] = {xsub(point[0], a1[0]), xsub(point[1], a1[1])};
        double fac = -xdiv(xdot2(nl, w), dp);
        double b[2] = {xadd(xadd(w[0], a1[0]), xmul(fac, v[0])), xadd(xadd(w[1], a1[1]), xmul(fac, v[1]))};
        if (b[0] > pt[0]) {
            double ba0[2] = {xsub(b[0], a0[0]), xsub(b[1], a0[1])};
            double ba1[2] = {xsub(b[0], a1[0]), xsub(b[1], a1[1])};
            double a10[2] = {xsub(a1[0], a0[0]), xsub(a1[1], a0[1])};
            if (fabs(xsub(xadd(xnorm2(ba0), xnorm2(ba1)), xnorm2(a10))) <= eta) {
                double bp[2] = {xsub(b[0], pt[0]), xsub(b[1], pt[1])};
                double s = xdot2(bp, nl);
                if (s > 0)
                    count += 1;
                else if (s < 0)
                    count -= 1;
            }
        }
    }
    return count != 0;
}

// geometry.py:841-909 `_basic_visibility` (with _project_to_plane :561-612).
__device__ bool exact_visibility(const double* vp, const double* ep, const double* sp, int nv, const double* n) {
    const double eta = 1e-6;
    bool vis_in = point_in_polygon(vp, sp, nv, n);
    bool eval_in = point_in_polygon(ep, sp, nv, n);
    if (!vis_in && !eval_in) {
        double v[3] = {xsub(ep[0], vp[0]), xsub(ep[1], vp[1]), xsub(ep[2], vp[2])};
        double dp = xdot3(v, n);
        if (fabs(dp) > 1e-6) {
            double w[3] = {xsub(ep[0], sp[0]), xsub(ep[1], sp[1]), xsub(ep[2], sp[2])};
            double fac = -xdiv(xdot3(n, w), dp);
            double pt[3];
            for (int d = 0; d < 3; ++d) pt[d] = xadd(xadd(w[d], sp[d]), xmul(fac, v[d]));
            if (point_in_polygon(pt, sp, nv, n)) {
                double a[3] = {xsub(pt[0], vp[0]), xsub(pt[1], vp[1]), xsub(pt[2], vp[2])};
                double b[3] = {xsub(pt[0], ep[0]), xsub(pt[1], ep[1]), xsub(pt[2], ep[2])};
                if (xdot3(a, b) < 0) return false;
            }
        }
        return true;
    }
    // geometry.py:895-906: each elif includes its half-space test, so a
    // failed test falls through to the coplanar case
    if (vis_in && !eval_in) {
        double d[3] = {xsub(ep[0], vp[0]), xsub(ep[1], vp[1]), xsub(ep[2], vp[2])};
        if (xdot3(n, d) < 0) return false;
    } else if (!vis_in && eval_in) {
        double d[3] = {xsub(vp[0], ep[0]), xsub(vp[1], ep[1]), xsub(vp[2], ep[2])};
        if (xdot3(n, d) < 0) return false;
    }
    double a[3] = {xsub(vp[0], sp[0]), xsub(vp[1], sp[1]), xsub(vp[2], sp[2])};
    double b[3] = {xsub(ep[0], sp[0]), xsub(ep[1], sp[1]), xsub(ep[2], sp[2])};
    return !(fabs(xdot3(a, n)) < eta && fabs(xdot3(b, n)) < eta);
}

// The blocker-only part of point_in_polygon, computed once per patch with
// the same FP64 operations: the first two rows of the rotation to the
// horizontal plane, the rotated vertices, and per edge the unit normal nl
// and the length |a1 - a0|.
struct PolyPre {
    double r[6];
    double a[kMaxVerts][2];
    double nl[kMaxVerts][2];
    double ns[kMaxVerts];
};

__device__ void poly_pre(const double* poly3, int nv, const double* n, PolyPre& P) {
    double rot[9];
    rotation_matrix(n, rot);
    for (int k = 0; k < 6; ++k) P.r[k] = rot[k];
    for (int i = 0; i < nv; ++i) {
        P.a[i][0] = xdot3(rot, poly3 + 3 * i);
        P.a[i][1] = xdot3(rot + 3, poly3 + 3 * i);
    }
    for (int i = 0; i < nv; ++i) {
        const double* a1 = P.a[(i + 1) % nv];
        const double* a0 = P.a[i];
        const double side[2] = {xsub(a1[0], a0[0]), xsub(a1[1], a0[1])};
        const double ns = xnorm2(side);
        P.ns[i] = ns;
        P.nl[i][0] = xdiv(-side[1], ns);
        P.nl[i][1] = xdiv(side[0], ns);
    }
}

// point_in_polygon with the blocker part from poly_pre (bit-identical).
__device__ bool point_in_polygon_pre(const double* p3, const double* v0, const double* n, const PolyPre& P, int nv) {
    const double eta = 1e-6;
    const double d0[3] = {xsub(p3[0], v0[0]), xsub(p3[1], v0[1]), xsub(p3[2], v0[2])};
    if (fabs(xdot3(d0, n)) > eta) return false;
    const double pt[2] = {xdot3(P.r, p3), xdot3(P.r + 3, p3)};
    int count = 0;
    for (int i = 0; i < nv; ++i) {
        const double* a1 = P.a[(i + 1) % nv];
        const double* a0 = P.a[i];
        const double* nl = P.nl[i];
        const double point[2] = {xadd(pt[0], 1.0), xadd(pt[1], 0.0)};
        const double v[2] = {xsub(point[0], pt[0]), xsub(point[1], pt[1])};
        const double dp = xdot2(v, nl);
        if (!(fabs(dp) > 1e-6)) continue;
        const double w[2] = {xsub(point[0], a1[0]), xsub(point[1], a1[1])};
        const double fac = -xdiv(xdot2(nl, w), dp);
        const double b[2] = {xadd(xadd(w[0], a1[0]), xmul(fac, v[0])), xadd(xadd(w[1], a1[1]), xmul(fac, v[1]))};
        if (b[0] > pt[0]) {
            const double ba0[2] = {xsub(b[0], a0[0]), xsub(b[1], a0[1])};
            const double ba1[2] = {xsub(b[0], a1[0]), xsub(b[1], a1[1])};
            if (fabs(xsub(xadd(xnorm2(ba0), xnorm2(ba1)), P.ns[i])) <= eta) {
                const double bp[2] = {xsub(b[0], pt[0]), xsub(b[1], pt[1])};
                const double sgn = xdot2(bp, nl);
                if (sgn > 0)
                    count += 1;
                else if (sgn < 0)
                    count -= 1;
            }
        }
    }
    return count != 0;
}

// exact_visibility with the blocker part from poly_pre (bit-identical); v0 =
// the blocker's first vertex.
__device__ bool exact_visibility_pre(const double* vp, const double* ep, const double* v0, const double* n,
                                     const PolyPre& P, int nv) {
    const double eta = 1e-6;
    const bool vis_in = point_in_polygon_pre(vp, v0, n, P, nv);
    const bool eval_in = point_in_polygon_pre(ep, v0, n, P, nv);
    if (!vis_in && !eval_in) {
        const double v[3] = {xsub(ep[0], vp[0]), xsub(ep[1], vp[1]), xsub(ep[2], vp[2])};
        const double dp = xdot3(v, n);
        if (fabs(dp) > 1e-6) {
            const double w[3] = {xsub(ep[0], v0[0]), xsub(ep[1], v0[1]), xsub(ep[2], v0[2])};
            const double fac = -xdiv(xdot3(n, w), dp);
            double pt[3];
            for (int d = 0; d < 3; ++d) pt[d] = xadd(xadd(w[d], v0[d]), xmul(fac, v[d]));
            if (point_in_polygon_pre(pt, v0, n, P, nv)) {
                const double a[3] = {xsub(pt[0], vp[0]), xsub(pt[1], vp[1]), xsub(pt[2], vp[2])};
                const double b[3] = {xsub(pt[0], ep[0]), xsub(pt[1], ep[1]), xsub(pt[2], ep[2])};
                if (xdot3(a, b) < 0) return false;
            }
        }
        return true;
    }
    if (vis_in && !eval_in) {
        const double d[3] = {xsub(ep[0], vp[0]), xsub(ep[1], vp[1]), xsub(ep[2], vp[2])};
        if (xdot3(n, d) < 0) return false;
    } else if (!vis_in && eval_in) {
        const double d[3] = {xsub(vp[0], ep[0]), xsub(vp[1], ep[1]), xsub(vp[2], ep[2])};
        if (xdot3(n, d) < 0) return false;
    }
    const double a[3] = {xsub(vp[0], v0[0]), xsub(vp[1], v0[1]), xsub(vp[2], v0[2])};
    const double b[3] = {xsub(ep[0], v0[0]), xsub(ep[1], v0[1]), xsub(ep[2], v0[2])};
    return !(fabs(xdot3(a, n)) < eta && fabs(xdot3(b, n)) < eta);
}

// Conservative segment/box overlap in FP32.  Boxes are already enlarged by a
// margin that covers the predicate's 1e-6 tolerances and the FP32 rounding
// of the segment end points, so a miss here proves the exact predicate
// returns "visible" for every blocker inside the box.
// d holds the segment direction in d[0..2] and its reciprocals in d[3..5]
// (seg_reciprocals, once per segment).
__device__ __forceinline__ void seg_reciprocals(float* d) {
#pragma unroll
    for (int k = 0; k < 3; ++k) d[3 + k] = d[k] != 0.0f ? 1.0f / d[k] : 0.0f;
}
__device__ __forceinline__ bool seg_hits_box(const float* a, const float* d, const float* lo, const float* hi) {
    float t0 = 0.0f, t1 = 1.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (d[k] == 0.0f) {
            if (a[k] < lo[k] || a[k] > hi[k]) return false;
        } else {
            const float inv = d[3 + k];
            float ta = (lo[k] - a[k]) * inv, tb = (hi[k] - a[k]) * inv;
            float tn = fminf(ta, tb), tx = fmaxf(ta, tb);
            t0 = fmaxf(t0, tn);
            t1 = fminf(t1, tx);
        }
    }
    return t0 <= t1 + 1e-5f;
}

__global__ void k_patch_geometry(int n, int nv, const double* __restrict__ pts, double* __restrict__ centers,
                                 double* __restrict__ areas) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* p = pts + (size_t)i * nv * 3;
    // geometry.py:412-413 `_calculate_center`: sequential sum then divide.
    for (int d = 0; d < 3; ++d) {
        double s = p[d];
        for (int k = 1; k < nv; ++k) s = xadd(s, p[3 * k + d]);
        centers[3 * i + d] = xdiv(s, (double)nv);
    }
    // geometry.py:420-448 `_polygon_area` (fan from vertex 0).
    double area = 0.0;
    for (int t = 0; t < nv - 2; ++t) {
        const double* p1 = p + 3 * (t + 1);
        const double* p2 = p + 3 * (t + 2);
        double a[3] = {xsub(p1[0], p[0]), xsub(p1[1], p[1]), xsub(p1[2], p[2])};
        double b[3] = {xsub(p2[0], p[0]), xsub(p2[1], p[1]), xsub(p2[2], p[2])};
        double c[3];
        xcross3(a, b, c);
        area = xadd(area, xmul(0.5, xnorm3(c)));
    }
    areas[i] = area;
}

// Enlarged FP32 bounding boxes of every blocker and of every group of
// kGroup consecutive blockers.  box layout: lo[3], hi[3].
__global__ void k_blocker_boxes(int n, int nv, const double* __restrict__ pts, float margin,
                                float* __restrict__ box, float* __restrict__ gbox) {
    int g = blockIdx.x;
    int lane = threadIdx.x;  // blockDim == kGroup
    int s = g * kGroup + lane;
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    if (s < n) {
        for (int k = 0; k < nv; ++k)
            for (int d = 0; d < 3; ++d) {
                double v = pts[((size_t)s * nv + k) * 3 + d];
                lo[d] = fminf(lo[d], __double2float_rd(v));
                hi[d] = fmaxf(hi[d], __double2float_ru(v));
            }
        for (int d = 0; d < 3; ++d) {
            float m = margin + 4e-6f * fmaxf(fabsf(lo[d]), fabsf(hi[d]));
            lo[d] -= m;
            hi[d] += m;
            box[6 * s + d] = lo[d];
            box[6 * s + 3 + d] = hi[d];
        }
    }
    for (int d = 0; d < 3; ++d) {
        for (int off = 16; off > 0; off >>= 1) {
            lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], off));
            hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], off));
        }
    }
    if (lane == 0)
        for (int d = 0; d < 3; ++d) {
            gbox[6 * g + d] = lo[d];
            gbox[6 * g + 3 + d] = hi[d];
        }
}

// geometry.py:750-797 `_check_patch2patch_visibility`.  One thread per pair
// (i < j) of a 16 x 16 pair tile; blockers are all patches.
__global__ void __launch_bounds__(256) k_patch_visibility(int n, int nv, const double* __restrict__ centers,
                                                          const double* __restrict__ normals,
                                                          const double* __restrict__ pts,
                                                          const float* __restrict__ box,
                                                          const float* __restrict__ gbox, int n_groups,
                                                          uint8_t* __restrict__ vis) {
    extern __shared__ float s_gbox[];
    int tile_i = blockIdx.y, tile_j = blockIdx.x;
    if (tile_j < tile_i) return;  // whole tile below the diagonal
    int i = tile_i * 16 + (threadIdx.x >> 4);
    int j = tile_j * 16 + (threadIdx.x & 15);
    bool active = (i < n) && (j < n) && (i < j);
    double ci[3] = {0, 0, 0}, cj[3] = {0, 0, 0};
    float a[3] = {0, 0, 0}, d[6] = {0, 0, 0, 0, 0, 0};
    if (active) {
        for (int k = 0; k < 3; ++k) {
            ci[k] = centers[3 * i + k];
            cj[k] = centers[3 * j + k];
            a[k] = (float)ci[k];
            d[k] = (float)cj[k] - a[k];
        }
        seg_reciprocals(d);
    }
    bool visible = true;
    for (int g0 = 0; g0 < n_groups; g0 += 1024) {
        int cnt = min(1024, n_groups - g0);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt * 6; t += blockDim.x) s_gbox[t] = gbox[6 * g0 + t];
        __syncthreads();
        if (!active || !visible) continue;
        for (int g = 0; g < cnt && visible; ++g) {
            if (!seg_hits_box(a, d, s_gbox + 6 * g, s_gbox + 6 * g + 3)) continue;
            int s_end = min(n, (g0 + g + 1) * kGroup);
            for (int s = (g0 + g) * kGroup; s < s_end; ++s) {
                const float* bx = box + 6 * s;
                float lo[3] = {bx[0], bx[1], bx[2]}, hi[3] = {bx[3], bx[4], bx[5]};
                if (!seg_hits_box(a, d, lo, hi)) continue;
                double nn[3] = {normals[3 * s], normals[3 * s + 1], normals[3 * s + 2]};
                double sp[kMaxVerts * 3];
                for (int k = 0; k < nv * 3; ++k) sp[k] = pts[(size_t)s * nv * 3 + k];
                if (!exact_visibility(ci, cj, sp, nv, nn)) {
                    visible = false;
                    break;
                }
            }
        }
    }
    if (i < n && j < n) vis[(size_t)i * n + j] = (active && visible) ? 1 : 0;
}

// Patch visibility in steps that keep the FP64 predicate on full warps:
// k_vis_self (the pair's own patches as blockers), then k_vis_cull (one
// 16 x 16 pair tile per block, one pair per thread) writes, after the FP32
// box culling, the (pair, blocker) candidates to a buffer, each warp
// reserving room per blocker group with one atomic; k_vis_exact evaluates
// one candidate per thread and clears the pair when the blocker hides it
// (visibility is the AND over blockers, so the order of evaluation does not
// change the result).  A tile whose candidates do not all fit is culled
// again in a later round.
constexpr int kCandBits = 20;  // i, j, s < 2^20
// Per patch: whether its centre lies inside it (the winding test of
// `_point_in_polygon`) and within eta of its plane, each in the reference
// predicate's arithmetic.  Both hold for every non-degenerate patch.
__global__ void k_own_patch(int n, int nv, const double* __restrict__ centers, const double* __restrict__ normals,
                            const double* __restrict__ pts, uint8_t* __restrict__ own_ok) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double c[3], nn[3], sp[kMaxVerts * 3];
    for (int q = 0; q < 3; ++q) {
        c[q] = centers[3 * i + q];
        nn[q] = normals[3 * i + q];
    }
    for (int q = 0; q < nv * 3; ++q) sp[q] = pts[(size_t)i * nv * 3 + q];
    const double a[3] = {xsub(c[0], sp[0]), xsub(c[1], sp[1]), xsub(c[2], sp[2])};
    own_ok[i] = (point_in_polygon(c, sp, nv, nn) && fabs(xdot3(a, nn)) < 1e-6) ? 1 : 0;
}

// exact_visibility for a blocker that is the patch of one end point, in
// closed form.  With own_ok for that patch (its centre inside it and on its
// plane), `_basic_visibility` (geometry.py:841-909) depends only on h, the
// distance of the other end point from the blocker's plane as
// `_point_in_polygon` computes it:
//   h > eta: that point is outside the blocker (no winding test), so the
//            segment is hidden iff it leaves the blocker's front side
//            (the vis_in / eval_in branch with its half-space test);
//   h < eta: both points are coplanar with the blocker and one is inside it:
//            hidden, whatever the winding test of the other point gives.
// Returns 1 visible, 0 hidden, -1 when exact_visibility has to decide
// (a degenerate patch, or h == eta).
__device__ __forceinline__ int own_patch_test(const double* vp, const double* ep, bool blocker_of_vp,
                                              const double* p0, const double* n, bool own_ok) {
    if (!own_ok) return -1;
    const double* other = blocker_of_vp ? ep : vp;
    const double d0[3] = {xsub(other[0], p0[0]), xsub(other[1], p0[1]), xsub(other[2], p0[2])};
    const double h = fabs(xdot3(d0, n));
    if (h > 1e-6) {
        const double* from = blocker_of_vp ? vp : ep;
        const double d[3] = {xsub(other[0], from[0]), xsub(other[1], from[1]), xsub(other[2], from[2])};
        return xdot3(n, d) < 0 ? 0 : 1;
    }
    return h < 1e-6 ? 0 : -1;
}

// The pair's own patches as blockers first: they hide every coplanar pair,
// whose segments would otherwise cross the boxes of all patches between
// them.  Two closed-form tests per pair (own_patch_test), the full predicate
// only where they cannot decide.  Writes the base value.
__global__ void __launch_bounds__(256) k_vis_self(int n, int nv, const int32_t* __restrict__ tiles,
                                                  const double* __restrict__ centers,
                                                  const double* __restrict__ normals, const double* __restrict__ pts,
                                                  const uint8_t* __restrict__ own_ok, uint8_t* __restrict__ vis) {
    const int tile = tiles[blockIdx.x];
    const int tile_i = tile >> 16, tile_j = tile & 0xffff;
    const int i = tile_i * 16 + (threadIdx.x >> 4);
    const int j = tile_j * 16 + (threadIdx.x & 15);
    if (i >= n || j >= n) return;
    bool visible = i < j;
    if (visible) {
        double ci[3], cj[3];
        for (int q = 0; q < 3; ++q) {
            ci[q] = centers[3 * i + q];
            cj[q] = centers[3 * j + q];
        }
        for (int k = 0; k < 2 && visible; ++k) {
            const int s = k == 0 ? i : j;
            double nn[3], p0[3];
            for (int q = 0; q < 3; ++q) {
                nn[q] = normals[3 * s + q];
                p0[q] = pts[(size_t)s * nv * 3 + q];
            }
            int r = own_patch_test(ci, cj, k == 0, p0, nn, own_ok[s] != 0);
            if (r < 0) {
                double sp[kMaxVerts * 3];
                for (int q = 0; q < nv * 3; ++q) sp[q] = pts[(size_t)s * nv * 3 + q];
                r = exact_visibility(ci, cj, sp, nv, nn) ? 1 : 0;
            }
            visible = r != 0;
        }
    }
    vis[(size_t)i * n + j] = visible ? 1 : 0;
}

// One pass: the warps of a 16 x 16 pair tile walk the blocker groups
// together.  Per group, a lane whose segment meets the group's box tests its
// 32 blockers (bit mask of box hits, the pair's own patches left out); the
// warp then reserves room for all its lanes' hits with one atomic (shuffle
// prefix sum) and writes them.  A reservation that would pass `cap` is not
// written and marks the tile for the next round, where it is culled again
// in full (candidates written twice are harmless: visibility is an AND).
__global__ void __launch_bounds__(256) k_vis_cull(int n, const int32_t* __restrict__ tiles,
                                                  const double* __restrict__ centers, const float* __restrict__ box,
                                                  const float* __restrict__ gbox, int n_groups,
                                                  uint8_t* __restrict__ vis, int64_t* __restrict__ cand,
                                                  long long cap, unsigned long long* __restrict__ counter,
                                                  int32_t* __restrict__ overflow, int* __restrict__ n_overflow) {
    extern __shared__ float s_gbox[];
    __shared__ int s_over;
    const int tile = tiles[blockIdx.x];
    const int tile_i = tile >> 16, tile_j = tile & 0xffff;
    const int i = tile_i * 16 + (threadIdx.x >> 4);
    const int j = tile_j * 16 + (threadIdx.x & 15);
    const int lane = threadIdx.x & 31;
    // pairs the own-patch pass (k_vis_self) already hid need no candidates
    const bool active = (i < n) && (j < n) && (i < j) && vis[(size_t)i * n + j] != 0;
    float a[3] = {0, 0, 0}, d[6] = {0, 0, 0, 0, 0, 0};
    if (active) {
        for (int k = 0; k < 3; ++k) {
            a[k] = (float)centers[3 * i + k];
            d[k] = (float)centers[3 * j + k] - a[k];
        }
        seg_reciprocals(d);
    }
    const int64_t code = ((int64_t)i << (2 * kCandBits)) | ((int64_t)j << kCandBits);
    if (threadIdx.x == 0) s_over = 0;
    for (int g0 = 0; g0 < n_groups; g0 += 1024) {
        const int cnt = min(1024, n_groups - g0);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt * 6; t += blockDim.x) s_gbox[t] = gbox[6 * g0 + t];
        __syncthreads();
        for (int g = 0; g < cnt; ++g) {
            const int s0 = (g0 + g) * kGroup;
            uint32_t mask = 0;
            if (active && seg_hits_box(a, d, s_gbox + 6 * g, s_gbox + 6 * g + 3)) {
                const int s_end = min(n, s0 + kGroup);
                for (int s = s0; s < s_end; ++s) {
                    const float* bx = box + 6 * s;
                    const float lo[3] = {bx[0], bx[1], bx[2]}, hi[3] = {bx[3], bx[4], bx[5]};
                    if (s != i && s != j && seg_hits_box(a, d, lo, hi)) mask |= 1u << (s - s0);
                }
            }
            if (__ballot_sync(0xffffffffu, mask != 0u) == 0u) continue;  // the same for the whole warp
            const int h = __popc(mask);
            int incl = h;
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += y;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            unsigned long long base = 0;
            if (lane == 31) base = atomicAdd(counter, (unsigned long long)total);
            base = __shfl_sync(0xffffffffu, base, 31);
            if (base + (unsigned long long)total > (unsigned long long)cap) {
                if (lane == 0) s_over = 1;
                continue;
            }
            long long pos = (long long)base + incl - h;
            while (mask) {
                const int b = __ffs(mask) - 1;
                mask &= mask - 1u;
                cand[pos++] = code | (int64_t)(s0 + b);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_over) overflow[atomicAdd(n_overflow, 1)] = tile;
}

// Per patch: the blocker part of the predicate (poly_pre).
__global__ void k_poly_pre(int n, int nv, const double* __restrict__ normals, const double* __restrict__ pts,
                           PolyPre* __restrict__ pre) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    double nn[3] = {normals[3 * s], normals[3 * s + 1], normals[3 * s + 2]};
    double sp[kMaxVerts * 3];
    for (int q = 0; q < nv * 3; ++q) sp[q] = pts[(size_t)s * nv * 3 + q];
    PolyPre P;
    poly_pre(sp, nv, nn, P);
    pre[s] = P;
}

__global__ void k_vis_exact(long long count, const int64_t* __restrict__ cand, int n, int nv,
                            const double* __restrict__ centers, const double* __restrict__ normals,
                            const double* __restrict__ pts, const PolyPre* __restrict__ pre,
                            uint8_t* __restrict__ vis) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int64_t c = cand[k];
    if (c < 0) return;  // slot of a block that did not fit
    const int mask = (1 << kCandBits) - 1;
    const int i = (int)(c >> (2 * kCandBits)), j = (int)((c >> kCandBits) & mask), s = (int)(c & mask);
    uint8_t* v = vis + (size_t)i * n + j;
    if (*v == 0) return;  // already hidden by another blocker
    double ci[3], cj[3], nn[3], v0[3];
    for (int q = 0; q < 3; ++q) {
        ci[q] = centers[3 * i + q];
        cj[q] = centers[3 * j + q];
        nn[q] = normals[3 * s + q];
        v0[q] = pts[(size_t)s * nv * 3 + q];
    }
    if (!exact_visibility_pre(ci, cj, v0, nn, pre[s], nv)) *v = 0;
}

// geometry.py:799-839 `_check_point2patch_visibility`: point -> each patch
// centre, blockers are the given surfaces (walls), tested in index order.
// One thread per (point, patch); out is (n_points, n).
__global__ void k_point_visibility(long long n_points, const double* __restrict__ points, int n,
                                   const double* __restrict__ centers, int n_surf, int nv,
                                   const double* __restrict__ surf_pts, const double* __restrict__ surf_normals,
                                   const float* __restrict__ sbox, uint8_t* __restrict__ out) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_points * n) return;
    const long long p = q / n;
    const int i = (int)(q - p * n);
    const double* point = points + 3 * p;
    double vp[3] = {point[0], point[1], point[2]};
    double ep[3] = {centers[3 * i], centers[3 * i + 1], centers[3 * i + 2]};
    float a[3], d[6];
    for (int k = 0; k < 3; ++k) {
        a[k] = (float)vp[k];
        d[k] = (float)ep[k] - a[k];
    }
    seg_reciprocals(d);
    bool visible = true;
    for (int s = 0; s < n_surf && visible; ++s) {
        const float* bx = sbox + 6 * s;
        float lo[3] = {bx[0], bx[1], bx[2]}, hi[3] = {bx[3], bx[4], bx[5]};
        if (!seg_hits_box(a, d, lo, hi)) continue;
        double nn[3] = {surf_normals[3 * s], surf_normals[3 * s + 1], surf_normals[3 * s + 2]};
        double sp[kMaxVerts * 3];
        for (int k = 0; k < nv * 3; ++k) sp[k] = surf_pts[(size_t)s * nv * 3 + k];
        visible = exact_visibility(vp, ep, sp, nv, nn);
    }
    out[q] = visible ? 1 : 0;
}

// Row counts of a 0/1 matrix restricted to columns > row (upper) or all
// columns (full).  One block per row.
__global__ void k_row_counts(int n, const uint8_t* __restrict__ m, int upper, int32_t* __restrict__ counts) {
    int r = blockIdx.x;
    const uint8_t* row = m + (size_t)r * n;
    int c0 = upper ? r + 1 : 0;
    int cnt = 0;
    for (int c = c0 + threadIdx.x; c < n; c += blockDim.x) cnt += row[c] ? 1 : 0;
    for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    __shared__ int s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
        counts[r] = t;
    }
}

// Exclusive scan of n counts into offsets[0..n] (single block, 1024 threads).
__global__ void k_exclusive_scan(int n, const int32_t* __restrict__ counts, int64_t* __restrict__ offsets) {
    __shared__ int64_t s_part[1024];
    int tid = threadIdx.x;
    int per = (n + 1023) / 1024;
    int b = tid * per, e = min(n, b + per);
    int64_t loc = 0;
    for (int k = b; k < e; ++k) loc += counts[k];
    s_part[tid] = loc;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        int64_t v = (tid >= off) ? s_part[tid - off] : 0;
        __syncthreads();
        s_part[tid] += v;
        __syncthreads();
    }
    int64_t run = s_part[tid] - loc;
    for (int k = b; k < e; ++k) {
        offsets[k] = run;
        run += counts[k];
    }
    if (tid == 1023) offsets[n] = s_part[1023];
}

// Ordered fill: entry (r, c) of a 0/1 matrix goes to slot offsets[r] + rank.
// upper: pairs (r, c) with c > r written as int32 pairs + optional index map.
// full:  column index written to cols[] and the row to rows[].
__global__ void k_fill_rows(int n, const uint8_t* __restrict__ m, int upper, const int64_t* __restrict__ offsets,
                            int32_t* __restrict__ pairs, int32_t* __restrict__ index_map,
                            int32_t* __restrict__ cols, int32_t* __restrict__ rows) {
    int r = blockIdx.x;
    const uint8_t* row = m + (size_t)r * n;
    int c0 = upper ? r + 1 : 0;
    __shared__ int s_warp[32];
    __shared__ int64_t s_base;
    if (threadIdx.x == 0) s_base = offsets[r];
    __syncthreads();
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int cb = c0; cb < n; cb += blockDim.x) {
        int c = cb + threadIdx.x;
        bool on = (c < n) && row[c];
        unsigned bal = __ballot_sync(0xffffffffu, on);
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < nw; ++w) {
            if (w < warp) before += s_warp[w];
            total += s_warp[w];
        }
        if (on) {
            int64_t slot = s_base + before + __popc(bal & ((1u << lane) - 1u));
            if (upper) {
                pairs[2 * slot] = r;
                pairs[2 * slot + 1] = c;
                if (index_map) index_map[(size_t)r * n + c] = (int32_t)slot;
            } else {
                cols[slot] = c;
                rows[slot] = r;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) s_base += total;
        __syncthreads();
    }
}

// Symmetric visibility: S[i, j] = V[i, j] | V[j, i] (32 x 32 tiles).
__global__ void k_symmetrize(int n, const uint8_t* __restrict__ v, uint8_t* __restrict__ s) {
    __shared__ uint8_t tile[32][33];
    int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (int k = ty; k < 32; k += 8) {
        int r = bx + k, c = by + tx;  // read the transposed block V[bx.., by..]
        tile[k][tx] = (r < n && c < n) ? v[(size_t)r * n + c] : 0;
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        int r = by + k, c = bx + tx;
        if (r < n && c < n) s[(size_t)r * n + c] = (v[(size_t)r * n + c] | tile[tx][k]) ? 1 : 0;
    }
}

// Per directed pair (src i -> dst j): outgoing direction index of i toward j
// (RadiosityFast.py:402-414), incoming index used by the ff_tilde BRDF row
// (:1264-1268), centre distance (:538-543), the normalised-vector length
// used for air attenuation (:1252-1262) and F'_ij (:1255-1256).
// The reference argmin (sp_nearest_dir) decided in FP32 where that is
// provably the same index.  With unit direction vectors:
// * each FP32 unit(diff) component is within 5.1e-7 of the FP64 one (inputs
//   truncated to 2^-23, square sum, square root, reciprocal, product);
// * each difference a = dir - u is within 7.5e-7;
// * so each value sum a^2 (sum |a| <= 2 sqrt 3) is within 1.1e-5 of its
//   FP64 counterpart.
// When the two smallest FP32 values differ by more than kDirGap = 3e-5 >
// 2 x 1.1e-5, the smallest one is the unique FP64 minimum.
// Returns the index, or -1 when the gap is smaller (or not a number) and the
// FP64 loop has to decide.
constexpr float kDirGap = 3e-5f;
__device__ __forceinline__ int nearest_dir_f32(const double* diff, const double* __restrict__ dirs, int nd) {
    const float x = f64_trunc_f32(diff[0]), y = f64_trunc_f32(diff[1]), z = f64_trunc_f32(diff[2]);
    const float inv = 1.0f / sqrtf(x * x + y * y + z * z);
    const float u[3] = {x * inv, y * inv, z * inv};
    float b1 = __int_as_float(0x7f800000), b2 = b1;
    int i1 = 0;
    for (int o = 0; o < nd; ++o) {
        const float a = f64_trunc_f32(dirs[3 * o]) - u[0];
        const float b = f64_trunc_f32(dirs[3 * o + 1]) - u[1];
        const float c = f64_trunc_f32(dirs[3 * o + 2]) - u[2];
        const float v = a * a + b * b + c * c;
        if (v < b1) {
            b2 = b1;
            b1 = v;
            i1 = o;
        } else if (v < b2) {
            b2 = v;
        }
    }
    return (b2 - b1 > kDirGap) ? i1 : -1;
}

__global__ void k_pair_setup(long long n_dir, int n, const int32_t* __restrict__ src, const int32_t* __restrict__ dst,
                             const double* __restrict__ centers, const double* __restrict__ areas,
                             const int32_t* __restrict__ pair_index, const double* __restrict__ ff,
                             const int32_t* __restrict__ wall_of, int n_in, const double* __restrict__ dirs_in,
                             int n_out, const double* __restrict__ dirs_out, int32_t* __restrict__ out_dir,
                             int32_t* __restrict__ in_dir, double* __restrict__ dist, double* __restrict__ unit_len,
                             double* __restrict__ fprime) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_dir) return;
    int i = src[e], j = dst[e];
    double ci[3] = {centers[3 * i], centers[3 * i + 1], centers[3 * i + 2]};
    double cj[3] = {centers[3 * j], centers[3 * j + 1], centers[3 * j + 2]};
    int w = wall_of[i];
    double dv[3] = {xsub(ci[0], cj[0]), xsub(ci[1], cj[1]), xsub(ci[2], cj[2])};
    if (out_dir) {
        int o = 0;
        if (n_out > 0 && dirs_out) {
            const double* tab = dirs_out + (size_t)w * n_out * 3;
            const double fwd[3] = {xsub(cj[0], ci[0]), xsub(cj[1], ci[1]), xsub(cj[2], ci[2])};
            o = nearest_dir_f32(fwd, tab, n_out);
            if (o < 0) o = sp_nearest_dir(ci, cj, tab, n_out);
        }
        out_dir[e] = o;
    }
    if (in_dir) {
        int o = 0;
        if (n_in > 0 && dirs_in) {
            const double* tab = dirs_in + (size_t)w * n_in * 3;
            o = nearest_dir_f32(dv, tab, n_in);
            if (o < 0) o = sp_nearest_dir(cj, ci, tab, n_in);
        }
        in_dir[e] = o;
    }
    double dd = xnorm3(dv);
    dist[e] = dd;
    double u[3] = {xdiv(dv[0], dd), xdiv(dv[1], dd), xdiv(dv[2], dd)};
    unit_len[e] = xnorm3(u);
    double f;
    if (i < j) {
        f = ff[pair_index[(size_t)i * n + j]];
    } else {
        f = xdiv(xmul(ff[pair_index[(size_t)j * n + i]], areas[j]), areas[i]);
    }
    fprime[e] = f;
}

// Dense (N, N) outgoing-direction map with sentinel n_out where not visible
// (RadiosityFast.py:402-414): out[i, j] = p2o(i -> j).
__global__ void k_fill_i64(long long count, int64_t value, int64_t* __restrict__ out) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) out[e] = value;
}
__global__ void k_scatter_outdir(long long n_dir, int n, const int32_t* __restrict__ src, const int32_t* __restrict__ dst,
                                 const int32_t* __restrict__ out_dir, int64_t* __restrict__ out) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_dir) return;
    out[(size_t)src[e] * n + dst[e]] = out_dir[e];
}

__global__ void k_scatter_ff(long long n_pairs, int n, const int32_t* __restrict__ pairs, const double* __restrict__ ff,
                             double* __restrict__ out) {
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_pairs) return;
    out[(size_t)pairs[2 * q] * n + pairs[2 * q + 1]] = ff[q];
}

// RadiosityFast.py:1234-1272 `_form_factors_with_directivity_dim`, dense
// output (n, n, nd, nb): ((F' * exp(-att_b |u|)) * BRDF[slot_i, s_ij, o, b]).
__global__ void k_ff_tilde(long long n_dir, int n, int nd, int nb, int n_in, const int32_t* __restrict__ src,
                           const int32_t* __restrict__ dst, const int32_t* __restrict__ in_dir,
                           const double* __restrict__ fprime, const double* __restrict__ unit_len,
                           const double* __restrict__ att, const int32_t* __restrict__ wall_of,
                           const int32_t* __restrict__ brdf_index, const double* __restrict__ brdf,
                           double* __restrict__ out) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_dir) return;
    int i = src[e], j = dst[e];
    double* o_ = out + ((size_t)i * n + j) * nd * nb;
    const double* row = brdf ? brdf + ((size_t)brdf_index[wall_of[i]] * n_in + in_dir[e]) * nd * nb : nullptr;
    for (int o = 0; o < nd; ++o)
        for (int b = 0; b < nb; ++b) {
            double v = fprime[e];
            if (att) v = v * exp(-att[b] * unit_len[e]);
            if (row) v = v * row[(size_t)o * nb + b];
            o_[(size_t)o * nb + b] = v;
        }
}

}  // namespace

extern "C" {

int sp_dense_form_factors(long long n_pairs, int n, const int32_t* pairs, const double* ff, double* out,
                          void* stream) {
    if (n_pairs < 0 || n < 0 || (n > 0 && !out) || (n_pairs > 0 && (!pairs || !ff))) return SP_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (n > 0) cudaMemsetAsync(out, 0, (size_t)n * n * sizeof(double), st);
    if (n_pairs > 0) k_scatter_ff<<<sp_blocks(n_pairs, 256), 256, 0, sp_counted(st)>>>(n_pairs, n, pairs, ff, out);
    return sp_check_launch();
}

int sp_form_factors_tilde(long long n_dir, int n, int nd, int nb, int n_in, const int32_t* src, const int32_t* dst,
                          const int32_t* in_dir, const double* fprime, const double* unit_len, const double* att,
                          const int32_t* wall_of, const int32_t* brdf_index, const double* brdf, double* out,
                          void* stream) {
    if (n_dir < 0 || n < 0 || nd < 1 || nb < 1 || (n > 0 && !out)) return SP_ERR_ARG;
    if (brdf && (n_in < 1 || !in_dir || !wall_of || !brdf_index)) return SP_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (n > 0) cudaMemsetAsync(out, 0, (size_t)n * n * nd * nb * sizeof(double), st);
    if (n_dir > 0)
        k_ff_tilde<<<sp_blocks(n_dir, 128), 128, 0, sp_counted(st)>>>(n_dir, n, nd, nb, n_in, src, dst, in_dir, fprime, unit_len,
                                                          att, wall_of, brdf_index, brdf, out);
    return sp_check_launch();
}

int sp_patch_geometry(int n, int nv, const double* pts, double* centers, double* areas, void* stream) {
    if (n < 0 || nv < 3 || nv > kMaxVerts || (n > 0 && (!pts || !centers || !areas))) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    k_patch_geometry<<<sp_blocks(n, 128), 128, 0, sp_counted((cudaStream_t)stream)>>>(n, nv, pts, centers, areas);
    return sp_check_launch();
}

// Workspace: blocker boxes, group boxes, the candidate buffer (at least 256 n
// entries, so one tile always fits an empty buffer), two tile lists, counters.
inline long long vis_cand_capacity(int n) {
    const long long pairs = (long long)n * (n - 1) / 2;
    long long cap = pairs * 4;
    if (cap < 256LL * n) cap = 256LL * n;
    if (cap > (128LL << 20)) cap = (128LL << 20) > 256LL * n ? (128LL << 20) : 256LL * n;
    return cap;
}
inline long long vis_tile_count(int n) {
    const long long t = (n + 15) / 16;
    return t * (t + 1) / 2;
}

size_t sp_patch_visibility_workspace(int n) {
    if (n <= 0) return 256;
    size_t groups = ((size_t)n + kGroup - 1) / kGroup;
    return sp_align((size_t)n * 6 * sizeof(float) + groups * 6 * sizeof(float)) +
           sp_align((size_t)vis_cand_capacity(n) * 8) + 2 * sp_align((size_t)vis_tile_count(n) * 4) +
           sp_align((size_t)n) + sp_align((size_t)n * sizeof(PolyPre)) + 256;
}

int sp_patch_visibility(int n, int nv, const double* centers, const double* normals, const double* pts,
                        uint8_t* vis, void* ws, size_t ws_bytes, void* stream) {
    if (n < 0 || nv < 3 || nv > kMaxVerts || n >= (1 << kCandBits)) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    if (!centers || !normals || !pts || !vis || !ws) return SP_ERR_ARG;
    if (ws_bytes < sp_patch_visibility_workspace(n)) return SP_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    const int n_groups = (n + kGroup - 1) / kGroup;
    const long long cap = vis_cand_capacity(n);
    const long long n_tiles = vis_tile_count(n);
    char* q = (char*)ws;
    float* box = (float*)q;
    float* gbox = box + (size_t)n * 6;
    q += sp_align((size_t)n * 6 * sizeof(float) + (size_t)n_groups * 6 * sizeof(float));
    int64_t* cand = (int64_t*)q;
    q += sp_align((size_t)cap * 8);
    int32_t* list[2];
    list[0] = (int32_t*)q;
    q += sp_align((size_t)n_tiles * 4);
    list[1] = (int32_t*)q;
    q += sp_align((size_t)n_tiles * 4);
    uint8_t* own_ok = (uint8_t*)q;
    q += sp_align((size_t)n);
    PolyPre* pre = (PolyPre*)q;
    q += sp_align((size_t)n * sizeof(PolyPre));
    unsigned long long* counter = (unsigned long long*)q;
    int* n_overflow = (int*)(q + 8);
    k_blocker_boxes<<<n_groups, kGroup, 0, sp_counted(st)>>>(n, nv, pts, 1e-3f, box, gbox);
    cudaMemsetAsync(vis, 0, (size_t)n * n, st);  // tiles below the diagonal are never visited
    // upper-triangle tiles (tile_j >= tile_i)
    const int nt = (n + 15) / 16;
    std::vector<int32_t> h_tiles;
    h_tiles.reserve((size_t)n_tiles);
    for (int ti = 0; ti < nt; ++ti)
        for (int tj = ti; tj < nt; ++tj) h_tiles.push_back((ti << 16) | tj);
    cudaMemcpyAsync(list[0], h_tiles.data(), h_tiles.size() * 4, cudaMemcpyHostToDevice, st);
    long long todo = (long long)h_tiles.size();
    k_own_patch<<<sp_blocks(n, 128), 128, 0, sp_counted(st)>>>(n, nv, centers, normals, pts, own_ok);
    k_poly_pre<<<sp_blocks(n, 128), 128, 0, sp_counted(st)>>>(n, nv, normals, pts, pre);
    k_vis_self<<<(unsigned)todo, 256, 0, sp_counted(st)>>>(n, nv, list[0], centers, normals, pts, own_ok, vis);
    int cur = 0;
    for (int round = 0; todo > 0; ++round) {
        cudaMemsetAsync(counter, 0, 16, st);
        cudaMemsetAsync(cand, 0xff, (size_t)cap * 8, st);
        k_vis_cull<<<(unsigned)todo, 256, 1024 * 6 * sizeof(float), sp_counted(st)>>>(
            n, list[cur], centers, box, gbox, n_groups, vis, cand, cap, counter, list[1 - cur], n_overflow);
        unsigned long long h[2] = {0, 0};
        cudaMemcpyAsync(h, counter, 16, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return SP_ERR_CUDA;
        const long long used = (long long)h[0] < cap ? (long long)h[0] : cap;
        const int overflowed = (int)(h[1] & 0xffffffffull);
        if (used > 0)
            k_vis_exact<<<sp_blocks(used, 256), 256, 0, sp_counted(st)>>>(used, cand, n, nv, centers, normals, pts,
                                                                         pre, vis);
        if (overflowed >= todo) return SP_ERR_CUDA;  // no progress: cannot happen with cap >= 256 n
        todo = overflowed;
        cur = 1 - cur;
    }
    return sp_check_launch();
}

size_t sp_point_visibility_workspace(int n_surf) {
    size_t groups = ((size_t)n_surf + kGroup - 1) / kGroup;
    return (size_t)n_surf * 6 * sizeof(float) + groups * 6 * sizeof(float) + 256;
}

int sp_points_visibility(int n_points, const double* points, int n, const double* centers, int n_surf, int nv,
                         const double* surf_pts, const double* surf_normals, uint8_t* out, void* ws,
                         size_t ws_bytes, void* stream) {
    if (n_points < 0 || n < 0 || n_surf < 0 || nv < 3 || nv > kMaxVerts) return SP_ERR_ARG;
    if (n == 0 || n_points == 0) return SP_OK;
    if (!points || !centers || !out || (n_surf > 0 && (!surf_pts || !surf_normals || !ws))) return SP_ERR_ARG;
    if (n_surf > 0 && ws_bytes < sp_point_visibility_workspace(n_surf)) return SP_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    float* sbox = (float*)ws;
    if (n_surf > 0) {
        int n_groups = (n_surf + kGroup - 1) / kGroup;
        k_blocker_boxes<<<n_groups, kGroup, 0, sp_counted(st)>>>(n_surf, nv, surf_pts, 1e-3f, sbox, sbox + (size_t)n_surf * 6);
    }
    const long long total = (long long)n_points * n;
    k_point_visibility<<<sp_blocks(total, 128), 128, 0, sp_counted(st)>>>(n_points, points, n, centers, n_surf, nv,
                                                                          surf_pts, surf_normals, sbox, out);
    return sp_check_launch();
}

int sp_point_visibility(const double* point, int n, const double* centers, int n_surf, int nv,
                        const double* surf_pts, const double* surf_normals, uint8_t* out, void* ws,
                        size_t ws_bytes, void* stream) {
    return sp_points_visibility(1, point, n, centers, n_surf, nv, surf_pts, surf_normals, out, ws, ws_bytes, stream);
}

int sp_visible_pairs(int n, const uint8_t* vis, int32_t* row_counts, int64_t* row_offset, int32_t* pairs,
                     int32_t* pair_index, void* stream) {
    if (n < 0 || (n > 0 && (!vis || !row_counts || !row_offset || !pairs))) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    cudaStream_t st = (cudaStream_t)stream;
    k_row_counts<<<n, 256, 0, sp_counted(st)>>>(n, vis, 1, row_counts);
    k_exclusive_scan<<<1, 1024, 0, sp_counted(st)>>>(n, row_counts, row_offset);
    k_fill_rows<<<n, 256, 0, sp_counted(st)>>>(n, vis, 1, row_offset, pairs, pair_index, nullptr, nullptr);
    return sp_check_launch();
}

int sp_count_directed(int n, const uint8_t* vis, uint8_t* sym, int32_t* row_counts, int64_t* row_offset,
                      void* stream) {
    if (n < 0 || (n > 0 && (!vis || !sym || !row_counts || !row_offset))) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    cudaStream_t st = (cudaStream_t)stream;
    dim3 g((n + 31) / 32, (n + 31) / 32), b(32, 8);
    k_symmetrize<<<g, b, 0, sp_counted(st)>>>(n, vis, sym);
    k_row_counts<<<n, 256, 0, sp_counted(st)>>>(n, sym, 0, row_counts);
    k_exclusive_scan<<<1, 1024, 0, sp_counted(st)>>>(n, row_counts, row_offset);
    return sp_check_launch();
}

int sp_directed_pairs(int n, const uint8_t* sym, const int64_t* row_offset, int32_t* src, int32_t* dst,
                      void* stream) {
    if (n < 0 || (n > 0 && (!sym || !row_offset || !src || !dst))) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    k_fill_rows<<<n, 256, 0, sp_counted((cudaStream_t)stream)>>>(n, sym, 0, row_offset, nullptr, nullptr, src, dst);
    return sp_check_launch();
}

int sp_pair_setup(long long n_dir, int n, const int32_t* src, const int32_t* dst, const double* centers,
                  const double* areas, const int32_t* pair_index, const double* ff, const int32_t* wall_of,
                  int n_in, const double* dirs_in, int n_out, const double* dirs_out, int32_t* out_dir,
                  int32_t* in_dir, double* dist, double* unit_len, double* fprime, void* stream) {
    if (n_dir < 0 || n < 0) return SP_ERR_ARG;
    if (n_dir == 0) return SP_OK;
    if (!src || !dst || !centers || !areas || !pair_index || !ff || !wall_of || !dist || !unit_len || !fprime)
        return SP_ERR_ARG;
    k_pair_setup<<<sp_blocks(n_dir, 128), 128, 0, sp_counted((cudaStream_t)stream)>>>(
        n_dir, n, src, dst, centers, areas, pair_index, ff, wall_of, n_in, dirs_in, n_out, dirs_out, out_dir, in_dir,
        dist, unit_len, fprime);
    return sp_check_launch();
}

int sp_outgoing_index_map(long long n_dir, int n, const int32_t* src, const int32_t* dst, const int32_t* out_dir,
                          int64_t sentinel, int64_t* out, void* stream) {
    if (n_dir < 0 || n < 0 || (n > 0 && !out)) return SP_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    long long nn = (long long)n * n;
    if (nn > 0) k_fill_i64<<<sp_blocks(nn, 256), 256, 0, sp_counted(st)>>>(nn, sentinel, out);
    if (n_dir > 0) k_scatter_outdir<<<sp_blocks(n_dir, 256), 256, 0, sp_counted(st)>>>(n_dir, n, src, dst, out_dir, out);
    return sp_check_launch();
}

}  // extern "C"

// ------------------------------------------------ allocation-free variant
// sp_patch_visibility_static: the results of sp_patch_visibility with the
// blocker-box scratch in a fixed array of this library's device image
// instead of a caller-provided workspace.  It runs the single-pass
// k_patch_visibility (one pair per thread), which needs no scratch beyond the
// boxes; the three-pass form needs the workspace for its candidate lists.
namespace {
constexpr int kStaticVisMaxPatches = 16384;
constexpr size_t kStaticVisScratchFloats =
    (size_t)kStaticVisMaxPatches * 6 + (((size_t)kStaticVisMaxPatches + kGroup - 1) / kGroup) * 6;
// 405,504 bytes, reserved when the module loads.  Every box the kernels read
// is written earlier in the same call, so nothing here has to start at zero.
static __device__ __align__(256) float g_static_vis_scratch[kStaticVisScratchFloats];
constexpr int kStaticMaxDevices = 64;
std::atomic<float*> g_static_vis_ptr[kStaticMaxDevices];  // per device, looked up once
}  // namespace

extern "C" int sp_patch_visibility_static(int n, int nv, const double* centers, const double* normals,
                                          const double* pts, uint8_t* vis, void* stream) {
    if (n > kStaticVisMaxPatches) return SP_ERR_WORKSPACE;
    if (n < 0 || nv < 3 || nv > kMaxVerts) return SP_ERR_ARG;
    if (n == 0) return SP_OK;
    if (!centers || !normals || !pts || !vis) return SP_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kStaticMaxDevices) return SP_ERR_CUDA;
    float* box = g_static_vis_ptr[dev].load(std::memory_order_acquire);
    if (!box) {
        // first call on this device (with it current): find the array's address
        void* addr = nullptr;
        if (cudaGetSymbolAddress(&addr, g_static_vis_scratch) != cudaSuccess || !addr) return SP_ERR_CUDA;
        box = static_cast<float*>(addr);
        g_static_vis_ptr[dev].store(box, std::memory_order_release);
    }
    cudaStream_t st = (cudaStream_t)stream;
    int n_groups = (n + kGroup - 1) / kGroup;
    float* gbox = box + (size_t)n * 6;
    k_blocker_boxes<<<n_groups, kGroup, 0, sp_counted(st)>>>(n, nv, pts, 1e-3f, box, gbox);
    cudaMemsetAsync(vis, 0, (size_t)n * n, st);
    int tiles = (n + 15) / 16;
    dim3 grid(tiles, tiles);
    k_patch_visibility<<<grid, 256, 1024 * 6 * sizeof(float), sp_counted(st)>>>(n, nv, centers, normals, pts, box,
                                                                                 gbox, n_groups, vis);
    return sp_check_launch();
}
