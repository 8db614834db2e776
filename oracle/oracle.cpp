// FP64 CPU oracle for the directional fast-radiosity path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, statement by statement, the
// numpy/numba loops of sparrowpy 1.0.1 that the GPU library replaces, so that
// the GPU results can be checked against a fast CPU reference at sizes where
// the pure-Python reference would take days.  Only the test suite, the smoke
// check and the CPU-baseline leg of the benchmark load it; the product path
// (sparrowpy_gb300) never does.
//
// Every function names the reference file:line it follows.  Floating-point
// operations keep the reference's operation order; the build uses
// -ffp-contract=off so that no multiply-add is fused behind our back.
//
// Build: see oracle/build_oracle.py (g++ -O2 -fopenmp -ffp-contract=off).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int kMaxPoly = 8;  // patch polygon vertices the form factors accept

inline double dot3(const double* a, const double* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
inline double norm3(const double* a) { return std::sqrt(dot3(a, a)); }
inline double dot2(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1]; }
inline double norm2(const double* a) { return std::sqrt(dot2(a, a)); }
inline void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// geometry.py:498-559 `_rotation_matrix(n_in)` with n_out = (0, 0, 1).
void rotation_matrix(const double* n_in, double* m) {
    if (n_in[0] == 0.0 && n_in[1] == 0.0 && n_in[2] == 1.0) {
        for (int i = 0; i < 9; ++i) m[i] = (i % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    double nn = norm3(n_in);
    double a[3] = {n_in[0] / nn, n_in[1] / nn, n_in[2] / nn};
    double b[3] = {0.0, 0.0, 1.0};
    double c = dot3(a, b);
    if (c != -1.0) {
        double v[3];
        cross3(a, b, v);
        double s = norm3(v);
        double k[9] = {0.0, -v[2], v[1], v[2], 0.0, -v[0], -v[1], v[0], 0.0};
        double kk[9];
        for (int r = 0; r < 3; ++r)
            for (int col = 0; col < 3; ++col)
                kk[r * 3 + col] = k[r * 3 + 0] * k[0 * 3 + col] + k[r * 3 + 1] * k[1 * 3 + col] +
                                  k[r * 3 + 2] * k[2 * 3 + col];
        double f = (1.0 - c) / (s * s);
        for (int i = 0; i < 9; ++i) m[i] = ((i % 4 == 0) ? 1.0 : 0.0) + k[i] + kk[i] * f;
    } else {
        const double flip[9] = {-1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, -1.0};
        for (int i = 0; i < 9; ++i) m[i] = flip[i];
    }
}

// geometry.py:474-496 `_matrix_vector_product`, keeping the first two rows.
inline void rot_xy(const double* m, const double* v, double* out2) {
    out2[0] = dot3(m + 0, v);
    out2[1] = dot3(m + 3, v);
}
inline void rot_xyz(const double* m, const double* v, double* out3) {
    out3[0] = dot3(m + 0, v);
    out3[1] = dot3(m + 3, v);
    out3[2] = dot3(m + 6, v);
}

// geometry.py:561-612 `_project_to_plane` (3-D form).  Returns false for None.
bool project_to_plane3(const double* origin, const double* point, const double* plane_pt,
                       const double* n, bool check_normal, double* out) {
    const double eps = 1e-6;
    double v[3] = {point[0] - origin[0], point[1] - origin[1], point[2] - origin[2]};
    double dp = dot3(v, n);
    bool cond = check_normal ? (dp < -eps) : (std::fabs(dp) > eps);
    if (!cond) return false;
    double w[3] = {point[0] - plane_pt[0], point[1] - plane_pt[1], point[2] - plane_pt[2]};
    double fac = -(dot3(n, w) / dp);
    for (int d = 0; d < 3; ++d) out[d] = w[d] + plane_pt[d] + fac * v[d];
    return true;
}

// geometry.py:614-686 `_point_in_polygon` (winding number, eta = 1e-6).
bool point_in_polygon(const double* p3, const double* poly3, int nv, const double* n) {
    const double eta = 1e-6;
    double d0[3] = {p3[0] - poly3[0], p3[1] - poly3[1], p3[2] - poly3[2]};
    if (std::fabs(dot3(d0, n)) > eta) return false;
    double rot[9];
    rotation_matrix(n, rot);
    double pt[2];
    rot_xy(rot, p3, pt);
    double poly[16][2];
    for (int i = 0; i < nv; ++i) rot_xy(rot, poly3 + 3 * i, poly[i]);
    int count = 0;
    for (int i = 0; i < nv; ++i) {
        const double* a1 = poly[(i + 1) % nv];
        const double* a0 = poly[i % nv];
        double side[2] = {a1[0] - a0[0], a1[1] - a0[1]};
        double ns = norm2(side);
        double nl[2] = {-side[1] / ns, side[0] / ns};
        // _project_to_plane(origin=pt, point=pt+[1,0], plane_pt=a1, nl, check_normal=False)
        double point[2] = {pt[0] + 1.0, pt[1] + 0.0};
        double v[2] = {point[0] - pt[0], point[1] - pt[1]};
        double dp = dot2(v, nl);
        if (!(std::fabs(dp) > 1e-6)) continue;
        double w[2] = {point[0] - a1[0], point[1] - a1[1]};
        double fac = -(dot2(nl, w) / dp);
        double b[2] = {w[0] + a1[0] + fac * v[0], w[1] + a1[1] + fac * v[1]};
        if (b[0] > pt[0]) {
            double ba0[2] = {b[0] - a0[0], b[1] - a0[1]};
            double ba1[2] = {b[0] - a1[0], b[1] - a1[1]};
            double a10[2] = {a1[0] - a0[0], a1[1] - a0[1]};
            if (std::fabs(norm2(ba0) + norm2(ba1) - norm2(a10)) <= eta) {
                double bp[2] = {b[0] - pt[0], b[1] - pt[1]};
                double s = dot2(bp, nl);
                if (s > 0)
                    count += 1;
                else if (s < 0)
                    count -= 1;
            }
        }
    }
    return count != 0;
}

// geometry.py:841-909 `_basic_visibility`.
bool basic_visibility(const double* vis_point, const double* eval_point, const double* surf_points,
                      int nv, const double* n) {
    const double eta = 1e-6;
    bool is_visible = true;
    bool vis_in = point_in_polygon(vis_point, surf_points, nv, n);
    bool eval_in = point_in_polygon(eval_point, surf_points, nv, n);
    if (!vis_in && !eval_in) {
        double pt[3];
        if (project_to_plane3(vis_point, eval_point, surf_points, n, false, pt)) {
            if (point_in_polygon(pt, surf_points, nv, n)) {
                double a[3] = {pt[0] - vis_point[0], pt[1] - vis_point[1], pt[2] - vis_point[2]};
                double b[3] = {pt[0] - eval_point[0], pt[1] - eval_point[1], pt[2] - eval_point[2]};
                if (dot3(a, b) < 0) is_visible = false;
            }
        }
        return is_visible;
    }
    // the elif chain of geometry.py:895-906: each condition includes its
    // half-space test, so a failed test falls through to the coplanar case
    double ev[3] = {eval_point[0] - vis_point[0], eval_point[1] - vis_point[1], eval_point[2] - vis_point[2]};
    double ve[3] = {vis_point[0] - eval_point[0], vis_point[1] - eval_point[1], vis_point[2] - eval_point[2]};
    if (vis_in && !eval_in && dot3(n, ev) < 0) return false;
    if (!vis_in && eval_in && dot3(n, ve) < 0) return false;
    double a[3] = {vis_point[0] - surf_points[0], vis_point[1] - surf_points[1], vis_point[2] - surf_points[2]};
    double b[3] = {eval_point[0] - surf_points[0], eval_point[1] - surf_points[1], eval_point[2] - surf_points[2]};
    if (std::fabs(dot3(a, n)) < eta && std::fabs(dot3(b, n)) < eta && (vis_in || eval_in)) return false;
    return is_visible;
}

// geometry.py:420-440 `_polygon_area` (fan triangulation from vertex 0).
double polygon_area(const double* pts, int nv, int stride) {
    double area = 0.0;
    for (int t = 0; t < nv - 2; ++t) {
        const double* p0 = pts;
        const double* p1 = pts + (t + 1) * stride;
        const double* p2 = pts + (t + 2) * stride;
        double a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
        double b[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
        double c[3];
        cross3(a, b, c);
        area += 0.5 * norm3(c);
    }
    return area;
}

// integration.py:608-651 `_sample_boundary_regular` (points only; the
// connectivity of segment s is [s*n_div, ..., s*n_div + n_div] modulo n).
void sample_boundary(const double* el, int nv, int npoints, double* pts) {
    int n_div = npoints - 1;
    for (int i = 0; i < nv; ++i) {
        const double* a = el + 3 * i;
        const double* b = el + 3 * ((i + 1) % nv);
        for (int ii = 0; ii < n_div; ++ii)
            for (int d = 0; d < 3; ++d)
                pts[3 * (i * n_div + ii) + d] = a[d] + (ii * (b[d] - a[d])) / n_div;
    }
}

// integration.py:462-486 `_newton_cotes_4th` (Boole's rule).
inline double newton_cotes_4th(const double* x, const double* y) {
    double h = x[1] - x[0];
    return 2 * h / 45 * (7 * y[0] + 32 * y[1] + 12 * y[2] + 32 * y[3] + 7 * y[4]);
}

// integration.py:38-114 `stokes_integration` with load_stokes_entries :12-36,
// for convex polygons of nvi and nvj vertices (4 nv boundary points each,
// nv segments of 5 points).
double stokes_integration(const double* pi, int nvi, const double* pj, int nvj, double area_i) {
    const int na = 4 * nvi, nb = 4 * nvj;
    std::vector<double> ib((size_t)na * 3), jb((size_t)nb * 3);
    sample_boundary(pi, nvi, 5, ib.data());
    sample_boundary(pj, nvj, 5, jb.data());
    std::vector<double> form((size_t)na * nb);
    for (int a = 0; a < na; ++a)
        for (int b = 0; b < nb; ++b) {
            double d[3] = {ib[3 * a] - jb[3 * b], ib[3 * a + 1] - jb[3 * b + 1], ib[3 * a + 2] - jb[3 * b + 2]};
            form[(size_t)a * nb + b] = std::log(norm3(d));
        }
    double outer = 0.0;
    std::vector<double> inner((size_t)na * 3, 0.0);
    for (int dim = 0; dim < 3; ++dim) {
        for (int a = 0; a < na; ++a) {
            for (int s = 0; s < nvj; ++s) {
                double xj[5], sub[5];
                for (int k = 0; k < 5; ++k) xj[k] = jb[3 * ((4 * s + k) % nb) + dim];
                if (std::fabs(xj[4] - xj[0]) > 1e-3) {
                    for (int k = 0; k < 5; ++k) sub[k] = form[(size_t)a * nb + (4 * s + k) % nb];
                    inner[3 * a + dim] += newton_cotes_4th(xj, sub);
                }
            }
        }
        for (int s = 0; s < nvi; ++s) {
            double xi[5], sub[5];
            for (int k = 0; k < 5; ++k) xi[k] = ib[3 * ((4 * s + k) % na) + dim];
            if (std::fabs(xi[4] - xi[0]) > 1e-3) {
                for (int k = 0; k < 5; ++k) sub[k] = inner[3 * ((4 * s + k) % na) + dim];
                outer += newton_cotes_4th(xi, sub);
            }
        }
    }
    return std::fabs(outer / (2 * kPi * area_i));
}

// 3x3 inverse by Gauss-Jordan with partial pivoting (stands in for
// np.linalg.inv in integration.py:380; agreement is to rounding only).
bool inv3(const double* a, double* out) {
    double m[3][6];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) m[r][c] = a[r * 3 + c];
        for (int c = 0; c < 3; ++c) m[r][3 + c] = (r == c) ? 1.0 : 0.0;
    }
    for (int col = 0; col < 3; ++col) {
        int piv = col;
        for (int r = col + 1; r < 3; ++r)
            if (std::fabs(m[r][col]) > std::fabs(m[piv][col])) piv = r;
        if (m[piv][col] == 0.0) return false;
        if (piv != col)
            for (int c = 0; c < 6; ++c) std::swap(m[piv][c], m[col][c]);
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

// integration.py:416-460 `_area_under_curve` (3 samples, order 2) with
// `_poly_estimation_Lagrange` :349-382 and `_poly_integration` :385-412.
double area_under_curve(const double ps[3][2]) {
    double f[2] = {ps[2][0] - ps[0][0], ps[2][1] - ps[0][1]};
    double nf = norm2(f);
    double rm[4] = {f[0] / nf, f[1] / nf, -f[1] / nf, f[0] / nf};
    double x[3] = {0, 0, 0}, y[3] = {0, 0, 0};
    for (int k = 1; k < 3; ++k) {
        double c[2] = {ps[k][0] - ps[0][0], ps[k][1] - ps[0][1]};
        x[k] = rm[0] * c[0] + rm[1] * c[1];
        y[k] = rm[2] * c[0] + rm[3] * c[1];
    }
    double b[3] = {0, 0, 0};
    if (!(std::fabs(x[2] - x[0]) < 1e-6)) {
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
        out += b[i] * std::pow(x[2], p) / p;
        out -= b[i] * std::pow(x[0], p) / p;
    }
    return out;
}

inline double sign(double v) { return (v > 0) ? 1.0 : ((v < 0) ? -1.0 : 0.0); }

// integration.py:116-230 `nusselt_analog` for a receiver polygon of nvp
// vertices (2 nvp boundary points, nvp segments of 3).
double nusselt_analog(const double* origin, const double* surf_normal, const double* pp, int nvp,
                      const double* patch_normal) {
    const int nbp = 2 * nvp;
    double bp[2 * kMaxPoly * 3];
    sample_boundary(pp, nvp, 3, bp);
    double e1[3] = {pp[3] - pp[0], pp[4] - pp[1], pp[5] - pp[2]};
    double e2[3] = {pp[6] - pp[3], pp[7] - pp[4], pp[8] - pp[5]};
    double cr[3];
    cross3(e1, e2, cr);
    double hand = sign(dot3(cr, patch_normal));
    double sph[2 * kMaxPoly][3], pln[2 * kMaxPoly][2], proj[2 * kMaxPoly][3];
    for (int ii = 0; ii < nbp; ++ii) {
        double d[3] = {bp[3 * ii] - origin[0], bp[3 * ii + 1] - origin[1], bp[3 * ii + 2] - origin[2]};
        double nd = norm3(d);
        for (int k = 0; k < 3; ++k) sph[ii][k] = d[k] / nd;
    }
    double rot[9];
    rotation_matrix(surf_normal, rot);
    for (int ii = 0; ii < nbp; ++ii) {
        rot_xy(rot, sph[ii], pln[ii]);
        proj[ii][0] = pln[ii][0];
        proj[ii][1] = pln[ii][1];
        proj[ii][2] = 0.0;
    }
    double corners[kMaxPoly][3];
    for (int c = 0; c < nvp; ++c)
        for (int k = 0; k < 3; ++k) corners[c][k] = proj[2 * c][k];
    double big_poly = polygon_area(&corners[0][0], nvp, 3);
    double curved = 0.0;
    for (int jj = 0; jj < nvp; ++jj) {
        int s0 = (2 * jj) % nbp, s1 = (2 * jj + 1) % nbp, s2 = (2 * jj + 2) % nbp;
        double cr2[3];
        cross3(proj[s2], proj[s0], cr2);
        if (norm3(cr2) > 1e-6) {
            if (dot2(pln[s2], pln[s0]) >= 1e-6) {
                double seg[3][2] = {{pln[s0][0], pln[s0][1]}, {pln[s1][0], pln[s1][1]},
                                    {pln[s2][0], pln[s2][1]}};
                curved += area_under_curve(seg);
            } else {
                double mp[3], marc[3], a[3], b[3];
                for (int k = 0; k < 3; ++k) mp[k] = sph[s0][k] + (sph[s2][k] - sph[s0][k]) / 2;
                double nm = norm3(mp);
                for (int k = 0; k < 3; ++k) marc[k] = mp[k] / nm;
                for (int k = 0; k < 3; ++k) a[k] = sph[s0][k] + (marc[k] - sph[s0][k]) / 2;
                for (int k = 0; k < 3; ++k) b[k] = marc[k] + (sph[s2][k] - marc[k]) / 2;
                double mp2[2], marc2[2], a2[2], b2[2];
                rot_xy(rot, mp, mp2);
                rot_xy(rot, marc, marc2);
                double na = norm3(a);
                for (int k = 0; k < 3; ++k) a[k] = a[k] / na;
                rot_xy(rot, a, a2);
                double nb = norm3(b);
                for (int k = 0; k < 3; ++k) b[k] = b[k] / nb;
                rot_xy(rot, b, b2);
                double d1[2] = {pln[s2][0] - pln[s0][0], pln[s2][1] - pln[s0][1]};
                double d2[2] = {mp2[0] - marc2[0], mp2[1] - marc2[1]};
                double lin_area = norm2(d1) * norm2(d2) / 2;
                double left_seg[3][2] = {{pln[s0][0], pln[s0][1]}, {a2[0], a2[1]}, {marc2[0], marc2[1]}};
                double right_seg[3][2] = {{marc2[0], marc2[1]}, {b2[0], b2[1]}, {pln[s2][0], pln[s2][1]}};
                double left = area_under_curve(left_seg);
                double right = area_under_curve(right_seg);
                curved += (lin_area * sign(left) + left + right);
            }
        }
    }
    return big_poly + hand * curved;
}

// Python's round() on a float64: round half to even.
inline long round_half_even(double v) { return (long)std::nearbyint(v); }

// integration.py:533-605 `_surf_sample_regulargrid`: a parallelogram
// spanned by el[1] - el[0] and el[nv - 1] - el[0], or (nv == 3) the
// triangle half of it, whose columns shorten along the first edge and whose
// points beyond the hypotenuse (s + t > 1 - thres) are left out.
int surf_sample_regulargrid(const double* el, int nv, int npoints, std::vector<double>& out) {
    const double* last = el + 3 * (nv - 1);
    double u[3] = {el[3] - el[0], el[4] - el[1], el[5] - el[2]};
    double v[3] = {last[0] - el[0], last[1] - el[1], last[2] - el[2]};
    const bool tri = nv == 3;
    const double a = tri ? 2.0 : 1.0;
    double nu = norm3(u), nvv = norm3(v);
    long npx = round_half_even(nu / nvv * std::sqrt(a * npoints));
    long npz = round_half_even(nvv / nu * std::sqrt(a * npoints));
    if (npz == 0) npz = 1;
    if (npx == 0) npx = 1;
    std::vector<double> tt(npx), tz(npz);
    // numpy.linspace(0, stop, num): k*step, last element exactly stop.
    double sstep = 1.0 / (npx * 2), sstepz = 1.0 / (npz * 2);
    {
        double stop = 1 - 1.0 / npx;
        double step = (npx > 1) ? (stop - 0.0) / (npx - 1) : 0.0;
        for (long k = 0; k < npx; ++k) tt[k] = k * step + 0.0;
        if (npx > 1) tt[npx - 1] = stop;
        for (long k = 0; k < npx; ++k) tt[k] += sstep;
    }
    {
        double stop = 1 - 1.0 / npz;
        double step = (npz > 1) ? (stop - 0.0) / (npz - 1) : 0.0;
        for (long k = 0; k < npz; ++k) tz[k] = k * step + 0.0;
        if (npz > 1) tz[npz - 1] = stop;
        for (long k = 0; k < npz; ++k) tz[k] += sstepz;
    }
    const double thres = std::sqrt(sstepz * sstepz + sstep * sstep) / 2;
    out.clear();
    for (long i = 0; i < npx; ++i) {
        const long jj = tri ? i : 0;
        // tz[0 : len(tz) - round(npz / npx * jj)] (never a negative stop for these sizes)
        long stop = npz - round_half_even((double)npz / (double)npx * (double)jj);
        if (stop < 0) stop = std::max(0L, npz + stop);
        for (long k = 0; k < stop; ++k) {
            const bool inside = tt[i] + tz[k] <= 1 - thres;
            if (tri && !inside) continue;
            for (int d = 0; d < 3; ++d) out.push_back(tt[i] * u[d] + tz[k] * v[d] + el[d]);
        }
    }
    return (int)(out.size() / 3);
}

// integration.py:232-289 `nusselt_integration` (regular grid, nsamples).
double nusselt_integration(const double* pi, int nvi, const double* pj, int nvj, const double* ni, const double* nj,
                           int nsamples) {
    std::vector<double> p0;
    int n = surf_sample_regulargrid(pi, nvi, nsamples, p0);
    double out = 0.0;
    for (int i = 0; i < n; ++i) out += nusselt_analog(&p0[3 * i], ni, pj, nvj, nj);
    out *= 1 / (kPi * n);
    return out;
}

// geometry.py:719-748 `_coincidence_check`.
bool coincidence_check(const double* p0, int nv0, const double* p1, int nv1) {
    for (int i = 0; i < nv0; ++i)
        for (int j = 0; j < nv1; ++j) {
            double d[3] = {p0[3 * i] - p1[3 * j], p0[3 * i + 1] - p1[3 * j + 1], p0[3 * i + 2] - p1[3 * j + 2]};
            if (norm3(d) < 1e-6) return true;
        }
    return false;
}

// universal.py:54-96 `universal_form_factor` (patches of nv vertices each).
double universal_form_factor(const double* src_pts, const double* src_n, double src_area,
                             const double* rcv_pts, const double* rcv_n, int nv) {
    if (coincidence_check(rcv_pts, nv, src_pts, nv))
        return nusselt_integration(src_pts, nv, rcv_pts, nv, src_n, rcv_n, 64);
    return stokes_integration(src_pts, nv, rcv_pts, nv, src_area);
}

// geometry.py:688-715 `_sphere_tangent_vector`.
void sphere_tangent_vector(const double* v0, const double* v1, double* out) {
    if (std::fabs(dot3(v0, v1)) > 1e-10) {
        double d[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
        double f = dot3(d, v0) / dot3(v0, v0);
        for (int k = 0; k < 3; ++k) out[k] = d[k] - f * v0[k];
        double n = norm3(out);
        for (int k = 0; k < 3; ++k) out[k] /= n;
    } else {
        double n = norm3(v1);
        for (int k = 0; k < 3; ++k) out[k] = v1[k] / n;
    }
}

// integration.py:295-344 `pt_solution`.  mode 0 = source, 1 = receiver.
double pt_solution(const double* point, const double* patch, int nv, int mode) {
    double source_area = (mode == 1) ? polygon_area(patch, nv, 3) : 4.0;
    double ons[16][3];
    for (int i = 0; i < nv; ++i) {
        double d[3] = {patch[3 * i] - point[0], patch[3 * i + 1] - point[1], patch[3 * i + 2] - point[2]};
        double n = norm3(d);
        for (int k = 0; k < 3; ++k) ons[i][k] = d[k] / n;
    }
    double s = 0.0;
    for (int i = 0; i < nv; ++i) {
        double v0[3], v1[3];
        sphere_tangent_vector(ons[i], ons[(i - 1 + nv) % nv], v0);
        sphere_tangent_vector(ons[i], ons[(i + 1) % nv], v1);
        s += std::acos(dot3(v0, v1));
    }
    double factor = s - (nv - 2) * kPi;
    return factor / (kPi * source_area);
}

// RadiosityFast.py:1277-1312 `get_scattering_data_receiver_index`, one row:
// argmin_k |dirs[k] - unit(to - from)|^2 (first index on ties).
int nearest_direction(const double* from, const double* to, const double* dirs, int nd) {
    double diff[3] = {to[0] - from[0], to[1] - from[1], to[2] - from[2]};
    double n = norm3(diff);
    for (int k = 0; k < 3; ++k) diff[k] /= n;
    int best = 0;
    double bv = 0.0;
    for (int o = 0; o < nd; ++o) {
        double a = dirs[3 * o] - diff[0], b = dirs[3 * o + 1] - diff[1], c = dirs[3 * o + 2] - diff[2];
        double v = a * a + b * b + c * c;
        if (o == 0 || v < bv) {
            bv = v;
            best = o;
        }
    }
    return best;
}

}  // namespace

extern "C" {

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

// geometry.py:750-797 `_check_patch2patch_visibility`.  V is (N, N) row-major,
// only i < j entries can be 1.  Blockers are all N patches, in index order.
int orc_patch_visibility(int n, int nv, const double* centers, const double* normals,
                         const double* points, uint8_t* vis) {
    std::memset(vis, 0, (size_t)n * n);
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
        for (int j = i + 1; j < n; ++j) {
            bool v = true;
            for (int s = 0; s < n && v; ++s)
                v = basic_visibility(centers + 3 * i, centers + 3 * j, points + (size_t)s * nv * 3, nv,
                                     normals + 3 * s);
            vis[(size_t)i * n + j] = v ? 1 : 0;
        }
    }
    return 0;
}

// geometry.py:799-839 `_check_point2patch_visibility` (blockers = surfaces).
int orc_point_visibility(const double* point, int n, const double* centers, int n_surf, int nv,
                         const double* surf_points, const double* surf_normals, uint8_t* out) {
    for (int i = 0; i < n; ++i) {
        bool v = true;
        for (int s = 0; s < n_surf && v; ++s)
            v = basic_visibility(point, centers + 3 * i, surf_points + (size_t)s * nv * 3, nv,
                                 surf_normals + 3 * s);
        out[i] = v ? 1 : 0;
    }
    return 0;
}

// universal.py:12-52 `patch2patch_ff_universal`: one value per listed pair
// (all patches with nv vertices, as the reference's arrays have).
int orc_form_factors(int n_pairs, const int32_t* pairs, const double* points, int nv, const double* normals,
                     const double* areas, double* out) {
    if (nv < 3 || nv > kMaxPoly) return -1;
#pragma omp parallel for schedule(dynamic, 64)
    for (int p = 0; p < n_pairs; ++p) {
        int i = pairs[2 * p], j = pairs[2 * p + 1];
        out[p] = universal_form_factor(points + 3 * (size_t)nv * i, normals + 3 * i, areas[i],
                                       points + 3 * (size_t)nv * j, normals + 3 * j, nv);
    }
    return 0;
}

double orc_stokes(const double* pi, int nvi, const double* pj, int nvj, double area_i) {
    return stokes_integration(pi, nvi, pj, nvj, area_i);
}
double orc_nusselt(const double* pi, int nvi, const double* pj, int nvj, const double* ni, const double* nj, int ns) {
    return nusselt_integration(pi, nvi, pj, nvj, ni, nj, ns);
}
double orc_pt_solution(const double* point, const double* patch, int nv, int mode) {
    return pt_solution(point, patch, nv, mode);
}
int orc_coincident(const double* p0, int nv0, const double* p1, int nv1) {
    return coincidence_check(p0, nv0, p1, nv1) ? 1 : 0;
}

// Per directed pair (i -> j): nearest direction index among `dirs[wall[i]]`
// toward unit(c_to - c_from).  Covers RadiosityFast.py:402-414 (outgoing map,
// from = c_i, to = c_j) and :1359-1390 (incoming index, from = c_j, to = c_i).
int orc_nearest_dirs(int n_pairs, const int32_t* from_idx, const int32_t* to_idx, const double* centers,
                     const int64_t* wall_of_pair, const double* dirs, int nd, int32_t* out) {
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n_pairs; ++p) {
        int f = from_idx[p], t = to_idx[p];
        out[p] = nearest_direction(centers + 3 * f, centers + 3 * t, dirs + (size_t)wall_of_pair[p] * nd * 3, nd);
    }
    return 0;
}

// Nearest direction from arbitrary points (source/receiver lookups):
// RadiosityFast.py:1386-1390 with pos_h = point, pos_i = c_k -> dirs of wall k
// (mode 0: unit(point - c_k)); :728-730 with pos_j = point (mode 1: unit(point - c_k)).
int orc_point_dirs(const double* point, int n, const double* centers, const int64_t* wall_of,
                   const double* dirs, int nd, int32_t* out) {
    for (int k = 0; k < n; ++k)
        out[k] = nearest_direction(centers + 3 * k, point, dirs + (size_t)wall_of[k] * nd * 3, nd);
    return 0;
}

// RadiosityFast.py:1073-1145 `_energy_exchange` (+ :1037-1070 init), on the
// compact pair form.  For directed pair p (i -> j) the reference row
// form_factors_tilde[i, j, o, b] equals
//   ((fprime[p] * att_fac[b]) * brdf[slot[p], s_in[p], o, b])
// (RadiosityFast.py:1255-1270), which is recomputed here with the same
// operation order.  Directed pairs are listed in the reference loop order:
// visible pair list row-major, first (i -> j) then (j -> i).  Per-output
// summation order matches the reference because every receiver j collects
// its contributions in list order.
int orc_exchange(int n, int nd, int nb, int nt, int max_order, const double* e0dir, const int64_t* delay0,
                 int n_dir_pairs, const int32_t* src, const int32_t* dst, const int32_t* p2o,
                 const int64_t* delay, const double* fprime, const double* att_fac, const int32_t* slot,
                 const int32_t* s_in, const double* brdf, int n_in, double* etot) {
    const size_t row = (size_t)nd * nb * nt;
    std::memset(etot, 0, sizeof(double) * row * n);
    for (int i = 0; i < n; ++i) {
        int64_t d = delay0[i];
        if (d < 0 || d >= nt) return -2;
        for (int o = 0; o < nd; ++o)
            for (int b = 0; b < nb; ++b)
                etot[i * row + ((size_t)o * nb + b) * nt + d] += e0dir[((size_t)i * nd + o) * nb + b];
    }
    if (max_order <= 0) return 0;
    std::vector<double> prev(etot, etot + row * n), cur(row * n);
    // stable CSR by destination
    std::vector<int> cnt(n + 1, 0), order(n_dir_pairs);
    for (int p = 0; p < n_dir_pairs; ++p) cnt[dst[p] + 1]++;
    for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    {
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (int p = 0; p < n_dir_pairs; ++p) order[fill[dst[p]]++] = p;
    }
    for (int k = 0; k < max_order; ++k) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int j = 0; j < n; ++j) {
            double* out = cur.data() + (size_t)j * row;
            std::memset(out, 0, sizeof(double) * row);
            for (int q = cnt[j]; q < cnt[j + 1]; ++q) {
                int p = order[q];
                int i = src[p];
                int o_src = p2o[p];
                int64_t nsh = delay[p];
                const double* brow = brdf + (((size_t)slot[p] * n_in + s_in[p]) * nd) * nb;
                for (int o = 0; o < nd; ++o)
                    for (int b = 0; b < nb; ++b) {
                        double f = (fprime[p] * att_fac[(size_t)p * nb + b]) * brow[(size_t)o * nb + b];
                        const double* in = prev.data() + (size_t)i * row + ((size_t)o_src * nb + b) * nt;
                        double* o_ = out + ((size_t)o * nb + b) * nt;
                        if (nsh > 0) {
                            for (int64_t t = nsh; t < nt; ++t) o_[t] += f * in[t - nsh];
                        } else {
                            for (int64_t t = 0; t < nt; ++t) o_[t] += f * in[t];
                        }
                    }
            }
        }
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < (int64_t)(row * n); ++e) etot[e] += cur[e];
        std::swap(prev, cur);
    }
    return 0;
}

// Timing samples for the CPU baseline (same loops as above, on a subset).
// Rows i0 <= i < i1 (step stride) of geometry.py:750-797; returns the
// visible count.  With full != 0 a row covers every j != i (the pair
// evaluated as (min, max), i.e. one row of the symmetric matrix), else j > i.
long long orc_patch_visibility_rows(int n, int nv, const double* centers, const double* normals,
                                    const double* points, int i0, int i1, int stride, int full, uint8_t* vis_rows) {
    long long total = 0;
    int rows = 0;
    for (int i = i0; i < i1; i += stride) ++rows;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
    for (int r = 0; r < rows; ++r) {
        int i = i0 + r * stride;
        for (int j = full ? 0 : i + 1; j < n; ++j) {
            if (j == i) continue;
            int a = i < j ? i : j, b = i < j ? j : i;
            bool v = true;
            for (int s = 0; s < n && v; ++s)
                v = basic_visibility(centers + 3 * a, centers + 3 * b, points + (size_t)s * nv * 3, nv,
                                     normals + 3 * s);
            if (vis_rows) vis_rows[(size_t)r * n + j] = v ? 1 : 0;
            total += v ? 1 : 0;
        }
    }
    return total;
}

// One order of RadiosityFast.py:1121-1143 for destination rows
// rows[0..n_rows) only, with the destination-major pair list (dst_off, src,
// ...).  Source rows are read from `prev` at row (src % prev_rows) (the cost
// does not depend on the values).  Returns the sum of the produced values.
double orc_exchange_rows_sample(int nd, int nb, int nt, const double* prev, int prev_rows, const int64_t* dst_off,
                                const int32_t* src, const int32_t* p2o, const int32_t* delay, const double* fprime,
                                const double* att_fac, const int32_t* slot, const int32_t* s_in, const double* brdf,
                                int n_in, int n_rows, const int32_t* rows) {
    const size_t row = (size_t)nd * nb * nt;
    double total = 0.0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
    for (int q = 0; q < n_rows; ++q) {
        int j = rows[q];
        std::vector<double> out(row, 0.0);
        for (int64_t e = dst_off[j]; e < dst_off[j + 1]; ++e) {
            int i = src[e] % prev_rows;
            int nsh = delay[e];
            const double* brow = brdf + (((size_t)slot[e] * n_in + s_in[e]) * nd) * nb;
            for (int o = 0; o < nd; ++o)
                for (int b = 0; b < nb; ++b) {
                    double f = (fprime[e] * att_fac[(size_t)e * nb + b]) * brow[(size_t)o * nb + b];
                    const double* in = prev + (size_t)i * row + ((size_t)p2o[e] * nb + b) * nt;
                    double* o_ = out.data() + ((size_t)o * nb + b) * nt;
                    for (int t = nsh; t < nt; ++t) o_[t] += f * in[t - nsh];
                }
        }
        double s = 0.0;
        for (size_t k = 0; k < row; ++k) s += out[k];
        total += s;
    }
    return total;
}

// One order of RadiosityFast.py:1121-1143 for the listed destination rows,
// written out: out (n_rows, nd, nb, nt) FP64.  The previous order's
// histograms come as FP32 rows (the GPU's own state): the source row of pair
// e is prev[prev_row[e]] (nb * nt values, bands then bins), so a caller can
// pass only the rows the sampled destinations read.  Same loop and summation
// order as orc_exchange.
int orc_exchange_rows_out(int nd, int nb, int nt, const float* prev, const int64_t* prev_row,
                          const int64_t* dst_off, const int32_t* delay, const double* fprime, const double* att_fac,
                          const int32_t* slot, const int32_t* s_in, const double* brdf, int n_in, int n_rows,
                          const int32_t* rows, double* out) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int q = 0; q < n_rows; ++q) {
        const int j = rows[q];
        double* o_row = out + (size_t)q * nd * nb * nt;
        std::memset(o_row, 0, sizeof(double) * (size_t)nd * nb * nt);
        std::vector<double> in(nt);
        for (int64_t e = dst_off[j]; e < dst_off[j + 1]; ++e) {
            const int64_t nsh = delay[e];
            const double* brow = brdf + (((size_t)slot[e] * n_in + s_in[e]) * nd) * nb;
            for (int b = 0; b < nb; ++b) {
                const float* src = prev + ((size_t)prev_row[e] * nb + b) * nt;
                for (int t = 0; t < nt; ++t) in[t] = (double)src[t];
                for (int o = 0; o < nd; ++o) {
                    double f = (fprime[e] * att_fac[(size_t)e * nb + b]) * brow[(size_t)o * nb + b];
                    double* o_ = o_row + ((size_t)o * nb + b) * nt;
                    for (int64_t t = nsh; t < nt; ++t) o_[t] += f * in[t - nsh];
                }
            }
        }
    }
    return 0;
}

// RadiosityFast.py:686-752 `_collect_energy_patches` + :1148-1185
// `_collect_receiver_energy` for one receiver: out is (N, B, T).
int orc_collect(int n, int nd, int nb, int nt, const double* etot, const int32_t* ridx, const double* rfac,
                const double* dist, double c, double dt, const double* att, double* out) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k) {
        int64_t shift = (int64_t)std::ceil(dist[k] / c / dt);
        for (int b = 0; b < nb; ++b) {
            const double* in = etot + (((size_t)k * nd + ridx[k]) * nb + b) * nt;
            double* o = out + ((size_t)k * nb + b) * nt;
            double a = std::exp(-att[b] * dist[k]);
            int64_t s = ((shift % nt) + nt) % nt;
            for (int64_t t = 0; t < nt; ++t) {
                double e = in[t] * rfac[k];
                o[(t + s) % nt] = e * a;
            }
        }
    }
    return 0;
}

}  // extern "C"
