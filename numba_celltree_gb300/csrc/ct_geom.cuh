// ct_geom.cuh -- exact float64 restatements of the upstream clipping, overlap,
// area and barycentric algorithms (numba_celltree 0.4.2 algorithms/*.py and
// geometry_utils.py), in upstream evaluation order.  Compiled with
// -fmad=false, so results are bit-identical to the upstream CPU code.
#pragma once

#include <cfloat>

#include "ct_common.cuh"
#include "ct_locf.cuh"

__device__ __forceinline__ double dnan() { return __longlong_as_double(0x7ff8000000000000ll); }

// ---------------------------------------------------------------------------
// Cohen-Sutherland (algorithms/cohen_sutherland.py:18-101)
// ---------------------------------------------------------------------------
enum { CS_INSIDE = 0, CS_LEFT = 1, CS_RIGHT = 2, CS_LOWER = 4, CS_UPPER = 8 };

__device__ __forceinline__ int cs_code(dpt a, const dbox& b) {
    int p = CS_INSIDE;
    if (a.x < b.xmin) p |= CS_LEFT;
    else if (a.x > b.xmax) p |= CS_RIGHT;
    if (a.y < b.ymin) p |= CS_LOWER;
    else if (a.y > b.ymax) p |= CS_UPPER;
    return p;
}

// Returns 1 (clipped segment c-d), 0 (no intersection, c = d = NaN) or -1
// when the loop did not settle within 64 rounds (upstream loops until done;
// each round fixes one outcode bit, so it settles in at most four).
__device__ __forceinline__ int cohen_sutherland(dpt a, dpt b, const dbox& box, dpt* c, dpt* d) {
    *c = mkp(dnan(), dnan());
    *d = *c;
    double dx = b.x - a.x, dy = b.y - a.y;
    if (dx == 0.0 && dy == 0.0) return 0;
    int k1 = cs_code(a, box), k2 = cs_code(b, box);
    int iter = 0;
    while ((k1 | k2) != CS_INSIDE) {
        if ((k1 & k2) != 0) return 0;
        if (++iter > 64) return -1;
        int opt = k1 ? k1 : k2;
        double x, y;
        if (opt & CS_UPPER) {
            x = a.x + dx * (box.ymax - a.y) / dy;
            y = box.ymax;
        } else if (opt & CS_LOWER) {
            x = a.x + dx * (box.ymin - a.y) / dy;
            y = box.ymin;
        } else if (opt & CS_RIGHT) {
            y = a.y + dy * (box.xmax - a.x) / dx;
            x = box.xmax;
        } else {
            y = a.y + dy * (box.xmin - a.x) / dx;
            x = box.xmin;
        }
        if (opt == k1) {
            a = mkp(x, y);
            k1 = cs_code(a, box);
        } else if (opt == k2) {
            b = mkp(x, y);
            k2 = cs_code(b, box);
        }
        dx = b.x - a.x;
        dy = b.y - a.y;
        if (dx == 0.0 && dy == 0.0) return 0;
    }
    *c = a;
    *d = b;
    return 1;
}

// ---------------------------------------------------------------------------
// Cyrus-Beck / Skala (algorithms/cyrus_beck.py:26-241)
// ---------------------------------------------------------------------------

// compute_intersection cyrus_beck.py:26-43
__device__ __forceinline__ double cb_param(dpt a, dpt s, dpt v0, dpt v1, bool* entering) {
    dpt si = vsub(v0, a);
    dpt n = mkp(-(v1.y - v0.y), (v1.x - v0.x));
    double n_si = dotp(n, si);
    double k = dotp(n, s);
    double t = n_si / k;
    *entering = n_si > 0;
    return t;
}

// aligned cyrus_beck.py:76-91
__device__ __forceinline__ bool cb_aligned(dpt U, dpt V) {
    if ((U.x == 0 && U.y == 0) || (V.x == 0 && V.y == 0)) return true;
    if (U.x != 0 && V.x != 0) return (U.x > 0) == (V.x > 0);
    if (U.y != 0 && V.y != 0) return (U.y > 0) == (V.y > 0);
    return false;
}

// collinear_case cyrus_beck.py:94-130 (overlap 66-73)
__device__ __forceinline__ bool cb_collinear(dpt a, dpt b, dpt v0, dpt v1, dpt* c, dpt* d) {
    dpt _b = mkp(b.x - a.x, b.y - a.y);
    dpt _v0 = mkp(v0.x - a.x, v0.y - a.y);
    dpt _v1 = mkp(v1.x - a.x, v1.y - a.y);
    if (!cb_aligned(_b, vsub(_v1, _v0))) {
        dpt t = v0;
        v0 = v1;
        v1 = t;
        t = _v0;
        _v0 = _v1;
        _v1 = t;
    }
    dpt n = mkp(-_b.y, _b.x);
    double ta = 0.0, tb = crossp(n, _b), t0 = crossp(n, _v0), t1 = crossp(n, _v1);
    double xa = ta, xb = tb, x0 = t0, x1 = t1;
    if (xa > xb) {
        double t = xa;
        xa = xb;
        xb = t;
    }
    if (x0 > x1) {
        double t = x0;
        x0 = x1;
        x1 = t;
    }
    double ov = pmin(xb, x1) - pmax(xa, x0);
    if (!(ov > 0.0)) return false;  // max(0, ov) > 0
    *c = (t0 < ta) ? v0 : a;
    *d = (t1 > tb) ? v1 : b;
    return true;
}

// cyrus_beck_line_polygon_clip cyrus_beck.py:133-241
__device__ __forceinline__ bool cyrus_beck(dpt a, dpt b, const dpt* poly, int length, double tol, dpt* c, dpt* d) {
    *c = mkp(dnan(), dnan());
    *d = *c;
    dpt s = vsub(b, a);
    if (s.x == 0 && s.y == 0) return false;
    bool a_inside = pip_or_edge(a, poly, length, tol);
    bool b_inside = pip_or_edge(b, poly, length, tol);
    if (a_inside && b_inside) {
        *c = a;
        *d = b;
        return true;
    }
    int i0 = -1, i1 = -1, i = 0, k = 0;
    double ksi = crossp(vsub(poly[0], a), s);
    while (i < length && k < 2) {
        dpt v0 = poly[i], v1 = poly[(i + 1) % length];
        double eta = crossp(vsub(v1, a), s);
        if ((ksi < 0.0) != (eta < 0.0)) {
            if (k == 0) i0 = i;
            else i1 = i;
            k++;
        } else if (ksi == 0.0 && eta == 0.0) {
            bool r = cb_collinear(a, b, v0, v1, c, d);
            if (!r) {
                *c = mkp(dnan(), dnan());
                *d = *c;
            }
            return r;
        }
        ksi = eta;
        i++;
    }
    if (k == 0) return false;
    // intersections cyrus_beck.py:46-63 (Python index -1 wraps)
    int j0 = i0 < 0 ? i0 + length : i0, j1 = i1 < 0 ? i1 + length : i1;
    dpt v0 = poly[j0], v01 = poly[(i0 + 1) % length];
    dpt v1 = poly[j1], v11 = poly[((i1 + 1) % length + length) % length];
    bool e0, e1;
    double t0 = cb_param(a, s, v0, v01, &e0);
    double t1 = cb_param(a, s, v1, v11, &e1);
    if (e1) {
        double t = t0;
        t0 = t1;
        t1 = t;
    }
    if (t0 == t1) {
        if (a_inside && t1 != 0.0) t0 = 0.0;
        else if (b_inside && t0 != 1.0) t1 = 1.0;
        else return false;
    }
    if (t1 < t0) {
        double t = t0;
        t0 = t1;
        t1 = t;
    }
    bool valid0 = t0 >= 0 && t0 < 1;
    bool valid1 = t1 > 0 && t1 <= 1;
    if (valid0 && valid1) {
        *c = mkp(a.x + t0 * s.x, a.y + t0 * s.y);
        *d = mkp(a.x + t1 * s.x, a.y + t1 * s.y);
        return true;
    } else if (valid0) {
        *c = mkp(a.x + t0 * s.x, a.y + t0 * s.y);
        *d = b;
        return true;
    } else if (valid1) {
        *c = a;
        *d = mkp(a.x + t1 * s.x, a.y + t1 * s.y);
        return true;
    }
    return false;
}

// ---------------------------------------------------------------------------
// lines_intersect geometry_utils.py:318-418
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool left_of(dpt a, dpt p, dpt U) { return U.x * (a.y - p.y) > U.y * (a.x - p.x); }
__device__ __forceinline__ bool has_overlap(double a, double b, double p, double q, double tol) {
    return ((pmin(a, b) - pmax(p, q)) < tol) && ((pmin(p, q) - pmax(a, b)) < tol);
}

__device__ __forceinline__ bool lines_intersect(dpt a, dpt b, dpt p, dpt q, double* x, double* y) {
    dpt V = vsub(b, a), U = vsub(q, p);
    *x = dnan();
    *y = dnan();
    if ((U.x == 0 && U.y == 0) || (V.x == 0 && V.y == 0)) return false;
    if ((U.x == 0) && (V.x == 0) && a.x != p.x) return false;
    if ((U.y == 0) && (V.y == 0) && a.y != p.y) return false;
    double tol = pmax(CT_MIN_TOLERANCE, CT_TOLERANCE_FACTOR * pmax(fabs(U.x), fabs(U.y)));
    if (!has_overlap(a.x, b.x, p.x, q.x, tol) || !has_overlap(a.y, b.y, p.y, q.y, tol)) return false;
    if ((left_of(a, p, U) != left_of(b, p, U)) && (left_of(p, a, V) != left_of(q, a, V))) {
        double denom = crossp(V, U);
        if (within_perp(denom, V, tol)) return true;  // parallel: NaN point
        dpt R = vsub(p, a);
        double t = crossp(R, U) / denom;
        *x = a.x + t * V.x;
        *y = a.y + t * V.y;
        return true;
    }
    dpt R = vsub(p, a), S = vsub(q, a);
    if (within_perp(crossp(V, R), V, tol) && within_perp(crossp(V, S), V, tol)) {
        dpt aa = a, bb = b, pp = p, qq = q, t;
        if (aa.x > bb.x || (aa.x == bb.x && aa.y > bb.y)) {
            t = aa;
            aa = bb;
            bb = t;
        }
        if (pp.x > qq.x || (pp.x == qq.x && pp.y > qq.y)) {
            t = pp;
            pp = qq;
            qq = t;
        }
        double sx = pmax(aa.x, pp.x), sy = pmax(aa.y, pp.y);
        double ex = pmin(bb.x, qq.x), ey = pmin(bb.y, qq.y);
        if (sx > ex || sy > ey) return true;  // no overlap: NaN point
        *x = 0.5 * (sx + ex);
        *y = 0.5 * (sy + ey);
        return true;
    }
    return false;
}

// ---------------------------------------------------------------------------
// separating axes (algorithms/separating_axis.py:17-55)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool separating_axes(const dpt* a, int la, const dpt* b, int lb) {
    dpt p = a[la - 1];
    for (int i = 0; i < la; i++) {
        dpt q = a[i];
        dpt norm = mkp(p.y - q.y, q.x - p.x);
        p = q;
        if (norm.x == 0.0 && norm.y == 0.0) continue;
        double mina = DBL_MAX, maxa = -DBL_MAX, minb = DBL_MAX, maxb = -DBL_MAX;
        for (int j = 0; j < la; j++) {
            double proj = dotp(a[j], norm);
            mina = pmin(mina, proj);
            maxa = pmax(maxa, proj);
        }
        for (int j = 0; j < lb; j++) {
            double proj = dotp(b[j], norm);
            minb = pmin(minb, proj);
            maxb = pmax(maxb, proj);
        }
        if (!(maxa > minb && maxb > mina)) return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Sutherland-Hodgman (algorithms/sutherland_hodgman.py:56-148) and
// polygon_area (geometry_utils.py:82-95)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double polygon_area(const dpt* poly, int len) {
    double area = 0.0;
    dpt a = poly[0], b = poly[1];
    dpt U = vsub(b, a);
    for (int i = 2; i < len; i++) {
        dpt c = poly[i];
        dpt V = vsub(a, c);
        area += fabs(crossp(U, V));
        U = V;
    }
    return 0.5 * area;
}

__device__ __forceinline__ bool sh_inside(dpt p, dpt r, dpt U) { return U.x * (p.y - r.y) > U.y * (p.x - r.x); }

__device__ __forceinline__ bool sh_intersection(dpt a, dpt V, dpt r, dpt N, dpt* out) {
    dpt W = mkp(r.x - a.x, r.y - a.y);
    double nw = dotp(N, W), nv = dotp(N, V);
    if (nv != 0) {
        double t = nw / nv;
        *out = mkp(a.x + t * V.x, a.y + t * V.y);
        return true;
    }
    return false;
}

// One clip edge of polygon_polygon_clip_area (sutherland_hodgman.py:104-138):
// `subject` (length vertices) clipped by the line through r with direction U
// (normal N) into `output`.  Returns the output length, or -1 when the output
// would exceed CT_CLIP_MAX vertices (upstream writes past its stack arrays).
__device__ __forceinline__ int sh_clip_edge_seq(const dpt* subject, int length, dpt* output, dpt r, dpt U, dpt N) {
    int n_output = 0;
    dpt a = subject[length - 1];
    bool a_inside = sh_inside(a, r, U);
    for (int j = 0; j < length; j++) {
        dpt b = subject[j];
        dpt V = mkp(b.x - a.x, b.y - a.y);
        if (V.x == 0 && V.y == 0) continue;
        bool b_inside = sh_inside(b, r, U);
        dpt pnt;
        if (b_inside) {
            if (!a_inside) {
                if (sh_intersection(a, V, r, N, &pnt)) {
                    if (n_output >= CT_CLIP_MAX) return -1;
                    output[n_output++] = pnt;
                }
            }
            if (n_output >= CT_CLIP_MAX) return -1;
            output[n_output++] = b;
        } else if (a_inside) {
            if (sh_intersection(a, V, r, N, &pnt)) {
                if (n_output >= CT_CLIP_MAX) return -1;
                output[n_output++] = pnt;
            } else {
                b_inside = true;
                if (n_output >= CT_CLIP_MAX) return -1;
                output[n_output++] = b;
            }
        }
        a = b;
        a_inside = b_inside;
    }
    return n_output;
}

// polygon_polygon_clip_area: `subject` is clipped by `clipper`.  Uses two
// CT_CLIP_MAX-vertex scratch polygons; returns NaN and sets *overflow if the
// clipped polygon would exceed them (upstream writes past its stack arrays).
__device__ __forceinline__ double clip_area(const dpt* polygon, int n_poly, const dpt* clipper, int n_clip, dpt* bufA,
                                            dpt* bufB, bool* overflow) {
    dpt* output = bufA;
    dpt* subject = bufB;
    int n_output = n_poly;
    for (int i = 0; i < n_poly; i++) output[i] = polygon[i];
    dpt r = clipper[n_clip - 1];
    for (int i = 0; i < n_clip; i++) {
        dpt s = clipper[i];
        dpt U = mkp(s.x - r.x, s.y - r.y);
        if (U.x == 0 && U.y == 0) continue;
        dpt N = mkp(-U.y, U.x);
        int length = n_output;
        dpt* t = subject;  // swap roles instead of copying output into subject
        subject = output;
        output = t;
        n_output = sh_clip_edge_seq(subject, length, output, r, U, N);
        if (n_output < 0) {
            *overflow = true;
            return dnan();
        }
        if (n_output < 3) return 0.0;
        r = s;
    }
    return polygon_area(output, n_output);
}

// ---------------------------------------------------------------------------
// The same clip with each clip edge's float64 work in converged passes.
//
// The sequential walk computes an intersection wherever it crosses the clip
// line.  The lanes of a warp cross at different steps, so on a GPU the
// intersection code runs at almost every step with a few lanes active, and
// the float64 pipe -- the bound of these kernels on GB300 -- spends most of
// its issue slots on idle lanes.  Here each clip edge runs
//   1. the inside test of every subject vertex, all lanes in step;
//   2. integer bookkeeping: the skipped steps (zero-length edges, b - a == 0
//      <=> finite and equal coordinates), the crossings and the output slot
//      of every pushed vertex, copying the vertices that stay;
//   3. one pass per crossing (usually two per clip edge, all lanes in step)
//      computing the intersection into its slot.
// The output polygon, its order and every value are those of the walk.  A
// crossing whose intersection fails (N.V == 0, where the walk pushes a
// vertex instead and flips its inside flag) sends the lane through the walk
// for that clip edge.  Order comparisons and zero tests run on integer keys.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool g_notnan(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull) <= 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool g_finite(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull) < 0x7ff0000000000000ull;
}
// x == 0.0 (either sign)
__device__ __forceinline__ bool g_zero(double x) { return ((unsigned long long)__double_as_longlong(x) << 1) == 0ull; }
// x > y, false when either is NaN (the float64 comparison)
__device__ __forceinline__ bool g_gt(double x, double y) { return g_notnan(x) && g_notnan(y) && fkey(x) > fkey(y); }
// x == y as values for finite x, y (bit patterns equal, or both zeros)
__device__ __forceinline__ bool g_eq_finite(double x, double y) {
    unsigned long long a = (unsigned long long)__double_as_longlong(x), b = (unsigned long long)__double_as_longlong(y);
    return a == b || ((a | b) << 1) == 0ull;
}
// b - a == (0, 0): both coordinates finite and equal
__device__ __forceinline__ bool g_zero_edge(dpt a, dpt b) {
    return g_finite(a.x) && g_finite(b.x) && g_finite(a.y) && g_finite(b.y) && g_eq_finite(a.x, b.x) &&
           g_eq_finite(a.y, b.y);
}

// Float32 local coordinates of a float64 point: v - o in a frame at the
// point split in O (each coordinate split exactly into float hi + lo), with
// the per-component error bound folded into *ed (a running maximum).
__device__ __forceinline__ float2 g_local(dpt v, const PtSplit& O, float* ed) {
    PtSplit P = split_point(v.x, v.y);
    float dx, dy, e;
    local_delta(P, make_float4(O.xh, O.xl, O.yh, O.yl), &dx, &dy, &e);
    *ed = fmaxf(*ed, e);
    return make_float2(dx, dy);
}

__device__ __forceinline__ double clip_area_conv(const dpt* polygon, int n_poly, const dpt* clipper, int n_clip,
                                                 dpt* bufA, dpt* bufB, bool* overflow) {
    static_assert(CT_CLIP_MAX <= 64, "vertex masks are 64-bit");
    const float u24 = 5.9604644775390625e-08f;  // 2^-24
    dpt* output = bufA;
    const dpt* subject = polygon;  // the first clip edge reads the polygon in place
    int n_output = n_poly;
    unsigned short xs[CT_CLIP_MAX];  // crossings: step j | last kept step << 6 (slot in xslot)
    unsigned char xslot[CT_CLIP_MAX];
    // float32 local coordinates (frame at the first clipper vertex) of the
    // subject, output and clipper vertices, for the filtered inside test
    float2 fP[CT_MAX_N_VERTEX], fA[CT_CLIP_MAX], fB[CT_CLIP_MAX], fC[CT_MAX_N_VERTEX];
    float ed = 0.0f;
    const PtSplit O = split_point(clipper[0].x, clipper[0].y);
    for (int k = 0; k < n_clip; k++) fC[k] = g_local(clipper[k], O, &ed);
    for (int k = 0; k < n_poly; k++) fP[k] = g_local(polygon[k], O, &ed);
    const float2* fsub = fP;
    float2* fout = fA;
    dpt r = clipper[n_clip - 1];
    float2 fr = fC[n_clip - 1];
    for (int i = 0; i < n_clip; i++) {
        dpt s = clipper[i];
        dpt U = mkp(s.x - r.x, s.y - r.y);
        if (g_zero(U.x) && g_zero(U.y)) continue;
        dpt N = mkp(-U.y, U.x);
        int length = n_output;
        // float32 U and its error against the float64 U
        const float2 fs = fC[i];
        const float ufx = fs.x - fr.x, ufy = fs.y - fr.y;
        const float eU = 2.0f * ed + 2.0f * u24 * fmaxf(fabsf(ufx), fabsf(ufy));
        const float Nu = fabsf(ufx) + fabsf(ufy) + 2.0f * eU;
        // 1. inside flags and zero-length steps.  The inside test is decided
        // in float32 when its margin clears the float32 error and the float64
        // rounding of both products; otherwise in float64 as upstream.
        unsigned long long inside = 0ull, skip = 0ull;
        dpt prev = subject[length - 1];
        for (int j = 0; j < length; j++) {
            dpt b = subject[j];
            const float2 fb = fsub[j];
            float wx = fb.x - fr.x, wy = fb.y - fr.y;
            float ew = 2.0f * ed + u24 * fmaxf(fabsf(wx), fabsf(wy));
            float M = fmaxf(fabsf(wx), fabsf(wy)) + ew;
            float est = ufx * wy - ufy * wx;
            float thr = 1.02f * (2.0f * eU * M + Nu * ew + 4.0f * u24 * Nu * M + 2.2204461e-16f * Nu * M) + 1e-37f;
            bool in;
            if (fabsf(est) > thr) {
                in = est > 0.0f;
            } else {
                double lhs = U.x * (b.y - r.y);
                double rhs = U.y * (b.x - r.x);
                in = g_gt(lhs, rhs);
            }
            if (in) inside |= 1ull << j;
            if (g_zero_edge(prev, b)) skip |= 1ull << j;
            prev = b;
        }
        // 2. walk on the flags: slots of the kept vertices and of the crossings
        bool a_in = (inside >> (length - 1)) & 1ull;
        int a_idx = length - 1;
        int n_out = 0, n_x = 0;
        for (int j = 0; j < length; j++) {
            if ((skip >> j) & 1ull) continue;
            bool b_in = (inside >> j) & 1ull;
            if (b_in != a_in) {
                xs[n_x] = (unsigned short)(j | (a_idx << 6));
                xslot[n_x] = (unsigned char)(n_out < 255 ? n_out : 255);
                n_x++;
                n_out++;
            }
            if (b_in) {
                if (n_out < CT_CLIP_MAX) {
                    output[n_out] = subject[j];
                    fout[n_out] = fsub[j];
                }
                n_out++;
            }
            a_in = b_in;
            a_idx = j;
        }
        // 3. intersections (sh_intersection), all lanes in step
        bool fail = false;
        for (int k = 0; k < n_x; k++) {
            int j = xs[k] & 63, ai = xs[k] >> 6;
            dpt a = subject[ai], b = subject[j];
            dpt V = mkp(b.x - a.x, b.y - a.y);
            dpt W = mkp(r.x - a.x, r.y - a.y);
            double nw = dotp(N, W), nv = dotp(N, V);
            if (!g_zero(nv)) {
                double t = nw / nv;
                int slot = xslot[k];
                dpt pnt = mkp(a.x + t * V.x, a.y + t * V.y);
                if (slot < CT_CLIP_MAX) {
                    output[slot] = pnt;
                    fout[slot] = g_local(pnt, O, &ed);
                }
            } else {
                fail = true;
            }
        }
        if (fail) {
            n_out = sh_clip_edge_seq(subject, length, output, r, U, N);
            for (int k = 0; k < n_out; k++) fout[k] = g_local(output[k], O, &ed);
        } else if (n_out > CT_CLIP_MAX) {
            n_out = -1;
        }
        if (n_out < 0) {
            *overflow = true;
            return dnan();
        }
        n_output = n_out;
        if (n_output < 3) return 0.0;
        // the output becomes the next subject
        subject = output;
        fsub = fout;
        output = (output == bufA) ? bufB : bufA;
        fout = (fout == fA) ? fB : fA;
        r = s;
        fr = fs;
    }
    return polygon_area(subject, n_output);
}

// ---------------------------------------------------------------------------
// barycentric weights (algorithms/barycentric_triangle.py:28-43,
// barycentric_wachspress.py:26-85)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tri_weights(dpt a, dpt b, dpt c, dpt p, double* w) {
    dpt ab = vsub(b, a), ac = vsub(c, a), ap = vsub(p, a);
    double Aa = fabs(crossp(ab, ap)), Ac = fabs(crossp(ac, ap)), A = fabs(crossp(ab, ac));
    double inv_denom = 1.0 / A;
    double ww = inv_denom * Aa, v = inv_denom * Ac;
    double u = 1.0 - v - ww;
    w[0] = u;
    w[1] = v;
    w[2] = ww;
}

__device__ __forceinline__ void interp_edge(dpt a, dpt U, dpt p, double* w, int K, int i, int j) {
    for (int k = 0; k < K; k++) w[k] = 0.0;
    dpt V = vsub(p, a);
    double ww = sqrt(dotp(V, V)) / sqrt(dotp(U, U));
    w[i] = 1.0 - ww;
    w[j] = ww;
}

__device__ __forceinline__ void wachspress(const dpt* poly, int n, dpt p, double* w, int K, double tol) {
    double w_sum = 0.0;
    dpt a = poly[n - 1], b = poly[0];
    dpt U = vsub(b, a), V = vsub(p, a);
    double Ai = fabs(crossp(U, V));
    if (within_perp(Ai, U, tol)) {
        interp_edge(a, U, p, w, K, n - 1, 0);
        return;
    }
    for (int i = 0; i < n; i++) {
        int i_next = (i + 1) % n;
        dpt c = poly[i_next];
        dpt W = vsub(c, a);
        double Ci = fabs(crossp(U, W));
        U = vsub(c, b);
        V = vsub(p, b);
        double Aj = fabs(crossp(U, V));
        if (within_perp(Aj, U, tol)) {
            interp_edge(b, U, p, w, K, i, i_next);
            return;
        }
        double ww = 2.0 * Ci / (Ai * Aj);
        w[i] = ww;
        w_sum += ww;
        a = b;
        b = c;
        Ai = Aj;
    }
    for (int i = 0; i < n; i++) w[i] /= w_sum;
}
