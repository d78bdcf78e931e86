// ct_common.cuh -- shared device types and exact float64 geometry predicates.
//
// Every float64 routine restates the upstream numba_celltree 0.4.2 function it
// names (file:line relative to the upstream project root) in the same
// evaluation order.  The library is compiled with -fmad=false, so no a*b+c is
// contracted into an FMA; together with IEEE division and sqrt this makes the
// results bit-identical to the upstream CPU code.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "celltree_gb300.h"

#define CT_FILL_VALUE (-1)
#define CT_MIN_TOLERANCE 1e-15    // constants.py:146
#define CT_TOLERANCE_FACTOR 1e-12 // constants.py:147
#define CT_MAX_N_VERTEX 32        // constants.py:134
#define CT_CLIP_MAX 64            // utils.py:101 (2 * MAX_N_VERTEX)

// device-side error word bits (see ct_status in celltree_gb300.h)
#define CT_DEVERR_STACK 1u      // traversal stack overflow
#define CT_DEVERR_BUCKET 2u     // a centroid fell outside every bucket
#define CT_DEVERR_CLIP 4u       // clip polygon scratch overflow
#define CT_DEVERR_CAPACITY 8u   // output capacity exceeded
#define CT_DEVERR_LOOP 16u      // bounded loop gave up

struct dpt {
    double x, y;
};

__device__ __forceinline__ dpt mkp(double x, double y) {
    dpt r;
    r.x = x;
    r.y = y;
    return r;
}
// to_vector(a, b) geometry_utils.py:23-25
__device__ __forceinline__ dpt vsub(dpt b, dpt a) { return mkp(b.x - a.x, b.y - a.y); }
// cross_product geometry_utils.py:57-59
__device__ __forceinline__ double crossp(dpt u, dpt v) { return u.x * v.y - u.y * v.x; }
// dot_product geometry_utils.py:62-64
__device__ __forceinline__ double dotp(dpt u, dpt v) { return u.x * v.x + u.y * v.y; }
// length_squared geometry_utils.py:67-69
__device__ __forceinline__ double len2(dpt v) { return v.x * v.x + v.y * v.y; }
// Python builtin min/max on floats: keep the first argument on ties.
__device__ __forceinline__ double pmin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double pmax(double a, double b) { return (b > a) ? b : a; }

// within_perpendicular_distance geometry_utils.py:150-166
__device__ __forceinline__ bool within_perp(double UxV, dpt U, double tol) {
    return (UxV * UxV) < ((tol * len2(U)) * tol);
}

// in_bounds geometry_utils.py:169-192
__device__ __forceinline__ bool in_bounds(dpt p, dpt a, dpt b) {
    double xmin = pmin(a.x, b.x), xmax = pmax(a.x, b.x);
    double ymin = pmin(a.y, b.y), ymax = pmax(a.y, b.y);
    double dx = xmax - xmin, dy = ymax - ymin;
    bool use_x = fabs(dx) >= fabs(dy);
    return (use_x && (p.x >= xmin && p.x <= xmax)) || (!use_x && (p.y >= ymin && p.y <= ymax));
}

// point_in_polygon_or_on_edge geometry_utils.py:195-223
__device__ __forceinline__ bool pip_or_edge(dpt p, const dpt* poly, int len, double tol) {
    dpt v0 = poly[len - 1];
    dpt U = vsub(v0, p);
    bool c = false;
    for (int i = 0; i < len; i++) {
        dpt v1 = poly[i];
        if (v1.x == v0.x && v1.y == v0.y) continue;
        dpt V = vsub(v1, p);
        double A = crossp(U, V);
        dpt W = vsub(v1, v0);
        if (within_perp(A, W, tol) && in_bounds(p, v0, v1)) return true;
        if (((v0.y > p.y) != (v1.y > p.y)) && p.x < ((v1.x - v0.x) * (p.y - v0.y) / (v1.y - v0.y) + v0.x)) c = !c;
        v0 = v1;
        U = V;
    }
    return c;
}

// point_on_edge geometry_utils.py:226-238
__device__ __forceinline__ bool point_on_edge(dpt p, dpt v0, dpt v1, double tol) {
    if (v1.x == v0.x && v1.y == v0.y) return false;
    dpt U = vsub(v0, p), V = vsub(v1, p), W = vsub(v1, v0);
    double A = crossp(U, V);
    return within_perp(A, W, tol) && in_bounds(p, v0, v1);
}

struct dbox {
    double xmin, xmax, ymin, ymax;
};
__device__ __forceinline__ dbox load_box(const double* b) {
    dbox r;
    r.xmin = b[0];
    r.xmax = b[1];
    r.ymin = b[2];
    r.ymax = b[3];
    return r;
}
// boxes_intersect geometry_utils.py:292-300
__device__ __forceinline__ bool boxes_intersect(const dbox& a, const dbox& b) {
    return a.xmin < b.xmax && b.xmin < a.xmax && a.ymin < b.ymax && b.ymin < a.ymax;
}
// box_contained geometry_utils.py:303-315
__device__ __forceinline__ bool box_contained(const dbox& a, const dbox& b) {
    return a.xmin >= b.xmin && a.xmax <= b.xmax && a.ymin >= b.ymin && a.ymax <= b.ymax;
}

// polygon_length geometry_utils.py:72-79
__device__ __forceinline__ int polygon_length(const int64_t* face, int n) {
    for (int i = 3; i < n; i++)
        if (face[i] == CT_FILL_VALUE) return i;
    return n;
}

// copy_vertices_into geometry_utils.py:501-510
__device__ __forceinline__ int gather_polygon(const double* __restrict__ v, const int64_t* __restrict__ face, int n,
                                              dpt* out) {
    int len = polygon_length(face, n);
    for (int i = 0; i < len; i++) {
        int64_t k = face[i];
        out[i] = mkp(v[2 * k], v[2 * k + 1]);
    }
    return len;
}

// Monotone 64-bit integer key of a float64 (non-NaN): x < y <=> key(x) < key(y),
// with -0.0 and +0.0 sharing one key (they compare equal as floats).
__device__ __forceinline__ unsigned long long fkey(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if (b == 0x8000000000000000ull) b = 0ull;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double fkey_inv(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// Diagonal of a box of sides dx, dy as numpy evaluates sqrt(dx**2 + dy**2)
// (bbox_distances, celltree_base.py:20-48): products and sum rounded
// separately (no fused multiply-add), so that the default tolerance derived
// from the largest diagonal is the same wherever it is computed.
__device__ __forceinline__ double box_diagonal(double dx, double dy) {
    return sqrt(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
}

__device__ __forceinline__ void set_error(unsigned int* err, unsigned int bit) {
    if (err) atomicOr(err, bit);
}
