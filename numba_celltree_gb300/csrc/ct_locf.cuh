// ct_locf.cuh -- float32 leaf data in a per-cell local frame and the float32
// filters of the leaf predicates.
//
// Layout of one cell in `poly_f32` (leaf order, stride ct_poly32_stride(K)
// float4 units): float4 (x0_hi, x0_lo, y0_hi, y0_lo) -- the cell's first
// vertex split exactly as hi + lo with hi the float64 truncated to 24
// significant bits and lo the remainder rounded to float -- followed by
// float2 (v_k - v_0) for the remaining vertices (repeated consecutive
// vertices removed, as the float64 predicate skips them,
// geometry_utils.py:203-204).  A query point is split the same way once; the
// point-to-vertex vector (p - v0) = (p_hi - v0_hi) + (p_lo - v0_lo) is then
// accurate to float32 rounding of the local difference, so the error bounds
// of the filters scale with the cell size, not with the coordinates'
// magnitude.
#pragma once

#include "ct_common.cuh"

// float4 units per cell for n_max_vert K
__host__ __device__ __forceinline__ int poly32_stride(int K) { return 1 + (K - 1 + 1) / 2; }

// x = hi + lo: hi is x with its mantissa truncated to 24 bits (exactly a
// float when in range), lo the dropped bits rounded to float (error at most
// 2^-24 |lo|).  Integer operations only.
__device__ __forceinline__ float split_hi(double x, float* lo) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    int e = (int)((b >> 52) & 0x7ff);
    unsigned sign = (b >> 63) ? 0x80000000u : 0u;
    if (e == 0) {  // zero or subnormal: below float range
        *lo = 0.0f;
        return __int_as_float(sign);
    }
    if (e == 0x7ff) {  // inf / nan
        *lo = 0.0f;
        return __int_as_float(sign | 0x7f800000u | ((b & 0x000fffffffffffffull) ? 0x400000u : 0u));
    }
    int fe = e - 1023 + 127;
    if (fe >= 255) {
        *lo = 0.0f;
        return __int_as_float(sign | 0x7f800000u);
    }
    if (fe <= 0) {  // |x| < 2^-126: treated as 0 (covered by the absolute floor of the bounds)
        *lo = 0.0f;
        return __int_as_float(sign);
    }
    float hf = __int_as_float(sign | ((unsigned)fe << 23) | (unsigned)((b >> 29) & 0x7fffffu));
    unsigned m = (unsigned)(b & 0x1fffffffull);
    float l = 0.0f;
    if (m) {
        // m * 2^(e - 1075): the power of two built from its exponent bits when
        // it is a normal float (the product is then exact), else ldexpf
        int pe = e - 1075 + 127;
        l = (pe >= 1 && pe <= 254) ? __uint2float_rn(m) * __int_as_float(pe << 23)
                                   : ldexpf(__uint2float_rn(m), e - 1075);
        if (sign) l = -l;
    }
    *lo = l;
    return hf;
}

struct PtSplit {
    float xh, xl, yh, yl;
};

__device__ __forceinline__ PtSplit split_point(double x, double y) {
    PtSplit P;
    P.xh = split_hi(x, &P.xl);
    P.yh = split_hi(y, &P.yl);
    return P;
}

// d = p - v0 in float32 and a bound on its per-component error
__device__ __forceinline__ void local_delta(const PtSplit& P, float4 o, float* dx, float* dy, float* errd) {
    float t1x = P.xh - o.x, t2x = P.xl - o.y;
    float t1y = P.yh - o.z, t2y = P.yl - o.w;
    float rx = t1x + t2x, ry = t1y + t2y;
    *dx = rx;
    *dy = ry;
    // three float32 roundings plus the conversions of the two lo parts
    float ex = fabsf(t1x) + fabsf(t2x) + fabsf(rx) + fabsf(P.xl) + fabsf(o.y);
    float ey = fabsf(t1y) + fabsf(t2y) + fabsf(ry) + fabsf(P.yl) + fabsf(o.w);
    *errd = 5.9604644775390625e-08f * fmaxf(ex, ey) + 1e-37f;
}

enum { LF_OUTSIDE = 0, LF_INSIDE = 1, LF_UNSURE = 2 };

// Float32 filter for point_in_polygon_or_on_edge (geometry_utils.py:195-223).
// U_k = v_k - p.  For an edge (U0, U1) with m the largest |component| and e the
// per-component error of the U's, the float32 cross product A differs from the
// exact cross product of the float64 geometry by at most
// 8u m^2 + 4 m e + 2 e^2 (u = 2^-24), and moving the vertices along the
// segment between their float64 and float32 positions changes A by at most
// 4 m e + 6 e^2.  If |A| > 2 (8u m^2 + 4 m e + 6 e^2) + tol (|Wx|+|Wy|+2e),
// then (1) the float64 on-edge test of the edge is false and (2) the point is
// off the edge line throughout, so the crossing parity of the float32
// configuration -- computed exactly from the signs of A and of the y
// components -- equals the float64 parity.  e includes `dabs`, the float64
// rounding of absolute coordinates, so the float64 crossing abscissa is also
// resolved.  Otherwise the polygon is UNSURE.
template <int KT>
__device__ __forceinline__ int leaf_filter_local(const PtSplit& P, float dabs, float tolf,
                                                 const float4* __restrict__ cell, int len) {
    const float u = 5.9604644775390625e-08f;
    if (len < 3) return LF_UNSURE;
    float4 o = cell[0];
    const float2* rel = reinterpret_cast<const float2*>(cell + 1);
    float dx, dy, errd;
    local_delta(P, o, &dx, &dy, &errd);
    float dmax = fmaxf(fabsf(dx), fabsf(dy));
    float2 rl = rel[len - 2];
    float ux = rl.x - dx, uy = rl.y - dy;
    int parity = 0;
#pragma unroll
    for (int k = 0; k < KT; k++) {
        if (k >= len) break;
        float vx, vy;
        if (k == 0) {
            vx = -dx;
            vy = -dy;
        } else {
            float2 r = rel[k - 1];
            vx = r.x - dx;
            vy = r.y - dy;
        }
        float A = ux * vy - uy * vx;
        float m = fmaxf(fmaxf(fabsf(ux), fabsf(uy)), fmaxf(fabsf(vx), fabsf(vy)));
        float e = errd + 1.1920928955078125e-07f * (m + dmax) + dabs;
        float wx = vx - ux, wy = vy - uy;
        float thr = 2.0f * (8.0f * u * m * m + 4.0f * m * e + 6.0f * e * e) +
                    tolf * (fabsf(wx) + fabsf(wy) + 2.0f * e) * 1.000001f + 1e-30f;
        if (!(fabsf(A) > thr)) return LF_UNSURE;
        if ((uy > 0.0f) != (vy > 0.0f)) parity ^= (int)((vy > uy) ? (A > 0.0f) : (A < 0.0f));
        ux = vx;
        uy = vy;
    }
    return parity ? LF_INSIDE : LF_OUTSIDE;
}

// Float32 filter for point_on_edge (geometry_utils.py:226-238): true when the
// point is certainly farther than the tolerance from the edge line.
__device__ __forceinline__ bool edge_surely_off_local(const PtSplit& P, float dabs, float tolf,
                                                      const float4* __restrict__ cell) {
    const float u = 5.9604644775390625e-08f;
    float4 o = cell[0];
    float2 r = reinterpret_cast<const float2*>(cell + 1)[0];
    float dx, dy, errd;
    local_delta(P, o, &dx, &dy, &errd);
    float dmax = fmaxf(fabsf(dx), fabsf(dy));
    float ux = -dx, uy = -dy, vx = r.x - dx, vy = r.y - dy;
    float A = ux * vy - uy * vx;
    float m = fmaxf(fmaxf(fabsf(ux), fabsf(uy)), fmaxf(fabsf(vx), fabsf(vy)));
    float e = errd + 1.1920928955078125e-07f * (m + dmax) + dabs;
    float wx = vx - ux, wy = vy - uy;
    float thr = 2.0f * (8.0f * u * m * m + 4.0f * m * e + 6.0f * e * e) +
                tolf * (fabsf(wx) + fabsf(wy) + 2.0f * e) * 1.000001f + 1e-30f;
    return fabsf(A) > thr;
}

// Cheaper variant of leaf_filter_local for the batched pass: one threshold
// per polygon from M = the largest |component| of all U_k (>= every edge's m)
// and e = errd + 2^-23 (M + dmax) + dabs (>= every edge's e); |W| <= 4M per
// edge.  Both bounds only grow, so every INSIDE / OUTSIDE decision remains
// exact; the polygon is UNSURE a little more often.
template <int KT>
__device__ __forceinline__ int leaf_filter_poly(const PtSplit& P, float dabs, float tolf,
                                                const float4* __restrict__ cell, int len) {
    const float u = 5.9604644775390625e-08f;
    if (len < 3 || len > KT) return LF_UNSURE;
    float4 o = cell[0];
    const float2* rel = reinterpret_cast<const float2*>(cell + 1);
    float dx, dy, errd;
    local_delta(P, o, &dx, &dy, &errd);
    float ux[KT], uy[KT];
    ux[0] = -dx;
    uy[0] = -dy;
    float M = fmaxf(fabsf(dx), fabsf(dy));
    float dmax = M;
#pragma unroll
    for (int k = 1; k < KT; k++) {
        if (k < len) {
            float2 r = rel[k - 1];
            ux[k] = r.x - dx;
            uy[k] = r.y - dy;
            M = fmaxf(M, fmaxf(fabsf(ux[k]), fabsf(uy[k])));
        }
    }
    float e = errd + 1.1920928955078125e-07f * (M + dmax) + dabs;
    float thr = 2.0f * (8.0f * u * M * M + 4.0f * M * e + 6.0f * e * e) + tolf * (4.0f * M + 2.0f * e) * 1.000001f +
                1e-30f;
    float px_ = ux[0], py_ = uy[0];
#pragma unroll
    for (int k = 1; k < KT; k++)
        if (k == len - 1) {
            px_ = ux[k];
            py_ = uy[k];
        }
    int parity = 0;
    bool unsure = false;
#pragma unroll
    for (int k = 0; k < KT; k++) {
        if (k < len) {
            float vx = ux[k], vy = uy[k];
            float A = px_ * vy - py_ * vx;
            unsure |= !(fabsf(A) > thr);
            if ((py_ > 0.0f) != (vy > 0.0f)) parity ^= (int)((vy > py_) ? (A > 0.0f) : (A < 0.0f));
            px_ = vx;
            py_ = vy;
        }
    }
    if (unsure) return LF_UNSURE;
    return parity ? LF_INSIDE : LF_OUTSIDE;
}

// One cell of the leaf-ordered polygon arrays: its K float64 vertices (NaN
// padded past its length) and its float32 local-frame record (first vertex
// split hi + lo, the other distinct consecutive vertices as float32 offsets),
// its length and the length without repeated consecutive vertices.
__device__ __forceinline__ void pack_cell(const int64_t* __restrict__ e, int K, bool is_edge,
                                          const double* __restrict__ v, double2* __restrict__ P,
                                          float4* __restrict__ C, uint8_t* plen, uint8_t* plen32) {
    int len = is_edge ? 2 : polygon_length(e, K);
    const int S4 = poly32_stride(K);
    float2* rel = reinterpret_cast<float2*>(C + 1);
    for (int k = 0; k < len; k++) P[k] = make_double2(v[2 * e[k]], v[2 * e[k] + 1]);
    for (int k = len; k < K; k++) P[k] = make_double2(__longlong_as_double(0x7ff8000000000000ll), 0.0);
    int m = 0;
    double2 v0 = make_double2(0.0, 0.0);
    if (len > 0) {
        double2 prev = P[len - 1];
        for (int k = 0; k < len; k++) {
            double2 c = P[k];
            if (c.x == prev.x && c.y == prev.y) continue;
            if (m == 0) {
                v0 = c;
                float xl, yl;
                float xh = split_hi(c.x, &xl), yh = split_hi(c.y, &yl);
                C[0] = make_float4(xh, xl, yh, yl);
            } else {
                rel[m - 1] = make_float2(__double2float_rn(c.x - v0.x), __double2float_rn(c.y - v0.y));
            }
            m++;
            prev = c;
        }
    }
    if (m == 0) C[0] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = (m > 0 ? m - 1 : 0); k < 2 * (S4 - 1); k++) rel[k] = make_float2(0.f, 0.f);
    if (plen) *plen = (uint8_t)len;
    *plen32 = (uint8_t)m;
}
