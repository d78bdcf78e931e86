// ct_extra.cu -- the two exported helpers that no query calls
// (liang_barsky_line_box_clip algorithms/liang_barsky.py:10-64,
// points_in_triangles geometry_utils.py:273-289), batched, and the step right
// after the intersection queries in regridding: a CSR weight matrix from the
// query-major (row, column, area) pairs of intersect_faces / intersect_boxes
// and its area-weighted mean (the dense weight-matrix aggregation of
// examples/spatial_indexing_2d_grids.py:245-313, done sparse).
#include <cmath>
#include <cstdint>

#include "ct_common.cuh"
#include "ct_internal.h"

extern "C" int ct_exclusive_scan(const int64_t* in, int64_t n, int64_t* out, void* ws, size_t ws_bytes,
                                 int64_t* total_host, void* stream);
extern "C" size_t ct_scan_workspace_size(int64_t n);

namespace cte {

// point_inside_box geometry_utils.py:528-529 (strict)
__device__ __forceinline__ bool inside_box(dpt a, double xmin, double xmax, double ymin, double ymax) {
    return xmin < a.x && a.x < xmax && ymin < a.y && a.y < ymax;
}

// liang_barsky_line_box_clip liang_barsky.py:10-64
__device__ bool liang_barsky(dpt a, dpt b, double xmin, double xmax, double ymin, double ymax, dpt* c, dpt* d) {
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    *c = mkp(nan, nan);
    *d = mkp(nan, nan);
    double dx = b.x - a.x, dy = b.y - a.y;
    if (dx == 0.0 && dy == 0.0) return false;
    if (inside_box(a, xmin, xmax, ymin, ymax) && inside_box(b, xmin, xmax, ymin, ymax)) {
        *c = a;
        *d = b;
        return true;
    }
    double t0 = 0.0, t1 = 1.0;
    const double P[4] = {-dx, dx, -dy, dy};
    const double Q[4] = {a.x - xmin, xmax - a.x, a.y - ymin, ymax - a.y};
    for (int k = 0; k < 4; k++) {
        double p = P[k], q = Q[k];
        if (p == 0) {
            if (q < 0) return false;
        } else {
            double t = q / p;
            if (p < 0) {
                if (t > t1) return false;
                if (t > t0) t0 = t;
            } else if (p > 0) {
                if (t < t0) return false;
                if (t < t1) t1 = t;
            }
        }
    }
    if (t0 == t1) return false;
    *c = mkp(a.x + t0 * dx, a.y + t0 * dy);
    *d = mkp(a.x + t1 * dx, a.y + t1 * dy);
    return true;
}

// point_in_triangle geometry_utils.py:241-270
__device__ bool point_in_triangle(dpt p, dpt a, dpt b, dpt c, double tol) {
    dpt ap = vsub(p, a), bp = vsub(p, b), cp = vsub(p, c);
    dpt ab = vsub(b, a), bc = vsub(c, b), ca = vsub(a, c);
    double A = crossp(ab, ap), B = crossp(bc, bp), C = crossp(ca, cp);
    bool sA = A > 0, sB = B > 0, sC = C > 0;
    if ((sA == sB) && (sB == sC)) return true;
    return (within_perp(A, ab, tol) && in_bounds(p, a, b)) || (within_perp(B, bc, tol) && in_bounds(p, b, c)) ||
           (within_perp(C, ca, tol) && in_bounds(p, c, a));
}

__global__ void k_liang_barsky(const double2* __restrict__ a, const double2* __restrict__ b,
                               const double4* __restrict__ box, int64_t n, uint8_t* __restrict__ ok,
                               double2* __restrict__ c, double2* __restrict__ d) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double4 bx = box[i];
        dpt cc, dd;
        bool r = liang_barsky(mkp(a[i].x, a[i].y), mkp(b[i].x, b[i].y), bx.x, bx.y, bx.z, bx.w, &cc, &dd);
        ok[i] = (uint8_t)r;
        c[i] = make_double2(cc.x, cc.y);
        d[i] = make_double2(dd.x, dd.y);
    }
}

__global__ void k_points_in_triangles(const double2* __restrict__ pts, const int64_t* __restrict__ fidx, int64_t n,
                                      const int64_t* __restrict__ faces, int K, const double* __restrict__ v,
                                      int64_t n_faces, double tol, uint8_t* __restrict__ out,
                                      unsigned int* __restrict__ bad) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t f = fidx[i];
        if (f < 0 || f >= n_faces) {  // upstream indexes without a check
            atomicOr(bad, 1u);
            out[i] = 0;
            continue;
        }
        const int64_t* t = faces + f * K;
        dpt A = mkp(v[2 * t[0]], v[2 * t[0] + 1]), B = mkp(v[2 * t[1]], v[2 * t[1] + 1]);
        dpt C = mkp(v[2 * t[2]], v[2 * t[2] + 1]);
        out[i] = (uint8_t)point_in_triangle(mkp(pts[i].x, pts[i].y), A, B, C, tol);
    }
}

// entries per row (rows = the first index of the pairs)
__global__ void k_row_counts(const int64_t* __restrict__ rows, int64_t n_pairs, int64_t n_rows,
                             unsigned long long* __restrict__ counts, unsigned int* __restrict__ bad) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n_pairs;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = rows[t];
        if (r < 0 || r >= n_rows) {
            atomicOr(bad, 1u);
            continue;
        }
        atomicAdd(&counts[r], 1ull);
    }
}

// rows must be non-decreasing (the pairs come query-major); checked
__global__ void k_rows_sorted(const int64_t* __restrict__ rows, int64_t n_pairs, unsigned int* __restrict__ bad) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x + 1; t < n_pairs;
         t += (int64_t)gridDim.x * blockDim.x)
        if (rows[t] < rows[t - 1]) atomicOr(bad, 2u);
}

// One warp per row: sum of weights and of weight * x over the row's entries
// in entry order (lane-strided partial sums, then a fixed-order tree), mean =
// sum(w x) / sum(w), NaN for rows without weight.
__global__ void k_csr_mean(const int64_t* __restrict__ row_ptr, const int64_t* __restrict__ cols,
                           const double* __restrict__ w, int64_t n_rows, int64_t n_cols,
                           const double* __restrict__ x, double* __restrict__ mean, double* __restrict__ wsum_out,
                           unsigned int* __restrict__ bad) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < n_rows; r += nw) {
        double sw = 0.0, swx = 0.0;
        for (int64_t k = row_ptr[r] + lane; k < row_ptr[r + 1]; k += 32) {
            int64_t c = cols[k];
            if (c < 0 || c >= n_cols) {
                atomicOr(bad, 1u);
                continue;
            }
            sw += w[k];
            swx += w[k] * x[c];
        }
        for (int o = 16; o > 0; o >>= 1) {
            sw += __shfl_down_sync(0xffffffffu, sw, o);
            swx += __shfl_down_sync(0xffffffffu, swx, o);
        }
        if (lane == 0) {
            const double nan = __longlong_as_double(0x7ff8000000000000ll);
            mean[r] = (sw > 0.0) ? swx / sw : nan;
            if (wsum_out) wsum_out[r] = sw;
        }
    }
}

static unsigned grid_for(int64_t n, int t) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + t - 1) / t, 152 * 16)); }

}  // namespace cte

using namespace cte;

extern "C" {

int ct_liang_barsky_line_box_clip(const double* a, const double* b, const double* boxes, int64_t n, uint8_t* ok,
                                  double* c, double* d, void* stream) {
    if (n < 0) return ct_fail(CT_ERR_ARG, "negative length");
    if (n == 0) return CT_OK;
    k_liang_barsky<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>((const double2*)a, (const double2*)b,
                                                                      (const double4*)boxes, n, ok, (double2*)c,
                                                                      (double2*)d);
    CT_CHECK_LAUNCH("liang_barsky");
    return CT_OK;
}

int ct_points_in_triangles(const double* points, const int64_t* face_indices, int64_t n, const int64_t* faces,
                           int32_t n_max_vert, int64_t n_faces, const double* vertices, double tolerance,
                           uint8_t* out, unsigned int* error_word, void* stream) {
    if (n < 0 || n_max_vert < 3) return ct_fail(CT_ERR_ARG, "bad sizes");
    if (n == 0) return CT_OK;
    k_points_in_triangles<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        (const double2*)points, face_indices, n, faces, n_max_vert, vertices, n_faces, tolerance, out, error_word);
    CT_CHECK_LAUNCH("points_in_triangles");
    return CT_OK;
}

size_t ct_csr_workspace_size(int64_t n_rows) {
    return ((size_t)8 * (size_t)(n_rows + 1) + 255) / 256 * 256 + ct_scan_workspace_size(n_rows + 1);
}

int ct_csr_row_ptr(const int64_t* rows, int64_t n_pairs, int64_t n_rows, int64_t* row_ptr, void* ws,
                   size_t ws_bytes, unsigned int* error_word, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n_pairs < 0 || n_rows < 0) return ct_fail(CT_ERR_ARG, "negative length");
    if (!ws || ws_bytes < ct_csr_workspace_size(n_rows)) return ct_fail(CT_ERR_WORKSPACE, "csr workspace too small");
    unsigned long long* counts = (unsigned long long*)ws;
    size_t head = ((size_t)8 * (size_t)(n_rows + 1) + 255) / 256 * 256;
    CT_CUDA(cudaMemsetAsync(counts, 0, 8 * (size_t)(n_rows + 1), st));
    if (n_pairs > 0) {
        k_rows_sorted<<<grid_for(n_pairs, 256), 256, 0, st>>>(rows, n_pairs, error_word);
        k_row_counts<<<grid_for(n_pairs, 256), 256, 0, st>>>(rows, n_pairs, n_rows, counts, error_word);
        CT_CHECK_LAUNCH("csr counts");
    }
    return ct_exclusive_scan((const int64_t*)counts, n_rows + 1, row_ptr, (char*)ws + head, ws_bytes - head, nullptr,
                             stream);
}

int ct_csr_weighted_mean(const int64_t* row_ptr, const int64_t* cols, const double* weights, int64_t n_rows,
                         int64_t n_cols, const double* x, double* mean, double* weight_sum, unsigned int* error_word,
                         void* stream) {
    if (n_rows < 0 || n_cols < 0) return ct_fail(CT_ERR_ARG, "negative length");
    if (n_rows == 0) return CT_OK;
    unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n_rows * 32 + 255) / 256, 152 * 32));
    k_csr_mean<<<blocks, 256, 0, (cudaStream_t)stream>>>(row_ptr, cols, weights, n_rows, n_cols, x, mean, weight_sum,
                                                         error_word);
    CT_CHECK_LAUNCH("csr weighted mean");
    return CT_OK;
}

}  // extern "C"
