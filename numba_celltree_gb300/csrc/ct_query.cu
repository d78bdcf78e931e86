// ct_query.cu -- geometry preparation, tree packing and point queries.
//
// Point location (locate_point query.py:63-107) has two forms:
//
//  CT_MODE_FP64  the plain form: float64 node tests and the float64
//                point_in_polygon_or_on_edge on leaf-ordered polygons.
//  CT_MODE_FP32  float32 node bounds (rounded outward, relative to the tree
//                centre) and float32 leaf tests, each carrying a rigorous
//                error band.  A decision outside its band provably equals the
//                float64 one; inside the band the node or polygon is re-decided
//                with the exact float64 code.  The traversal order, the visited
//                nodes and the returned cell are therefore identical to the
//                float64 form (and to upstream) -- only the arithmetic that
//                reaches them is cheaper.  GB300 executes float32 about 68x
//                faster than float64, which is what this form exploits.
#include <cfloat>
#include <cmath>
#include <mutex>

#include "ct_common.cuh"
#include "ct_internal.h"
#include "ct_locf.cuh"

namespace ctq {

// Device view of a packed tree, passed to kernels by value.
struct TreeDev {
    const float4* nf;       // Lmax_f, Rmin_f, a, b (a/b as int bits)
    const double2* nd;      // Lmax, Rmin
    const double2* poly;    // leaf-ordered float64 polygons, K per cell
    const float4* polyf;    // leaf-ordered float32 cells in their local frame (ct_locf.cuh)
    const uint8_t* plen;    // polygon length (nullptr: all K)
    const uint8_t* plen32;  // deduplicated length
    const int64_t* bbi;     // bb_indices
    unsigned int* err;
    int64_t n_nodes;
    double ox, oy;
    float dabs;             // float64 rounding scale of absolute coordinates
    int K;
    int S4;                 // float4 units per cell in polyf
};

__device__ __forceinline__ int node_a(const float4& q) { return __float_as_int(q.z); }
__device__ __forceinline__ int node_b(const float4& q) { return __float_as_int(q.w); }

// Error band of a float32 value obtained by (directed or nearest) rounding of
// a float64 difference: 2^-22 relative covers both roundings with margin.
__device__ __forceinline__ float band(float x) { return fabsf(x) * 2.384185791015625e-07f + 1e-30f; }

template <int STACK>
struct Stack {
    int s[STACK];
    int n;
};

// Float64 node step (locate_point query.py:87-105).
template <int STACK>
__device__ __forceinline__ bool push_fp64(Stack<STACK>& st, double pd, double Lmax, double Rmin, int child,
                                          unsigned int* err) {
    bool left = pd <= Lmax;
    bool right = pd >= Rmin;
    if (st.n + 2 > STACK) {
        set_error(err, CT_DEVERR_STACK);
        return false;
    }
    if (left && right) {
        if ((Lmax - pd) < (pd - Rmin)) {
            st.s[st.n++] = child;
            st.s[st.n++] = child + 1;
        } else {
            st.s[st.n++] = child + 1;
            st.s[st.n++] = child;
        }
    } else if (left) {
        st.s[st.n++] = child;
    } else if (right) {
        st.s[st.n++] = child + 1;
    }
    return true;
}

// Float32 node step with exactness bands; falls back to float64 per decision.
template <int STACK>
__device__ __forceinline__ bool push_fp32(Stack<STACK>& st, const TreeDev& T, int v, const float4& q, int dim,
                                          float x, float dx, double pd) {
    float Lf = q.x, Rf = q.y;
    float bL = band(Lf) + dx, bR = band(Rf) + dx;
    bool left, right;
    double2 nd;
    bool have = false;
    float dl = x - Lf;
    if (dl > bL) left = false;
    else if (-dl > bL) left = true;
    else {
        nd = T.nd[v];
        have = true;
        left = pd <= nd.x;
    }
    float dr = x - Rf;
    if (dr > bR) right = true;
    else if (-dr > bR) right = false;
    else {
        if (!have) {
            nd = T.nd[v];
            have = true;
        }
        right = pd >= nd.y;
    }
    int child = node_a(q);
    if (st.n + 2 > STACK) {
        set_error(T.err, CT_DEVERR_STACK);
        return false;
    }
    if (left && right) {
        float aF = Lf - x, bF = x - Rf;
        float bo = bL + bR + 2.384185791015625e-07f * (fabsf(aF) + fabsf(bF)) + 1e-30f;
        bool near_first;
        if (fabsf(aF - bF) > bo) near_first = aF < bF;
        else {
            if (!have) nd = T.nd[v];
            near_first = (nd.x - pd) < (pd - nd.y);
        }
        if (near_first) {
            st.s[st.n++] = child;
            st.s[st.n++] = child + 1;
        } else {
            st.s[st.n++] = child + 1;
            st.s[st.n++] = child;
        }
    } else if (left) {
        st.s[st.n++] = child;
    } else if (right) {
        st.s[st.n++] = child + 1;
    }
    return true;
}

template <int MODE, int STACK, int KT>
__global__ void __launch_bounds__(256) k_locate_points(TreeDev T, const double2* __restrict__ pts, int64_t n,
                                                       double tol, float tolf, int64_t* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 pp = pts[i];
    dpt p = mkp(pp.x, pp.y);
    float px = 0.f, py = 0.f, dpx = 0.f, dpy = 0.f;
    PtSplit P;
    if (MODE == CT_MODE_FP32) {
        px = __double2float_rn(p.x - T.ox);
        py = __double2float_rn(p.y - T.oy);
        dpx = band(px);
        dpy = band(py);
        P = split_point(p.x, p.y);
    }
    const int K = KT == 32 ? T.K : KT;
    Stack<STACK> st;
    st.n = 1;
    st.s[0] = 0;
    int64_t res = -1;
    int64_t budget = T.n_nodes;  // each node is visited at most once per query
    while (st.n > 0) {
        if (--budget < 0) {
            set_error(T.err, CT_DEVERR_LOOP);
            break;
        }
        int v = st.s[--st.n];
        float4 q = T.nf[v];
        int b = node_b(q);
        if (b >= 0) {  // leaf: cells bb_indices[ptr : ptr + size]
            int ptr = node_a(q);
            bool hit = false;
            for (int j = ptr; j < ptr + b; j++) {
                const dpt* poly = reinterpret_cast<const dpt*>(T.poly + (size_t)j * K);
                int len = (KT == 3) ? 3 : (T.plen ? (int)T.plen[j] : K);
                if (MODE == CT_MODE_FP32) {
                    int r = leaf_filter_local<KT>(P, T.dabs, tolf, T.polyf + (size_t)j * T.S4, (int)T.plen32[j]);
                    if (r == LF_INSIDE) hit = true;
                    else if (r == LF_UNSURE) hit = pip_or_edge(p, poly, len, tol);
                } else {
                    hit = pip_or_edge(p, poly, len, tol);
                }
                if (hit) {
                    res = T.bbi[j];
                    break;
                }
            }
            if (hit) break;
            continue;
        }
        int dim = -1 - b;
        double pd = dim ? p.y : p.x;
        bool ok;
        if (MODE == CT_MODE_FP32) {
            ok = push_fp32<STACK>(st, T, v, q, dim, dim ? py : px, dim ? dpy : dpx, pd);
        } else {
            double2 nd = T.nd[v];
            ok = push_fp64<STACK>(st, pd, nd.x, nd.y, node_a(q), T.err);
        }
        if (!ok) break;
    }
    out[i] = res;
}

// ------------------------------------------------------------------------
// Trees deeper than the stacks: the same depth-first traversal without a
// stack.  A node's children and their visiting order depend only on the
// query and the node, so the walk goes down to the first child it would have
// popped, and on the way back up (through node_parent) recomputes the order
// at the parent to find the sibling still to visit.  Every node is entered at
// most twice per query.
// ------------------------------------------------------------------------

// Children of internal node v in locate_point's visiting order (query.py:87-105):
// both: the one pushed last first; *second = -1 when there is only one.
__device__ __forceinline__ int order_fp64(const TreeDev& T, int v, const float4& q, double pd, int* second) {
    double2 nd = T.nd[v];
    bool left = pd <= nd.x, right = pd >= nd.y;
    int child = node_a(q);
    *second = -1;
    if (left && right) {
        if ((nd.x - pd) < (pd - nd.y)) {  // pushed left, then right
            *second = child;
            return child + 1;
        }
        *second = child + 1;
        return child;
    }
    if (left) return child;
    if (right) return child + 1;
    return -1;
}

template <int KT>
__global__ void __launch_bounds__(256) k_locate_points_deep(TreeDev T, const int* __restrict__ parent,
                                                            const double2* __restrict__ pts, int64_t n, double tol,
                                                            int64_t* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 pp = pts[i];
    dpt p = mkp(pp.x, pp.y);
    const int K = KT == 32 ? T.K : KT;
    int64_t res = -1;
    int v = 0, from = -1;
    bool down = true;
    int64_t budget = 2 * T.n_nodes + 2;
    while (v >= 0) {
        if (--budget < 0) {
            set_error(T.err, CT_DEVERR_LOOP);
            break;
        }
        float4 q = T.nf[v];
        int b = node_b(q);
        int next;
        if (b >= 0) {  // leaf
            if (down) {
                int ptr = node_a(q);
                for (int j = ptr; j < ptr + b && res < 0; j++) {
                    const dpt* poly = reinterpret_cast<const dpt*>(T.poly + (size_t)j * K);
                    int len = (KT == 3) ? 3 : (T.plen ? (int)T.plen[j] : K);
                    if (pip_or_edge(p, poly, len, tol)) res = T.bbi[j];
                }
                if (res >= 0) break;
            }
            next = -1;
        } else {
            int second;
            int first = order_fp64(T, v, q, (-1 - b) ? p.y : p.x, &second);
            next = down ? first : ((from == first) ? second : -1);
        }
        if (next >= 0) {
            from = v;
            v = next;
            down = true;
        } else {
            from = v;
            v = parent[v];
            down = false;
        }
    }
    out[i] = res;
}

__global__ void __launch_bounds__(256) k_locate_on_edge_deep(TreeDev T, const int* __restrict__ parent,
                                                             const double2* __restrict__ pts, int64_t n, double tol,
                                                             int64_t* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 pp = pts[i];
    dpt p = mkp(pp.x, pp.y);
    int64_t res = -1;
    int v = 0, from = -1;
    bool down = true;
    int64_t budget = 2 * T.n_nodes + 2;
    while (v >= 0) {
        if (--budget < 0) {
            set_error(T.err, CT_DEVERR_LOOP);
            break;
        }
        float4 q = T.nf[v];
        int b = node_b(q);
        int next;
        if (b >= 0) {
            if (down) {
                int ptr = node_a(q);
                for (int j = ptr; j < ptr + b && res < 0; j++) {
                    const double2* e = T.poly + (size_t)j * 2;
                    if (point_on_edge(p, mkp(e[0].x, e[0].y), mkp(e[1].x, e[1].y), tol)) res = T.bbi[j];
                }
                if (res >= 0) break;
            }
            next = -1;
        } else {
            int second;
            int first = order_fp64(T, v, q, (-1 - b) ? p.y : p.x, &second);
            next = down ? first : ((from == first) ? second : -1);
        }
        if (next >= 0) {
            from = v;
            v = next;
            down = true;
        } else {
            from = v;
            v = parent[v];
            down = false;
        }
    }
    out[i] = res;
}

// locate_point_on_edge query.py:121-164 (edge trees, K == 2).
template <int STACK>
__global__ void __launch_bounds__(256) k_locate_on_edge(TreeDev T, const double2* __restrict__ pts, int64_t n,
                                                        double tol, float tolf, int64_t* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 pp = pts[i];
    dpt p = mkp(pp.x, pp.y);
    float px = __double2float_rn(p.x - T.ox), py = __double2float_rn(p.y - T.oy);
    float dpx = band(px), dpy = band(py);
    PtSplit P = split_point(p.x, p.y);
    Stack<STACK> st;
    st.n = 1;
    st.s[0] = 0;
    int64_t res = -1;
    int64_t budget = T.n_nodes;
    while (st.n > 0) {
        if (--budget < 0) {
            set_error(T.err, CT_DEVERR_LOOP);
            break;
        }
        int v = st.s[--st.n];
        float4 q = T.nf[v];
        int b = node_b(q);
        if (b >= 0) {
            int ptr = node_a(q);
            bool hit = false;
            for (int j = ptr; j < ptr + b; j++) {
                if (T.plen32[j] == 2 && edge_surely_off_local(P, T.dabs, tolf, T.polyf + (size_t)j * T.S4)) continue;
                const double2* e = T.poly + (size_t)j * 2;
                if (point_on_edge(p, mkp(e[0].x, e[0].y), mkp(e[1].x, e[1].y), tol)) {
                    hit = true;
                    res = T.bbi[j];
                    break;
                }
            }
            if (hit) break;
            continue;
        }
        int dim = -1 - b;
        if (!push_fp32<STACK>(st, T, v, q, dim, dim ? py : px, dim ? dpy : dpx, dim ? p.y : p.x)) break;
    }
    out[i] = res;
}

// ------------------------------------------------------------------------
// geometry preparation
// ------------------------------------------------------------------------

// Index validation: the first `min_len` entries of every element and every
// entry before its first fill value must name a vertex.
__global__ void k_validate(const int64_t* __restrict__ e, int64_t n, int K, int min_len, int64_t nv,
                           unsigned int* __restrict__ bad) {
    int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n) return;
    const int64_t* x = e + f * K;
    for (int k = 0; k < K; k++) {
        int64_t idx = x[k];
        if (k >= min_len && idx == CT_FILL_VALUE) break;
        if (idx < 0 || idx >= nv) {
            atomicOr(bad, 1u);
            return;
        }
    }
}

// counter_clockwise geometry_utils.py:541-561 (flip 532-538)
__global__ void k_ccw(const double* __restrict__ v, int64_t* __restrict__ faces, int64_t n, int K) {
    int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n) return;
    int64_t* face = faces + f * K;
    int len = polygon_length(face, K);
    dpt a = mkp(v[2 * face[len - 2]], v[2 * face[len - 2] + 1]);
    dpt b = mkp(v[2 * face[len - 1]], v[2 * face[len - 1] + 1]);
    for (int i = 0; i < len; i++) {
        dpt c = mkp(v[2 * face[i]], v[2 * face[i] + 1]);
        double product = crossp(vsub(b, a), vsub(c, a));
        if (product == 0) {
            a = b;
            b = c;
        } else if (product < 0) {
            int end = len - 1;
            for (int k = 0; k < len / 2; k++) {
                int j = end - k;
                int64_t t = face[k];
                face[k] = face[j];
                face[j] = t;
            }
        } else {
            break;
        }
    }
}

// bounding_box / build_face_bboxes geometry_utils.py:421-456
__global__ void k_face_bboxes(const double* __restrict__ v, const int64_t* __restrict__ faces, int64_t n, int K,
                              double* __restrict__ bb) {
    int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n) return;
    const int64_t* face = faces + f * K;
    double xmin = v[2 * face[0]], xmax = xmin, ymin = v[2 * face[0] + 1], ymax = ymin;
    for (int i = 1; i < K; i++) {
        int64_t idx = face[i];
        if (idx == CT_FILL_VALUE) break;
        double x = v[2 * idx], y = v[2 * idx + 1];
        xmin = pmin(xmin, x);
        xmax = pmax(xmax, x);
        ymin = pmin(ymin, y);
        ymax = pmax(ymax, y);
    }
    double4 o;
    o.x = xmin;
    o.y = xmax;
    o.z = ymin;
    o.w = ymax;
    reinterpret_cast<double4*>(bb)[f] = o;
}

// edge_bounding_box / build_edge_bboxes geometry_utils.py:459-487
__global__ void k_edge_bboxes(const double* __restrict__ v, const int64_t* __restrict__ edges, int64_t n, double tol,
                              double* __restrict__ bb) {
    int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n) return;
    int64_t a = edges[2 * f], b = edges[2 * f + 1];
    double x0 = v[2 * a], y0 = v[2 * a + 1], x1 = v[2 * b], y1 = v[2 * b + 1];
    double4 o;
    o.x = pmin(x0 - tol, x1 - tol);
    o.y = pmax(x0 + tol, x1 + tol);
    o.z = pmin(y0 - tol, y1 - tol);
    o.w = pmax(y0 + tol, y1 + tol);
    reinterpret_cast<double4*>(bb)[f] = o;
}

// bbox_tree / bbox_distances celltree_base.py:20-48 (reduction by keys)
__global__ void k_bbox_summary(const double* __restrict__ bb, int64_t n, double* __restrict__ dist,
                               unsigned long long* __restrict__ red) {
    unsigned long long k[5] = {~0ull, ~0ull, ~0ull, ~0ull, ~0ull};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double4 b = reinterpret_cast<const double4*>(bb)[i];
        double dx = b.y - b.x, dy = b.w - b.z;
        double dxy = box_diagonal(dx, dy);
        if (dist) {
            dist[3 * i] = dx;
            dist[3 * i + 1] = dy;
            dist[3 * i + 2] = dxy;
        }
        k[0] = min(k[0], fkey(b.x));
        k[1] = min(k[1], ~fkey(b.y));
        k[2] = min(k[2], fkey(b.z));
        k[3] = min(k[3], ~fkey(b.w));
        k[4] = min(k[4], ~fkey(dxy));
    }
    for (int j = 0; j < 5; j++) {
        unsigned long long m = k[j];
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
            m = min(m, t);
        }
        if ((threadIdx.x & 31) == 0) atomicMin(&red[j], m);
    }
}

__global__ void k_vertex_extent(const double* __restrict__ v, int64_t n, unsigned long long* __restrict__ red) {
    unsigned long long k[4] = {~0ull, ~0ull, ~0ull, ~0ull};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double x = v[2 * i], y = v[2 * i + 1];
        k[0] = min(k[0], fkey(x));
        k[1] = min(k[1], ~fkey(x));
        k[2] = min(k[2], fkey(y));
        k[3] = min(k[3], ~fkey(y));
    }
    for (int j = 0; j < 4; j++) {
        unsigned long long m = k[j];
        for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) atomicMin(&red[j], m);
    }
}

// ------------------------------------------------------------------------
// packing
// ------------------------------------------------------------------------

__global__ void k_check_finite(const double* __restrict__ x, int64_t n, unsigned int* __restrict__ flag) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (!isfinite(x[i])) atomicOr(flag, 2u);
}

__global__ void k_pack_nodes(int64_t n_nodes, const int64_t* __restrict__ child, const double* __restrict__ Lmax,
                             const double* __restrict__ Rmin, const int64_t* __restrict__ ptr,
                             const int64_t* __restrict__ size, const uint8_t* __restrict__ dim, double ox, double oy,
                             int64_t n_elem, float4* __restrict__ nf, double2* __restrict__ nd,
                             int* __restrict__ parent, unsigned int* __restrict__ bad) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_nodes) return;
    // structure check: children after their parent and in range, leaf ranges
    // inside bb_indices -- guarantees every traversal terminates in bounds
    int64_t c = child[v];
    if (c != -1 && (c <= v || c + 1 >= n_nodes)) atomicOr(bad, 1u);
    if (parent && c > v && c + 1 < n_nodes) {
        parent[c] = (int)v;
        parent[c + 1] = (int)v;
    }
    if (c == -1 && (ptr[v] < 0 || size[v] < 0 || ptr[v] + size[v] > n_elem)) atomicOr(bad, 1u);
    double L = Lmax[v], R = Rmin[v];
    if (!isfinite(L) || !isfinite(R)) atomicOr(bad, 2u);  // not an error: queries keep the literal float64 path
    nd[v] = make_double2(L, R);
    float4 q;
    if (child[v] == -1) {
        q.x = 0.f;
        q.y = 0.f;
        q.z = __int_as_float((int)ptr[v]);
        q.w = __int_as_float((int)size[v]);
    } else {
        int d = dim[v] ? 1 : 0;
        double o = d ? oy : ox;
        // rounded outward: the float32 interval [Rmin_f, Lmax_f] contains the float64 one
        q.x = __double2float_ru(L - o);
        q.y = __double2float_rd(R - o);
        q.z = __int_as_float((int)child[v]);
        q.w = __int_as_float(-1 - d);
    }
    nf[v] = q;
}

// Leaf-ordered polygons: the float64 copy as given, and the float32 cell in
// its local frame (ct_locf.cuh) with repeated consecutive vertices removed
// (the float64 predicate skips them: `if v1 == v0: continue`,
// geometry_utils.py:203-204).
__global__ void k_pack_polys(int64_t n, int K, bool is_edge, const int64_t* __restrict__ elems,
                             const int64_t* __restrict__ bbi, const double* __restrict__ v,
                             double2* __restrict__ poly, float4* __restrict__ polyf, uint8_t* __restrict__ plen,
                             uint8_t* __restrict__ plen32) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    pack_cell(elems + bbi[j] * K, K, is_edge, v, poly + j * K, polyf + j * poly32_stride(K), plen ? plen + j : nullptr,
              plen32 + j);
}

TreeDev make_dev(const ct_tree* t) {
    TreeDev T;
    T.nf = (const float4*)t->nodes_f32;
    T.nd = (const double2*)t->nodes_f64;
    T.poly = (const double2*)t->poly_f64;
    T.polyf = (const float4*)t->poly_f32;
    T.plen = t->n_max_vert == 3 ? nullptr : t->poly_len;
    T.plen32 = t->poly_len32;
    T.bbi = t->bb_indices;
    T.err = t->error_word;
    T.n_nodes = t->n_nodes;
    T.ox = t->origin[0];
    T.oy = t->origin[1];
    T.dabs = t->abs_eps;
    T.K = t->n_max_vert;
    T.S4 = poly32_stride(t->n_max_vert);
    return T;
}

static inline int grid_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }

}  // namespace ctq

using namespace ctq;

// Reduction scratch for the summaries and checks lives in a small static
// device array shared by ct_validate_elements, ct_bbox_summary,
// ct_vertex_extent and ct_pack_tree.  Each of them holds g_red_mutex from
// the reset of the array to the read-back of its result (all four
// synchronise their stream before returning), so calls from several host
// threads or on several streams run one after another instead of clearing
// or overwriting each other's counters.
static __device__ unsigned long long g_red[8];
static std::mutex g_red_mutex;

extern "C" {

int ct_validate_elements(const int64_t* elements, int64_t n, int32_t K, int32_t min_len, int64_t n_vertices,
                         int32_t* bad_host, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    unsigned int* red = nullptr;
    std::lock_guard<std::mutex> red_lock(g_red_mutex);
    CT_CUDA(cudaGetSymbolAddress((void**)&red, g_red));
    CT_CUDA(cudaMemsetAsync(red, 0, sizeof(unsigned int), st));
    if (n > 0) {
        k_validate<<<grid_for(n, 256), 256, 0, st>>>(elements, n, K, min_len, n_vertices, red);
        CT_CHECK_LAUNCH("validate");
    }
    unsigned int h = 0;
    CT_CUDA(cudaMemcpyAsync(&h, red, sizeof(h), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    *bad_host = (int32_t)h;
    return CT_OK;
}

int ct_counter_clockwise(const double* vertices, int64_t* faces, int64_t n, int32_t K, void* stream) {
    if (n == 0) return CT_OK;
    if (K < 3 || K > CT_MAX_N_VERTEX) return ct_fail(CT_ERR_ARG, "n_max_vert must be in [3, 32]");
    k_ccw<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(vertices, faces, n, K);
    CT_CHECK_LAUNCH("ccw");
    return CT_OK;
}

int ct_face_bboxes(const double* vertices, const int64_t* faces, int64_t n, int32_t K, double* bb, void* stream) {
    if (n == 0) return CT_OK;
    if (K < 1 || K > CT_MAX_N_VERTEX) return ct_fail(CT_ERR_ARG, "n_max_vert must be in [1, 32]");
    k_face_bboxes<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(vertices, faces, n, K, bb);
    CT_CHECK_LAUNCH("face_bboxes");
    return CT_OK;
}

int ct_edge_bboxes(const double* vertices, const int64_t* edges, int64_t n, double tol, double* bb, void* stream) {
    if (n == 0) return CT_OK;
    k_edge_bboxes<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(vertices, edges, n, tol, bb);
    CT_CHECK_LAUNCH("edge_bboxes");
    return CT_OK;
}


int ct_bbox_summary(const double* bb, int64_t n, double* dist, double* out5, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long* red = nullptr;
    std::lock_guard<std::mutex> red_lock(g_red_mutex);
    CT_CUDA(cudaGetSymbolAddress((void**)&red, g_red));
    unsigned long long init[5] = {~0ull, ~0ull, ~0ull, ~0ull, ~0ull};
    CT_CUDA(cudaMemcpyAsync(red, init, sizeof(init), cudaMemcpyHostToDevice, st));
    if (n > 0) {
        int g = (int)std::min<int64_t>(grid_for(n, 256), 152 * 8);
        k_bbox_summary<<<g, 256, 0, st>>>(bb, n, dist, red);
        CT_CHECK_LAUNCH("bbox_summary");
    }
    unsigned long long h[5];
    CT_CUDA(cudaMemcpyAsync(h, red, sizeof(h), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    auto inv = [](unsigned long long k) {
        unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
        double d;
        memcpy(&d, &b, 8);
        return d;
    };
    out5[0] = inv(h[0]);
    out5[1] = inv(~h[1]);
    out5[2] = inv(h[2]);
    out5[3] = inv(~h[3]);
    out5[4] = inv(~h[4]);
    return CT_OK;
}

int ct_vertex_extent(const double* v, int64_t n, double* out4, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long* red = nullptr;
    std::lock_guard<std::mutex> red_lock(g_red_mutex);
    CT_CUDA(cudaGetSymbolAddress((void**)&red, g_red));
    unsigned long long init[4] = {~0ull, ~0ull, ~0ull, ~0ull};
    CT_CUDA(cudaMemcpyAsync(red, init, sizeof(init), cudaMemcpyHostToDevice, st));
    if (n > 0) {
        int g = (int)std::min<int64_t>(grid_for(n, 256), 152 * 8);
        k_vertex_extent<<<g, 256, 0, st>>>(v, n, red);
        CT_CHECK_LAUNCH("vertex_extent");
    }
    unsigned long long h[4];
    CT_CUDA(cudaMemcpyAsync(h, red, sizeof(h), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    auto inv = [](unsigned long long k) {
        unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
        double d;
        memcpy(&d, &b, 8);
        return d;
    };
    out4[0] = inv(h[0]);
    out4[1] = inv(~h[1]);
    out4[2] = inv(h[2]);
    out4[3] = inv(~h[3]);
    return CT_OK;
}

int ct_pack_tree(ct_tree* t, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!t) return ct_fail(CT_ERR_ARG, "tree is null");
    if (t->n_max_vert < 2 || t->n_max_vert > CT_MAX_N_VERTEX) return ct_fail(CT_ERR_ARG, "n_max_vert out of range");
    double ox = 0.5 * (t->bbox[0] + t->bbox[1]);
    double oy = 0.5 * (t->bbox[2] + t->bbox[3]);
    if (!std::isfinite(ox) || !std::isfinite(oy)) {
        ox = 0.0;
        oy = 0.0;
    }
    bool is_edge = t->n_max_vert == 2;
    unsigned int* red = nullptr;
    std::lock_guard<std::mutex> red_lock(g_red_mutex);
    CT_CUDA(cudaGetSymbolAddress((void**)&red, g_red));
    CT_CUDA(cudaMemsetAsync(red, 0, 2 * sizeof(unsigned int), st));
    t->origin[0] = ox;
    t->origin[1] = oy;
    if (t->n_nodes > 0) {
        if (t->node_parent) CT_CUDA(cudaMemsetAsync(t->node_parent, 0xff, (size_t)t->n_nodes * sizeof(int), st));
        k_pack_nodes<<<grid_for(t->n_nodes, 256), 256, 0, st>>>(
            t->n_nodes, t->node_child, t->node_Lmax, t->node_Rmin, t->node_ptr, t->node_size, t->node_dim, ox, oy,
            t->n_elements, (float4*)t->nodes_f32, (double2*)t->nodes_f64, t->node_parent, red + 1);
        CT_CHECK_LAUNCH("pack_nodes");
    }
    if (t->n_elements > 0) {
        k_pack_polys<<<grid_for(t->n_elements, 256), 256, 0, st>>>(
            t->n_elements, t->n_max_vert, is_edge, t->elements, t->bb_indices, t->vertices, (double2*)t->poly_f64,
            (float4*)t->poly_f32, t->poly_len, t->poly_len32);
        CT_CHECK_LAUNCH("pack_polys");
    }
    if (t->n_elements > 0 && t->bb_coords)
        k_check_finite<<<(unsigned)std::min<int64_t>(grid_for(4 * t->n_elements, 256), 152 * 8), 256, 0, st>>>(
            t->bb_coords, 4 * t->n_elements, red + 1);
    unsigned int hv[2] = {0, 0};
    CT_CUDA(cudaMemcpyAsync(hv, red, sizeof(hv), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    if (hv[1] & 1u) return ct_fail(CT_ERR_DEVICE, "tree structure check failed (child or leaf range out of order)");
    t->bounds_finite = (hv[1] & 2u) ? 0 : 1;
    t->vmax = 0.0f;  // unused by the local-frame float32 cells
    // float64 rounding of absolute vertex coordinates (the float64 predicate
    // rounds relative to them): 2^-50 * max |coordinate|
    double amax = std::max(std::max(std::fabs(t->bbox[0]), std::fabs(t->bbox[1])),
                           std::max(std::fabs(t->bbox[2]), std::fabs(t->bbox[3])));
    if (!std::isfinite(amax)) amax = 0.0;
    t->abs_eps = (float)(amax * 8.881784197001252e-16) + 1e-30f;
    return CT_OK;
}

// traversal stack of the float64 / in-line float32 forms: the tree's launch
// shape when it fits the tree, else the smallest stack that does
static int stack_for(const ct_tree* t) {
    int need = t->max_depth + 2;
    if (need > 512) return -1;
    if (t->tune_fp64_stack == 512) return 512;
    return need <= 64 ? 64 : 512;
}

int ct_locate_points(const ct_tree* t, const double* points, int64_t n, double tol, int32_t mode, int64_t* out,
                     void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!t) return ct_fail(CT_ERR_ARG, "tree is null");
    if (n == 0) return CT_OK;
    if (t->n_nodes <= 0) return ct_fail(CT_ERR_ARG, "tree has no nodes");
    int S = stack_for(t);
    if (S < 0 && !t->node_parent) return ct_fail(CT_ERR_ARG, "tree deeper than 510 levels (no node_parent)");
    TreeDev T = make_dev(t);
    if (S < 0) {  // deeper than the stacks: the stackless float64 traversal (same results)
        const double2* P = (const double2*)points;
        int g = grid_for(n, 256);
        if (t->n_max_vert == 3) k_locate_points_deep<3><<<g, 256, 0, st>>>(T, t->node_parent, P, n, tol, out);
        else if (t->n_max_vert == 4) k_locate_points_deep<4><<<g, 256, 0, st>>>(T, t->node_parent, P, n, tol, out);
        else k_locate_points_deep<32><<<g, 256, 0, st>>>(T, t->node_parent, P, n, tol, out);
        CT_CHECK_LAUNCH("locate_points (deep tree)");
        return CT_OK;
    }
    float tolf = __builtin_nanf("");
    {
        // float32 tolerance rounded up (conservative for the filter)
        float f = (float)tol;
        if ((double)f < tol) f = nextafterf(f, INFINITY);
        tolf = f;
    }
    const double2* P = (const double2*)points;
    int g = grid_for(n, 256);
    int K = t->n_max_vert;
#define CT_LAUNCH_LOCATE(MODE, STK)                                                        \
    do {                                                                                   \
        if (K == 3) k_locate_points<MODE, STK, 3><<<g, 256, 0, st>>>(T, P, n, tol, tolf, out); \
        else if (K == 4) k_locate_points<MODE, STK, 4><<<g, 256, 0, st>>>(T, P, n, tol, tolf, out); \
        else k_locate_points<MODE, STK, 32><<<g, 256, 0, st>>>(T, P, n, tol, tolf, out);     \
    } while (0)
    if (mode == CT_MODE_FP32) {
        if (S == 64) CT_LAUNCH_LOCATE(CT_MODE_FP32, 64);
        else CT_LAUNCH_LOCATE(CT_MODE_FP32, 512);
    } else {
        if (S == 64) CT_LAUNCH_LOCATE(CT_MODE_FP64, 64);
        else CT_LAUNCH_LOCATE(CT_MODE_FP64, 512);
    }
#undef CT_LAUNCH_LOCATE
    CT_CHECK_LAUNCH("locate_points");
    return CT_OK;
}

int ct_locate_points_on_edge(const ct_tree* t, const double* points, int64_t n, double tol, int64_t* out,
                             void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!t) return ct_fail(CT_ERR_ARG, "tree is null");
    if (n == 0) return CT_OK;
    if (t->n_max_vert != 2) return ct_fail(CT_ERR_ARG, "not an edge tree");
    int S = stack_for(t);
    if (S < 0 && !t->node_parent) return ct_fail(CT_ERR_ARG, "tree deeper than 510 levels (no node_parent)");
    TreeDev T = make_dev(t);
    if (S < 0) {
        k_locate_on_edge_deep<<<grid_for(n, 256), 256, 0, st>>>(T, t->node_parent, (const double2*)points, n, tol,
                                                                 out);
        CT_CHECK_LAUNCH("locate_points_on_edge (deep tree)");
        return CT_OK;
    }
    float f = (float)tol;
    if ((double)f < tol) f = nextafterf(f, INFINITY);
    int g = grid_for(n, 256);
    if (S == 64) k_locate_on_edge<64><<<g, 256, 0, st>>>(T, (const double2*)points, n, tol, f, out);
    else k_locate_on_edge<512><<<g, 256, 0, st>>>(T, (const double2*)points, n, tol, f, out);
    CT_CHECK_LAUNCH("locate_points_on_edge");
    return CT_OK;
}

}  // extern "C"
