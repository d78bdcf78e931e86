// ct_multi.cu -- multi-result queries, per-pair kernels, barycentric weights
// and node-bound diagnostics.
//
// Multi-result queries (locate_boxes query.py:177-289, _locate_edges
// query.py:357-533) are rebuilt as count -> exclusive scan -> write: the
// count and write kernels run the same traversal, so the write pass knows
// each query's output offset.  Results come out query-major and, within a
// query, in traversal order -- exactly upstream's concatenated order.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "ct_common.cuh"
#include "ct_geom.cuh"
#include "ct_internal.h"
#include "ct_locf.cuh"

extern "C" size_t ct_radix_pass_workspace_size(void);
extern "C" int ct_radix_pass(const unsigned* kin, const int* iin, int64_t n, int32_t shift, unsigned* kout, int* iout,
                             void* ws, size_t ws_bytes, void* stream);

namespace ctm {

struct TreeQ {
    const float4* nf;    // packed node meta: z = child / ptr, w = -1 - dim / size
    const double2* nd;   // Lmax, Rmin
    const double2* poly; // leaf-ordered polygons (K per cell)
    const uint8_t* plen;
    const int64_t* bbi;
    const double* bb;    // bb_coords (cell order)
    unsigned int* err;
    int64_t n_nodes;
    dbox bbox;
    int K;
    bool finite;  // all node bounds and cell boxes finite: order comparisons on integer keys
    // box index (ct_pack_box_index; null when not built)
    const double4* bbl;        // cell boxes in leaf order
    const struct NodeBox* nbx; // per node: bounding box of its cells (float32 frame, outward) and leaf range
    const int* lstart;         // per leaf position: first position of its leaf
    double ox, oy;             // float32 frame origin
    const int* parent;         // node parents (trees deeper than the stacks are walked through them)
    // float32 leaf data (ct_locf.cuh) for the filters of the segment test
    const float4* polyf;
    const uint8_t* plen32;
    int S4;
    float dabs;                // float64 rounding of absolute coordinates
    // line filter of the segment traversal (null bbl32: off)
    const float4* bbl32;       // cell boxes in leaf order, float32 frame, rounded outward
    float fX, fY;              // largest |x - ox|, |y - oy| over the tree's bbox
    double babs;               // largest |coordinate| of the tree's bbox
    double mext;               // 2^-37 x the tree's largest extent + 2^-47
};

// Bounding box of a node's cells in the float32 frame of the tree (x - ox,
// y - oy rounded outward) and the node's range of leaf positions.  32 bytes.
struct NodeBox {
    float xmin, xmax, ymin, ymax;
    int ptr, size, pad0, pad1;
};

// x < y for finite (or infinite, non-NaN) doubles as one 64-bit integer
// comparison of order-preserving keys (-0.0 and +0.0 share a key, as they
// compare equal): the comparisons of the box and segment traversals run on
// the integer pipes instead of GB300's narrow float64 pipe.
__device__ __forceinline__ bool not_nan(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull) <= 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool is_fin(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull) < 0x7ff0000000000000ull;
}

__device__ __forceinline__ int na(const float4& q) { return __float_as_int(q.z); }
__device__ __forceinline__ int nb(const float4& q) { return __float_as_int(q.w); }

constexpr int STK = 128;  // traversal stack (tree depth + 2 must fit; checked on the host)

// bb_coords of the cell at leaf position j: from the leaf-ordered copy of the
// box index when it is built, else through bb_indices
__device__ __forceinline__ dbox leaf_box(const TreeQ& T, int64_t j) {
    if (T.bbl) {
        double4 c4 = T.bbl[j];
        dbox b;
        b.xmin = c4.x;
        b.xmax = c4.y;
        b.ymin = c4.z;
        b.ymax = c4.w;
        return b;
    }
    return load_box(T.bb + 4 * T.bbi[j]);
}

// ---------------------------------------------------------------------------
// locate_box query.py:177-244
// ---------------------------------------------------------------------------
// A subtree wholly inside a query box whose cells the writing pass leaves to
// k_box_jobs: its output offset, the query box and its leaf range.
struct BoxJob {
    int64_t out, box;
    int ptr, size, pad0, pad1;
};
constexpr int BOX_JOB_MIN = 8;  // default: smaller subtrees are written in line

template <bool WRITE, bool DEEP>
__global__ void __launch_bounds__(256) k_boxes(TreeQ T, const double4* __restrict__ boxes, int64_t n,
                                               const int* __restrict__ order, int64_t* __restrict__ cnt_or_off,
                                               int64_t* __restrict__ ii, int64_t* __restrict__ jj,
                                               BoxJob* __restrict__ jobs = nullptr,
                                               unsigned long long* __restrict__ njobs = nullptr, int64_t job_cap = 0,
                                               int job_min = BOX_JOB_MIN, int* __restrict__ spec = nullptr,
                                               int spec_cap = 0, const int64_t* __restrict__ spec_cnt = nullptr) {
    int64_t tq = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tq >= n) return;
    // queries in work order (similar work in one warp); results by query index
    int64_t i = order ? (int64_t)order[tq] : tq;
    // writing pass after a speculative count: boxes whose pairs all fit the
    // per-box scratch were written from it (k_boxes_spec_emit)
    if (WRITE && spec_cnt && spec_cnt[i] <= spec_cap) return;
    int* sp_out = (!WRITE && spec) ? spec + i * (int64_t)spec_cap : nullptr;
    double4 q4 = boxes[i];
    dbox box;
    box.xmin = q4.x;
    box.xmax = q4.y;
    box.ymin = q4.z;
    box.ymax = q4.w;
    int64_t count = 0;
    int64_t base = WRITE ? cnt_or_off[i] : 0;
    // key path: every value non-NaN, so the order comparisons equal the
    // float64 ones (NaN boxes keep the float64 comparisons)
    const bool keys = T.finite && not_nan(box.xmin) && not_nan(box.xmax) && not_nan(box.ymin) && not_nan(box.ymax);
    const unsigned long long kx0 = fkey(box.xmin), kx1 = fkey(box.xmax), ky0 = fkey(box.ymin), ky1 = fkey(box.ymax);
    // box index: a node whose cells' bounding box lies strictly inside the
    // query box has every cell overlapping it (boxes_intersect is strict and
    // cell.xmax >= node.xmin > box.xmin, ...); the traversal would visit all
    // of it.  The query box in the float32 frame is rounded inward, the node
    // boxes outward, so a float32 "strictly inside" implies the float64 one.
    // A node whose cells' bounding box lies strictly beyond a side of the
    // query box has no overlapping cell (boxes_intersect needs
    // box.xmin < cell.xmax <= node.xmax, ...): its subtree is skipped.  The
    // query box rounded outward, the node boxes outward: since x -> fl(x - o)
    // is monotonic, node.xmax_f32 < float_rd(fl(box.xmin - o)) implies
    // node.xmax < box.xmin.  Skipped subtrees hold no result, so the output
    // and its order are unchanged.
    const bool idx = keys && T.nbx != nullptr;
    float qx0 = 0.0f, qx1 = 0.0f, qy0 = 0.0f, qy1 = 0.0f;
    float ox0 = 0.0f, ox1 = 0.0f, oy0 = 0.0f, oy1 = 0.0f;
    if (idx) {
        qx0 = __double2float_ru(box.xmin - T.ox);
        qx1 = __double2float_rd(box.xmax - T.ox);
        qy0 = __double2float_ru(box.ymin - T.oy);
        qy1 = __double2float_rd(box.ymax - T.oy);
        ox0 = __double2float_rd(box.xmin - T.ox);
        ox1 = __double2float_ru(box.xmax - T.ox);
        oy0 = __double2float_rd(box.ymin - T.oy);
        oy1 = __double2float_ru(box.ymax - T.oy);
    }
    if (boxes_intersect(box, T.bbox)) {
        // depth-first walk: a stack, or (DEEP, trees deeper than the stack)
        // the parent links -- down to the child that would be popped first,
        // back up to the parent to find the sibling still to visit
        int st[DEEP ? 1 : STK];
        int sp = 1;
        st[0] = 0;
        int dv = 0, from = -1;
        bool down = true;
        int64_t budget = DEEP ? 2 * T.n_nodes + 2 : T.n_nodes;
        while (DEEP ? dv >= 0 : sp > 0) {
            if (--budget < 0) {
                set_error(T.err, CT_DEVERR_LOOP);
                break;
            }
            const int v = DEEP ? dv : st[--sp];
            bool terminal = false;
            // the node's three records loaded together (one memory round trip
            // per visited node instead of a chain of three)
            const float4 q = T.nf[v];
            const double2 nd_v = T.nd[v];
            NodeBox nbv;
            if (idx && (!DEEP || down)) nbv = T.nbx[v];
            if (!DEEP || down) {
                if (idx) {
                    if (nbv.xmax < ox0 || nbv.xmin > ox1 || nbv.ymax < oy0 || nbv.ymin > oy1) {
                        terminal = true;  // no cell below overlaps the box
                    } else if (qx0 < nbv.xmin && nbv.xmax < qx1 && qy0 < nbv.ymin && nbv.ymax < qy1) {
                        // the whole subtree, in upstream's visiting order: right
                        // child first, i.e. leaves by decreasing position, each
                        // leaf's cells by increasing position
                        int64_t jk = -1;
                        if (WRITE && jobs && nbv.size >= job_min) {
                            jk = (int64_t)atomicAdd(njobs, 1ull);
                            if (jk < job_cap) {
                                BoxJob J;
                                J.out = base + count;
                                J.box = i;
                                J.ptr = nbv.ptr;
                                J.size = nbv.size;
                                J.pad0 = J.pad1 = 0;
                                jobs[jk] = J;
                            } else {
                                jk = -1;  // no room (cannot happen with the sized buffer): write in line
                            }
                        }
                        if ((WRITE && jk < 0) || (sp_out && count < spec_cap)) {
                            int qq = nbv.ptr + nbv.size;
                            int64_t c = count;
                            while (qq > nbv.ptr && (WRITE || c < spec_cap)) {
                                int s = T.lstart[qq - 1];
                                if (s < nbv.ptr || s >= qq) {  // corrupt index: stop rather than loop
                                    set_error(T.err, CT_DEVERR_LOOP);
                                    break;
                                }
                                for (int j = s; j < qq; j++) {
                                    if (WRITE) {
                                        ii[base + c] = i;
                                        jj[base + c] = T.bbi[j];
                                    } else if (c < spec_cap) {
                                        sp_out[c] = (int)T.bbi[j];
                                    }
                                    c++;
                                }
                                qq = s;
                            }
                        }
                        count += nbv.size;
                        terminal = true;
                    }
                }
                if (!terminal) {
                    int b = nb(q);
                    if (b >= 0) {
                        int ptr = na(q);
                        for (int j = ptr; j < ptr + b; j++) {
                            dbox lb = leaf_box(T, j);
                            // boxes_intersect geometry_utils.py:292-300
                            bool hit = keys ? (kx0 < fkey(lb.xmax) && fkey(lb.xmin) < kx1 && ky0 < fkey(lb.ymax) &&
                                               fkey(lb.ymin) < ky1)
                                            : boxes_intersect(box, lb);
                            if (hit) {
                                if (WRITE) {
                                    ii[base + count] = i;
                                    jj[base + count] = T.bbi[j];
                                } else if (sp_out && count < spec_cap) {
                                    sp_out[count] = (int)T.bbi[j];
                                }
                                count++;
                            }
                        }
                        terminal = true;
                    }
                }
            }
            int first = -1, second = -1;
            if (!terminal) {
                int dim = -1 - nb(q);
                const double2 d = nd_v;
                bool left, right;
                if (keys) {
                    left = (dim ? ky0 : kx0) <= fkey(d.x);
                    right = (dim ? ky1 : kx1) >= fkey(d.y);
                } else {
                    double bmin = dim ? box.ymin : box.xmin, bmax = dim ? box.ymax : box.xmax;
                    left = bmin <= d.x;
                    right = bmax >= d.y;
                }
                // pushed left, then right: the right child is visited first
                int child = na(q);
                first = right ? child + 1 : (left ? child : -1);
                second = (left && right) ? child : -1;
            }
            if (DEEP) {
                int next = terminal ? -1 : (down ? first : ((from == first) ? second : -1));
                from = dv;
                if (next >= 0) {
                    dv = next;
                    down = true;
                } else {
                    dv = T.parent[dv];
                    down = false;
                }
            } else if (!terminal) {
                if (sp + 2 > STK) {
                    set_error(T.err, CT_DEVERR_STACK);
                    break;
                }
                if (second >= 0) st[sp++] = second;
                if (first >= 0) st[sp++] = first;
            }
        }
    }
    if (!WRITE) cnt_or_off[i] = count;
}

// The cells of each deferred subtree, one warp per subtree, in upstream's
// visiting order (leaves by decreasing position, each leaf's cells by
// increasing position): output o takes reversed position q = end - 1 - o,
// whose leaf [s, e) contributes position s + (e - 1 - q).  Writes and the
// bb_indices reads are coalesced across the warp.
__global__ void __launch_bounds__(256) k_box_jobs(const BoxJob* __restrict__ jobs,
                                                  const unsigned long long* __restrict__ njobs,
                                                  int64_t job_cap, const int* __restrict__ lstart,
                                                  const int64_t* __restrict__ bbi, int64_t* __restrict__ ii,
                                                  int64_t* __restrict__ jj, unsigned int* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t nj = (int64_t)min(*njobs, (unsigned long long)job_cap);
    for (int64_t k = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < nj; k += warps) {
        const BoxJob J = jobs[k];
        const int end = J.ptr + J.size;
        bool bad = false;
        for (int o = lane; o < J.size; o += 32) {
            const int q = end - 1 - o;
            const int s0 = lstart[q];
            int e = q + 1;
            while (e < end && lstart[e] == s0) e++;
            const int p = s0 + (e - 1 - q);
            if (s0 < J.ptr || s0 > q) {  // corrupt index: leave the slot, report
                bad = true;
                continue;
            }
            ii[J.out + o] = J.box;
            jj[J.out + o] = bbi[p];
        }
        if (bad) set_error(err, CT_DEVERR_LOOP);
    }
}

// Pairs of the boxes whose count fits the speculative scratch: one thread per
// scratch slot, box-major, so the writes of a box's pairs are contiguous.
__global__ void k_boxes_spec_emit(const int64_t* __restrict__ cnt, const int64_t* __restrict__ off, int64_t n,
                                  const int* __restrict__ spec, int cap, int64_t* __restrict__ ii,
                                  int64_t* __restrict__ jj) {
    const int64_t total = n * (int64_t)cap;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k / cap;
        const int c = (int)(k - i * cap);
        const int64_t m = cnt[i];
        if (m > cap || c >= m) continue;
        ii[off[i] + c] = i;
        jj[off[i] + c] = spec[k];
    }
}

// Candidates of the segments whose count fits the counting pass's scratch.
__global__ void k_edge_spec_emit(const int64_t* __restrict__ cnt, const int64_t* __restrict__ off, int64_t n,
                                 const int* __restrict__ spec, int cap, int* __restrict__ cseg,
                                 int* __restrict__ cpos) {
    const int64_t total = n * (int64_t)cap;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k / cap;
        const int c = (int)(k - i * cap);
        const int64_t m = cnt[i];
        if (m > cap || c >= m) continue;
        cseg[off[i] + c] = (int)i;
        cpos[off[i] + c] = spec[k];
    }
}

// ---------------------------------------------------------------------------
// locate_edge query.py:357-455 with compute_edge_edge_intersect (292-306,
// mode 0) or compute_edge_face_intersect (309-328, mode 1)
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// locate_edge (query.py:357-455) in two phases: the traversal collects
// candidate (segment, cell) pairs in upstream traversal order; one thread per
// candidate then runs the float64 cell test.  Clipping inside the traversal
// would run with a few lanes of a warp active (every segment's traversal
// differs); per candidate it runs with full warps.  Phase 1 drops only the
// cells that the cell test's own first step (Cohen-Sutherland's
// shared-outcode reject, an exact order comparison) rejects.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int cs_code_keys(unsigned long long kx, unsigned long long ky, unsigned long long x0,
                                            unsigned long long x1, unsigned long long y0, unsigned long long y1) {
    int p = CS_INSIDE;
    if (kx < x0) p |= CS_LEFT;
    else if (kx > x1) p |= CS_RIGHT;
    if (ky < y0) p |= CS_LOWER;
    else if (ky > y1) p |= CS_UPPER;
    return p;
}

// Line filter of the segment traversal (no upstream counterpart).  A cell
// whose box the segment's line misses by more than a margin m cannot be a
// result: Cohen-Sutherland (cohen_sutherland.py:32-101) then rejects it --
// each clipping step puts an endpoint on a box edge line at most a few
// float64 roundings (of the coordinates' magnitude C) off the line, so every
// point it computes stays outside the box, on the side the exact algorithm's
// does, and the exact algorithm rejects a segment that misses the box (a
// segment whose line meets the box beyond an endpoint shares an outcode bit
// and is rejected by the outcode test) -- and for edge trees
// lines_intersect (geometry_utils.py:361-418) finds both tree edge
// endpoints strictly on one side of the segment's line and not within its
// tolerance (1e-12 of the edge length) of it.  m = 2^-40 C (C: the largest
// |coordinate| of the segment and the tree's bbox) + 2^-37 x the tree's
// extent + 2^-47 covers both by orders of magnitude.  The test runs in
// float32 in the tree's frame on node boxes and cell boxes rounded outward:
// f = n . (corner - a) at the corner nearest the line's side, against a
// bound on the float32 and conversion errors (2^-19 of the products'
// magnitudes plus the frame magnitudes) plus m |n|.  Pruning only removes
// cells that produce no result, so results and their order are unchanged.
struct LineF {
    float ax, ay, nx, ny, K, em;
    bool on;
};

__device__ __forceinline__ LineF line_filter(const TreeQ& T, dpt a, dpt b, dpt V, bool keys) {
    LineF L;
    L.on = keys && T.bbl32 != nullptr;
    L.ax = L.ay = L.nx = L.ny = L.K = L.em = 0.0f;
    if (!L.on) return L;
    L.ax = __double2float_rn(a.x - T.ox);
    L.ay = __double2float_rn(a.y - T.oy);
    L.nx = __double2float_rn(-V.y);
    L.ny = __double2float_rn(V.x);
    const float anx = fabsf(L.nx), any = fabsf(L.ny);
    L.K = __fadd_ru(__fmul_ru(anx, __fadd_ru(fabsf(L.ax), T.fX)), __fmul_ru(any, __fadd_ru(fabsf(L.ay), T.fY)));
    const double C = fmax(fmax(fmax(fabs(a.x), fabs(a.y)), fmax(fabs(b.x), fabs(b.y))), T.babs);
    const float m = __double2float_ru(__dadd_ru(__dmul_ru(C, 0x1p-40), T.mext));
    L.em = __fmul_ru(__fmul_ru(m, __fadd_ru(anx, any)), 1.0f + 0x1p-18f);
    // a non-finite term switches the filter off (its comparisons would be false anyway)
    L.on = isfinite(L.K) && isfinite(L.em) && isfinite(L.ax) && isfinite(L.ay);
    return L;
}

// Whether the segment's line surely misses the float32 box (frame of the tree).
__device__ __forceinline__ bool line_misses(const LineF& L, float x0, float x1, float y0, float y1) {
    const float px = L.nx > 0.0f ? x0 : x1, qx = L.nx > 0.0f ? x1 : x0;
    const float py = L.ny > 0.0f ? y0 : y1, qy = L.ny > 0.0f ? y1 : y0;
    const float dpx = __fsub_rn(px, L.ax), dpy = __fsub_rn(py, L.ay);
    const float dqx = __fsub_rn(qx, L.ax), dqy = __fsub_rn(qy, L.ay);
    const float t1 = __fmul_rn(L.nx, dpx), t2 = __fmul_rn(L.ny, dpy);
    const float u1 = __fmul_rn(L.nx, dqx), u2 = __fmul_rn(L.ny, dqy);
    const float fmin = __fadd_rn(t1, t2), fmax_ = __fadd_rn(u1, u2);
    const float emin = __fadd_ru(__fmul_ru(__fadd_ru(__fadd_ru(fabsf(t1), fabsf(t2)), L.K), 0x1p-19f),
                                 __fadd_ru(L.em, 0x1p-100f));
    const float emax = __fadd_ru(__fmul_ru(__fadd_ru(__fadd_ru(fabsf(u1), fabsf(u2)), L.K), 0x1p-19f),
                                 __fadd_ru(L.em, 0x1p-100f));
    return fmin > emin || fmax_ < -emax;
}

// Segment a -> b against the cells of leaf `v` (nf q): the candidates that
// Cohen-Sutherland's shared-outcode test does not reject (mode 1), or every
// cell (mode 0), counted and, with WRITE, written at cseg / cj[base + count].
template <bool WRITE, int MODE>
__device__ __forceinline__ void edge_leaf(const TreeQ& T, float4 q, dpt a, dpt b, bool keys, unsigned long long kax,
                                          unsigned long long kay, unsigned long long kbx, unsigned long long kby,
                                          int64_t i, int64_t base, int64_t& count, int* __restrict__ cseg,
                                          int* __restrict__ cj, const LineF* lf = nullptr, int spcap = 0) {
    int ptr = na(q), bq = nb(q);
    for (int j = ptr; j < ptr + bq; j++) {
        if (lf && lf->on) {
            const float4 c = T.bbl32[j];
            if (line_misses(*lf, c.x, c.y, c.z, c.w)) continue;
        }
        bool cand = true;
        if (MODE == 1) {
            dbox bx = leaf_box(T, j);
            int k1, k2;
            if (keys) {
                unsigned long long x0 = fkey(bx.xmin), x1 = fkey(bx.xmax), y0 = fkey(bx.ymin), y1 = fkey(bx.ymax);
                k1 = cs_code_keys(kax, kay, x0, x1, y0, y1);
                k2 = cs_code_keys(kbx, kby, x0, x1, y0, y1);
            } else {
                k1 = cs_code(a, bx);
                k2 = cs_code(b, bx);
            }
            cand = (k1 & k2) == 0;
        }
        if (cand) {
            if (WRITE) {
                cseg[base + count] = (int)i;
                cj[base + count] = j;
            } else if (count < spcap) {
                cj[count] = j;  // counting pass: the segment's scratch row
            }
            count++;
        }
    }
}

// Children of internal node v the segment's traversal enters (locate_edge
// query.py:410-441): `first` is visited first (the right child when both).
__device__ __forceinline__ void edge_children(const TreeQ& T, double2 nd, float4 q, dpt a, dpt b, dpt V, bool keys,
                                              unsigned long long kax, unsigned long long kay,
                                              unsigned long long kbx, unsigned long long kby, int* first,
                                              int* second) {
    int dim = -1 - nb(q);
    double dx = dim ? V.y : V.x;
    bool left, right;
    if (keys) {
        unsigned long long ka = dim ? kay : kax, kb = dim ? kby : kbx;
        bool pos = dx > 0.0;
        left = fkey(nd.x) >= (pos ? ka : kb);
        right = fkey(nd.y) <= (pos ? kb : ka);
    } else {
        double an = dim ? a.y : a.x, bn = dim ? b.y : b.x;
        double dx_left, dx_right;
        if (dx > 0.0) {
            dx_left = nd.x - an;
            dx_right = nd.y - bn;
        } else {
            dx_left = nd.x - bn;
            dx_right = nd.y - an;
        }
        left = dx_left >= 0.0;
        right = dx_right <= 0.0;
        if (dx > 0.0) {
            if (left) left = (dx_left / dx) >= 0.0;
            if (right) right = (dx_right / dx) <= 1.0;
        } else if (dx < 0.0) {
            if (left) left = (1.0 - (dx_left / dx)) >= 0.0;
            if (right) right = (1.0 - (dx_right / dx)) <= 1.0;
        }
    }
    // pushed left, then right: the right child is visited first
    int child = na(q);
    *first = right ? child + 1 : (left ? child : -1);
    *second = (left && right) ? child : -1;
}

struct EdgeKeys {
    bool keys;
    unsigned long long kax, kay, kbx, kby;
};

__device__ __forceinline__ EdgeKeys edge_keys(const TreeQ& T, dpt a, dpt b) {
    dpt V = vsub(b, a);
    EdgeKeys k;
    k.keys = T.finite && is_fin(a.x) && is_fin(a.y) && is_fin(b.x) && is_fin(b.y) && is_fin(V.x) && is_fin(V.y);
    k.kax = fkey(a.x);
    k.kay = fkey(a.y);
    k.kbx = fkey(b.x);
    k.kby = fkey(b.y);
    return k;
}

// Depth-first traversal of segment i from node `start` (stack form).  With
// CUT the walk stops at the nodes `cut` levels below the start (and at
// leaves above them) and, instead of their candidates, counts / writes those
// nodes (item_seg / item_node): the cut splits one segment's traversal into
// subtrees whose candidate lists, concatenated in this order, are the
// traversal's.
template <bool WRITE, int MODE, bool CUT>
__device__ __forceinline__ int64_t edge_dfs(const TreeQ& T, dpt a, dpt b, int64_t i, int start, int cut,
                                            int64_t base, int* __restrict__ cseg, int* __restrict__ cj,
                                            int spcap = 0) {
    const dpt V = vsub(b, a);
    const EdgeKeys K = edge_keys(T, a, b);
    const LineF LF = line_filter(T, a, b, V, K.keys);
    int st[STK];
    unsigned char sd[CUT ? STK : 1];
    int sp = 1;
    st[0] = start;
    sd[0] = 0;
    int64_t count = 0;
    int64_t budget = T.n_nodes;
    while (sp > 0) {
        if (--budget < 0) {
            set_error(T.err, CT_DEVERR_LOOP);
            break;
        }
        --sp;
        const int v = st[sp];
        const int depth = CUT ? sd[sp] : 0;
        // the node's records loaded together (one round trip per node)
        const float4 q = T.nf[v];
        const double2 nd_v = T.nd[v];
        if (LF.on) {
            const float4 nbx = *reinterpret_cast<const float4*>(T.nbx + v);
            if (line_misses(LF, nbx.x, nbx.y, nbx.z, nbx.w)) continue;
        }
        const bool terminal = nb(q) >= 0;
        if (CUT && (terminal || depth >= cut)) {
            if (WRITE) {
                cseg[base + count] = (int)i;
                cj[base + count] = v;
            }
            count++;
            continue;
        }
        if (terminal) {
            edge_leaf<WRITE, MODE>(T, q, a, b, K.keys, K.kax, K.kay, K.kbx, K.kby, i, base, count, cseg, cj, &LF,
                                   spcap);
            continue;
        }
        int first, second;
        edge_children(T, nd_v, q, a, b, V, K.keys, K.kax, K.kay, K.kbx, K.kby, &first, &second);
        if (sp + 2 > STK) {
            set_error(T.err, CT_DEVERR_STACK);
            break;
        }
        const unsigned char nd1 = (unsigned char)min(depth + 1, 255);
        if (second >= 0) {
            st[sp] = second;
            if (CUT) sd[sp] = nd1;
            sp++;
        }
        if (first >= 0) {
            st[sp] = first;
            if (CUT) sd[sp] = nd1;
            sp++;
        }
    }
    return count;
}

// spcap > 0: in the counting pass cj is a scratch of spcap entries per
// segment that keeps its first candidates; in the writing pass spec_cnt
// holds the counts and segments whose candidates fit were copied from the
// scratch (k_edge_spec_emit), so they return at once.
template <bool WRITE, int MODE, bool DEEP>
__global__ void __launch_bounds__(128) k_edge_cands(TreeQ T, const double4* __restrict__ segs, int64_t n,
                                                    const int* __restrict__ order, int64_t* __restrict__ cnt_or_off,
                                                    int* __restrict__ cseg, int* __restrict__ cj, int spcap = 0,
                                                    const int64_t* __restrict__ spec_cnt = nullptr) {
    int64_t tq = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tq >= n) return;
    int64_t i = order ? (int64_t)order[tq] : tq;
    if (WRITE && spec_cnt && spec_cnt[i] <= spcap) return;
    if (!WRITE && spcap > 0) cj += i * (int64_t)spcap;
    double4 s4 = segs[i];
    dpt a = mkp(s4.x, s4.y), b = mkp(s4.z, s4.w);
    int64_t count = 0;
    int64_t base = WRITE ? cnt_or_off[i] : 0;
    dpt c, d;
    int r = cohen_sutherland(a, b, T.bbox, &c, &d);
    if (r < 0) set_error(T.err, CT_DEVERR_LOOP);
    if (r == 1) {
        if (!DEEP) {
            count = edge_dfs<WRITE, MODE, false>(T, a, b, i, 0, -1, base, cseg, cj, WRITE ? 0 : spcap);
        } else {
            // depth-first walk through the parent links (see k_boxes)
            const dpt V = vsub(b, a);
            const EdgeKeys K = edge_keys(T, a, b);
            int dv = 0, from = -1;
            bool down = true;
            int64_t budget = 2 * T.n_nodes + 2;
            while (dv >= 0) {
                if (--budget < 0) {
                    set_error(T.err, CT_DEVERR_LOOP);
                    break;
                }
                const int v = dv;
                float4 q = T.nf[v];
                int first = -1, second = -1;
                const bool terminal = nb(q) >= 0;
                if (terminal && down)
                    edge_leaf<WRITE, MODE>(T, q, a, b, K.keys, K.kax, K.kay, K.kbx, K.kby, i, base, count, cseg, cj,
                                           nullptr, WRITE ? 0 : spcap);
                if (!terminal)
                    edge_children(T, T.nd[v], q, a, b, V, K.keys, K.kax, K.kay, K.kbx, K.kby, &first, &second);
                int next = terminal ? -1 : (down ? first : ((from == first) ? second : -1));
                from = dv;
                if (next >= 0) {
                    dv = next;
                    down = true;
                } else {
                    dv = T.parent[dv];
                    down = false;
                }
            }
        }
    }
    if (!WRITE) cnt_or_off[i] = count;
}

// The traversal of every segment cut `cut` levels below the root into work
// items (segment, node) in traversal order: counts per segment (WRITE
// false), then the items at their offsets.  Segments that miss the tree's
// bbox (Cohen-Sutherland, as the uncut traversal) have none.
template <bool WRITE, int MODE>
__global__ void __launch_bounds__(128) k_edge_items(TreeQ T, const double4* __restrict__ segs, int64_t n,
                                                    const int* __restrict__ order, int cut,
                                                    int64_t* __restrict__ cnt_or_off, int* __restrict__ item_seg,
                                                    int* __restrict__ item_node) {
    int64_t tq = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tq >= n) return;
    int64_t i = order ? (int64_t)order[tq] : tq;
    double4 s4 = segs[i];
    dpt a = mkp(s4.x, s4.y), b = mkp(s4.z, s4.w);
    int64_t count = 0;
    dpt c, d;
    int r = cohen_sutherland(a, b, T.bbox, &c, &d);
    if (r < 0) set_error(T.err, CT_DEVERR_LOOP);
    if (r == 1)
        count = edge_dfs<WRITE, MODE, true>(T, a, b, i, 0, cut, WRITE ? cnt_or_off[i] : 0, item_seg, item_node);
    if (!WRITE) cnt_or_off[i] = count;
}

// The candidates of every work item (the uncut traversal from the item's
// node): counts per item, then the candidates at the items' offsets.
template <bool WRITE, int MODE>
__global__ void __launch_bounds__(128) k_item_cands(TreeQ T, const double4* __restrict__ segs,
                                                    const int* __restrict__ item_seg,
                                                    const int* __restrict__ item_node, int64_t n_items,
                                                    int64_t* __restrict__ cnt_or_off, int* __restrict__ cseg,
                                                    int* __restrict__ cj) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_items) return;
    const int64_t i = item_seg[k];
    double4 s4 = segs[i];
    dpt a = mkp(s4.x, s4.y), b = mkp(s4.z, s4.w);
    int64_t count = edge_dfs<WRITE, MODE, false>(T, a, b, i, item_node[k], -1, WRITE ? cnt_or_off[k] : 0, cseg, cj);
    if (!WRITE) cnt_or_off[k] = count;
}

// Per segment: the offset and count of its candidates, from its items'
// (items are segment-major; a segment's items are [ioff[s], ioff[s] + icnt[s])).
__global__ void k_seg_from_items(const int64_t* __restrict__ ioff, const int64_t* __restrict__ icnt, int64_t n,
                                 const int64_t* __restrict__ item_coff, const int64_t* __restrict__ item_ccnt,
                                 int64_t n_items, int64_t* __restrict__ coff, int64_t* __restrict__ ccnt) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k0 = ioff[s], k1 = k0 + icnt[s];
        const int64_t total = n_items > 0 ? item_coff[n_items - 1] + item_ccnt[n_items - 1] : 0;
        const int64_t c0 = k0 < n_items ? item_coff[k0] : total;
        const int64_t c1 = k1 < n_items ? item_coff[k1] : total;
        coff[s] = c0;
        ccnt[s] = c1 - c0;
    }
}

// Sign of the cross product (v - a) x s used by Cyrus-Beck's crossing walk
// (cyrus_beck.py:162-180: ksi / eta) decided in float32 in the cell's local
// frame: -1 / +1 when sure (then also nonzero), 0 when the float64 product
// must be computed.  dv, da: float32 local coordinates of v and a (error ev
// per component), sf: float32 s with error es.  The float64 value is
// fl(fl(U.x * s.y) - fl(U.y * s.x)) with U = fl(v - a): within
// 3.0001 u (|U.x||s.y| + |U.y||s.x|) (u = 2^-53) of the exact product of the
// float64 inputs, so a float32 margin above that bound plus the float32
// error fixes its sign.
__device__ __forceinline__ int cb_sign32(float2 dv, float2 da, float ev, float2 sf, float es) {
    const float u24 = 5.9604644775390625e-08f;
    float ux = dv.x - da.x, uy = dv.y - da.y;
    float eu = 2.0f * ev + u24 * fmaxf(fabsf(ux), fabsf(uy));
    float M = fmaxf(fabsf(ux), fabsf(uy)) + eu;
    float Ns = fabsf(sf.x) + fabsf(sf.y) + 2.0f * es;
    float est = ux * sf.y - uy * sf.x;
    float thr = 1.02f * (2.0f * es * M + Ns * eu + 4.0f * u24 * Ns * M + 3.3307e-16f * Ns * M) + 1e-37f;
    if (!(fabsf(est) > thr)) return 0;
    return est > 0.0f ? 1 : -1;
}

// cyrus_beck_line_polygon_clip (cyrus_beck.py:133-241) with its float64
// decisions screened in float32: the two point_in_polygon_or_on_edge tests by
// the certified leaf filter (ct_locf.cuh), the crossing walk's signs by
// cb_sign32; undecided ones run in float64.  The intersection parameters and
// clipped points are the float64 computations of cyrus_beck().
template <int KT>
__device__ __forceinline__ bool cyrus_beck_f32(dpt a, dpt b, const dpt* poly, int length, double tol,
                                               const float4* __restrict__ cellf, int len32, float dabs, dpt* c,
                                               dpt* d) {
    *c = mkp(dnan(), dnan());
    *d = *c;
    dpt s = vsub(b, a);
    if (s.x == 0 && s.y == 0) return false;
    float tolf = (float)tol;
    if ((double)tolf < tol) tolf = nextafterf(tolf, INFINITY);
    PtSplit Pa = split_point(a.x, a.y), Pb = split_point(b.x, b.y);
    int ra = leaf_filter_local<KT>(Pa, dabs, tolf, cellf, len32);
    int rb = leaf_filter_local<KT>(Pb, dabs, tolf, cellf, len32);
    bool a_inside = (ra == LF_UNSURE) ? pip_or_edge(a, poly, length, tol) : (ra == LF_INSIDE);
    bool b_inside = (rb == LF_UNSURE) ? pip_or_edge(b, poly, length, tol) : (rb == LF_INSIDE);
    if (a_inside && b_inside) {
        *c = a;
        *d = b;
        return true;
    }
    // float32 local coordinates of a and s (frame: the cell's first vertex)
    float da_x, da_y, ea, db_x, db_y, eb;
    local_delta(Pa, cellf[0], &da_x, &da_y, &ea);
    local_delta(Pb, cellf[0], &db_x, &db_y, &eb);
    const float u24 = 5.9604644775390625e-08f;
    const float ed = fmaxf(ea, eb) + dabs;
    const float2 da = make_float2(da_x, da_y);
    const float2 sf = make_float2(db_x - da_x, db_y - da_y);
    const float es = 2.0f * ed + 2.0f * u24 * fmaxf(fabsf(sf.x), fabsf(sf.y));
    const float2* rel = reinterpret_cast<const float2*>(cellf + 1);
    // poly[i] in the local frame: vertex 0 at the origin, the others as their
    // stored float32 offsets (rounded by 2^-24 of their size)
    float vmax = 0.0f;
    for (int i = 1; i < len32 && i < KT; i++) vmax = fmaxf(vmax, fmaxf(fabsf(rel[i - 1].x), fabsf(rel[i - 1].y)));
    const float ev = ed + u24 * vmax + dabs;
    // the float32 cell lists the same vertices as poly unless repeated ones were dropped
    const bool use32 = (len32 == length);
    int i0 = -1, i1 = -1, i = 0, k = 0;
    int sk = use32 ? cb_sign32(make_float2(0.0f, 0.0f), da, ev, sf, es) : 0;
    bool ksi64 = sk == 0;
    double ksi = ksi64 ? crossp(vsub(poly[0], a), s) : 0.0;
    while (i < length && k < 2) {
        const int in = (i + 1) % length;
        int se = use32 ? cb_sign32(in == 0 ? make_float2(0.0f, 0.0f) : rel[in - 1], da, ev, sf, es) : 0;
        const bool eta64 = se == 0;
        const double eta = eta64 ? crossp(vsub(poly[in], a), s) : 0.0;
        const bool ksi_neg = ksi64 ? (ksi < 0.0) : (sk < 0);
        const bool eta_neg = eta64 ? (eta < 0.0) : (se < 0);
        if (ksi_neg != eta_neg) {
            if (k == 0) i0 = i;
            else i1 = i;
            k++;
        } else if (ksi64 && eta64 && ksi == 0.0 && eta == 0.0) {
            bool r = cb_collinear(a, b, poly[i], poly[in], c, d);
            if (!r) {
                *c = mkp(dnan(), dnan());
                *d = *c;
            }
            return r;
        }
        ksi = eta;
        sk = se;
        ksi64 = eta64;
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
// Cohen-Sutherland's verdict in float32 intervals (no upstream counterpart)
// ---------------------------------------------------------------------------
// cohen_sutherland() above is replayed in the cell's local frame (the float32
// cell: its first vertex split hi + lo, the other vertices as offsets) on
// intervals with directed rounding.  Every interval encloses the float64 value
// upstream's code computes at that step: inputs enclose the exact local
// coordinates, each operation's result is widened by the float64 rounding of
// that operation (2^-51 of its magnitude, plus 2^-50 of the largest absolute
// coordinate where the result is an absolute coordinate).  When every outcode
// test and every dx == dy == 0 test is decided for the whole interval, the
// float64 run takes the same path, so its verdict is known: 1 accept, 0
// reject; -1 when any test is undecided (the caller runs the float64 clip).
// Only the verdict is used: upstream overwrites the clipped points with
// Cyrus-Beck's.
struct FI {
    float lo, hi;
};
__device__ __forceinline__ FI fi_sub(FI a, FI b) { return FI{__fsub_rd(a.lo, b.hi), __fsub_ru(a.hi, b.lo)}; }
__device__ __forceinline__ FI fi_add(FI a, FI b) { return FI{__fadd_rd(a.lo, b.lo), __fadd_ru(a.hi, b.hi)}; }
__device__ __forceinline__ FI fi_mul(FI a, FI b) {
    const float l = fminf(fminf(__fmul_rd(a.lo, b.lo), __fmul_rd(a.lo, b.hi)),
                          fminf(__fmul_rd(a.hi, b.lo), __fmul_rd(a.hi, b.hi)));
    const float h = fmaxf(fmaxf(__fmul_ru(a.lo, b.lo), __fmul_ru(a.lo, b.hi)),
                          fmaxf(__fmul_ru(a.hi, b.lo), __fmul_ru(a.hi, b.hi)));
    return FI{l, h};
}
// b must exclude 0
__device__ __forceinline__ FI fi_div(FI a, FI b) {
    const float l = fminf(fminf(__fdiv_rd(a.lo, b.lo), __fdiv_rd(a.lo, b.hi)),
                          fminf(__fdiv_rd(a.hi, b.lo), __fdiv_rd(a.hi, b.hi)));
    const float h = fmaxf(fmaxf(__fdiv_ru(a.lo, b.lo), __fdiv_ru(a.lo, b.hi)),
                          fmaxf(__fdiv_ru(a.hi, b.lo), __fdiv_ru(a.hi, b.hi)));
    return FI{l, h};
}
__device__ __forceinline__ bool fi_ok(FI a) { return isfinite(a.lo) && isfinite(a.hi) && a.lo <= a.hi; }
__device__ __forceinline__ bool fi_has0(FI a) { return !(a.lo > 0.0f || a.hi < 0.0f); }
// float64 rounding of one operation: 2^-51 of the result's magnitude, plus
// `w` (2^-50 of the largest absolute coordinate) for absolute coordinates
__device__ __forceinline__ FI fi_round(FI a, float w) {
    const float e = __fadd_ru(__fmul_ru(fmaxf(fabsf(a.lo), fabsf(a.hi)), 0x1p-51f), w + 0x1p-126f);
    return FI{__fsub_rd(a.lo, e), __fadd_ru(a.hi, e)};
}

// Outcode of an interval point (-1: undecided); a coordinate set to a box
// side (tag >= 0) is exactly that side.
__device__ __forceinline__ int fi_code(FI x, FI y, int tx, int ty, const FI* B) {
    int p = 0;
    if (tx < 0) {
        if (x.hi < B[0].lo) p |= CS_LEFT;
        else if (x.lo >= B[0].hi && x.lo > B[1].hi) p |= CS_RIGHT;
        else if (!(x.lo >= B[0].hi && x.hi <= B[1].lo)) return -1;
    }
    if (ty < 0) {
        if (y.hi < B[2].lo) p |= CS_LOWER;
        else if (y.lo >= B[2].hi && y.lo > B[3].hi) p |= CS_UPPER;
        else if (!(y.lo >= B[2].hi && y.hi <= B[3].lo)) return -1;
    }
    return p;
}

__device__ __forceinline__ int cs_f32(dpt a, dpt b, const dbox& box, const float4* __restrict__ cellf, int len32,
                                      float dabs) {
    // non-finite endpoints and cells of fewer than two distinct vertices
    // (no float32 frame) take the float64 clip
    if (!(is_fin(a.x) && is_fin(a.y) && is_fin(b.x) && is_fin(b.y)) || len32 < 2) return -1;
    // the exact tests on the inputs, as upstream
    if (g_eq_finite(a.x, b.x) && g_eq_finite(a.y, b.y)) return 0;
    int k1 = cs_code(a, box), k2 = cs_code(b, box);
    if ((k1 | k2) == 0) return 1;
    if ((k1 & k2) != 0) return 0;
    // local frame: intervals of the endpoints and the box sides
    const PtSplit Pa = split_point(a.x, a.y), Pb = split_point(b.x, b.y);
    float ax, ay, ea, bx, by, eb;
    local_delta(Pa, cellf[0], &ax, &ay, &ea);
    local_delta(Pb, cellf[0], &bx, &by, &eb);
    const float2* rel = reinterpret_cast<const float2*>(cellf + 1);
    float x0 = 0.0f, x1 = 0.0f, y0 = 0.0f, y1 = 0.0f, vmax = 0.0f;
    for (int i = 1; i < len32 && i < 8; i++) {
        const float2 r = rel[i - 1];
        x0 = fminf(x0, r.x);
        x1 = fmaxf(x1, r.x);
        y0 = fminf(y0, r.y);
        y1 = fmaxf(y1, r.y);
        vmax = fmaxf(vmax, fmaxf(fabsf(r.x), fabsf(r.y)));
    }
    // stored offsets: float32 roundings of the float64 differences
    const float ev = __fadd_ru(__fmul_ru(vmax, 0x1p-22f), dabs + 0x1p-126f);
    const float ep = fmaxf(ea, eb) + dabs + 0x1p-126f;
    FI B[4] = {FI{__fsub_rd(x0, ev), __fadd_ru(x0, ev)}, FI{__fsub_rd(x1, ev), __fadd_ru(x1, ev)},
               FI{__fsub_rd(y0, ev), __fadd_ru(y0, ev)}, FI{__fsub_rd(y1, ev), __fadd_ru(y1, ev)}};
    FI Ax{__fsub_rd(ax, ep), __fadd_ru(ax, ep)}, Ay{__fsub_rd(ay, ep), __fadd_ru(ay, ep)};
    FI Bx{__fsub_rd(bx, ep), __fadd_ru(bx, ep)}, By{__fsub_rd(by, ep), __fadd_ru(by, ep)};
    int tax = -1, tay = -1, tbx = -1, tby = -1;
    // 2^-50 of the largest absolute coordinate of the segment and the cell
    const float C = fmaxf(fmaxf(fmaxf(fabsf(Pa.xh), fabsf(Pa.yh)), fmaxf(fabsf(Pb.xh), fabsf(Pb.yh))),
                          fmaxf(fabsf(cellf[0].x), fabsf(cellf[0].z)) + vmax);
    const float w = __fmul_ru(__fmul_ru(C, 1.0f + 0x1p-20f), 0x1p-50f);
    if (!(fi_ok(Ax) && fi_ok(Ay) && fi_ok(Bx) && fi_ok(By) && isfinite(w))) return -1;
    for (int iter = 0; iter < 8; iter++) {
        if ((k1 | k2) == 0) return 1;
        if ((k1 & k2) != 0) return 0;
        const int opt = k1 ? k1 : k2;
        const FI DX = fi_round(fi_sub(Bx, Ax), 0.0f), DY = fi_round(fi_sub(By, Ay), 0.0f);
        FI x, y;
        int tx = -1, ty = -1;
        if (opt & (CS_UPPER | CS_LOWER)) {
            if (fi_has0(DY)) return -1;
            const int side = (opt & CS_UPPER) ? 3 : 2;
            const FI t = fi_round(fi_div(fi_round(fi_mul(DX, fi_round(fi_sub(B[side], Ay), 0.0f)), 0.0f), DY), 0.0f);
            x = fi_round(fi_add(Ax, t), w);
            y = B[side];
            ty = side;
        } else {
            if (fi_has0(DX)) return -1;
            const int side = (opt & CS_RIGHT) ? 1 : 0;
            const FI t = fi_round(fi_div(fi_round(fi_mul(DY, fi_round(fi_sub(B[side], Ax), 0.0f)), 0.0f), DX), 0.0f);
            y = fi_round(fi_add(Ay, t), w);
            x = B[side];
            tx = side;
        }
        if (!(fi_ok(x) && fi_ok(y))) return -1;
        if (opt == k1) {
            Ax = x;
            Ay = y;
            tax = tx;
            tay = ty;
            k1 = fi_code(Ax, Ay, tax, tay, B);
            if (k1 < 0) return -1;
        } else {
            Bx = x;
            By = y;
            tbx = tx;
            tby = ty;
            k2 = fi_code(Bx, By, tbx, tby, B);
            if (k2 < 0) return -1;
        }
        // dx == 0 and dy == 0: equal coordinates are certain when both were
        // set to the same box side, unequal when the intervals are disjoint
        const bool xeq = tax >= 0 && tax == tbx, yeq = tay >= 0 && tay == tby;
        const bool xne = Ax.hi < Bx.lo || Bx.hi < Ax.lo, yne = Ay.hi < By.lo || By.hi < Ay.lo;
        if (xeq && yeq) return 0;
        if (!(xne || yne)) return -1;
    }
    return -1;
}

// The float64 cell test of every candidate (compute_edge_face_intersect
// query.py:309-328 / compute_edge_edge_intersect 292-306).
template <int MODE>
__global__ void __launch_bounds__(128) k_edge_test(TreeQ T, const double4* __restrict__ segs,
                                                   const int* __restrict__ cseg, const int* __restrict__ cj,
                                                   int64_t nc, int64_t* __restrict__ keep, double4* __restrict__ xy) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nc; t += (int64_t)gridDim.x * blockDim.x) {
        double4 s4 = segs[cseg[t]];
        dpt a = mkp(s4.x, s4.y), b = mkp(s4.z, s4.w);
        int j = cj[t];
        dpt c, d;
        bool hit;
        if (MODE == 0) {
            double2 p0 = T.poly[(size_t)j * 2], p1 = T.poly[(size_t)j * 2 + 1];
            double x, y;
            hit = lines_intersect(a, b, mkp(p0.x, p0.y), mkp(p1.x, p1.y), &x, &y);
            c = mkp(x, y);
            d = c;
        } else {
            dbox bx = leaf_box(T, j);
            int rr = -1;
            if (T.polyf && T.K <= 8) rr = cs_f32(a, b, bx, T.polyf + (size_t)j * T.S4, (int)T.plen32[j], T.dabs);
            if (rr < 0) {
                rr = cohen_sutherland(a, b, bx, &c, &d);
                if (rr < 0) set_error(T.err, CT_DEVERR_LOOP);
            }
            hit = rr == 1;
            if (hit) {
                const dpt* poly = reinterpret_cast<const dpt*>(T.poly + (size_t)j * T.K);
                int len = T.plen ? (int)T.plen[j] : T.K;
                double tol = pmax(CT_MIN_TOLERANCE, CT_TOLERANCE_FACTOR * pmax(bx.xmax - bx.xmin, bx.ymax - bx.ymin));
                if (T.polyf && T.K <= 8)
                    hit = cyrus_beck_f32<8>(a, b, poly, len, tol, T.polyf + (size_t)j * T.S4, (int)T.plen32[j],
                                            T.dabs, &c, &d);
                else
                    hit = cyrus_beck(a, b, poly, len, tol, &c, &d);
            }
        }
        keep[t] = hit ? 1 : 0;
        xy[t] = make_double4(c.x, c.y, d.x, d.y);
    }
}

// Diagnostics of the segment test's float32 certificates (tests only): per
// pair, upstream's float64 Cohen-Sutherland verdict (1 accept, 0 reject, -1
// loop cap), the float32 interval verdict (cs_f32: 1, 0, -1 undecided) and
// whether the traversal's line filter surely misses the cell's box (1/0; 0
// when the filter is off).
__global__ void k_cs_certificates(TreeQ T, const double4* __restrict__ segs, const int* __restrict__ cseg,
                                  const int* __restrict__ cj, int64_t nc, int8_t* __restrict__ out) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nc; t += (int64_t)gridDim.x * blockDim.x) {
        double4 s4 = segs[cseg[t]];
        dpt a = mkp(s4.x, s4.y), b = mkp(s4.z, s4.w);
        const int j = cj[t];
        dbox bx = leaf_box(T, j);
        dpt c, d;
        out[3 * t] = (int8_t)cohen_sutherland(a, b, bx, &c, &d);
        out[3 * t + 1] = (int8_t)((T.polyf && T.K <= 8)
                                      ? cs_f32(a, b, bx, T.polyf + (size_t)j * T.S4, (int)T.plen32[j], T.dabs)
                                      : -1);
        const EdgeKeys K = edge_keys(T, a, b);
        const LineF LF = line_filter(T, a, b, vsub(b, a), K.keys);
        int miss = 0;
        if (LF.on) {
            const float4 q = T.bbl32[j];
            miss = line_misses(LF, q.x, q.y, q.z, q.w) ? 1 : 0;
        }
        out[3 * t + 2] = (int8_t)miss;
    }
}

// Hits in candidate order (segment-major, traversal order within a segment),
// and every segment's hit offset and count.
__global__ void k_edge_compact(const int64_t* __restrict__ keep, const int64_t* __restrict__ pos, int64_t nc,
                               const int* __restrict__ cseg, const int* __restrict__ cj,
                               const int64_t* __restrict__ bbi, const double4* __restrict__ xy_c,
                               int64_t* __restrict__ ii, int64_t* __restrict__ jj, double4* __restrict__ xy) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nc; t += (int64_t)gridDim.x * blockDim.x) {
        if (!keep[t]) continue;
        int64_t p = pos[t];
        ii[p] = cseg[t];
        jj[p] = bbi[cj[t]];
        xy[p] = xy_c[t];
    }
}

__global__ void k_edge_seg_counts(const int64_t* __restrict__ coff, const int64_t* __restrict__ ccnt,
                                  const int64_t* __restrict__ keep, const int64_t* __restrict__ pos, int64_t nc,
                                  int64_t n, int64_t* __restrict__ off, int64_t* __restrict__ cnt) {
    const int64_t total = nc > 0 ? pos[nc - 1] + keep[nc - 1] : 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t c0 = coff[i], c1 = c0 + ccnt[i];
        int64_t p0 = c0 < nc ? pos[c0] : total, p1 = c1 < nc ? pos[c1] : total;
        off[i] = p0;
        cnt[i] = p1 - p0;
    }
}

// ---------------------------------------------------------------------------
// exclusive scan of int64 counts
// ---------------------------------------------------------------------------
constexpr int SCAN_T = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_T * SCAN_ITEMS;

// Block-wide exclusive scan; every thread receives the block total in *total.
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* total) {
    __shared__ int64_t warp_sums[SCAN_T / 32];
    __shared__ int64_t block_total;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t s = lane < SCAN_T / 32 ? warp_sums[lane] : 0;
        int64_t y = s;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t t = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y += t;
        }
        if (lane < SCAN_T / 32) warp_sums[lane] = y - s;
        if (lane == SCAN_T / 32 - 1) block_total = y;
    }
    __syncthreads();
    int64_t r = x - v + warp_sums[w];
    *total = block_total;
    __syncthreads();
    return r;
}

__global__ void k_scan_reduce(const int64_t* __restrict__ in, int64_t n, int64_t* __restrict__ sums) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int64_t s = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t i = base + (int64_t)k * SCAN_T + threadIdx.x;
        if (i < n) s += in[i];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ int64_t ws[SCAN_T / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int k = 0; k < SCAN_T / 32; k++) t += ws[k];
        sums[blockIdx.x] = t;
    }
}

// single block: exclusive scan of the block sums in place, total at sums[nb]
__global__ void k_scan_sums(int64_t* sums, int64_t nblocks) {
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < nblocks; base += SCAN_T) {
        int64_t i = base + threadIdx.x;
        int64_t v = i < nblocks ? sums[i] : 0;
        int64_t tot;
        int64_t ex = block_exclusive_scan(v, &tot);
        if (i < nblocks) sums[i] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[nblocks] = carry;
}

__global__ void k_scan_down(const int64_t* __restrict__ in, int64_t n, const int64_t* __restrict__ sums,
                            int64_t* __restrict__ out) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int64_t v[SCAN_ITEMS];
    int64_t s = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t i = base + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    int64_t tot;
    int64_t ex = block_exclusive_scan(s, &tot) + sums[blockIdx.x];
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t i = base + k;
        if (i < n) out[i] = ex;
        ex += v[k];
    }
}

// ---------------------------------------------------------------------------
// per-segment stable sort by t (sort_intersections_by_edge
// geometry_utils.py:564-574: np.lexsort((t, ii)), NaN last)
// ---------------------------------------------------------------------------

// sortable key of t: NaN greatest, otherwise the float order
__device__ __forceinline__ unsigned long long tkey(double t) {
    unsigned long long b = (unsigned long long)__double_as_longlong(t);
    if ((b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) return ~0ull;
    return fkey(t);
}

__global__ void k_tkeys(const double4* __restrict__ segs, const int64_t* __restrict__ ii,
                        const double4* __restrict__ xy, int64_t total, unsigned long long* __restrict__ key,
                        int64_t* __restrict__ idx) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= total) return;
    double4 s = segs[ii[r]];
    double4 c = xy[r];
    double abx = s.z - s.x, aby = s.w - s.y;
    double acx = c.x - s.x, acy = c.y - s.y;
    double t = acx * abx + acy * aby;
    key[r] = tkey(t);
    idx[r] = r;
}

__device__ __forceinline__ bool kless(unsigned long long ka, int64_t ia, unsigned long long kb, int64_t ib) {
    return ka < kb || (ka == kb && ia < ib);
}

constexpr int SORT_T = 128;
constexpr int SORT_SMEM = 1024;  // 2 x 1024 x (8 + 8) B = 32 KB static shared memory

// One block per segment: stable sort of (key, idx) pairs of the segment by
// bottom-up merging; (key, idx) pairs are unique, so each element's output
// rank is its rank in its own run plus the number of smaller elements in the
// partner run (binary search).  Small segments are sorted in shared memory,
// large ones in global memory (A/B ping-pong); the result lands in `idx_out`.
// Segments of more than WARP_SORT_MAX results (listed by k_segsort_warp).
__global__ void __launch_bounds__(SORT_T) k_segsort(const int64_t* __restrict__ off, const int64_t* __restrict__ cnt,
                                                    const int* __restrict__ list,
                                                    const unsigned long long* __restrict__ nlist,
                                                    unsigned long long* __restrict__ kA, int64_t* __restrict__ iA,
                                                    unsigned long long* __restrict__ kB, int64_t* __restrict__ iB,
                                                    int64_t* __restrict__ idx_out) {
    __shared__ unsigned long long sk[2][SORT_SMEM];
    __shared__ int64_t si[2][SORT_SMEM];
    const int64_t nl = (int64_t)*nlist;
    for (int64_t li = blockIdx.x; li < nl; li += gridDim.x) {
    __syncthreads();
    const int64_t sgi = list[li];
    int64_t c = cnt[sgi], o = off[sgi];
    bool smem = c <= SORT_SMEM;
    unsigned long long* k0 = smem ? sk[0] : kA + o;
    int64_t* i0 = smem ? si[0] : iA + o;
    unsigned long long* k1 = smem ? sk[1] : kB + o;
    int64_t* i1 = smem ? si[1] : iB + o;
    if (smem) {
        for (int64_t t = threadIdx.x; t < c; t += blockDim.x) {
            sk[0][t] = kA[o + t];
            si[0][t] = iA[o + t];
        }
    }
    __syncthreads();
    for (int64_t w = 1; w < c; w <<= 1) {
        for (int64_t t = threadIdx.x; t < c; t += blockDim.x) {
            int64_t run = t / w;
            int64_t r0 = (run ^ 1) * w;  // partner run start
            bool left = (run & 1) == 0;
            int64_t own0 = run * w;
            int64_t pair0 = left ? own0 : r0;
            unsigned long long mk = k0[t];
            int64_t mi = i0[t];
            int64_t plo = r0, phi = min(r0 + w, c);
            if (plo > c) plo = c;
            int64_t lo = plo, hi = phi;  // count partner elements smaller than (mk, mi)
            while (lo < hi) {
                int64_t mid = (lo + hi) >> 1;
                if (kless(k0[mid], i0[mid], mk, mi)) lo = mid + 1;
                else hi = mid;
            }
            int64_t dst = pair0 + (t - own0) + (lo - plo);
            k1[dst] = mk;
            i1[dst] = mi;
        }
        __syncthreads();
        unsigned long long* tk = k0;
        k0 = k1;
        k1 = tk;
        int64_t* ti = i0;
        i0 = i1;
        i1 = ti;
    }
    for (int64_t t = threadIdx.x; t < c; t += blockDim.x) idx_out[o + t] = i0[t];
    }
}

// One warp per segment: bitonic sort of up to 32 x E (key, idx) pairs in
// registers (element r * 32 + lane in register r of the lane; pads sort
// last).  (key, idx) pairs are unique, so the order is the stable sort's.
constexpr int WARP_SORT_MAX = 128;

template <int E>
__device__ __forceinline__ void warp_bitonic(unsigned long long (&k)[E], int64_t (&x)[E], int lane) {
    const unsigned FULL = 0xffffffffu;
#pragma unroll
    for (int size = 2; size <= 32 * E; size <<= 1) {
#pragma unroll
        for (int j = size >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int rj = j >> 5;
#pragma unroll
                for (int r = 0; r < E; r++) {
                    const int rp = r ^ rj;
                    if (rp > r) {
                        const bool asc = ((r * 32 + lane) & size) == 0;
                        const bool less_rp = kless(k[rp], x[rp], k[r], x[r]);
                        if (asc ? less_rp : !less_rp) {
                            const unsigned long long tk = k[r];
                            k[r] = k[rp];
                            k[rp] = tk;
                            const int64_t tx = x[r];
                            x[r] = x[rp];
                            x[rp] = tx;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < E; r++) {
                    const unsigned long long pk = __shfl_xor_sync(FULL, k[r], j);
                    const int64_t px = __shfl_xor_sync(FULL, x[r], j);
                    const bool asc = ((r * 32 + lane) & size) == 0;
                    const bool lower = (lane & j) == 0;
                    const bool pless = kless(pk, px, k[r], x[r]);
                    if ((lower == asc) ? pless : !pless) {
                        k[r] = pk;
                        x[r] = px;
                    }
                }
            }
        }
    }
}

template <int E>
__device__ __forceinline__ void warp_sort_segment(const unsigned long long* __restrict__ kA,
                                                  const int64_t* __restrict__ iA, int64_t o, int64_t c, int lane,
                                                  int64_t* __restrict__ idx_out) {
    unsigned long long k[E];
    int64_t x[E];
#pragma unroll
    for (int r = 0; r < E; r++) {
        const int64_t e = r * 32 + lane;
        k[r] = e < c ? kA[o + e] : ~0ull;
        x[r] = e < c ? iA[o + e] : INT64_MAX;
    }
    warp_bitonic<E>(k, x, lane);
#pragma unroll
    for (int r = 0; r < E; r++) {
        const int64_t e = r * 32 + lane;
        if (e < c) idx_out[o + e] = x[r];
    }
}

// Segments of up to WARP_SORT_MAX results sorted by a warp each; longer ones
// are listed for k_segsort.
__global__ void __launch_bounds__(256) k_segsort_warp(const int64_t* __restrict__ off,
                                                      const int64_t* __restrict__ cnt, int64_t nseg,
                                                      const unsigned long long* __restrict__ kA,
                                                      const int64_t* __restrict__ iA, int64_t* __restrict__ idx_out,
                                                      int* __restrict__ list, unsigned long long* __restrict__ nlist) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t sgi = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); sgi < nseg; sgi += warps) {
        const int64_t c = cnt[sgi], o = off[sgi];
        if (c <= 0) continue;
        if (c == 1) {
            if (lane == 0) idx_out[o] = iA[o];
        } else if (c <= 32) {
            warp_sort_segment<1>(kA, iA, o, c, lane, idx_out);
        } else if (c <= 64) {
            warp_sort_segment<2>(kA, iA, o, c, lane, idx_out);
        } else if (c <= WARP_SORT_MAX) {
            warp_sort_segment<4>(kA, iA, o, c, lane, idx_out);
        } else if (lane == 0) {
            list[atomicAdd(nlist, 1ull)] = (int)sgi;
        }
    }
}

__global__ void k_gather_results(const int64_t* __restrict__ perm, int64_t total, const int64_t* __restrict__ jj_in,
                                 const double4* __restrict__ xy_in, int64_t* __restrict__ jj_out,
                                 double4* __restrict__ xy_out) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= total) return;
    int64_t s = perm[r];
    jj_out[r] = jj_in[s];
    xy_out[r] = xy_in[s];
}

// ---------------------------------------------------------------------------
// per-pair kernels
// ---------------------------------------------------------------------------

__device__ __forceinline__ int load_poly(const double* __restrict__ v, const int64_t* __restrict__ faces, int K,
                                         int64_t f, dpt* out) {
    return gather_polygon(v, faces + f * K, K, out);
}

// Float32 filter of polygons_intersect (separating_axis.py:17-75).
//
// For the axis of edge p -> q the upstream test compares float64
// projections v . n with n = (p.y - q.y, q.x - p.x) (both float64).  Each
// projection is within D = 2u(1+u) |v|max (|n.x| + |n.y|) (u = 2^-53) of the
// exact projection on that same n, so a comparison of a maximum with a
// minimum whose exact values differ by more than 2D has the float64 outcome
// of the exact one.  Here the projections are evaluated in float32 in a frame
// at the first vertex of a (each coordinate split exactly into float hi + lo,
// as the leaf filter does), within E of the exact ones (error terms of the
// local coordinates, of n and of the float32 dot products).  An axis whose
// two comparisons clear 2(D + E) is decided: separating or not.  Any
// decided separating axis makes the answer false (upstream stops at the
// first separating axis, but the answer is the same boolean); all axes
// decided and none separating makes it true; otherwise the float64 test runs.
// Returns 0 / 1 for a decided answer, 2 when undecided.
template <int KA, int KB>
__device__ __forceinline__ int sat_filter(const dpt* a, int la, const dpt* b, int lb) {
    constexpr int KM = KA + KB;
    const float u32 = 5.9604644775390625e-08f;  // 2^-24
    float dx[KM], dy[KM];
    float vmax = 0.0f, dmax = 0.0f, ed = 0.0f;
    PtSplit O = split_point(a[0].x, a[0].y);
    bool finite = true;
#pragma unroll
    for (int j = 0; j < KM; j++) {
        if (j < KA ? j < la : (j - KA) < lb) {
            dpt v = j < KA ? a[j] : b[j - KA];
            finite = finite && g_finite(v.x) && g_finite(v.y);
            PtSplit P = split_point(v.x, v.y);
            float4 o = make_float4(O.xh, O.xl, O.yh, O.yl);
            float e;
            local_delta(P, o, &dx[j], &dy[j], &e);
            ed = fmaxf(ed, e);
            dmax = fmaxf(dmax, fmaxf(fabsf(dx[j]), fabsf(dy[j])));
            vmax = fmaxf(vmax, fmaxf(fabsf(P.xh), fabsf(P.yh)));
        } else {
            dx[j] = dy[j] = 0.0f;
        }
    }
    if (!finite) return 2;
    vmax *= 1.0000003f;
    dmax += ed;
    bool undecided = false;
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const int base = side ? KA : 0, len = side ? lb : la;
        const int KS = side ? KB : KA;
#pragma unroll
        for (int i = 0; i < KS; i++) {
            if (i >= len) break;
            const int ip = (i == 0) ? base + len - 1 : base + i - 1, iq = base + i;
            dpt p = side ? b[ip - KA] : a[ip], q = side ? b[iq - KA] : a[iq];
            if (g_zero_edge(p, q)) continue;  // norm == (0, 0): upstream skips the axis
            float nx = dy[ip] - dy[iq], ny = dx[iq] - dx[ip];
            float nm = fabsf(nx) + fabsf(ny);
            float en = 2.0f * ed + 2.0f * u32 * fmaxf(fabsf(nx), fabsf(ny));
            float mina = 3.0e38f, maxa = -3.0e38f, minb = 3.0e38f, maxb = -3.0e38f;
#pragma unroll
            for (int j = 0; j < KM; j++) {
                if (j < KA ? j < la : (j - KA) < lb) {
                    float pr = dx[j] * nx + dy[j] * ny;
                    if (j < KA) {
                        mina = fminf(mina, pr);
                        maxa = fmaxf(maxa, pr);
                    } else {
                        minb = fminf(minb, pr);
                        maxb = fmaxf(maxb, pr);
                    }
                }
            }
            float E = ed * nm + 2.0f * dmax * en + 4.0f * u32 * dmax * (nm + 2.0f * en);
            float D = 2.2204461e-16f * 1.0001f * vmax * (nm + 2.0f * en);
            float thr = 2.03f * (E + D) + 1e-37f;
            float d1 = maxa - minb, d2 = maxb - mina;
            bool sure1 = fabsf(d1) * (1.0f - 4.0f * u32) > thr, sure2 = fabsf(d2) * (1.0f - 4.0f * u32) > thr;
            // separating for sure: one comparison surely false
            if ((sure1 && d1 < 0.0f) || (sure2 && d2 < 0.0f)) return 0;
            if (!(sure1 && sure2)) undecided = true;
        }
    }
    return undecided ? 2 : 1;
}

// polygons_intersect separating_axis.py:58-75
__global__ void k_sat(const double* __restrict__ va, const int64_t* __restrict__ fa, int Ka,
                      const double* __restrict__ vb, const int64_t* __restrict__ fb, int Kb,
                      const int64_t* __restrict__ ia, const int64_t* __restrict__ ib, int64_t n,
                      uint8_t* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dpt a[CT_MAX_N_VERTEX], b[CT_MAX_N_VERTEX];
    int la = load_poly(va, fa, Ka, ia[i], a);
    int lb = load_poly(vb, fb, Kb, ib[i], b);
    int r = 2;
    if (Ka <= 4 && Kb <= 4) r = sat_filter<4, 4>(a, la, b, lb);
    else if (Ka <= 8 && Kb <= 8) r = sat_filter<8, 8>(a, la, b, lb);
    if (r == 2) r = (int)(separating_axes(a, la, b, lb) && separating_axes(b, lb, a, la));
    out[i] = (uint8_t)r;
}

// area_of_intersection sutherland_hodgman.py:151-168 (subject: face of a,
// clipper: face of b)
// `order`: NULL, or a permutation of the pairs (processing order only:
// pairs of equal polygon lengths side by side, so a warp's lanes run the
// same number of clip edges; results stay at their pair's index).
__global__ void k_clip_area(const double* __restrict__ va, const int64_t* __restrict__ fa, int Ka,
                            const double* __restrict__ vb, const int64_t* __restrict__ fb, int Kb,
                            const int64_t* __restrict__ ia, const int64_t* __restrict__ ib, int64_t n,
                            const int* __restrict__ order, double* __restrict__ out, unsigned int* __restrict__ err) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int64_t i = order ? (int64_t)order[t] : t;
    dpt a[CT_MAX_N_VERTEX], b[CT_MAX_N_VERTEX];
    dpt A[CT_CLIP_MAX], B[CT_CLIP_MAX];
    int la = load_poly(va, fa, Ka, ia[i], a);
    int lb = load_poly(vb, fb, Kb, ib[i], b);
    bool of = false;
    out[i] = clip_area_conv(a, la, b, lb, A, B, &of);
    if (of) set_error(err, CT_DEVERR_CLIP);
}

// box_area_of_intersection sutherland_hodgman.py:171-187 (subject: the box)
__global__ void k_box_area(const double4* __restrict__ boxes, const double* __restrict__ vb,
                           const int64_t* __restrict__ fb, int Kb, const int64_t* __restrict__ ibox,
                           const int64_t* __restrict__ iface, int64_t n, const int* __restrict__ order,
                           double* __restrict__ out, unsigned int* __restrict__ err) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int64_t i = order ? (int64_t)order[t] : t;
    double4 q = boxes[ibox[i]];
    dpt a[4] = {mkp(q.x, q.z), mkp(q.y, q.z), mkp(q.y, q.w), mkp(q.x, q.w)};
    dpt b[CT_MAX_N_VERTEX];
    dpt A[CT_CLIP_MAX], B[CT_CLIP_MAX];
    int lb = load_poly(vb, fb, Kb, iface[i], b);
    bool of = false;
    out[i] = clip_area_conv(a, 4, b, lb, A, B, &of);
    if (of) set_error(err, CT_DEVERR_CLIP);
}

// 6-bit class of a pair: the polygon lengths (3 .. 10) of its two faces
// (fa NULL: boxes, length 4)
__global__ void k_pair_keys(const int64_t* __restrict__ fa, int Ka, const int64_t* __restrict__ ia,
                            const int64_t* __restrict__ fb, int Kb, const int64_t* __restrict__ ib, int64_t n,
                            unsigned* __restrict__ key) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int la = fa ? polygon_length(fa + ia[i] * Ka, Ka) : 4;
        int lb = polygon_length(fb + ib[i] * Kb, Kb);
        key[i] = (unsigned)(min(la - 3, 7) * 8 + min(lb - 3, 7));
    }
}

// keep = area > 0 (celltree.py:183, 268) or keep = flag
__global__ void k_keep(const double* __restrict__ area, const uint8_t* __restrict__ flag, int64_t n,
                       int64_t* __restrict__ keep) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keep[i] = area ? (int64_t)(area[i] > 0) : (int64_t)(flag[i] != 0);
}

__global__ void k_compact(const int64_t* __restrict__ keep, const int64_t* __restrict__ pos, int64_t n,
                          const int64_t* __restrict__ ii, const int64_t* __restrict__ jj,
                          const double* __restrict__ vals, int64_t* __restrict__ ii_out, int64_t* __restrict__ jj_out,
                          double* __restrict__ vals_out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !keep[i]) return;
    int64_t p = pos[i];
    ii_out[p] = ii[i];
    jj_out[p] = jj[i];
    if (vals) vals_out[p] = vals[i];
}

// ---------------------------------------------------------------------------
// barycentric weights (barycentric_triangle.py:46-64,
// barycentric_wachspress.py:88-107)
// ---------------------------------------------------------------------------
__global__ void k_barycentric(const double2* __restrict__ pts, const int64_t* __restrict__ fidx, int64_t n,
                              const double* __restrict__ v, const int64_t* __restrict__ faces, int K, int KW,
                              double tol, double* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double* w = out + i * KW;
    for (int k = 0; k < KW; k++) w[k] = 0.0;
    int64_t f = fidx[i];
    if (f == -1) return;
    double2 pp = pts[i];
    dpt p = mkp(pp.x, pp.y);
    const int64_t* face = faces + f * K;
    if (K > 3) {
        dpt poly[CT_MAX_N_VERTEX];
        double ww[CT_MAX_N_VERTEX];
        int len = gather_polygon(v, face, K, poly);
        for (int k = 0; k < K; k++) ww[k] = 0.0;
        wachspress(poly, len, p, ww, K, tol);
        for (int k = 0; k < K; k++) w[k] = ww[k];
    } else {
        double ww[3];
        tri_weights(mkp(v[2 * face[0]], v[2 * face[0] + 1]), mkp(v[2 * face[1]], v[2 * face[1] + 1]),
                    mkp(v[2 * face[2]], v[2 * face[2] + 1]), p, ww);
        w[0] = ww[0];
        w[1] = ww[1];
        w[2] = ww[2];
    }
}

// ---------------------------------------------------------------------------
// node-bound diagnostics (collect_node_bounds query.py:568-622,
// validate_node_bounds 625-663)
// ---------------------------------------------------------------------------
__global__ void k_parents(const int64_t* __restrict__ child, int64_t n_nodes, int64_t* __restrict__ parent) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_nodes) return;
    if (v == 0) parent[0] = -1;
    int64_t c = child[v];
    if (c > v && c + 1 < n_nodes) {
        parent[c] = v;
        parent[c + 1] = v;
    }
}

// A node's bounds are its parent's with one coordinate overwritten (left
// child: max of the parent's dim = Lmax; right child: min = Rmin).  Walking up
// from the node, the first ancestor edge that sets a coordinate wins.
__global__ void k_node_bounds(const int64_t* __restrict__ child, const double* __restrict__ Lmax,
                              const double* __restrict__ Rmin, const uint8_t* __restrict__ dim,
                              const int64_t* __restrict__ parent, int64_t n_nodes, double4 bbox,
                              double4* __restrict__ out) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_nodes) return;
    double b[4] = {bbox.x, bbox.y, bbox.z, bbox.w};
    bool set[4] = {false, false, false, false};
    int64_t u = v;
    int64_t guard = n_nodes;
    while (u > 0 && guard-- > 0) {
        int64_t p = parent[u];
        if (p < 0) break;
        int d = dim[p] ? 1 : 0;
        int side = (u == child[p]) ? 1 : 0;  // left child: side 1 (max), right: side 0 (min)
        int k = d * 2 + side;
        if (!set[k]) {
            b[k] = side ? Lmax[p] : Rmin[p];
            set[k] = true;
        }
        u = p;
    }
    out[v] = make_double4(b[0], b[1], b[2], b[3]);
}

__global__ void k_validate_bounds(const int64_t* __restrict__ child, const int64_t* __restrict__ ptr,
                                  const int64_t* __restrict__ size, const int64_t* __restrict__ bbi,
                                  const double* __restrict__ bb, const double4* __restrict__ nbnd, int64_t n_nodes,
                                  uint8_t* __restrict__ valid) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_nodes) return;
    double4 q = nbnd[v];
    dbox bx;
    bx.xmin = q.x;
    bx.xmax = q.y;
    bx.ymin = q.z;
    bx.ymax = q.w;
    int64_t c = child[v];
    bool ok = true;
    if (c == -1) {
        for (int64_t i = ptr[v]; i < ptr[v] + size[v]; i++) ok = ok && box_contained(load_box(bb + 4 * bbi[i]), bx);
    } else {
        double4 l = nbnd[c], r = nbnd[c + 1];
        dbox lb, rb;
        lb.xmin = l.x;
        lb.xmax = l.y;
        lb.ymin = l.z;
        lb.ymax = l.w;
        rb.xmin = r.x;
        rb.xmax = r.y;
        rb.ymin = r.z;
        rb.ymax = r.w;
        ok = box_contained(lb, bx) && box_contained(rb, bx);
    }
    valid[v] = (uint8_t)ok;
}

// 8-bit work class of a box (kind 0: area with a cell-size margin) or a
// segment (kind 1: length plus a cell size): 4 * log2(work) + 128, clamped.
__global__ void k_work_keys(const double4* __restrict__ q, int64_t n, int kind, float cell,
                            unsigned* __restrict__ key) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double4 v = q[i];
        float w;
        if (kind == 0) {
            float dx = (float)(v.y - v.x), dy = (float)(v.w - v.z);
            w = (fabsf(dx) + cell) * (fabsf(dy) + cell);
        } else {
            float dx = (float)(v.z - v.x), dy = (float)(v.w - v.y);
            w = sqrtf(dx * dx + dy * dy) + cell;
        }
        int k = (w > 0.0f) ? (int)floorf(4.0f * log2f(w)) + 128 : 0;  // NaN -> 0
        key[i] = (unsigned)min(max(k, 0), 255);
    }
}

TreeQ make_q(const ct_tree* t) {
    TreeQ T;
    T.nf = (const float4*)t->nodes_f32;
    T.nd = (const double2*)t->nodes_f64;
    T.poly = (const double2*)t->poly_f64;
    T.plen = t->n_max_vert == 3 || t->n_max_vert == 2 ? nullptr : t->poly_len;
    T.bbi = t->bb_indices;
    T.bb = t->bb_coords;
    T.err = t->error_word;
    T.n_nodes = t->n_nodes;
    T.bbox.xmin = t->bbox[0];
    T.bbox.xmax = t->bbox[1];
    T.bbox.ymin = t->bbox[2];
    T.bbox.ymax = t->bbox[3];
    T.K = t->n_max_vert;
    T.finite = t->bounds_finite != 0;
    const bool box_index = t->node_box && t->leaf_start && t->bb_leaf && T.finite;
    T.bbl = box_index ? (const double4*)t->bb_leaf : nullptr;
    T.nbx = box_index ? (const NodeBox*)t->node_box : nullptr;
    T.lstart = box_index ? t->leaf_start : nullptr;
    T.ox = t->origin[0];
    T.oy = t->origin[1];
    T.bbl32 = (box_index && t->bb_leaf32) ? (const float4*)t->bb_leaf32 : nullptr;
    T.fX = (float)std::max(std::fabs(t->bbox[0] - T.ox), std::fabs(t->bbox[1] - T.ox)) * (1.0f + 0x1p-20f);
    T.fY = (float)std::max(std::fabs(t->bbox[2] - T.oy), std::fabs(t->bbox[3] - T.oy)) * (1.0f + 0x1p-20f);
    T.babs = std::max(std::max(std::fabs(t->bbox[0]), std::fabs(t->bbox[1])),
                      std::max(std::fabs(t->bbox[2]), std::fabs(t->bbox[3])));
    T.mext = 0x1p-37 * std::max(t->bbox[1] - t->bbox[0], t->bbox[3] - t->bbox[2]) + 0x1p-47;
    if (!(T.fX <= 3.0e38f && T.fY <= 3.0e38f && T.babs <= 1.0e300 && T.mext <= 1.0e300)) T.bbl32 = nullptr;
    T.parent = t->node_parent;
    T.polyf = (const float4*)t->poly_f32;
    T.plen32 = t->poly_len32;
    T.S4 = poly32_stride(t->n_max_vert);
    T.dabs = t->abs_eps;
    return T;
}

// ---------------------------------------------------------------------------
// Box index (no upstream counterpart), built once per tree:
//  * bb_leaf: bb_coords in leaf order (the leaf loop reads them in sequence
//    instead of through bb_indices);
//  * leaf_start: for every leaf position the first position of its leaf;
//  * node_box: per node the bounding box of the cells below it (leaves from
//    their cells, then up the parent chain with integer-key atomics; a leaf
//    stops climbing where its box is already covered, since whichever leaf
//    widened that node carries the wider box further up) and its leaf range.
// ---------------------------------------------------------------------------
__global__ void k_bi_leaf_boxes(const int64_t* __restrict__ bbi, const double4* __restrict__ bb, int64_t n,
                                double4* __restrict__ bbl) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
        bbl[p] = bb[bbi[p]];
}

// bb_leaf in the float32 frame, rounded outward (the subtraction of the
// origin rounded outward too): contains the cell's box exactly.
__global__ void k_bi_leaf32(const double4* __restrict__ bbl, int64_t n, double ox, double oy,
                            float4* __restrict__ out) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const double4 b = bbl[p];
        out[p] = make_float4(__double2float_rd(__dsub_rd(b.x, ox)), __double2float_ru(__dsub_ru(b.y, ox)),
                             __double2float_rd(__dsub_rd(b.z, oy)), __double2float_ru(__dsub_ru(b.w, oy)));
    }
}

__global__ void k_bi_parents(const int64_t* __restrict__ child, int64_t nn, int* __restrict__ parent,
                             unsigned long long* __restrict__ keys) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nn) return;
    int64_t c = child[v];
    if (c >= 0 && c + 1 < nn) {
        parent[c] = (int)v;
        parent[c + 1] = (int)v;
    }
    keys[4 * v + 0] = ~0ull;
    keys[4 * v + 1] = 0ull;
    keys[4 * v + 2] = ~0ull;
    keys[4 * v + 3] = 0ull;
}

__global__ void k_bi_leaves(const int64_t* __restrict__ child, const int64_t* __restrict__ ptr,
                            const int64_t* __restrict__ size, int64_t nn, const double4* __restrict__ bbl, int64_t n,
                            const int* __restrict__ parent, unsigned long long* __restrict__ keys,
                            int* __restrict__ lstart, unsigned int* __restrict__ err) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nn || child[v] >= 0) return;
    int64_t p0 = ptr[v], sz = size[v];
    if (p0 < 0 || sz < 0 || p0 + sz > n) {
        set_error(err, CT_DEVERR_CAPACITY);
        return;
    }
    if (sz == 0) return;
    unsigned long long x0 = ~0ull, x1 = 0ull, y0 = ~0ull, y1 = 0ull;
    for (int64_t p = p0; p < p0 + sz; p++) {
        lstart[p] = (int)p0;
        double4 b = bbl[p];
        x0 = min(x0, fkey(b.x));
        x1 = max(x1, fkey(b.y));
        y0 = min(y0, fkey(b.z));
        y1 = max(y1, fkey(b.w));
    }
    int u = (int)v;
    for (int64_t guard = nn; u >= 0 && guard > 0; guard--) {
        unsigned long long* k = keys + 4 * (int64_t)u;
        unsigned long long o0 = atomicMin(k + 0, x0), o1 = atomicMax(k + 1, x1);
        unsigned long long o2 = atomicMin(k + 2, y0), o3 = atomicMax(k + 3, y1);
        if (o0 <= x0 && o1 >= x1 && o2 <= y0 && o3 >= y1) break;
        u = parent[u];
    }
}

__global__ void k_bi_nodes(const int64_t* __restrict__ ptr, const int64_t* __restrict__ size, int64_t nn,
                           const unsigned long long* __restrict__ keys, double ox, double oy,
                           NodeBox* __restrict__ out) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nn) return;
    NodeBox b;
    const unsigned long long* k = keys + 4 * v;
    if (k[0] == ~0ull) {  // no cells: never "inside" a query box
        b.xmin = b.ymin = __int_as_float(0x7fc00000);
        b.xmax = b.ymax = __int_as_float(0x7fc00000);
    } else {
        b.xmin = __double2float_rd(fkey_inv(k[0]) - ox);
        b.xmax = __double2float_ru(fkey_inv(k[1]) - ox);
        b.ymin = __double2float_rd(fkey_inv(k[2]) - oy);
        b.ymax = __double2float_ru(fkey_inv(k[3]) - oy);
    }
    b.ptr = (int)ptr[v];
    b.size = (int)size[v];
    b.pad0 = b.pad1 = 0;
    out[v] = b;
}

static inline unsigned grid_of(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace ctm

using namespace ctm;

extern "C" {

size_t ct_scan_workspace_size(int64_t n) {
    int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    return (size_t)(nb + 1) * sizeof(int64_t);
}

int ct_exclusive_scan(const int64_t* in, int64_t n, int64_t* out, void* ws, size_t ws_bytes, int64_t* total_host,
                      void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n < 0) return ct_fail(CT_ERR_ARG, "negative length");
    if (ws_bytes < ct_scan_workspace_size(n) || !ws) return ct_fail(CT_ERR_WORKSPACE, "scan workspace too small");
    int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    int64_t* sums = (int64_t*)ws;
    if (nb > 0) {
        k_scan_reduce<<<(unsigned)nb, SCAN_T, 0, st>>>(in, n, sums);
        k_scan_sums<<<1, SCAN_T, 0, st>>>(sums, nb);
        k_scan_down<<<(unsigned)nb, SCAN_T, 0, st>>>(in, n, sums, out);
    } else {
        CT_CUDA(cudaMemsetAsync(sums, 0, sizeof(int64_t), st));
    }
    CT_CHECK_LAUNCH("scan");
    if (total_host) {
        CT_CUDA(cudaMemcpyAsync(total_host, sums + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CT_CUDA(cudaStreamSynchronize(st));
    }
    return CT_OK;
}

size_t ct_box_index_scratch_size(const ct_tree* t) {
    if (!t || t->n_nodes <= 0) return 0;
    return (size_t)t->n_nodes * (4 * sizeof(unsigned long long) + sizeof(int)) + 256;
}

int ct_pack_box_index(ct_tree* t, void* scratch, size_t scratch_bytes, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!t) return ct_fail(CT_ERR_ARG, "tree is null");
    if (!t->bb_leaf || !t->node_box || !t->leaf_start) return ct_fail(CT_ERR_ARG, "box index arrays not set");
    if (t->n_nodes <= 0 || t->n_nodes >= INT32_MAX || t->n_elements >= INT32_MAX)
        return ct_fail(CT_ERR_ARG, "tree size out of range");
    if (!scratch || scratch_bytes < ct_box_index_scratch_size(t))
        return ct_fail(CT_ERR_WORKSPACE, "box index scratch too small");
    int64_t nn = t->n_nodes, n = t->n_elements;
    unsigned long long* keys = (unsigned long long*)scratch;
    int* parent = (int*)(keys + 4 * nn);
    CT_CUDA(cudaMemsetAsync(parent, 0xff, (size_t)nn * sizeof(int), st));
    if (n > 0) {
        k_bi_leaf_boxes<<<(unsigned)std::min<int64_t>(grid_of(n, 256), 152 * 8), 256, 0, st>>>(
            t->bb_indices, (const double4*)t->bb_coords, n, (double4*)t->bb_leaf);
        if (t->bb_leaf32)
            k_bi_leaf32<<<(unsigned)std::min<int64_t>(grid_of(n, 256), 152 * 8), 256, 0, st>>>(
                (const double4*)t->bb_leaf, n, t->origin[0], t->origin[1], (float4*)t->bb_leaf32);
    }
    k_bi_parents<<<grid_of(nn, 256), 256, 0, st>>>(t->node_child, nn, parent, keys);
    k_bi_leaves<<<grid_of(nn, 128), 128, 0, st>>>(t->node_child, t->node_ptr, t->node_size, nn,
                                                  (const double4*)t->bb_leaf, n, parent, keys, t->leaf_start,
                                                  t->error_word);
    k_bi_nodes<<<grid_of(nn, 256), 256, 0, st>>>(t->node_ptr, t->node_size, nn, keys, t->origin[0], t->origin[1],
                                                 (NodeBox*)t->node_box);
    CT_CHECK_LAUNCH("pack_box_index");
    return CT_OK;
}

// block sizes of the traversal kernels (the tree's launch shape, else the defaults)
static int box_threads(const ct_tree* t) {
    int b = t->tune_query_threads;
    return (b == 64 || b == 128 || b == 256) ? b : 256;
}
static int seg_threads(const ct_tree* t) {
    int b = t->tune_query_threads;
    return (b == 64 || b == 128) ? b : 128;
}

static int check_tree(const ct_tree* t) {
    if (!t) return ct_fail(CT_ERR_ARG, "tree is null");
    if (t->n_nodes <= 0) return ct_fail(CT_ERR_ARG, "tree has no nodes");
    if (t->max_depth + 2 > STK && !t->node_parent)
        return ct_fail(CT_ERR_ARG, "tree deeper than 126 levels for multi-result queries (no node_parent)");
    return CT_OK;
}

// trees deeper than the traversal stack are walked through the node parents
static bool deep_tree(const ct_tree* t) { return t->max_depth + 2 > STK; }

int ct_count_boxes(const ct_tree* t, const double* boxes, int64_t n, const int32_t* order, int64_t* counts,
                   void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n == 0) return CT_OK;
    const int bt = box_threads(t);
    if (deep_tree(t))
        k_boxes<false, true><<<grid_of(n, bt), bt, 0, (cudaStream_t)stream>>>(make_q(t), (const double4*)boxes, n,
                                                                              order, counts, nullptr, nullptr);
    else
        k_boxes<false, false><<<grid_of(n, bt), bt, 0, (cudaStream_t)stream>>>(make_q(t), (const double4*)boxes, n,
                                                                               order, counts, nullptr, nullptr);
    CT_CHECK_LAUNCH("count_boxes");
    return CT_OK;
}

int ct_write_boxes(const ct_tree* t, const double* boxes, int64_t n, const int32_t* order, const int64_t* offsets,
                   int64_t* ii, int64_t* jj, void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n == 0) return CT_OK;
    const int bt = box_threads(t);
    if (deep_tree(t))
        k_boxes<true, true><<<grid_of(n, bt), bt, 0, (cudaStream_t)stream>>>(make_q(t), (const double4*)boxes, n,
                                                                             order, (int64_t*)offsets, ii, jj);
    else
        k_boxes<true, false><<<grid_of(n, bt), bt, 0, (cudaStream_t)stream>>>(make_q(t), (const double4*)boxes, n,
                                                                              order, (int64_t*)offsets, ii, jj);
    CT_CHECK_LAUNCH("write_boxes");
    return CT_OK;
}

static int box_job_min(int32_t m) { return m > 0 ? (m < 2 ? 2 : m) : BOX_JOB_MIN; }

size_t ct_write_boxes_workspace_size(int64_t total_pairs, int32_t min_job_cells) {
    const int64_t cap = (total_pairs > 0 ? total_pairs : 0) / box_job_min(min_job_cells) + 1;
    return 256 + (size_t)cap * sizeof(BoxJob);
}

int ct_write_boxes_ws(const ct_tree* t, const double* boxes, int64_t n, const int32_t* order,
                      const int64_t* offsets, int64_t total_pairs, int32_t min_job_cells, int64_t* ii, int64_t* jj,
                      void* ws, size_t ws_bytes, void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n == 0) return CT_OK;
    if (total_pairs < 0) return ct_fail(CT_ERR_ARG, "negative pair count");
    if (!ws || ws_bytes < ct_write_boxes_workspace_size(total_pairs, min_job_cells))
        return ct_fail(CT_ERR_WORKSPACE, "write_boxes workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    TreeQ T = make_q(t);
    if (!T.nbx) return ct_write_boxes(t, boxes, n, order, offsets, ii, jj, stream);  // no box index: no subtrees
    const int jm = box_job_min(min_job_cells);
    unsigned long long* njobs = (unsigned long long*)ws;
    BoxJob* jobs = (BoxJob*)((char*)ws + 256);
    const int64_t cap = (total_pairs > 0 ? total_pairs : 0) / jm + 1;
    CT_CUDA(cudaMemsetAsync(njobs, 0, sizeof(unsigned long long), st));
    const int bt = box_threads(t);
    if (deep_tree(t))
        k_boxes<true, true><<<grid_of(n, bt), bt, 0, st>>>(T, (const double4*)boxes, n, order, (int64_t*)offsets,
                                                           ii, jj, jobs, njobs, cap, jm);
    else
        k_boxes<true, false><<<grid_of(n, bt), bt, 0, st>>>(T, (const double4*)boxes, n, order, (int64_t*)offsets,
                                                            ii, jj, jobs, njobs, cap, jm);
    k_box_jobs<<<152 * 8, 256, 0, st>>>(jobs, njobs, cap, T.lstart, T.bbi, ii, jj, T.err);
    CT_CHECK_LAUNCH("write_boxes");
    return CT_OK;
}

int ct_count_boxes_spec(const ct_tree* t, const double* boxes, int64_t n, const int32_t* order, int64_t* counts,
                        int32_t* spec, int32_t spec_cap, void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n == 0) return CT_OK;
    if (!spec || spec_cap < 1 || spec_cap > 4096) return ct_fail(CT_ERR_ARG, "spec_cap must be in [1, 4096]");
    if (t->n_elements >= INT32_MAX) return ct_fail(CT_ERR_ARG, "tree size out of range");
    const int bt = box_threads(t);
    cudaStream_t st = (cudaStream_t)stream;
    const TreeQ T = make_q(t);
    const double4* B = (const double4*)boxes;
    if (deep_tree(t))
        k_boxes<false, true><<<grid_of(n, bt), bt, 0, st>>>(T, B, n, order, counts, nullptr, nullptr, nullptr, nullptr,
                                                            0, BOX_JOB_MIN, spec, spec_cap, nullptr);
    else
        k_boxes<false, false><<<grid_of(n, bt), bt, 0, st>>>(T, B, n, order, counts, nullptr, nullptr, nullptr,
                                                             nullptr, 0, BOX_JOB_MIN, spec, spec_cap, nullptr);
    CT_CHECK_LAUNCH("count_boxes_spec");
    return CT_OK;
}

int ct_write_boxes_spec(const ct_tree* t, const double* boxes, int64_t n, const int32_t* order,
                        const int64_t* counts, const int64_t* offsets, const int32_t* spec, int32_t spec_cap,
                        int64_t total_pairs, int32_t min_job_cells, int64_t* ii, int64_t* jj, void* ws,
                        size_t ws_bytes, void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n == 0) return CT_OK;
    if (!spec || spec_cap < 1 || spec_cap > 4096) return ct_fail(CT_ERR_ARG, "spec_cap must be in [1, 4096]");
    if (total_pairs < 0) return ct_fail(CT_ERR_ARG, "negative pair count");
    if (!ws || ws_bytes < ct_write_boxes_workspace_size(total_pairs, min_job_cells))
        return ct_fail(CT_ERR_WORKSPACE, "write_boxes workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    const TreeQ T = make_q(t);
    k_boxes_spec_emit<<<(unsigned)std::min<int64_t>(grid_of(n * (int64_t)spec_cap, 256), 152 * 16), 256, 0, st>>>(
        counts, offsets, n, spec, spec_cap, ii, jj);
    const int jm = box_job_min(min_job_cells);
    unsigned long long* njobs = (unsigned long long*)ws;
    BoxJob* jobs = T.nbx ? (BoxJob*)((char*)ws + 256) : nullptr;
    const int64_t cap = (total_pairs > 0 ? total_pairs : 0) / jm + 1;
    CT_CUDA(cudaMemsetAsync(njobs, 0, sizeof(unsigned long long), st));
    const int bt = box_threads(t);
    const double4* B = (const double4*)boxes;
    int64_t* off = (int64_t*)offsets;
    if (deep_tree(t))
        k_boxes<true, true><<<grid_of(n, bt), bt, 0, st>>>(T, B, n, order, off, ii, jj, jobs, njobs, cap, jm,
                                                           nullptr, spec_cap, counts);
    else
        k_boxes<true, false><<<grid_of(n, bt), bt, 0, st>>>(T, B, n, order, off, ii, jj, jobs, njobs, cap, jm,
                                                            nullptr, spec_cap, counts);
    if (jobs) k_box_jobs<<<152 * 8, 256, 0, st>>>(jobs, njobs, cap, T.lstart, T.bbi, ii, jj, T.err);
    CT_CHECK_LAUNCH("write_boxes_spec");
    return CT_OK;
}

size_t ct_sort_workspace_size(int64_t total) {
    const size_t t = (size_t)(total > 0 ? total : 1);
    return t * 4 * 8 + (t / (WARP_SORT_MAX + 1) + 2) * sizeof(int) + 1024 + 256;
}

int ct_sort_intersections(const double* segs, int64_t n_segs, const int64_t* offsets, const int64_t* counts,
                          const int64_t* ii, const int64_t* jj_in, const double* xy_in, int64_t total,
                          int64_t* jj_out, double* xy_out, void* ws, size_t ws_bytes, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (total == 0) return CT_OK;
    if (!ws || ws_bytes < ct_sort_workspace_size(total)) return ct_fail(CT_ERR_WORKSPACE, "sort workspace too small");
    unsigned long long* kA = (unsigned long long*)ws;
    int64_t* iA = (int64_t*)(kA + total);
    unsigned long long* kB = (unsigned long long*)(iA + total);
    int64_t* iB = (int64_t*)(kB + total);
    unsigned long long* nlist = (unsigned long long*)(iB + total);  // 8 B, then the list of long segments
    int* list = (int*)(nlist + 1);
    if (n_segs > INT32_MAX) return ct_fail(CT_ERR_ARG, "at most 2^31 - 1 segments");
    CT_CUDA(cudaMemsetAsync(nlist, 0, sizeof(unsigned long long), st));
    k_tkeys<<<grid_of(total, 256), 256, 0, st>>>((const double4*)segs, ii, (const double4*)xy_in, total, kA, iA);
    k_segsort_warp<<<(unsigned)std::min<int64_t>(grid_of(n_segs * 32, 256), 152 * 32), 256, 0, st>>>(
        offsets, counts, n_segs, kA, iA, iB, list, nlist);
    k_segsort<<<152 * 4, SORT_T, 0, st>>>(offsets, counts, list, nlist, kA, iA, kB, iB, iB);
    // iB now holds, per segment, the sorted source positions (segments of one
    // result write them directly)
    k_gather_results<<<grid_of(total, 256), 256, 0, st>>>(iB, total, jj_in, (const double4*)xy_in, jj_out,
                                                          (double4*)xy_out);
    CT_CHECK_LAUNCH("sort_intersections");
    return CT_OK;
}

int ct_polygons_intersect(const double* va, const int64_t* fa, int32_t Ka, const double* vb, const int64_t* fb,
                          int32_t Kb, const int64_t* ia, const int64_t* ib, int64_t n, uint8_t* out, void* stream) {
    if (n == 0) return CT_OK;
    k_sat<<<grid_of(n, 128), 128, 0, (cudaStream_t)stream>>>(va, fa, Ka, vb, fb, Kb, ia, ib, n, out);
    CT_CHECK_LAUNCH("polygons_intersect");
    return CT_OK;
}

int ct_area_of_intersection_ordered(const double* va, const int64_t* fa, int32_t Ka, const double* vb,
                                    const int64_t* fb, int32_t Kb, const int64_t* ia, const int64_t* ib, int64_t n,
                                    const int32_t* order, double* out, unsigned int* error_word, void* stream) {
    if (n == 0) return CT_OK;
    k_clip_area<<<grid_of(n, 128), 128, 0, (cudaStream_t)stream>>>(va, fa, Ka, vb, fb, Kb, ia, ib, n, order, out,
                                                                    error_word);
    CT_CHECK_LAUNCH("area_of_intersection");
    return CT_OK;
}

int ct_area_of_intersection(const double* va, const int64_t* fa, int32_t Ka, const double* vb, const int64_t* fb,
                            int32_t Kb, const int64_t* ia, const int64_t* ib, int64_t n, double* out,
                            unsigned int* error_word, void* stream) {
    return ct_area_of_intersection_ordered(va, fa, Ka, vb, fb, Kb, ia, ib, n, nullptr, out, error_word, stream);
}

int ct_box_area_of_intersection_ordered(const double* boxes, const double* vb, const int64_t* fb, int32_t Kb,
                                        const int64_t* ibox, const int64_t* iface, int64_t n, const int32_t* order,
                                        double* out, unsigned int* error_word, void* stream) {
    if (n == 0) return CT_OK;
    k_box_area<<<grid_of(n, 128), 128, 0, (cudaStream_t)stream>>>((const double4*)boxes, vb, fb, Kb, ibox, iface, n,
                                                                   order, out, error_word);
    CT_CHECK_LAUNCH("box_area_of_intersection");
    return CT_OK;
}

int ct_box_area_of_intersection(const double* boxes, const double* vb, const int64_t* fb, int32_t Kb,
                                const int64_t* ibox, const int64_t* iface, int64_t n, double* out,
                                unsigned int* error_word, void* stream) {
    return ct_box_area_of_intersection_ordered(boxes, vb, fb, Kb, ibox, iface, n, nullptr, out, error_word, stream);
}

size_t ct_pair_order_workspace_size(int64_t n) {
    size_t part = ((size_t)(n > 0 ? n : 1) * sizeof(unsigned) + 255) / 256 * 256;
    return 2 * part + ct_radix_pass_workspace_size();
}

int ct_pair_order(const int64_t* fa, int32_t Ka, const int64_t* ia, const int64_t* fb, int32_t Kb, const int64_t* ib,
                  int64_t n, int32_t* order, void* ws, size_t ws_bytes, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n < 0 || n > INT32_MAX) return ct_fail(CT_ERR_ARG, "pair count out of range");
    if (!ws || ws_bytes < ct_pair_order_workspace_size(n)) return ct_fail(CT_ERR_WORKSPACE, "pair order workspace");
    if (n == 0) return CT_OK;
    size_t part = ((size_t)n * sizeof(unsigned) + 255) / 256 * 256;
    unsigned* kin = (unsigned*)ws;
    unsigned* kout = (unsigned*)((char*)ws + part);
    k_pair_keys<<<(unsigned)std::min<int64_t>(grid_of(n, 256), 152 * 8), 256, 0, st>>>(fa, Ka, ia, fb, Kb, ib, n, kin);
    CT_CHECK_LAUNCH("pair keys");
    return ct_radix_pass(kin, nullptr, n, 0, kout, order, (char*)ws + 2 * part, ws_bytes - 2 * part, stream);
}

int ct_compact_pairs(const double* area, const uint8_t* flag, int64_t n, const int64_t* ii, const int64_t* jj,
                     int64_t* ii_out, int64_t* jj_out, double* area_out, void* ws, size_t ws_bytes,
                     int64_t* total_host, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n == 0) {
        if (total_host) *total_host = 0;
        return CT_OK;
    }
    size_t scan_ws = ct_scan_workspace_size(n);
    if (!ws || ws_bytes < scan_ws + 2 * (size_t)n * sizeof(int64_t))
        return ct_fail(CT_ERR_WORKSPACE, "compaction workspace too small");
    int64_t* keep = (int64_t*)ws;
    int64_t* pos = keep + n;
    void* sws = pos + n;
    k_keep<<<grid_of(n, 256), 256, 0, st>>>(area, flag, n, keep);
    int s = ct_exclusive_scan(keep, n, pos, sws, scan_ws, total_host, stream);
    if (s) return s;
    k_compact<<<grid_of(n, 256), 256, 0, st>>>(keep, pos, n, ii, jj, area, ii_out, jj_out, area_out);
    CT_CHECK_LAUNCH("compact");
    return CT_OK;
}

size_t ct_compact_workspace_size(int64_t n) {
    return ct_scan_workspace_size(n) + 2 * (size_t)(n > 0 ? n : 1) * sizeof(int64_t);
}

int ct_barycentric_weights(const ct_tree* t, const double* points, const int64_t* face_indices, int64_t n,
                           double tolerance, double* weights, void* stream) {
    if (!t) return ct_fail(CT_ERR_ARG, "tree is null");
    if (n == 0) return CT_OK;
    int K = t->n_max_vert;
    int KW = K > 3 ? K : 3;
    k_barycentric<<<grid_of(n, 128), 128, 0, (cudaStream_t)stream>>>((const double2*)points, face_indices, n,
                                                                      t->vertices, t->elements, K, KW, tolerance,
                                                                      weights);
    CT_CHECK_LAUNCH("barycentric");
    return CT_OK;
}

int ct_node_bounds(const int64_t* child, const double* Lmax, const double* Rmin, const uint8_t* dim, int64_t n_nodes,
                   const double* bbox_host4, int64_t* parent_ws, double* out, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n_nodes <= 0) return CT_OK;
    CT_CUDA(cudaMemsetAsync(parent_ws, 0xff, sizeof(int64_t) * n_nodes, st));
    k_parents<<<grid_of(n_nodes, 256), 256, 0, st>>>(child, n_nodes, parent_ws);
    double4 b = make_double4(bbox_host4[0], bbox_host4[1], bbox_host4[2], bbox_host4[3]);
    k_node_bounds<<<grid_of(n_nodes, 256), 256, 0, st>>>(child, Lmax, Rmin, dim, parent_ws, n_nodes, b,
                                                          (double4*)out);
    CT_CHECK_LAUNCH("node_bounds");
    return CT_OK;
}

int ct_validate_node_bounds(const int64_t* child, const int64_t* ptr, const int64_t* size, int64_t n_nodes,
                            const int64_t* bb_indices, const double* bb_coords, const double* node_bounds,
                            uint8_t* valid, void* stream) {
    if (n_nodes <= 0) return CT_OK;
    k_validate_bounds<<<grid_of(n_nodes, 256), 256, 0, (cudaStream_t)stream>>>(
        child, ptr, size, bb_indices, bb_coords, (const double4*)node_bounds, n_nodes, valid);
    CT_CHECK_LAUNCH("validate_node_bounds");
    return CT_OK;
}

size_t ct_work_order_workspace_size(int64_t n) {
    size_t nn = (size_t)(n > 0 ? n : 1);
    return 2 * ((4 * nn + 255) / 256 * 256) + ct_radix_pass_workspace_size();
}

int ct_work_order(const double* queries, int64_t n, int32_t kind, double cell_size, int32_t* order, void* ws,
                  size_t ws_bytes, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n < 0 || (kind != 0 && kind != 1)) return ct_fail(CT_ERR_ARG, "bad work-order arguments");
    if (!ws || ws_bytes < ct_work_order_workspace_size(n)) return ct_fail(CT_ERR_WORKSPACE, "workspace too small");
    if (n == 0) return CT_OK;
    size_t part = (4 * (size_t)n + 255) / 256 * 256;
    unsigned* kin = (unsigned*)ws;
    unsigned* kout = (unsigned*)((char*)ws + part);
    unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16);
    k_work_keys<<<blocks, 256, 0, st>>>((const double4*)queries, n, kind, (float)cell_size, kin);
    CT_CHECK_LAUNCH("work keys");
    return ct_radix_pass(kin, nullptr, n, 0, kout, order, (char*)ws + 2 * part, ws_bytes - 2 * part, stream);
}

int ct_count_edge_candidates(const ct_tree* t, int32_t mode, const double* segs, int64_t n, const int32_t* order,
                              int64_t* counts, void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n == 0) return CT_OK;
    if (mode == 0 && t->n_max_vert != 2) return ct_fail(CT_ERR_ARG, "edge-edge mode needs an edge tree");
    cudaStream_t st = (cudaStream_t)stream;
    TreeQ T = make_q(t);
    const int et = seg_threads(t);
    const double4* S = (const double4*)segs;
    const unsigned g = grid_of(n, et);
    if (deep_tree(t)) {
        if (mode == 0) k_edge_cands<false, 0, true><<<g, et, 0, st>>>(T, S, n, order, counts, 0, 0);
        else k_edge_cands<false, 1, true><<<g, et, 0, st>>>(T, S, n, order, counts, 0, 0);
    } else {
        if (mode == 0) k_edge_cands<false, 0, false><<<g, et, 0, st>>>(T, S, n, order, counts, 0, 0);
        else k_edge_cands<false, 1, false><<<g, et, 0, st>>>(T, S, n, order, counts, 0, 0);
    }
    CT_CHECK_LAUNCH("count_edge_candidates");
    return CT_OK;
}

int ct_write_edge_candidates(const ct_tree* t, int32_t mode, const double* segs, int64_t n, const int32_t* order,
                              const int64_t* offsets, int32_t* cand_seg, int32_t* cand_pos, void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n == 0) return CT_OK;
    if (n > INT32_MAX) return ct_fail(CT_ERR_ARG, "at most 2^31 - 1 segments");
    cudaStream_t st = (cudaStream_t)stream;
    TreeQ T = make_q(t);
    const int et = seg_threads(t);
    const double4* S = (const double4*)segs;
    const unsigned g = grid_of(n, et);
    int64_t* off = (int64_t*)offsets;
    if (deep_tree(t)) {
        if (mode == 0) k_edge_cands<true, 0, true><<<g, et, 0, st>>>(T, S, n, order, off, cand_seg, cand_pos);
        else k_edge_cands<true, 1, true><<<g, et, 0, st>>>(T, S, n, order, off, cand_seg, cand_pos);
    } else {
        if (mode == 0) k_edge_cands<true, 0, false><<<g, et, 0, st>>>(T, S, n, order, off, cand_seg, cand_pos);
        else k_edge_cands<true, 1, false><<<g, et, 0, st>>>(T, S, n, order, off, cand_seg, cand_pos);
    }
    CT_CHECK_LAUNCH("write_edge_candidates");
    return CT_OK;
}

static int check_split(const ct_tree* t, int32_t mode, int32_t cut) {
    int s = check_tree(t);
    if (s) return s;
    if (mode != 0 && mode != 1) return ct_fail(CT_ERR_ARG, "mode must be 0 or 1");
    if (mode == 0 && t->n_max_vert != 2) return ct_fail(CT_ERR_ARG, "edge-edge mode needs an edge tree");
    if (cut < 0 || cut > 64) return ct_fail(CT_ERR_ARG, "cut depth must be in [0, 64]");
    if (deep_tree(t)) return ct_fail(CT_ERR_ARG, "tree too deep for the split traversal");
    return CT_OK;
}

int ct_count_edge_items(const ct_tree* t, int32_t mode, const double* segs, int64_t n, const int32_t* order,
                        int32_t cut, int64_t* counts, void* stream) {
    int s = check_split(t, mode, cut);
    if (s) return s;
    if (n == 0) return CT_OK;
    cudaStream_t st = (cudaStream_t)stream;
    TreeQ T = make_q(t);
    const int et = seg_threads(t);
    const unsigned g = grid_of(n, et);
    const double4* S = (const double4*)segs;
    if (mode == 0) k_edge_items<false, 0><<<g, et, 0, st>>>(T, S, n, order, cut, counts, 0, 0);
    else k_edge_items<false, 1><<<g, et, 0, st>>>(T, S, n, order, cut, counts, 0, 0);
    CT_CHECK_LAUNCH("count_edge_items");
    return CT_OK;
}

int ct_write_edge_items(const ct_tree* t, int32_t mode, const double* segs, int64_t n, const int32_t* order,
                        int32_t cut, const int64_t* offsets, int32_t* item_seg, int32_t* item_node, void* stream) {
    int s = check_split(t, mode, cut);
    if (s) return s;
    if (n == 0) return CT_OK;
    if (n > INT32_MAX) return ct_fail(CT_ERR_ARG, "at most 2^31 - 1 segments");
    cudaStream_t st = (cudaStream_t)stream;
    TreeQ T = make_q(t);
    const int et = seg_threads(t);
    const unsigned g = grid_of(n, et);
    const double4* S = (const double4*)segs;
    int64_t* off = (int64_t*)offsets;
    if (mode == 0) k_edge_items<true, 0><<<g, et, 0, st>>>(T, S, n, order, cut, off, item_seg, item_node);
    else k_edge_items<true, 1><<<g, et, 0, st>>>(T, S, n, order, cut, off, item_seg, item_node);
    CT_CHECK_LAUNCH("write_edge_items");
    return CT_OK;
}

int ct_count_item_candidates(const ct_tree* t, int32_t mode, const double* segs, const int32_t* item_seg,
                             const int32_t* item_node, int64_t n_items, int64_t* counts, void* stream) {
    int s = check_split(t, mode, 0);
    if (s) return s;
    if (n_items == 0) return CT_OK;
    cudaStream_t st = (cudaStream_t)stream;
    TreeQ T = make_q(t);
    const int et = seg_threads(t);
    const unsigned g = grid_of(n_items, et);
    const double4* S = (const double4*)segs;
    if (mode == 0) k_item_cands<false, 0><<<g, et, 0, st>>>(T, S, item_seg, item_node, n_items, counts, 0, 0);
    else k_item_cands<false, 1><<<g, et, 0, st>>>(T, S, item_seg, item_node, n_items, counts, 0, 0);
    CT_CHECK_LAUNCH("count_item_candidates");
    return CT_OK;
}

int ct_write_item_candidates(const ct_tree* t, int32_t mode, const double* segs, const int32_t* item_seg,
                             const int32_t* item_node, int64_t n_items, const int64_t* offsets, int32_t* cand_seg,
                             int32_t* cand_pos, void* stream) {
    int s = check_split(t, mode, 0);
    if (s) return s;
    if (n_items == 0) return CT_OK;
    cudaStream_t st = (cudaStream_t)stream;
    TreeQ T = make_q(t);
    const int et = seg_threads(t);
    const unsigned g = grid_of(n_items, et);
    const double4* S = (const double4*)segs;
    int64_t* off = (int64_t*)offsets;
    if (mode == 0)
        k_item_cands<true, 0><<<g, et, 0, st>>>(T, S, item_seg, item_node, n_items, off, cand_seg, cand_pos);
    else
        k_item_cands<true, 1><<<g, et, 0, st>>>(T, S, item_seg, item_node, n_items, off, cand_seg, cand_pos);
    CT_CHECK_LAUNCH("write_item_candidates");
    return CT_OK;
}

int ct_segment_candidate_ranges(const int64_t* item_off, const int64_t* item_cnt, int64_t n,
                                const int64_t* item_cand_off, const int64_t* item_cand_cnt, int64_t n_items,
                                int64_t* cand_off, int64_t* cand_cnt, void* stream) {
    if (n < 0 || n_items < 0) return ct_fail(CT_ERR_ARG, "negative count");
    if (n == 0) return CT_OK;
    cudaStream_t st = (cudaStream_t)stream;
    k_seg_from_items<<<(unsigned)std::min<int64_t>(grid_of(n, 256), 152 * 32), 256, 0, st>>>(
        item_off, item_cnt, n, item_cand_off, item_cand_cnt, n_items, cand_off, cand_cnt);
    CT_CHECK_LAUNCH("segment_candidate_ranges");
    return CT_OK;
}

int ct_count_edge_candidates_spec(const ct_tree* t, int32_t mode, const double* segs, int64_t n,
                                  const int32_t* order, int64_t* counts, int32_t* spec, int32_t spec_cap,
                                  void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n == 0) return CT_OK;
    if (mode != 0 && mode != 1) return ct_fail(CT_ERR_ARG, "mode must be 0 or 1");
    if (mode == 0 && t->n_max_vert != 2) return ct_fail(CT_ERR_ARG, "edge-edge mode needs an edge tree");
    if (!spec || spec_cap < 1 || spec_cap > 4096) return ct_fail(CT_ERR_ARG, "spec_cap must be in [1, 4096]");
    cudaStream_t st = (cudaStream_t)stream;
    TreeQ T = make_q(t);
    const int et = seg_threads(t);
    const double4* S = (const double4*)segs;
    const unsigned g = grid_of(n, et);
    if (deep_tree(t)) {
        if (mode == 0) k_edge_cands<false, 0, true><<<g, et, 0, st>>>(T, S, n, order, counts, 0, spec, spec_cap);
        else k_edge_cands<false, 1, true><<<g, et, 0, st>>>(T, S, n, order, counts, 0, spec, spec_cap);
    } else {
        if (mode == 0) k_edge_cands<false, 0, false><<<g, et, 0, st>>>(T, S, n, order, counts, 0, spec, spec_cap);
        else k_edge_cands<false, 1, false><<<g, et, 0, st>>>(T, S, n, order, counts, 0, spec, spec_cap);
    }
    CT_CHECK_LAUNCH("count_edge_candidates_spec");
    return CT_OK;
}

int ct_write_edge_candidates_spec(const ct_tree* t, int32_t mode, const double* segs, int64_t n,
                                  const int32_t* order, const int64_t* counts, const int64_t* offsets,
                                  const int32_t* spec, int32_t spec_cap, int32_t* cand_seg, int32_t* cand_pos,
                                  void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n == 0) return CT_OK;
    if (n > INT32_MAX) return ct_fail(CT_ERR_ARG, "at most 2^31 - 1 segments");
    if (mode != 0 && mode != 1) return ct_fail(CT_ERR_ARG, "mode must be 0 or 1");
    if (!spec || spec_cap < 1 || spec_cap > 4096) return ct_fail(CT_ERR_ARG, "spec_cap must be in [1, 4096]");
    cudaStream_t st = (cudaStream_t)stream;
    TreeQ T = make_q(t);
    k_edge_spec_emit<<<(unsigned)std::min<int64_t>(grid_of(n * (int64_t)spec_cap, 256), 152 * 16), 256, 0, st>>>(
        counts, offsets, n, spec, spec_cap, cand_seg, cand_pos);
    const int et = seg_threads(t);
    const double4* S = (const double4*)segs;
    const unsigned g = grid_of(n, et);
    int64_t* off = (int64_t*)offsets;
    if (deep_tree(t)) {
        if (mode == 0)
            k_edge_cands<true, 0, true><<<g, et, 0, st>>>(T, S, n, order, off, cand_seg, cand_pos, spec_cap, counts);
        else
            k_edge_cands<true, 1, true><<<g, et, 0, st>>>(T, S, n, order, off, cand_seg, cand_pos, spec_cap, counts);
    } else {
        if (mode == 0)
            k_edge_cands<true, 0, false><<<g, et, 0, st>>>(T, S, n, order, off, cand_seg, cand_pos, spec_cap, counts);
        else
            k_edge_cands<true, 1, false><<<g, et, 0, st>>>(T, S, n, order, off, cand_seg, cand_pos, spec_cap, counts);
    }
    CT_CHECK_LAUNCH("write_edge_candidates_spec");
    return CT_OK;
}

int ct_cs_certificates(const ct_tree* t, const double* segs, const int32_t* cand_seg, const int32_t* cand_pos,
                       int64_t n_cand, int8_t* out, void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n_cand == 0) return CT_OK;
    cudaStream_t st = (cudaStream_t)stream;
    k_cs_certificates<<<(unsigned)std::min<int64_t>(grid_of(n_cand, 128), 152 * 64), 128, 0, st>>>(
        make_q(t), (const double4*)segs, cand_seg, cand_pos, n_cand, out);
    CT_CHECK_LAUNCH("cs_certificates");
    return CT_OK;
}

int ct_test_edge_candidates(const ct_tree* t, int32_t mode, const double* segs, const int32_t* cand_seg,
                            const int32_t* cand_pos, int64_t n_cand, int64_t* keep, double* xy, void* stream) {
    int s = check_tree(t);
    if (s) return s;
    if (n_cand == 0) return CT_OK;
    cudaStream_t st = (cudaStream_t)stream;
    TreeQ T = make_q(t);
    unsigned g = (unsigned)std::min<int64_t>(grid_of(n_cand, 128), 152 * 64);
    if (mode == 0)
        k_edge_test<0><<<g, 128, 0, st>>>(T, (const double4*)segs, cand_seg, cand_pos, n_cand, keep, (double4*)xy);
    else
        k_edge_test<1><<<g, 128, 0, st>>>(T, (const double4*)segs, cand_seg, cand_pos, n_cand, keep, (double4*)xy);
    CT_CHECK_LAUNCH("test_edge_candidates");
    return CT_OK;
}

int ct_compact_edge_hits(const ct_tree* t, const int64_t* keep, const int64_t* pos, int64_t n_cand,
                         const int32_t* cand_seg, const int32_t* cand_pos, const double* xy_cand,
                         const int64_t* cand_off, const int64_t* cand_cnt, int64_t n, int64_t* ii, int64_t* jj,
                         double* xy, int64_t* offsets, int64_t* counts, void* stream) {
    if (!t) return ct_fail(CT_ERR_ARG, "tree is null");
    cudaStream_t st = (cudaStream_t)stream;
    if (n_cand > 0)
        k_edge_compact<<<(unsigned)std::min<int64_t>(grid_of(n_cand, 256), 152 * 32), 256, 0, st>>>(
            keep, pos, n_cand, cand_seg, cand_pos, t->bb_indices, (const double4*)xy_cand, ii, jj, (double4*)xy);
    if (n > 0)
        k_edge_seg_counts<<<(unsigned)std::min<int64_t>(grid_of(n, 256), 152 * 32), 256, 0, st>>>(
            cand_off, cand_cnt, keep, pos, n_cand, n, offsets, counts);
    CT_CHECK_LAUNCH("compact_edge_hits");
    return CT_OK;
}

}  // extern "C"
