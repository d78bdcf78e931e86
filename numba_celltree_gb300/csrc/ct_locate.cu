// ct_locate.cu -- the batched point-location pipeline (locate_points
// query.py:63-117), float32 form, for one tree or a batch of trees.
//
//   1. order    queries are sorted along a Morton curve over the tree bbox
//               (LSD radix sort with 8-bit digits: per-block shared-memory
//               histograms, one scan, shared-memory-staged scatter), so
//               neighbouring threads take nearly the same paths;
//   2a. cells   per query the candidate list of its grid cell (cells whose
//               widened bbox meets the grid cell): a float32 bbox reject,
//               then the float32 leaf filter in each cell's local frame.
//               One sure hit and sure misses elsewhere, or sure misses only,
//               is final; anything else leaves the query open;
//   2b. fast    open queries: float32 traversal from the start-node grid
//               (bounds inside their error band re-decided out of line in
//               float64).  A polygon the filter cannot decide (UNSURE)
//               becomes a candidate and the traversal continues, in upstream
//               order, until a polygon is surely hit or it ends.  Queries
//               without candidates are final; the others get a record and a
//               dense (record, ordinal, polygon) list of candidates;
//   3. pip      the exact float64 point_in_polygon_or_on_edge of every
//               candidate pair, one pair per thread (full warps); a true
//               result lowers the record's first-true ordinal;
//   4. resolve  per record: the first candidate whose exact test is true,
//               else the surely-hit cell of the fast pass, else -1 -- which is
//               exactly upstream's first hit, since node decisions do not
//               depend on polygon results;
//   5. exact    queries with more than CMAX candidates (or beyond the record
//               capacity) run the float32-with-float64-fallback traversal.
//
// Query order does not affect any result (queries are independent and every
// result is written to the query's own index), so the sort is safe.  The
// traversal stacks live in shared memory.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "ct_common.cuh"
#include "ct_internal.h"
#include "ct_locf.cuh"

extern "C" int ct_exclusive_scan(const int64_t* in, int64_t n, int64_t* out, void* ws, size_t ws_bytes,
                                 int64_t* total_host, void* stream);
extern "C" size_t ct_scan_workspace_size(int64_t n);

namespace ctl {

constexpr int CMAX = 6;             // candidates kept per query
constexpr int LOC_THREADS = 256;
constexpr int GRID_STRIDE = 152 * 8;

struct TreeL {
    const float4* nf;
    const double2* nd;
    const double2* poly;
    const float4* polyf;
    const uint8_t* plen;
    const uint8_t* plen32;
    const int64_t* bbi;
    unsigned int* err;
    int64_t n_nodes;
    double ox, oy;
    float dabs;
    float bandG;  // error band of every float32 node bound: 2^-22 * max |bound - origin|
    int K;
    int S4;     // float4 units per cell in polyf
    int stack;  // stack entries per thread (>= max_depth + 2)
    const int* gstart;  // start-node grid (null: start at the root)
    int gnx, gny;
    float gx0, gy0, gsx, gsy;
    const int64_t* coff;  // candidate lists (null: off)
    const int* cidx;
    const float4* cbox;   // widened box of each list entry
    double tol;           // query tolerance
    float tolf;           // tol rounded up to float32
    float ohx, olx, ohy, oly;  // float32 frame origin, split hi + lo
};

// The tree of a query: the kernel's own (one tree) or the query's entry of a
// device array of trees (a batch of meshes, tree index per query).
template <bool MULTI>
__device__ __forceinline__ const TreeL& tree_of(const TreeL& T0, const TreeL* __restrict__ forest,
                                                const int* __restrict__ qtree, int oi) {
    if (MULTI) return forest[qtree[oi]];
    return T0;
}

struct Recs {
    int* orig;                 // query index in the caller's order
    int64_t* res;              // surely-hit cell of the fast pass or -1
    unsigned long long* first; // (ordinal << 32 | polygon) of the first true candidate
    int4* pairs;               // (record, ordinal, polygon, -)
    int cap;
};

__device__ __forceinline__ int na(const float4& q) { return __float_as_int(q.z); }
__device__ __forceinline__ int nbq(const float4& q) { return __float_as_int(q.w); }
__device__ __forceinline__ float bandf(float x) { return fabsf(x) * 2.384185791015625e-07f + 1e-30f; }

__device__ __forceinline__ unsigned lane_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// float32 value of (x - o) in the global frame and its error bound (no
// float64 instruction): x split exactly into hi + lo, o = ohi + olo.
__device__ __forceinline__ void to_frame(double x, float ohi, float olo, float* v, float* err, float* xh_out,
                                         float* xl_out) {
    float lo;
    float hi = split_hi(x, &lo);
    float t1 = hi - ohi, t2 = lo - olo, r = t1 + t2;
    *v = r;
    *err = 5.9604644775390625e-08f * (fabsf(t1) + fabsf(t2) + fabsf(r) + fabsf(lo) + fabsf(olo)) + 1e-30f;
    *xh_out = hi;
    *xl_out = lo;
}

// Warp-aggregated append of `idx` to a list.
__device__ __forceinline__ void append(bool d, int idx, int* list, int* count) {
    unsigned m = __ballot_sync(__activemask(), d);
    if (!d) return;
    int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(m, base, leader);
    list[base + __popc(m & lane_lt())] = idx;
}

// Node step of the float32 traversal with in-line float64 re-decisions for
// bounds inside their band (locate_point query.py:87-105).  Returns false on
// stack overflow.
__device__ __forceinline__ bool node_step(const TreeL& T, int* s, int B, int& sp, int v, const float4& q, float x,
                                          float dx, const double2* __restrict__ pts, int i, int dim) {
    float Lf = q.x, Rf = q.y;
    float bL = dx, bR = dx;  // dx already holds the point's error plus the tree-wide bound band
    float dl = x - Lf, dr = x - Rf;
    bool left, right, have = false;
    double2 nd;
    double pd = 0.0;
    if (dl > bL) left = false;
    else if (-dl > bL) left = true;
    else {
        nd = T.nd[v];
        double2 p2 = pts[i];
        pd = dim ? p2.y : p2.x;
        have = true;
        left = pd <= nd.x;
    }
    if (dr > bR) right = true;
    else if (-dr > bR) right = false;
    else {
        if (!have) {
            nd = T.nd[v];
            double2 p2 = pts[i];
            pd = dim ? p2.y : p2.x;
            have = true;
        }
        right = pd >= nd.y;
    }
    int child = na(q);
    if (sp + 2 > T.stack) return false;
    if (left && right) {
        float aF = Lf - x, bF = x - Rf;
        float bo = 2.0f * dx + 2.384185791015625e-07f * (fabsf(aF) + fabsf(bF)) + 1e-30f;
        bool near_first;
        if (fabsf(aF - bF) > bo) near_first = aF < bF;
        else {
            if (!have) {
                nd = T.nd[v];
                double2 p2 = pts[i];
                pd = dim ? p2.y : p2.x;
            }
            near_first = (nd.x - pd) < (pd - nd.y);
        }
        if (near_first) {
            s[(sp++) * B] = child;
            s[(sp++) * B] = child + 1;
        } else {
            s[(sp++) * B] = child + 1;
            s[(sp++) * B] = child;
        }
    } else if (left) {
        s[(sp++) * B] = child;
    } else if (right) {
        s[(sp++) * B] = child + 1;
    }
    return true;
}

// float64 re-decision of node v (locate_point query.py:87-105) for a query
// whose float32 margins were inside the band: bit 0 left child, bit 1 right
// child, bit 2 right child first.  Kept out of line so that no float64
// instruction is scheduled on the float32 path (GB300 runs float64 at 1/64
// of the float32 rate).
__device__ __noinline__ int node_exact_code(const double2* __restrict__ nd_all, int v, const double2* __restrict__ pts,
                                            int oi, int dim) {
    double2 nd = nd_all[v];
    double2 p2 = pts[oi];
    double pd = dim ? p2.y : p2.x;
    int left = pd <= nd.x, right = pd >= nd.y;
    int rf = (nd.x - pd) < (pd - nd.y);
    return left | (right << 1) | (rf << 2);
}

// Children of internal node v for the float32 traversal: returns the child to
// visit next, or -1 when neither child contains the point, and pushes the
// second child of a two-child visit (the reference pushes both and pops the
// nearer bound's child first).  Decisions whose float32 margin is within the
// band `dx` are taken from node_exact_code.  `ok` is cleared on stack
// overflow.
__device__ __forceinline__ int node_next(const TreeL& T, int* s, int B, int& sp, int v, const float4& q, float x,
                                         float dx, const double2* __restrict__ pts, int oi, int dim, bool& ok) {
    const float Lf = q.x, Rf = q.y;
    const float dl = x - Lf, dr = x - Rf;
    const int child = na(q);
    bool left = dl < 0.0f, right = dr > 0.0f;
    bool sure = fabsf(dl) > dx && fabsf(dr) > dx;
    bool right_first = false;
    if (sure && left && right) {
        float aF = Lf - x, bF = x - Rf;
        float bo = 2.0f * dx + 2.384185791015625e-07f * (fabsf(aF) + fabsf(bF)) + 1e-30f;
        sure = fabsf(aF - bF) > bo;
        right_first = aF < bF;
    }
    if (!sure) {
        int c = node_exact_code(T.nd, v, pts, oi, dim);
        // float32-sure decisions stand; only the uncertain ones are replaced
        if (!(fabsf(dl) > dx)) left = c & 1;
        if (!(fabsf(dr) > dx)) right = (c >> 1) & 1;
        right_first = (c >> 2) & 1;
    }
    if (!(left && right)) return left ? child : (right ? child + 1 : -1);
    if (sp + 1 > T.stack) {
        ok = false;
        return -1;
    }
    s[(sp++) * B] = right_first ? child : child + 1;
    return right_first ? child + 1 : child;
}

// Stage 2b: float32 traversal with candidate collection, over every query
// (qlist null) or over the queries stage 2a left open (qlist, *qcount).
template <int KT, bool MULTI>
__global__ void __launch_bounds__(LOC_THREADS)
    k_fast(const __grid_constant__ TreeL T0, const TreeL* __restrict__ forest, const int* __restrict__ qtree,
           const double2* __restrict__ pts, const int* __restrict__ order, int64_t n, int64_t* __restrict__ out, Recs R,
           int* __restrict__ counters, int* __restrict__ ovf, const int* __restrict__ qlist,
           const int* __restrict__ qcount) {
    extern __shared__ int stk[];
    const int64_t nq = qlist ? (int64_t)min(*qcount, (int)min(n, (int64_t)INT32_MAX)) : n;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nq; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tq = base + threadIdx.x;
        bool active = tq < nq;
        const int64_t i = active ? (qlist ? (int64_t)qlist[tq] : tq) : 0;
        int nc = 0;
        int cand[CMAX];
        bool overflow = false;
        int64_t res = -1;
        // queries are taken in the sorted order; oi is the query's own index
        const int oi = active ? (order ? order[i] : (int)i) : 0;
        if (active) {
            const TreeL& T = tree_of<MULTI>(T0, forest, qtree, oi);
            double2 pp = pts[oi];
            float px, py, dpx, dpy;
            PtSplit P;
            to_frame(pp.x, T.ohx, T.olx, &px, &dpx, &P.xh, &P.xl);
            to_frame(pp.y, T.ohy, T.oly, &py, &dpy, &P.yh, &P.yl);
            dpx += T.bandG;
            dpy += T.bandG;
            const int B = blockDim.x;
            int* s = stk + threadIdx.x;
            int sp = 0;
            int v = 0;
            if (T.gstart) {
                // grid cell of the point; outside the grid (or NaN): the root
                float fx = (px - T.gx0) * T.gsx, fy = (py - T.gy0) * T.gsy;
                if (fx >= 0.0f && fx < (float)T.gnx && fy >= 0.0f && fy < (float)T.gny)
                    v = T.gstart[(int64_t)(int)fy * T.gnx + (int)fx];
            }
            // at most n_nodes visits; v = -1: the root path ends without a child
            int budget = (v < 0) ? 0 : (int)min(T.n_nodes, (int64_t)INT32_MAX - 1) + 1;
            while (budget > 0) {
                if (--budget == 0) {
                    set_error(T.err, CT_DEVERR_LOOP);
                    break;
                }
                float4 q = T.nf[v];
                int b = nbq(q);
                if (b < 0) {
                    int dim = -1 - b;
                    bool ok = true;
                    int nx = node_next(T, s, B, sp, v, q, dim ? py : px, dim ? dpy : dpx, pts, oi, dim, ok);
                    if (nx >= 0) {
                        v = nx;
                        continue;
                    }
                    if (!ok) {
                        set_error(T.err, CT_DEVERR_STACK);
                        break;
                    }
                } else {
                    int ptr = na(q);
                    bool done = false;
                    for (int j = ptr; j < ptr + b; j++) {
                        int r = (KT <= 4) ? leaf_filter_poly<(KT <= 4 ? KT : 4)>(
                                                P, T.dabs, T.tolf, T.polyf + (size_t)j * T.S4, (int)T.plen32[j])
                                          : leaf_filter_local<KT>(P, T.dabs, T.tolf, T.polyf + (size_t)j * T.S4,
                                                                  (int)T.plen32[j]);
                        if (r == LF_INSIDE) {
                            res = T.bbi[j];
                            done = true;
                            break;
                        }
                        if (r == LF_UNSURE) {
                            if (nc < CMAX) {
                                cand[nc++] = j;
                            } else {
                                overflow = true;
                                done = true;
                                break;
                            }
                        }
                    }
                    if (done) break;
                }
                if (sp == 0) break;
                v = s[(--sp) * B];
            }
        }
        if (active && !overflow && nc == 0) out[oi] = res;
        // records for queries with candidates
        bool want = active && !overflow && nc > 0;
        unsigned m = __ballot_sync(0xffffffffu, want);
        if (want) {
            int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(&counters[1], __popc(m));
            base = __shfl_sync(m, base, leader);
            int rec = base + __popc(m & lane_lt());
            if (rec >= R.cap) {
                overflow = true;  // no record left: the exact pass takes it
            } else {
                R.orig[rec] = oi;
                R.res[rec] = res;
                R.first[rec] = ~0ull;
                int pb = atomicAdd(&counters[2], nc);
                for (int c = 0; c < CMAX; c++)
                    if (c < nc) R.pairs[pb + c] = make_int4(rec, c, cand[c], 0);
            }
        }
        append(active && overflow, oi, ovf, &counters[0]);
    }
}

constexpr int RES_OPEN = INT32_MIN;  // sorted-order result of a query left open

// One query of stage 2a: the cells listed for its grid cell, a float32 bbox
// reject, then the float32 leaf filter.  Returns whether the query stays
// open (its result is then left to stage 2b).
template <int KT>
__device__ __forceinline__ bool cells_one(const TreeL& T, double2 pp, int64_t i, int oi, int64_t* __restrict__ out,
                                          int* __restrict__ res_sorted) {
    bool open = false;
    float px, py, dpx, dpy;
    PtSplit P;
    to_frame(pp.x, T.ohx, T.olx, &px, &dpx, &P.xh, &P.xl);
    to_frame(pp.y, T.ohy, T.oly, &py, &dpy, &P.yh, &P.yl);
    float fx = (px - T.gx0) * T.gsx, fy = (py - T.gy0) * T.gsy;
    if (T.coff && fx >= 0.0f && fx < (float)T.gnx && fy >= 0.0f && fy < (float)T.gny) {
        const int64_t g = (int64_t)(int)fy * T.gnx + (int)fx;
        const int64_t s0 = T.coff[g], s1 = T.coff[g + 1];
        // the point's float32 interval
        const float xl = __fsub_rd(px, dpx), xh = __fadd_ru(px, dpx);
        const float yl = __fsub_rd(py, dpy), yh = __fadd_ru(py, dpy);
        int hits = 0, hit = -1;
        // entry k+1 is loaded while entry k is tested
        int jn = 0;
        float4 bn = make_float4(0.f, 0.f, 0.f, 0.f);
        if (s0 < s1) {
            jn = T.cidx[s0];
            bn = T.cbox[s0];
        }
        // Rounds of two phases: (1) collect up to four entries whose box
        // holds the point's interval, (2) filter them.  The filter then
        // runs for the lanes that have a polygon to test, not once per
        // iteration of a loop whose trip count is the longest list of
        // the warp.  The decision does not depend on the order of the
        // tests.
        int64_t k = s0;
        while (!open && k < s1) {
            int np = 0, c0 = 0, c1 = 0, c2 = 0, c3 = 0;
            for (; k < s1 && np < 4; k++) {
                const int j = jn;
                const float4 b = bn;
                if (k + 1 < s1) {
                    jn = T.cidx[k + 1];
                    bn = T.cbox[k + 1];
                }
                if (xh < b.x || xl > b.y || yh < b.z || yl > b.w) continue;  // outside: predicate false
                c3 = c2;
                c2 = c1;
                c1 = c0;
                c0 = j;
                np++;
            }
            for (int c = 0; c < np; c++) {
                const int j = c0;
                c0 = c1;
                c1 = c2;
                c2 = c3;
                int r = (KT <= 4) ? leaf_filter_poly<(KT <= 4 ? KT : 4)>(
                                        P, T.dabs, T.tolf, T.polyf + (size_t)j * T.S4, (int)T.plen32[j])
                                  : leaf_filter_local<KT>(P, T.dabs, T.tolf, T.polyf + (size_t)j * T.S4,
                                                          (int)T.plen32[j]);
                if (r == LF_UNSURE) {
                    open = true;
                    break;
                }
                if (r == LF_INSIDE) {
                    hit = j;
                    if (++hits > 1) {
                        open = true;
                        break;
                    }
                }
            }
        }
        if (!open) {
            const int r = hits ? (int)T.bbi[hit] : -1;
            if (res_sorted) res_sorted[i] = r;
            else out[oi] = r;
        }
    } else {
        open = true;
    }
    if (open && res_sorted) res_sorted[i] = RES_OPEN;
    return open;
}

// Warp-aggregated append of the open queries' sorted positions.
__device__ __forceinline__ void append_open(bool open, int64_t i, int* __restrict__ qlist, int* __restrict__ qcount) {
    unsigned m = __ballot_sync(0xffffffffu, open);
    if (m) {
        const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
        int b0 = 0;
        if (lane == leader) b0 = atomicAdd(qcount, __popc(m));
        b0 = __shfl_sync(0xffffffffu, b0, leader);
        if (open) qlist[b0 + __popc(m & lane_lt())] = (int)i;
    }
}

// Stage 2a: candidate lists.  Per query the cells listed for its grid cell:
// a float32 bbox reject, then the float32 leaf filter.  Exactly one sure hit
// with sure misses elsewhere, or sure misses only, is final; otherwise the
// query's sorted position goes to the list of stage 2b.  With `res_sorted`
// the results go there by sorted position (RES_OPEN for open queries; a
// bucketed scatter takes them to `out`), else straight to out[oi].
// 6 blocks of 256 threads per SM (40 registers): measured faster than the
// 48-register build at 5 blocks despite a few spilled values.
template <int KT, bool MULTI, int MINB = 6>
__global__ void __launch_bounds__(LOC_THREADS, MINB)
    k_cells(const __grid_constant__ TreeL T0, const TreeL* __restrict__ forest, const int* __restrict__ qtree,
            const double2* __restrict__ pts, const int* __restrict__ order, int64_t n, int64_t* __restrict__ out,
            int* __restrict__ res_sorted, int* __restrict__ qlist, int* __restrict__ qcount) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool open = false;
    if (i < n) {
        const int oi = order ? order[i] : (int)i;
        const TreeL& T = tree_of<MULTI>(T0, forest, qtree, oi);
        open = cells_one<KT>(T, pts[oi], i, oi, out, res_sorted);
    }
    append_open(open, i, qlist, qcount);
}

// Results by sorted position -> out[order[i]], in two passes so that the
// random 8-byte writes land in an L2-sized window at a time and leave the
// cache as whole sectors: (1) regroup the (query, result) pairs by the
// bucket (query >> shift) of their destination -- at most 256 buckets,
// bucket d owning the range [d << shift, (d + 1) << shift) of the pair
// arrays, filled through a per-bucket cursor; (2) walk the pair arrays in
// order and write every result that is not RES_OPEN.  `order` is a
// permutation of 0 .. n-1, so bucket d receives exactly the queries of its
// range; a pair that would fall outside it is dropped with an error bit.
constexpr int RB_T = 256, RB_IPT = 16, RB_TILE = RB_T * RB_IPT;

__global__ void __launch_bounds__(RB_T)
    k_res_bucket(const int* __restrict__ res_sorted, const int* __restrict__ order, int64_t n, int shift,
                 unsigned long long* __restrict__ cursor, int* __restrict__ pq, int* __restrict__ pr,
                 unsigned int* __restrict__ err) {
    __shared__ int cnt[256];
    __shared__ int tbase[256];
    __shared__ int wsum[RB_T / 32];
    __shared__ long long gbase[256];
    __shared__ int sq[RB_TILE];
    __shared__ int sr[RB_TILE];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int64_t base = (int64_t)blockIdx.x * RB_TILE;
    cnt[t] = 0;
    __syncthreads();
    int q[RB_IPT], r[RB_IPT], rk[RB_IPT];
#pragma unroll
    for (int k = 0; k < RB_IPT; k++) {
        const int64_t i = base + k * RB_T + t;
        const bool v = i < n;
        q[k] = v ? order[i] : -1;
        r[k] = v ? res_sorted[i] : 0;
    }
#pragma unroll
    for (int k = 0; k < RB_IPT; k++) rk[k] = (q[k] >= 0) ? atomicAdd(&cnt[(q[k] >> shift) & 255], 1) : 0;
    __syncthreads();
    const int c = cnt[t];
    int x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    int pre = 0;
    for (int ww = 0; ww < w; ww++) pre += wsum[ww];
    tbase[t] = pre + x - c;
    gbase[t] = c ? (long long)atomicAdd(&cursor[t], (unsigned long long)c) : 0;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < RB_IPT; k++)
        if (q[k] >= 0) {
            const int pos = tbase[(q[k] >> shift) & 255] + rk[k];
            sq[pos] = q[k];
            sr[pos] = r[k];
        }
    __syncthreads();
    const int m = (int)min((int64_t)RB_TILE, n - base);
    for (int j = t; j < m; j += RB_T) {
        const int qq = sq[j];
        const int d = (qq >> shift) & 255;
        const int64_t lo = (int64_t)d << shift, hi = min(n, (int64_t)(d + 1) << shift);
        const int64_t dst = lo + gbase[d] + (j - tbase[d]);
        if (dst >= hi) {
            set_error(err, CT_DEVERR_CAPACITY);
            continue;
        }
        pq[dst] = qq;
        pr[dst] = sr[j];
    }
}

__global__ void __launch_bounds__(256)
    k_res_unbucket(const int* __restrict__ pq, const int* __restrict__ pr, int64_t n, int64_t* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        const int r = pr[t];
        const int q = pq[t];
        if (r != RES_OPEN && q >= 0 && q < n) out[q] = r;
    }
}

// Stage 3: exact float64 test of every candidate pair.
template <bool MULTI>
__global__ void __launch_bounds__(LOC_THREADS)
    k_pip(const __grid_constant__ TreeL T0, const TreeL* __restrict__ forest, const int* __restrict__ qtree,
          const double2* __restrict__ pts, Recs R, const int* __restrict__ counters) {
    int npairs = counters[2];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npairs; t += gridDim.x * blockDim.x) {
        int4 pr = R.pairs[t];
        const int oi = R.orig[pr.x];
        const TreeL& T = tree_of<MULTI>(T0, forest, qtree, oi);
        double2 pp = pts[oi];
        int j = pr.z;
        const dpt* poly = reinterpret_cast<const dpt*>(T.poly + (size_t)j * T.K);
        int len = T.plen ? (int)T.plen[j] : T.K;
        if (pip_or_edge(mkp(pp.x, pp.y), poly, len, T.tol))
            atomicMin(&R.first[pr.x], ((unsigned long long)(unsigned)pr.y << 32) | (unsigned)j);
    }
}

// Stage 4: first true candidate, else the fast pass's hit.
template <bool MULTI>
__global__ void k_resolve(const __grid_constant__ TreeL T0, const TreeL* __restrict__ forest,
                          const int* __restrict__ qtree, Recs R, const int* __restrict__ counters,
                          int64_t* __restrict__ out) {
    int nrec = min(counters[1], R.cap);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += gridDim.x * blockDim.x) {
        unsigned long long f = R.first[r];
        const int oi = R.orig[r];
        const TreeL& T = tree_of<MULTI>(T0, forest, qtree, oi);
        out[oi] = (f != ~0ull) ? T.bbi[(int)(f & 0xffffffffull)] : R.res[r];
    }
}

// Stage 5: overflow queries, float32 bands with float64 re-decisions.
template <int KT, bool MULTI>
__global__ void __launch_bounds__(LOC_THREADS)
    k_exact(const __grid_constant__ TreeL T0, const TreeL* __restrict__ forest, const int* __restrict__ qtree,
            const double2* __restrict__ pts, const int* __restrict__ list, const int* __restrict__ counters,
            int64_t* __restrict__ out) {
    extern __shared__ int stk[];
    const int B = blockDim.x;
    int* s = stk + threadIdx.x;
    int cnt = counters[0];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += gridDim.x * blockDim.x) {
        int i = list[t];
        const TreeL& T = tree_of<MULTI>(T0, forest, qtree, i);
        const double tol = T.tol;
        const float tolf = T.tolf;
        double2 pp = pts[i];
        dpt p = mkp(pp.x, pp.y);
        float px, py, dpx, dpy;
        PtSplit P;
        to_frame(pp.x, T.ohx, T.olx, &px, &dpx, &P.xh, &P.xl);
        to_frame(pp.y, T.ohy, T.oly, &py, &dpy, &P.yh, &P.yl);
        dpx += T.bandG;
        dpy += T.bandG;
        int sp = 1;
        s[0] = 0;
        int64_t res = -1;
        int64_t budget = T.n_nodes;
        while (sp > 0) {
            if (--budget < 0) {
                set_error(T.err, CT_DEVERR_LOOP);
                break;
            }
            int v = s[(--sp) * B];
            float4 q = T.nf[v];
            int b = nbq(q);
            if (b >= 0) {
                int ptr = na(q);
                bool hit = false;
                for (int j = ptr; j < ptr + b; j++) {
                    int r = leaf_filter_local<KT>(P, T.dabs, tolf, T.polyf + (size_t)j * T.S4, (int)T.plen32[j]);
                    if (r == LF_UNSURE) {
                        const dpt* poly = reinterpret_cast<const dpt*>(T.poly + (size_t)j * T.K);
                        int len = T.plen ? (int)T.plen[j] : T.K;
                        r = pip_or_edge(p, poly, len, tol) ? LF_INSIDE : LF_OUTSIDE;
                    }
                    if (r == LF_INSIDE) {
                        hit = true;
                        res = T.bbi[j];
                        break;
                    }
                }
                if (hit) break;
                continue;
            }
            int dim = -1 - b;
            if (!node_step(T, s, B, sp, v, q, dim ? py : px, dim ? dpy : dpx, pts, i, dim)) {
                set_error(T.err, CT_DEVERR_STACK);
                break;
            }
        }
        out[i] = res;
    }
}

// ---------------------------------------------------------------------------
// query ordering: LSD radix sort of (Morton key, index) pairs
// ---------------------------------------------------------------------------
constexpr int RS_BLOCKS = 152 * 8;  // fixed grid (8 blocks per SM); each block owns a contiguous chunk
constexpr int RS_T = 256;
constexpr int RS_IPT = 16;  // keys per thread per tile of the scatter
constexpr int RS_TILE = RS_T * RS_IPT;

struct Grid {
    float x0, y0, sx, sy;  // cell = floor((x - x0) * sx), 2^12 cells per axis
};

__device__ __forceinline__ unsigned spread12(unsigned v) {  // 12 bits -> even bit positions
    v &= 0xfff;
    v = (v | (v << 8)) & 0x00ff00ff;
    v = (v | (v << 4)) & 0x0f0f0f0f;
    v = (v | (v << 2)) & 0x33333333;
    v = (v | (v << 1)) & 0x55555555;
    return v;
}

__device__ __forceinline__ unsigned morton24(const Grid& g, double2 p) {
    float lo;
    float fx = (split_hi(p.x, &lo) - g.x0) * g.sx;
    float fy = (split_hi(p.y, &lo) - g.y0) * g.sy;
    unsigned bx = (fx > 0.0f) ? (unsigned)fminf(fx, 4095.0f) : 0u;  // NaN -> 0
    unsigned by = (fy > 0.0f) ? (unsigned)fminf(fy, 4095.0f) : 0u;
    return spread12(bx) | (spread12(by) << 1);
}

// Every sort kernel runs on RS_BLOCKS blocks; block b owns the chunk
// [b * chunk, min((b + 1) * chunk, n)) of its input (chunk a multiple of
// RS_TILE, so each chunk starts 16-byte aligned).  hist[d * RS_BLOCKS + b]
// counts digit d in block b's chunk; its exclusive scan is where block b
// writes its keys of digit d.

// Keys of the queries and the histogram of the first digit (the indices of
// the first pass are implicit: the scatter takes a null index input as i).
__global__ void __launch_bounds__(RS_T) k_keys(const double2* __restrict__ pts, int64_t n, int64_t chunk, Grid g,
                                                int shift, unsigned* __restrict__ key, int64_t* __restrict__ hist) {
    __shared__ int h[RS_T / 32][256];
    const int t = threadIdx.x, w = t >> 5;
    for (int k = 0; k < RS_T / 32; k++) h[k][t] = 0;
    __syncthreads();
    // chunks past the end are empty (e = s): a negative length would make the
    // vector loop bound below round down into the next chunk
    int64_t s = (int64_t)blockIdx.x * chunk, e = max(s, min(s + chunk, n));
    // four points in flight per thread (one at a time left the loads too few
    // to cover the memory latency)
    constexpr int U = 4;
    for (int64_t i0 = s + t; i0 < e; i0 += U * RS_T) {
        double2 q[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int64_t i = i0 + (int64_t)u * RS_T;
            if (i < e) q[u] = pts[i];
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int64_t i = i0 + (int64_t)u * RS_T;
            if (i < e) {
                const unsigned k = morton24(g, q[u]);
                key[i] = k;
                atomicAdd(&h[w][(k >> shift) & 255u], 1);
            }
        }
    }
    __syncthreads();
    int c = 0;
    for (int k = 0; k < RS_T / 32; k++) c += h[k][t];
    hist[(int64_t)t * gridDim.x + blockIdx.x] = c;
}

// Keys of a batch of trees: the point's tree (binary search of the point
// offsets) in the high bits, the top `mbits` bits of its Morton key over its
// own tree's bbox below; histogram of the lowest digit.
__global__ void __launch_bounds__(RS_T) k_keys_forest(const double2* __restrict__ pts, int64_t n, int64_t chunk,
                                                       const Grid* __restrict__ grids,
                                                       const int64_t* __restrict__ poff, int n_trees, int mbits,
                                                       unsigned* __restrict__ key, int* __restrict__ qtree,
                                                       int64_t* __restrict__ hist) {
    __shared__ int h[RS_T / 32][256];
    const int t = threadIdx.x, w = t >> 5;
    for (int k = 0; k < RS_T / 32; k++) h[k][t] = 0;
    __syncthreads();
    // chunks past the end are empty (e = s): a negative length would make the
    // vector loop bound below round down into the next chunk
    int64_t s = (int64_t)blockIdx.x * chunk, e = max(s, min(s + chunk, n));
    for (int64_t i = s + t; i < e; i += RS_T) {
        int lo = 0, hi = n_trees;  // poff[lo] <= i < poff[hi]
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (poff[mid] <= i) lo = mid;
            else hi = mid;
        }
        unsigned m = morton24(grids[lo], pts[i]) >> (24 - mbits);
        unsigned k = ((unsigned)lo << mbits) | m;
        key[i] = k;
        qtree[i] = lo;
        atomicAdd(&h[w][k & 255u], 1);
    }
    __syncthreads();
    int c = 0;
    for (int k = 0; k < RS_T / 32; k++) c += h[k][t];
    hist[(int64_t)t * gridDim.x + blockIdx.x] = c;
}

// Histogram of one 8-bit digit per block chunk (warp-private counters).
__global__ void __launch_bounds__(RS_T) k_rs_hist(const unsigned* __restrict__ key, int64_t n, int64_t chunk,
                                                   int shift, int64_t* __restrict__ hist) {
    __shared__ int h[RS_T / 32][256];
    const int t = threadIdx.x, w = t >> 5;
    for (int k = 0; k < RS_T / 32; k++) h[k][t] = 0;
    __syncthreads();
    // chunks past the end are empty (e = s): a negative length would make the
    // vector loop bound below round down into the next chunk
    int64_t s = (int64_t)blockIdx.x * chunk, e = max(s, min(s + chunk, n));
    int64_t ev = s + ((e - s) & ~(int64_t)3);  // end of the whole uint4 groups
    for (int64_t i = s + 4 * t; i < ev; i += 4 * RS_T) {
        uint4 k4 = *reinterpret_cast<const uint4*>(key + i);
        atomicAdd(&h[w][(k4.x >> shift) & 255u], 1);
        atomicAdd(&h[w][(k4.y >> shift) & 255u], 1);
        atomicAdd(&h[w][(k4.z >> shift) & 255u], 1);
        atomicAdd(&h[w][(k4.w >> shift) & 255u], 1);
    }
    for (int64_t i = ev + t; i < e; i += RS_T) atomicAdd(&h[w][(key[i] >> shift) & 255u], 1);
    __syncthreads();
    int c = 0;
    for (int k = 0; k < RS_T / 32; k++) c += h[k][t];
    hist[(int64_t)t * gridDim.x + blockIdx.x] = c;
}

// The same for one-byte digits (written by the previous pass).
__global__ void __launch_bounds__(RS_T) k_rs_hist8(const uint8_t* __restrict__ key, int64_t n, int64_t chunk,
                                                    int64_t* __restrict__ hist) {
    __shared__ int h[RS_T / 32][256];
    const int t = threadIdx.x, w = t >> 5;
    for (int k = 0; k < RS_T / 32; k++) h[k][t] = 0;
    __syncthreads();
    int64_t s = (int64_t)blockIdx.x * chunk, e = max(s, min(s + chunk, n));
    int64_t ev = s + ((e - s) & ~(int64_t)15);  // end of the whole 16-byte groups
    for (int64_t i = s + 16 * t; i < ev; i += 16 * RS_T) {
        const uint4 k4 = *reinterpret_cast<const uint4*>(key + i);
        const unsigned wd[4] = {k4.x, k4.y, k4.z, k4.w};
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int b = 0; b < 4; b++) atomicAdd(&h[w][(wd[q] >> (8 * b)) & 255u], 1);
    }
    for (int64_t i = ev + t; i < e; i += RS_T) atomicAdd(&h[w][key[i]], 1);
    __syncthreads();
    int c = 0;
    for (int k = 0; k < RS_T / 32; k++) c += h[k][t];
    hist[(int64_t)t * gridDim.x + blockIdx.x] = c;
}

// Scatter of one digit.  The block walks its chunk in tiles of RS_TILE
// keys; a key's rank within its digit in the tile comes from a shared-memory
// atomic (so equal digits of one tile may be permuted -- the order of the
// queries only has to be coherent, every result is written by the query's
// own index), the tile is regrouped by digit in shared memory and written
// out in runs.  A null `iin` stands for the indices 0 .. n-1; a null `kout`
// (the last pass) writes the indices only.  Keys are read as KI and written
// as KO after a right shift by `oshift`: a pass whose successor sorts the
// last 8 bits writes just that byte.
template <typename KI, typename KO>
__global__ void __launch_bounds__(RS_T) k_rs_scatter(const KI* __restrict__ kin, const int* __restrict__ iin,
                                                      int64_t n, int64_t chunk, int shift,
                                                      const int64_t* __restrict__ offs, KO* __restrict__ kout,
                                                      int oshift, int* __restrict__ iout) {
    __shared__ int cur[256];    // output position of the digit's next key
    __shared__ int cnt[256];    // digit counts of the tile
    __shared__ int tbase[256];  // exclusive scan of cnt
    __shared__ int wsum[RS_T / 32];
    __shared__ unsigned sk[RS_TILE];
    __shared__ int si[RS_TILE];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    cur[t] = (int)offs[(int64_t)t * gridDim.x + blockIdx.x];
    // chunks past the end are empty (e = s): a negative length would make the
    // vector loop bound below round down into the next chunk
    int64_t s = (int64_t)blockIdx.x * chunk, e = max(s, min(s + chunk, n));
    for (int64_t base = s; base < e; base += RS_TILE) {
        cnt[t] = 0;
        __syncthreads();
        unsigned key[RS_IPT];
        int id[RS_IPT], rk[RS_IPT];
#pragma unroll
        for (int k = 0; k < RS_IPT; k++) {
            int64_t i = base + k * RS_T + t;
            bool v = i < e;
            key[k] = v ? (unsigned)kin[i] : 0u;
            id[k] = v ? (iin ? iin[i] : (int)i) : -1;
        }
#pragma unroll
        for (int k = 0; k < RS_IPT; k++) rk[k] = (id[k] >= 0) ? atomicAdd(&cnt[(key[k] >> shift) & 255u], 1) : 0;
        __syncthreads();
        int c = cnt[t];
        int x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        int pre = 0;
        for (int ww = 0; ww < w; ww++) pre += wsum[ww];
        tbase[t] = pre + x - c;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < RS_IPT; k++)
            if (id[k] >= 0) {
                int pos = tbase[(key[k] >> shift) & 255u] + rk[k];
                sk[pos] = key[k];
                si[pos] = id[k];
            }
        __syncthreads();
        int m = (int)min((int64_t)RS_TILE, e - base);
        for (int j = t; j < m; j += RS_T) {
            unsigned kk = sk[j];
            int dd = (int)((kk >> shift) & 255u);
            int dst = cur[dd] + (j - tbase[dd]);
            if (kout) kout[dst] = (KO)(kk >> oshift);
            iout[dst] = si[j];
        }
        __syncthreads();
        cur[t] += c;
    }
}

// ---------------------------------------------------------------------------
// start-node grid
// ---------------------------------------------------------------------------
// Start node of grid cell (gx, gy): follow the root path while every point of
// the cell (its range widened by `m`) takes one and the same single child.
// The float32 node bounds are within `band` of the float64 bounds, so a
// decision is certain when the cell range clears bound -/+ band (directed
// rounding).
// cw = 1 / sx and ch = 1 / sy (cell sizes, divided once by the caller): the
// products differ from the quotients by an ulp or two, far inside the margin m.
__device__ __forceinline__ int grid_cell_start(const float4* __restrict__ nf, int gx, int gy, float x0, float y0,
                                               double cw, double ch, double m, float band, int max_steps) {
    float xlo = __double2float_rd((double)x0 + (double)gx * cw - m);
    float xhi = __double2float_ru((double)x0 + (double)(gx + 1) * cw + m);
    float ylo = __double2float_rd((double)y0 + (double)gy * ch - m);
    float yhi = __double2float_ru((double)y0 + (double)(gy + 1) * ch + m);
    int v = 0;
    for (int k = 0; k < max_steps; k++) {
        float4 q = nf[v];
        int b = nbq(q);
        if (b >= 0) break;  // leaf
        int dim = -1 - b;
        float lo = dim ? ylo : xlo, hi = dim ? yhi : xhi;
        bool all_left = hi < __fsub_rd(q.x, band), no_left = lo > __fadd_ru(q.x, band);
        bool all_right = lo > __fadd_ru(q.y, band), no_right = hi < __fsub_rd(q.y, band);
        if (!((all_left || no_left) && (all_right || no_right))) break;  // a bound inside the cell
        if (all_left && all_right) break;                                // both children taken
        if (all_left) v = na(q);
        else if (all_right) v = na(q) + 1;
        else {
            v = -1;  // no child: locate_point returns -1
            break;
        }
    }
    return v;
}

// One thread per grid cell of one tree.
__global__ void k_grid_start(const float4* __restrict__ nf, int gnx, int gny, float x0, float y0, double cw, double ch,
                             double m, float band, int max_steps, int* __restrict__ start) {
    int64_t total = (int64_t)gnx * gny;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < total; c += (int64_t)gridDim.x * blockDim.x)
        start[c] = grid_cell_start(nf, (int)(c % gnx), (int)(c / gnx), x0, y0, cw, ch, m, band, max_steps);
}

// ---------------------------------------------------------------------------
// candidate lists
// ---------------------------------------------------------------------------
// Widened bbox of every cell (leaf order) in the float32 frame, rounded
// outward: the region where the cell's predicate can be true.
__global__ void k_cand_box(const double* __restrict__ bb, const int64_t* __restrict__ bbi, int64_t n, double ox,
                           double oy, double M, float4* __restrict__ box) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double* b = bb + 4 * bbi[j];
        box[j] = make_float4(__double2float_rd((b[0] - ox) - M), __double2float_ru((b[1] - ox) + M),
                             __double2float_rd((b[2] - oy) - M), __double2float_ru((b[3] - oy) + M));
    }
}

// Grid cells met by a widened box: cell gx spans [x0 + gx / sx, x0 + (gx + 1) / sx]
// widened by m.
__device__ __forceinline__ bool cand_range(float4 b, int gnx, int gny, double x0, double y0, double sx, double sy,
                                           double m, int* gx0, int* gx1, int* gy0, int* gy1) {
    double ax = ((double)b.x - m - x0) * sx, bx = ((double)b.y + m - x0) * sx;
    double ay = ((double)b.z - m - y0) * sy, by = ((double)b.w + m - y0) * sy;
    if (!(bx >= 0.0 && ax < (double)gnx && by >= 0.0 && ay < (double)gny)) return false;  // also NaN
    *gx0 = (int)fmax(floor(ax - 1e-9), 0.0);
    *gx1 = (int)fmin(floor(bx + 1e-9), (double)(gnx - 1));
    *gy0 = (int)fmax(floor(ay - 1e-9), 0.0);
    *gy1 = (int)fmin(floor(by + 1e-9), (double)(gny - 1));
    return true;
}

// Box of polygon L (len vertices, float32, frame of the grid cell) clipped
// to the rectangle [X0, X1] x [Y0, Y1], enlarged by the rounding of this
// float32 computation (callers add a slack much larger than it): the union of
// the edges' pieces inside the rectangle (Liang-Barsky, the parameter range
// widened by its rounding bound, so a piece is never cut short) and of the
// rectangle corners the crossing-parity test does not certainly place outside
// (each edge's cross product with the corner beyond its error bound -- the
// parity is then that of the exact polygon).  Extreme points of the
// polygon's inside (crossing-parity) region within the rectangle lie on such
// pieces or corners.  False when the box is empty.
// S bounds every |coordinate|; each vertex of L is within u S + ea of the
// exact vertex (float32 and float64 rounding).
template <int KMAX>
__device__ bool clip_box(const float2* L, int len, float X0, float X1, float Y0, float Y1, float S, float ea,
                         float4* out) {
    const float u = 5.9604644775390625e-08f;
    float bx0 = FLT_MAX, bx1 = -FLT_MAX, by0 = FLT_MAX, by1 = -FLT_MAX;
    for (int k = 0; k < len; k++) {
        const float2 P = L[k], Q = L[(k + 1 == len) ? 0 : k + 1];
        const float dx = Q.x - P.x, dy = Q.y - P.y;
        float t0 = 0.0f, t1 = 1.0f;
        bool ok = true;
        if (dx == 0.0f) {
            ok = P.x >= X0 && P.x <= X1;
        } else {
            float ta = (X0 - P.x) / dx, tb = (X1 - P.x) / dx;
            float e = 4.0f * u * (fabsf(ta) + fabsf(tb));
            t0 = fmaxf(t0, fminf(ta, tb) - e);
            t1 = fminf(t1, fmaxf(ta, tb) + e);
        }
        if (dy == 0.0f) {
            ok = ok && P.y >= Y0 && P.y <= Y1;
        } else {
            float ta = (Y0 - P.y) / dy, tb = (Y1 - P.y) / dy;
            float e = 4.0f * u * (fabsf(ta) + fabsf(tb));
            t0 = fmaxf(t0, fminf(ta, tb) - e);
            t1 = fminf(t1, fmaxf(ta, tb) + e);
        }
        if (!ok || !(t0 <= t1)) continue;
        const float ex0 = P.x + t0 * dx, ex1 = P.x + t1 * dx;
        const float ey0 = P.y + t0 * dy, ey1 = P.y + t1 * dy;
        bx0 = fminf(bx0, fminf(ex0, ex1));
        bx1 = fmaxf(bx1, fmaxf(ex0, ex1));
        by0 = fminf(by0, fminf(ey0, ey1));
        by1 = fmaxf(by1, fmaxf(ey0, ey1));
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const float cx = (c & 1) ? X1 : X0, cy = (c & 2) ? Y1 : Y0;
        int parity = 0;
        bool unsure = false;
        float2 U = make_float2(L[len - 1].x - cx, L[len - 1].y - cy);
        for (int k = 0; k < len; k++) {
            const float2 V = make_float2(L[k].x - cx, L[k].y - cy);
            if (V.x == U.x && V.y == U.y) continue;  // repeated vertex: no edge (geometry_utils.py:203-204)
            const float A = U.x * V.y - U.y * V.x;
            const float m = fmaxf(fmaxf(fabsf(U.x), fabsf(U.y)), fmaxf(fabsf(V.x), fabsf(V.y)));
            // rounding of U, V and A, and the rounding of the vertices
            // themselves (below u S + ea each)
            const float thr = 16.0f * u * m * m + 8.0f * (u * S + ea) * m + 1e-30f;
            unsure |= !(fabsf(A) > thr);
            if ((U.y > 0.0f) != (V.y > 0.0f)) parity ^= (int)((V.y > U.y) ? (A > 0.0f) : (A < 0.0f));
            U = V;
        }
        if (unsure || parity) {
            bx0 = fminf(bx0, cx);
            bx1 = fmaxf(bx1, cx);
            by0 = fminf(by0, cy);
            by1 = fmaxf(by1, cy);
        }
    }
    *out = make_float4(bx0, bx1, by0, by1);
    return bx0 <= bx1 && by0 <= by1;
}

// Box of a surely counter-clockwise triangle V clipped to [X0, X1] x [Y0, Y1]
// (same contract as clip_box, registers only): edge k runs from V[k] with
// direction D[k] (reciprocals rx, ry; 0 where the component is 0) and
// constant cc[k] = V[k] x V[k + 1], so that the cross product of
// (V[k] - C, V[k + 1] - C) is cc[k] - C x D[k].  A corner is left out only
// when one edge puts it surely on its outer side (the triangle is convex).
// Lm, Dm: largest |component| of the vertices and of the edges; each vertex
// is within d = u Lm + ea of the exact one.
__device__ __forceinline__ bool tri_box(const float2 (&V)[3], const float2 (&D)[3], const float (&rx)[3],
                                        const float (&ry)[3], const float (&cc)[3], float Lm, float Dm, float d,
                                        float X0, float X1, float Y0, float Y1, float4* out) {
    const float u = 5.9604644775390625e-08f;
    float bx0 = FLT_MAX, bx1 = -FLT_MAX, by0 = FLT_MAX, by1 = -FLT_MAX;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float2 P = V[k];
        float t0 = 0.0f, t1 = 1.0f;
        bool ok = true;
        if (D[k].x == 0.0f) {
            ok = P.x >= X0 && P.x <= X1;
        } else {
            // the reciprocal, the differences and the products are each
            // rounded once: 8 u of the parameter covers them
            const float ta = (X0 - P.x) * rx[k], tb = (X1 - P.x) * rx[k];
            const float e = 8.0f * u * (fabsf(ta) + fabsf(tb));
            t0 = fmaxf(t0, fminf(ta, tb) - e);
            t1 = fminf(t1, fmaxf(ta, tb) + e);
        }
        if (D[k].y == 0.0f) {
            ok = ok && P.y >= Y0 && P.y <= Y1;
        } else {
            const float ta = (Y0 - P.y) * ry[k], tb = (Y1 - P.y) * ry[k];
            const float e = 8.0f * u * (fabsf(ta) + fabsf(tb));
            t0 = fmaxf(t0, fminf(ta, tb) - e);
            t1 = fminf(t1, fmaxf(ta, tb) + e);
        }
        if (ok && t0 <= t1) {
            const float ex0 = P.x + t0 * D[k].x, ex1 = P.x + t1 * D[k].x;
            const float ey0 = P.y + t0 * D[k].y, ey1 = P.y + t1 * D[k].y;
            bx0 = fminf(bx0, fminf(ex0, ex1));
            bx1 = fmaxf(bx1, fmaxf(ex0, ex1));
            by0 = fminf(by0, fminf(ey0, ey1));
            by1 = fmaxf(by1, fmaxf(ey0, ey1));
        }
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const float cx = (c & 1) ? X1 : X0, cy = (c & 2) ? Y1 : Y0;
        const float c1 = fabsf(cx) + fabsf(cy);
        // rounding of cc, D, the products and the difference; then the
        // vertices' own rounding (d each)
        const float thr = 8.0f * u * (Lm * Lm + c1 * Dm) + 8.0f * d * (2.0f * c1 + 2.0f * Lm) + 1e-30f;
        bool outside = false;
#pragma unroll
        for (int k = 0; k < 3; k++) outside |= (cc[k] - (cx * D[k].y - cy * D[k].x)) < -thr;
        if (!outside) {
            bx0 = fminf(bx0, cx);
            bx1 = fmaxf(bx1, cx);
            by0 = fminf(by0, cy);
            by1 = fmaxf(by1, cy);
        }
    }
    *out = make_float4(bx0, bx1, by0, by1);
    return bx0 <= bx1 && by0 <= by1;
}

// Per cell (leaf order j) and grid cell g of its widened bbox's range: the
// part of the cell within g widened by e2 = m + M (cell-assignment margin
// plus the predicate's reach), its box widened by M and by the float32
// slack, intersected with the cell's widened bbox.  Counted (FILL = false)
// or written to g's list (FILL = true); both passes take the same decisions.
// The vertices are taken once per cell, in float32 relative to the cell's
// first vertex (the anchor, float64); a grid cell's rectangle is placed
// relative to the anchor in float32 with an error far below the slack.
// Triangles that are surely counter-clockwise take tri_box; other cells of
// up to 4 vertices clip_box; cells with fewer than 3 vertices, more than 4
// (clipping them cost more build time than it saved queries in measurements
// on mixed meshes) or non-finite coordinates keep the widened bbox in every
// grid cell of its range.
// Entries of one cell kept in its record slots by the counting pass (more
// go through the geometry again in the filling pass).
constexpr int CAND_SLOTS = 8;
constexpr unsigned char CAND_OVERFLOW = 255;

// Records of the counting pass: the kept (grid cell, clipped box) pairs of
// every cell, so that the filling pass scatters them without repeating the
// geometry.
struct CandRecs {
    int* g;           // n x CAND_SLOTS grid cells
    float4* r;        // n x CAND_SLOTS clipped boxes
    unsigned char* n; // kept pairs per cell, CAND_OVERFLOW when more than CAND_SLOTS
    int* ovf;         // cells with more than CAND_SLOTS pairs
    int* ovf_count;
};

// MODE 0: count the (cell, grid cell) pairs per grid cell; MODE 2: count and
// record them (CandRecs); MODE 1: write the entries of the cells listed in
// `cells` (all cells when null) at off[g] + cursor.
// One cell j (leaf order) with widened box b: the grid cells its predicate
// region meets, each counted in count[g] and, by MODE, recorded or written.
template <int MODE, int KMAX>
__device__ __forceinline__ void cand_cell(int64_t j, float4 b, const double2* __restrict__ poly,
                                          const uint8_t* __restrict__ plen, int K, double ox, double oy, int gnx,
                                          int gny, double x0, double y0, double sx, double sy, double cw, double ch,
                                          double m, float Mf, float e2f, float ea,
                                          unsigned long long* __restrict__ count, const int64_t* __restrict__ off,
                                          int* __restrict__ idx, float4* __restrict__ lbox,
                                          unsigned int* __restrict__ err, const CandRecs& rec) {
    const float u = 5.9604644775390625e-08f;
    int a0, a1, b0, b1;
    int kept = 0;
    if (!cand_range(b, gnx, gny, x0, y0, sx, sy, m, &a0, &a1, &b0, &b1)) {
        if (MODE == 2) rec.n[j] = 0;
        return;
    }
    const int len = plen ? (int)plen[j] : K;
    const double2* pv = poly + (size_t)j * K;
    bool clip = KMAX <= 4 && len >= 3 && len <= KMAX;
    for (int k = 0; k < len && clip; k++) clip = isfinite(pv[k].x) && isfinite(pv[k].y);
    double ax = 0.0, ay = 0.0;
    float2 L[KMAX];
    float Lm = 0.0f;
    if (clip) {
        ax = pv[0].x - ox;
        ay = pv[0].y - oy;
        for (int k = 0; k < len; k++) {
            L[k] = make_float2((float)((pv[k].x - ox) - ax), (float)((pv[k].y - oy) - ay));
            Lm = fmaxf(Lm, fmaxf(fabsf(L[k].x), fabsf(L[k].y)));
        }
    }
    const float d = u * Lm + ea;
    // triangle fast path: edges, reciprocals, constants, orientation
    float2 V[3], D[3];
    float rx[3], ry[3], cc[3];
    bool tri = clip && len == 3;
    float Dm = 0.0f;
    if (tri) {
#pragma unroll
        for (int k = 0; k < 3; k++) V[k] = L[k];
        float area2 = 0.0f, csum = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float2 P = V[k], Q = V[(k + 1) % 3];
            D[k] = make_float2(Q.x - P.x, Q.y - P.y);
            rx[k] = (D[k].x != 0.0f) ? __frcp_rn(D[k].x) : 0.0f;
            ry[k] = (D[k].y != 0.0f) ? __frcp_rn(D[k].y) : 0.0f;
            cc[k] = P.x * Q.y - P.y * Q.x;
            area2 += cc[k];
            csum += fabsf(cc[k]);
            Dm = fmaxf(Dm, fmaxf(fabsf(D[k].x), fabsf(D[k].y)));
        }
        // twice the signed area, beyond its rounding and the vertices' own
        tri = area2 > 4.0f * u * csum + 32.0f * u * Lm * Lm + 16.0f * d * Lm;
    }
    // cw = 1 / sx, ch = 1 / sy: grid cell sizes, divided once on the host
    const float fcw = (float)cw, fch = (float)ch;
    // lower-left corner of the range's first grid cell relative to the anchor
    const float fbx0 = (float)((x0 + (double)a0 * cw) - ax), fby0 = (float)((y0 + (double)b0 * ch) - ay);
    const float axf = (float)ax, ayf = (float)ay;
    for (int gy = b0; gy <= b1; gy++) {
        const float ry0 = fby0 + (float)(gy - b0) * fch;
        for (int gx = a0; gx <= a1; gx++) {
            float4 r = b;
            bool keep = true;
            if (clip) {
                const float rx0 = fbx0 + (float)(gx - a0) * fcw;
                const float S = Lm + fabsf(rx0) + fabsf(ry0) + fcw + fch + 2.0f * e2f;
                // slack: far above every rounding of the rectangle's
                // placement, of the clip and of the vertices
                const float w = ldexpf(S, -14) + 4.0f * ea;
                const float X0 = rx0 - e2f - w, X1 = rx0 + fcw + e2f + w;
                const float Y0 = ry0 - e2f - w, Y1 = ry0 + fch + e2f + w;
                float4 c;
                keep = tri ? tri_box(V, D, rx, ry, cc, Lm, Dm, d, X0, X1, Y0, Y1, &c)
                           : clip_box<KMAX>(L, len, X0, X1, Y0, Y1, S, ea, &c);
                if (keep) {
                    // back to the frame: the anchor's float32 rounding,
                    // then M and the slack; rounded outward
                    const float px = Mf + 2.0f * w + 2.0f * u * (fabsf(axf) + fabsf(c.x) + fabsf(c.y)) + 1e-30f;
                    const float py = Mf + 2.0f * w + 2.0f * u * (fabsf(ayf) + fabsf(c.z) + fabsf(c.w)) + 1e-30f;
                    r.x = fmaxf(b.x, __fsub_rd(__fadd_rd(axf, c.x), px));
                    r.y = fminf(b.y, __fadd_ru(__fadd_ru(axf, c.y), px));
                    r.z = fmaxf(b.z, __fsub_rd(__fadd_rd(ayf, c.z), py));
                    r.w = fminf(b.w, __fadd_ru(__fadd_ru(ayf, c.w), py));
                }
            }
            if (!keep) continue;
            int64_t g = (int64_t)gy * gnx + gx;
            unsigned long long k = atomicAdd(&count[g], 1ull);
            if (MODE == 1) {
                const int64_t e = off[g] + (int64_t)k;
                if (e >= off[g + 1]) {  // the counting pass decided otherwise: never write past g
                    set_error(err, CT_DEVERR_CAPACITY);
                    continue;
                }
                idx[e] = (int)j;
                lbox[e] = r;
            } else if (MODE == 2) {
                if (kept < CAND_SLOTS) {
                    rec.g[j * CAND_SLOTS + kept] = (int)g;
                    rec.r[j * CAND_SLOTS + kept] = r;
                }
                kept++;
            }
        }
    }
    if (MODE == 2) {
        if (kept > CAND_SLOTS) {
            rec.n[j] = CAND_OVERFLOW;
            rec.ovf[atomicAdd(rec.ovf_count, 1)] = (int)j;
        } else {
            rec.n[j] = (unsigned char)kept;
        }
    }
}

template <int MODE, int KMAX>
__global__ void k_cand_lists(const float4* __restrict__ box, const double2* __restrict__ poly,
                             const uint8_t* __restrict__ plen, int K, int64_t n, double ox, double oy, int gnx,
                             int gny, double x0, double y0, double sx, double sy, double cw, double ch, double m,
                             float Mf, float e2f, float ea, unsigned long long* __restrict__ count,
                             const int64_t* __restrict__ off,
                             int* __restrict__ idx, float4* __restrict__ lbox, unsigned int* __restrict__ err,
                             CandRecs rec, const int* __restrict__ cells, const int* __restrict__ cells_count) {
    const int64_t nj = cells ? (int64_t)*cells_count : n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nj; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = cells ? (int64_t)cells[t] : t;
        cand_cell<MODE, KMAX>(j, box[j], poly, plen, K, ox, oy, gnx, gny, x0, y0, sx, sy, cw, ch, m, Mf, e2f, ea, count,
                              off, idx, lbox, err, rec);
    }
}

// Filling pass from the records: every recorded pair of a cell to its grid
// cell's list (off[g] + cursor); cells that overflowed their slots are left
// to the geometry pass (MODE 1 over rec.ovf).
__global__ void k_cand_scatter(int64_t n, CandRecs rec, unsigned long long* __restrict__ cursor,
                               const int64_t* __restrict__ off, int* __restrict__ idx, float4* __restrict__ lbox,
                               unsigned int* __restrict__ err) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const int c = rec.n[j];
        if (c == CAND_OVERFLOW) continue;
        for (int k = 0; k < c; k++) {
            const int64_t g = rec.g[j * CAND_SLOTS + k];
            const int64_t e = off[g] + (int64_t)atomicAdd(&cursor[g], 1ull);
            if (e >= off[g + 1]) {
                set_error(err, CT_DEVERR_CAPACITY);
                continue;
            }
            idx[e] = (int)j;
            lbox[e] = rec.r[j * CAND_SLOTS + k];
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static inline size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

struct LocWS {
    unsigned* keyA;
    int* order;       // sorted position -> input index (idxA after the last pass)
    unsigned* keyB;
    int* idxB;
    int* ovf;
    int* open;  // sorted positions left open by the candidate-list stage
    Recs R;
    int64_t* hist;
    void* scan_ws;
    size_t scan_bytes;
    int* counters;  // [0] overflow, [1] records, [2] pairs, [3] open after the candidate lists
};

static int rec_cap_for(int64_t n) { return (int)std::min<int64_t>(n / 8 + 4096, (int64_t)INT32_MAX / 8); }

static size_t carve_loc(void* ws, int64_t n, int32_t sort_bits, LocWS* L) {
    size_t nn = (size_t)(n > 0 ? n : 1);
    size_t rc = (size_t)rec_cap_for(n);
    size_t nh = (size_t)256 * RS_BLOCKS;
    size_t off = 0;
    char* base = (char*)ws;
    auto take = [&](size_t b) {
        char* p = base ? base + off : nullptr;
        off += a256(b);
        return p;
    };
    LocWS l;
    bool sorted = sort_bits > 0;
    l.keyA = (unsigned*)take(sorted ? 4 * nn : 16);
    l.order = (int*)take(sorted ? 4 * nn : 16);
    l.keyB = (unsigned*)take(sorted ? 4 * nn : 16);
    l.idxB = (int*)take(sorted ? 4 * nn : 16);
    l.ovf = (int*)take(4 * nn);
    l.open = (int*)take(4 * nn);
    l.R.orig = (int*)take(4 * rc);
    l.R.res = (int64_t*)take(8 * rc);
    l.R.first = (unsigned long long*)take(8 * rc);
    l.R.pairs = (int4*)take(16 * rc * CMAX);
    l.R.cap = (int)rc;
    l.hist = (int64_t*)take(8 * nh);
    l.scan_bytes = ct_scan_workspace_size((int64_t)nh);
    l.scan_ws = take(l.scan_bytes);
    l.counters = (int*)take(64);
    if (L) *L = l;
    return off;
}

static void origin_split(double o, float* hi, float* lo) {
    *hi = (float)o;
    *lo = (float)(o - (double)*hi);
}

// Device-side view of one packed tree for queries at tolerance `tol`.
static int fill_tree(const ct_tree* t, double tol, TreeL* T) {
    if (!t) return ct_fail(CT_ERR_ARG, "tree is null");
    if (t->n_nodes <= 0) return ct_fail(CT_ERR_ARG, "tree has no nodes");
    memset(T, 0, sizeof(*T));
    T->nf = (const float4*)t->nodes_f32;
    T->nd = (const double2*)t->nodes_f64;
    T->poly = (const double2*)t->poly_f64;
    T->polyf = (const float4*)t->poly_f32;
    T->plen = (t->n_max_vert == 3) ? nullptr : t->poly_len;
    T->plen32 = t->poly_len32;
    T->bbi = t->bb_indices;
    T->err = t->error_word;
    T->n_nodes = t->n_nodes;
    T->ox = t->origin[0];
    T->oy = t->origin[1];
    T->dabs = t->abs_eps;
    {
        double F = std::max(std::max(t->bbox[1] - t->origin[0], t->origin[0] - t->bbox[0]),
                            std::max(t->bbox[3] - t->origin[1], t->origin[1] - t->bbox[2]));
        if (!(F >= 0.0) || !std::isfinite(F)) F = 0.0;
        T->bandG = (float)(F * 2.384185791015625e-07 * 1.0001) + 1e-30f;  // bounds are inside the bbox
    }
    T->gstart = (t->grid_start && t->grid_nx > 0 && t->grid_ny > 0) ? t->grid_start : nullptr;
    T->gnx = T->gstart ? t->grid_nx : 0;
    T->gny = T->gstart ? t->grid_ny : 0;
    // candidate lists only when they cover this tolerance
    T->coff = (T->gstart && t->cand_off && t->cand_idx && t->cand_lbox && t->cand_tol > 0.0 && tol <= t->cand_tol)
                  ? t->cand_off
                  : nullptr;
    T->cidx = t->cand_idx;
    T->cbox = (const float4*)t->cand_lbox;
    T->gx0 = t->grid_x0;
    T->gy0 = t->grid_y0;
    T->gsx = t->grid_sx;
    T->gsy = t->grid_sy;
    T->K = t->n_max_vert;
    T->S4 = poly32_stride(t->n_max_vert);
    T->stack = t->max_depth + 2;
    T->tol = tol;
    T->tolf = (float)tol;
    if ((double)T->tolf < tol) T->tolf = nextafterf(T->tolf, INFINITY);
    origin_split(T->ox, &T->ohx, &T->olx);
    origin_split(T->oy, &T->ohy, &T->oly);
    if (T->stack > 128) return ct_fail(CT_ERR_ARG, "tree deeper than 126 levels for the batched form");
    return CT_OK;
}

static int make_tree(const ct_tree* t, int64_t n, int32_t G, double tol, void* ws, size_t ws_bytes, TreeL* T) {
    if (n >= INT32_MAX / 2) return ct_fail(CT_ERR_ARG, "at most 2^30 points per call");
    if (G != 0 && G != 8 && G != 16 && G != 24) return ct_fail(CT_ERR_ARG, "sort_bits must be 0, 8, 16 or 24");
    if (!ws || ws_bytes < carve_loc(nullptr, n, G, nullptr))
        return ct_fail(CT_ERR_WORKSPACE, "locate workspace too small");
    return fill_tree(t, tol, T);
}

template <int KT, bool MULTI>
static void smem_attr(size_t smem) {
    if (smem > 48 * 1024) {
        cudaFuncSetAttribute(k_fast<KT, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_exact<KT, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
}

static Grid morton_grid(const ct_tree* t) {
    Grid g;
    double xmin = t->bbox[0], xmax = t->bbox[1], ymin = t->bbox[2], ymax = t->bbox[3];
    double wx = xmax - xmin, wy = ymax - ymin;
    g.x0 = (float)xmin;
    g.y0 = (float)ymin;
    g.sx = (wx > 0) ? (float)(4096.0 / wx) : 0.0f;
    g.sy = (wy > 0) ? (float)(4096.0 / wy) : 0.0f;
    return g;
}

// Batch of trees: device array of the trees, their Morton grids, the point
// offsets of every tree and the tree of every point, after the LocWS part.
struct ForestWS {
    TreeL* trees;
    Grid* grids;
    int64_t* poff;
    int* qtree;
};

static size_t carve_forest(void* ws, int64_t n, int n_trees, LocWS* L, ForestWS* F) {
    size_t off = carve_loc(ws, n, 32, L);
    char* base = (char*)ws;
    auto take = [&](size_t b) {
        char* p = base ? base + off : nullptr;
        off += a256(b);
        return p;
    };
    ForestWS f;
    f.trees = (TreeL*)take(sizeof(TreeL) * (size_t)n_trees);
    f.grids = (Grid*)take(sizeof(Grid) * (size_t)n_trees);
    f.poff = (int64_t*)take(sizeof(int64_t) * ((size_t)n_trees + 1));
    f.qtree = (int*)take(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (F) *F = f;
    return off;
}

// Results of the candidate-list stage, written by sorted position into the
// sort's key buffer A (free once the permutation is in L.order), scattered to
// out[order[i]] through the sort's key buffer B and index buffer B; the
// bucket cursors reuse the radix histogram.  Needs a sorted workspace.
static int* sorted_results(const LocWS& L) { return (int*)L.keyA; }

// The scatter pays off once one tree's queries span more output than L2
// holds comfortably (2^23 int64 = 64 MB): below that, direct writes from
// k_cells already land in a cache-resident window.
constexpr int64_t RES_SCATTER_MIN = (int64_t)1 << 23;

static int scatter_results(const LocWS& L, int64_t n, unsigned int* err, int64_t* out, cudaStream_t st) {
    int shift = 0;
    while (((n - 1) >> shift) >= 256) shift++;
    CT_CUDA(cudaMemsetAsync(L.hist, 0, 256 * sizeof(int64_t), st));
    k_res_bucket<<<(unsigned)((n + RB_TILE - 1) / RB_TILE), RB_T, 0, st>>>(
        sorted_results(L), L.order, n, shift, (unsigned long long*)L.hist, (int*)L.keyB, L.idxB, err);
    k_res_unbucket<<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const int*)L.keyB, L.idxB, n, out);
    return CT_OK;
}

// ---------------------------------------------------------------------------
// Device-side index of a batch built by ct_build_forest_async: the per-tree
// summaries and records that ct_bbox_summary, ct_pack_tree, ct_pack_grid and
// ct_forest_locate_prepare derive on the host for single trees, computed
// here so that no value has to come back to the host between the build and
// the locate.
// ---------------------------------------------------------------------------
constexpr int FX_WORDS = 16;  // summary words per tree: 5 reduction keys, grid margin, grid cell sizes,
                              // candidate-list reach

// Stand-in tree of a build that overflowed its node capacity (its node
// ranges are not usable): one empty leaf, so that every query of the batch
// ends at once with -1 while the error word reports the overflow.
__device__ float4 g_fx_empty_leaf = {0.0f, 0.0f, 0.0f, 0.0f};
__device__ double2 g_fx_empty_bounds = {0.0, 0.0};

// std::max as the host computes it ((a < b) ? b : a)
__device__ __forceinline__ double hmax(double a, double b) { return (a < b) ? b : a; }

// Tree of row r of a batch: the largest t with off[t] <= r (trees with no
// rows share their offset with the next tree).
__device__ __forceinline__ int tree_of_row(const int64_t* __restrict__ off, int n_trees, int64_t r) {
    int lo = 0, hi = n_trees - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= r) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_fx_reset(unsigned long long* __restrict__ summary, int n_trees, unsigned int* __restrict__ err) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)n_trees * FX_WORDS;
         i += (int64_t)gridDim.x * blockDim.x)
        summary[i] = ~0ull;
    if (blockIdx.x == 0 && threadIdx.x == 0 && err) *err = 0u;
}

// Per-tree bbox and largest box diagonal (bbox_tree / bbox_distances,
// celltree_base.py:20-48) as order-preserving keys reduced with atomicMin;
// a warp whose rows all belong to one tree reduces in registers first.
__global__ void k_fx_summary(const double* __restrict__ bb, int64_t n, const int64_t* __restrict__ tree_off,
                             int n_trees, unsigned long long* __restrict__ summary, unsigned int* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int64_t i = base + lane;
        const bool valid = i < n;
        unsigned long long k[5] = {~0ull, ~0ull, ~0ull, ~0ull, ~0ull};
        int t = -1;
        if (valid) {
            t = tree_of_row(tree_off, n_trees, i);
            double4 b = reinterpret_cast<const double4*>(bb)[i];
            if (!isfinite(b.x) || !isfinite(b.y) || !isfinite(b.z) || !isfinite(b.w))
                set_error(err, CT_DEVERR_NONFINITE);
            k[0] = fkey(b.x);
            k[1] = ~fkey(b.y);
            k[2] = fkey(b.z);
            k[3] = ~fkey(b.w);
            k[4] = ~fkey(box_diagonal(b.y - b.x, b.w - b.z));
        }
        const int t0 = __shfl_sync(0xffffffffu, t, 0);  // lane 0 is valid (base < n)
        if (__all_sync(0xffffffffu, !valid || t == t0)) {
            for (int j = 0; j < 5; j++) {
                unsigned long long m = k[j];
                for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
                if (lane == 0) atomicMin(&summary[(int64_t)t0 * FX_WORDS + j], m);
            }
        } else if (valid) {
            for (int j = 0; j < 5; j++) atomicMin(&summary[(int64_t)t * FX_WORDS + j], k[j]);
        }
    }
}

// One thread per tree: the tree record of the batched locate (the fields
// fill_tree takes from a packed ct_tree), its Morton grid, and the margin of
// its start-node grid (summary word 5).
__global__ void k_fx_records(const __grid_constant__ ct_forest_index X, TreeL* __restrict__ trees,
                             Grid* __restrict__ grids) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= X.n_trees) return;
    unsigned long long* S = X.summary + (int64_t)t * FX_WORDS;
    const double b0 = fkey_inv(S[0]), b1 = fkey_inv(~S[1]), b2 = fkey_inv(S[2]), b3 = fkey_inv(~S[3]);
    const double diag = fkey_inv(~S[4]);
    const int64_t e0 = X.tree_off[t];
    const int K = X.tree_K[t];
    // origin: bbox centre (ct_pack_tree)
    double ox = 0.5 * (b0 + b1), oy = 0.5 * (b2 + b3);
    if (!isfinite(ox) || !isfinite(oy)) {
        ox = 0.0;
        oy = 0.0;
    }
    TreeL T;
    memset(&T, 0, sizeof(T));
    T.nf = (const float4*)X.nodes_f32 + X.node_off[t];
    T.nd = (const double2*)X.nodes_f64 + X.node_off[t];
    T.poly = (const double2*)X.poly_f64 + X.face_off[t];
    T.polyf = (const float4*)X.poly_f32 + X.poly32_off[t];
    T.plen = (K == 3) ? nullptr : X.poly_len + e0;
    T.plen32 = X.poly_len32 + e0;
    T.bbi = X.bb_indices + e0;
    T.err = X.error_word;
    T.n_nodes = X.node_off[t + 1] - X.node_off[t];
    const bool over = X.node_off[X.n_trees] > X.node_capacity;
    if (over) {
        set_error(X.error_word, CT_DEVERR_CAPACITY);
        T.nf = &g_fx_empty_leaf;
        T.nd = &g_fx_empty_bounds;
        T.n_nodes = 1;
    }
    T.ox = ox;
    T.oy = oy;
    double amax = hmax(hmax(fabs(b0), fabs(b1)), hmax(fabs(b2), fabs(b3)));
    if (!isfinite(amax)) amax = 0.0;
    T.dabs = __double2float_rn(amax * 8.881784197001252e-16) + 1e-30f;
    const double F = hmax(hmax(b1 - ox, ox - b0), hmax(b3 - oy, oy - b2));
    const double Fb = (!(F >= 0.0) || !isfinite(F)) ? 0.0 : F;
    T.bandG = __double2float_rn(Fb * 2.384185791015625e-07 * 1.0001) + 1e-30f;
    // start-node grid of the caller's shape over this build's bbox (ct_pack_grid)
    const int gnx = X.grid_nx[t], gny = X.grid_ny[t];
    const double ex = b1 - b0, ey = b3 - b2;
    bool grid_ok = !over && gnx > 0 && gny > 0 && ex > 0.0 && ey > 0.0 && isfinite(ex) && isfinite(ey) && isfinite(F);
    if (grid_ok) {
        T.gx0 = __double2float_rn(b0 - ox);
        T.gy0 = __double2float_rn(b2 - oy);
        T.gsx = __double2float_rn((double)gnx / ex);
        T.gsy = __double2float_rn((double)gny / ey);
        grid_ok = T.gsx > 0.0f && T.gsy > 0.0f && isfinite(T.gsx) && isfinite(T.gsy);
    }
    T.gstart = grid_ok ? X.grid_start + X.grid_off[t] : nullptr;
    T.gnx = grid_ok ? gnx : 0;
    T.gny = grid_ok ? gny : 0;
    S[5] = (unsigned long long)__double_as_longlong(grid_ok ? ldexp(hmax(ex, ey) + F, -19) : 0.0);
    S[6] = (unsigned long long)__double_as_longlong(grid_ok ? 1.0 / (double)T.gsx : 0.0);  // grid cell sizes
    S[7] = (unsigned long long)__double_as_longlong(grid_ok ? 1.0 / (double)T.gsy : 0.0);
    T.coff = nullptr;  // no candidate lists
    T.K = K;
    T.S4 = poly32_stride(K);
    const int need = X.max_depth[t] + 2;
    if (need > X.stack) set_error(X.error_word, CT_DEVERR_STACK);
    T.stack = need < X.stack ? need : X.stack;
    // query tolerance: the given one, or default_tolerance (celltree_base.py:51-52)
    double tol = X.tolerance;
    if (!(tol > 0.0)) {
        const double d = 1e-12 * diag;
        tol = (d > 1e-15) ? d : 1e-15;
    }
    T.tol = tol;
    T.tolf = __double2float_ru(tol);
    // reach of the candidate lists built for this tolerance (cand_reach)
    S[8] = (unsigned long long)__double_as_longlong(grid_ok ? 2.0 * tol * (1.0 + 1e-6) + 16.0 * (double)T.dabs +
                                                                  ldexp(F, -48)
                                                            : 0.0);
    T.ohx = __double2float_rn(ox);
    T.olx = __double2float_rn(ox - (double)T.ohx);
    T.ohy = __double2float_rn(oy);
    T.oly = __double2float_rn(oy - (double)T.ohy);
    trees[t] = T;
    // Morton grid of the query sort (morton_grid)
    Grid g;
    g.x0 = __double2float_rn(b0);
    g.y0 = __double2float_rn(b2);
    g.sx = (ex > 0.0) ? __double2float_rn(4096.0 / ex) : 0.0f;
    g.sy = (ey > 0.0) ? __double2float_rn(4096.0 / ey) : 0.0f;
    grids[t] = g;
}

// Packed nodes of every tree (k_pack_nodes over the batch): node v of the
// batch belongs to the tree whose node range holds it; child and ptr are
// relative to the tree.  The structure check of k_pack_nodes (children after
// their parent and inside the tree, leaf ranges inside the tree's cells)
// turns a bad node into an empty leaf and reports it, so that no traversal
// leaves the tree's arrays.
__global__ void k_fx_pack_nodes(const __grid_constant__ ct_forest_index X, const TreeL* __restrict__ trees) {
    const int64_t total = X.node_off[X.n_trees];
    if (total > X.node_capacity) return;  // overflowed build: the records use the stand-in tree
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < total; v += (int64_t)gridDim.x * blockDim.x) {
        const int t = tree_of_row(X.node_off, X.n_trees, v);
        const int64_t local = v - X.node_off[t], nn = X.node_off[t + 1] - X.node_off[t];
        const int64_t rows = X.tree_off[t + 1] - X.tree_off[t];
        const double L = X.node_Lmax[v], R = X.node_Rmin[v];
        if (!isfinite(L) || !isfinite(R)) set_error(X.error_word, CT_DEVERR_NONFINITE);
        reinterpret_cast<double2*>(X.nodes_f64)[v] = make_double2(L, R);
        int64_t c = X.node_child[v];
        const bool bad = (c != -1 && (c <= local || c + 1 >= nn)) ||
                         (c == -1 && (X.node_ptr[v] < 0 || X.node_size[v] < 0 || X.node_ptr[v] + X.node_size[v] > rows));
        float4 q;
        if (bad) {
            set_error(X.error_word, CT_DEVERR_CAPACITY);
            q = make_float4(0.f, 0.f, 0.f, 0.f);  // empty leaf
        } else if (c == -1) {
            q.x = 0.f;
            q.y = 0.f;
            q.z = __int_as_float((int)X.node_ptr[v]);
            q.w = __int_as_float((int)X.node_size[v]);
        } else {
            const int d = X.node_dim[v] ? 1 : 0;
            const double o = d ? trees[t].oy : trees[t].ox;
            q.x = __double2float_ru(L - o);
            q.y = __double2float_rd(R - o);
            q.z = __int_as_float((int)c);
            q.w = __int_as_float(-1 - d);
        }
        reinterpret_cast<float4*>(X.nodes_f32)[v] = q;
    }
}

// Leaf-ordered cells of every tree (k_pack_polys over the batch).
__global__ void k_fx_pack_cells(const __grid_constant__ ct_forest_index X) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < X.n_total;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int t = tree_of_row(X.tree_off, X.n_trees, p);
        const int64_t j = p - X.tree_off[t];
        const int K = X.tree_K[t];
        const int64_t b = X.bb_indices[p];
        if (b < 0 || b >= X.tree_off[t + 1] - X.tree_off[t]) {  // only after an overflowed build
            set_error(X.error_word, CT_DEVERR_CAPACITY);
            X.poly_len[p] = 0;
            X.poly_len32[p] = 0;
            continue;
        }
        pack_cell(X.faces + X.face_off[t] + b * K, K, false, X.vertices, (double2*)X.poly_f64 + X.face_off[t] + j * K,
                  (float4*)X.poly_f32 + X.poly32_off[t] + j * poly32_stride(K), X.poly_len + p, X.poly_len32 + p);
    }
}

// Start nodes of every tree's grid (k_grid_start over the batch).
__global__ void k_fx_grid_start(const __grid_constant__ ct_forest_index X, const TreeL* __restrict__ trees) {
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < X.grid_cells;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int t = tree_of_row(X.grid_off, X.n_trees, c);
        const TreeL& T = trees[t];
        if (!T.gstart) {
            X.grid_start[c] = 0;  // grid off for this build: queries start at the root
            continue;
        }
        const int64_t local = c - X.grid_off[t];
        const double m = __longlong_as_double((long long)X.summary[(int64_t)t * FX_WORDS + 5]);
        const double cw = __longlong_as_double((long long)X.summary[(int64_t)t * FX_WORDS + 6]);
        const double ch = __longlong_as_double((long long)X.summary[(int64_t)t * FX_WORDS + 7]);
        X.grid_start[c] = grid_cell_start(T.nf, (int)(local % T.gnx), (int)(local / T.gnx), T.gx0, T.gy0, cw, ch, m,
                                          T.bandG, X.max_depth[t] + 2);
    }
}

// Candidate lists of every tree (k_cand_box / k_cand_lists over the batch):
// the widened box of each cell, then the counting (MODE 0) or filling
// (MODE 1) pass with the cell's tree parameters; grid cell g of tree t is
// entry grid_off[t] + g of the batch-wide counts and offsets, and an entry
// stores the cell's leaf position within its tree.
__global__ void k_fx_cand_box(const __grid_constant__ ct_forest_index X, const TreeL* __restrict__ trees) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < X.n_total;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int t = tree_of_row(X.tree_off, X.n_trees, p);
        const TreeL& T = trees[t];
        const double M = __longlong_as_double((long long)X.summary[(int64_t)t * FX_WORDS + 8]);
        const int64_t bi = X.bb_indices[p];
        const int64_t rows = X.tree_off[t + 1] - X.tree_off[t];
        if (!T.gstart || bi < 0 || bi >= rows) continue;
        const double* b = X.bb_coords + 4 * (X.tree_off[t] + bi);
        reinterpret_cast<float4*>(X.cand_box)[p] =
            make_float4(__double2float_rd((b[0] - T.ox) - M), __double2float_ru((b[1] - T.ox) + M),
                        __double2float_rd((b[2] - T.oy) - M), __double2float_ru((b[3] - T.oy) + M));
    }
}

template <int MODE>
__global__ void k_fx_cand_lists(const __grid_constant__ ct_forest_index X, const TreeL* __restrict__ trees) {
    if (MODE == 1 && X.cand_off[X.grid_cells] > X.cand_capacity) return;  // lists off for this build
    CandRecs none;
    memset(&none, 0, sizeof(none));
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < X.n_total;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int t = tree_of_row(X.tree_off, X.n_trees, p);
        const TreeL& T = trees[t];
        if (!T.gstart) continue;  // no grid for this build: no lists
        const unsigned long long* S = X.summary + (int64_t)t * FX_WORDS;
        const double m = __longlong_as_double((long long)S[5]);
        const double cw = __longlong_as_double((long long)S[6]), ch = __longlong_as_double((long long)S[7]);
        const double M = __longlong_as_double((long long)S[8]);
        const float Mf = __double2float_ru(M), e2f = __double2float_ru(m + M);
        const float ea = __double2float_rn(4.0 * (double)T.dabs);
        const int64_t j = p - X.tree_off[t];
        const int64_t go = X.grid_off[t];
        const float4 b = reinterpret_cast<const float4*>(X.cand_box)[p];
        unsigned long long* count = X.cand_count + go;
        const int64_t* off = MODE == 1 ? X.cand_off + go : nullptr;
        if (T.K <= 4)
            cand_cell<MODE, 4>(j, b, T.poly, T.plen, T.K, T.ox, T.oy, T.gnx, T.gny, (double)T.gx0, (double)T.gy0,
                               (double)T.gsx, (double)T.gsy, cw, ch, m, Mf, e2f, ea, count, off, X.cand_idx,
                               (float4*)X.cand_lbox, X.error_word, none);
        else
            cand_cell<MODE, 32>(j, b, T.poly, T.plen, T.K, T.ox, T.oy, T.gnx, T.gny, (double)T.gx0, (double)T.gy0,
                                (double)T.gsx, (double)T.gsy, cw, ch, m, Mf, e2f, ea, count, off, X.cand_idx,
                                (float4*)X.cand_lbox, X.error_word, none);
    }
}

// Lists on for every tree with a grid when the batch's entries fit.
__global__ void k_fx_cand_enable(const __grid_constant__ ct_forest_index X, TreeL* __restrict__ trees) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= X.n_trees || !trees[t].gstart) return;
    if (X.cand_off[X.grid_cells] > X.cand_capacity) return;
    trees[t].coff = X.cand_off + X.grid_off[t];
    trees[t].cidx = X.cand_idx;
    trees[t].cbox = (const float4*)X.cand_lbox;
}

}  // namespace ctl

using namespace ctl;

extern "C" {

int ct_poly32_stride(int32_t K) { return poly32_stride(K); }

size_t ct_abi_sizeof(int32_t which) {
    switch (which) {
        case 0: return sizeof(ct_tree);
        case 1: return sizeof(ct_forest_plan);
        case 2: return sizeof(ct_forest_index);
        default: return 0;
    }
}

int ct_grid_shape(int64_t n_elements, double width, double height, double cells_per_element, int32_t* nx,
                  int32_t* ny) {
    if (!nx || !ny) return ct_fail(CT_ERR_ARG, "null argument");
    if (!(cells_per_element > 0.0) || !std::isfinite(cells_per_element))
        return ct_fail(CT_ERR_ARG, "cells_per_element must be finite and > 0");
    double target = std::min(std::max((double)std::max<int64_t>(n_elements, 0) * cells_per_element, 256.0),
                             (double)(1 << 26));
    double a = width / height;  // aspect; 1 for a degenerate bbox (the grid is then switched off)
    if (!(a > 0.0) || !std::isfinite(a)) a = 1.0;
    a = std::min(std::max(a, 1.0 / 4096.0), 4096.0);
    const double sx = std::sqrt(target * a), sy = std::sqrt(target / a);  // ideal cells per axis
    int64_t gx = std::min<int64_t>(65536, std::max<int64_t>(16, (int64_t)std::llround(sx)));
    int64_t gy = std::min<int64_t>(65536, std::max<int64_t>(16, (int64_t)std::llround(sy)));
    // rounding (or the minimum of 16 on one axis) can step over the cap:
    // drop a row or column of the axis furthest above its ideal count
    while (gx * gy > ((int64_t)1 << 26) && (gx > 16 || gy > 16)) {
        if (gy <= 16 || (gx > 16 && (double)gx * sy >= (double)gy * sx)) gx--;
        else gy--;
    }
    *nx = (int32_t)gx;
    *ny = (int32_t)gy;
    return CT_OK;
}

int ct_pack_grid(ct_tree* t, void* stream) {
    if (!t) return ct_fail(CT_ERR_ARG, "tree is null");
    if (!t->grid_start || t->grid_nx <= 0 || t->grid_ny <= 0) {
        t->grid_nx = t->grid_ny = 0;
        return CT_OK;
    }
    if (t->grid_nx > 65536 || t->grid_ny > 65536 || (int64_t)t->grid_nx * t->grid_ny > ((int64_t)1 << 28))
        return ct_fail(CT_ERR_ARG, "grid too large");
    if (t->n_nodes <= 0 || !t->nodes_f32) return ct_fail(CT_ERR_ARG, "tree is not packed");
    double ex = t->bbox[1] - t->bbox[0], ey = t->bbox[3] - t->bbox[2];
    double F = std::max(std::max(t->bbox[1] - t->origin[0], t->origin[0] - t->bbox[0]),
                        std::max(t->bbox[3] - t->origin[1], t->origin[1] - t->bbox[2]));
    if (!(ex > 0.0 && ey > 0.0) || !std::isfinite(ex) || !std::isfinite(ey) || !std::isfinite(F)) {
        t->grid_nx = t->grid_ny = 0;  // degenerate bbox: every query starts at the root
        return CT_OK;
    }
    const int gnx = t->grid_nx, gny = t->grid_ny;
    t->grid_x0 = (float)(t->bbox[0] - t->origin[0]);
    t->grid_y0 = (float)(t->bbox[2] - t->origin[1]);
    t->grid_sx = (float)(gnx / ex);
    t->grid_sy = (float)(gny / ey);
    if (!(t->grid_sx > 0.0f && t->grid_sy > 0.0f && std::isfinite(t->grid_sx) && std::isfinite(t->grid_sy))) {
        t->grid_nx = t->grid_ny = 0;
        return CT_OK;
    }
    // margin over the cell of a point: float32 rounding of the point in the
    // frame and of (p - x0) * s is below 2^-21 (extent + F); 4x that
    double m = std::ldexp(std::max(ex, ey) + F, -19);
    float band = (float)(F * 2.384185791015625e-07 * 1.0001) + 1e-30f;
    int64_t total = (int64_t)gnx * gny;
    unsigned blocks = (unsigned)std::min<int64_t>((total + 255) / 256, 152 * 16);
    k_grid_start<<<blocks, 256, 0, (cudaStream_t)stream>>>((const float4*)t->nodes_f32, gnx, gny, t->grid_x0,
                                                          t->grid_y0, 1.0 / (double)t->grid_sx,
                                                          1.0 / (double)t->grid_sy, m, band, t->max_depth + 2,
                                                          t->grid_start);
    CT_CHECK_LAUNCH("pack grid");
    return CT_OK;
}

// cell-assignment margin of the grid (same bound as the start-node grid)
static double grid_margin(const ct_tree* t) {
    double ex = t->bbox[1] - t->bbox[0], ey = t->bbox[3] - t->bbox[2];
    double F = std::max(std::max(t->bbox[1] - t->origin[0], t->origin[0] - t->bbox[0]),
                        std::max(t->bbox[3] - t->origin[1], t->origin[1] - t->bbox[2]));
    return std::ldexp(std::max(ex, ey) + F, -19);
}

// Scratch of the candidate lists: grid-cell counts (then cursors), the scan's
// workspace, and the counting pass's records.
struct CandScratch {
    unsigned long long* count;
    void* scan_ws;
    size_t scan_bytes;
    CandRecs rec;
};

static size_t carve_cand(const ct_tree* t, void* scratch, CandScratch* C) {
    const int64_t cells = (int64_t)t->grid_nx * t->grid_ny;
    const size_t n = (size_t)std::max<int64_t>(t->n_elements, 1);
    char* base = (char*)scratch;
    size_t off = 0;
    auto take = [&](size_t b) {
        char* p = base ? base + off : nullptr;
        off += a256(b);
        return p;
    };
    CandScratch c;
    c.count = (unsigned long long*)take(8 * (size_t)(cells + 1));
    c.scan_bytes = ct_scan_workspace_size(cells + 1);
    c.scan_ws = take(c.scan_bytes);
    c.rec.g = (int*)take(sizeof(int) * CAND_SLOTS * n);
    c.rec.r = (float4*)take(sizeof(float4) * CAND_SLOTS * n);
    c.rec.n = (unsigned char*)take(n);
    c.rec.ovf = (int*)take(sizeof(int) * n);
    c.rec.ovf_count = (int*)take(sizeof(int));
    if (C) *C = c;
    return off + 256;
}

size_t ct_cand_scratch_size(const ct_tree* t) {
    if (!t || t->grid_nx <= 0 || t->grid_ny <= 0) return 256;
    return carve_cand(t, nullptr, nullptr);
}

// widening of the region where a cell's predicate can be true: the on-edge
// test reaches 2 tol beyond an edge's bbox; float64 rounding of the
// coordinates (abs_eps each) moves the tests by a few ulp
static double cand_reach(const ct_tree* t, double cover_tol) {
    double F = std::max(std::max(t->bbox[1] - t->origin[0], t->origin[0] - t->bbox[0]),
                        std::max(t->bbox[3] - t->origin[1], t->origin[1] - t->bbox[2]));
    return 2.0 * cover_tol * (1.0 + 1e-6) + 16.0 * (double)t->abs_eps + std::ldexp(F, -48);
}

// v rounded up to float32
static float float_up(double v) {
    float f = (float)v;
    if ((double)f < v) f = std::nextafter(f, INFINITY);
    return f;
}

// Counting-and-recording pass (fill = false) or the geometry filling pass
// over the cells that overflowed their record slots (fill = true).
static void launch_cand_lists(const ct_tree* t, bool fill, double M, const CandScratch& C, cudaStream_t st) {
    int64_t n = t->n_elements;
    unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
    const uint8_t* plen = (t->n_max_vert == 3) ? nullptr : t->poly_len;
#define CT_CAND_LISTS(MODE, KMAX)                                                                                  \
    k_cand_lists<MODE, KMAX><<<blocks, 256, 0, st>>>(                                                              \
        (const float4*)t->cand_box, (const double2*)t->poly_f64, plen, t->n_max_vert, n, t->origin[0],             \
        t->origin[1], t->grid_nx, t->grid_ny, t->grid_x0, t->grid_y0, t->grid_sx, t->grid_sy,                     \
        1.0 / (double)t->grid_sx, 1.0 / (double)t->grid_sy, grid_margin(t),                                       \
        float_up(M), float_up(grid_margin(t) + M), (float)(4.0 * (double)t->abs_eps),                             \
        C.count, MODE == 1 ? t->cand_off : nullptr, MODE == 1 ? t->cand_idx : nullptr,                             \
        MODE == 1 ? (float4*)t->cand_lbox : nullptr, t->error_word, C.rec, MODE == 1 ? C.rec.ovf : nullptr,         \
        C.rec.ovf_count)
    if (t->n_max_vert <= 4) {
        if (fill) CT_CAND_LISTS(1, 4);
        else CT_CAND_LISTS(2, 4);
    } else {
        if (fill) CT_CAND_LISTS(1, 32);
        else CT_CAND_LISTS(2, 32);
    }
#undef CT_CAND_LISTS
}

int ct_cand_count(ct_tree* t, double cover_tol, void* scratch, size_t scratch_bytes, int64_t* total_host,
                  void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!t || !total_host) return ct_fail(CT_ERR_ARG, "null argument");
    *total_host = 0;
    t->cand_n = 0;
    t->cand_tol = 0.0;
    if (t->grid_nx <= 0 || t->grid_ny <= 0 || !t->grid_start) return CT_OK;  // no grid: lists off
    if (!t->cand_off || !t->cand_box) return ct_fail(CT_ERR_ARG, "cand_off / cand_box not set");
    if (!t->poly_f64) return ct_fail(CT_ERR_ARG, "tree is not packed");
    if (!(cover_tol >= 0.0) || !std::isfinite(cover_tol)) return ct_fail(CT_ERR_ARG, "cover_tol must be finite and >= 0");
    if (!scratch || scratch_bytes < ct_cand_scratch_size(t)) return ct_fail(CT_ERR_WORKSPACE, "scratch too small");
    const int64_t cells = (int64_t)t->grid_nx * t->grid_ny;
    CandScratch C;
    carve_cand(t, scratch, &C);  // counts: cells + 1 entries, the last stays 0
    const double M = cand_reach(t, cover_tol);
    int64_t n = t->n_elements;
    unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
    k_cand_box<<<blocks, 256, 0, st>>>(t->bb_coords, t->bb_indices, n, t->origin[0], t->origin[1], M,
                                       (float4*)t->cand_box);
    CT_CUDA(cudaMemsetAsync(C.count, 0, 8 * (size_t)(cells + 1), st));
    CT_CUDA(cudaMemsetAsync(C.rec.ovf_count, 0, sizeof(int), st));
    launch_cand_lists(t, false, M, C, st);
    CT_CHECK_LAUNCH("candidate counts");
    int64_t total = 0;
    int s = ct_exclusive_scan((const int64_t*)C.count, cells + 1, t->cand_off, C.scan_ws, C.scan_bytes, &total,
                              stream);
    if (s) return s;
    if (total > INT32_MAX) return CT_OK;  // too many entries for int offsets of the pairs: lists off
    t->cand_n = total;
    t->cand_tol = cover_tol > 0.0 ? cover_tol : 1e-300;
    *total_host = total;
    return CT_OK;
}

int ct_cand_fill(ct_tree* t, void* scratch, size_t scratch_bytes, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!t) return ct_fail(CT_ERR_ARG, "tree is null");
    if (t->cand_tol <= 0.0 || t->grid_nx <= 0 || t->grid_ny <= 0) return CT_OK;
    if ((!t->cand_idx || !t->cand_lbox) && t->cand_n > 0) return ct_fail(CT_ERR_ARG, "cand_idx / cand_lbox not set");
    if (!scratch || scratch_bytes < ct_cand_scratch_size(t)) return ct_fail(CT_ERR_WORKSPACE, "scratch too small");
    const int64_t cells = (int64_t)t->grid_nx * t->grid_ny;
    CandScratch C;
    carve_cand(t, scratch, &C);
    CT_CUDA(cudaMemsetAsync(C.count, 0, 8 * (size_t)cells, st));  // now the lists' cursors
    const int64_t n = t->n_elements;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
    k_cand_scatter<<<blocks, 256, 0, st>>>(n, C.rec, C.count, t->cand_off, t->cand_idx, (float4*)t->cand_lbox,
                                           t->error_word);
    const double cover = (t->cand_tol == 1e-300) ? 0.0 : t->cand_tol;  // the count's cover_tol
    launch_cand_lists(t, true, cand_reach(t, cover), C, st);  // cells with more pairs than record slots
    CT_CHECK_LAUNCH("candidate lists");
    return CT_OK;
}

size_t ct_locate_workspace_size(int64_t n, int32_t sort_bits) {
    if (sort_bits != 0 && sort_bits != 8 && sort_bits != 16 && sort_bits != 24) return 0;
    return carve_loc(nullptr, n, sort_bits, nullptr);
}

// Stage 1: order the queries along a Morton curve over the tree bbox (4096 x
// 4096 grid): the top `sort_bits` bits of the 24-bit key, LSD radix sort with
// 8-bit digits; the last pass writes the permutation (the points stay where
// they are).  No-op when sort_bits == 0.
int ct_locate_bin(const ct_tree* t, const double* points, int64_t n, int32_t sort_bits, void* ws, size_t ws_bytes,
                  void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    TreeL T;
    int s = make_tree(t, n, sort_bits, 0.0, ws, ws_bytes, &T);
    if (s) return s;
    if (n == 0 || sort_bits == 0) return CT_OK;
    LocWS L;
    carve_loc(ws, n, sort_bits, &L);
    Grid g = morton_grid(t);
    int passes = sort_bits / 8;
    // ping-pong so that the last pass writes the permutation into L.order
    unsigned* kin = (passes & 1) ? L.keyB : L.keyA;
    int* iin = (passes & 1) ? L.idxB : L.order;
    unsigned* kout = (passes & 1) ? L.keyA : L.keyB;
    int* iout = (passes & 1) ? L.order : L.idxB;
    int64_t chunk = (n + RS_BLOCKS - 1) / RS_BLOCKS;
    chunk = (chunk + RS_TILE - 1) / RS_TILE * RS_TILE;
    const int64_t nh = (int64_t)256 * RS_BLOCKS;
    for (int pss = 0; pss < passes; pss++) {
        int shift = 24 - sort_bits + 8 * pss;
        // the pass before the last writes the last digit as one byte
        const bool byte_in = pss > 0 && pss + 1 == passes, byte_out = pss + 2 == passes;
        if (pss == 0)
            k_keys<<<RS_BLOCKS, RS_T, 0, st>>>((const double2*)points, n, chunk, g, shift, kin, L.hist);
        else if (byte_in)
            k_rs_hist8<<<RS_BLOCKS, RS_T, 0, st>>>((const uint8_t*)kin, n, chunk, L.hist);
        else
            k_rs_hist<<<RS_BLOCKS, RS_T, 0, st>>>(kin, n, chunk, shift, L.hist);
        s = ct_exclusive_scan(L.hist, nh, L.hist, L.scan_ws, L.scan_bytes, nullptr, stream);
        if (s) return s;
        const int* ii = pss ? iin : nullptr;
        if (byte_in)  // last pass: indices only
            k_rs_scatter<uint8_t, uint8_t><<<RS_BLOCKS, RS_T, 0, st>>>((const uint8_t*)kin, ii, n, chunk, 0, L.hist,
                                                                       nullptr, 0, iout);
        else if (byte_out)
            k_rs_scatter<unsigned, uint8_t><<<RS_BLOCKS, RS_T, 0, st>>>(kin, ii, n, chunk, shift, L.hist,
                                                                        (uint8_t*)kout, shift + 8, iout);
        else
            k_rs_scatter<unsigned, unsigned><<<RS_BLOCKS, RS_T, 0, st>>>(
                kin, ii, n, chunk, shift, L.hist, pss + 1 < passes ? kout : nullptr, 0, iout);
        std::swap(kin, kout);
        std::swap(iin, iout);
    }
    CT_CHECK_LAUNCH("locate order");
    return CT_OK;
}

int ct_locate_fast(const ct_tree* t, const double* points, int64_t n, double tol, int32_t G, int64_t* out, void* ws,
                   size_t ws_bytes, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    TreeL T;
    int s = make_tree(t, n, G, tol, ws, ws_bytes, &T);
    if (s) return s;
    LocWS L;
    carve_loc(ws, n, G, &L);
    CT_CUDA(cudaMemsetAsync(L.counters, 0, 64, st));
    if (n == 0) return CT_OK;
    const double2* P = (const double2*)points;
    const int* ord = G > 0 ? L.order : nullptr;
    size_t smem = (size_t)T.stack * LOC_THREADS * sizeof(int);
    unsigned grid = (unsigned)((n + LOC_THREADS - 1) / LOC_THREADS);
    // stage 2a (candidate lists) when they cover this tolerance; stage 2b
    // then traverses only the queries left open
    const bool lists = T.coff != nullptr;
    const int* qlist = lists ? L.open : nullptr;
    const int* qcount = lists ? &L.counters[3] : nullptr;
    const int cells_bpsm = t->tune_cells_bpsm;
    int sms = 152;
    {
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    const int fast_bpsm = (t->tune_fast_bpsm >= 1 && t->tune_fast_bpsm <= 32) ? t->tune_fast_bpsm : 16;
    unsigned grid_b =
        lists ? (unsigned)std::min<int64_t>((n + LOC_THREADS - 1) / LOC_THREADS, (int64_t)sms * fast_bpsm) : grid;
    // many sorted queries: list results by sorted position, then one bucketed scatter
    int* res_sorted = (lists && ord && n > RES_SCATTER_MIN) ? sorted_results(L) : nullptr;
#define CT_FAST_STAGES(KT)                                                                                        \
    if (lists) {                                                                                                   \
        if (cells_bpsm == 4)                                                                                       \
            k_cells<KT, false, 4><<<grid, LOC_THREADS, 0, st>>>(T, nullptr, nullptr, P, ord, n, out, res_sorted,   \
                                                                L.open, &L.counters[3]);                           \
        else if (cells_bpsm == 8)                                                                                  \
            k_cells<KT, false, 8><<<grid, LOC_THREADS, 0, st>>>(T, nullptr, nullptr, P, ord, n, out, res_sorted,   \
                                                                L.open, &L.counters[3]);                           \
        else                                                                                                       \
            k_cells<KT, false, 6><<<grid, LOC_THREADS, 0, st>>>(T, nullptr, nullptr, P, ord, n, out, res_sorted,   \
                                                                L.open, &L.counters[3]);                           \
    }                                                                                                              \
    smem_attr<KT, false>(smem);                                                                                    \
    k_fast<KT, false><<<grid_b, LOC_THREADS, smem, st>>>(T, nullptr, nullptr, P, ord, n, out, L.R, L.counters,    \
                                                         L.ovf, qlist, qcount);
    if (T.K == 3) {
        CT_FAST_STAGES(3)
    } else if (T.K == 4) {
        CT_FAST_STAGES(4)
    } else {
        CT_FAST_STAGES(32)
    }
#undef CT_FAST_STAGES
    if (res_sorted) scatter_results(L, n, T.err, out, st);
    CT_CHECK_LAUNCH("locate fast");
    return CT_OK;
}

int ct_locate_exact(const ct_tree* t, const double* points, int64_t n, double tol, int32_t G, int64_t* out, void* ws,
                    size_t ws_bytes, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    TreeL T;
    int s = make_tree(t, n, G, tol, ws, ws_bytes, &T);
    if (s) return s;
    if (n == 0) return CT_OK;
    LocWS L;
    carve_loc(ws, n, G, &L);
    const double2* P = (const double2*)points;
    k_pip<false><<<GRID_STRIDE, LOC_THREADS, 0, st>>>(T, nullptr, nullptr, P, L.R, L.counters);
    k_resolve<false><<<GRID_STRIDE, LOC_THREADS, 0, st>>>(T, nullptr, nullptr, L.R, L.counters, out);
    size_t smem = (size_t)T.stack * LOC_THREADS * sizeof(int);
    if (T.K == 3)
        k_exact<3, false><<<GRID_STRIDE, LOC_THREADS, smem, st>>>(T, nullptr, nullptr, P, L.ovf, L.counters, out);
    else if (T.K == 4)
        k_exact<4, false><<<GRID_STRIDE, LOC_THREADS, smem, st>>>(T, nullptr, nullptr, P, L.ovf, L.counters, out);
    else
        k_exact<32, false><<<GRID_STRIDE, LOC_THREADS, smem, st>>>(T, nullptr, nullptr, P, L.ovf, L.counters, out);
    CT_CHECK_LAUNCH("locate exact");
    return CT_OK;
}

int ct_locate_deferred_count(const void* ws, int64_t n, int32_t G, int64_t* counts_host4, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    LocWS L;
    carve_loc((void*)ws, n, G, &L);
    int c[4] = {0, 0, 0, 0};
    CT_CUDA(cudaMemcpyAsync(c, L.counters, sizeof(c), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < 4; k++) counts_host4[k] = c[k];
    return CT_OK;
}

int ct_locate_points_batched(const ct_tree* t, const double* points, int64_t n, double tol, int32_t G, int64_t* out,
                             void* ws, size_t ws_bytes, void* stream) {
    int s = ct_locate_bin(t, points, n, G, ws, ws_bytes, stream);
    if (s) return s;
    s = ct_locate_fast(t, points, n, tol, G, out, ws, ws_bytes, stream);
    if (s) return s;
    return ct_locate_exact(t, points, n, tol, G, out, ws, ws_bytes, stream);
}

// ---------------------------------------------------------------------------
// a batch of trees: one pipeline for the points of every tree
// ---------------------------------------------------------------------------

size_t ct_forest_locate_workspace_size(int64_t n_points, int32_t n_trees) {
    if (n_points < 0 || n_trees < 1) return 0;
    return carve_forest(nullptr, n_points, n_trees, nullptr, nullptr);
}

int ct_forest_locate_prepare(const ct_tree* trees, int32_t n_trees, const double* tolerances,
                             const int64_t* point_off, int64_t n_points, ct_forest_plan* plan, void* ws,
                             size_t ws_bytes, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!trees || !tolerances || !point_off || !plan || n_trees < 1) return ct_fail(CT_ERR_ARG, "null argument");
    if (n_points < 0 || n_points >= INT32_MAX / 2) return ct_fail(CT_ERR_ARG, "at most 2^30 points per call");
    if (point_off[0] != 0 || point_off[n_trees] != n_points)
        return ct_fail(CT_ERR_ARG, "point offsets must start at 0 and end at n_points");
    for (int i = 0; i < n_trees; i++)
        if (point_off[i + 1] < point_off[i]) return ct_fail(CT_ERR_ARG, "point offsets must not decrease");
    if (!ws || ws_bytes < carve_forest(nullptr, n_points, n_trees, nullptr, nullptr))
        return ct_fail(CT_ERR_WORKSPACE, "forest locate workspace too small");
    LocWS L;
    ForestWS F;
    carve_forest(ws, n_points, n_trees, &L, &F);
    std::vector<TreeL> tl((size_t)n_trees);
    std::vector<Grid> gr((size_t)n_trees);
    int kmax = 0, stack = 0;
    for (int i = 0; i < n_trees; i++) {
        int s = fill_tree(&trees[i], tolerances[i], &tl[i]);
        if (s) return s;
        gr[i] = morton_grid(&trees[i]);
        kmax = std::max(kmax, tl[i].K);
        stack = std::max(stack, tl[i].stack);
    }
    int tree_bits = 0;
    while ((1 << tree_bits) < n_trees) tree_bits++;
    if (tree_bits > 24) return ct_fail(CT_ERR_ARG, "at most 2^24 trees per batch");
    int mbits = std::min(24, 32 - tree_bits) & ~1;
    plan->n_points = n_points;
    plan->n_trees = n_trees;
    plan->kt = (kmax <= 3) ? 3 : (kmax <= 4 ? 4 : 32);
    plan->stack = stack;
    plan->morton_bits = mbits;
    plan->error_word = trees[0].error_word;
    plan->max_tree_points = 0;
    for (int32_t i = 0; i < n_trees; i++)
        plan->max_tree_points = std::max<int64_t>(plan->max_tree_points, point_off[i + 1] - point_off[i]);
    CT_CUDA(cudaMemcpyAsync(F.trees, tl.data(), sizeof(TreeL) * tl.size(), cudaMemcpyHostToDevice, st));
    CT_CUDA(cudaMemcpyAsync(F.grids, gr.data(), sizeof(Grid) * gr.size(), cudaMemcpyHostToDevice, st));
    CT_CUDA(cudaMemcpyAsync(F.poff, point_off, sizeof(int64_t) * ((size_t)n_trees + 1), cudaMemcpyHostToDevice, st));
    CT_CUDA(cudaStreamSynchronize(st));  // the host vectors go out of scope
    size_t smem = (size_t)stack * LOC_THREADS * sizeof(int);
    if (plan->kt == 3) smem_attr<3, true>(smem);
    else if (plan->kt == 4) smem_attr<4, true>(smem);
    else smem_attr<32, true>(smem);
    return CT_OK;
}

// Kernel launches only (no host synchronisation, no host copies): can be
// captured in a CUDA graph once prepared.
int ct_forest_locate(const ct_forest_plan* plan, const double* points, int64_t* out, void* ws, size_t ws_bytes,
                     void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!plan || plan->n_trees < 1) return ct_fail(CT_ERR_ARG, "plan not prepared");
    const int64_t n = plan->n_points;
    if (!ws || ws_bytes < carve_forest(nullptr, n, plan->n_trees, nullptr, nullptr))
        return ct_fail(CT_ERR_WORKSPACE, "forest locate workspace too small");
    LocWS L;
    ForestWS F;
    carve_forest(ws, n, plan->n_trees, &L, &F);
    CT_CUDA(cudaMemsetAsync(L.counters, 0, 64, st));
    if (n == 0) return CT_OK;
    const double2* P = (const double2*)points;
    // stage 1: sort by (tree, Morton key), 4 passes of 8 bits; the last pass
    // writes the permutation into L.order
    unsigned* kin = L.keyA;
    int* iin = L.order;
    unsigned* kout = L.keyB;
    int* iout = L.idxB;
    int64_t chunk = (n + RS_BLOCKS - 1) / RS_BLOCKS;
    chunk = (chunk + RS_TILE - 1) / RS_TILE * RS_TILE;
    const int64_t nh = (int64_t)256 * RS_BLOCKS;
    for (int pss = 0; pss < 4; pss++) {
        int shift = 8 * pss;
        if (pss == 0)
            k_keys_forest<<<RS_BLOCKS, RS_T, 0, st>>>(P, n, chunk, F.grids, F.poff, plan->n_trees, plan->morton_bits,
                                                      kin, F.qtree, L.hist);
        else
            k_rs_hist<<<RS_BLOCKS, RS_T, 0, st>>>(kin, n, chunk, shift, L.hist);
        int s = ct_exclusive_scan(L.hist, nh, L.hist, L.scan_ws, L.scan_bytes, nullptr, stream);
        if (s) return s;
        k_rs_scatter<unsigned, unsigned><<<RS_BLOCKS, RS_T, 0, st>>>(kin, pss ? iin : nullptr, n, chunk, shift,
                                                                     L.hist, pss < 3 ? kout : nullptr, 0, iout);
        std::swap(kin, kout);
        std::swap(iin, iout);
    }
    // 4 passes: the permutation is back in L.order
    TreeL T0;
    memset(&T0, 0, sizeof(T0));
    size_t smem = (size_t)plan->stack * LOC_THREADS * sizeof(int);
    unsigned grid = (unsigned)((n + LOC_THREADS - 1) / LOC_THREADS);
    int sms = 152;
    {
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    const int fast_bpsm = (plan->tune_fast_bpsm >= 1 && plan->tune_fast_bpsm <= 32) ? plan->tune_fast_bpsm : 16;
    const int cells_bpsm = plan->tune_cells_bpsm;
    unsigned grid_b = (unsigned)std::min<int64_t>((n + LOC_THREADS - 1) / LOC_THREADS, (int64_t)sms * fast_bpsm);
    // queries are sorted by tree first: one tree's results land in its own
    // range of `out`, so only a tree with many queries needs the scatter
    int* res_sorted = plan->max_tree_points > RES_SCATTER_MIN ? sorted_results(L) : nullptr;
#define CT_FOREST_STAGES(KT)                                                                                      \
    if (cells_bpsm == 8)                                                                                          \
        k_cells<KT, true, 8><<<grid, LOC_THREADS, 0, st>>>(T0, F.trees, F.qtree, P, L.order, n, out, res_sorted, \
                                                           L.open, &L.counters[3]);                              \
    else                                                                                                          \
        k_cells<KT, true, 6><<<grid, LOC_THREADS, 0, st>>>(T0, F.trees, F.qtree, P, L.order, n, out, res_sorted, \
                                                           L.open, &L.counters[3]);                              \
    k_fast<KT, true><<<grid_b, LOC_THREADS, smem, st>>>(T0, F.trees, F.qtree, P, L.order, n, out, L.R,          \
                                                        L.counters, L.ovf, L.open, &L.counters[3]);              \
    k_pip<true><<<GRID_STRIDE, LOC_THREADS, 0, st>>>(T0, F.trees, F.qtree, P, L.R, L.counters);                  \
    k_resolve<true><<<GRID_STRIDE, LOC_THREADS, 0, st>>>(T0, F.trees, F.qtree, L.R, L.counters, out);            \
    k_exact<KT, true><<<GRID_STRIDE, LOC_THREADS, smem, st>>>(T0, F.trees, F.qtree, P, L.ovf, L.counters, out);
    if (plan->kt == 3) {
        CT_FOREST_STAGES(3)
    } else if (plan->kt == 4) {
        CT_FOREST_STAGES(4)
    } else {
        CT_FOREST_STAGES(32)
    }
#undef CT_FOREST_STAGES
    if (res_sorted) scatter_results(L, n, plan->error_word, out, st);
    CT_CHECK_LAUNCH("forest locate");
    return CT_OK;
}

static int check_index(const ct_forest_index* X) {
    if (!X) return ct_fail(CT_ERR_ARG, "index is null");
    if (X->n_trees < 1 || X->n_total < X->n_trees) return ct_fail(CT_ERR_ARG, "index sizes out of range");
    if (X->k_max < 3 || X->k_max > CT_MAX_N_VERTEX) return ct_fail(CT_ERR_ARG, "k_max must be in [3, 32]");
    if (X->stack < 2 || X->stack > 128) return ct_fail(CT_ERR_ARG, "stack must be in [2, 128]");
    if (X->grid_cells < 0 || X->node_capacity < 1) return ct_fail(CT_ERR_ARG, "index sizes out of range");
    if (!X->vertices || !X->faces || !X->face_off || !X->poly32_off || !X->tree_K || !X->bb_coords ||
        !X->tree_off || !X->node_off || !X->max_depth || !X->node_child || !X->node_Lmax || !X->node_Rmin ||
        !X->node_ptr || !X->node_size || !X->node_dim || !X->bb_indices || !X->grid_off || !X->grid_nx ||
        !X->grid_ny || (X->grid_cells > 0 && !X->grid_start) || !X->nodes_f32 || !X->nodes_f64 || !X->poly_f64 ||
        !X->poly_f32 || !X->poly_len || !X->poly_len32 || !X->summary || !X->error_word)
        return ct_fail(CT_ERR_ARG, "index has a null array");
    if (X->cand_capacity < 0) return ct_fail(CT_ERR_ARG, "cand_capacity must be >= 0");
    if (X->cand_capacity > 0 &&
        (!X->cand_count || !X->cand_off || !X->cand_box || !X->cand_idx || !X->cand_lbox || !X->cand_scan_ws ||
         X->cand_scan_bytes < ct_scan_workspace_size(X->grid_cells + 1)))
        return ct_fail(CT_ERR_ARG, "candidate-list arrays of the index are missing or too small");
    return CT_OK;
}

int ct_forest_index_prepare(const ct_forest_index* X, const int64_t* point_off, int64_t n_points,
                            ct_forest_plan* plan, void* ws, size_t ws_bytes, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    int s = check_index(X);
    if (s) return s;
    if (!point_off || !plan) return ct_fail(CT_ERR_ARG, "null argument");
    const int32_t n_trees = X->n_trees;
    if (n_points < 0 || n_points >= INT32_MAX / 2) return ct_fail(CT_ERR_ARG, "at most 2^30 points per call");
    if (point_off[0] != 0 || point_off[n_trees] != n_points)
        return ct_fail(CT_ERR_ARG, "point offsets must start at 0 and end at n_points");
    for (int i = 0; i < n_trees; i++)
        if (point_off[i + 1] < point_off[i]) return ct_fail(CT_ERR_ARG, "point offsets must not decrease");
    if (!ws || ws_bytes < carve_forest(nullptr, n_points, n_trees, nullptr, nullptr))
        return ct_fail(CT_ERR_WORKSPACE, "forest locate workspace too small");
    int tree_bits = 0;
    while ((1 << tree_bits) < n_trees) tree_bits++;
    if (tree_bits > 24) return ct_fail(CT_ERR_ARG, "at most 2^24 trees per batch");
    LocWS L;
    ForestWS F;
    carve_forest(ws, n_points, n_trees, &L, &F);
    plan->n_points = n_points;
    plan->n_trees = n_trees;
    plan->kt = (X->k_max <= 3) ? 3 : (X->k_max <= 4 ? 4 : 32);
    plan->stack = X->stack;
    plan->morton_bits = std::min(24, 32 - tree_bits) & ~1;
    plan->error_word = X->error_word;
    plan->max_tree_points = 0;
    for (int32_t i = 0; i < n_trees; i++)
        plan->max_tree_points = std::max<int64_t>(plan->max_tree_points, point_off[i + 1] - point_off[i]);
    CT_CUDA(cudaMemcpyAsync(F.poff, point_off, sizeof(int64_t) * ((size_t)n_trees + 1), cudaMemcpyHostToDevice, st));
    CT_CUDA(cudaStreamSynchronize(st));
    size_t smem = (size_t)plan->stack * LOC_THREADS * sizeof(int);
    if (plan->kt == 3) smem_attr<3, true>(smem);
    else if (plan->kt == 4) smem_attr<4, true>(smem);
    else smem_attr<32, true>(smem);
    return CT_OK;
}

int ct_forest_index_build(const ct_forest_index* X, const ct_forest_plan* plan, void* ws, size_t ws_bytes,
                          void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    int s = check_index(X);
    if (s) return s;
    if (!plan || plan->n_trees != X->n_trees || plan->stack != X->stack)
        return ct_fail(CT_ERR_ARG, "plan not prepared for this index");
    if (!ws || ws_bytes < carve_forest(nullptr, plan->n_points, plan->n_trees, nullptr, nullptr))
        return ct_fail(CT_ERR_WORKSPACE, "forest locate workspace too small");
    LocWS L;
    ForestWS F;
    carve_forest(ws, plan->n_points, plan->n_trees, &L, &F);
    int sms = 152;
    {
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    auto blocks = [&](int64_t n, int per_sm) {
        return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * per_sm));
    };
    k_fx_reset<<<blocks((int64_t)X->n_trees * FX_WORDS, 4), 256, 0, st>>>(X->summary, X->n_trees, X->error_word);
    k_fx_summary<<<blocks(X->n_total, 8), 256, 0, st>>>(X->bb_coords, X->n_total, X->tree_off, X->n_trees,
                                                        X->summary, X->error_word);
    k_fx_records<<<(unsigned)((X->n_trees + 127) / 128), 128, 0, st>>>(*X, F.trees, F.grids);
    k_fx_pack_nodes<<<blocks(X->node_capacity, 16), 256, 0, st>>>(*X, F.trees);
    k_fx_pack_cells<<<blocks(X->n_total, 16), 256, 0, st>>>(*X);
    if (X->grid_cells > 0) k_fx_grid_start<<<blocks(X->grid_cells, 16), 256, 0, st>>>(*X, F.trees);
    if (X->cand_capacity > 0 && X->grid_cells > 0) {
        const size_t cbytes = 8 * (size_t)(X->grid_cells + 1);
        k_fx_cand_box<<<blocks(X->n_total, 16), 256, 0, st>>>(*X, F.trees);
        CT_CUDA(cudaMemsetAsync(X->cand_count, 0, cbytes, st));
        k_fx_cand_lists<0><<<blocks(X->n_total, 16), 256, 0, st>>>(*X, F.trees);
        int sc = ct_exclusive_scan((const int64_t*)X->cand_count, X->grid_cells + 1, X->cand_off, X->cand_scan_ws,
                                   X->cand_scan_bytes, nullptr, stream);
        if (sc) return sc;
        k_fx_cand_enable<<<(unsigned)((X->n_trees + 127) / 128), 128, 0, st>>>(*X, F.trees);
        CT_CUDA(cudaMemsetAsync(X->cand_count, 0, cbytes, st));  // now the lists' cursors
        k_fx_cand_lists<1><<<blocks(X->n_total, 16), 256, 0, st>>>(*X, F.trees);
    }
    CT_CHECK_LAUNCH("forest index");
    return CT_OK;
}

// ---------------------------------------------------------------------------
// one 8-bit radix pass, shared with the multi-result queries
// ---------------------------------------------------------------------------
size_t ct_radix_pass_workspace_size(void) {
    return a256(8 * (size_t)256 * RS_BLOCKS) + a256(ct_scan_workspace_size((int64_t)256 * RS_BLOCKS));
}

int ct_radix_pass(const unsigned* kin, const int* iin, int64_t n, int32_t shift, unsigned* kout, int* iout, void* ws,
                  size_t ws_bytes, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n < 0 || shift < 0 || shift > 24) return ct_fail(CT_ERR_ARG, "bad radix pass");
    if (!ws || ws_bytes < ct_radix_pass_workspace_size()) return ct_fail(CT_ERR_WORKSPACE, "radix workspace too small");
    if (n == 0) return CT_OK;
    int64_t* hist = (int64_t*)ws;
    const int64_t nh = (int64_t)256 * RS_BLOCKS;
    void* scan_ws = (char*)ws + a256(8 * (size_t)nh);
    size_t scan_bytes = ws_bytes - a256(8 * (size_t)nh);
    int64_t chunk = (n + RS_BLOCKS - 1) / RS_BLOCKS;
    chunk = (chunk + RS_TILE - 1) / RS_TILE * RS_TILE;
    k_rs_hist<<<RS_BLOCKS, RS_T, 0, st>>>(kin, n, chunk, shift, hist);
    int s = ct_exclusive_scan(hist, nh, hist, scan_ws, scan_bytes, nullptr, stream);
    if (s) return s;
    k_rs_scatter<unsigned, unsigned><<<RS_BLOCKS, RS_T, 0, st>>>(kin, iin, n, chunk, shift, hist, kout, 0, iout);
    CT_CHECK_LAUNCH("radix pass");
    return CT_OK;
}

}  // extern "C"
