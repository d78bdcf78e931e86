// ct_build.cu -- GPU construction of the cell tree (creation.py:27-413).
//
// The upstream builder (build creation.py:233-381) is a serial depth-first
// loop.  Every node's work -- the bounds of its range, the n_buckets
// equal-width centroid buckets, the stable partition of its bb_indices range
// and the split decision -- depends only on the node's own range, never on
// the order in which nodes are processed.  This builder therefore processes
// nodes breadth first:
//
//   phase A  nodes with more than SMALL cells, one level at a time, many CTAs
//            per node: a stats pass (per-bucket counts and first-occurrence
//            bounds for both dimensions, warp-aggregated), a decide pass (one
//            warp per node, upstream split logic), a stable scatter pass
//            (match_any ranks + per-tile prefixes).  Child bounds come from the
//            parent's per-bucket stats, so no separate bounds pass is needed.
//   phase B  every node of <= SMALL cells roots a subtree that one warp builds
//            depth first in shared memory, in upstream order.
//   phase C  the node numbering.  Upstream appends the two children of every
//            split node at the end of the node array in depth-first
//            (pre-order, left first) processing order, so a split node v gets
//            child = 1 + 2 * (number of split nodes before v in pre-order).
//            Phase C computes per-subtree split counts bottom-up and pre-order
//            ranks top-down and writes every node to its upstream position.
//
// Float64 comparisons use monotone 64-bit integer keys (fkey): the order is the
// float order, and -0.0 / +0.0 share a key; where a first-occurrence minimum
// or maximum is 0 the sign is taken from the first zero-valued element, so the
// stored bits equal upstream's.  The float64 arithmetic of the split logic is
// written in upstream's evaluation order (library compiled with -fmad=false).
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "ct_common.cuh"
#include "ct_internal.h"

namespace ct {

constexpr int SMALL = 128;         // subtree size handled by one warp
constexpr int NBMAX = 32;          // maximum n_buckets
constexpr int STATS_THREADS = 256; // threads of the stats / scatter CTAs
constexpr int TILE_MIN = 2048;     // minimum cells per tile
constexpr int MAX_TILES = 512;     // maximum tiles per node
constexpr int SUB_WARPS = 2;       // warps per CTA in the subtree kernel (8.1 KB of shared memory each)

enum : int { K_PENDING = 0, K_SPLIT = 1, K_LEAF = 2, K_SUBTREE = 3 };

// Phase-A node record.
struct ARec {
    double bnd[4];  // first-occurrence xmin, xmax, ymin, ymax of the node's boxes
    double Lmax, Rmin;
    long long splits;  // split nodes in the subtree rooted here
    long long S;       // split nodes before this node in pre-order
    long long pos;     // final node index
    int ptr, size;
    int dim, kind;
    int child, parity; // child: record id of the left child (right = +1)
    int level, tile0;
    int tile1, split_dim;
    int nlocal, err;
    int tree, pad_;    // tree of the node (forest builds; 0 otherwise)
};

// Phase-B local node record (subtree numbering, local ids).
struct LRec {
    double Lmax, Rmin;
    int child, ptr, size, dim;
};

struct Counters {
    int rec_count;
    int tile_count;
    int small_count;
    unsigned int err;
    int max_depth;
    int lb, le;  // current level record range
    int pad;
    unsigned long long root_key[4];
    int root_zp[4];
    int done;    // device-driven level loop: no pending record left (or an error)
    int nlev;    // device-driven level loop: phase-A levels recorded in lvl_b / lvl_e
};

// most phase-A levels the device-driven level loop runs (a balanced tree of
// 2^31 cells needs about 30; more sets CT_DEVERR_LOOP in the status)
constexpr int DEV_MAX_LEVELS = 64;

struct WS {
    double* f[2][4];  // lo_x, hi_x, lo_y, hi_y (two ping-pong buffers); centroids are recomputed (centroid_of)
    int* idx[2];
    int* final_idx;
    ARec* recs;
    int rec_cap;
    unsigned int* st_cnt;            // [rec_cap][2][NB]
    unsigned long long* st_key;      // [rec_cap][2][NB][4]
    int* st_zp;                      // [rec_cap][2][NB][4]
    int* nb_base;                    // [rec_cap][NB]
    int* tile_rec;
    int* tile_start;
    int* tile_end;
    unsigned int* tile_cnt;          // [tile_cap][2][NB]
    int* tile_pref;                  // [tile_cap][NB]
    int tile_cap;
    int* small_list;                 // [rec_cap]
    LRec* lrec;                      // [2 * n]
    Counters* cnt;
    int* level_begin;                // [rec_cap + 1] host mirror written per level
    int* lvl_b;                      // [DEV_MAX_LEVELS + 1] level record ranges (device-driven loop)
    int* lvl_e;
    // per tree (a forest build has n_roots trees, root records 0 .. n_roots-1)
    int n_roots;
    int64_t* tree_off;               // [n_roots + 1] element offsets
    int* elem_tree;                  // [n] tree of each element position
    unsigned long long* root_key;    // [n_roots][4]
    int* root_zp;                    // [n_roots][4]
    int* tree_depth;                 // [n_roots]
};

static inline size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

// Carves the workspace; returns total bytes.  base == nullptr -> size only.
// `forest`: the layout of the forest builds, whose per-element tree index is
// written and read for every element even when the batch holds one tree.
static size_t carve(char* base, int64_t n, int NB, int factor, WS* ws, int n_trees = 1, bool forest = false) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> char* {
        char* p = base ? base + off : nullptr;
        off += align_up(bytes);
        return p;
    };
    int64_t nn = n > 0 ? n : 1;
    int rec_cap = (int)std::min<int64_t>(INT32_MAX / 4,
                                         (int64_t)factor * (8 * (nn / SMALL) + 64) + 3 * (int64_t)n_trees);
    int tile_cap = (int)std::min<int64_t>(INT32_MAX / 4, 2 * (nn / TILE_MIN) + 2 * (int64_t)rec_cap + 64);
    WS w;
    for (int b = 0; b < 2; b++) {
        for (int k = 0; k < 4; k++) w.f[b][k] = (double*)take(sizeof(double) * nn);
        w.idx[b] = (int*)take(sizeof(int) * nn);
    }
    w.final_idx = (int*)take(sizeof(int) * nn);
    w.recs = (ARec*)take(sizeof(ARec) * rec_cap);
    w.rec_cap = rec_cap;
    w.st_cnt = (unsigned int*)take(sizeof(unsigned int) * (size_t)rec_cap * 2 * NB);
    w.st_key = (unsigned long long*)take(sizeof(unsigned long long) * (size_t)rec_cap * 2 * NB * 4);
    w.st_zp = (int*)take(sizeof(int) * (size_t)rec_cap * 2 * NB * 4);
    w.nb_base = (int*)take(sizeof(int) * (size_t)rec_cap * NB);
    w.tile_rec = (int*)take(sizeof(int) * tile_cap);
    w.tile_start = (int*)take(sizeof(int) * tile_cap);
    w.tile_end = (int*)take(sizeof(int) * tile_cap);
    w.tile_cnt = (unsigned int*)take(sizeof(unsigned int) * (size_t)tile_cap * 2 * NB);
    w.tile_pref = (int*)take(sizeof(int) * (size_t)tile_cap * NB);
    w.tile_cap = tile_cap;
    w.small_list = (int*)take(sizeof(int) * rec_cap);
    w.lrec = (LRec*)take(sizeof(LRec) * 2 * nn);
    w.cnt = (Counters*)take(sizeof(Counters));
    w.level_begin = nullptr;
    w.lvl_b = (int*)take(sizeof(int) * (DEV_MAX_LEVELS + 1));
    w.lvl_e = (int*)take(sizeof(int) * (DEV_MAX_LEVELS + 1));
    w.n_roots = n_trees;
    w.tree_off = (int64_t*)take(sizeof(int64_t) * ((size_t)n_trees + 1));
    w.elem_tree = (int*)take((forest || n_trees > 1) ? sizeof(int) * nn : 16);
    w.root_key = (unsigned long long*)take(sizeof(unsigned long long) * 4 * (size_t)n_trees);
    w.root_zp = (int*)take(sizeof(int) * 4 * (size_t)n_trees);
    w.tree_depth = (int*)take(sizeof(int) * (size_t)n_trees);
    if (ws) *ws = w;
    return off;
}

// ------------------------------------------------------------------------
// small device helpers
// ------------------------------------------------------------------------

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// (key, pos) lexicographic minimum over the lanes of `mask` (all call).
__device__ __forceinline__ void group_min_kp(unsigned mask, unsigned long long k, unsigned pos,
                                             unsigned long long* ko, unsigned* po) {
    unsigned hi = (unsigned)(k >> 32), lo = (unsigned)k;
    unsigned mh = __reduce_min_sync(mask, hi);
    unsigned ml = __reduce_min_sync(mask, hi == mh ? lo : 0xffffffffu);
    unsigned mp = __reduce_min_sync(mask, (hi == mh && lo == ml) ? pos : 0xffffffffu);
    *ko = ((unsigned long long)mh << 32) | ml;
    *po = mp;
}

__device__ __forceinline__ unsigned long long group_min_k(unsigned mask, unsigned long long k) {
    unsigned hi = (unsigned)(k >> 32), lo = (unsigned)k;
    unsigned mh = __reduce_min_sync(mask, hi);
    unsigned ml = __reduce_min_sync(mask, hi == mh ? lo : 0xffffffffu);
    return ((unsigned long long)mh << 32) | ml;
}

__device__ __forceinline__ bool is_zero(double x) { return (__double_as_longlong(x) & 0x7fffffffffffffffll) == 0; }
__device__ __forceinline__ bool is_nan_bits(double x) {
    return (unsigned long long)(__double_as_longlong(x) & 0x7fffffffffffffffll) > 0x7ff0000000000000ull;
}

// Bucket of centroid key kc given the NB+1 boundary keys K (non-decreasing):
// the b with K[b] <= kc < K[b+1] (centroid_test creation.py:44-51), or -1.
__device__ __forceinline__ int find_bucket(const unsigned long long* K, int NB, unsigned long long kc) {
    if (kc < K[0] || kc >= K[NB]) return -1;
    int lo = 0, hi = NB;  // K[lo] <= kc < K[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (K[mid] <= kc) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Boundary j of the equal-width buckets: Min of bucket j (= Max of bucket j-1),
// `i * bucket_length + range_Rmin` (creation.py:283-293).
__device__ __forceinline__ double bucket_edge(int j, double bl, double R) { return exact_i2d(j) * bl + R; }

// bucket_length = (range_Lmax - range_Rmin) / n_buckets (creation.py:278).
// For a power-of-two n_buckets the quotient equals the product with the exact
// reciprocal (same real number, same rounding), which avoids a float64 divide.
__device__ __forceinline__ double bucket_len(double L, double R, int NB) {
    double diff = L - R;
    if ((NB & (NB - 1)) == 0) return diff * exact_pow2_inv(NB);
    return diff / exact_i2d(NB);
}

struct Decision {
    int kind;     // 0: all cells in one bucket, 1: split, -1: error
    int nleft;    // cells in the left child
    int rbucket;  // first bucket of the right child
    double Lmax, Rmin;
};

// Split decision of one node for one dimension, lane-parallel (all 32 lanes
// call, NB <= 32).  cnt / bRmin / bLmax hold the per-bucket sizes and bounds
// (empty buckets: DBL_MAX / -DBL_MAX, get_bounds creation.py:153-171).
// Restates the empty-bucket merge (creation.py:322-341), the all-in-one test
// (343-358) and split_plane (174-213) on the list of non-empty buckets.
__device__ Decision warp_decide(const int* cnt, const double* bRmin, const double* bLmax, int NB, int size,
                                double R, double L, double bl) {
    const unsigned FULL = 0xffffffffu;
    int lane = threadIdx.x & 31;
    Decision D;
    D.kind = -1;
    D.nleft = 0;
    D.rbucket = -1;
    D.Lmax = -1.0;
    D.Rmin = -1.0;
    bool ne = lane < NB && cnt[lane] > 0;
    unsigned mask = __ballot_sync(FULL, ne);
    int m = __popc(mask);
    if (m <= 1) {
        D.kind = (m == 1) ? 0 : -1;
        return D;
    }
    int bk = (lane < m) ? (int)__fns(mask, 0, lane + 1) : 0;
    int ck = (lane < m) ? cnt[bk] : 0;
    int pre = ck;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(FULL, pre, o);
        if (lane >= o) pre += t;
    }
    int nL = pre - ck;  // cells of the first `lane` non-empty buckets
    int bprev = __shfl_up_sync(FULL, bk, 1);
    int plane = -1;
    if (m == 2) {
        plane = 1;
    } else {
        // Float32 screening of split_plane's costs: the numerators are the
        // upstream float64 differences; the volumes and the cost are then
        // within 6u (u = 2^-24) of the exact real cost, all terms being
        // non-negative, and the float64 costs within a few 2^-53.  A
        // minimum below every other cost by more than 32u relative is
        // therefore the float64 argmin as well; anything else (ties, zero
        // or non-finite values, costs near FLOAT_MAX) takes the float64
        // path below.
        float c32 = FLT_MAX;
        bool ok = true;
        if (lane >= 1 && lane < m) {
            const double dl = bLmax[bprev] - R, dr = L - bRmin[bk];
            const float fbl = (float)bl;
            ok = dl >= 0.0 && dr >= 0.0 && dl < 1e30 && dr < 1e30 && fbl > 1e-30f && fbl < 1e30f;
            if (ok) {
                const float vl = (float)dl / fbl, vr = (float)dr / fbl;
                // no float32 denormals (their relative error is unbounded)
                ok = (dl == 0.0 || ((float)dl >= 1e-30f && vl >= 1e-30f)) &&
                     (dr == 0.0 || ((float)dr >= 1e-30f && vr >= 1e-30f));
                c32 = vl * (float)nL + vr * (float)(size - nL);
                ok = ok && c32 < 1e30f;
            }
        }
        if (__all_sync(FULL, ok)) {
            float cmin = c32;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) cmin = fminf(cmin, __shfl_xor_sync(FULL, cmin, o));
            const float u = 5.9604644775390625e-08f;
            const bool near = c32 <= cmin * (1.0f + 32.0f * u) + 1e-37f;
            const unsigned nm = __ballot_sync(FULL, near && lane >= 1 && lane < m);
            if (__popc(nm) == 1) plane = __ffs(nm) - 1;
        }
    }
    if (plane < 0) {
        unsigned long long key = ~0ull;
        if (lane >= 1 && lane < m) {
            double left_volume = (bLmax[bprev] - R) / bl;
            double right_volume = (L - bRmin[bk]) / bl;
            double cost = left_volume * exact_i2d(nL) + right_volume * exact_i2d(size - nL);
            // `plane_cost < plane_min_cost` with plane_min_cost = FLOAT_MAX (NaN never qualifies)
            if (!is_nan_bits(cost) && fkey(cost) < fkey(DBL_MAX)) key = fkey(cost);
        }
        unsigned long long kmin;
        unsigned pmin_;
        group_min_kp(FULL, key, (unsigned)lane, &kmin, &pmin_);
        if (kmin == ~0ull) return D;  // no finite cost: upstream indexes past its buckets
        plane = (int)pmin_;
    }
    // Lmax = first maximum of bucket Lmax left of the plane, Rmin = first
    // minimum of bucket Rmin right of it (split_plane creation.py:202-211).
    unsigned long long kl = (lane < plane) ? ~fkey(bLmax[bk]) : ~0ull;
    unsigned long long kr = (lane >= plane && lane < m) ? fkey(bRmin[bk]) : ~0ull;
    unsigned long long ko;
    unsigned pl, pr;
    group_min_kp(FULL, kl, (unsigned)lane, &ko, &pl);
    group_min_kp(FULL, kr, (unsigned)lane, &ko, &pr);
    int bl_w = __shfl_sync(FULL, bk, (int)pl);
    int br_w = __shfl_sync(FULL, bk, (int)pr);
    D.Lmax = bLmax[bl_w];
    D.Rmin = bRmin[br_w];
    D.nleft = __shfl_sync(FULL, pre, plane - 1);
    D.rbucket = __shfl_sync(FULL, bk, plane);
    D.kind = 1;
    return D;
}

// ------------------------------------------------------------------------
// initial element buffers and root bounds
// ------------------------------------------------------------------------

// centroid creation.py:50: box[2d] + 0.5 * (box[2d + 1] - box[2d]), each
// operation rounded on its own (no fused multiply-add); recomputed wherever a
// cell's bucket is needed instead of being stored and moved with the cell
__device__ __forceinline__ double centroid_of(double lo, double hi) {
    return __dadd_rn(lo, __dmul_rn(0.5, __dsub_rn(hi, lo)));
}

__global__ void k_init_elems(const double* __restrict__ bb, int n, WS ws) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double x0 = bb[4 * (size_t)i], x1 = bb[4 * (size_t)i + 1], y0 = bb[4 * (size_t)i + 2], y1 = bb[4 * (size_t)i + 3];
        ws.f[0][0][i] = x0;
        ws.f[0][1][i] = x1;
        ws.f[0][2][i] = y0;
        ws.f[0][3][i] = y1;
        ws.idx[0][i] = i;
    }
}

__global__ void k_reset(WS ws, int n, int cpl_small_root, int root_dim) {
    Counters* c = ws.cnt;
    c->rec_count = 1;
    c->tile_count = 0;
    c->small_count = 0;
    c->err = 0;
    c->max_depth = 0;
    c->lb = 0;
    c->le = 1;
    c->done = 0;
    c->nlev = 1;
    for (int f = 0; f < 4; f++) {
        c->root_key[f] = ~0ull;
        c->root_zp[f] = INT32_MAX;
    }
    ARec r;
    memset(&r, 0, sizeof(r));
    r.ptr = 0;
    r.size = n;
    r.dim = root_dim;
    r.kind = (n > SMALL) ? K_PENDING : K_SUBTREE;
    r.child = -1;
    r.parity = 0;
    r.level = 0;
    r.split_dim = -1;
    r.Lmax = -1.0;
    r.Rmin = -1.0;
    ws.recs[0] = r;
    ws.tree_depth[0] = 0;
    if (n <= SMALL) {
        ws.small_list[0] = 0;
        c->small_count = 1;
    }
    (void)cpl_small_root;
}

// First-occurrence bounds of all boxes, both dimensions (root get_bounds).
__global__ void k_root_bounds(WS ws, int n) {
    const unsigned FULL = 0xffffffffu;
    unsigned long long k[4] = {~0ull, ~0ull, ~0ull, ~0ull};
    int stride = gridDim.x * blockDim.x;
    int iters = (n + stride - 1) / stride;
    for (int it = 0; it < iters; it++) {
        int i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        if (i < n) {
            for (int f = 0; f < 4; f++) {
                double v = ws.f[0][f][i];
                unsigned long long kk = (f & 1) ? ~fkey(v) : fkey(v);
                if (kk < k[f]) k[f] = kk;
                if (is_zero(v)) atomicMin(&ws.cnt->root_zp[f], i);
            }
        }
    }
    for (int f = 0; f < 4; f++) {
        unsigned long long m = group_min_k(FULL, k[f]);
        if ((threadIdx.x & 31) == 0) atomicMin(&ws.cnt->root_key[f], m);
    }
}

__device__ __forceinline__ double resolve_key(unsigned long long key_min_form, int f, int zp, const double* src) {
    // key_min_form: the minimum of the min-form key (complemented for maxima)
    unsigned long long k = (f & 1) ? ~key_min_form : key_min_form;
    if (k == fkey(0.0)) return src[zp];
    return fkey_inv(k);
}

__global__ void k_root_resolve(WS ws, int n) {
    if (n <= 0) return;
    for (int f = 0; f < 4; f++)
        ws.recs[0].bnd[f] = resolve_key(ws.cnt->root_key[f], f, ws.cnt->root_zp[f], ws.f[0][f]);
}

// ------------------------------------------------------------------------
// phase A
// ------------------------------------------------------------------------

__device__ __forceinline__ int tile_len_for(int size) {
    int t = (size + MAX_TILES - 1) / MAX_TILES;
    if (t < TILE_MIN) t = TILE_MIN;
    t = (t + STATS_THREADS - 1) / STATS_THREADS * STATS_THREADS;
    return t;
}

// One warp per record of the current level: make tiles for pending nodes and
// reset their stats slots.
__global__ void k_make_tiles(WS ws, int NB) {
    if (ws.cnt->done) return;
    int lb = ws.cnt->lb, le = ws.cnt->le;
    int lane = threadIdx.x & 31;
    int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int nw = (gridDim.x * blockDim.x) >> 5;
    for (int r = lb + wid; r < le; r += nw) {
        ARec* R = &ws.recs[r];
        if (R->kind != K_PENDING) continue;
        int size = R->size;
        int tl = tile_len_for(size);
        int nt = (size + tl - 1) / tl;
        int t0 = 0;
        if (lane == 0) t0 = atomicAdd(&ws.cnt->tile_count, nt);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 + nt > ws.tile_cap) {
            if (lane == 0) atomicOr(&ws.cnt->err, 0x80000000u);
            continue;
        }
        for (int j = lane; j < nt; j += 32) {
            ws.tile_rec[t0 + j] = r;
            ws.tile_start[t0 + j] = R->ptr + j * tl;
            ws.tile_end[t0 + j] = min(R->ptr + (j + 1) * tl, R->ptr + size);
        }
        if (lane == 0) {
            R->tile0 = t0;
            R->tile1 = t0 + nt;
        }
        size_t s = (size_t)(r - lb);
        for (int j = lane; j < 2 * NB; j += 32) ws.st_cnt[s * 2 * NB + j] = 0u;
        for (int j = lane; j < 2 * NB * 4; j += 32) {
            ws.st_key[s * 2 * NB * 4 + j] = ~0ull;
            ws.st_zp[s * 2 * NB * 4 + j] = INT32_MAX;
        }
    }
}

// Per tile: bucket membership in both dimensions; per (dim, bucket): count,
// first-occurrence min of lo_x / lo_y and max of hi_x / hi_y (as min-form
// keys) and the first position of a zero value.
// LOOP: the device-driven level loop's form -- a fixed grid walks the tiles
// whose count the make-tiles pass left on the device.
template <bool LOOP>
__global__ void __launch_bounds__(STATS_THREADS) k_stats(WS ws, int parity, int NB) {
    __shared__ unsigned long long K[2][NBMAX + 1];
    __shared__ unsigned int cnt[2][NBMAX];
    __shared__ unsigned long long key[2][NBMAX][4];
    __shared__ int zp[2][NBMAX][4];
    const unsigned FULL = 0xffffffffu;
    const int nt = LOOP ? (ws.cnt->done ? 0 : ws.cnt->tile_count) : (int)gridDim.x;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
    if (LOOP) __syncthreads();  // the previous tile's readers are done with the shared arrays
    int r = ws.tile_rec[t];
    int s = ws.tile_start[t], e = ws.tile_end[t];
    int lb = ws.cnt->lb;
    const ARec* R = &ws.recs[r];
    int tid = threadIdx.x;
    for (int j = tid; j < 2 * NBMAX; j += blockDim.x) (&cnt[0][0])[j] = 0u;
    for (int j = tid; j < 2 * NBMAX * 4; j += blockDim.x) {
        (&key[0][0][0])[j] = ~0ull;
        (&zp[0][0][0])[j] = INT32_MAX;
    }
    if (tid < 2 * (NB + 1)) {
        int d = tid / (NB + 1), j = tid % (NB + 1);
        double Rd = R->bnd[2 * d], Ld = R->bnd[2 * d + 1];
        K[d][j] = fkey(bucket_edge(j, bucket_len(Ld, Rd, NB), Rd));
    }
    __syncthreads();
    const double* F0 = ws.f[parity][0];
    const double* F1 = ws.f[parity][1];
    const double* F2 = ws.f[parity][2];
    const double* F3 = ws.f[parity][3];
    for (int base = s; base < e; base += blockDim.x) {
        int i = base + tid;
        bool valid = i < e;
        double v0 = 0, v1 = 0, v2 = 0, v3 = 0, c0 = 0, c1 = 0;
        if (valid) {
            v0 = F0[i];
            v1 = F1[i];
            v2 = F2[i];
            v3 = F3[i];
            c0 = centroid_of(v0, v1);
            c1 = centroid_of(v2, v3);
        }
        unsigned long long k0 = fkey(v0), k1 = ~fkey(v1), k2 = fkey(v2), k3 = ~fkey(v3);
#pragma unroll
        for (int d = 0; d < 2; d++) {
            int b = -2;
            if (valid) {
                b = find_bucket(K[d], NB, fkey(d ? c1 : c0));
                if (b < 0) atomicOr(&ws.cnt->err, CT_DEVERR_BUCKET);
            }
            unsigned grp = __match_any_sync(FULL, b);
            if (b >= 0) {
                unsigned long long m0 = group_min_k(grp, k0);
                unsigned long long m1 = group_min_k(grp, k1);
                unsigned long long m2 = group_min_k(grp, k2);
                unsigned long long m3 = group_min_k(grp, k3);
                if ((int)(__ffs(grp) - 1) == (tid & 31)) {
                    atomicAdd(&cnt[d][b], (unsigned)__popc(grp));
                    atomicMin(&key[d][b][0], m0);
                    atomicMin(&key[d][b][1], m1);
                    atomicMin(&key[d][b][2], m2);
                    atomicMin(&key[d][b][3], m3);
                }
                if (is_zero(v0)) atomicMin(&zp[d][b][0], i);
                if (is_zero(v1)) atomicMin(&zp[d][b][1], i);
                if (is_zero(v2)) atomicMin(&zp[d][b][2], i);
                if (is_zero(v3)) atomicMin(&zp[d][b][3], i);
            }
        }
    }
    __syncthreads();
    size_t sidx = (size_t)(r - lb);
    for (int j = tid; j < 2 * NB; j += blockDim.x) {
        int d = j / NB, b = j % NB;
        unsigned c = cnt[d][b];
        ws.tile_cnt[(size_t)t * 2 * NB + j] = c;
        if (c) atomicAdd(&ws.st_cnt[sidx * 2 * NB + j], c);
    }
    for (int j = tid; j < 2 * NB * 4; j += blockDim.x) {
        int d = j / (NB * 4), b = (j / 4) % NB, f = j % 4;
        if (cnt[d][b]) {
            atomicMin(&ws.st_key[sidx * 2 * NB * 4 + j], key[d][b][f]);
            if (zp[d][b][f] != INT32_MAX) atomicMin(&ws.st_zp[sidx * 2 * NB * 4 + j], zp[d][b][f]);
        }
    }
    }
}

// One warp per record of the current level: the upstream split decision for
// pending nodes, children records, bucket bases and tile prefixes.
template <bool LOOP>
__global__ void k_decide(WS ws, int NB, long long cpl) {
    __shared__ int s_cnt[4][2][NBMAX];
    __shared__ double s_Rmin[4][2][NBMAX];
    __shared__ double s_Lmax[4][2][NBMAX];
    const unsigned FULL = 0xffffffffu;
    int lane = threadIdx.x & 31;
    int w = threadIdx.x >> 5;  // blockDim = 128
    if (LOOP && ws.cnt->done) return;
    int lb = ws.cnt->lb, le = ws.cnt->le;
    const int step = LOOP ? (int)gridDim.x * 4 : INT32_MAX / 2;
    for (int r = lb + blockIdx.x * 4 + w; r < le; r += step) {
    __syncwarp();
    ARec* R = &ws.recs[r];
    if (R->kind != K_PENDING) continue;
    int parity = R->parity;
    size_t sidx = (size_t)(r - lb);
    int size = R->size, ptr = R->ptr;
    // resolve per-bucket bounds of both dimensions
    for (int j = lane; j < 2 * NB; j += 32) {
        int d = j / NB, b = j % NB;
        int c = (int)ws.st_cnt[sidx * 2 * NB + j];
        s_cnt[w][d][b] = c;
        double rmin = DBL_MAX, lmax = -DBL_MAX;
        if (c > 0) {
            size_t kb = (sidx * 2 * NB + j) * 4;
            int flo = 2 * d, fhi = 2 * d + 1;
            rmin = resolve_key(ws.st_key[kb + flo], flo, ws.st_zp[kb + flo], ws.f[parity][flo]);
            lmax = resolve_key(ws.st_key[kb + fhi], fhi, ws.st_zp[kb + fhi], ws.f[parity][fhi]);
        }
        s_Rmin[w][d][b] = rmin;
        s_Lmax[w][d][b] = lmax;
    }
    __syncwarp();
    int d0 = R->dim;
    int stored_dim = d0;
    int ds = -1;
    Decision D;
    D.kind = -1;
    bool bad = false;
    if ((long long)size <= cpl) {
        D.kind = 2;  // leaf (creation.py:267)
    } else {
        for (int attempt = 0; attempt < 2; attempt++) {
            int d = attempt == 0 ? d0 : 1 - d0;
            int tot = 0;
            for (int b = 0; b < NB; b++) tot += s_cnt[w][d][b];
            if (tot != size) {
                bad = true;
                break;
            }
            double Rd = R->bnd[2 * d], Ld = R->bnd[2 * d + 1];
            double bl = bucket_len(Ld, Rd, NB);
            D = warp_decide(s_cnt[w][d], s_Rmin[w][d], s_Lmax[w][d], NB, size, Rd, Ld, bl);
            if (D.kind == 1) {
                ds = d;
                break;
            }
            if (D.kind < 0) {
                bad = true;
                break;
            }
            // all cells in one bucket: flip the stored dim once, then give up
            if (attempt == 0) stored_dim = 1 - d0;
            else D.kind = 2;
        }
    }
    if (bad) {
        if (lane == 0) atomicOr(&ws.cnt->err, CT_DEVERR_BUCKET);
        D.kind = 2;
    }
    if (D.kind == 2) {
        if (lane == 0) {
            R->kind = K_LEAF;
            R->dim = stored_dim;
            R->split_dim = -1;
            R->Lmax = -1.0;
            R->Rmin = -1.0;
        }
        continue;
    }
    // split in ds
    int c = 0;
    if (lane == 0) c = atomicAdd(&ws.cnt->rec_count, 2);
    c = __shfl_sync(FULL, c, 0);
    if (c + 2 > ws.rec_cap) {
        if (lane == 0) {
            atomicOr(&ws.cnt->err, 0x80000000u);
            R->kind = K_LEAF;
            R->split_dim = -1;
        }
        continue;
    }
    int rb = D.rbucket;
    // child bounds: first occurrence over the child's buckets in order
    size_t kb0 = sidx * 2 * NB * 4 + (size_t)ds * NB * 4;
    double cb[2][4];
    for (int f = 0; f < 4; f++) {
        for (int side = 0; side < 2; side++) {
            int b0 = side ? rb : 0, b1 = side ? NB : rb;
            unsigned long long best = ~0ull;
            int bb = -1;
            for (int b = b0; b < b1; b++) {
                if (s_cnt[w][ds][b] == 0) continue;
                unsigned long long k = ws.st_key[kb0 + (size_t)b * 4 + f];
                if (k < best) {
                    best = k;
                    bb = b;
                }
            }
            cb[side][f] = (bb < 0) ? ((f & 1) ? -DBL_MAX : DBL_MAX)
                                   : resolve_key(best, f, ws.st_zp[kb0 + (size_t)bb * 4 + f], ws.f[parity][f]);
        }
    }
    int child_dim = 1 - ds;
    if (lane < 2) {
        ARec ch;
        memset(&ch, 0, sizeof(ch));
        ch.ptr = lane ? ptr + D.nleft : ptr;
        ch.size = lane ? size - D.nleft : D.nleft;
        ch.dim = child_dim;
        ch.child = -1;
        ch.parity = 1 - parity;
        ch.level = R->level + 1;
        ch.tree = R->tree;
        ch.split_dim = -1;
        ch.Lmax = -1.0;
        ch.Rmin = -1.0;
        for (int f = 0; f < 4; f++) ch.bnd[f] = cb[lane][f];
        ch.kind = (ch.size > SMALL) ? K_PENDING : K_SUBTREE;
        ws.recs[c + lane] = ch;
        if (ch.kind == K_SUBTREE) {
            int sl = atomicAdd(&ws.cnt->small_count, 1);
            ws.small_list[sl] = c + lane;
        }
        atomicMax(&ws.cnt->max_depth, ch.level);
        atomicMax(&ws.tree_depth[R->tree], ch.level);
    }
    if (lane == 0) {
        R->kind = K_SPLIT;
        R->dim = stored_dim;
        R->split_dim = ds;
        R->Lmax = D.Lmax;
        R->Rmin = D.Rmin;
        R->child = c;
    }
    // bucket bases in the node and per-tile prefixes
    if (lane == 0) {
        int acc = ptr;
        for (int b = 0; b < NB; b++) {
            ws.nb_base[sidx * NB + b] = acc;
            acc += s_cnt[w][ds][b];
        }
    }
    int t0 = R->tile0, t1 = R->tile1;
    int nt = t1 - t0;
    int per = (nt + 31) / 32;
    int my0 = t0 + lane * per, my1 = min(t0 + (lane + 1) * per, t1);
    for (int b = 0; b < NB; b++) {
        int sum = 0;
        for (int t = my0; t < my1; t++) sum += (int)ws.tile_cnt[(size_t)t * 2 * NB + ds * NB + b];
        int incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += v;
        }
        int run = incl - sum;
        for (int t = my0; t < my1; t++) {
            ws.tile_pref[(size_t)t * NB + b] = run;
            run += (int)ws.tile_cnt[(size_t)t * 2 * NB + ds * NB + b];
        }
    }
}
}

// Per tile: stable partition of split nodes into the other buffer; leaf cells
// go straight to their final position.
template <bool LOOP>
__global__ void __launch_bounds__(STATS_THREADS) k_scatter(WS ws, int parity, int NB) {
    __shared__ unsigned long long K[NBMAX + 1];
    __shared__ int base[NBMAX];
    __shared__ int run[NBMAX];
    __shared__ int wcnt[STATS_THREADS / 32][NBMAX];
    const unsigned FULL = 0xffffffffu;
    const int nt = LOOP ? (ws.cnt->done ? 0 : ws.cnt->tile_count) : (int)gridDim.x;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
    if (LOOP) __syncthreads();
    int r = ws.tile_rec[t];
    int s = ws.tile_start[t], e = ws.tile_end[t];
    int lb = ws.cnt->lb;
    const ARec* R = &ws.recs[r];
    int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int* idx_in = ws.idx[parity];
    if (R->kind != K_SPLIT) {
        for (int i = s + tid; i < e; i += blockDim.x) ws.final_idx[i] = idx_in[i];
        continue;
    }
    int ds = R->split_dim;
    size_t sidx = (size_t)(r - lb);
    if (tid <= NB) {
        double Rd = R->bnd[2 * ds], Ld = R->bnd[2 * ds + 1];
        K[tid] = fkey(bucket_edge(tid, bucket_len(Ld, Rd, NB), Rd));
    }
    if (tid < NB) {
        base[tid] = ws.nb_base[sidx * NB + tid] + ws.tile_pref[(size_t)t * NB + tid];
        run[tid] = 0;
    }
    __syncthreads();
    const double* Lo = ws.f[parity][2 * ds];
    const double* Hi = ws.f[parity][2 * ds + 1];
    for (int b0 = s; b0 < e; b0 += blockDim.x) {
        int i = b0 + tid;
        bool valid = i < e;
        int b = valid ? find_bucket(K, NB, fkey(centroid_of(Lo[i], Hi[i]))) : -2;
        if (valid && b < 0) b = -1;  // counted nowhere: flagged by k_stats
        unsigned grp = __match_any_sync(FULL, b);
        int rank = __popc(grp & lanemask_lt());
        for (int j = tid; j < (STATS_THREADS / 32) * NBMAX; j += blockDim.x) (&wcnt[0][0])[j] = 0;
        __syncthreads();
        if (b >= 0 && (int)(__ffs(grp) - 1) == lane) wcnt[w][b] = __popc(grp);
        __syncthreads();
        int off = 0;
        if (b >= 0) {
            for (int ww = 0; ww < w; ww++) off += wcnt[ww][b];
            int dst = base[b] + run[b] + off + rank;
            int op = 1 - parity;
#pragma unroll
            for (int k = 0; k < 4; k++) ws.f[op][k][dst] = ws.f[parity][k][i];
            ws.idx[op][dst] = idx_in[i];
        }
        __syncthreads();
        if (tid < NB) {
            int tot = 0;
            for (int ww = 0; ww < STATS_THREADS / 32; ww++) tot += wcnt[ww][tid];
            run[tid] += tot;
        }
        __syncthreads();
    }
    }
}

// ------------------------------------------------------------------------
// phase B: one warp builds a subtree of <= SMALL cells in shared memory
// ------------------------------------------------------------------------

// Per-warp shared memory of a subtree: the four box fields of its cells
// (the centroids are recomputed from them with the expression that produced
// them, so the same bits), and the node stack as packed arrays.  8.1 KB, so
// that more warps are resident (the kernel is bound by issue latency).
struct SubSmem {
    double F[4][SMALL];
    unsigned long long K[NBMAX + 1];
    double bRmin[NBMAX];
    double bLmax[NBMAX];
    int gid[SMALL];
    int stk_v[SMALL + 2];      // node
    int stk_depth[SMALL + 2];  // depth
    int cnt[NBMAX];
    int bstart[NBMAX];
    int brun[NBMAX];
    unsigned short perm[SMALL];
    unsigned short tmp[SMALL];
    unsigned short stk_p[SMALL + 2];  // local ptr
    unsigned short stk_n[SMALL + 2];  // size
    unsigned char bkt[SMALL];         // bucket of each position before the partition
    unsigned char nbkt[SMALL];        // bucket of each position after it
    signed char stk_flag[SMALL + 2];  // dim, or dim - 2 after an all-in-one-bucket flip
};
static_assert(SMALL <= 65535, "subtree positions are 16-bit");

__device__ __forceinline__ void sub_push(SubSmem& S, int sp, int v, int p, int n, int flag, int depth) {
    S.stk_v[sp] = v;
    S.stk_p[sp] = (unsigned short)p;
    S.stk_n[sp] = (unsigned short)n;
    S.stk_flag[sp] = (signed char)flag;
    S.stk_depth[sp] = depth;
}


// First-occurrence min over perm[p .. p+n) of field f (min-form key: maxima
// complemented when `is_max`); returns the exact value.  All lanes call.
__device__ __forceinline__ double warp_range_extreme(const SubSmem& S, int f, bool is_max, int p, int n) {
    const unsigned FULL = 0xffffffffu;
    int lane = threadIdx.x & 31;
    unsigned long long best = ~0ull;
    unsigned bpos = 0;  // always a valid position, even for NaN-only ranges
    for (int i = lane; i < n; i += 32) {
        unsigned long long k = fkey(S.F[f][S.perm[p + i]]);
        if (is_max) k = ~k;
        if (k < best) {
            best = k;
            bpos = (unsigned)i;
        }
    }
    unsigned long long ko;
    unsigned po;
    group_min_kp(FULL, best, bpos, &ko, &po);
    return S.F[f][S.perm[p + (int)po]];
}

template <bool LOOP>
__global__ void __launch_bounds__(SUB_WARPS * 32) k_subtree(WS ws, int NB, long long cpl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned FULL = 0xffffffffu;
    int lane = threadIdx.x & 31;
    int w = threadIdx.x >> 5;
    SubSmem& S = reinterpret_cast<SubSmem*>(smem_raw)[w];
    const int nsmall = ws.cnt->small_count;
    const int step = LOOP ? (int)gridDim.x * SUB_WARPS : INT32_MAX / 2;
    for (int sidx = blockIdx.x * SUB_WARPS + w; sidx < nsmall; sidx += step) {
    __syncwarp();
    int r = ws.small_list[sidx];
    ARec* RR = &ws.recs[r];
    int p0 = RR->ptr, s = RR->size, par = RR->parity, d0 = RR->dim, lvl = RR->level;
    for (int i = lane; i < s; i += 32) {
        for (int k = 0; k < 4; k++) S.F[k][i] = ws.f[par][k][p0 + i];
        S.gid[i] = ws.idx[par][p0 + i];
        S.perm[i] = (unsigned short)i;
    }
    LRec* L = ws.lrec + 2 * (size_t)p0;
    if (lane == 0) {
        LRec z;
        z.Lmax = -1.0;
        z.Rmin = -1.0;
        z.child = -1;
        z.ptr = p0;
        z.size = s;
        z.dim = d0;
        L[0] = z;
        sub_push(S, 0, 0, 0, s, d0, lvl);
    }
    __syncwarp();
    int sp = 1, nloc = 1, maxd = lvl;
    bool err = false;
    while (sp > 0) {
        sp--;
        int v = S.stk_v[sp], p = S.stk_p[sp], n = S.stk_n[sp], flag = S.stk_flag[sp], depth = S.stk_depth[sp];
        __syncwarp();
        int d = flag < 0 ? flag + 2 : flag;
        if ((long long)n <= cpl) continue;
        // get_bounds of the node (creation.py:271-277)
        double R = warp_range_extreme(S, 2 * d, false, p, n);
        double Lr = warp_range_extreme(S, 2 * d + 1, true, p, n);
        double bl = bucket_len(Lr, R, NB);
        for (int j = lane; j <= NB; j += 32) S.K[j] = fkey(bucket_edge(j, bl, R));  // NB + 1 edges
        if (lane < NB) {
            S.cnt[lane] = 0;
            S.brun[lane] = 0;
        }
        __syncwarp();
        bool lbad = false;
        for (int i = lane; i < n; i += 32) {
            const int e = S.perm[p + i];
            int b = find_bucket(S.K, NB, fkey(centroid_of(S.F[2 * d][e], S.F[2 * d + 1][e])));
            if (b < 0) {
                lbad = true;
                b = 0;
            }
            S.bkt[i] = (unsigned char)b;
            atomicAdd(&S.cnt[b], 1);
        }
        if (__any_sync(FULL, lbad)) {
            err = true;
            continue;  // upstream indexes past its buckets; keep a leaf
        }
        __syncwarp();
        if (lane < 32) {
            int c = lane < NB ? S.cnt[lane] : 0;
            int incl = c;
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += t;
            }
            if (lane < NB) S.bstart[lane] = incl - c;
        }
        __syncwarp();
        // stable partition (stable_partition / sort_bbox_indices creation.py:54-150)
        for (int c0 = 0; c0 < n; c0 += 32) {
            int i = c0 + lane;
            int b = i < n ? (int)S.bkt[i] : 255;
            unsigned grp = __match_any_sync(FULL, b);
            int rank = __popc(grp & lanemask_lt());
            if (i < n) {
                const int dst = S.bstart[b] + S.brun[b] + rank;
                S.tmp[dst] = S.perm[p + i];
                S.nbkt[dst] = (unsigned char)b;
            }
            __syncwarp();
            if (i < n && (int)(__ffs(grp) - 1) == lane) S.brun[b] += __popc(grp);
            __syncwarp();
        }
        for (int i = lane; i < n; i += 32) S.perm[p + i] = S.tmp[i];
        __syncwarp();
        // special case creation.py:311-320
        if (cpl == 1 && n == 2) {
            if (lane == 0) {
                L[v].Lmax = Lr;
                L[v].Rmin = R;
                L[v].child = nloc;
                LRec a;
                a.Lmax = -1.0;
                a.Rmin = -1.0;
                a.child = -1;
                a.size = 1;
                a.dim = 1 - d;
                a.ptr = p0 + p;
                L[nloc] = a;
                a.ptr = p0 + p + 1;
                L[nloc + 1] = a;
            }
            nloc += 2;
            maxd = max(maxd, depth + 1);
            __syncwarp();
            continue;
        }
        // per-bucket bounds (creation.py:300-306): the first-occurrence
        // minimum of Rmin and maximum of Lmax of every bucket in one pass over
        // the node's positions (after the partition bucket b is a contiguous
        // run).  The lanes of one bucket reduce (key, position) together and
        // their first lane folds the result into the bucket's running minimum
        // (a later chunk never wins a tie: first occurrence).  Keys and
        // positions use scratch the partition is done with: S.K (Rmin keys),
        // S.bLmax viewed as keys (Lmax), S.brun / S.bstart (positions).
        {
            unsigned long long* kR = S.K;
            unsigned long long* kL = reinterpret_cast<unsigned long long*>(S.bLmax);
            if (lane < NB) {
                kR[lane] = ~0ull;
                kL[lane] = ~0ull;
                S.brun[lane] = S.bstart[lane];  // positions when every key of the bucket ties at ~0
            }
            __syncwarp();
            for (int c0 = 0; c0 < n; c0 += 32) {
                const int i = c0 + lane;
                int b = -1;
                unsigned long long kr = ~0ull, kl = ~0ull;
                if (i < n) {
                    b = S.nbkt[i];
                    const int e = S.perm[p + i];
                    kr = fkey(S.F[2 * d][e]);
                    kl = ~fkey(S.F[2 * d + 1][e]);
                }
                const unsigned grp = __match_any_sync(FULL, b);
                unsigned long long mr, ml;
                unsigned pr, pl;
                group_min_kp(grp, kr, (unsigned)i, &mr, &pr);
                group_min_kp(grp, kl, (unsigned)i, &ml, &pl);
                if (b >= 0 && lane == (int)(__ffs(grp) - 1)) {
                    if (mr < kR[b]) {
                        kR[b] = mr;
                        S.brun[b] = (int)pr;
                    }
                    if (ml < kL[b]) {
                        kL[b] = ml;
                        S.bstart[b] = (int)pl;
                    }
                }
                __syncwarp();
            }
            if (lane < NB) {
                const bool any = S.cnt[lane] > 0;
                const double rmin = any ? S.F[2 * d][S.perm[p + S.brun[lane]]] : DBL_MAX;
                const double lmax = any ? S.F[2 * d + 1][S.perm[p + S.bstart[lane]]] : -DBL_MAX;
                S.bRmin[lane] = rmin;
                S.bLmax[lane] = lmax;  // replaces this bucket's key
            }
            __syncwarp();
        }
        Decision D = warp_decide(S.cnt, S.bRmin, S.bLmax, NB, n, R, Lr, bl);
        if (D.kind == 0) {
            // all cells in one bucket (creation.py:345-358)
            if (flag >= 0) {
                if (lane == 0) {
                    L[v].dim = 1 - L[v].dim;
                    sub_push(S, sp, v, p, n, (1 - d) - 2, depth);
                }
                sp++;
            } else if (lane == 0) {
                L[v].Lmax = -1.0;
                L[v].Rmin = -1.0;
            }
            __syncwarp();
            continue;
        }
        if (D.kind < 0) {
            err = true;
            continue;
        }
        int nl = D.nleft;
        if (lane == 0) {
            L[v].Lmax = D.Lmax;
            L[v].Rmin = D.Rmin;
            L[v].child = nloc;
            LRec a;
            a.Lmax = -1.0;
            a.Rmin = -1.0;
            a.child = -1;
            a.dim = 1 - d;
            a.ptr = p0 + p;
            a.size = nl;
            L[nloc] = a;
            a.ptr = p0 + p + nl;
            a.size = n - nl;
            L[nloc + 1] = a;
            // push right, then left (creation.py:378-379)
            sub_push(S, sp, nloc + 1, p + nl, n - nl, 1 - d, depth + 1);
            sub_push(S, sp + 1, nloc, p, nl, 1 - d, depth + 1);
        }
        sp += 2;
        nloc += 2;
        maxd = max(maxd, depth + 1);
        __syncwarp();
    }
    __syncwarp();
    for (int i = lane; i < s; i += 32) ws.final_idx[p0 + i] = S.gid[S.perm[i]];
    if (lane == 0) {
        RR->splits = (nloc - 1) / 2;
        RR->nlocal = nloc;
        RR->err = err ? 1 : 0;
        atomicMax(&ws.cnt->max_depth, maxd);
        atomicMax(&ws.tree_depth[RR->tree], maxd);
        if (err) atomicOr(&ws.cnt->err, CT_DEVERR_BUCKET);
    }
    }
}

// ------------------------------------------------------------------------
// phase C: numbering and emission
// ------------------------------------------------------------------------

// ---- the device-driven level loop: per-level bookkeeping on the device ----
__global__ void k_level_start(WS ws) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && !ws.cnt->done) ws.cnt->tile_count = 0;
}

// After a level's scatter: the records it created are the next level; none
// (or a capacity error) ends the loop.
__global__ void k_level_next(WS ws, int L) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Counters* c = ws.cnt;
    if (c->done) return;
    int nb = c->le, ne = c->rec_count;
    if ((c->err & 0x80000000u) || ne == nb) {
        c->done = 1;
        return;
    }
    if (L + 1 >= DEV_MAX_LEVELS) {  // more levels than the loop runs
        c->done = 1;
        c->err |= CT_DEVERR_LOOP;
        return;
    }
    c->lb = nb;
    c->le = ne;
    ws.lvl_b[L + 1] = nb;
    ws.lvl_e[L + 1] = ne;
    c->nlev = L + 2;
}

__global__ void k_count_up_dev(WS ws, int L) {
    if (L >= ws.cnt->nlev) return;
    int b = ws.lvl_b[L], e = ws.lvl_e[L];
    for (int r = b + blockIdx.x * blockDim.x + threadIdx.x; r < e; r += gridDim.x * blockDim.x) {
        ARec* R = &ws.recs[r];
        if (R->kind == K_SPLIT) R->splits = 1 + ws.recs[R->child].splits + ws.recs[R->child + 1].splits;
        else if (R->kind == K_LEAF) R->splits = 0;
    }
}

__global__ void k_number_down_dev(WS ws, int L) {
    if (L >= ws.cnt->nlev) return;
    int b = ws.lvl_b[L], e = ws.lvl_e[L];
    for (int r = b + blockIdx.x * blockDim.x + threadIdx.x; r < e; r += gridDim.x * blockDim.x) {
        ARec* R = &ws.recs[r];
        if (r < ws.n_roots) {
            R->S = 0;
            R->pos = 0;
        }
        if (R->kind == K_SPLIT) {
            ARec* A = &ws.recs[R->child];
            ARec* B = &ws.recs[R->child + 1];
            A->S = R->S + 1;
            B->S = R->S + 1 + A->splits;
            A->pos = 1 + 2 * R->S;
            B->pos = 2 + 2 * R->S;
        }
    }
}

// Node counts (1 + 2 splits of the root), their offsets (one block, serial
// prefix in chunks of the block) and depths per tree; the status word gets
// the builder's error bits and whether the node capacity holds the trees.
__global__ void k_forest_counts(WS ws, int64_t* n_nodes, int64_t* node_off, int* depth, int64_t capacity,
                                unsigned int* status) {
    __shared__ long long carry;
    __shared__ long long part[256];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ws.n_roots; base += blockDim.x) {
        int t = base + threadIdx.x;
        long long v = 0;
        if (t < ws.n_roots) {
            v = 1 + 2 * ws.recs[t].splits;
            n_nodes[t] = v;
            depth[t] = ws.tree_depth[t];
        }
        part[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < (int)blockDim.x; o <<= 1) {
            long long y = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
            __syncthreads();
            part[threadIdx.x] += y;
            __syncthreads();
        }
        if (t < ws.n_roots) node_off[t] = carry + part[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += part[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        node_off[ws.n_roots] = carry;
        unsigned st = ws.cnt->err & (CT_DEVERR_BUCKET | CT_DEVERR_LOOP);
        if (ws.cnt->err & 0x80000000u) st |= CT_DEVERR_CAPACITY;
        if (!ws.cnt->done && ws.cnt->nlev > 0 && ws.cnt->tile_count > 0) st |= CT_DEVERR_LOOP;
        if (carry > capacity) st |= CT_DEVERR_CAPACITY;
        *status = st;
    }
}

__global__ void k_count_up(WS ws, int b, int e) {
    int r = b + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= e) return;
    ARec* R = &ws.recs[r];
    if (R->kind == K_SPLIT) R->splits = 1 + ws.recs[R->child].splits + ws.recs[R->child + 1].splits;
    else if (R->kind == K_LEAF) R->splits = 0;
    // K_SUBTREE: set by k_subtree
}

__global__ void k_number_down(WS ws, int b, int e) {
    int r = b + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= e) return;
    ARec* R = &ws.recs[r];
    if (r < ws.n_roots) {  // every tree is numbered from its own root
        R->S = 0;
        R->pos = 0;
    }
    if (R->kind == K_SPLIT) {
        ARec* A = &ws.recs[R->child];
        ARec* B = &ws.recs[R->child + 1];
        A->S = R->S + 1;
        B->S = R->S + 1 + A->splits;
        A->pos = 1 + 2 * R->S;
        B->pos = 2 + 2 * R->S;
    }
}

struct NodesOut {
    int64_t* child;
    double* Lmax;
    double* Rmin;
    int64_t* ptr;
    int64_t* size;
    uint8_t* dim;
};

__device__ __forceinline__ void put_node(const NodesOut& o, long long pos, long long child, double Lmax, double Rmin,
                                         long long ptr, long long size, int dim) {
    o.child[pos] = child;
    o.Lmax[pos] = Lmax;
    o.Rmin[pos] = Rmin;
    o.ptr[pos] = ptr;
    o.size[pos] = size;
    o.dim[pos] = (uint8_t)(dim != 0);
}

// node_off (forest builds): first output node of every tree; node counts
// n_nodes of one tree are node_off[t + 1] - node_off[t].  Positions, children
// and ptr are written relative to the node's own tree.
__device__ __forceinline__ void tree_frame(const WS& ws, const int64_t* node_off, long long n_nodes, int t,
                                           long long* noff, long long* nn, long long* eoff) {
    if (node_off) {
        *noff = node_off[t];
        *nn = node_off[t + 1] - node_off[t];
        *eoff = ws.tree_off[t];
    } else {
        *noff = 0;
        *nn = n_nodes;
        *eoff = 0;
    }
}

__global__ void k_emit_phaseA(WS ws, int nrec, long long n_nodes, NodesOut o, const int64_t* node_off) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const ARec* R = &ws.recs[r];
    if (R->kind != K_SPLIT && R->kind != K_LEAF) return;
    long long noff, nn, eoff;
    tree_frame(ws, node_off, n_nodes, R->tree, &noff, &nn, &eoff);
    if (R->pos < 0 || R->pos >= nn) {
        atomicOr(&ws.cnt->err, 0x40000000u);
        return;
    }
    if (R->kind == K_SPLIT) put_node(o, noff + R->pos, 1 + 2 * R->S, R->Lmax, R->Rmin, R->ptr - eoff, R->size, R->dim);
    else put_node(o, noff + R->pos, -1, R->Lmax, R->Rmin, R->ptr - eoff, R->size, R->dim);
}

// One warp per subtree root: local records to their final positions.
__global__ void k_emit_subtrees(WS ws, long long n_nodes, NodesOut o, const int64_t* node_off) {
    int lane = threadIdx.x & 31;
    int sidx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (sidx >= ws.cnt->small_count) return;
    const ARec* R = &ws.recs[ws.small_list[sidx]];
    const LRec* L = ws.lrec + 2 * (size_t)R->ptr;
    long long off = 2 * R->S;
    long long noff, nn, eoff;
    tree_frame(ws, node_off, n_nodes, R->tree, &noff, &nn, &eoff);
    for (int j = lane; j < R->nlocal; j += 32) {
        LRec a = L[j];
        long long pos = (j == 0) ? R->pos : (long long)j + off;
        long long child = (a.child < 0) ? -1 : (long long)a.child + off;
        if (pos < 0 || pos >= nn || child >= nn) {
            atomicOr(&ws.cnt->err, 0x40000000u);
            continue;
        }
        put_node(o, noff + pos, child, a.Lmax, a.Rmin, a.ptr - eoff, a.size, a.dim);
    }
}

__global__ void k_emit_indices(WS ws, int n, int64_t* bb_indices, bool forest) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        bb_indices[i] = forest ? ws.final_idx[i] - ws.tree_off[ws.elem_tree[i]] : ws.final_idx[i];
}

__global__ void k_emit_phaseA_dev(WS ws, NodesOut o, const int64_t* node_off, const unsigned int* status) {
    if (*status) return;
    int nrec = ws.cnt->rec_count;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += gridDim.x * blockDim.x) {
        const ARec* R = &ws.recs[r];
        if (R->kind != K_SPLIT && R->kind != K_LEAF) continue;
        long long noff, nn, eoff;
        tree_frame(ws, node_off, 0, R->tree, &noff, &nn, &eoff);
        if (R->pos < 0 || R->pos >= nn) {
            atomicOr(&ws.cnt->err, 0x40000000u);
            continue;
        }
        if (R->kind == K_SPLIT)
            put_node(o, noff + R->pos, 1 + 2 * R->S, R->Lmax, R->Rmin, R->ptr - eoff, R->size, R->dim);
        else put_node(o, noff + R->pos, -1, R->Lmax, R->Rmin, R->ptr - eoff, R->size, R->dim);
    }
}

__global__ void k_emit_subtrees_dev(WS ws, NodesOut o, const int64_t* node_off, const unsigned int* status) {
    if (*status) return;
    int lane = threadIdx.x & 31;
    int nsmall = ws.cnt->small_count;
    for (int sidx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sidx < nsmall;
         sidx += (gridDim.x * blockDim.x) >> 5) {
        const ARec* R = &ws.recs[ws.small_list[sidx]];
        const LRec* Lr = ws.lrec + 2 * (size_t)R->ptr;
        long long off = 2 * R->S;
        long long noff, nn, eoff;
        tree_frame(ws, node_off, 0, R->tree, &noff, &nn, &eoff);
        for (int j = lane; j < R->nlocal; j += 32) {
            LRec a = Lr[j];
            long long pos = (j == 0) ? R->pos : (long long)j + off;
            long long child = (a.child < 0) ? -1 : (long long)a.child + off;
            if (pos < 0 || pos >= nn || child >= nn) {
                atomicOr(&ws.cnt->err, 0x40000000u);
                continue;
            }
            put_node(o, noff + pos, child, a.Lmax, a.Rmin, a.ptr - eoff, a.size, a.dim);
        }
    }
}

// emission errors (a node position outside its tree's range) into the status
__global__ void k_forest_status_final(WS ws, unsigned int* status) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && (ws.cnt->err & 0x40000000u)) *status |= CT_DEVERR_CAPACITY;
}

// ------------------------------------------------------------------------
// forest initialisation: one root record per tree
// ------------------------------------------------------------------------

__global__ void k_forest_reset(WS ws) {
    Counters* c = ws.cnt;
    c->rec_count = ws.n_roots;
    c->tile_count = 0;
    c->small_count = 0;
    c->err = 0;
    c->max_depth = 0;
    c->lb = 0;
    c->le = ws.n_roots;
    c->done = 0;
    c->nlev = 1;
    ws.lvl_b[0] = 0;
    ws.lvl_e[0] = ws.n_roots;
}

__global__ void k_forest_roots(WS ws) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ws.n_roots; t += gridDim.x * blockDim.x) {
        ARec r;
        memset(&r, 0, sizeof(r));
        r.ptr = (int)ws.tree_off[t];
        r.size = (int)(ws.tree_off[t + 1] - ws.tree_off[t]);
        r.dim = 0;
        r.kind = (r.size > SMALL) ? K_PENDING : K_SUBTREE;
        r.child = -1;
        r.level = 0;
        r.split_dim = -1;
        r.Lmax = -1.0;
        r.Rmin = -1.0;
        r.tree = t;
        ws.recs[t] = r;
        ws.tree_depth[t] = 0;
        for (int f = 0; f < 4; f++) {
            ws.root_key[4 * t + f] = ~0ull;
            ws.root_zp[4 * t + f] = INT32_MAX;
        }
        if (r.kind == K_SUBTREE) ws.small_list[atomicAdd(&ws.cnt->small_count, 1)] = t;
    }
}

__global__ void k_forest_elem_tree(WS ws, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int lo = 0, hi = ws.n_roots;  // tree_off[lo] <= i < tree_off[hi]
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (ws.tree_off[mid] <= i) lo = mid;
            else hi = mid;
        }
        ws.elem_tree[i] = lo;
    }
}

// First-occurrence bounds of every tree's boxes (root get_bounds, per tree).
__global__ void k_forest_root_bounds(WS ws, int n) {
    const unsigned FULL = 0xffffffffu;
    int stride = gridDim.x * blockDim.x;
    int iters = (n + stride - 1) / stride;
    for (int it = 0; it < iters; it++) {
        int i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool valid = i < n;
        int t = valid ? ws.elem_tree[i] : -1;
        unsigned same = __match_any_sync(FULL, t);
        for (int f = 0; f < 4; f++) {
            unsigned long long kk = ~0ull;
            if (valid) {
                double v = ws.f[0][f][i];
                kk = (f & 1) ? ~fkey(v) : fkey(v);
                if (is_zero(v)) atomicMin(&ws.root_zp[4 * t + f], i);
            }
            if (same == FULL) {
                unsigned long long m = group_min_k(FULL, kk);
                if ((threadIdx.x & 31) == 0 && t >= 0) atomicMin(&ws.root_key[4 * t + f], m);
            } else if (valid) {
                atomicMin(&ws.root_key[4 * t + f], kk);
            }
        }
    }
}

__global__ void k_forest_root_resolve(WS ws) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ws.n_roots; t += gridDim.x * blockDim.x) {
        if (ws.tree_off[t + 1] <= ws.tree_off[t]) continue;
        for (int f = 0; f < 4; f++)
            ws.recs[t].bnd[f] = resolve_key(ws.root_key[4 * t + f], f, ws.root_zp[4 * t + f], ws.f[0][f]);
    }
}

}  // namespace ct

using namespace ct;

extern "C" {

int64_t ct_pessimistic_n_nodes(int64_t n) {
    // creation.py:216-230
    int64_t n_nodes = n;
    int64_t nodes = (n + 1) / 2;
    while (nodes > 1) {
        n_nodes += nodes;
        nodes = (nodes + 1) / 2;
    }
    return n_nodes + 1;
}

size_t ct_build_workspace_size(int64_t n, int32_t NB, int32_t factor) {
    if (NB < 2 || NB > NBMAX || n < 0 || factor < 1) return 0;
    return carve(nullptr, n, NB, factor, nullptr);
}

}  // extern "C"

namespace ct {

// Phases A, B and C over the root records already in place (one per tree).
// Returns the record count through *nrec_out; one host synchronisation per
// phase-A level.
static int build_levels(WS& ws, cudaStream_t st, int NB, int64_t cpl, bool run_phase_a, int n_roots,
                        Counters* hc_out) {
    // a function attribute belongs to the current device (and context): set
    // it on every call rather than once per process
    CT_CUDA(cudaFuncSetAttribute(k_subtree<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(SUB_WARPS * sizeof(SubSmem))));
    std::vector<int> level_b, level_e;
    level_b.push_back(0);
    level_e.push_back(n_roots);
    int parity = 0;
    Counters hc;
    if (run_phase_a) {
        while (true) {
            int lb = level_b.back(), le = level_e.back();
            int width = le - lb;
            // tiles for pending nodes of this level
            cudaMemsetAsync(&ws.cnt->tile_count, 0, sizeof(int), st);
            int g = std::max(1, std::min((width + 3) / 4, 4096));
            k_make_tiles<<<g, 128, 0, st>>>(ws, NB);
            CT_CHECK_LAUNCH("make_tiles");
            CT_CUDA(cudaMemcpyAsync(&hc, ws.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, st));
            CT_CUDA(cudaStreamSynchronize(st));
            if (hc.err & 0x80000000u) return ct_fail(CT_ERR_WORKSPACE, "builder tile capacity exceeded");
            int ntiles = hc.tile_count;
            if (ntiles == 0) break;
            k_stats<false><<<ntiles, STATS_THREADS, 0, st>>>(ws, parity, NB);
            k_decide<false><<<(width + 3) / 4, 128, 0, st>>>(ws, NB, (long long)cpl);
            k_scatter<false><<<ntiles, STATS_THREADS, 0, st>>>(ws, parity, NB);
            CT_CHECK_LAUNCH("phase A level");
            CT_CUDA(cudaMemcpyAsync(&hc, ws.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, st));
            CT_CUDA(cudaStreamSynchronize(st));
            if (hc.err & 0x80000000u)
                return ct_fail(CT_ERR_WORKSPACE, "builder node-record capacity exceeded (unbalanced tree)");
            int nb_ = le, ne_ = hc.rec_count;
            if (ne_ == nb_) break;
            level_b.push_back(nb_);
            level_e.push_back(ne_);
            parity = 1 - parity;
            // publish the next level range to the device
            int range[2] = {nb_, ne_};
            CT_CUDA(cudaMemcpyAsync(&ws.cnt->lb, range, 2 * sizeof(int), cudaMemcpyHostToDevice, st));
            CT_CUDA(cudaStreamSynchronize(st));
        }
    }
    CT_CUDA(cudaMemcpyAsync(&hc, ws.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    int nsmall = hc.small_count;
    if (nsmall > 0) {
        int blocks = (nsmall + SUB_WARPS - 1) / SUB_WARPS;
        k_subtree<false><<<blocks, SUB_WARPS * 32, SUB_WARPS * sizeof(SubSmem), st>>>(ws, NB, (long long)cpl);
        CT_CHECK_LAUNCH("subtree");
    }
    // phase C: split counts bottom-up, pre-order ranks top-down
    for (int L = (int)level_b.size() - 1; L >= 0; L--) {
        int b = level_b[L], e = level_e[L];
        k_count_up<<<(e - b + 255) / 256, 256, 0, st>>>(ws, b, e);
    }
    for (size_t L = 0; L < level_b.size(); L++) {
        int b = level_b[L], e = level_e[L];
        k_number_down<<<(e - b + 255) / 256, 256, 0, st>>>(ws, b, e);
    }
    CT_CHECK_LAUNCH("numbering");
    CT_CUDA(cudaMemcpyAsync(&hc, ws.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    if (hc.err & CT_DEVERR_BUCKET)
        return ct_fail(CT_ERR_DEVICE, "tree construction failed: a cell centroid fell outside every bucket");
    // remember the record count for the emit call
    CT_CUDA(cudaMemcpyAsync(&ws.cnt->pad, &hc.rec_count, sizeof(int), cudaMemcpyHostToDevice, st));
    CT_CUDA(cudaStreamSynchronize(st));
    *hc_out = hc;
    return CT_OK;
}

static int emit_nodes(const WS& ws, int64_t n, long long n_nodes, const int64_t* node_off, int64_t* child,
                      double* Lmax, double* Rmin, int64_t* ptr, int64_t* size, uint8_t* dim, int64_t* bb_indices,
                      cudaStream_t st) {
    Counters hc;
    CT_CUDA(cudaMemcpyAsync(&hc, ws.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    int nrec = hc.pad;
    NodesOut o{child, Lmax, Rmin, ptr, size, dim};
    k_emit_phaseA<<<(nrec + 255) / 256, 256, 0, st>>>(ws, nrec, n_nodes, o, node_off);
    if (hc.small_count > 0)
        k_emit_subtrees<<<(hc.small_count * 32 + 127) / 128, 128, 0, st>>>(ws, n_nodes, o, node_off);
    if (n > 0) {
        int g = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
        k_emit_indices<<<g, 256, 0, st>>>(ws, (int)n, bb_indices, node_off != nullptr);
    }
    CT_CHECK_LAUNCH("emit");
    CT_CUDA(cudaMemcpyAsync(&hc, ws.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    if (hc.err & 0x40000000u) return ct_fail(CT_ERR_DEVICE, "tree emission: node position out of range");
    return CT_OK;
}

}  // namespace ct

extern "C" {

int ct_build_tree(const double* bb, int64_t n, int32_t NB, int64_t cpl, int32_t factor, void* workspace,
                  size_t ws_bytes, int64_t* n_nodes_host, int32_t* max_depth_host, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (NB < 2 || NB > NBMAX) return ct_fail(CT_ERR_ARG, "n_buckets must be in [2, 32] for the GPU builder");
    if (cpl < 1) return ct_fail(CT_ERR_ARG, "cells_per_leaf must be >= 1");
    if (n < 0 || n >= (int64_t)INT32_MAX / 2) return ct_fail(CT_ERR_ARG, "n_elements out of range");
    if (factor < 1) return ct_fail(CT_ERR_ARG, "capacity_factor must be >= 1");
    size_t need = carve(nullptr, n, NB, factor, nullptr);
    if (!workspace || ws_bytes < need) return ct_fail(CT_ERR_WORKSPACE, "build workspace too small");
    if (n > 0 && !bb) return ct_fail(CT_ERR_ARG, "bb_coords is null");
    WS ws;
    carve((char*)workspace, n, NB, factor, &ws);
    int ni = (int)n;
    int root_dim = 0;
    k_reset<<<1, 1, 0, st>>>(ws, ni, 0, root_dim);
    if (ni > 0) {
        int g = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
        k_init_elems<<<g, 256, 0, st>>>(bb, ni, ws);
        k_root_bounds<<<g, 256, 0, st>>>(ws, ni);
        k_root_resolve<<<1, 1, 0, st>>>(ws, ni);
    }
    CT_CHECK_LAUNCH("build init");
    Counters hc;
    int s = build_levels(ws, st, NB, cpl, ni > SMALL, 1, &hc);
    if (s) return s;
    long long root_splits = 0;
    CT_CUDA(cudaMemcpyAsync(&root_splits, &ws.recs[0].splits, sizeof(long long), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    if (n_nodes_host) *n_nodes_host = 1 + 2 * root_splits;
    if (max_depth_host) *max_depth_host = hc.max_depth;
    return CT_OK;
}

int ct_build_emit(const void* workspace, int64_t n, int32_t NB, int32_t factor, int64_t* child, double* Lmax,
                  double* Rmin, int64_t* ptr, int64_t* size, uint8_t* dim, int64_t* bb_indices, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (NB < 2 || NB > NBMAX || factor < 1) return ct_fail(CT_ERR_ARG, "bad n_buckets / capacity_factor");
    WS ws;
    carve((char*)workspace, n, NB, factor, &ws);
    long long root_splits = 0;
    CT_CUDA(cudaMemcpyAsync(&root_splits, &ws.recs[0].splits, sizeof(long long), cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    return emit_nodes(ws, n, 1 + 2 * root_splits, nullptr, child, Lmax, Rmin, ptr, size, dim, bb_indices, st);
}

size_t ct_build_forest_workspace_size(int64_t n_total, int32_t n_trees, int32_t NB, int32_t factor) {
    if (NB < 2 || NB > NBMAX || n_total < 0 || factor < 1 || n_trees < 1) return 0;
    return carve(nullptr, n_total, NB, factor, nullptr, n_trees, true);
}

int ct_build_forest(const double* bb, int64_t n_total, const int64_t* tree_off_host, int32_t n_trees, int32_t NB,
                    int64_t cpl, int32_t factor, void* workspace, size_t ws_bytes, int64_t* n_nodes_host,
                    int32_t* max_depth_host, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (NB < 2 || NB > NBMAX) return ct_fail(CT_ERR_ARG, "n_buckets must be in [2, 32] for the GPU builder");
    if (cpl < 1) return ct_fail(CT_ERR_ARG, "cells_per_leaf must be >= 1");
    if (n_trees < 1 || !tree_off_host) return ct_fail(CT_ERR_ARG, "need at least one tree");
    if (n_total < 0 || n_total >= (int64_t)INT32_MAX / 2) return ct_fail(CT_ERR_ARG, "n_elements out of range");
    if (factor < 1) return ct_fail(CT_ERR_ARG, "capacity_factor must be >= 1");
    if (tree_off_host[0] != 0 || tree_off_host[n_trees] != n_total)
        return ct_fail(CT_ERR_ARG, "tree offsets must start at 0 and end at n_total");
    bool any_large = false;
    for (int t = 0; t < n_trees; t++) {
        int64_t m = tree_off_host[t + 1] - tree_off_host[t];
        if (m < 1) return ct_fail(CT_ERR_ARG, "every tree needs at least one element");
        any_large |= m > SMALL;
    }
    size_t need = carve(nullptr, n_total, NB, factor, nullptr, n_trees, true);
    if (!workspace || ws_bytes < need) return ct_fail(CT_ERR_WORKSPACE, "build workspace too small");
    if (!bb) return ct_fail(CT_ERR_ARG, "bb_coords is null");
    WS ws;
    carve((char*)workspace, n_total, NB, factor, &ws, n_trees, true);
    int ni = (int)n_total;
    CT_CUDA(cudaMemcpyAsync(ws.tree_off, tree_off_host, sizeof(int64_t) * ((size_t)n_trees + 1),
                            cudaMemcpyHostToDevice, st));
    int g = (int)std::min<int64_t>((n_total + 255) / 256, 152 * 8);
    int gt = (int)std::min<int64_t>((n_trees + 255) / 256, 152 * 8);
    k_forest_reset<<<1, 1, 0, st>>>(ws);
    k_forest_roots<<<gt, 256, 0, st>>>(ws);
    k_init_elems<<<g, 256, 0, st>>>(bb, ni, ws);
    k_forest_elem_tree<<<g, 256, 0, st>>>(ws, ni);
    k_forest_root_bounds<<<g, 256, 0, st>>>(ws, ni);
    k_forest_root_resolve<<<gt, 256, 0, st>>>(ws);
    CT_CHECK_LAUNCH("forest init");
    Counters hc;
    int s = build_levels(ws, st, NB, cpl, any_large, n_trees, &hc);
    if (s) return s;
    std::vector<ARec> roots(n_trees);
    std::vector<int> depth(n_trees);
    CT_CUDA(cudaMemcpyAsync(roots.data(), ws.recs, sizeof(ARec) * n_trees, cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaMemcpyAsync(depth.data(), ws.tree_depth, sizeof(int) * n_trees, cudaMemcpyDeviceToHost, st));
    CT_CUDA(cudaStreamSynchronize(st));
    for (int t = 0; t < n_trees; t++) {
        if (n_nodes_host) n_nodes_host[t] = 1 + 2 * roots[t].splits;
        if (max_depth_host) max_depth_host[t] = depth[t];
    }
    return CT_OK;
}

// Build + emit of a forest with every level driven on the device: a fixed
// sequence of launches (the level loop runs DEV_MAX_LEVELS times; levels past
// the last one find nothing to do), no host synchronisation, so the whole
// call can be captured in a CUDA graph and replayed.  The trees' sizes are
// fixed by the host-side offsets; everything that depends on the boxes --
// levels, node counts and offsets, depths -- stays on the device.
int ct_build_forest_async(const double* bb, int64_t n_total, const int64_t* tree_off_host,
                          const int64_t* tree_off_dev, int32_t n_trees, int32_t NB, int64_t cpl, int32_t factor,
                          void* workspace, size_t ws_bytes, int64_t node_capacity, int64_t* child, double* Lmax,
                          double* Rmin, int64_t* ptr, int64_t* size, uint8_t* dim, int64_t* bb_indices,
                          int64_t* n_nodes_dev, int64_t* node_off_dev, int32_t* max_depth_dev,
                          unsigned int* status_dev, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (NB < 2 || NB > NBMAX) return ct_fail(CT_ERR_ARG, "n_buckets must be in [2, 32] for the GPU builder");
    if (cpl < 1) return ct_fail(CT_ERR_ARG, "cells_per_leaf must be >= 1");
    if (n_trees < 1 || !tree_off_host || !tree_off_dev) return ct_fail(CT_ERR_ARG, "need at least one tree");
    if (n_total < 1 || n_total >= (int64_t)INT32_MAX / 2) return ct_fail(CT_ERR_ARG, "n_elements out of range");
    if (factor < 1) return ct_fail(CT_ERR_ARG, "capacity_factor must be >= 1");
    if (tree_off_host[0] != 0 || tree_off_host[n_trees] != n_total)
        return ct_fail(CT_ERR_ARG, "tree offsets must start at 0 and end at n_total");
    if (!n_nodes_dev || !node_off_dev || !max_depth_dev || !status_dev || !bb_indices || !child)
        return ct_fail(CT_ERR_ARG, "null output");
    bool any_large = false;
    for (int t = 0; t < n_trees; t++) {
        int64_t m = tree_off_host[t + 1] - tree_off_host[t];
        if (m < 1) return ct_fail(CT_ERR_ARG, "every tree needs at least one element");
        any_large |= m > SMALL;
    }
    size_t need = carve(nullptr, n_total, NB, factor, nullptr, n_trees, true);
    if (!workspace || ws_bytes < need) return ct_fail(CT_ERR_WORKSPACE, "build workspace too small");
    if (!bb) return ct_fail(CT_ERR_ARG, "bb_coords is null");
    WS ws;
    carve((char*)workspace, n_total, NB, factor, &ws, n_trees, true);
    CT_CUDA(cudaMemcpyAsync(ws.tree_off, tree_off_dev, sizeof(int64_t) * ((size_t)n_trees + 1),
                            cudaMemcpyDeviceToDevice, st));
    const int ni = (int)n_total;
    const int g = (int)std::min<int64_t>((n_total + 255) / 256, 152 * 8);
    const int gt = (int)std::min<int64_t>((n_trees + 255) / 256, 152 * 8);
    k_forest_reset<<<1, 1, 0, st>>>(ws);
    k_forest_roots<<<gt, 256, 0, st>>>(ws);
    k_init_elems<<<g, 256, 0, st>>>(bb, ni, ws);
    k_forest_elem_tree<<<g, 256, 0, st>>>(ws, ni);
    k_forest_root_bounds<<<g, 256, 0, st>>>(ws, ni);
    k_forest_root_resolve<<<gt, 256, 0, st>>>(ws);
    CT_CHECK_LAUNCH("forest init");
    CT_CUDA(cudaFuncSetAttribute(k_subtree<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(SUB_WARPS * sizeof(SubSmem))));
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int G = sms * 8;
    if (any_large) {
        for (int L = 0; L < DEV_MAX_LEVELS; L++) {
            const int parity = L & 1;
            k_level_start<<<1, 32, 0, st>>>(ws);
            k_make_tiles<<<G, 128, 0, st>>>(ws, NB);
            k_stats<true><<<G, STATS_THREADS, 0, st>>>(ws, parity, NB);
            k_decide<true><<<G, 128, 0, st>>>(ws, NB, (long long)cpl);
            k_scatter<true><<<G, STATS_THREADS, 0, st>>>(ws, parity, NB);
            k_level_next<<<1, 32, 0, st>>>(ws, L);
        }
    }
    // enough blocks to fill every SM with resident subtree warps (the grid strides over the subtrees)
    k_subtree<true><<<sms * 16, SUB_WARPS * 32, SUB_WARPS * sizeof(SubSmem), st>>>(ws, NB, (long long)cpl);
    for (int L = DEV_MAX_LEVELS - 1; L >= 0; L--) k_count_up_dev<<<sms * 4, 256, 0, st>>>(ws, L);
    for (int L = 0; L < DEV_MAX_LEVELS; L++) k_number_down_dev<<<sms * 4, 256, 0, st>>>(ws, L);
    k_forest_counts<<<1, 256, 0, st>>>(ws, n_nodes_dev, node_off_dev, max_depth_dev, node_capacity, status_dev);
    NodesOut o{child, Lmax, Rmin, ptr, size, dim};
    k_emit_phaseA_dev<<<G, 256, 0, st>>>(ws, o, node_off_dev, status_dev);
    k_emit_subtrees_dev<<<G, 256, 0, st>>>(ws, o, node_off_dev, status_dev);
    k_emit_indices<<<g, 256, 0, st>>>(ws, ni, bb_indices, true);
    k_forest_status_final<<<1, 32, 0, st>>>(ws, status_dev);
    CT_CHECK_LAUNCH("forest build (device-driven)");
    return CT_OK;
}

int ct_build_forest_emit(const void* workspace, int64_t n_total, int32_t n_trees, int32_t NB, int32_t factor,
                         const int64_t* node_off, int64_t* child, double* Lmax, double* Rmin, int64_t* ptr,
                         int64_t* size, uint8_t* dim, int64_t* bb_indices, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (NB < 2 || NB > NBMAX || factor < 1 || n_trees < 1) return ct_fail(CT_ERR_ARG, "bad arguments");
    if (!node_off) return ct_fail(CT_ERR_ARG, "node_off is null");
    WS ws;
    carve((char*)workspace, n_total, NB, factor, &ws, n_trees, true);
    return emit_nodes(ws, n_total, 0, node_off, child, Lmax, Rmin, ptr, size, dim, bb_indices, st);
}

}  // extern "C"

// ------------------------------------------------------------------------
// Allocation-free build
//
// Some callers cannot call cudaMalloc: code running inside another runtime
// that owns all device memory (a host application with its own pool, a
// plugin that may not touch the allocator), or code on a path where an
// allocation could block or fail.  ct_build_tree_noalloc builds a tree for
// them with its scratch in the fixed device array below instead of a caller
// workspace.  The array is 8 MiB, enough for 16384 cells with any n_buckets
// <= 32; every GPU that loads the library holds it until the process exits.
// Host code only sees a stand-in for the array's name, so the device address
// is looked up once per device (with that device current) and cached; a
// device whose context was re-created (cudaDeviceReset) is looked up again.
// ------------------------------------------------------------------------

namespace ct {

constexpr int64_t NOALLOC_MAX_CELLS = 16384;
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(8) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mutex;

// One cached address per device, valid for the context it was looked up in.
// A symbol's device address belongs to a CUDA context: after cudaDeviceReset
// (or after the primary context is released and created again) the module is
// loaded anew, so the cache is keyed by the context's unique id as well.
struct NoallocSlot {
    unsigned long long ctx_id;
    void* ptr;
};
static NoallocSlot g_noalloc_slot[256] = {};

typedef int (*pfn_ctx_get_current)(void**);
typedef int (*pfn_ctx_get_id)(void*, unsigned long long*);

// Unique id of the context current on this thread (0 when none is current).
static int current_context_id(unsigned long long* id) {
    static pfn_ctx_get_current get_current = nullptr;
    static pfn_ctx_get_id get_id = nullptr;
    if (!get_current || !get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return ct_fail(CT_ERR_CUDA, "driver entry points cuCtxGetCurrent / cuCtxGetId unavailable");
        get_current = (pfn_ctx_get_current)f1;
        get_id = (pfn_ctx_get_id)f2;
    }
    void* ctx = nullptr;
    if (get_current(&ctx) != 0) return ct_fail(CT_ERR_CUDA, "cuCtxGetCurrent failed");
    *id = 0;
    if (ctx && get_id(ctx, id) != 0) return ct_fail(CT_ERR_CUDA, "cuCtxGetId failed");
    return CT_OK;
}

// Device address of g_noalloc_scratch on the current device: looked up once
// per device and context (with that device current), then reused.
static int noalloc_scratch(void** out) {
    int dev = 0;
    CT_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return ct_fail(CT_ERR_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    unsigned long long id = 0;
    int s = current_context_id(&id);
    if (s != CT_OK) return s;
    NoallocSlot& slot = g_noalloc_slot[dev];
    if (id == 0 || slot.ptr == nullptr || slot.ctx_id != id) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return ct_fail(CT_ERR_CUDA, cudaGetErrorString(e));
        // the lookup makes the runtime's context current if none was
        if (id == 0) {
            s = current_context_id(&id);
            if (s != CT_OK) return s;
        }
        slot.ctx_id = id;
        slot.ptr = p;
    }
    *out = slot.ptr;
    return CT_OK;
}

}  // namespace ct

extern "C" int ct_build_tree_noalloc(const double* bb, int64_t n, int32_t NB, int64_t cpl, int64_t* child,
                                     double* Lmax, double* Rmin, int64_t* ptr, int64_t* size, uint8_t* dim,
                                     int64_t node_capacity, int64_t* bb_indices, int64_t* n_nodes_host,
                                     int32_t* max_depth_host, void* stream) {
    if (n < 0 || n > NOALLOC_MAX_CELLS)
        return ct_fail(CT_ERR_ARG, "ct_build_tree_noalloc: n_elements must be in [0, 16384] (8 MiB static scratch)");
    if (NB < 2 || NB > NBMAX) return ct_fail(CT_ERR_ARG, "n_buckets must be in [2, 32] for the GPU builder");
    size_t need = carve(nullptr, n, NB, 1, nullptr);
    if (need > NOALLOC_SCRATCH_BYTES) return ct_fail(CT_ERR_ARG, "ct_build_tree_noalloc: static scratch too small");
    void* scratch = nullptr;
    int s = noalloc_scratch(&scratch);
    if (s != CT_OK) return s;
    // The array keeps the previous call's contents: start from zeroed counters.
    WS ws;
    carve((char*)scratch, n, NB, 1, &ws);
    CT_CUDA(cudaMemsetAsync(ws.cnt, 0, sizeof(Counters), (cudaStream_t)stream));
    int64_t nn = 0;
    int32_t md = 0;
    s = ct_build_tree(bb, n, NB, cpl, 1, scratch, NOALLOC_SCRATCH_BYTES, &nn, &md, stream);
    if (s != CT_OK) return s;
    if (nn > node_capacity)
        return ct_fail(CT_ERR_ARG, "node_capacity too small: pass ct_pessimistic_n_nodes(n_elements)");
    s = ct_build_emit(scratch, n, NB, 1, child, Lmax, Rmin, ptr, size, dim, bb_indices, stream);
    if (s != CT_OK) return s;
    if (n_nodes_host) *n_nodes_host = nn;
    if (max_depth_host) *max_depth_host = md;
    return CT_OK;
}
