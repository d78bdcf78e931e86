/*
 * celltree_oracle.c -- CPU restatement of the numba_celltree algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the test-suite,
 * `__graft_entry__.smoke()` and the `cpu_baseline` / reference arm of
 * `bench.py` call it as the checker and as the timed host-core baseline.  The
 * product path (numba_celltree_gb300) never links or calls it.
 *
 * Every routine restates one function of the upstream package and cites it as
 * `file:line` relative to the upstream project root (numba_celltree 0.4.2).
 * The arithmetic is written in the upstream evaluation order; the file must be
 * compiled with -ffp-contract=off so that no a*b+c is fused (numba does not
 * fuse either), which keeps every float64 result bit-identical.
 *
 * Parity is pinned against the upstream package itself, run in its own
 * pure-Python mode (see tests/golden/make_golden.py) and against the golden
 * values of the upstream test-suite.
 *
 * Index type: int64 (numpy intp on 64-bit hosts, constants.py:27).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define FILL_VALUE (-1)                 /* constants.py:135 */
#define MIN_TOLERANCE 1e-15             /* constants.py:146 */
#define TOLERANCE_FACTOR 1e-12          /* constants.py:147 */
#define MAX_N_VERTEX 32                 /* constants.py:134 */
#define CLIP_MAX_N_VERTEX (2 * MAX_N_VERTEX) /* utils.py:101 */

typedef struct { double x, y; } pt;
typedef struct { double xmin, xmax, ymin, ymax; } box4;

/* ----------------------------------------------------------------------- */
/* Python scalar semantics                                                  */
/* ----------------------------------------------------------------------- */

/* builtin min(a, b): returns a unless b < a (keeps the first on ties). */
static inline double pmin(double a, double b) { return (b < a) ? b : a; }
/* builtin max(a, b): returns a unless b > a. */
static inline double pmax(double a, double b) { return (b > a) ? b : a; }

static inline pt P(double x, double y) { pt r; r.x = x; r.y = y; return r; }
static inline pt vsub(pt b, pt a) { return P(b.x - a.x, b.y - a.y); }  /* to_vector(a, b) geometry_utils.py:23-25 */
static inline double cross(pt u, pt v) { return u.x * v.y - u.y * v.x; } /* geometry_utils.py:57-59 */
static inline double dot(pt u, pt v) { return u.x * v.x + u.y * v.y; }   /* geometry_utils.py:62-64 */
static inline double len2(pt v) { return v.x * v.x + v.y * v.y; }        /* geometry_utils.py:67-69 */

/* ----------------------------------------------------------------------- */
/* geometry_utils.py                                                        */
/* ----------------------------------------------------------------------- */

/* polygon_length geometry_utils.py:72-79 */
static inline int64_t polygon_length(const int64_t* face, int64_t n) {
    for (int64_t i = 3; i < n; i++)
        if (face[i] == FILL_VALUE) return i;
    return n;
}

/* copy_vertices_into geometry_utils.py:501-510 */
static inline int64_t gather_polygon(const double* vertices, const int64_t* face, int64_t n, pt* out) {
    int64_t len = polygon_length(face, n);
    for (int64_t i = 0; i < len; i++) out[i] = P(vertices[2 * face[i]], vertices[2 * face[i] + 1]);
    return len;
}

/* polygon_area geometry_utils.py:82-95 */
static double polygon_area(const pt* poly, int64_t len) {
    double area = 0.0;
    pt a = poly[0], b = poly[1];
    pt U = vsub(b, a);
    for (int64_t i = 2; i < len; i++) {
        pt c = poly[i];
        pt V = vsub(a, c);
        area += fabs(cross(U, V));
        b = c;
        U = V;
    }
    (void)b;
    return 0.5 * area;
}

/* within_perpendicular_distance geometry_utils.py:150-166 */
static inline int within_perp(double UxV, pt U, double tol) {
    return (UxV * UxV) < ((tol * len2(U)) * tol);
}

/* in_bounds geometry_utils.py:169-192 */
static inline int in_bounds(pt p, pt a, pt b) {
    double xmin = pmin(a.x, b.x), xmax = pmax(a.x, b.x);
    double ymin = pmin(a.y, b.y), ymax = pmax(a.y, b.y);
    double dx = xmax - xmin, dy = ymax - ymin;
    int use_x = fabs(dx) >= fabs(dy);
    return (use_x && (p.x >= xmin && p.x <= xmax)) || (!use_x && (p.y >= ymin && p.y <= ymax));
}

/* point_in_polygon geometry_utils.py:98-147 */
static int point_in_polygon(pt p, const pt* poly, int64_t len) {
    pt v0 = poly[len - 1];
    int c = 0;
    for (int64_t i = 0; i < len; i++) {
        pt v1 = poly[i];
        if (((v0.y > p.y) != (v1.y > p.y)) &&
            p.x < ((v1.x - v0.x) * (p.y - v0.y) / (v1.y - v0.y) + v0.x))
            c = !c;
        v0 = v1;
    }
    return c;
}

/* point_in_polygon_or_on_edge geometry_utils.py:195-223 */
static int point_in_polygon_or_on_edge(pt p, const pt* poly, int64_t len, double tol) {
    pt v0 = poly[len - 1];
    pt U = vsub(v0, p);
    int c = 0;
    for (int64_t i = 0; i < len; i++) {
        pt v1 = poly[i];
        if (v1.x == v0.x && v1.y == v0.y) continue;
        pt V = vsub(v1, p);
        double A = cross(U, V);
        pt W = vsub(v1, v0);
        if (within_perp(A, W, tol) && in_bounds(p, v0, v1)) return 1;
        if (((v0.y > p.y) != (v1.y > p.y)) &&
            p.x < ((v1.x - v0.x) * (p.y - v0.y) / (v1.y - v0.y) + v0.x))
            c = !c;
        v0 = v1;
        U = V;
    }
    return c;
}

/* point_on_edge geometry_utils.py:226-238 */
static int point_on_edge(pt p, pt v0, pt v1, double tol) {
    if (v1.x == v0.x && v1.y == v0.y) return 0;
    pt U = vsub(v0, p), V = vsub(v1, p), W = vsub(v1, v0);
    double A = cross(U, V);
    return within_perp(A, W, tol) && in_bounds(p, v0, v1);
}

/* point_in_triangle geometry_utils.py:241-270 */
static int point_in_triangle(pt p, pt a, pt b, pt c, double tol) {
    pt ap = vsub(p, a), bp = vsub(p, b), cp = vsub(p, c);
    pt ab = vsub(b, a), bc = vsub(c, b), ca = vsub(a, c);
    double A = cross(ab, ap), B = cross(bc, bp), C = cross(ca, cp);
    int sA = A > 0, sB = B > 0, sC = C > 0;
    if ((sA == sB) && (sB == sC)) return 1;
    if ((within_perp(A, ab, tol) && in_bounds(p, a, b)) || (within_perp(B, bc, tol) && in_bounds(p, b, c)) ||
        (within_perp(C, ca, tol) && in_bounds(p, c, a)))
        return 1;
    return 0;
}

/* boxes_intersect geometry_utils.py:292-300 */
static inline int boxes_intersect(box4 a, box4 b) {
    return a.xmin < b.xmax && b.xmin < a.xmax && a.ymin < b.ymax && b.ymin < a.ymax;
}

/* box_contained geometry_utils.py:303-315 */
static inline int box_contained(box4 a, box4 b) {
    return a.xmin >= b.xmin && a.xmax <= b.xmax && a.ymin >= b.ymin && a.ymax <= b.ymax;
}

static inline box4 as_box(const double* a) { box4 b; b.xmin = a[0]; b.xmax = a[1]; b.ymin = a[2]; b.ymax = a[3]; return b; }

/* left_of geometry_utils.py:318-322 */
static inline int left_of(pt a, pt p, pt U) { return U.x * (a.y - p.y) > U.y * (a.x - p.x); }

/* has_overlap geometry_utils.py:325-329 */
static inline int has_overlap(double a, double b, double p, double q, double tol) {
    return ((pmin(a, b) - pmax(p, q)) < tol) && ((pmin(p, q) - pmax(a, b)) < tol);
}

/* lines_intersect geometry_utils.py:332-418 (with intersection_location_point
 * 332-345 and midpoint_collinear_lines 348-374). */
static int lines_intersect(pt a, pt b, pt p, pt q, double* x, double* y) {
    pt V = vsub(b, a), U = vsub(q, p);
    *x = NAN; *y = NAN;
    if ((U.x == 0 && U.y == 0) || (V.x == 0 && V.y == 0)) return 0;
    if ((U.x == 0) && (V.x == 0) && a.x != p.x) return 0;
    if ((U.y == 0) && (V.y == 0) && a.y != p.y) return 0;
    double tol = pmax(MIN_TOLERANCE, TOLERANCE_FACTOR * pmax(fabs(U.x), fabs(U.y)));
    if (!has_overlap(a.x, b.x, p.x, q.x, tol) || !has_overlap(a.y, b.y, p.y, q.y, tol)) return 0;
    if ((left_of(a, p, U) != left_of(b, p, U)) && (left_of(p, a, V) != left_of(q, a, V))) {
        double denom = cross(V, U);
        if (within_perp(denom, V, tol)) return 1; /* parallel: NaN point */
        pt R = vsub(p, a);
        double t = cross(R, U) / denom;
        *x = a.x + t * V.x;
        *y = a.y + t * V.y;
        return 1;
    }
    pt R = vsub(p, a), S = vsub(q, a);
    if (within_perp(cross(V, R), V, tol) && within_perp(cross(V, S), V, tol)) {
        pt aa = a, bb = b, pp = p, qq = q, t;
        if (aa.x > bb.x || (aa.x == bb.x && aa.y > bb.y)) { t = aa; aa = bb; bb = t; }
        if (pp.x > qq.x || (pp.x == qq.x && pp.y > qq.y)) { t = pp; pp = qq; qq = t; }
        double sx = pmax(aa.x, pp.x), sy = pmax(aa.y, pp.y);
        double ex = pmin(bb.x, qq.x), ey = pmin(bb.y, qq.y);
        if (sx > ex || sy > ey) return 1; /* no overlap: NaN point */
        *x = 0.5 * (sx + ex);
        *y = 0.5 * (sy + ey);
        return 1;
    }
    return 0;
}

/* bounding_box geometry_utils.py:421-440 */
static void bounding_box(const int64_t* face, int64_t n, const double* v, double* out) {
    double xmin = v[2 * face[0]], xmax = xmin, ymin = v[2 * face[0] + 1], ymax = ymin;
    for (int64_t i = 1; i < n; i++) {
        int64_t idx = face[i];
        if (idx == FILL_VALUE) break;
        double x = v[2 * idx], y = v[2 * idx + 1];
        xmin = pmin(xmin, x); xmax = pmax(xmax, x);
        ymin = pmin(ymin, y); ymax = pmax(ymax, y);
    }
    out[0] = xmin; out[1] = xmax; out[2] = ymin; out[3] = ymax;
}

/* build_face_bboxes geometry_utils.py:443-456 */
void cto_build_face_bboxes(const int64_t* faces, int64_t n_faces, int64_t n_max_vert, const double* vertices,
                           double* bb_coords) {
    for (int64_t i = 0; i < n_faces; i++) bounding_box(faces + i * n_max_vert, n_max_vert, vertices, bb_coords + 4 * i);
}

/* edge_bounding_box / build_edge_bboxes geometry_utils.py:459-487 */
void cto_build_edge_bboxes(const int64_t* edges, int64_t n_edges, const double* v, double tol, double* bb) {
    for (int64_t i = 0; i < n_edges; i++) {
        double x0 = v[2 * edges[2 * i]], y0 = v[2 * edges[2 * i] + 1];
        double x1 = v[2 * edges[2 * i + 1]], y1 = v[2 * edges[2 * i + 1] + 1];
        bb[4 * i + 0] = pmin(x0 - tol, x1 - tol);
        bb[4 * i + 1] = pmax(x0 + tol, x1 + tol);
        bb[4 * i + 2] = pmin(y0 - tol, y1 - tol);
        bb[4 * i + 3] = pmax(y0 + tol, y1 + tol);
    }
}

/* flip / counter_clockwise geometry_utils.py:532-561 (in place) */
void cto_counter_clockwise(const double* v, int64_t* faces, int64_t n_faces, int64_t n_max_vert) {
    for (int64_t f = 0; f < n_faces; f++) {
        int64_t* face = faces + f * n_max_vert;
        int64_t len = polygon_length(face, n_max_vert);
        pt a = P(v[2 * face[len - 2]], v[2 * face[len - 2] + 1]);
        pt b = P(v[2 * face[len - 1]], v[2 * face[len - 1] + 1]);
        for (int64_t i = 0; i < len; i++) {
            pt c = P(v[2 * face[i]], v[2 * face[i] + 1]);
            double product = cross(vsub(b, a), vsub(c, a));
            if (product == 0) {
                a = b;
                b = c;
            } else if (product < 0) {
                int64_t end = len - 1;
                for (int64_t k = 0; k < len / 2; k++) {
                    int64_t j = end - k, t = face[k];
                    face[k] = face[j];
                    face[j] = t;
                }
            } else {
                break;
            }
        }
    }
}

/* point_in_triangle over a point list: points_in_triangles geometry_utils.py:273-289 */
void cto_points_in_triangles(const double* points, const int64_t* face_indices, const int64_t* faces,
                             int64_t n_max_vert, const double* v, int64_t n, double tol, uint8_t* out) {
    for (int64_t i = 0; i < n; i++) {
        const int64_t* f = faces + face_indices[i] * n_max_vert;
        pt a = P(v[2 * f[0]], v[2 * f[0] + 1]), b = P(v[2 * f[1]], v[2 * f[1] + 1]), c = P(v[2 * f[2]], v[2 * f[2] + 1]);
        out[i] = (uint8_t)point_in_triangle(P(points[2 * i], points[2 * i + 1]), a, b, c, tol);
    }
}

/* ----------------------------------------------------------------------- */
/* creation.py                                                              */
/* ----------------------------------------------------------------------- */

typedef struct { double Max, Min, Rmin, Lmax; int64_t index, size; } bucket_t; /* constants.py:109-122 */

/* pessimistic_n_nodes creation.py:216-230 */
int64_t cto_pessimistic_n_nodes(int64_t n) {
    int64_t n_nodes = n;
    int64_t nodes = (int64_t)ceil((double)n / 2.0);
    while (nodes > 1) {
        n_nodes += nodes;
        nodes = (int64_t)ceil((double)nodes / 2.0);
    }
    return n_nodes + 1;
}

/* get_bounds creation.py:153-171 */
static void get_bounds(int64_t index, int64_t size, const double* bb, const int64_t* bbi, int dim, double* Rmin_o,
                       double* Lmax_o) {
    double Rmin = DBL_MAX, Lmax = -DBL_MAX;
    for (int64_t i = index; i < index + size; i++) {
        int64_t d = bbi[i];
        double value = bb[4 * d + 2 * dim];
        if (value < Rmin) Rmin = value;
        value = bb[4 * d + 2 * dim + 1];
        if (value > Lmax) Lmax = value;
    }
    *Rmin_o = Rmin;
    *Lmax_o = Lmax;
}

/* centroid_test creation.py:44-51 */
static inline int centroid_test(const bucket_t* b, const double* box, int dim) {
    double c = box[2 * dim] + 0.5 * (box[2 * dim + 1] - box[2 * dim]);
    return (c >= b->Min) && (c < b->Max);
}

/* stable_partition creation.py:54-112 */
static int64_t stable_partition(int64_t* bbi, const double* bb, int64_t begin, int64_t end, const bucket_t* b, int dim,
                                int64_t* tmp) {
    int64_t nt = 0, nf = 0, n = end - begin;
    for (int64_t i = begin; i < end; i++) {
        int64_t idx = bbi[i];
        if (centroid_test(b, bb + 4 * idx, dim))
            bbi[begin + nt++] = idx; /* trues are compacted in place: never overtakes i */
        else
            tmp[nf++] = idx;
    }
    (void)n;
    for (int64_t i = 0; i < nf; i++) bbi[begin + nt + i] = tmp[i];
    return begin + nt;
}

/* split_plane creation.py:174-213 */
static int64_t split_plane(const bucket_t* bk, int64_t nbk, int64_t root_size, double range_Lmax, double range_Rmin,
                           double bucket_length, double* Lmax_o, double* Rmin_o) {
    double plane_min_cost = DBL_MAX;
    int64_t plane = INT64_MAX;
    int64_t bbs_in_left = 0, bbs_in_right = 0;
    for (int64_t i = 1; i < nbk; i++) {
        const bucket_t* cur = &bk[i - 1];
        const bucket_t* nxt = &bk[i];
        bbs_in_left += cur->size;
        bbs_in_right = root_size - bbs_in_left;
        double left_volume = (cur->Lmax - range_Rmin) / bucket_length;
        double right_volume = (range_Lmax - nxt->Rmin) / bucket_length;
        double plane_cost = left_volume * (double)bbs_in_left + right_volume * (double)bbs_in_right;
        if (plane_cost < plane_min_cost) {
            plane_min_cost = plane_cost;
            plane = i;
        }
    }
    double Lmax = -DBL_MAX, Rmin = DBL_MAX;
    if (plane == INT64_MAX) return -1;
    for (int64_t i = 0; i < plane; i++)
        if (bk[i].Lmax > Lmax) Lmax = bk[i].Lmax;
    for (int64_t i = plane; i < nbk; i++)
        if (bk[i].Rmin < Rmin) Rmin = bk[i].Rmin;
    *Lmax_o = Lmax;
    *Rmin_o = Rmin;
    return plane;
}

typedef struct {
    int64_t* child;
    double* Lmax;
    double* Rmin;
    int64_t* ptr;
    int64_t* size;
    uint8_t* dim;
} nodes_out;

static inline int64_t push_node(nodes_out* nd, int64_t index, int64_t ptr, int64_t size, int dim) {
    nd->child[index] = -1;
    nd->Lmax[index] = -1.0;
    nd->Rmin[index] = -1.0;
    nd->ptr[index] = ptr;
    nd->size[index] = size;
    nd->dim[index] = (uint8_t)(dim != 0);
    return index + 1;
}

/* build creation.py:233-381 and initialize creation.py:384-413.
 * Returns the number of nodes, or -1 when a centroid falls in no bucket (the
 * upstream code indexes past its bucket list in that case). */
int64_t cto_build_tree(const double* bb, int64_t n, int64_t n_buckets, int64_t cells_per_leaf, int64_t* child,
                       double* Lmax, double* Rmin, int64_t* ptr, int64_t* size, uint8_t* dim, int64_t* bb_indices) {
    nodes_out nd = {child, Lmax, Rmin, ptr, size, dim};
    for (int64_t i = 0; i < n; i++) bb_indices[i] = i;
    int64_t node_index = push_node(&nd, 0, 0, n, 0);

    int64_t cap = 32, sz = 1;
    int64_t* stack = (int64_t*)malloc(sizeof(int64_t) * 2 * cap);
    int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    bucket_t* bk = (bucket_t*)malloc(sizeof(bucket_t) * n_buckets);
    int64_t result = 0;
    stack[0] = 0;
    stack[1] = 0;

    while (sz > 0) {
        sz--;
        int64_t root_index = stack[2 * sz];
        int64_t dimv = stack[2 * sz + 1];
        int64_t dim_flag = dimv;
        if (dimv < 0) dimv += 2;
        int d = (int)dimv;

        int64_t r_ptr = nd.ptr[root_index], r_size = nd.size[root_index];
        int r_dim = nd.dim[root_index];
        if (r_size <= cells_per_leaf) continue;

        double range_Rmin, range_Lmax;
        get_bounds(r_ptr, r_size, bb, bb_indices, d, &range_Rmin, &range_Lmax);
        double bucket_length = (range_Lmax - range_Rmin) / (double)n_buckets;

        for (int64_t i = 0; i < n_buckets; i++) {
            bk[i].Max = (double)(i + 1) * bucket_length + range_Rmin;
            bk[i].Min = (double)i * bucket_length + range_Rmin;
            bk[i].Rmin = -1.0;
            bk[i].Lmax = -1.0;
            bk[i].index = -1;
            bk[i].size = 0;
        }

        /* sort_bbox_indices creation.py:115-150 */
        {
            int64_t current = r_ptr, end = r_ptr + r_size;
            bk[0].index = r_ptr;
            int64_t i = 1;
            while (current != end) {
                if (i - 1 >= n_buckets) { result = -1; goto done; }
                bucket_t b = bk[i - 1];
                current = stable_partition(bb_indices, bb, current, end, &b, d, tmp);
                int64_t start = b.index;
                bk[i - 1].size = current - start;
                if (i < n_buckets) bk[i].index = bk[i - 1].index + bk[i - 1].size;
                i++;
            }
        }
        for (int64_t i = 0; i < n_buckets; i++) {
            double a, b;
            get_bounds(bk[i].index, bk[i].size, bb, bb_indices, d, &a, &b);
            bk[i].Rmin = a;
            bk[i].Lmax = b;
        }

        if (cells_per_leaf == 1 && r_size == 2) {
            nd.Lmax[root_index] = range_Lmax;
            nd.Rmin[root_index] = range_Rmin;
            nd.child[root_index] = node_index;
            node_index = push_node(&nd, node_index, r_ptr, 1, !d);
            node_index = push_node(&nd, node_index, r_ptr + 1, 1, !d);
            continue;
        }

        int64_t nbk = n_buckets;
        bucket_t* bl = bk;
        while (bl[0].size == 0) {
            bl[1].Min = bl[0].Min;
            bl++;
            nbk--;
        }
        {
            int64_t i = 1;
            while (i < nbk) {
                if (bl[i].size == 0) {
                    bl[i - 1].Max = bl[i].Max;
                    memmove(&bl[i], &bl[i + 1], sizeof(bucket_t) * (size_t)(nbk - i - 1));
                    nbk--;
                } else {
                    i++;
                }
            }
        }

        int needs_continue = 0;
        for (int64_t i = 0; i < nbk; i++) {
            if (bl[i].size == r_size) {
                needs_continue = 1;
                if (dim_flag >= 0) {
                    dim_flag = (int64_t)(!d) - 2;
                    nd.dim[root_index] = (uint8_t)(!r_dim);
                    if (sz >= cap) {
                        cap *= 2;
                        stack = (int64_t*)realloc(stack, sizeof(int64_t) * 2 * cap);
                    }
                    stack[2 * sz] = root_index;
                    stack[2 * sz + 1] = dim_flag;
                    sz++;
                } else {
                    nd.Lmax[root_index] = -1;
                    nd.Rmin[root_index] = -1;
                }
                break;
            }
        }
        if (needs_continue) continue;

        double sLmax, sRmin;
        int64_t plane = split_plane(bl, nbk, r_size, range_Lmax, range_Rmin, bucket_length, &sLmax, &sRmin);
        if (plane < 0) { result = -1; goto done; }
        int64_t right_index = bl[plane].index;
        int64_t right_size = r_ptr + r_size - right_index;
        int64_t left_index = r_ptr;
        int64_t left_size = r_size - right_size;
        nd.Lmax[root_index] = sLmax;
        nd.Rmin[root_index] = sRmin;
        nd.child[root_index] = node_index;
        int64_t child_ind = node_index;
        node_index = push_node(&nd, node_index, left_index, left_size, !d);
        node_index = push_node(&nd, node_index, right_index, right_size, !d);

        if (sz + 2 > cap) {
            cap *= 2;
            stack = (int64_t*)realloc(stack, sizeof(int64_t) * 2 * cap);
        }
        stack[2 * sz] = child_ind + 1;
        stack[2 * sz + 1] = !d;
        sz++;
        stack[2 * sz] = child_ind;
        stack[2 * sz + 1] = !d;
        sz++;
    }
    result = node_index;
done:
    free(stack);
    free(tmp);
    free(bk);
    return result;
}

/* ----------------------------------------------------------------------- */
/* query.py                                                                 */
/* ----------------------------------------------------------------------- */

typedef struct {
    const int64_t* elements; /* faces or edges, n_elem x n_max_vert */
    int64_t n_max_vert;
    const double* vertices;
    const int64_t* child;
    const double* Lmax;
    const double* Rmin;
    const int64_t* ptr;
    const int64_t* size;
    const uint8_t* dim;
    int64_t n_nodes;
    const int64_t* bb_indices;
    const double* bb_coords;
    const double* bbox; /* xmin, xmax, ymin, ymax */
} cto_tree;

typedef struct {
    int64_t* data;
    int64_t n, cap;
} istack;

static inline void ipush(istack* s, int64_t v) {
    if (s->n >= s->cap) {
        s->cap *= 2;
        s->data = (int64_t*)realloc(s->data, sizeof(int64_t) * s->cap);
    }
    s->data[s->n++] = v;
}

static inline istack inew(void) {
    istack s;
    s.cap = 32; /* INITIAL_STACK_LENGTH constants.py:144 */
    s.n = 0;
    s.data = (int64_t*)malloc(sizeof(int64_t) * 32);
    return s;
}

/* locate_point query.py:63-107 */
static int64_t locate_point(pt p, const cto_tree* t, double tol, istack* st, pt* poly) {
    st->n = 0;
    ipush(st, 0);
    while (st->n > 0) {
        int64_t ni = st->data[--st->n];
        if (t->child[ni] == -1) {
            for (int64_t i = t->ptr[ni]; i < t->ptr[ni] + t->size[ni]; i++) {
                int64_t bi = t->bb_indices[i];
                int64_t len = gather_polygon(t->vertices, t->elements + bi * t->n_max_vert, t->n_max_vert, poly);
                if (point_in_polygon_or_on_edge(p, poly, len, tol)) return bi;
            }
            continue;
        }
        int d = t->dim[ni] ? 1 : 0;
        double pd = d ? p.y : p.x;
        int left = pd <= t->Lmax[ni];
        int right = pd >= t->Rmin[ni];
        int64_t lc = t->child[ni], rc = lc + 1;
        if (left && right) {
            if ((t->Lmax[ni] - pd) < (pd - t->Rmin[ni])) {
                ipush(st, lc);
                ipush(st, rc);
            } else {
                ipush(st, rc);
                ipush(st, lc);
            }
        } else if (left) {
            ipush(st, lc);
        } else if (right) {
            ipush(st, rc);
        }
    }
    return -1;
}

/* locate_points query.py:110-117 */
void cto_locate_points(const cto_tree* t, const double* points, int64_t n, double tol, int64_t* out) {
#pragma omp parallel
    {
        istack st = inew();
        pt poly[MAX_N_VERTEX];
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < n; i++) out[i] = locate_point(P(points[2 * i], points[2 * i + 1]), t, tol, &st, poly);
        free(st.data);
    }
}

/* locate_point_on_edge query.py:121-164 */
static int64_t locate_point_on_edge(pt p, const cto_tree* t, double tol, istack* st) {
    st->n = 0;
    ipush(st, 0);
    while (st->n > 0) {
        int64_t ni = st->data[--st->n];
        if (t->child[ni] == -1) {
            for (int64_t i = t->ptr[ni]; i < t->ptr[ni] + t->size[ni]; i++) {
                int64_t bi = t->bb_indices[i];
                const int64_t* e = t->elements + bi * t->n_max_vert;
                pt v0 = P(t->vertices[2 * e[0]], t->vertices[2 * e[0] + 1]);
                pt v1 = P(t->vertices[2 * e[1]], t->vertices[2 * e[1] + 1]);
                if (point_on_edge(p, v0, v1, tol)) return bi;
            }
            continue;
        }
        int d = t->dim[ni] ? 1 : 0;
        double pd = d ? p.y : p.x;
        int left = pd <= t->Lmax[ni];
        int right = pd >= t->Rmin[ni];
        int64_t lc = t->child[ni], rc = lc + 1;
        if (left && right) {
            if ((t->Lmax[ni] - pd) < (pd - t->Rmin[ni])) {
                ipush(st, lc);
                ipush(st, rc);
            } else {
                ipush(st, rc);
                ipush(st, lc);
            }
        } else if (left) {
            ipush(st, lc);
        } else if (right) {
            ipush(st, rc);
        }
    }
    return -1;
}

/* locate_points_on_edge query.py:167-174 */
void cto_locate_points_on_edge(const cto_tree* t, const double* points, int64_t n, double tol, int64_t* out) {
#pragma omp parallel
    {
        istack st = inew();
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < n; i++) out[i] = locate_point_on_edge(P(points[2 * i], points[2 * i + 1]), t, tol, &st);
        free(st.data);
    }
}

/* locate_box query.py:177-244.  Counts when jj == NULL, else writes. */
static int64_t locate_box(box4 box, const cto_tree* t, istack* st, int64_t qi, int64_t* ii, int64_t* jj) {
    if (!boxes_intersect(box, as_box(t->bbox))) return 0;
    int64_t count = 0;
    st->n = 0;
    ipush(st, 0);
    while (st->n > 0) {
        int64_t ni = st->data[--st->n];
        if (t->child[ni] == -1) {
            for (int64_t i = t->ptr[ni]; i < t->ptr[ni] + t->size[ni]; i++) {
                int64_t bi = t->bb_indices[i];
                if (boxes_intersect(box, as_box(t->bb_coords + 4 * bi))) {
                    if (jj) {
                        ii[count] = qi;
                        jj[count] = bi;
                    }
                    count++;
                }
            }
        } else {
            int d = t->dim[ni] ? 1 : 0;
            double bmin = d ? box.ymin : box.xmin, bmax = d ? box.ymax : box.xmax;
            int left = bmin <= t->Lmax[ni];
            int right = bmax >= t->Rmin[ni];
            int64_t lc = t->child[ni], rc = lc + 1;
            if (left && right) {
                ipush(st, lc);
                ipush(st, rc);
            } else if (left) {
                ipush(st, lc);
            } else if (right) {
                ipush(st, rc);
            }
        }
    }
    return count;
}

/* locate_boxes query.py:247-289: per-box counts, then an ordered write at the
 * exclusive-scan offsets (the upstream chunked concatenation yields the same
 * box-major, traversal-ordered sequence). */
void cto_count_boxes(const cto_tree* t, const double* boxes, int64_t n, int64_t* counts) {
#pragma omp parallel
    {
        istack st = inew();
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; i++) counts[i] = locate_box(as_box(boxes + 4 * i), t, &st, i, NULL, NULL);
        free(st.data);
    }
}

void cto_write_boxes(const cto_tree* t, const double* boxes, int64_t n, const int64_t* offsets, int64_t* ii,
                     int64_t* jj) {
#pragma omp parallel
    {
        istack st = inew();
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; i++) locate_box(as_box(boxes + 4 * i), t, &st, i, ii + offsets[i], jj + offsets[i]);
        free(st.data);
    }
}

/* ----------------------------------------------------------------------- */
/* algorithms/cohen_sutherland.py                                           */
/* ----------------------------------------------------------------------- */

enum { CS_INSIDE = 0, CS_LEFT = 1, CS_RIGHT = 2, CS_LOWER = 4, CS_UPPER = 8 };

/* get_clip cohen_sutherland.py:18-33 */
static inline int get_clip(pt a, box4 b) {
    int p = CS_INSIDE;
    if (a.x < b.xmin) p |= CS_LEFT;
    else if (a.x > b.xmax) p |= CS_RIGHT;
    if (a.y < b.ymin) p |= CS_LOWER;
    else if (a.y > b.ymax) p |= CS_UPPER;
    return p;
}

/* cohen_sutherland_line_box_clip cohen_sutherland.py:36-101 */
int cto_cohen_sutherland(pt a, pt b, box4 box, pt* c, pt* d) {
    *c = P(NAN, NAN);
    *d = P(NAN, NAN);
    double dx = b.x - a.x, dy = b.y - a.y;
    if (dx == 0.0 && dy == 0.0) return 0;
    int k1 = get_clip(a, box), k2 = get_clip(b, box);
    int iter = 0;
    while ((k1 | k2) != CS_INSIDE) {
        if ((k1 & k2) != 0) return 0;
        if (++iter > 64) return -1; /* bounded; upstream loops until done */
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
            a = P(x, y);
            k1 = get_clip(a, box);
        } else if (opt == k2) {
            b = P(x, y);
            k2 = get_clip(b, box);
        }
        dx = b.x - a.x;
        dy = b.y - a.y;
        if (dx == 0.0 && dy == 0.0) return 0;
    }
    *c = a;
    *d = b;
    return 1;
}

/* ----------------------------------------------------------------------- */
/* algorithms/liang_barsky.py                                               */
/* ----------------------------------------------------------------------- */

/* liang_barsky_line_box_clip liang_barsky.py:10-64 (point_inside_box
 * geometry_utils.py:527-529) */
int cto_liang_barsky(pt a, pt b, box4 box, pt* c, pt* d) {
    *c = P(NAN, NAN);
    *d = P(NAN, NAN);
    double dx = b.x - a.x, dy = b.y - a.y;
    if (dx == 0.0 && dy == 0.0) return 0;
    int ain = box.xmin < a.x && a.x < box.xmax && box.ymin < a.y && a.y < box.ymax;
    int bin = box.xmin < b.x && b.x < box.xmax && box.ymin < b.y && b.y < box.ymax;
    if (ain && bin) {
        *c = a;
        *d = b;
        return 1;
    }
    double t0 = 0.0, t1 = 1.0;
    double Pv[4] = {-dx, dx, -dy, dy};
    double Qv[4] = {a.x - box.xmin, box.xmax - a.x, a.y - box.ymin, box.ymax - a.y};
    for (int k = 0; k < 4; k++) {
        double p_i = Pv[k], q_i = Qv[k];
        if (p_i == 0) {
            if (q_i < 0) return 0;
        } else {
            double t = q_i / p_i;
            if (p_i < 0) {
                if (t > t1) return 0;
                else if (t > t0) t0 = t;
            } else if (p_i > 0) {
                if (t < t0) return 0;
                else if (t < t1) t1 = t;
            }
        }
    }
    if (t0 == t1) return 0;
    *c = P(a.x + t0 * dx, a.y + t0 * dy);
    *d = P(a.x + t1 * dx, a.y + t1 * dy);
    return 1;
}

/* ----------------------------------------------------------------------- */
/* algorithms/cyrus_beck.py                                                 */
/* ----------------------------------------------------------------------- */

/* compute_intersection cyrus_beck.py:26-43 */
static inline double cb_intersect(pt a, pt s, pt v0, pt v1, int* entering) {
    pt si = vsub(v0, a);
    pt n = P(-(v1.y - v0.y), (v1.x - v0.x));
    double n_si = dot(n, si);
    double k = dot(n, s);
    double t = n_si / k;
    *entering = n_si > 0;
    return t;
}

/* aligned cyrus_beck.py:76-91 */
static inline int aligned(pt U, pt V) {
    if ((U.x == 0 && U.y == 0) || (V.x == 0 && V.y == 0)) return 1;
    if (U.x != 0 && V.x != 0) return (U.x > 0) == (V.x > 0);
    if (U.y != 0 && V.y != 0) return (U.y > 0) == (V.y > 0);
    return 0;
}

/* collinear_case cyrus_beck.py:94-130 (overlap 66-73) */
static int cb_collinear(pt a, pt b, pt v0, pt v1, pt* c, pt* d) {
    pt _b = P(b.x - a.x, b.y - a.y);
    pt _v0 = P(v0.x - a.x, v0.y - a.y);
    pt _v1 = P(v1.x - a.x, v1.y - a.y);
    pt U = _b;
    pt V = vsub(_v1, _v0);
    if (!aligned(U, V)) {
        pt t = v0; v0 = v1; v1 = t;
        t = _v0; _v0 = _v1; _v1 = t;
    }
    pt n = P(-_b.y, _b.x);
    double ta = 0.0, tb = cross(n, _b), t0 = cross(n, _v0), t1 = cross(n, _v1);
    {
        double xa = ta, xb = tb, x0 = t0, x1 = t1, tmp;
        if (xa > xb) { tmp = xa; xa = xb; xb = tmp; }
        if (x0 > x1) { tmp = x0; x0 = x1; x1 = tmp; }
        double ov = pmin(xb, x1) - pmax(xa, x0);
        if (!(ov > 0.0)) return 0; /* max(0, ov) > 0  <=>  ov > 0 */
    }
    *c = (t0 < ta) ? v0 : a;
    *d = (t1 > tb) ? v1 : b;
    return 1;
}

/* cyrus_beck_line_polygon_clip cyrus_beck.py:133-241 */
int cto_cyrus_beck(pt a, pt b, const pt* poly, int64_t length, double tol, pt* c, pt* d) {
    *c = P(NAN, NAN);
    *d = P(NAN, NAN);
    pt s = vsub(b, a);
    if (s.x == 0 && s.y == 0) return 0;
    int a_inside = point_in_polygon_or_on_edge(a, poly, length, tol);
    int b_inside = point_in_polygon_or_on_edge(b, poly, length, tol);
    if (a_inside && b_inside) {
        *c = a;
        *d = b;
        return 1;
    }
    int64_t i0 = -1, i1 = -1, i = 0, k = 0;
    double ksi = cross(vsub(poly[0], a), s);
    while (i < length && k < 2) {
        pt v0 = poly[i], v1 = poly[(i + 1) % length];
        double eta = cross(vsub(v1, a), s);
        if ((ksi < 0.0) ^ (eta < 0.0)) {
            if (k == 0) i0 = i;
            else i1 = i;
            k++;
        } else if (ksi == 0.0 && eta == 0.0) {
            int r = cb_collinear(a, b, v0, v1, c, d);
            if (!r) { *c = P(NAN, NAN); *d = P(NAN, NAN); }
            return r;
        }
        ksi = eta;
        i++;
    }
    if (k == 0) return 0;
    /* intersections cyrus_beck.py:46-63; Python index -1 wraps to the end */
    int64_t j0 = (i0 < 0) ? i0 + length : i0, j1 = (i1 < 0) ? i1 + length : i1;
    pt v0 = poly[j0], v01 = poly[(i0 + 1) % length];
    pt v1 = poly[j1], v11 = poly[((i1 + 1) % length + length) % length];
    int e0, e1;
    double t0 = cb_intersect(a, s, v0, v01, &e0);
    double t1 = cb_intersect(a, s, v1, v11, &e1);
    if (e1) {
        double t = t0; t0 = t1; t1 = t;
    }
    if (t0 == t1) {
        if (a_inside && t1 != 0.0) t0 = 0.0;
        else if (b_inside && t0 != 1.0) t1 = 1.0;
        else return 0;
    }
    if (t1 < t0) {
        double t = t0; t0 = t1; t1 = t;
    }
    int valid0 = t0 >= 0 && t0 < 1;
    int valid1 = t1 > 0 && t1 <= 1;
    if (valid0 && valid1) {
        *c = P(a.x + t0 * s.x, a.y + t0 * s.y);
        *d = P(a.x + t1 * s.x, a.y + t1 * s.y);
        return 1;
    } else if (valid0) {
        *c = P(a.x + t0 * s.x, a.y + t0 * s.y);
        *d = b;
        return 1;
    } else if (valid1) {
        *c = a;
        *d = P(a.x + t1 * s.x, a.y + t1 * s.y);
        return 1;
    }
    return 0;
}

/* ----------------------------------------------------------------------- */
/* query.py: segment queries                                                */
/* ----------------------------------------------------------------------- */

/* compute_edge_face_intersect query.py:309-328 / compute_edge_edge_intersect
 * query.py:292-306 */
static int edge_leaf_intersect(int mode, const cto_tree* t, int64_t bi, pt a, pt b, pt* c, pt* d, pt* poly) {
    if (mode == 0) {
        const int64_t* e = t->elements + bi * t->n_max_vert;
        pt p = P(t->vertices[2 * e[0]], t->vertices[2 * e[0] + 1]);
        pt q = P(t->vertices[2 * e[1]], t->vertices[2 * e[1] + 1]);
        double x, y;
        int r = lines_intersect(a, b, p, q, &x, &y);
        *c = P(x, y);
        *d = *c;
        return r;
    }
    box4 bx = as_box(t->bb_coords + 4 * bi);
    int r = cto_cohen_sutherland(a, b, bx, c, d);
    if (r == 1) {
        int64_t len = gather_polygon(t->vertices, t->elements + bi * t->n_max_vert, t->n_max_vert, poly);
        double tol = pmax(MIN_TOLERANCE, TOLERANCE_FACTOR * pmax(bx.xmax - bx.xmin, bx.ymax - bx.ymin));
        r = cto_cyrus_beck(a, b, poly, len, tol, c, d);
    }
    return r == 1;
}

/* locate_edge query.py:357-455.  Counts when jj == NULL, else writes. */
static int64_t locate_edge(int mode, pt a, pt b, const cto_tree* t, istack* st, int64_t qi, int64_t* ii, int64_t* jj,
                           double* xy) {
    pt c, d;
    pt poly[MAX_N_VERTEX];
    if (cto_cohen_sutherland(a, b, as_box(t->bbox), &c, &d) != 1) return 0;
    pt V = vsub(b, a);
    int64_t count = 0;
    st->n = 0;
    ipush(st, 0);
    while (st->n > 0) {
        int64_t ni = st->data[--st->n];
        if (t->child[ni] == -1) {
            for (int64_t i = t->ptr[ni]; i < t->ptr[ni] + t->size[ni]; i++) {
                int64_t bi = t->bb_indices[i];
                if (edge_leaf_intersect(mode, t, bi, a, b, &c, &d, poly)) {
                    if (jj) {
                        ii[count] = qi;
                        jj[count] = bi;
                        xy[4 * count + 0] = c.x;
                        xy[4 * count + 1] = c.y;
                        xy[4 * count + 2] = d.x;
                        xy[4 * count + 3] = d.y;
                    }
                    count++;
                }
            }
            continue;
        }
        int nd = t->dim[ni] ? 1 : 0;
        double dx = nd ? V.y : V.x;
        double an = nd ? a.y : a.x, bn = nd ? b.y : b.x;
        double dx_left, dx_right;
        if (dx > 0.0) {
            dx_left = t->Lmax[ni] - an;
            dx_right = t->Rmin[ni] - bn;
        } else {
            dx_left = t->Lmax[ni] - bn;
            dx_right = t->Rmin[ni] - an;
        }
        int left = dx_left >= 0.0;
        int right = dx_right <= 0.0;
        if (dx > 0.0) {
            if (left) left = (dx_left / dx) >= 0.0;
            if (right) right = (dx_right / dx) <= 1.0;
        } else if (dx < 0.0) {
            if (left) left = (1.0 - (dx_left / dx)) >= 0.0;
            if (right) right = (1.0 - (dx_right / dx)) <= 1.0;
        }
        int64_t lc = t->child[ni], rc = lc + 1;
        if (left && right) {
            ipush(st, lc);
            ipush(st, rc);
        } else if (left) {
            ipush(st, lc);
        } else if (right) {
            ipush(st, rc);
        }
    }
    return count;
}

/* _locate_edges query.py:500-533, count pass.  mode 0: edge-edge, 1: edge-face. */
void cto_count_edges(int mode, const cto_tree* t, const double* edges, int64_t n, int64_t* counts) {
#pragma omp parallel
    {
        istack st = inew();
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; i++)
            counts[i] = locate_edge(mode, P(edges[4 * i], edges[4 * i + 1]), P(edges[4 * i + 2], edges[4 * i + 3]), t,
                                    &st, i, NULL, NULL, NULL);
        free(st.data);
    }
}

/* _locate_edges query.py:500-533, write pass. */
void cto_write_edges(int mode, const cto_tree* t, const double* edges, int64_t n, const int64_t* offsets, int64_t* ii,
                     int64_t* jj, double* xy) {
#pragma omp parallel
    {
        istack st = inew();
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; i++)
            locate_edge(mode, P(edges[4 * i], edges[4 * i + 1]), P(edges[4 * i + 2], edges[4 * i + 3]), t, &st, i,
                        ii + offsets[i], jj + offsets[i], xy + 4 * offsets[i]);
        free(st.data);
    }
}

/* sort_intersections_by_edge geometry_utils.py:564-574: the permutation of a
 * stable lexsort by (ii, t), t = (c - a) . (b - a); NaN sorts last. */
static inline int t_less(double x, double y) {
    if (isnan(x)) return 0;
    if (isnan(y)) return 1;
    return x < y;
}

void cto_sort_intersections(const int64_t* ii, const double* xy, int64_t n, const double* edges, int64_t* order) {
    double* t = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    for (int64_t i = 0; i < n; i++) {
        const double* e = edges + 4 * ii[i];
        double abx = e[2] - e[0], aby = e[3] - e[1];
        double acx = xy[4 * i] - e[0], acy = xy[4 * i + 1] - e[1];
        t[i] = acx * abx + acy * aby; /* np.sum over axis 1: left to right */
        order[i] = i;
    }
    /* stable insertion sort within runs of equal ii (ii arrives grouped and
     * non-decreasing from the locate pass), then a stable merge by ii for the
     * general case. */
    int64_t* buf = (int64_t*)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    for (int64_t w = 1; w < n; w *= 2) {
        for (int64_t lo = 0; lo < n; lo += 2 * w) {
            int64_t mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
            int64_t p = lo, q = mid, k = lo;
            while (p < mid && q < hi) {
                int64_t A = order[p], B = order[q];
                int take_b = (ii[B] < ii[A]) || (ii[B] == ii[A] && t_less(t[B], t[A]));
                buf[k++] = take_b ? order[q++] : order[p++];
            }
            while (p < mid) buf[k++] = order[p++];
            while (q < hi) buf[k++] = order[q++];
        }
        memcpy(order, buf, sizeof(int64_t) * (size_t)n);
    }
    free(buf);
    free(t);
}

/* ----------------------------------------------------------------------- */
/* algorithms/separating_axis.py                                            */
/* ----------------------------------------------------------------------- */

/* extrema_projected / is_separating_axis / separating_axes
 * separating_axis.py:17-55 */
static int separating_axes(const pt* a, int64_t la, const pt* b, int64_t lb) {
    pt p = a[la - 1];
    for (int64_t i = 0; i < la; i++) {
        pt q = a[i];
        pt norm = P(p.y - q.y, q.x - p.x);
        p = q;
        if (norm.x == 0.0 && norm.y == 0.0) continue;
        double mina = DBL_MAX, maxa = -DBL_MAX, minb = DBL_MAX, maxb = -DBL_MAX;
        for (int64_t j = 0; j < la; j++) {
            double proj = dot(a[j], norm);
            mina = pmin(mina, proj);
            maxa = pmax(maxa, proj);
        }
        for (int64_t j = 0; j < lb; j++) {
            double proj = dot(b[j], norm);
            minb = pmin(minb, proj);
            maxb = pmax(maxb, proj);
        }
        if (!(maxa > minb && maxb > mina)) return 0;
    }
    return 1;
}

int cto_separating_axes(const double* a, int64_t la, const double* b, int64_t lb) {
    return separating_axes((const pt*)a, la, (const pt*)b, lb);
}

/* polygons_intersect separating_axis.py:58-75 */
void cto_polygons_intersect(const double* va, const double* vb, const int64_t* fa, int64_t Ka, const int64_t* fb,
                            int64_t Kb, const int64_t* ia, const int64_t* ib, int64_t n, uint8_t* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        pt a[MAX_N_VERTEX], b[MAX_N_VERTEX];
        int64_t la = gather_polygon(va, fa + ia[i] * Ka, Ka, a);
        int64_t lb = gather_polygon(vb, fb + ib[i] * Kb, Kb, b);
        out[i] = (uint8_t)(separating_axes(a, la, b, lb) && separating_axes(b, lb, a, la));
    }
}

/* ----------------------------------------------------------------------- */
/* algorithms/sutherland_hodgman.py                                         */
/* ----------------------------------------------------------------------- */

/* inside sutherland_hodgman.py:56-60 */
static inline int sh_inside(pt p, pt r, pt U) { return U.x * (p.y - r.y) > U.y * (p.x - r.x); }

/* intersection sutherland_hodgman.py:63-74 */
static inline int sh_intersection(pt a, pt V, pt r, pt N, pt* out) {
    pt W = P(r.x - a.x, r.y - a.y);
    double nw = dot(N, W), nv = dot(N, V);
    if (nv != 0) {
        double t = nw / nv;
        *out = P(a.x + t * V.x, a.y + t * V.y);
        return 1;
    }
    *out = P(NAN, NAN);
    return 0;
}

/* polygon_polygon_clip_area sutherland_hodgman.py:84-148.  Returns NaN if the
 * 64-vertex scratch polygon would overflow (upstream writes past it). */
double cto_clip_area(const pt* polygon, int64_t n_poly, const pt* clipper, int64_t n_clip) {
    pt subject[CLIP_MAX_N_VERTEX], output[CLIP_MAX_N_VERTEX];
    int64_t n_output = n_poly;
    for (int64_t i = 0; i < n_poly; i++) output[i] = polygon[i];
    pt r = clipper[n_clip - 1];
    for (int64_t i = 0; i < n_clip; i++) {
        pt s = clipper[i];
        pt U = P(s.x - r.x, s.y - r.y);
        if (U.x == 0 && U.y == 0) continue;
        pt N = P(-U.y, U.x);
        int64_t length = n_output;
        for (int64_t k = 0; k < length; k++) subject[k] = output[k];
        n_output = 0;
        pt a = subject[length - 1];
        int a_inside = sh_inside(a, r, U);
        for (int64_t j = 0; j < length; j++) {
            pt b = subject[j];
            pt V = P(b.x - a.x, b.y - a.y);
            if (V.x == 0 && V.y == 0) continue;
            int b_inside = sh_inside(b, r, U);
            pt pnt;
            if (b_inside) {
                if (!a_inside) {
                    if (sh_intersection(a, V, r, N, &pnt)) {
                        if (n_output >= CLIP_MAX_N_VERTEX) return NAN;
                        output[n_output++] = pnt;
                    }
                }
                if (n_output >= CLIP_MAX_N_VERTEX) return NAN;
                output[n_output++] = b;
            } else if (a_inside) {
                if (sh_intersection(a, V, r, N, &pnt)) {
                    if (n_output >= CLIP_MAX_N_VERTEX) return NAN;
                    output[n_output++] = pnt;
                } else {
                    b_inside = 1;
                    if (n_output >= CLIP_MAX_N_VERTEX) return NAN;
                    output[n_output++] = b;
                }
            }
            a = b;
            a_inside = b_inside;
        }
        if (n_output < 3) return 0.0;
        r = s;
    }
    return polygon_area(output, n_output);
}

double cto_polygon_polygon_clip_area(const double* polygon, int64_t n_poly, const double* clipper, int64_t n_clip) {
    return cto_clip_area((const pt*)polygon, n_poly, (const pt*)clipper, n_clip);
}

double cto_polygon_area(const double* polygon, int64_t n) { return polygon_area((const pt*)polygon, n); }

/* area_of_intersection sutherland_hodgman.py:151-168 */
void cto_area_of_intersection(const double* va, const double* vb, const int64_t* fa, int64_t Ka, const int64_t* fb,
                              int64_t Kb, const int64_t* ia, const int64_t* ib, int64_t n, double* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        pt a[MAX_N_VERTEX], b[MAX_N_VERTEX];
        int64_t la = gather_polygon(va, fa + ia[i] * Ka, Ka, a);
        int64_t lb = gather_polygon(vb, fb + ib[i] * Kb, Kb, b);
        out[i] = cto_clip_area(a, la, b, lb);
    }
}

/* box_area_of_intersection sutherland_hodgman.py:171-187 (copy_box_vertices
 * geometry_utils.py:513-524) */
void cto_box_area_of_intersection(const double* boxes, const double* v, const int64_t* faces, int64_t K,
                                  const int64_t* ibox, const int64_t* iface, int64_t n, double* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        const double* bx = boxes + 4 * ibox[i];
        pt a[4] = {P(bx[0], bx[2]), P(bx[1], bx[2]), P(bx[1], bx[3]), P(bx[0], bx[3])};
        pt b[MAX_N_VERTEX];
        int64_t lb = gather_polygon(v, faces + iface[i] * K, K, b);
        out[i] = cto_clip_area(a, 4, b, lb);
    }
}

/* ----------------------------------------------------------------------- */
/* algorithms/barycentric_*.py                                              */
/* ----------------------------------------------------------------------- */

/* compute_weights barycentric_triangle.py:28-43 */
static void tri_weights(pt a, pt b, pt c, pt p, double* w) {
    pt ab = vsub(b, a), ac = vsub(c, a), ap = vsub(p, a);
    double Aa = fabs(cross(ab, ap)), Ac = fabs(cross(ac, ap)), A = fabs(cross(ab, ac));
    double inv_denom = 1.0 / A;
    double ww = inv_denom * Aa, v = inv_denom * Ac;
    double u = 1.0 - v - ww;
    w[0] = u;
    w[1] = v;
    w[2] = ww;
}

/* barycentric_triangle_weights barycentric_triangle.py:46-64 */
void cto_barycentric_triangle(const double* points, const int64_t* fidx, const int64_t* faces, int64_t K,
                              const double* v, int64_t n, double* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double* w = out + 3 * i;
        w[0] = w[1] = w[2] = 0.0;
        if (fidx[i] == -1) continue;
        const int64_t* f = faces + fidx[i] * K;
        tri_weights(P(v[2 * f[0]], v[2 * f[0] + 1]), P(v[2 * f[1]], v[2 * f[1] + 1]), P(v[2 * f[2]], v[2 * f[2] + 1]),
                    P(points[2 * i], points[2 * i + 1]), w);
    }
}

/* interp_edge_case barycentric_wachspress.py:26-35 */
static void interp_edge(pt a, pt U, pt p, double* w, int64_t K, int64_t i, int64_t j) {
    for (int64_t k = 0; k < K; k++) w[k] = 0.0;
    pt V = vsub(p, a);
    double ww = sqrt(dot(V, V)) / sqrt(dot(U, U));
    w[i] = 1.0 - ww;
    w[j] = ww;
}

/* compute_weights barycentric_wachspress.py:38-85 */
static void wachspress_weights(const pt* poly, int64_t n, pt p, double* w, int64_t K, double tol) {
    double w_sum = 0.0;
    pt a = poly[n - 1], b = poly[0];
    pt U = vsub(b, a), V = vsub(p, a);
    double Ai = fabs(cross(U, V));
    if (within_perp(Ai, U, tol)) {
        interp_edge(a, U, p, w, K, n - 1, 0);
        return;
    }
    for (int64_t i = 0; i < n; i++) {
        int64_t i_next = (i + 1) % n;
        pt c = poly[i_next];
        pt W = vsub(c, a);
        double Ci = fabs(cross(U, W));
        U = vsub(c, b);
        V = vsub(p, b);
        double Aj = fabs(cross(U, V));
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
    for (int64_t i = 0; i < n; i++) w[i] /= w_sum;
}

void cto_wachspress_weights(const double* poly, int64_t n, double px, double py, double* w, int64_t K, double tol) {
    wachspress_weights((const pt*)poly, n, P(px, py), w, K, tol);
}

/* barycentric_wachspress_weights barycentric_wachspress.py:88-107 */
void cto_barycentric_wachspress(const double* points, const int64_t* fidx, const int64_t* faces, int64_t K,
                                const double* v, int64_t n, double tol, double* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double* w = out + K * i;
        for (int64_t k = 0; k < K; k++) w[k] = 0.0;
        if (fidx[i] == -1) continue;
        pt poly[MAX_N_VERTEX];
        int64_t len = gather_polygon(v, faces + fidx[i] * K, K, poly);
        wachspress_weights(poly, len, P(points[2 * i], points[2 * i + 1]), w, K, tol);
    }
}

/* ----------------------------------------------------------------------- */
/* query.py: node-bound diagnostics                                         */
/* ----------------------------------------------------------------------- */

/* collect_node_bounds query.py:568-622 */
void cto_collect_node_bounds(const cto_tree* t, double* nb) {
    nb[0] = t->bbox[0]; nb[1] = t->bbox[1]; nb[2] = t->bbox[2]; nb[3] = t->bbox[3];
    if (t->n_nodes < 2) return;
    int64_t cap = 64, sz = 0;
    int64_t* st = (int64_t*)malloc(sizeof(int64_t) * 3 * cap);
    st[0] = 2; st[1] = 0; st[2] = 0; /* right child */
    st[3] = 1; st[4] = 0; st[5] = 1; /* left child */
    sz = 2;
    while (sz > 0) {
        sz--;
        int64_t ni = st[3 * sz], pi = st[3 * sz + 1], side = st[3 * sz + 2];
        int d = t->dim[pi] ? 1 : 0;
        for (int k = 0; k < 4; k++) nb[4 * ni + k] = nb[4 * pi + k];
        nb[4 * ni + d * 2 + side] = side ? t->Lmax[pi] : t->Rmin[pi];
        if (t->child[ni] == -1) continue;
        int64_t lc = t->child[ni], rc = lc + 1;
        if (sz + 2 > cap) {
            cap *= 2;
            st = (int64_t*)realloc(st, sizeof(int64_t) * 3 * cap);
        }
        st[3 * sz] = rc; st[3 * sz + 1] = ni; st[3 * sz + 2] = 0; sz++;
        st[3 * sz] = lc; st[3 * sz + 1] = ni; st[3 * sz + 2] = 1; sz++;
    }
    free(st);
}

/* validate_node_bounds query.py:625-663 */
void cto_validate_node_bounds(const cto_tree* t, const double* nb, uint8_t* valid) {
    for (int64_t i = 0; i < t->n_nodes; i++) valid[i] = 0;
    istack st = inew();
    ipush(&st, 0);
    while (st.n > 0) {
        int64_t ni = st.data[--st.n];
        box4 bx = as_box(nb + 4 * ni);
        if (t->child[ni] == -1) {
            int v = 1;
            for (int64_t i = t->ptr[ni]; i < t->ptr[ni] + t->size[ni]; i++)
                v = v && box_contained(as_box(t->bb_coords + 4 * t->bb_indices[i]), bx);
            valid[ni] = (uint8_t)v;
            continue;
        }
        int64_t lc = t->child[ni], rc = lc + 1;
        valid[ni] = (uint8_t)(box_contained(as_box(nb + 4 * lc), bx) && box_contained(as_box(nb + 4 * rc), bx));
        ipush(&st, rc);
        ipush(&st, lc);
    }
    free(st.data);
}

int cto_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
