/*
 * celltree_gb300.h -- C ABI of the GB300 cell-tree library (libcelltree_gb300.so).
 *
 * Plain pointers and sizes only.  Every array argument is DEVICE memory unless
 * its comment says "host".  `stream` is a cudaStream_t passed as void*
 * (NULL = legacy default stream).  Functions return a ct_status; on error
 * ct_last_error_message() gives a readable reason (thread-local).  No function
 * allocates device memory: callers pass workspaces sized by the *_workspace_size
 * queries.
 *
 * Upstream interface that each entry point replaces is cited as file:line of
 * the numba_celltree 0.4.2 sources (relative to the upstream project root).
 * Index arrays use int64 (numpy intp, constants.py:27); coordinates float64
 * (constants.py:28).
 */
#ifndef CELLTREE_GB300_H
#define CELLTREE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CT_ABI_VERSION 3

typedef enum ct_status {
    CT_OK = 0,
    CT_ERR_CUDA = 1,      /* a CUDA call failed */
    CT_ERR_ARG = 2,       /* invalid argument (shape, size, null pointer) */
    CT_ERR_WORKSPACE = 3, /* workspace too small or builder capacity exceeded */
    CT_ERR_DEVICE = 4     /* a kernel reported an error word (see ct_device_error) */
} ct_status;

/* Device-side error bits, OR-ed into the error word of a tree descriptor. */
#define CT_DEVERR_STACK 1u    /* traversal stack overflow */
#define CT_DEVERR_BUCKET 2u   /* a centroid fell outside every bucket (upstream raises IndexError) */
#define CT_DEVERR_CLIP 4u     /* clip polygon scratch (64 vertices) overflow */
#define CT_DEVERR_CAPACITY 8u /* output capacity exceeded */
#define CT_DEVERR_LOOP 16u    /* a bounded loop gave up (Cohen-Sutherland) */
#define CT_DEVERR_NONFINITE 32u /* a coordinate of a batch index is not finite */

int ct_abi_version(void);
const char* ct_last_error_message(void);
/* Page-lock (register) host memory in place for direct DMA, and release it
 * (no upstream counterpart; the chunked host-array path registers a caller's
 * ordinary array chunk by chunk instead of copying it into a pinned staging
 * buffer).  ptr / bytes should cover whole pages; read_only registers pages
 * the process may only read.  A failure returns CT_ERR_CUDA and leaves no
 * error pending in the CUDA runtime. */
int ct_host_register(void* ptr, size_t bytes, int32_t read_only);
int ct_host_unregister(void* ptr);

/* ---------------------------------------------------------------------- */
/* Tree descriptor                                                         */
/* ---------------------------------------------------------------------- */

/* Device arrays of one built tree.  The reference-layout members mirror
 * CellTreeData (constants.py:82-89) with the packed NodeDType record
 * (constants.py:92-106) stored as separate arrays.  The packed members are
 * written by ct_pack_tree and read by the query kernels. */
typedef struct ct_tree {
    /* reference layout */
    const int64_t* elements;  /* faces (n_elements x n_max_vert) or edges (n_elements x 2) */
    const double* vertices;   /* n_vertices x 2 */
    const int64_t* bb_indices;/* n_elements */
    const double* bb_coords;  /* n_elements x 4: xmin, xmax, ymin, ymax */
    const int64_t* node_child;
    const double* node_Lmax;
    const double* node_Rmin;
    const int64_t* node_ptr;
    const int64_t* node_size;
    const uint8_t* node_dim;
    int64_t n_elements;
    int64_t n_vertices;
    int64_t n_nodes;
    int32_t n_max_vert;
    int32_t max_depth;        /* deepest node (root = 0), from ct_build_tree */
    double bbox[4];           /* host copy: xmin, xmax, ymin, ymax (bbox_tree celltree_base.py:20-25) */
    /* packed traversal arrays (filled by ct_pack_tree) */
    void* nodes_f32;          /* n_nodes x 16 B: float Lmax, float Rmin, int a, int b */
    void* nodes_f64;          /* n_nodes x 16 B: double Lmax, double Rmin */
    void* poly_f64;           /* n_elements x n_max_vert x 16 B, leaf (bb_indices) order */
    void* poly_f32;           /* n_elements x ct_poly32_stride(n_max_vert) x 16 B, leaf order, local frame */
    uint8_t* poly_len;        /* n_elements: polygon length (polygon_length geometry_utils.py:72-79) */
    uint8_t* poly_len32;      /* n_elements: length after removing repeated consecutive vertices */
    double origin[2];         /* host: origin of the float32 frame (centre of bbox) */
    float vmax;               /* host: unused (kept for layout stability) */
    float abs_eps;            /* host: float64 rounding scale of absolute coordinates */
    unsigned int* error_word; /* device: one uint32, OR-ed CT_DEVERR_* bits */
    /* start-node grid of the batched float32 locate (filled by ct_pack_grid;
     * grid_nx = 0 disables it) */
    int32_t* grid_start;      /* device: grid_ny rows of grid_nx node ids (-1: no cell) */
    int32_t grid_nx, grid_ny; /* cells along x and y */
    float grid_x0, grid_y0;   /* host: grid origin in the float32 frame */
    float grid_sx, grid_sy;   /* host: cells per unit length */
    /* per-grid-cell candidate lists of the batched float32 locate (filled by
     * ct_cand_count + ct_cand_fill; cand_tol = 0 disables them) */
    int64_t* cand_off;        /* device: grid_nx * grid_ny + 1 offsets into cand_idx */
    int32_t* cand_idx;        /* device: leaf-order cell ids of each grid cell */
    void* cand_lbox;          /* device: cand_n x float4, per entry the box where the cell's predicate
                                 can be true for a point of the grid cell */
    void* cand_box;           /* device: n_elements x float4 widened bbox (xmin, xmax, ymin, ymax),
                                 float32 frame, leaf order */
    int64_t cand_n;           /* host: entries of cand_idx */
    double cand_tol;          /* host: largest query tolerance the lists cover */
    int32_t bounds_finite;    /* host (ct_pack_tree): every node bound and bb_coords value is finite */
    /* box index of the multi-result queries (filled by ct_pack_box_index;
     * all three NULL disables it) */
    void* bb_leaf;            /* device: n_elements x 4 doubles, bb_coords in leaf (bb_indices) order */
    void* node_box;           /* device: n_nodes x 32 B: float32 bbox of the node's cells (frame of origin,
                                 rounded outward), int32 leaf ptr, int32 size, 8 B padding */
    int32_t* leaf_start;      /* device: n_elements: first leaf position of the leaf holding each position */
    /* launch shapes (host; 0 = the library default).  They change speed,
     * never results; an autotuner picks them per GPU and problem size. */
    int32_t tune_cells_bpsm;  /* candidate-list pass compiled for 4, 6 or 8 resident blocks per SM (default 6) */
    int32_t tune_fast_bpsm;   /* grid of the open-query traversal in blocks per SM, 1 .. 32 (default 16) */
    int32_t tune_query_threads; /* block size of the box and segment traversals: 64, 128 or 256
                                   (default 256 boxes, 128 segments; segments take at most 128) */
    int32_t tune_fp64_stack;  /* stack entries of the plain float64 locate: 0 = smallest that fits, 64 or 512 */
    /* parent of every node (device, n_nodes int32, -1 for the root; filled by
     * ct_pack_tree when not NULL).  Trees deeper than the traversal stacks
     * (510 levels for point location, 126 for the multi-result queries) are
     * then traversed without a stack, in the same order; without it such
     * trees are refused. */
    int32_t* node_parent;
    /* device, optional part of the box index: n_elements x float4, bb_leaf in
     * the float32 frame rounded outward (filled by ct_pack_box_index when not
     * NULL).  With it the segment traversals skip nodes and cells whose box
     * the segment's line surely misses (they produce no results). */
    void* bb_leaf32;
} ct_tree;

/* ---------------------------------------------------------------------- */
/* Geometry preparation                                                    */
/* ---------------------------------------------------------------------- */

/* ct_validate_elements, ct_bbox_summary, ct_vertex_extent and ct_pack_tree
 * share one small reduction array inside the library.  Each holds a
 * process-wide lock from clearing it to reading its result back (all four
 * synchronise their stream), so concurrent calls from several host threads
 * or streams are safe and run one after another. */

/* Input check for faces / edges (no upstream counterpart: upstream indexes
 * without checks).  *bad_host = 1 when an element's first min_len entries, or
 * any entry before its first fill value (-1), is not a vertex index in
 * [0, n_vertices).  Synchronises the stream. */
int ct_validate_elements(const int64_t* elements, int64_t n, int32_t n_max_vert, int32_t min_len, int64_t n_vertices,
                         int32_t* bad_host, void* stream);

/* counter_clockwise geometry_utils.py:541-561: flips clockwise faces in place. */
int ct_counter_clockwise(const double* vertices, int64_t* faces, int64_t n_faces, int32_t n_max_vert, void* stream);

/* build_face_bboxes geometry_utils.py:443-456. bb_coords: n_faces x 4. */
int ct_face_bboxes(const double* vertices, const int64_t* faces, int64_t n_faces, int32_t n_max_vert,
                   double* bb_coords, void* stream);

/* build_edge_bboxes geometry_utils.py:473-487 (edges: n_edges x 2). */
int ct_edge_bboxes(const double* vertices, const int64_t* edges, int64_t n_edges, double tolerance,
                   double* bb_coords, void* stream);

/* bbox_tree + bbox_distances + max diagonal (celltree_base.py:20-52).
 * out (host, 5 doubles): xmin, xmax, ymin, ymax, max bb diagonal.
 * distances (device, n x 3, may be NULL): dx, dy, dxy per box.
 * Synchronises the stream. */
int ct_bbox_summary(const double* bb_coords, int64_t n, double* distances, double* out_host5, void* stream);

/* Vertex extent for EdgeCellTree2d's tolerance (edge_celltree.py:59-62).
 * out (host, 4 doubles): xmin, xmax, ymin, ymax.  Synchronises the stream. */
int ct_vertex_extent(const double* vertices, int64_t n, double* out_host4, void* stream);

/* ---------------------------------------------------------------------- */
/* Tree construction (creation.py:27-413)                                  */
/* ---------------------------------------------------------------------- */

/* pessimistic_n_nodes creation.py:216-230 */
int64_t ct_pessimistic_n_nodes(int64_t n_elements);

/* Workspace bytes for ct_build_tree.  capacity_factor >= 1 scales the
 * builder's node-record capacity for very unbalanced trees (retry with a larger
 * factor when ct_build_tree returns CT_ERR_WORKSPACE). */
size_t ct_build_workspace_size(int64_t n_elements, int32_t n_buckets, int32_t capacity_factor);

/* initialize / build creation.py:233-413 on the GPU.  Builds the tree inside
 * the workspace and returns the node count and maximum depth (host outputs).
 * The nodes are then written by ct_build_emit, which must be called with the
 * same workspace before it is reused. Synchronises the stream. */
int ct_build_tree(const double* bb_coords, int64_t n_elements, int32_t n_buckets, int64_t cells_per_leaf,
                  int32_t capacity_factor, void* workspace, size_t workspace_bytes, int64_t* n_nodes_host,
                  int32_t* max_depth_host, void* stream);

/* Writes the nodes (reference numbering, NodeDType fields as arrays of
 * n_nodes) and bb_indices (n_elements) built by the last ct_build_tree. */
int ct_build_emit(const void* workspace, int64_t n_elements, int32_t n_buckets, int32_t capacity_factor,
                  int64_t* child, double* Lmax, double* Rmin, int64_t* ptr, int64_t* size, uint8_t* dim,
                  int64_t* bb_indices, void* stream);

/* Allocation-free variant of ct_build_tree + ct_build_emit, for callers that
 * cannot allocate device memory (code inside a runtime that owns the device
 * memory, plugins that may not call cudaMalloc).  No counterpart in the
 * upstream package.  Its scratch is a fixed 8 MiB device array inside the
 * library, so n_elements must be <= 16384 (larger inputs return CT_ERR_ARG);
 * every GPU that loads the library holds the array until the process exits.
 * The outputs are the caller's: node arrays of node_capacity >=
 * ct_pessimistic_n_nodes(n_elements) entries and bb_indices of n_elements.
 * The first call on each device looks up the array's device address (and so
 * does the first call after that device's context is re-created, e.g. by
 * cudaDeviceReset).  All calls share the one array: calls that overlap on
 * the GPU (other streams, other host threads) race.
 * Extremely unbalanced trees that exceed the builder's record capacity return
 * CT_ERR_WORKSPACE; use ct_build_tree with a larger capacity_factor.
 * Not capturable in a CUDA graph: it synchronises the stream once per tree
 * level (ct_build_forest_async is the capturable build). */
int ct_build_tree_noalloc(const double* bb_coords, int64_t n_elements, int32_t n_buckets, int64_t cells_per_leaf,
                          int64_t* child, double* Lmax, double* Rmin, int64_t* ptr, int64_t* size, uint8_t* dim,
                          int64_t node_capacity, int64_t* bb_indices, int64_t* n_nodes_host, int32_t* max_depth_host,
                          void* stream);

/* float4 units of one cell in ct_tree.poly_f32: the cell's first vertex as
 * float hi/lo pairs, then the other vertices relative to it (float2). */
int ct_poly32_stride(int32_t n_max_vert);
/* sizeof(ct_tree) (which = 0) or sizeof(ct_forest_plan) (which = 1), else 0:
 * lets a binding check its mirror of the structures against the library. */
size_t ct_abi_sizeof(int32_t which);

/* Fills the packed traversal arrays of `tree` (nodes_f32, nodes_f64,
 * poly_f64, poly_f32, poly_len, poly_len32) and its origin / vmax / abs_eps.
 * `tree` is updated in place (host struct).  Synchronises the stream. */
int ct_pack_tree(ct_tree* tree, void* stream);

/* ---------------------------------------------------------------------- */
/* Point queries                                                           */
/* ---------------------------------------------------------------------- */

#define CT_MODE_FP64 0 /* float64 traversal and leaf tests (plain form) */
#define CT_MODE_FP32 1 /* float32 traversal + float32 leaf filter, exact float64 fallback */

/* Start-node grid (no upstream counterpart; an index over the tree that
 * shortens the batched float32 locate).  For each cell of a grid_nx x grid_ny
 * grid over the tree bbox it stores the first node of the root path of
 * locate_point (query.py:63-107) at which the points of that cell (plus a
 * rounding margin) stop taking one and the same single child -- a leaf, a
 * node with a bound inside the cell, or a node whose two children are both
 * taken -- or -1 when the path ends without a child.  Every traversal of the
 * reference from the root reaches that node with an empty stack, so starting
 * there gives the same result.  ct_grid_shape: grid_nx, grid_ny for
 * n_elements cells in a width x height bbox -- nearly square grid cells,
 * about cells_per_element grid cells per mesh cell, at least 16 per axis,
 * at most 2^26 in all.  ct_pack_grid needs the packed tree (ct_pack_tree) and
 * tree->grid_start / grid_nx / grid_ny set by the caller; it sets
 * grid_nx = grid_ny = 0 for a degenerate bbox. */
int ct_grid_shape(int64_t n_elements, double width, double height, double cells_per_element, int32_t* grid_nx,
                  int32_t* grid_ny);
int ct_pack_grid(ct_tree* tree, void* stream);

/* Candidate lists (no upstream counterpart; an index that lets most batched
 * float32 queries skip the traversal).  The region where
 * point_in_polygon_or_on_edge (geometry_utils.py:195-223) can be true for a
 * cell lies within M = 2 * cover_tol plus the float64 rounding of the
 * coordinates of the cell.  For grid cell g (widened by the cell-assignment
 * margin m) the list holds every cell that meets g widened by m + M, each
 * with the box of that part of the cell widened by M (and by the rounding of
 * the float32 clipping that computes it; cells of more than 4 vertices keep
 * their widened bbox): every cell whose predicate can be true for a point of
 * g, and a box that holds every such point.  A query tests the boxes of its
 * list and the float32 leaf filter of the cells whose box holds it; one sure
 * hit and sure misses elsewhere is locate_point's answer (a sure hit is an
 * interior point, inside the cell's bbox, so the reference reaches that
 * leaf), all sure misses is -1, anything else goes through the traversal.
 * Needs ct_pack_grid first and the caller's arrays cand_off
 * (grid_nx * grid_ny + 1 int64) and cand_box (n_elements float4).
 * ct_cand_count fills the boxes and offsets and returns the number of
 * entries (sets cand_n, cand_tol; synchronises); the caller then allocates
 * cand_idx and cand_lbox (cand_n entries each) and calls ct_cand_fill, which
 * sets CT_DEVERR_CAPACITY in the tree's error word should its decisions
 * differ from the count's (no write goes past a grid cell's range).
 * scratch: ct_cand_scratch_size bytes. */
size_t ct_cand_scratch_size(const ct_tree* tree);
int ct_cand_count(ct_tree* tree, double cover_tol, void* scratch, size_t scratch_bytes, int64_t* total_host,
                  void* stream);
int ct_cand_fill(ct_tree* tree, void* scratch, size_t scratch_bytes, void* stream);

/* locate_points query.py:110-117 (locate_point 63-107).  out: n (int64). */
int ct_locate_points(const ct_tree* tree, const double* points, int64_t n, double tolerance, int32_t mode,
                     int64_t* out, void* stream);

/* Batched float32 form of locate_points (query.py:110-117): queries are
 * ordered along a Morton curve over the tree bbox (radix sort by the top
 * sort_bits of a 24-bit key, 4096 x 4096 grid; sort_bits 0 = input order,
 * else 8, 16 or 24), located through the candidate lists (a float32 pass that
 * settles most queries) and a float32 traversal of the rest that collects
 * candidate cells for queries whose float32 leaf test is ambiguous, then
 * finished by float64 tests of those candidates (and a float64 traversal for
 * the rare query with too many candidates).  Above 2^23 queries the list
 * results go out through a bucketed scatter (the workspace's sort buffers).
 * Output identical to ct_locate_points.
 * Workspace: ct_locate_workspace_size(n, sort_bits) bytes. */
size_t ct_locate_workspace_size(int64_t n, int32_t sort_bits);
int ct_locate_points_batched(const ct_tree* tree, const double* points, int64_t n, double tolerance, int32_t sort_bits,
                             int64_t* out, void* workspace, size_t workspace_bytes, void* stream);
/* The three stages of ct_locate_points_batched, callable separately (same
 * arguments and workspace): order, float32 pass, float64 pass over the
 * deferred queries.  ct_locate_deferred_count reports what the last float32
 * pass deferred (synchronises). */
int ct_locate_bin(const ct_tree* tree, const double* points, int64_t n, int32_t sort_bits, void* workspace,
                  size_t workspace_bytes, void* stream);
int ct_locate_fast(const ct_tree* tree, const double* points, int64_t n, double tolerance, int32_t sort_bits,
                   int64_t* out, void* workspace, size_t workspace_bytes, void* stream);
int ct_locate_exact(const ct_tree* tree, const double* points, int64_t n, double tolerance, int32_t sort_bits,
                    int64_t* out, void* workspace, size_t workspace_bytes, void* stream);
/* counts_host4: queries sent to the overflow pass, queries with candidate
 * records, candidate pairs, queries the candidate lists left to the
 * traversal -- of the last float32 pass (synchronises). */
int ct_locate_deferred_count(const void* workspace, int64_t n, int32_t sort_bits, int64_t* counts_host4, void* stream);

/* A batch of face trees (no upstream counterpart): the points of every tree
 * located by one pipeline -- queries sorted by (tree, Morton key over that
 * tree's bbox), then the candidate-list, traversal, float64-pair, resolve and
 * overflow stages with the tree looked up per query.  Results equal
 * ct_locate_points on each tree.  points: n_points x 2, the points of tree i
 * at rows point_off[i] .. point_off[i + 1] - 1; tolerances: one per tree.
 * ct_forest_locate_prepare uploads the tree records (synchronises; call it
 * again when a tree or a tolerance changes); ct_forest_locate only enqueues
 * kernels and memsets, so it can be captured in a CUDA graph and replayed. */
typedef struct ct_forest_plan {
    int64_t n_points;
    int32_t n_trees;
    int32_t kt;           /* leaf-filter width: 3, 4 or 32 (largest n_max_vert) */
    int32_t stack;        /* traversal stack entries per query (deepest tree + 2) */
    int32_t morton_bits;  /* Morton bits of the sort key below the tree bits */
    unsigned int* error_word; /* device: error bits of the batch-wide stages (the first tree's word) */
    int64_t max_tree_points;  /* most points of one tree */
    int32_t tune_cells_bpsm;  /* as ct_tree.tune_cells_bpsm (set before ct_forest_locate; 0 = default) */
    int32_t tune_fast_bpsm;   /* as ct_tree.tune_fast_bpsm */
} ct_forest_plan;
size_t ct_forest_locate_workspace_size(int64_t n_points, int32_t n_trees);
int ct_forest_locate_prepare(const ct_tree* trees, int32_t n_trees, const double* tolerances,
                             const int64_t* point_off, int64_t n_points, ct_forest_plan* plan, void* workspace,
                             size_t workspace_bytes, void* stream);
int ct_forest_locate(const ct_forest_plan* plan, const double* points, int64_t* out, void* workspace,
                     size_t workspace_bytes, void* stream);

/* The index and query records of a batch built by ct_build_forest_async,
 * computed on the device (no upstream counterpart).  With it a batch's
 * build and point location run as one sequence of launches with no host
 * synchronisation -- ct_counter_clockwise and ct_face_bboxes over the faces,
 * ct_build_forest_async, ct_forest_index_build, ct_forest_locate -- which can
 * be captured in one CUDA graph and replayed when the vertices and points
 * change (the mesh topology and the point counts stay).  Per tree it computes
 * on the device what ct_bbox_summary, ct_pack_tree and ct_pack_grid compute
 * for a single tree (bbox, default tolerance, float32 frame, packed nodes and
 * cells, start-node grid of a fixed shape) and writes the tree records of
 * ct_forest_locate into its workspace.  The batch locate then runs without
 * candidate lists (every query traverses from its start node); results equal
 * ct_locate_points on each tree.  Errors are reported in error_word:
 * CT_DEVERR_STACK (a tree deeper than `stack` - 2 levels), CT_DEVERR_NONFINITE
 * (a box or node bound is not finite). */
typedef struct ct_forest_index {
    /* inputs (device) */
    const double* vertices;     /* all meshes' vertices, x y */
    const int64_t* faces;       /* tree i: n_i x K_i indices into `vertices` (-1 padded) from face_off[i] */
    const int64_t* face_off;    /* n_trees: first int64 of tree i's faces (also its float64 cells' offset) */
    const int64_t* poly32_off;  /* n_trees: first float4 of tree i's float32 cells */
    const int32_t* tree_K;      /* n_trees: n_max_vert of tree i */
    const double* bb_coords;    /* n_total x 4, the boxes the trees were built from */
    const int64_t* tree_off;    /* n_trees + 1 face offsets of the trees */
    const int64_t* node_off;    /* n_trees + 1 node offsets (ct_build_forest_async) */
    const int32_t* max_depth;   /* n_trees (ct_build_forest_async) */
    const int64_t* node_child;
    const double* node_Lmax;
    const double* node_Rmin;
    const int64_t* node_ptr;
    const int64_t* node_size;
    const uint8_t* node_dim;
    const int64_t* bb_indices;  /* n_total, relative to each tree */
    /* start-node grids: tree i has grid_nx[i] x grid_ny[i] cells at
     * grid_start + grid_off[i] (shapes fixed by the caller, e.g. from
     * ct_grid_shape; the origin and scale follow each build's boxes) */
    int32_t* grid_start;
    const int64_t* grid_off;    /* n_trees + 1 */
    const int32_t* grid_nx;
    const int32_t* grid_ny;
    /* sizes and settings (host) */
    int64_t n_total;
    int64_t node_capacity;
    int64_t grid_cells;         /* grid_off[n_trees] */
    int32_t n_trees;
    int32_t k_max;              /* largest K_i */
    int32_t stack;              /* traversal stack entries per query (deepest tree + 2, at most 128) */
    int32_t pad_;
    double tolerance;           /* query tolerance of every tree; <= 0: each tree's default */
    /* outputs (device), written by ct_forest_index_build */
    void* nodes_f32;            /* node_capacity x 16 B */
    void* nodes_f64;            /* node_capacity x 16 B */
    void* poly_f64;             /* 16 B per face vertex, tree i from face_off[i], leaf order */
    void* poly_f32;             /* 16 B units, tree i from poly32_off[i] (ct_poly32_stride(K_i) per cell) */
    uint8_t* poly_len;          /* n_total */
    uint8_t* poly_len32;        /* n_total */
    unsigned long long* summary; /* scratch: n_trees x 16 words */
    unsigned int* error_word;   /* device: CT_DEVERR_* bits */
    /* candidate lists of the batch locate (as ct_cand_count / ct_cand_fill for
     * one tree, covering each tree's query tolerance), built when
     * cand_capacity > 0; a build whose entries exceed cand_capacity runs the
     * locate without them (same results, slower) */
    unsigned long long* cand_count; /* scratch: grid_cells + 1 */
    int64_t* cand_off;          /* grid_cells + 1 offsets (of all trees' grid cells) */
    void* cand_box;             /* n_total x 16 B */
    int32_t* cand_idx;          /* cand_capacity entries: leaf positions within the tree */
    void* cand_lbox;            /* cand_capacity x 16 B */
    void* cand_scan_ws;         /* ct_scan_workspace_size(grid_cells + 1) bytes */
    size_t cand_scan_bytes;
    int64_t cand_capacity;
} ct_forest_index;
/* Fills `plan` (points per tree from point_off_host, n_trees + 1 host
 * offsets; kt and stack from the index's k_max and stack) and uploads the
 * point offsets into the ct_forest_locate workspace (synchronises; call once
 * per set of sizes). */
int ct_forest_index_prepare(const ct_forest_index* index, const int64_t* point_off_host, int64_t n_points,
                            ct_forest_plan* plan, void* workspace, size_t workspace_bytes, void* stream);
/* Enqueues the device-side index of the current build (kernels and memsets
 * only). */
int ct_forest_index_build(const ct_forest_index* index, const ct_forest_plan* plan, void* workspace,
                          size_t workspace_bytes, void* stream);

/* locate_points_on_edge query.py:167-174 (locate_point_on_edge 121-164). */
int ct_locate_points_on_edge(const ct_tree* tree, const double* points, int64_t n, double tolerance,
                             int64_t* out, void* stream);

/* ---------------------------------------------------------------------- */
/* Multi-result queries: count -> exclusive scan -> write                  */
/* (the upstream chunked grow-and-retry, query.py:46-59, 247-289, 458-533) */
/* ---------------------------------------------------------------------- */

/* Workspace bytes / exclusive scan of n int64 values; *total_host receives
 * the sum (synchronises the stream when total_host is not NULL). */
size_t ct_scan_workspace_size(int64_t n);
int ct_exclusive_scan(const int64_t* in, int64_t n, int64_t* out, void* workspace, size_t workspace_bytes,
                      int64_t* total_host, void* stream);

/* Work order of box (kind 0) or segment (kind 1) queries (no upstream
 * counterpart): a permutation grouping queries of similar size (box area /
 * segment length with a cell-size margin, 8-bit log classes), so one
 * warp's queries take similar time.  Passing it as `order` below changes no
 * result: counts and pairs stay indexed and ordered by query. */
size_t ct_work_order_workspace_size(int64_t n);
int ct_work_order(const double* queries, int64_t n, int32_t kind, double cell_size, int32_t* order, void* workspace,
                  size_t workspace_bytes, void* stream);
/* One LSD pass on 8 bits of 32-bit keys (bits shift .. shift + 7):
 * kin/iin -> kout/iout, iin null for the indices 0 .. n-1.  Keys of one digit
 * keep the order of the 4096-key tiles they come from but may be permuted
 * within a tile (callers need grouping, not stability).  Workspace:
 * ct_radix_pass_workspace_size() bytes. */
size_t ct_radix_pass_workspace_size(void);
int ct_radix_pass(const unsigned* kin, const int* iin, int64_t n, int32_t shift, unsigned* kout, int* iout,
                  void* workspace, size_t workspace_bytes, void* stream);

/* Box index of a packed face or edge tree (no upstream counterpart): the
 * cell boxes in leaf order, every node's bounding box and leaf range, and
 * every leaf position's leaf start, in caller-allocated arrays set in the
 * descriptor (bb_leaf, node_box, leaf_start; bb_leaf32 optional).  With it
 * the box queries stop descending at nodes whose cells' bounding box lies
 * strictly inside the query box -- every cell below overlaps it -- and count
 * or write that subtree's cells in the upstream visiting order directly; with
 * bb_leaf32 too, the segment traversals skip nodes and cells whose box the
 * segment's line misses by more than the float64 rounding of the clipping
 * tests (certified in float32).  Results are unchanged.  scratch: ct_box_index_scratch_size(tree) bytes; the call only
 * enqueues work, so the scratch must stay allocated until that work has run
 * (stream order). */
size_t ct_box_index_scratch_size(const ct_tree* tree);
int ct_pack_box_index(ct_tree* tree, void* scratch, size_t scratch_bytes, void* stream);

/* locate_box query.py:177-244: per box (xmin, xmax, ymin, ymax) the number of
 * cells whose bbox overlaps it (strict, boxes_intersect geometry_utils.py:292-300).
 * order: NULL or a permutation of the boxes (processing order only). */
int ct_count_boxes(const ct_tree* tree, const double* boxes, int64_t n, const int32_t* order, int64_t* counts,
                   void* stream);
/* Writes (box index, cell index) pairs at the scanned offsets, box-major and
 * in traversal order -- upstream's locate_boxes output order. */
int ct_write_boxes(const ct_tree* tree, const double* boxes, int64_t n, const int32_t* order, const int64_t* offsets,
                   int64_t* ii, int64_t* jj, void* stream);
/* The same output; subtrees of at least min_job_cells cells (0: 8) wholly
 * inside a query box (box index) are queued in the workspace and their cells
 * written by one warp per subtree, coalesced, after the traversal, instead
 * of by the box's own thread.  total_pairs: the scanned total (sizes the
 * queue); workspace: ct_write_boxes_workspace_size(total_pairs,
 * min_job_cells) bytes, in use until the enqueued work has run. */
size_t ct_write_boxes_workspace_size(int64_t total_pairs, int32_t min_job_cells);
int ct_write_boxes_ws(const ct_tree* tree, const double* boxes, int64_t n, const int32_t* order,
                      const int64_t* offsets, int64_t total_pairs, int32_t min_job_cells, int64_t* ii, int64_t* jj,
                      void* workspace, size_t workspace_bytes, void* stream);

/* Small batches in one traversal (no upstream counterpart): the counting
 * pass also writes each box's first spec_cap cells (in output order) into
 * spec (n x spec_cap int32, 1 <= spec_cap <= 4096); the writing call then
 * copies the boxes whose count fits from spec and traverses again only for
 * the others (workspace as ct_write_boxes_ws).  Same output as
 * ct_count_boxes + ct_write_boxes. */
int ct_count_boxes_spec(const ct_tree* tree, const double* boxes, int64_t n, const int32_t* order, int64_t* counts,
                        int32_t* spec, int32_t spec_cap, void* stream);
int ct_write_boxes_spec(const ct_tree* tree, const double* boxes, int64_t n, const int32_t* order,
                        const int64_t* counts, const int64_t* offsets, const int32_t* spec, int32_t spec_cap,
                        int64_t total_pairs, int32_t min_job_cells, int64_t* ii, int64_t* jj, void* workspace,
                        size_t workspace_bytes, void* stream);

/* locate_edge query.py:357-455 over segments (n x 2 x 2).  mode 1: edge vs
 * face (Cohen-Sutherland + Cyrus-Beck, compute_edge_face_intersect
 * query.py:309-328); mode 0: edge vs edge (lines_intersect,
 * compute_edge_edge_intersect query.py:292-306, edge trees only).  In two
 * phases: the traversal writes candidate (segment, leaf position) pairs in
 * traversal order -- every visited cell, minus (mode 1) those
 * Cohen-Sutherland rejects by a shared outcode -- then one thread per
 * candidate runs the float64 cell test (keep = 0/1, xy: n_cand x 2 x 2), and
 * the hits are compacted in candidate order (pos = exclusive scan of keep)
 * with each segment's offset / count: upstream's pairs, order and clipped
 * coordinates (before sort_intersections_by_edge). */
int ct_count_edge_candidates(const ct_tree* tree, int32_t mode, const double* segs, int64_t n, const int32_t* order,
                              int64_t* counts, void* stream);
int ct_write_edge_candidates(const ct_tree* tree, int32_t mode, const double* segs, int64_t n, const int32_t* order,
                              const int64_t* offsets, int32_t* cand_seg, int32_t* cand_pos, void* stream);
/* One traversal for most segments (no upstream counterpart): the counting
 * pass also keeps each segment's first spec_cap candidates (leaf positions,
 * traversal order) in spec (n x spec_cap int32, 1 <= spec_cap <= 4096); the
 * writing call copies the segments whose count fits from spec and traverses
 * again only for the others.  Same candidates as the uncut pair above. */
int ct_count_edge_candidates_spec(const ct_tree* tree, int32_t mode, const double* segs, int64_t n,
                                  const int32_t* order, int64_t* counts, int32_t* spec, int32_t spec_cap,
                                  void* stream);
int ct_write_edge_candidates_spec(const ct_tree* tree, int32_t mode, const double* segs, int64_t n,
                                  const int32_t* order, const int64_t* counts, const int64_t* offsets,
                                  const int32_t* spec, int32_t spec_cap, int32_t* cand_seg, int32_t* cand_pos,
                                  void* stream);
/* The same candidates with each segment's traversal split across threads
 * (no upstream counterpart; a long segment's traversal otherwise runs on one
 * thread).  ct_count/write_edge_items cut every segment's traversal `cut`
 * levels below the root: the nodes at that depth (and the leaves above it)
 * it reaches, in traversal order, as work items (segment, node), segment-
 * major at the scanned per-segment offsets.  ct_count/write_item_candidates
 * run the traversal from each item's node: concatenated in item order the
 * candidates are ct_write_edge_candidates' (same pairs, same order).
 * ct_segment_candidate_ranges turns the items' candidate offsets / counts
 * into each segment's (for ct_compact_edge_hits).  Trees deeper than the
 * stacked traversal allows (max_depth + 2 > 128) are refused (CT_ERR_ARG):
 * they take the uncut entry points. */
int ct_count_edge_items(const ct_tree* tree, int32_t mode, const double* segs, int64_t n, const int32_t* order,
                        int32_t cut, int64_t* counts, void* stream);
int ct_write_edge_items(const ct_tree* tree, int32_t mode, const double* segs, int64_t n, const int32_t* order,
                        int32_t cut, const int64_t* offsets, int32_t* item_seg, int32_t* item_node, void* stream);
int ct_count_item_candidates(const ct_tree* tree, int32_t mode, const double* segs, const int32_t* item_seg,
                             const int32_t* item_node, int64_t n_items, int64_t* counts, void* stream);
int ct_write_item_candidates(const ct_tree* tree, int32_t mode, const double* segs, const int32_t* item_seg,
                             const int32_t* item_node, int64_t n_items, const int64_t* offsets, int32_t* cand_seg,
                             int32_t* cand_pos, void* stream);
int ct_segment_candidate_ranges(const int64_t* item_off, const int64_t* item_cnt, int64_t n,
                                const int64_t* item_cand_off, const int64_t* item_cand_cnt, int64_t n_items,
                                int64_t* cand_off, int64_t* cand_cnt, void* stream);
/* Diagnostics for tests of the segment test's float32 certificates (face
 * trees): per (segment, leaf position) pair, out[3t] = upstream's float64
 * Cohen-Sutherland verdict (1 accept, 0 reject), out[3t+1] = the float32
 * interval verdict used by ct_test_edge_candidates (1, 0, or -1 undecided),
 * out[3t+2] = 1 when the traversal's line filter surely misses the cell's
 * box (needs bb_leaf32).  A certificate is sound when out[3t+1] is -1 or
 * equals out[3t], and out[3t+2] = 1 only where out[3t] = 0. */
int ct_cs_certificates(const ct_tree* tree, const double* segs, const int32_t* cand_seg, const int32_t* cand_pos,
                       int64_t n_cand, int8_t* out, void* stream);
int ct_test_edge_candidates(const ct_tree* tree, int32_t mode, const double* segs, const int32_t* cand_seg,
                            const int32_t* cand_pos, int64_t n_cand, int64_t* keep, double* xy, void* stream);
int ct_compact_edge_hits(const ct_tree* tree, const int64_t* keep, const int64_t* pos, int64_t n_cand,
                         const int32_t* cand_seg, const int32_t* cand_pos, const double* xy_cand,
                         const int64_t* cand_off, const int64_t* cand_cnt, int64_t n, int64_t* ii, int64_t* jj,
                         double* xy, int64_t* offsets, int64_t* counts, void* stream);

/* sort_intersections_by_edge geometry_utils.py:564-574: stable sort of each
 * segment's results by t = (c - a) . (b - a), NaN last; writes the permuted
 * jj / xy (ii is unchanged: results are already grouped by segment). */
size_t ct_sort_workspace_size(int64_t total);
int ct_sort_intersections(const double* segs, int64_t n_segs, const int64_t* offsets, const int64_t* counts,
                          const int64_t* ii, const int64_t* jj_in, const double* xy_in, int64_t total,
                          int64_t* jj_out, double* xy_out, void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------- */
/* Per-pair kernels                                                        */
/* ---------------------------------------------------------------------- */

/* polygons_intersect algorithms/separating_axis.py:58-75 (out: 1 = overlap or touch). */
int ct_polygons_intersect(const double* vertices_a, const int64_t* faces_a, int32_t n_max_vert_a,
                          const double* vertices_b, const int64_t* faces_b, int32_t n_max_vert_b,
                          const int64_t* indices_a, const int64_t* indices_b, int64_t n, uint8_t* out, void* stream);

/* area_of_intersection algorithms/sutherland_hodgman.py:151-168 (subject: face a, clipper: face b). */
int ct_area_of_intersection(const double* vertices_a, const int64_t* faces_a, int32_t n_max_vert_a,
                            const double* vertices_b, const int64_t* faces_b, int32_t n_max_vert_b,
                            const int64_t* indices_a, const int64_t* indices_b, int64_t n, double* out,
                            unsigned int* error_word, void* stream);

/* box_area_of_intersection algorithms/sutherland_hodgman.py:171-187 (subject: the box). */
int ct_box_area_of_intersection(const double* boxes, const double* vertices, const int64_t* faces,
                                int32_t n_max_vert, const int64_t* indices_box, const int64_t* indices_face,
                                int64_t n, double* out, unsigned int* error_word, void* stream);

/* The two above with the pairs processed in `order` (a permutation of 0 ..
 * n-1, e.g. from ct_pair_order; NULL = index order).  Results are written
 * at each pair's own index, so they do not depend on the order. */
int ct_area_of_intersection_ordered(const double* vertices_a, const int64_t* faces_a, int32_t n_max_vert_a,
                                    const double* vertices_b, const int64_t* faces_b, int32_t n_max_vert_b,
                                    const int64_t* indices_a, const int64_t* indices_b, int64_t n,
                                    const int32_t* order, double* out, unsigned int* error_word, void* stream);
int ct_box_area_of_intersection_ordered(const double* boxes, const double* vertices, const int64_t* faces,
                                        int32_t n_max_vert, const int64_t* indices_box, const int64_t* indices_face,
                                        int64_t n, const int32_t* order, double* out, unsigned int* error_word,
                                        void* stream);

/* Processing order for the per-pair kernels (no upstream counterpart): the
 * pairs grouped by the polygon lengths of their two faces (faces_a NULL:
 * the pairs' first members are boxes), so that the lanes of a warp clip
 * polygons of the same lengths.  order: n int32.  Workspace:
 * ct_pair_order_workspace_size(n) bytes. */
size_t ct_pair_order_workspace_size(int64_t n);
int ct_pair_order(const int64_t* faces_a, int32_t n_max_vert_a, const int64_t* indices_a, const int64_t* faces_b,
                  int32_t n_max_vert_b, const int64_t* indices_b, int64_t n, int32_t* order, void* workspace,
                  size_t workspace_bytes, void* stream);

/* Keeps the pairs with area > 0 (area != NULL) or flag != 0 (celltree.py:183,
 * 226, 268); outputs have capacity n; *total_host = kept count (synchronises). */
size_t ct_compact_workspace_size(int64_t n);
int ct_compact_pairs(const double* area, const uint8_t* flag, int64_t n, const int64_t* ii, const int64_t* jj,
                     int64_t* ii_out, int64_t* jj_out, double* area_out, void* workspace, size_t workspace_bytes,
                     int64_t* total_host, void* stream);

/* compute_barycentric_weights celltree.py:306-351: triangle weights
 * (barycentric_triangle.py:46-64) when n_max_vert <= 3, else Wachspress
 * (barycentric_wachspress.py:88-107); rows of points not found are zero.
 * weights: n x max(3, n_max_vert). */
int ct_barycentric_weights(const ct_tree* tree, const double* points, const int64_t* face_indices, int64_t n,
                           double tolerance, double* weights, void* stream);

/* ---------------------------------------------------------------------- */
/* Batched build (no upstream counterpart)                                 */
/* ---------------------------------------------------------------------- */

/* build (creation.py:233-381) of n_trees trees at once: the bounding boxes of
 * all trees concatenated (tree i at rows tree_off[i] .. tree_off[i + 1] - 1,
 * tree_off host memory, every tree non-empty), built level by level together
 * (one host synchronisation per level for the whole batch).  n_nodes_host /
 * max_depth_host: one entry per tree.  Each tree's nodes and bb_indices are
 * identical to ct_build_tree on its own boxes. */
size_t ct_build_forest_workspace_size(int64_t n_total, int32_t n_trees, int32_t n_buckets, int32_t capacity_factor);
int ct_build_forest(const double* bb_coords, int64_t n_total, const int64_t* tree_off, int32_t n_trees,
                    int32_t n_buckets, int64_t cells_per_leaf, int32_t capacity_factor, void* workspace,
                    size_t workspace_bytes, int64_t* n_nodes_host, int32_t* max_depth_host, void* stream);
/* ct_build_forest + ct_build_forest_emit with every tree level driven on
 * the device: a fixed sequence of launches and no host synchronisation (the
 * call only enqueues work, so it can be captured in a CUDA graph and
 * replayed while the boxes change and the tree sizes do not).  tree_off_host
 * and tree_off_dev hold the same n_trees + 1 offsets.  Outputs on the device:
 * per tree its node count (n_nodes_dev), node offset into the node arrays
 * (node_off_dev, n_trees + 1; the arrays hold node_capacity nodes -- the sum
 * of ct_pessimistic_n_nodes over the trees always suffices), depth
 * (max_depth_dev); status_dev = 0, or CT_DEVERR_* bits: BUCKET (a centroid
 * outside every bucket), CAPACITY (record or node capacity exceeded: retry
 * with a larger capacity_factor), LOOP (more than 64 tree levels above the
 * subtree size of 128 cells: use ct_build_forest).  Nodes and bb_indices are
 * those of ct_build_forest whenever status_dev is 0. */
int ct_build_forest_async(const double* bb_coords, int64_t n_total, const int64_t* tree_off_host,
                          const int64_t* tree_off_dev, int32_t n_trees, int32_t n_buckets, int64_t cells_per_leaf,
                          int32_t capacity_factor, void* workspace, size_t workspace_bytes, int64_t node_capacity,
                          int64_t* child, double* Lmax, double* Rmin, int64_t* ptr, int64_t* size, uint8_t* dim,
                          int64_t* bb_indices, int64_t* n_nodes_dev, int64_t* node_off_dev, int32_t* max_depth_dev,
                          unsigned int* status_dev, void* stream);

/* node_off: device, n_trees + 1 node offsets (prefix sums of n_nodes); the
 * node arrays hold every tree's nodes at its offset (child, ptr relative to
 * the tree); bb_indices (n_total) hold each tree's indices at its rows. */
int ct_build_forest_emit(const void* workspace, int64_t n_total, int32_t n_trees, int32_t n_buckets,
                         int32_t capacity_factor, const int64_t* node_off, int64_t* child, double* Lmax, double* Rmin,
                         int64_t* ptr, int64_t* size, uint8_t* dim, int64_t* bb_indices, void* stream);

/* ---------------------------------------------------------------------- */
/* Adjoints (no upstream counterpart)                                      */
/* ---------------------------------------------------------------------- */

/* Reverse-mode derivative of ct_area_of_intersection (polygon_polygon_clip_area
 * sutherland_hodgman.py:83-148 + polygon_area geometry_utils.py:82-95) with
 * the pairs held fixed: grad_va (n_vertices_a x 2) and grad_vb
 * (n_vertices_b x 2) are ACCUMULATED (+=) with sum_t grad_area[t] *
 * d area[t] / d vertex.  The clip is replayed with a tape of at most 160
 * vertices per pair; CT_DEVERR_CLIP in *error_word if it overflows. */
int ct_area_of_intersection_grad(const double* vertices_a, const int64_t* faces_a, int32_t n_max_vert_a,
                                 const double* vertices_b, const int64_t* faces_b, int32_t n_max_vert_b,
                                 const int64_t* indices_a, const int64_t* indices_b, int64_t n,
                                 const double* grad_area, double* grad_va, double* grad_vb,
                                 unsigned int* error_word, void* stream);

/* Reverse-mode derivative of ct_barycentric_weights (barycentric_triangle.py:28-43,
 * barycentric_wachspress.py:26-85, on-edge branch included) with the face
 * indices held fixed.  grad_weights: n x n_weights (n_weights = max(3, n_max_vert));
 * grad_vertices (n_vertices x 2) is ACCUMULATED; grad_points (n x 2, may be
 * NULL) is written. */
int ct_barycentric_weights_grad(const double* points, const int64_t* face_indices, int64_t n, const double* vertices,
                                const int64_t* faces, int32_t n_max_vert, int32_t n_weights, double tolerance,
                                const double* grad_weights, double* grad_vertices, double* grad_points,
                                void* stream);

/* ---------------------------------------------------------------------- */
/* Exported helpers and the regridding step                                */
/* ---------------------------------------------------------------------- */

/* liang_barsky_line_box_clip algorithms/liang_barsky.py:10-64, one segment
 * per row: a, b (n x 2), boxes (n x 4: xmin, xmax, ymin, ymax) -> ok (n),
 * clipped c, d (n x 2; NaN when not ok). */
int ct_liang_barsky_line_box_clip(const double* a, const double* b, const double* boxes, int64_t n, uint8_t* ok,
                                  double* c, double* d, void* stream);

/* points_in_triangles geometry_utils.py:273-289: out[i] = point_in_triangle
 * (241-270) of point i in triangle face_indices[i] (first three vertices of
 * the face).  A face index outside [0, n_faces) sets bit 1 of *error_word
 * (upstream indexes without a check) and gives 0. */
int ct_points_in_triangles(const double* points, const int64_t* face_indices, int64_t n, const int64_t* faces,
                           int32_t n_max_vert, int64_t n_faces, const double* vertices, double tolerance,
                           uint8_t* out, unsigned int* error_word, void* stream);

/* Regridding step after intersect_faces / intersect_boxes (no upstream
 * counterpart; the upstream example builds a dense weight matrix,
 * examples/spatial_indexing_2d_grids.py:245-313).  The query-major pairs
 * (rows non-decreasing, checked: bit 2 of *error_word) are a CSR matrix once
 * row_ptr (n_rows + 1) is known: ct_csr_row_ptr.  ct_csr_weighted_mean:
 * mean[r] = sum(w x[col]) / sum(w) over row r (NaN without weight),
 * weight_sum[r] = sum(w) (may be NULL). */
size_t ct_csr_workspace_size(int64_t n_rows);
int ct_csr_row_ptr(const int64_t* rows, int64_t n_pairs, int64_t n_rows, int64_t* row_ptr, void* workspace,
                   size_t workspace_bytes, unsigned int* error_word, void* stream);
int ct_csr_weighted_mean(const int64_t* row_ptr, const int64_t* cols, const double* weights, int64_t n_rows,
                         int64_t n_cols, const double* x, double* mean, double* weight_sum, unsigned int* error_word,
                         void* stream);

/* ---------------------------------------------------------------------- */
/* Node-bound diagnostics                                                  */
/* ---------------------------------------------------------------------- */

/* collect_node_bounds query.py:568-622 (out: n_nodes x 4; parent_ws: n_nodes int64). */
int ct_node_bounds(const int64_t* child, const double* Lmax, const double* Rmin, const uint8_t* dim, int64_t n_nodes,
                   const double* bbox_host4, int64_t* parent_ws, double* out, void* stream);
/* validate_node_bounds query.py:625-663 (valid: n_nodes). */
int ct_validate_node_bounds(const int64_t* child, const int64_t* ptr, const int64_t* size, int64_t n_nodes,
                            const int64_t* bb_indices, const double* bb_coords, const double* node_bounds,
                            uint8_t* valid, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CELLTREE_GB300_H */
