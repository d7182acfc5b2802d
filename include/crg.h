/*
 * crg.h -- C ABI of the GB300-native conservative-regridding library.
 *
 * This is the drop-in boundary for ConservativeRegridding.jl v0.2.5's two hot
 * paths.  Each entry point names the reference interface it replaces
 * (paths relative to the ConservativeRegridding.jl repository).  Plain
 * pointers and sizes only; no exceptions cross it; every call returns a
 * crg_status and crg_last_error() gives the message of the last failure on
 * the calling thread.
 *
 * Index conventions.  Cells are numbered from 0.  A curvilinear block with
 * nx x ny cells has (nx+1) x (ny+1) points stored i-fastest; cell (i, j) has
 * index block_offset + i + j*nx and the ring p(i,j), p(i+1,j), p(i+1,j+1),
 * p(i,j+1) -- the reference's CellBasedGrid (src/trees/grids.jl:71-85) and
 * cartesian_to_linear_idx (src/trees/interfaces.jl:241-243) shifted to
 * 0-based, with blocks laid out like the cubed-sphere face offsets
 * (ext/ConservativeRegriddingClimaCoreExt.jl:56-61).
 *
 * Field layout.  A field array holds nfields fields of n cells; element
 * (cell c, field f) is at base[c*stride_cell + f*stride_field] (in elements).
 * stride_cell = 1 is the reference's dims=1 N-D layout; stride_field = 1
 * puts the fields of one cell side by side (dims = last).
 */
#ifndef CRG_H
#define CRG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CRG_ABI_VERSION 2

typedef enum {
    CRG_OK = 0,
    CRG_ERR_INVALID_ARGUMENT = 1,   /* reference: ArgumentError (src/regridder/regrid.jl:242-245) */
    CRG_ERR_DIMENSION_MISMATCH = 2, /* reference: DimensionMismatch (src/regridder/regrid.jl:289-296) */
    CRG_ERR_CUDA = 3,
    CRG_ERR_OUT_OF_MEMORY = 4,
    CRG_ERR_NOT_SUPPORTED = 5,
    CRG_ERR_GEOMETRY = 6,           /* a clipped polygon exceeded its vertex capacity (non-convex input) */
    CRG_ERR_INTERNAL = 7
} crg_status;

typedef enum { CRG_PLANAR = 0, CRG_SPHERICAL = 1 } crg_manifold;
typedef enum { CRG_GRID_CURVILINEAR = 0, CRG_GRID_CELLS = 1 } crg_grid_kind;
typedef enum { CRG_F64 = 0, CRG_F32 = 1, CRG_BF16 = 2 } crg_dtype;

/* A grid of convex cells.  Pointers may be host or device memory (detected).
 * Spherical coordinates are unit vectors (x, y, z); planar ones are (x, y).
 * Replaces the grids the reference turns into trees with Trees.treeify
 * (src/trees/interfaces.jl:94-129): vertex matrices (CellBasedGrid,
 * TopDownQuadtreeCursor), cubed-sphere faces (CubedSphereToplevelTree,
 * src/trees/wrappers.jl:140-159) and per-cell polygons (HEALPix pixels,
 * ext/ConservativeRegriddingHealpixExt.jl:159-167; FlatNoTree polygon lists). */
typedef struct crg_grid_desc {
    int32_t kind;               /* crg_grid_kind */
    int32_t manifold;           /* crg_manifold */
    int32_t nblocks;            /* CURVILINEAR: number of blocks, 1..12 */
    int32_t max_verts;          /* CELLS: vertex slots per cell, 3..8 */
    int64_t ncells;             /* total number of cells */
    const int64_t* block_nx;    /* CURVILINEAR: [nblocks] cells along i (host memory) */
    const int64_t* block_ny;    /* CURVILINEAR: [nblocks] cells along j (host memory) */
    const double* points;       /* CURVILINEAR: blocks back to back, (nx+1)*(ny+1) points each, i fastest */
    const double* cell_verts;   /* CELLS: [ncells][max_verts][dim] in ring order (not closed) */
    const int32_t* cell_nverts; /* CELLS: [ncells] vertex counts, or NULL when all are max_verts */
} crg_grid_desc;

typedef struct crg_build_opts {
    int32_t normalize;  /* divide A and both area vectors by maximum(A): normalize!(::Regridder),
                           src/regridder/regridder.jl:54-62 (the reference's keyword default is false) */
    int32_t flags;      /* reserved, must be 0 */
    void* stream;       /* cudaStream_t for the build; NULL = legacy default stream */
} crg_build_opts;

typedef struct crg_regridder crg_regridder;

typedef struct crg_info {
    int64_t n_dst, n_src, nnz, n_candidates;
    int32_t manifold, normalized;
    double normalizer;       /* maximum(A) before normalisation (1.0 when not normalised) */
    double t_build_ms;       /* wall time of crg_build on the stream (CUDA events) */
    double t_search_ms;      /* caps, ordering, hierarchy and dual traversal */
    double t_clip_ms;        /* per-pair clip + area */
    double t_assemble_ms;    /* CSR/CSC assembly, areas, normalisation, weight derivation */
    int64_t clip_overflows;  /* pairs whose clip exceeded the vertex capacity */
    int32_t device;
    int32_t pad;
    /* merge-path layout of the batched cell-major apply, [0] = forward, [1] = transpose */
    int64_t merge_tasks[2];  /* tasks of about 64 entries, cut at row starts */
    int64_t cut_rows[2];     /* rows longer than 16 entries cut between tasks */
    int64_t carry_slots[2];  /* pieces of the cut rows (512-byte partial sums each) */
    int64_t empty_rows[2];   /* rows without entries (written as zeros) */
    int64_t n_clipped;       /* candidate pairs left for the clip after the FP32 separation filter */
} crg_info;

/* Build the regridder from `src` to `dst`.
 * Replaces Regridder(dst, src; normalize) (src/regridder/regridder.jl:105-163):
 * candidate search (src/regridder/intersection_areas.jl:48-65, :67-122), the
 * per-pair DefaultIntersectionOperator (src/regridder/regridder.jl:96-103),
 * SparseArrays.sparse assembly (src/regridder/intersection_areas.jl:115-121),
 * per-cell areas (src/regridder/regridder.jl:165-178) and normalize!.
 * Mixed planar/spherical inputs are rejected: promote on the host, as the
 * reference's Regridder(dst, src) does (src/regridder/regridder.jl:109-117).
 * Indices are 32-bit: a grid of 2^31 cells or more, a search of 2^31 candidate
 * pairs or more (or of 2^26 leaf pairs of 8-cell blocks, whose count could
 * pass 2^32) is refused with CRG_ERR_NOT_SUPPORTED. */
crg_status crg_build(const crg_grid_desc* dst, const crg_grid_desc* src, const crg_build_opts* opts,
                     crg_regridder** out);

/* Reference counting: transpose(R) (src/regridder/regridder.jl:49-50) shares
 * the same arrays; a host wrapper that hands out a transposed view retains the
 * handle and releases it when the view dies.  The last release frees it. */
crg_status crg_regridder_retain(crg_regridder* r);
crg_status crg_regridder_release(crg_regridder* r);

crg_status crg_regridder_info(const crg_regridder* r, crg_info* out);

/* dst = (A src) ./ a_d  (transpose = 0)   or   dst = (A^T src) ./ a_s  (transpose = 1);
 * without the division when normalize = 0.
 * Replaces regrid!(dst, R, src; dims) with its pipeline extract/initialize/
 * perform_regridding!/finalize_regridding! (src/regridder/regrid.jl:63-118),
 * the N-D NDSliceLoop one-mul!-per-slice loop (src/regridder/regrid.jl:225-318)
 * by a single SpMM over all fields, and regrid!(dst, transpose(R), src).
 * dtype CRG_F64 accumulates in FP64 in the reference's summation order;
 * CRG_F32 / CRG_BF16 read FP32 weights and accumulate in FP32.
 * src and dst may be host or device pointers; host buffers are staged through
 * device memory on `stream`, which the call synchronises before returning. */
crg_status crg_apply(const crg_regridder* r, int32_t transpose, int32_t dtype,
                     const void* src, int64_t src_stride_cell, int64_t src_stride_field,
                     void* dst, int64_t dst_stride_cell, int64_t dst_stride_field,
                     int64_t nfields, int32_t normalize, void* stream);

/* Adjoint of crg_apply with the same arguments: given gdst = dL/d(dst), write
 * gsrc = dL/d(src) = A^T (gdst ./ a_d) (transpose = 0), or A (gdst ./ a_s)
 * (transpose = 1); without the division when normalize = 0.  It reads the
 * opposite-direction copy of A, so no atomics are needed.  The reference has
 * no derivative rules (Project.toml has no ChainRulesCore); this is the
 * backward of regrid! for an rrule. */
crg_status crg_apply_adjoint(const crg_regridder* r, int32_t transpose, int32_t dtype,
                             const void* gdst, int64_t gdst_stride_cell, int64_t gdst_stride_field,
                             void* gsrc, int64_t gsrc_stride_cell, int64_t gsrc_stride_field,
                             int64_t nfields, int32_t normalize, void* stream);

/* Builds n regridders at once, out[k] from src[k] to dst[k] (k < n), with the
 * options in *opts (opts->stream is ignored).  No counterpart in the
 * reference, which builds one Regridder at a time
 * (src/regridder/regridder.jl:105-163); for many small grid pairs, whose
 * builds are short kernels separated by host synchronisations, nthreads host
 * threads (0: up to 8) build concurrently, each on its own stream.  On a
 * failure every regridder of the call is released, out[] is all NULL and the
 * lowest failing k's status is returned (its message names k). */
crg_status crg_build_batch(int64_t n, const crg_grid_desc* dst, const crg_grid_desc* src, const crg_build_opts* opts,
                           int32_t nthreads, crg_regridder** out);

/* One apply of a batch: the arguments of crg_apply (adjoint = 1 for
 * crg_apply_adjoint), device pointers only. */
typedef struct crg_apply_item {
    const crg_regridder* regridder;
    int32_t transpose, dtype;
    const void* src;
    int64_t src_stride_cell, src_stride_field;
    void* dst;
    int64_t dst_stride_cell, dst_stride_field;
    int64_t nfields;
    int32_t normalize, adjoint;
} crg_apply_item;

/* A CUDA graph of the applies of n items, captured once and replayed by
 * crg_apply_plan_launch with one launch: the batched form of regrid! over
 * many regridders (no counterpart in the reference).  The items are parallel
 * branches of the graph, so their outputs must not overlap (inputs may be
 * shared).  The plan retains the regridders and keeps the field pointers:
 * launch it again after writing new values into the same buffers.  Its
 * temporaries are graph allocations; launches of one plan must not overlap. */
/* The applies of n items (the arguments of crg_apply; host or device fields)
 * run concurrently on up to nthreads host threads (0: 4), each on its own
 * stream, after the work queued on `stream`; `stream` continues after all of
 * them, and items with host fields are complete on return.  Independent
 * applies with host fields thus share both directions of the host link (e.g.
 * R on one field set and transpose(R) on another).  Outputs must not overlap.
 * On failure the first failing item is named.  No reference counterpart: the
 * reference applies one regridder, one slice at a time. */
crg_status crg_apply_batch(int64_t n, const crg_apply_item* items, int32_t nthreads, void* stream);

typedef struct crg_apply_plan crg_apply_plan;
crg_status crg_apply_plan_create(int64_t n, const crg_apply_item* items, crg_apply_plan** out);
crg_status crg_apply_plan_launch(crg_apply_plan* plan, void* stream);
crg_status crg_apply_plan_destroy(crg_apply_plan* plan);
/* How a plan runs (no reference counterpart): the kernel launches of one
 * replay, and how many of its items the persistent batch launch covers.  The
 * items whose own apply cannot fill the GPU -- cell-major FP32 / BF16 fields
 * of more than 128 fields on a matrix with fewer merge-path tasks than the GPU
 * holds resident warps -- run as one launch over all their (task, 128-field
 * pass) units, plus one launch that sums the rows cut between tasks and zeroes
 * empty rows; the others are captured as their own, autotuned applies on graph
 * branches beside it.  With the environment variable CRG_PLAN_BATCH=all every
 * cell-major FP32 / BF16 or single-field item joins the persistent launch
 * (groups of rows for the items below 32 fields), with CRG_PLAN_BATCH=0 none
 * does.  Each item's result has the bits of its own crg_apply either way.
 * Either pointer may be NULL. */
crg_status crg_apply_plan_info(const crg_apply_plan* plan, int64_t* kernels, int64_t* batched_items);

/* Derivatives of the areas with respect to the destination grid's vertices.
 * No counterpart in the reference (it has no derivatives, Project.toml:10-23);
 * with crg_apply_adjoint it gives the pullback of regrid! for a ChainRulesCore
 * rrule.  Computes, into grad (zeroed first),
 *     G = sum_ij row_weight[i] * src_field[j] * dA_ij/dV + sum_i area_weight[i] * da_i/dV,
 * where A_ij is the unnormalised intersection area of destination cell i and
 * source cell j (the nonzeros of r), a_i the unnormalised area of destination
 * cell i, and V the destination vertex coordinates exactly as `dst` lays them
 * out: [points][dim] for CRG_GRID_CURVILINEAR (shared corners accumulate),
 * [ncells][max_verts][dim] for CRG_GRID_CELLS; dim is 3 (x, y, z of the unit
 * vectors; project onto longitude/latitude tangents for angle derivatives) or
 * 2 on the plane.  dst and src must be the grids r was built from.
 * row_weight and src_field may both be NULL (area term only); area_weight
 * may be NULL.  For d = (A s) ./ a and an output cotangent g:
 * row_weight = g ./ a, area_weight = -g .* d ./ a.  Host or device pointers;
 * returns after the result is in grad.  Derivatives with respect to the
 * SOURCE vertices are this same call on the regridder built the other way
 * round (crg_build(src, dst)), with dst and src swapped and row_weight and
 * src_field exchanged: A_ij is the area of the intersection of two cells,
 * symmetric in them (the source cell areas do not enter regrid!). */
crg_status crg_area_grad(const crg_regridder* r, const crg_grid_desc* dst, const crg_grid_desc* src,
                         const double* row_weight, const double* src_field, const double* area_weight, double* grad,
                         void* stream);

/* Scratch held by crg_apply_noalloc, in bytes (per GPU that loads the library). */
#define CRG_NOALLOC_SCRATCH_BYTES (16u << 20)

/* crg_apply without any device allocation.  It has no counterpart in the
 * reference; it exists for callers that cannot call cudaMalloc: an
 * application whose memory pool owns the whole device (a Julia CUDA.jl or
 * PyTorch caching allocator sized to the GPU, a model that pre-allocates
 * everything at start-up and forbids allocation while it runs).  Same
 * arguments as crg_apply, restricted to the cell-major merge-path kernels (the
 * narrow one below 32 fields), whose results it has bit for bit: device
 * pointers only, dtype CRG_F32 or CRG_BF16, src_stride_field = dst_stride_field
 * = 1, nfields and both cell strides multiples of 4, 16-byte aligned (FP32) /
 * 8-byte aligned (BF16) base pointers.  The partial sums of rows cut between
 * work blocks (crg_info.carry_slots, 512 bytes each) go to a scratch array the
 * library declares statically (CRG_NOALLOC_SCRATCH_BYTES per GPU, kept until
 * the process exits): at most 32,768 pieces.  With the default task length
 * of 64 entries every regridder with at most 1,048,576 nonzeros fits (at most
 * 2 pieces per 64 entries; the tuning variable CRG_TASK_NNZ = 32 halves that
 * bound); a larger one fits unless many of its rows are longer than 16
 * entries, and one that does not fit is refused with CRG_ERR_NOT_SUPPORTED.
 * The array is reserved on a GPU when the part of the library holding it is
 * loaded there: by the first crg_build (or crg_build_* / crg_build_batch) on
 * that GPU, which also looks up its device address (cudaGetSymbolAddress) --
 * so build before the application's pool takes the whole device.  A call in
 * a CUDA context other than the one of the last lookup (after a
 * cudaDeviceReset, say) looks the address up again; make that call before any
 * stream capture.  The scratch is shared by every call on the device and
 * keeps the previous call's contents (each call writes every slot it reads
 * before reading it), so calls that may overlap on the GPU -- on different
 * streams without ordering -- race on it. */
crg_status crg_apply_noalloc(const crg_regridder* r, int32_t transpose, int32_t dtype,
                             const void* src, int64_t src_stride_cell, int64_t src_stride_field,
                             void* dst, int64_t dst_stride_cell, int64_t dst_stride_field,
                             int64_t nfields, int32_t normalize, void* stream);

/* Copy A out as CSC (rows = dst cells, columns = src cells), i.e. the
 * reference's R.intersections::SparseMatrixCSC (src/regridder/regridder.jl:25-36)
 * with rows ascending inside each column.  index_base 1 gives Julia's 1-based
 * colptr/rowval.  Host or device destination pointers; colptr has n_src+1
 * entries, rowval and nzval have nnz. */
crg_status crg_get_csc(const crg_regridder* r, int32_t index_base, int64_t* colptr, int64_t* rowval, double* nzval);

/* The same matrix as CSR (rows = dst cells, columns ascending in each row). */
crg_status crg_get_csr(const crg_regridder* r, int32_t index_base, int64_t* rowptr, int64_t* colval, double* nzval);

/* Folded (tripolar) grids, RightCenterFolded: in the top cell row (j = ny,
 * 1-based) cell i and cell nx+1-i are the same physical quadrilateral.  As in
 * the reference (ext/ConservativeRegriddingOceananigansExt.jl:117-175), the
 * grid handed to crg_build keeps one slot of each pair as a real cell (slots
 * 1..nx/4 and nx/2+1..nx/2+nx/4) and makes the partner a ghost: a
 * CRG_GRID_CELLS cell with 0 vertices, which has no area and is never a
 * candidate.  After an apply to such a destination, crg_mirror_fold copies
 * each primary's value into its partner (the reference's
 * mirror_fold_partners!, :205-240), for every field: cells are numbered
 * i + j * nx, the field is (cells, fields) with the given strides, nx is a
 * multiple of 4.  Device pointers run a kernel on `stream`; host pointers are
 * copied on the host after the stream's work. */
crg_status crg_mirror_fold(int32_t dtype, void* field, int64_t stride_cell, int64_t stride_field, int64_t nfields,
                           int64_t nx, int64_t ny, void* stream);

/* The ESMF offline-weights arrays of save_esmf_weights
 * (ext/ConservativeRegriddingNCDatasetsExt.jl:18-60): entries in CSC order
 * (source column ascending, destination row ascending inside it, as findnz
 * returns them), row = destination cell, col = source cell (index_base 1
 * for ESMF files), S = A_ij / a_i ("destarea" normalisation); frac_a =
 * column sums of A / source areas, frac_b = row sums / destination areas
 * (Kahan sums); area_a, area_b = the cell areas.  frac_*, area_* may be NULL.
 * Host or device pointers.  Like the reference, the weights follow ESMF
 * conventions for a regridder built without normalize (S and frac_* are the
 * same either way; the areas are divided by the normaliser). */
crg_status crg_get_esmf_weights(const crg_regridder* r, int32_t index_base, int64_t* row, int64_t* col, double* S,
                                double* frac_a, double* frac_b, double* area_a, double* area_b);

/* Per-cell areas R.dst_areas and R.src_areas (src/regridder/regridder.jl:149-150),
 * divided by the normaliser when the regridder was built with normalize. */
crg_status crg_get_areas(const crg_regridder* r, double* dst_areas, double* src_areas);

/* Kahan-summed row sums (length n_dst) and column sums (length n_src) of A:
 * the quantities the reference's area-agreement test compares with the cell
 * areas (lib/ConservativeRegriddingTestHelpers/src/ConservativeRegriddingTestHelpers.jl:70-73).
 * Computed on the first call (or the first crg_get_esmf_weights), not by the
 * build; thread-safe. */
crg_status crg_get_row_col_sums(const crg_regridder* r, double* row_sums, double* col_sums);

/* ------------------------------------------------------------------------
 * Spectral-element (SE) <-> finite-volume (FV) regridders on the sphere, the
 * ClimaCore extension of the reference (ext/ConservativeRegriddingClimaCoreExt.jl).
 *
 * An SE space is a set of quadrilateral elements with nq x nq Gauss-Lobatto-
 * Legendre (GLL) nodes each.  Element e maps the reference square (xi, eta) in
 * [-1, 1]^2 onto the sphere by the normalised bilinear map of its corners
 * (vertex k of the element at reference corner k: (-1,-1), (1,-1), (1,1),
 * (-1,1)); its edges are great-circle arcs.  Node (e, i, j) -- xi = x_i,
 * eta = x_j, i fastest -- is entry e * nq^2 + i + j * nq of an SE field
 * (ClimaCore's flattened nodal order, se_field_to_vec :368-370).
 * ------------------------------------------------------------------------ */
typedef struct crg_se_space {
    crg_grid_desc elements;      /* spherical quadrilaterals (curvilinear blocks or 4-vertex cells) */
    int32_t nq;                  /* GLL nodes per direction (ClimaCore n_quad_points), 2..8 */
    int32_t pad;
    const double* node_weights;  /* [nelem * nq * nq] weighted Jacobian W = J w_i w_j of every node
                                    (Spaces.weighted_jacobian, se_node_weights :153-156), host or device;
                                    NULL = computed from the element map on a sphere of opts->radius */
} crg_se_space;

typedef struct crg_se_opts {
    int32_t triangle_quad_degree;  /* degree of the Dunavant triangle rule for the overlap integrals,
                                      1..8; 0 = 2 (nq - 1), the reference's default (:434, :583) */
    int32_t flags;                 /* reserved, must be 0 */
    double radius;                 /* sphere radius: areas and computed node weights scale by radius^2;
                                      0 = 1 (the unit sphere) */
    void* stream;                  /* cudaStream_t of the build; NULL = legacy default stream */
} crg_se_opts;

/* SE source -> FV destination, the "principled" weights (se_to_fv_principled,
 * :416-486, accumulate_principled_b :260-305): A[k, (e,i,j)] = integral over cell k ∩ element e of phi_i(xi) phi_j(eta),
 * by fan triangulation of each overlap from its normalised vertex mean and a
 * Dunavant rule on every triangle, (xi, eta) from the inverse element map.
 * dst_areas = the FV cell areas, src_areas = the node weights; not normalised.
 * regrid! then gives d = (A s) ./ a_d; constants are preserved exactly up to
 * rounding.  Errors: CRG_ERR_INVALID_ARGUMENT for a non-spherical grid, an
 * element without 4 vertices, nq outside 2..8 or a rule degree above 8;
 * CRG_ERR_NOT_SUPPORTED for 2^31 nodes or more and for 2^26 overlapping
 * (element, cell) pairs or more (32-bit counts). */
crg_status crg_build_se_to_fv(const crg_grid_desc* dst, const crg_se_space* src, const crg_se_opts* opts,
                              crg_regridder** out);

/* FV source -> SE destination, the per-element L2 projection
 * (fv_to_se_l2_projection :573-689, compute_local_mass_matrix :522-560): the same overlap integrals b(e, k) per
 * element and cell, then per element the local mass matrix M^e (GLL rule of
 * ceil((3 nq - 2) / 2) + 1 points, Jacobian interpolated from the node
 * weights) restricted to the nodes with nonzero total b, each of its rows
 * scaled to that total, inverted (Gauss-Jordan, partial pivoting) and applied
 * to every cell's b.  dst_areas = ones, src_areas = the FV cell areas.  Like
 * the reference's regrid! into a ClimaCore field, follow the apply by
 * crg_se_dss to make shared nodes agree.  CRG_ERR_GEOMETRY if a local mass
 * matrix is singular. */
crg_status crg_build_fv_to_se(const crg_se_space* dst, const crg_grid_desc* src, const crg_se_opts* opts,
                              crg_regridder** out);

/* Positions (unit vectors, [nnodes][3]) and weighted Jacobians ([nnodes]) of
 * all nodes of an SE space (se_node_positions / se_node_weights, :139-156);
 * either output may be NULL; host or device pointers. */
crg_status crg_se_nodes(const crg_se_space* space, const crg_se_opts* opts, double* points, double* weights);

/* Weighted direct stiffness summation (ClimaCore Spaces.weighted_dss!, the
 * finalize step of regrid! into an SE field, :709-715): every group of node
 * copies that are the same point gets the weighted mean
 * sum(w_n f_n) / sum(w_n) of its copies, for every field.  Groups are
 * group_nodes[group_ptr[g] .. group_ptr[g+1]) (device memory, ascending node
 * numbers), w = the node weights (device memory); the field is
 * (nodes, fields) with the given strides, on `stream`. */
crg_status crg_se_dss(int32_t dtype, void* field, int64_t stride_node, int64_t stride_field, int64_t nfields,
                      const int32_t* group_ptr, const int32_t* group_nodes, const double* weights, int64_t ngroups,
                      void* stream);

const char* crg_last_error(void);
const char* crg_status_string(crg_status s);
int32_t crg_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CRG_H */
