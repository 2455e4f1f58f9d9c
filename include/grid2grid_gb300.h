/*
 * grid2grid_gb300 -- C ABI of the GB300-native grid2grid transform path.
 *
 * A matrix is split into a grid of blocks (grid2D: rows_split, cols_split);
 * every block is owned by one rank (assigned_grid2D: ranks[i][j]) and stored
 * column-major at an arbitrary pointer with an arbitrary stride (block<T>).
 * A transform redistributes the matrix from an initial layout into a final
 * layout:  final = beta * final + alpha * op(initial),  op in {N, T, C}.
 *
 * On one GPU the P ranks of a layout are *virtual ranks*: every rank's local
 * blocks live in the same device memory, so a layout descriptor carries the
 * local blocks of all ranks at once, each tagged with its rank. The
 * reference's pack / MPI exchange / unpack collapses into one device
 * gather-scatter over a work list that the device builds from the grid cover.
 *
 * Conventions
 *  - Every function returns a g2g_status; on failure a human-readable message
 *    is available from g2g_last_error_string() (thread-local).
 *  - Pointers in g2g_block_desc.data are DEVICE addresses owned by the caller,
 *    or addresses in PINNED host memory (cudaHostAlloc / cudaHostRegister),
 *    which the gather-scatter then reads or writes in place over the host
 *    link. Pageable host memory is refused (G2G_ERROR_INVALID_ARGUMENT).
 *    The library never frees them and never touches a destination block's
 *    padding (rows < stride).
 *  - A `stream` argument is a cudaStream_t passed as void* (NULL = legacy
 *    default stream). All device work is stream-ordered.
 *  - No function takes or returns a framework (torch/numpy) type.
 *
 * Reference interfaces replaced (paths inside kabicm/grid2grid):
 *  - grid2grid::transform, 4 overloads           src/grid2grid/transform.hpp:13-43
 *  - grid2grid::transformer<T>                    src/grid2grid/transformer.hpp:8-62
 *  - grid2grid::grid_cover / get_decomp_cover     src/grid2grid/grid_cover.hpp:38-65,
 *                                                 src/grid2grid/grid_cover.cpp:54-121
 *  - grid_layout / assigned_grid2D / block<T>     src/grid2grid/grid_layout.hpp:7-63,
 *                                                 src/grid2grid/grid2D.hpp:46-125,
 *                                                 src/grid2grid/block.hpp:60-190
 *  - communication_volume, optimal_reordering     src/grid2grid/transform.cpp:9-39,
 *                                                 src/grid2grid/ranks_reordering.cpp:4-61
 *  - get_scalapack_grid (as a ScaLAPACK front end) src/grid2grid/scalapack_layout.cpp:152-278
 */
#ifndef GRID2GRID_GB300_H
#define GRID2GRID_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define G2G_VERSION_MAJOR 0
#define G2G_VERSION_MINOR 1

/* Status codes replace the reference's exceptions (std::runtime_error from
 * interval.cpp:5-17, grid2D.cpp:29-43, block.cpp:167-174,
 * grid_cover.hpp:57-62, scalapack_layout.cpp:12-15,43-48) and its asserts
 * (communication_data.cpp:227-239, grid_cover.cpp:70). */
typedef enum g2g_status {
    G2G_SUCCESS = 0,
    G2G_ERROR_INVALID_ARGUMENT = 1, /* descriptor violates a layout invariant   */
    G2G_ERROR_CUDA = 2,             /* a CUDA runtime call failed               */
    G2G_ERROR_OUT_OF_MEMORY = 3,    /* device allocation for plan metadata      */
    G2G_ERROR_BUDGET = 4,           /* request exceeds the server's HBM budget  */
    G2G_ERROR_TIMEOUT = 5,          /* a bounded wait expired                   */
    G2G_ERROR_NOT_READY = 6,        /* asynchronous result not available yet    */
    G2G_ERROR_UNSUPPORTED = 7       /* valid request this build cannot serve    */
} g2g_status;

/* The four element types the reference instantiates (transform.cpp:206-298,
 * mpi_type_wrapper.hpp:9-70). Complex types are {real, imag} pairs, the
 * layout of std::complex<float> / std::complex<double>. */
typedef enum g2g_dtype {
    G2G_FLOAT32 = 0,    /* float                 4 bytes */
    G2G_FLOAT64 = 1,    /* double                8 bytes */
    G2G_COMPLEX64 = 2,  /* std::complex<float>   8 bytes */
    G2G_COMPLEX128 = 3  /* std::complex<double> 16 bytes */
} g2g_dtype;

/* One locally stored block (block<T>, block.hpp:60-146). Its row and column
 * intervals are the grid's intervals at (row, col). With transpose_on_copy
 * set, the grid coordinates are those of the (already transposed) layout and
 * the memory holds the un-transposed block, exactly as block<T> after
 * transpose_or_conjugate (block.cpp:249-288). */
typedef struct g2g_block_desc {
    int32_t rank;              /* virtual rank whose local_blocks hold it   */
    int32_t row;               /* block_coordinates::row                    */
    int32_t col;               /* block_coordinates::col                    */
    int32_t transpose_on_copy; /* block<T>::transpose_on_copy (0/1)         */
    int32_t conjugate_on_copy; /* block<T>::conjugate_on_copy (0/1)         */
    int32_t reserved;
    int64_t stride;            /* leading dimension in elements             */
    void *data;                /* address of element (0,0): device or pinned host */
} g2g_block_desc;

/* A grid_layout over P virtual ranks (grid_layout.hpp:7-63): the grid, the
 * owner matrix (with optional rank reordering, grid2D.cpp:112-122) and the
 * local blocks of ALL ranks. */
typedef struct g2g_layout_desc {
    int32_t n_block_rows;       /* grid2D::n_rows (number of row intervals)  */
    int32_t n_block_cols;       /* grid2D::n_cols                            */
    const int32_t *rows_split;  /* n_block_rows + 1 non-decreasing entries   */
    const int32_t *cols_split;  /* n_block_cols + 1 non-decreasing entries   */
    const int32_t *owners;      /* row-major n_block_rows x n_block_cols:
                                   owners[i*n_block_cols + j] = ranks[i][j]  */
    int32_t n_ranks;            /* assigned_grid2D::num_ranks()              */
    int32_t n_reordering;       /* 0, or number of entries in `reordering`   */
    const int32_t *reordering;  /* owner(i,j) = reordering[ranks[i][j]]      */
    int32_t n_blocks;           /* local blocks over all virtual ranks       */
    int32_t reserved;
    const g2g_block_desc *blocks;
} g2g_layout_desc;

/* The (trans, alpha, beta) of transform.hpp:20-25. alpha/beta are given as
 * {real, imag} doubles and converted to the element type (the imaginary part
 * must be 0 for real types). (alpha, beta) == (1, 0) is a pure bit copy, as
 * in memory_utils.hpp:92-95. trans is 'N', 'T' or 'C' (any case); 'T'/'C'
 * transpose the initial layout first (grid_layout.hpp:18-25); the caller's
 * descriptor is not modified. */
typedef struct g2g_op {
    char trans;
    char reserved[7];
    double alpha[2];
    double beta[2];
} g2g_op;

/* Knobs of the gather-scatter kernels. Zero fields mean "library default".
 * g2g_plan_autotune picks them by measurement. */
typedef struct g2g_tuning {
    int32_t tile_bytes;       /* target bytes per non-transposed tile       */
    int32_t tile_dim;         /* edge (elements) of a transposed tile: 16 or 32 */
    int32_t ctas_per_sm;      /* persistent grid = ctas_per_sm x SM count   */
    int32_t threads;          /* threads per CTA: 256 or 512                */
    int32_t unroll;           /* 16-byte chunks per lane and step: 1, 2 or 4 */
    int32_t stages;           /* plain copies: -1 = not TMA-staged,
                                 2..4 = TMA bulk copies into a ring of that
                                 many shared-memory stages (0 = default)    */
    int32_t ring;             /* plain copies when not TMA-staged: 1 = per-warp
                                 cp.async ring in shared memory, -1 = loads
                                 through registers (0 = default). Launches of
                                 transposes of one element size only (plain,
                                 or scaled 4- or 8-byte ones): 1 = their
                                 staged cp.async ring, -1 = the register path */
    int32_t tile_run;         /* ring: a warp takes runs of this many
                                 consecutive tiles (1, 2, 4 .. 64; 0 = default) */
    int32_t l2_prefetch;      /* ring: 1 = a warp entering a tile asks L2 for
                                 the tile's source columns in bulk, -1 = no
                                 (0 = default: no)                          */
    int32_t tensor_boxes;     /* plain copies of a plan whose blocks are
                                 16-byte aligned with 16-byte multiple strides
                                 and whose pieces are whole boxes of one shape
                                 (e.g. block-cyclic to block-cyclic): 1 = move
                                 them as 2-D TMA boxes through tensor maps,
                                 -1 = no (0 = default: no); ignored when the
                                 plan does not qualify                      */
} g2g_tuning;

typedef struct g2g_plan_info {
    int32_t n_pairs;          /* layout pairs in the plan                    */
    int32_t n_ranks;          /* largest virtual-rank count over the pairs   */
    int64_t n_pieces;         /* non-empty (initial block x final block) pieces */
    int64_t n_tiles;          /* work items of the gather-scatter kernel     */
    int64_t bytes_moved;      /* sum of m*n*sizeof(T) over the pairs         */
    int64_t bytes_min_traffic;/* 2x bytes_moved (3x for pieces with beta!=0) */
    int64_t metadata_bytes;   /* device memory held by the plan              */
    int32_t graph_captured;   /* 1 after g2g_plan_capture_graph              */
    int32_t device_status;    /* 0, or the error a kernel of the plan raised
                                 (1 = a bounded wait expired); reading it
                                 synchronises with the plan's last execution */
    int32_t tensor_boxes_ok;  /* 1 if the plan qualifies for tensor_boxes    */
    int32_t tile_paths;       /* tile kinds of the work list: 1 copy, 2 transpose,
                                 4 scaled real, 8 scaled complex, 16 cast,
                                 32 transposes of 4- or 8-byte elements,
                                 64 / 128 / 256 transposes of 4- / 8- /
                                 16-byte elements only (they run on the
                                 staged cp.async ring when no copy tiles
                                 come with them, the
                                 tuning's ring is not -1 and no block is in
                                 host memory), 1024 / 2048 scaled transposes
                                 of 4- / 8-byte elements only (their staged
                                 ring, on the same conditions)                */
    g2g_tuning tuning;        /* knobs in effect                             */
} g2g_plan_info;

typedef struct g2g_plan g2g_plan;

/* ---- errors and version ------------------------------------------------ */
const char *g2g_last_error_string(void);
const char *g2g_version_string(void);

/* ---- planning ---------------------------------------------------------- */

/* Plans one transform (transform.hpp:13-25; utils::prepare_to_send/recv,
 * utils.hpp:146-212). Host side: validates both descriptors and builds the
 * per-layout block tables. Device side (stream-ordered, no host sync): the
 * grid cover by a parallel merge of the split vectors, per-block piece counts,
 * a scan, and the emission of the piece and tile work lists. `op` may be NULL
 * (= 'N', 1, 0). */
g2g_status g2g_plan_create(const g2g_layout_desc *initial,
                           const g2g_layout_desc *final_,
                           g2g_dtype dtype, const g2g_op *op,
                           void *stream, g2g_plan **plan);

/* Plans n_pairs transforms executed together, the vector overloads
 * (transform.hpp:30-43) and transformer<T>::transform (transformer.hpp:44-53).
 * Unlike the reference, each pair may have its own dtype. ops may be NULL.
 * Destinations of different pairs must not overlap. */
g2g_status g2g_plan_create_batch(int32_t n_pairs,
                                 const g2g_layout_desc *initials,
                                 const g2g_layout_desc *finals,
                                 const g2g_dtype *dtypes, const g2g_op *ops,
                                 void *stream, g2g_plan **plan);

/* Runs the plan's gather-scatter on `stream` (exchange_async,
 * transform.cpp:41-124, as one kernel). Replays the captured graph if
 * g2g_plan_capture_graph was called. */
g2g_status g2g_plan_execute(g2g_plan *plan, void *stream);

/* Executes several plans as ONE launch of the persistent gather-scatter
 * (the concatenation of their work lists; up to 256 plans per launch, more
 * are split into further launches; cast plans, from g2g_plan_create_cast,
 * launch apart from the others). Plans must live on one device and their
 * destinations must not overlap. Used for continuous batching of cached
 * plans. */
g2g_status g2g_plans_execute(int32_t n_plans, g2g_plan *const *plans, void *stream);

/* Captures one execution into a CUDA graph; later executes replay it. */
g2g_status g2g_plan_capture_graph(g2g_plan *plan, void *stream);

g2g_status g2g_plan_set_tuning(g2g_plan *plan, const g2g_tuning *tuning);

/* Times candidate tunings on `stream` (each executes the plan, so the
 * destination is written) and keeps the fastest; *best may be NULL. */
g2g_status g2g_plan_autotune(g2g_plan *plan, void *stream, int32_t iters,
                             g2g_tuning *best);

g2g_status g2g_plan_get_info(const g2g_plan *plan, g2g_plan_info *info);

/* Frees the plan's device metadata after work queued on the plan's last
 * stream has finished (stream-ordered free). */
g2g_status g2g_plan_destroy(g2g_plan *plan);

/* ---- fused dtype cast (beyond the reference) --------------------------- */

/* A transform that converts the element type on the way:
 * final = convert(op(initial)), the initial layout holding src_dtype
 * elements and the final one dst_dtype elements. Supported: float <-> double
 * and complex<float> <-> complex<double> (each part rounded to nearest even),
 * real -> complex (imaginary part +0); complex -> real is
 * G2G_ERROR_UNSUPPORTED. op: trans 'N', 'T' or 'C' ('C' conjugates after the
 * conversion); alpha and beta must be 1 and 0 (op may be NULL). The reference
 * has no such operation; results are checked against numpy's conversions. */
g2g_status g2g_plan_create_cast(const g2g_layout_desc *initial, g2g_dtype src_dtype,
                                const g2g_layout_desc *final_, g2g_dtype dst_dtype,
                                const g2g_op *op, void *stream, g2g_plan **plan);

/* Plans, executes and destroys a cast transform; returns after completion. */
g2g_status g2g_transform_cast(const g2g_layout_desc *initial, g2g_dtype src_dtype,
                              const g2g_layout_desc *final_, g2g_dtype dst_dtype,
                              const g2g_op *op, void *stream);

/* ---- one-shot transform ------------------------------------------------ */

/* plan + execute, returning after the transform completed: the reference's
 * blocking transform() call (transform.cpp:126-164). The reference re-plans
 * on every call; here plans are cached, keyed by a 128-bit signature of the
 * descriptors, dtype and op (at most G2G_PLAN_CACHE_ENTRIES plans, default
 * 64, 0 = plan and free on every call). A cached plan holds device metadata
 * only, never the caller's buffers. */
g2g_status g2g_transform(const g2g_layout_desc *initial,
                         const g2g_layout_desc *final_, g2g_dtype dtype,
                         const g2g_op *op, void *stream);

g2g_status g2g_transform_batch(int32_t n_pairs,
                               const g2g_layout_desc *initials,
                               const g2g_layout_desc *finals,
                               const g2g_dtype *dtypes, const g2g_op *ops,
                               void *stream);

/* The one-shot transform of g2g_transform for callers that cannot allocate
 * device memory (an application that gives all of HBM to its own pool and
 * forbids other allocations, a process under a strict memory quota, a
 * latency-critical loop that cannot take cudaFree's implicit device
 * synchronisation). No counterpart in the reference. It calls no CUDA or
 * library allocation routine: plan metadata and the work list live in a
 * fixed 32 MiB device array inside the library, held on every GPU where the
 * library's device code is loaded until the process exits. Limits: a
 * transform needing more metadata than the array holds is rejected with
 * G2G_ERROR_OUT_OF_MEMORY before any device work; all calls share the array,
 * so calls that overlap on the GPU race (the call synchronises `stream` and
 * returns after its transform has completed; issue calls one at a time per
 * device). The first call on a device resolves the array's address. One
 * dtype and op as in g2g_transform; `op` may be NULL. */
g2g_status g2g_transform_noalloc(const g2g_layout_desc *initial,
                                 const g2g_layout_desc *final_, g2g_dtype dtype,
                                 const g2g_op *op, void *stream);

/* Frees every cached plan of g2g_transform / g2g_transform_batch that no
 * call is using. */
g2g_status g2g_plan_cache_clear(void);

/* ---- grid cover -------------------------------------------------------- */

/* grid_cover of two split vectors (get_decomp_cover, grid_cover.cpp:54-121),
 * computed on the device by a parallel merge. Host arrays in and out:
 * for k in [0, n_a-1): start_index[k] = max i with b[i] <= a[k],
 * end_index[k] = min i with b[i] >= a[k+1]. Requires a[0] == b[0] and
 * a[n_a-1] == b[n_b-1]. Synchronises `stream`. */
g2g_status g2g_grid_cover(const int32_t *splits_a, int32_t n_a,
                          const int32_t *splits_b, int32_t n_b,
                          int32_t *start_index, int32_t *end_index,
                          void *stream);

/* ---- rank reordering --------------------------------------------------- */

/* communication_volume (transform.cpp:9-39): the elements each pair of
 * virtual ranks exchanges in a transform from `initial` to `final_`, owners
 * taken through the layouts' reorderings (grid2D.cpp:116-122). `volume` is
 * an n_ranks x n_ranks row-major array: entry [r*n_ranks + s], r <= s, holds
 * the elements moved between r and s (r == s: elements that stay on r);
 * entries below the diagonal are 0. Only splits and owners are read (no
 * blocks, no device work). n_ranks must cover every owner. */
g2g_status g2g_communication_volume(const g2g_layout_desc *initial,
                                    const g2g_layout_desc *final_, int32_t n_ranks,
                                    int64_t *volume);

/* optimal_reordering (ranks_reordering.cpp:4-61): a greedy matching on the
 * volumes that relabels ranks so that more data stays local. Edge r-s weighs
 * vol(r,s) - vol(r,r) - vol(s,s) (a rank kept where it is weighs 1); edges
 * are taken by decreasing weight, each rank in at most one, and a taken edge
 * r-s swaps r and s. Ties are taken in (r, s) order. permutation[r] is r's
 * new label; *reordered = 1 if it is not the identity. */
g2g_status g2g_optimal_reordering(const int64_t *volume, int32_t n_ranks,
                                  int32_t *permutation, int32_t *reordered);

/* The two functions above computed on the device, where a sharded
 * transform keeps its data, to pick the rank-to-GPU map
 * (transform.cpp:9-39, ranks_reordering.cpp:4-61). `volume` is a DEVICE
 * array of n_ranks x n_ranks int64 (the layout of g2g_communication_volume),
 * `permutation` a DEVICE array of n_ranks int32 and `reordered` a DEVICE
 * int32; both calls are asynchronous on `stream` and give the same results
 * as the host functions. The matching runs as the locally dominant
 * matching (every free rank points at its best edge, mutual choices are
 * matched, repeated), which under the same strict edge order -- weight,
 * then (r, s) -- is the greedy matching. */
g2g_status g2g_communication_volume_device(const g2g_layout_desc *initial,
                                           const g2g_layout_desc *final_, int32_t n_ranks,
                                           int64_t *volume, void *stream);
g2g_status g2g_optimal_reordering_device(const int64_t *volume, int32_t n_ranks,
                                         int32_t *permutation, int32_t *reordered,
                                         void *stream);

/* ---- ScaLAPACK-descriptor front end ------------------------------------ */

/* A block-cyclic matrix as a ScaLAPACK array descriptor describes it
 * (M_, N_, MB_, NB_, RSRC_, CSRC_), over an nprow x npcol grid of virtual
 * ranks. The local leading dimensions (LLD_) are passed per rank. */
typedef struct g2g_scalapack_desc {
    int32_t m, n;         /* global rows, columns                              */
    int32_t mb, nb;       /* rows, columns of a block                          */
    int32_t rsrc, csrc;   /* process row, column holding the first block       */
    int32_t nprow, npcol; /* process grid                                      */
    int32_t row_major;    /* rank = prow*npcol + pcol (1) or pcol*nprow + prow (0) */
    int32_t reserved;
} g2g_scalapack_desc;

/* A layout built by the library; it owns the arrays its descriptor points to. */
typedef struct g2g_layout g2g_layout;

/* The layout of the submatrix A(ia:ia+m-1, ja:ja+n-1) (1-based, as in
 * ScaLAPACK) of the block-cyclic matrix `desc`, rank r's local array at
 * DEVICE address rank_data[r] with leading dimension lld[r] elements
 * (lld == NULL: the rank's local block rows x mb, the reference's default).
 * Same grid, owners, local offsets and strides as get_scalapack_grid
 * (scalapack_layout.cpp:178-278) for every rank. m == 0 or n == 0 is an
 * empty layout. Host only: nothing is read from rank_data. */
g2g_status g2g_layout_create_scalapack(const g2g_scalapack_desc *desc, int32_t ia,
                                       int32_t ja, int32_t m, int32_t n,
                                       void *const *rank_data, const int32_t *lld,
                                       g2g_dtype dtype, g2g_layout **layout);

/* Points *out at the layout's arrays (valid until g2g_layout_destroy). */
g2g_status g2g_layout_get_desc(const g2g_layout *layout, g2g_layout_desc *out);

g2g_status g2g_layout_destroy(g2g_layout *layout);

/* p?gemr2d on one GPU: sub(B) = sub(A) between two block-cyclic
 * distributions, sub(A) = A(ia:ia+m-1, ja:ja+n-1) and sub(B) =
 * B(ib:ib+m-1, jb:jb+n-1); with `op`, sub(B) = beta*sub(B) + alpha*op(sub(A))
 * where sub(A) is n x m for 'T' / 'C'. Builds both layouts and runs the
 * one-shot transform (plans cached, returns after completion). */
g2g_status g2g_gemr2d(int32_t m, int32_t n,
                      void *const *a_data, int32_t ia, int32_t ja,
                      const g2g_scalapack_desc *desc_a, const int32_t *lld_a,
                      void *const *b_data, int32_t ib, int32_t jb,
                      const g2g_scalapack_desc *desc_b, const int32_t *lld_b,
                      g2g_dtype dtype, const g2g_op *op, void *stream);

/* ---- sharded transform: virtual ranks spread over several GPUs --------- */

/* A transform whose virtual ranks are spread over several GPUs (shards), one
 * process per GPU, each holding the blocks of its ranks: the reference's
 * exchange between ranks (exchange_async, transform.cpp:41-124, driven by
 * communication_data, communication_data.cpp:51-99) with a GPU in place of
 * an MPI rank. Every shard's process calls these functions with the same
 * grids, owners, dtype, op and rank-to-shard map, and descriptors that list
 * exactly the blocks of its own ranks (blocks of other shards' ranks are not
 * listed). A shard's part is:
 *   g2g_exchange_pack    local pieces (source and destination rank on this
 *                        shard) straight into their destination blocks, and
 *                        pieces bound for other shards, op applied, into the
 *                        send buffer -- one launch;
 *   (the caller exchanges the buffers: an all-to-all with the per-shard byte
 *    counts of g2g_exchange_get_counts, e.g. NCCL);
 *   g2g_exchange_unpack  received pieces into their destination blocks,
 *                        alpha/beta applied.
 * Buffer layout: the section for (or from) shard h starts at the sum of the
 * byte counts of shards 0..h-1. Inside a section, for each source rank and
 * then each destination rank (ascending), the pieces between them in the
 * order of the reference's message sort (column interval, then row
 * interval; communication_data.cpp:26-30), each packed column-major with its
 * rows as leading dimension in final orientation: a (source rank,
 * destination rank) segment holds what the reference's rank sends to the
 * other in its own buffer. */
typedef struct g2g_exchange g2g_exchange;

enum { G2G_EXCHANGE_LOCAL = 0, G2G_EXCHANGE_SEND = 1, G2G_EXCHANGE_RECV = 2 };

/* One piece of a shard's part: a cell of the grid cover (both grids' split
 * points merged), in final coordinates. */
typedef struct g2g_exchange_piece {
    int32_t row_start, row_end;  /* [row_start, row_end)                        */
    int32_t col_start, col_end;  /* [col_start, col_end)                        */
    int32_t src_rank, dst_rank;  /* owner in the initial (after op) / final grid */
    int64_t offset;              /* elements from the start of the shard's send
                                    or receive buffer; -1 for local pieces      */
} g2g_exchange_piece;

/* Plans shard `shard`'s part of a transform over n_shards shards.
 * shard_of_rank has one entry per virtual rank (max of both layouts'
 * n_ranks). Host only: validates the descriptors, computes the grid cover,
 * the piece lists and counts; no device work. */
g2g_status g2g_exchange_create(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                               g2g_dtype dtype, const g2g_op *op, int32_t n_shards,
                               const int32_t *shard_of_rank, int32_t shard,
                               g2g_exchange **ex);

/* Bytes this shard sends to / receives from each shard (n_shards entries
 * each; the shard's own entries are 0). Either pointer may be NULL. */
g2g_status g2g_exchange_get_counts(const g2g_exchange *ex, int64_t *send_bytes,
                                   int64_t *recv_bytes);

/* Elements each virtual rank sends to each other one, over the whole
 * transform (n_ranks x n_ranks, row-major: counts[s*n_ranks + d]; the
 * diagonal holds the elements that stay on a rank). Row s, diagonal set to
 * zero, is the reference's communication_data send counts of rank s
 * (communication_data.cpp:51-99), column d its receive counts of rank d. */
g2g_status g2g_exchange_get_rank_counts(const g2g_exchange *ex, int32_t n_ranks,
                                        int64_t *counts);

/* The local, send or receive pieces (G2G_EXCHANGE_*) of this shard, in
 * buffer order. pieces may be NULL to ask for the number only. */
g2g_status g2g_exchange_get_pieces(const g2g_exchange *ex, int32_t which, int64_t capacity,
                                   g2g_exchange_piece *pieces, int64_t *n_pieces);

/* Binds the device send and receive buffers (at least the sum of the send /
 * receive byte counts each, element aligned) and plans the local, pack and
 * unpack gather-scatters on the device. Rebinding replaces the plans. */
g2g_status g2g_exchange_bind(g2g_exchange *ex, void *send_buffer, void *recv_buffer,
                             void *stream);

g2g_status g2g_exchange_pack(g2g_exchange *ex, void *stream);
g2g_status g2g_exchange_unpack(g2g_exchange *ex, void *stream);

/* Plan info of the local, pack (G2G_EXCHANGE_SEND) or unpack
 * (G2G_EXCHANGE_RECV) gather-scatter; all zero when it has no pieces. */
g2g_status g2g_exchange_get_plan_info(const g2g_exchange *ex, int32_t which,
                                      g2g_plan_info *info);

g2g_status g2g_exchange_destroy(g2g_exchange *ex);

/* ---- serving: continuous batching ------------------------------------- */

/* A request loop for transforms of device-resident layouts (no counterpart
 * in the reference, which serves one collective call at a time). Requests
 * are queued by g2g_server_submit and admitted while the bytes of admitted,
 * unfinished requests (source + destination) stay within the HBM budget;
 * a dispatcher thread launches all admissible queued requests as ONE launch
 * (g2g_plans_execute over their cached plans) on one of several streams, so
 * requests that arrive while others are on the GPU start as soon as a
 * launch slot and budget free up and overlap with them on the device. */
typedef struct g2g_server g2g_server;

typedef struct g2g_server_config {
    int64_t hbm_budget_bytes;      /* admission budget (0 = 120 GB)              */
    int32_t max_launches_in_flight;/* concurrent launches / streams (0 = 3)      */
    int32_t max_batch_requests;    /* requests per launch, 1..256 (0 = 256);
                                      1 gives plain per-request launches        */
    int32_t plan_cache_entries;    /* cached plans (0 = 4096)                    */
    int32_t reserved[3];
} g2g_server_config;

typedef struct g2g_request_times {
    int64_t submit_ns;    /* steady clock, when the request was queued   */
    int64_t launch_ns;    /* when its launch was issued                  */
    int64_t complete_ns;  /* when its launch was seen complete           */
    int64_t bytes;        /* m*n*sizeof(T) of the request                */
    int32_t status;       /* g2g_status of the request                   */
    int32_t batch_size;   /* requests in the launch that carried it      */
} g2g_request_times;

typedef struct g2g_server_stats {
    int64_t submitted, completed, launches, plan_cache_hits, plan_cache_misses;
    int64_t bytes_completed;
    int64_t inflight_bytes_peak;
} g2g_server_stats;

/* Creates the server on the current device and loads every gather-scatter
 * kernel instance a launch can select there, so that no request waits for a
 * lazily loaded module. */
g2g_status g2g_server_create(const g2g_server_config *config, g2g_server **server);

/* Queues a transform; *ticket identifies it. Fails with G2G_ERROR_BUDGET if
 * the request alone exceeds the budget. Planning happens here (cached). */
g2g_status g2g_server_submit(g2g_server *server, const g2g_layout_desc *initial,
                             const g2g_layout_desc *final_, g2g_dtype dtype,
                             const g2g_op *op, uint64_t *ticket);

/* Waits up to timeout_us (< 0: forever) for a request; G2G_ERROR_NOT_READY if
 * it is still pending. `times` may be NULL. A finished ticket is released
 * by this call. */
g2g_status g2g_server_wait(g2g_server *server, uint64_t ticket, int64_t timeout_us,
                           g2g_request_times *times);

/* Open-loop replay: submits request k (pair pair_index[k] of the given
 * layout pairs) at arrival_s[k] seconds after the call starts, from a native
 * thread, then waits for all and fills times[k]. */
g2g_status g2g_server_replay(g2g_server *server, int32_t n_pairs,
                             const g2g_layout_desc *initials,
                             const g2g_layout_desc *finals, const g2g_dtype *dtypes,
                             const g2g_op *ops, int64_t n_requests,
                             const int32_t *pair_index, const double *arrival_s,
                             g2g_request_times *times);

g2g_status g2g_server_get_stats(const g2g_server *server, g2g_server_stats *stats);

/* Finishes every queued request, then frees the server and its plans. */
g2g_status g2g_server_destroy(g2g_server *server);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* GRID2GRID_GB300_H */
