/*
 * pbig2.h — C ABI of the GB300 pairwise box-intersection engine.
 *
 * Plain pointers and sizes only; no C++ or torch types. Every entry point
 * returns a pbig2_status; pbig2_last_error() gives a message for the last
 * failure on the calling thread.
 *
 * Boxes use PBIG's RectInfo layout (rect.h): per box 2*dims+1 unsigned ints
 * {xmin,xmax,ymin,ymax[,zmin,zmax],rid}, rid equal to the box's index in its
 * scene, every coordinate < range, min <= max. Two boxes overlap when their
 * closed intervals intersect on every axis (touching faces count); a box
 * never pairs with itself. Each overlapping pair is reported once.
 *
 * Reference interfaces replaced (paths in the awatch/pbig project):
 *   pbig2_self_intersect    <- void pbig_check(RectInfo*, report*)
 *                              src/pbig/pbig.h:10, src/pbig/pbig.cu:1962
 *   pbig2_create/destroy    <- pbig_init / pbig_finalize
 *                              src/pbig/pbig.h:9,11, src/pbig/pbig.cu:2139,141
 *   pairs in device memory  <- the per-batch output stream + decode()
 *                              src/pbig/pbig.cu:1694-1960, src/pbig/decode.cc:26
 */
#ifndef PBIG2_H_
#define PBIG2_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define PBIG2_API __attribute__((visibility("default")))
#else
#define PBIG2_API
#endif

typedef enum {
    PBIG2_OK = 0,
    PBIG2_EINVAL = 1,    /* bad argument (null pointer, dims, sizes) */
    PBIG2_ENOMEM = 2,    /* device or pinned allocation failed */
    PBIG2_ECUDA = 3,     /* CUDA runtime error */
    PBIG2_EINPUT = 4,    /* some boxes violate the input contract; they were
                            skipped and the pairs of the others reported */
    PBIG2_ETIMEOUT = 5,  /* a bounded device wait gave up */
    PBIG2_ECAPACITY = 6, /* caller buffer too small; *count holds the need */
    PBIG2_EBUSY = 7      /* serving queue full / admission refused */
} pbig2_status;

/* memory location flags for input/output buffers */
#define PBIG2_HOST 0
#define PBIG2_DEVICE 1

typedef struct pbig2_ctx pbig2_ctx;

/* Statistics of the last query on a context (all counts exact). */
typedef struct {
    uint64_t boxes;        /* boxes in the query */
    uint64_t bad_boxes;    /* boxes rejected by the input contract */
    uint64_t cells;        /* grid cells (sum over scenes) */
    uint64_t entries;      /* cell entries E (box-in-cell records) */
    uint64_t pair_tests;   /* sum over cells of n(n-1)/2 */
    uint64_t pairs;        /* overlapping pairs reported */
    uint32_t cell_shift;   /* log2(cell size) of the (first) scene */
    uint32_t scenes;
    uint32_t kernels;      /* kernel launches of the query */
    uint32_t grid_retries; /* automatic cell size: passes rerun on a coarser
                              grid because a box outside the tuner's sample
                              covered 2^26 cells or more */
    double device_ms;      /* device time of the query (CUDA events) */
    /* device time per phase of the last pipeline pass (CUDA events on the
     * query's stream): count, scan, expand, scatter, pair test (all three
     * pair kernels), grouping by scene, and within the pair test: the
     * small-cell, medium-cell and block kernels */
    double phase_ms[9];
    /* the reference's own work statistics for the same grid (sched_phase,
     * src/pbig/pbig.cu:1586-1688): numCompPairs = sum of n*n/2, jobs = sum
     * of ceil(n/256), over the cells -- or merged blocks -- of n >= 2 boxes;
     * max_cell = the largest of them; merged_blocks = merged blocks of two
     * or more cells (merged mode) */
    uint64_t comp_pairs;
    uint64_t jobs;
    uint32_t max_cell;
    uint32_t merged_blocks;
    /* the class map the query used (PBIG2_OPT_CLASS_MAP) and the merged
     * mode's block limit (PBIG2_OPT_MERGE_LIMIT) */
    uint64_t class_map;
    uint32_t merge_limit;
    uint32_t pad;
} pbig2_stats;

/* Context: one device, owns its buffers and streams. Not thread-safe; use
 * one context per host thread. */
PBIG2_API int pbig2_create(int device, pbig2_ctx** out);
PBIG2_API int pbig2_destroy(pbig2_ctx* ctx);
PBIG2_API const char* pbig2_last_error(void);
PBIG2_API int pbig2_version(void);

/* Self-intersection of one scene. `boxes` holds n RectInfo records in host
 * (PBIG2_HOST) or device (PBIG2_DEVICE) memory. cell_shift selects the cell
 * size 2^cell_shift; pass PBIG2_AUTO for the autotuner. `stream` is a
 * cudaStream_t (NULL = the context's stream). The pairs stay resident on the
 * device (pbig2_result_pairs) until the next query on the context; the call
 * returns once the pair count is known and writes it to *npairs. */
#define PBIG2_AUTO 0xffffffffu
PBIG2_API int pbig2_self_intersect(pbig2_ctx* ctx, const uint32_t* boxes, uint64_t n, uint32_t dims,
                                   uint32_t range, uint32_t cell_shift, int boxes_loc, void* stream,
                                   uint64_t* npairs);

/* Red/blue intersection: only pairs with one red and one blue box are
 * reported, as (red index, blue index). */
PBIG2_API int pbig2_bipartite_intersect(pbig2_ctx* ctx, const uint32_t* red, uint64_t n_red,
                                        const uint32_t* blue, uint64_t n_blue, uint32_t dims,
                                        uint32_t range, uint32_t cell_shift, int boxes_loc,
                                        void* stream, uint64_t* npairs);

/* Batched self-intersection of independent scenes in one launch sequence.
 * `boxes` is the concatenation of all scenes (each scene's rid counts from
 * 0); scene_offsets has n_scenes+1 entries (host memory). Pairs are grouped
 * by scene: scene s owns result pairs [pair_offsets[s], pair_offsets[s+1])
 * with scene-local indices (pbig2_result_scene_offsets). cell_shifts may be
 * NULL (every scene's cell size is chosen on the device, one warp per scene
 * running the autotuner's cost model on up to 64 of its boxes) or hold one
 * shift per scene. */
PBIG2_API int pbig2_batch_intersect(pbig2_ctx* ctx, const uint32_t* boxes,
                                    const uint64_t* scene_offsets, uint32_t n_scenes, uint32_t dims,
                                    uint32_t range, const uint32_t* cell_shifts, int boxes_loc,
                                    void* stream, uint64_t* npairs);

/* Result of the last query: pointer to npairs uint32 pairs (a<b for self
 * queries; (red,blue) for bipartite), valid until the next query on the
 * context -- the context's device buffer, or the caller's buffer given to
 * pbig2_set_pair_output when the pairs went there. */
PBIG2_API int pbig2_result_pairs(pbig2_ctx* ctx, const uint32_t** dev_pairs, uint64_t* npairs);

/* Record mode results (PBIG2_OPT_RICE): device pointers to the stream
 * (nwords 8-byte words), StartI (ncells values) and Recs (nentries values),
 * valid until the next query; *npairs of the query counts the pairs in the
 * records. pbig2_copy_records copies them to host or device buffers (any of
 * the three may be NULL). pbig2_decode_records decodes a stream held in host
 * memory into (min, max) pairs. */
PBIG2_API int pbig2_result_records(pbig2_ctx* ctx, const uint64_t** words, uint64_t* nwords,
                                   const uint32_t** start_i, uint64_t* ncells, const uint32_t** recs,
                                   uint64_t* nentries);
PBIG2_API int pbig2_copy_records(pbig2_ctx* ctx, uint64_t* words, uint32_t* start_i, uint32_t* recs);
PBIG2_API int pbig2_decode_records(const uint64_t* words, uint64_t nwords, const uint32_t* start_i, uint64_t ncells,
                                   const uint32_t* recs, uint64_t nentries, uint32_t* pairs, uint64_t cap,
                                   uint64_t* npairs);

/* Direct pair output (no counterpart in the reference, whose decode() always
 * copies batches out). Later self and bipartite queries on ctx store their
 * pairs straight into dst, cap_pairs pairs of it: device memory, or
 * page-locked host memory (pbig2_host_alloc) that the pair kernels write
 * over the host link while they run, so no separate device-to-host copy is
 * needed. A result of more than cap_pairs pairs is redone into the context's
 * own device buffer (pbig2_result_pairs says where the pairs are; the copy
 * functions work from either). dst = NULL restores the default. Batched
 * queries always use the context's buffers. dst must stay valid while it is
 * set. */
PBIG2_API int pbig2_set_pair_output(pbig2_ctx* ctx, uint32_t* dst, uint64_t cap_pairs);

/* Copy pairs [first, first+count) of the last result into dst (host or
 * device memory), in the result's order; nothing to do when dst is where
 * the result already is. */
PBIG2_API int pbig2_copy_pairs(pbig2_ctx* ctx, uint32_t* dst, uint64_t first, uint64_t count,
                               int dst_loc, void* stream);

/* Per-scene pair offsets of the last batched query (n_scenes+1 values,
 * host memory). */
PBIG2_API int pbig2_result_scene_offsets(pbig2_ctx* ctx, uint64_t* offsets, uint32_t n_scenes);

/* Cell size (log2) each scene of the last query ran with: n_scenes values
 * for a batched query, 1 for a self or red/blue query (host memory). With
 * automatic cell sizes these are the autotuner's choices, after any coarser
 * rerun (pbig2_stats.grid_retries). */
PBIG2_API int pbig2_result_scene_shifts(pbig2_ctx* ctx, uint32_t* shifts, uint32_t n_scenes);

/* Asynchronous variant of pbig2_copy_pairs: enqueues the copy on `stream`
 * and returns; pbig2_sync waits for it. */
PBIG2_API int pbig2_copy_pairs_async(pbig2_ctx* ctx, uint32_t* dst, uint64_t first, uint64_t count,
                                     int dst_loc, void* stream);
PBIG2_API int pbig2_sync(pbig2_ctx* ctx, void* stream);

/* Page-locked host memory for fast host<->device copies. */
PBIG2_API int pbig2_host_alloc(size_t bytes, void** ptr);
PBIG2_API int pbig2_host_free(void* ptr);

PBIG2_API int pbig2_get_stats(pbig2_ctx* ctx, pbig2_stats* stats);

/* Context options. PBIG2_OPT_GRAPH (default 1): batched queries capture
 * their pipeline (kernels and copies, sizes read from device memory) into a
 * CUDA graph once, and replay it for later batches with the same box buffer,
 * dims, range and no more boxes, cells or scenes than the captured one. */
#define PBIG2_OPT_GRAPH 1
/* PBIG2_OPT_MERGED (default 0): the reference's MERGED=1 build. After the
 * count, sparse neighbouring cells are merged greedily into blocks of at
 * most 256 box entries (h_merge_grids, src/pbig/pbig.cu:1066-1251; on the
 * host, as there), every box enters a block once at the minimum corner of
 * (box range x block) (d_postcounting, :223-318), and the pair test runs per
 * block. The pair set is the same; the work statistics (pbig2_stats) are
 * the merged build's. Self and red/blue queries only. */
#define PBIG2_OPT_MERGED 2
/* PBIG2_OPT_RICE (default 0): self queries return the reference's Rice
 * record stream (RICE_COMPRESSION with 8-byte words, writer
 * src/pbig/pbig.cu:788-920, reader src/pbig/decode.cc:38-131) instead of
 * flat pairs, for tools that consume that stream: blocks of {0x0fffff11, cell
 * id} then records {row tile u8, column tile u8, row index u16, hits u16, one
 * column index u8 per hit} padded to 8 bytes, rows and columns being indices
 * into the cell's entry list. pbig2_result_records gives the stream and the
 * two arrays that decode it (StartI: first entry of each cell; Recs: the box
 * index of each entry); pbig2_decode_records is the reference's decode with
 * its column-offset bug fixed. Cells of 65536 boxes or more cannot be
 * written (PBIG2_ECAPACITY). Blocks are per emission step, so one cell can
 * have several (as the reference's cells of several jobs do). */
#define PBIG2_OPT_RICE 3
/* PBIG2_OPT_HOST_SPLIT (default 0 = automatic): when the pair output set by
 * pbig2_set_pair_output is page-locked host memory, the pair phase is bound
 * by the host link; the small-cell and block kernels then run on their own
 * stream over this many SMs (automatic: a quarter) beside the medium-cell
 * kernel on the rest, so the link is not idle while they compute. A
 * negative value runs the three kernels one after another. */
#define PBIG2_OPT_HOST_SPLIT 4
/* PBIG2_OPT_ONE_LAUNCH (default 1): a self query of at most 262 144 boxes
   with an automatic cell size (or a given one whose grid has at most 2^20
   cells), outside merged and record mode, runs as one cooperative kernel
   launch: cell size, count, scan, scatter and pair test, separated by grid
   barriers. A result that does not fit the buffers the launch was given is
   redone by the regular pipeline. 0 sends every query to the regular
   pipeline. The value 2 tests the barriers' bounded wait: in the next
   one-launch query no barrier completes, every block gives up after about a
   second and the query returns PBIG2_ETIMEOUT; later queries run normally. */
#define PBIG2_OPT_ONE_LAUNCH 5
/* PBIG2_OPT_CLASS_MAP (default 0 = automatic): which pair kernel takes a cell
   of n boxes. Nibble L (L = ceil(log2 n), 1..15; 15 also for larger cells)
   names the list: 0..3 lane groups of 4, 8, 16, 32 lanes (cells up to that
   many boxes), 4 one warp per cell staged whole (up to 128), 5 one block per
   cell (up to 512), 6 tile tasks (any size; required for L = 15). A map that
   sends a bucket to a list too small for it is refused. */
#define PBIG2_OPT_CLASS_MAP 6
/* PBIG2_OPT_MERGE_LIMIT (default 256, the reference's NTPB): merged mode's
   block limit -- a block grows while its boxes stay within the limit. The
   pair set does not depend on it; the merged build's statistics do. */
#define PBIG2_OPT_MERGE_LIMIT 7

/* The automatic class map: the work lists a query takes when no map is set
   (one_launch: a small scene's one-launch query). Measured on GB300: the
   default map (each cell to the smallest list that holds it) is the fastest
   on the clustered 4M-box, red/blue and 4096-scene workloads; in a one-launch
   query cells of 5..32 boxes go to the one-warp-per-cell pass instead (all
   passes run at one block per SM there, and a warp per cell keeps more
   independent load chains in flight). No
   counterpart in the reference: its cell classes are fixed at build time. */
PBIG2_API uint64_t pbig2_class_map_auto(uint32_t one_launch);
/* 0 when every bucket of the class map names a list that can hold its cells,
   else the first bucket that does not. */
PBIG2_API uint32_t pbig2_class_map_check(uint64_t map);
PBIG2_API int pbig2_set_option(pbig2_ctx* ctx, int option, int64_t value);

/* One batch of the serving loop (no counterpart in the reference; the
 * request loop in pbig_gb300/serve.py decides the batches and where each
 * scene lives). Runs, without returning to the caller in between: the cell
 * size of every item whose shift is PBIG2_AUTO (tuned on a sample of its host
 * rows; the choice is written back), the moved rows of updates (written into
 * the item's host rows, and into its device rows unless the item is
 * uploaded), uploads of items marked upload (host rows -> device rows), the
 * concatenation of the items into cat_dev (cat_rows rows; not needed for one
 * item), the batched query of the items as separate scenes, and the copy of
 * the pairs (scene-local indices, grouped by item) into pairs_host (page-
 * locked, pairs_cap pairs); scene_pair_off[n_items+1] gives each item's
 * range. stage_host (page-locked) and stage_dev hold stage_rows staged update
 * rows of 8 words. 3-D only. PBIG2_ECAPACITY: a buffer is too small (*npairs
 * holds the pair count when the pair buffer was; the result stays on the
 * device for pbig2_copy_pairs). */
typedef struct {
    uint32_t* dev;          /* the scene's rows on the device (n x 7 words) */
    uint32_t* host;         /* the scene's rows on the host (n x 7 words) */
    uint64_t n;             /* boxes of the scene */
    const uint32_t* rows;   /* update: k new rows (7 words each), else null */
    const uint32_t* idx;    /* update: their box indices */
    uint64_t k;
    uint32_t upload;        /* 1: copy the host rows to the device rows first */
    uint32_t shift;         /* cell size; PBIG2_AUTO: tuned here, written back */
} pbig2_batch_item;
PBIG2_API int pbig2_serve_batch(pbig2_ctx* ctx, pbig2_batch_item* items, uint32_t n_items, uint32_t range,
                                uint32_t* cat_dev, uint64_t cat_rows, uint32_t* stage_host, uint32_t* stage_dev,
                                uint64_t stage_rows, void* stream, uint32_t* pairs_host, uint64_t pairs_cap,
                                uint64_t* npairs, uint64_t* scene_pair_off, double* phase_ms);

/* Allocation-free self-intersection (no counterpart in the reference).
 * For callers that cannot allocate device memory during the query -- a
 * process whose device memory is owned by another allocator, or a
 * latency-critical loop that cannot afford cudaMalloc/cudaFree and their
 * device-wide synchronization. Boxes and the output pairs (pair_cap uint32
 * pairs, a<b) are caller-owned device buffers; every intermediate buffer
 * lives in a fixed 16 MiB scratch array inside the library, held by every
 * GPU that loads the library until exit. Limits: n <= 262144 boxes, a grid
 * of at most 2^20 cells (the cell size is coarsened to fit) and at most
 * 524288 box-in-cell entries; larger queries return PBIG2_ECAPACITY. The
 * scratch is shared by all calls, so calls that overlap on the GPU race; the
 * first call on a device sets the device up and should come before any
 * stream capture. d_pairs must be 8-byte aligned (PBIG2_EINVAL otherwise).
 * *npairs receives the pair count, also when the pair buffer is too small;
 * it is 0 when the scene needs more cell entries than the scratch holds.
 * Error text: pbig2_noalloc_last_error(). */
PBIG2_API int pbig2_self_intersect_noalloc(const uint32_t* d_boxes, uint64_t n, uint32_t dims, uint32_t range,
                                           uint32_t cell_shift, uint32_t* d_pairs, uint64_t pair_cap,
                                           uint64_t* npairs, void* stream);
PBIG2_API const char* pbig2_noalloc_last_error(void);

/* Resident scenes and incremental updates (no counterpart in the reference,
 * which re-runs pbig_check from scratch). pbig2_scene_create runs the full
 * self-intersection of n boxes on ctx (autotuned when cell_shift is
 * PBIG2_AUTO; every box must be valid) and keeps the boxes, a grid with
 * slack in every cell and the full pair list on the device; *npairs gets the
 * pair count. pbig2_scene_move gives k boxes new coordinates (idx: their
 * indices, distinct; new_boxes: k RectInfo records with rid = the index,
 * host or device memory) and re-bins only those boxes. *n_removed gets the
 * number of pairs the moved boxes had before the move, *n_added the number
 * they have after it (pbig2_scene_delta: both lists, device memory, a pair
 * of two moved boxes once); the full list (pbig2_scene_pairs) becomes the
 * old list without the removed pairs plus the added ones -- an O(pairs)
 * step that flags = PBIG2_SCENE_DELTA_ONLY leaves out. The scene uses
 * ctx's stream and buffers: one scene call at a time per context, and the
 * context's last-result pointers are overwritten by pbig2_scene_create. */
typedef struct pbig2_scene pbig2_scene;
#define PBIG2_SCENE_DELTA_ONLY 1u /* flags: moves report their delta only; no full list is kept */
PBIG2_API int pbig2_scene_create(pbig2_ctx* ctx, const uint32_t* boxes, uint64_t n, uint32_t dims, uint32_t range,
                                 uint32_t cell_shift, int boxes_loc, uint32_t flags, pbig2_scene** scene,
                                 uint64_t* npairs);
PBIG2_API int pbig2_scene_destroy(pbig2_scene* scene);
PBIG2_API int pbig2_scene_move(pbig2_scene* scene, const uint32_t* idx, uint64_t k, const uint32_t* new_boxes,
                               int boxes_loc, uint64_t* n_removed, uint64_t* n_added);
PBIG2_API int pbig2_scene_delta(pbig2_scene* scene, const uint32_t** removed, uint64_t* n_removed,
                                const uint32_t** added, uint64_t* n_added);
PBIG2_API int pbig2_scene_pairs(pbig2_scene* scene, const uint32_t** pairs, uint64_t* npairs);
PBIG2_API int pbig2_scene_boxes(pbig2_scene* scene, const uint32_t** boxes, uint64_t* n);
/* Copy the first count pairs of the full list (which = 0), the removed
 * (1) or the added (2) pairs of the last move into dst (host or device). */
PBIG2_API int pbig2_scene_copy(pbig2_scene* scene, int which, uint32_t* dst, uint64_t count);

/* Cells of the grid a query at cell size 2^shift uses over [0, range) in
 * dims dimensions: ceil(range / 2^shift)^dims, saturating at UINT64_MAX
 * (no counterpart in the reference, whose 32-bit nCells wraps). Queries
 * refuse grids of 2^32 - 1 cells or more. */
PBIG2_API uint64_t pbig2_grid_cells(uint32_t range, uint32_t shift, uint32_t dims);

/* Cell-size autotuner: the shift the engine would pick for these boxes
 * (host memory), from a sample of at most `sample` boxes. */
PBIG2_API int pbig2_tune_shift(const uint32_t* boxes, uint64_t n, uint32_t dims, uint32_t range,
                               uint64_t sample, uint32_t* shift);

#ifdef __cplusplus
}
#endif
#endif /* PBIG2_H_ */
