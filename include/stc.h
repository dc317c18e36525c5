/*
 * stc.h -- C ABI of the GB300-native STCDB co-occurrence pipeline.
 *
 * One context owns one GPU-resident pipeline: the partitioning quadtree
 * (schema), the per-step leaf lists, the open-addressed meeting table and the
 * buffer of emitted meetings. Plain pointers and sizes only; no C++ or torch
 * types cross this boundary.
 *
 * Reference interface replaced (paths inside the tengdj/STCDB checkout):
 *   stc_create          <- partitioner::build_schema (tracing/filter.cpp:27-93,
 *                          declared tracing/partitioner.h:218) followed by
 *                          cuda_create_device_bench (cuda/geometry.cu:1395,
 *                          declared tracing/process.cpp:374)
 *   stc_step / stc_step_device
 *                       <- process_with_gpu (cuda/geometry.cu:1573, declared
 *                          tracing/process.cpp:375) and its CPU twin in
 *                          tracer::process (tracing/process.cpp:452-459, 608-612):
 *                          filter + reachability + update_meetings + update_schema
 *   stc_step_window     <- the per-step loop of tracer::process
 *                          (tracing/process.cpp:401-612) over a window of
 *                          steps, with the step replayed from a CUDA graph
 *   stc_server_*        (no reference counterpart: the reference answers
 *                          one query at a time from its experiment loops,
 *                          tools/load_search.cpp)
 *   stc_autotune        (no reference counterpart: the reference takes
 *                          grid_capacity from its command line, config.h:29)
 *   stc_drain_meetings  <- reading h_meetings_ps[0..kv_count) after
 *                          update_meetings (tracing/meeting.cpp:11-24)
 *   stc_get_stats       <- workbench counters grid_check_counter,
 *                          num_taken_buckets, num_active_meetings
 *                          (tracing/workbench.h:136, 152-153)
 *   stc_destroy         <- workbench::clear / gpu_info::clear
 *                          (tracing/workbench.cpp:62-73)
 *   stc_last_error      <- (none: the reference exits on CUDA errors,
 *                          cuda/cuda_util.cuh:19-27)
 *
 * Error behaviour: every call returns a status and never exits or hangs.
 * Device-side loops are bounded; a bound that runs out is reported as
 * STC_ERR_TIMEOUT or STC_ERR_CAPACITY and the context stays usable for
 * stc_destroy.
 *
 * Threading: a context is driven by one host thread at a time.
 */
#ifndef STC_H
#define STC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum stc_status {
  STC_OK = 0,
  STC_ERR_INVALID_ARG = 1,
  STC_ERR_CUDA = 2,
  STC_ERR_CAPACITY = 3,   /* a fixed-size device structure overflowed */
  STC_ERR_TIMEOUT = 4,    /* a bounded device loop ran out of iterations */
  STC_ERR_UNSUPPORTED = 5,
  STC_ERR_STATE = 6       /* call out of order, or context already failed */
} stc_status;

/* Pipeline parameters. Field meanings follow the reference's
 * `configuration` class (util/config.h:15-114). */
typedef struct stc_config {
  uint32_t num_objects;          /* objects per step (config.h:21) */
  uint32_t min_meet_time;        /* steps a meeting must last (config.h:39) */
  uint32_t max_meet_time;        /* longer meetings go to the oversize buffer (config.h:40) */
  uint32_t grid_capacity;        /* quadtree leaf split threshold (config.h:29) */
  double grid_amplify;           /* leaf list capacity = amplify*grid_capacity (config.h:33) */
  double reach_distance;         /* metres (config.h:41) */
  uint64_t num_meeting_buckets;  /* meeting table slots (config.h:31, default 2N config.h:306-308) */
  uint32_t refine_size;          /* border checking units per object (config.h:34) */
  uint32_t schema_update_delay;  /* consecutive over/underflows before split/merge (config.h:38) */
  int32_t dynamic_schema;        /* update the quadtree after every step (config.h:35) */
  int32_t mbr_filter;            /* drop meetings whose MBR leaves the map box (cuda/geometry.cu:667-670) */
  uint64_t candidate_capacity;   /* new-meeting candidates per step; 0 = auto */
  uint64_t emit_capacity;        /* emitted meetings held between drains; 0 = auto */
  uint64_t hit_capacity;         /* pairs buffered between refinement and table update; 0 = auto:
                                    max(4M, 8 n), grown after a step (or window) that found more */
  uint32_t device;               /* CUDA device ordinal */
  uint32_t flags;                /* STC_FLAG_* (0 for normal operation) */
  /* Memtable and flush into a contact tracing block (CTB) of CTFs, the
   * reference's GPU flush (cuda/geometry.cu:1752-2138). Off while
   * kv_restriction is 0. */
  uint64_t kv_restriction;       /* flush after a step that leaves more directed keys than this
                                    in the memtable (config.h:55, 80) */
  uint64_t kv_capacity;          /* memtable size in directed keys; 0 = kv_restriction + 1,000,000
                                    (config.h:81) */
  uint32_t ctf_count;            /* CTFs per block, a perfect square <= 3969; 0 = 100 (config.h:59, 83-84) */
  uint32_t start_time;           /* time of the first step; the first block's key times count from
                                    start_time + min_meet_time (config.h:28, process.cpp:404) */
  double area_restriction;       /* an object whose box over all its keys has a larger area (deg^2)
                                    goes to the oversize buffer (process.cpp:408-411); 0 = 100, no cut */
  uint32_t ctb_retain;           /* flushed blocks kept on the device for queries; the oldest is
                                    dropped beyond this; 0 = 8 */
  uint32_t step_slices;          /* launches each long step kernel (pair tests, table update,
                                    sweep) is cut into, so that queries running on another thread
                                    get the GPU between them; results do not change; 0 = 1 */
  /* Launch shape of the refinement (stc_autotune picks it; results do not
   * depend on it: new meetings take their slots by priority, not by
   * arrival). */
  uint32_t job_chunk;            /* refinement jobs (32 rows against their candidate ranges) a warp
                                    takes at a time; 0 = 8, at most 64 */
  uint32_t refine_blocks_per_sm; /* pair-test blocks launched per SM; 0 = 8, at most 32 */
  uint32_t hits_blocks_per_sm;   /* table-update blocks launched per SM; 0 = 16, at most 64 */
  uint32_t window_graphs;        /* stc_step_window replays each step from a captured CUDA graph:
                                    0 = automatic: when the context's last step took under 1.5 ms
                                    of device time (up to 2^21 objects), or, before any step, up to
                                    2^18 objects (graphs save launch costs on short steps; a
                                    replayed graph ran long steps up to 10% slower than direct
                                    launches); 1 = always, 2 = never */
  uint32_t bitmap_edge;          /* edge of a block's map bitmap, the oversize buffer's spatial
                                    bitmap over the map box (DEFAULT_bitmap_edge, util/util.h:47,
                                    a compile-time 256 in the reference): bitmap_edge^2 bits;
                                    0 = 256; a multiple of 32 from 32 to 1024 */
  uint32_t refine_chunk;         /* refinement tile length: a job tests 32 rows against this many
                                    positions of their candidate windows (launch shape, results do
                                    not depend on it); a multiple of 32 from 32 to 4096; 0 =
                                    automatic, per step: 64 when the step before tested more than 16
                                    candidates per checking unit (dense leaves), else 256 */
} stc_config;

/* Replay quadtree splits/merges on one device thread only (tests compare it
 * with the default parallel replay). */
#define STC_FLAG_SERIAL_SCHEMA 1u
/* How the pair tests hand over their hits (results do not depend on it; by
 * default the library picks by the last step's hits per checking unit):
 * straight to the hit buffer, or through a per-warp queue. Tests force each. */
#define STC_FLAG_DIRECT_HITS 2u
#define STC_FLAG_QUEUED_HITS 4u
/* stc_step_window copies page-locked host input with a copy engine instead
 * of having each step's descent read it from the host pages (the default
 * without graphs and while no request loop is attached). Tests force it. */
#define STC_FLAG_COPY_INPUT 8u

/* One finished meeting. pid_lo < pid_hi; start/end are the first and last
 * step in which the pair was within reach; mbr is the float bounding box of
 * both objects over those steps (low x, low y, high x, high y). */
typedef struct stc_meeting {
  uint32_t pid_lo, pid_hi, start, end;
  float mbr[4];
} stc_meeting;

/* Counters of the last completed step. */
typedef struct stc_stats {
  uint32_t step;                 /* time stamp of the last step */
  uint32_t leaves;               /* live quadtree leaves */
  uint32_t schema_nodes;         /* live quadtree nodes */
  uint32_t overflow_objects;     /* objects dropped from full leaf lists */
  uint64_t checking_units;       /* own-leaf + border units (grid_check_counter) */
  uint64_t border_units;
  uint64_t pair_tests;           /* candidate pairs tested */
  uint64_t exact_tests;          /* tests that needed the fp64 reference arithmetic */
  uint64_t hits;                 /* pairs within reach */
  uint64_t new_candidates;       /* meetings started by the step (ordered insertions) */
  uint64_t taken_buckets;        /* occupied slots after the step */
  uint64_t emitted;              /* meetings emitted by the step */
  uint64_t pending;              /* emitted meetings not yet drained */
  uint32_t splits, merges;       /* schema updates applied after the step */
  uint32_t kernel_launches;      /* kernels launched by the step */
  uint32_t schema_path;          /* split/merge replay used: 1 parallel, 0 or 2 one-thread */
  uint32_t ambiguous_tests;      /* distance decisions within a few ulp of reach, where
                                    the last bit of sin() could matter */
  float step_ms;                 /* device time of the step */
  float phase_ms[8];             /* partition, border+jobs, refine, insert, sweep, schema, copy-in, memtable append */
  uint64_t memtable_keys;        /* directed keys in the memtable after the step (and any flush) */
  uint32_t flushes;              /* blocks flushed so far */
  float flush_ms;                /* device time of the last flush */
  /* The last stc_step_window call: the device time of its steps (core and
   * memtable append, flushes excluded) and the call's wall time on the host;
   * their ratio is how busy the window kept the GPU. window_input_wait_ms is
   * the part of the device time its steps spent waiting for their positions'
   * copy (a slow host link shows here). */
  float window_device_ms;
  float window_wall_ms;
  float window_input_wait_ms;
  float window_copy_ms;          /* the window's input copies, start to end (each beside a step);
                                    0 when the steps' descent read the input from the host pages */
  /* The last flush's stages (device time on the library's stream, the host's
   * reads of the device state between them included): object order (oversize
   * cut, STR sorts, slabs, sids), key sort, per-CTF limits and metadata, key
   * encoding with the bitmaps, and the block's store with its query index. */
  float flush_stage_ms[5];
  /* The last stc_compact's stages (device time on the library's stream, host
   * work between them included): scratch allocation, decode of the inputs,
   * STR order and sids, key sort, per-CTF limits and metadata with the new
   * block's allocation, key encoding with the bitmaps, and the query index. */
  float compact_stage_ms[7];
} stc_stats;

/* Fills *cfg with the reference defaults for n objects (util/config.h:29-41,
 * 303-317): grid_capacity 50, grid_amplify 2, refine_size 4, reach 2 m,
 * min_meet_time 5, max_meet_time 4096, buckets 2n, dynamic schema on. */
void stc_config_default(stc_config *cfg, uint32_t num_objects);

typedef struct stc_ctx stc_ctx;

/* Builds the quadtree from the step-0 positions xy0 (n (lon, lat) f64 pairs
 * in host memory) inside the map box mbr (lon/lat low x, low y, high x,
 * high y) and allocates all device state. */
stc_status stc_create(const stc_config *cfg, const double mbr[4], const double *xy0, uint32_t n,
                      stc_ctx **out);

/* Processes one time step. xy: num_objects (lon, lat) f64 pairs, layout
 * [oid], in host memory (copied in) or device memory (stc_step_device). */
stc_status stc_step(stc_ctx *ctx, const double *xy, uint32_t t);
stc_status stc_step_device(stc_ctx *ctx, const double *xy_device, uint32_t t);

/* Result of stc_autotune. */
typedef struct stc_tune_result {
  stc_config config;             /* the configuration given, with the chosen grid_capacity,
                                    job_chunk, refine_chunk, refine_blocks_per_sm and
                                    hits_blocks_per_sm */
  float base_step_ms;            /* device time per timed step of the configuration given */
  float best_step_ms;            /* the same for the chosen one */
  uint32_t trials;               /* candidate settings run */
  uint32_t reserved;
} stc_tune_result;

/* Autotuner: picks the quadtree leaf capacity and the refinement's launch
 * shape for positions like those given (steps x n (lon, lat) f64 pairs in
 * host memory, layout [step][oid], steps >= 3). Every candidate runs the same
 * steps from a fresh context (memtable off) and is scored by the device time
 * of its steps after the first two; the leaf capacity is chosen first among
 * `capacities` (n_capacities values; null = {grid_capacity / 2,
 * grid_capacity, 2 * grid_capacity}; cfg's own grid_capacity is always tried
 * and gives base_step_ms), then job_chunk (2-32), refine_chunk (the tile
 * length: the automatic choice or 64-512), refine_blocks_per_sm and
 * hits_blocks_per_sm one after the other. The launch shape never changes
 * results; the leaf capacity is part of the reference's configuration (it
 * orders the reference's table inserts), so a run with the chosen capacity
 * matches the reference run with that capacity. */
stc_status stc_autotune(const stc_config *cfg, const double mbr[4], const double *xy, uint32_t n, uint32_t steps,
                        const uint32_t *capacities, uint32_t n_capacities, stc_tune_result *out);

/* Processes a window of `steps` consecutive steps t0, t0 + 1, ...: xy holds
 * steps x num_objects (lon, lat) f64 pairs, layout [step][oid], in host
 * memory (on_device 0) or device memory (on_device 1). Device input is read
 * where it lies. Page-locked host input (the whole range in one page-locked
 * allocation) is read from the host pages by each step's descent, which
 * writes the device copy the rest of the step reads, unless the steps replay
 * graphs, a request loop (stc_server) is attached to the context, or
 * STC_FLAG_COPY_INPUT is set. Otherwise each step's positions are copied into
 * one of three input buffers once the step three before it has run, beside
 * the sweep of the step queued before it (page-locked host memory by DMA,
 * pageable memory staged by the driver). The window is pipelined one step
 * deep: step i + 1 is queued on the GPU before
 * the host reads step i's state, so the GPU does not wait for the host
 * between steps. The memtable
 * append of step i + 1 is queued only after step i's flush decision (a flush
 * runs behind the next step's core, which never touches the memtable), so
 * results equal those of stc_step called step by step, flushes included.
 * Small windows replay each step's core from a CUDA graph captured once
 * (stc_config.window_graphs; captured again after a flush or a change of the
 * slice count), so such a step costs one launch instead of one per kernel.
 * When out is given, each step's meetings are drained into out[*n_out..cap)
 * beside the next step and *n_out counts them. When they do not fit the call
 * returns STC_ERR_CAPACITY (the context stays usable): at most one step
 * beyond the one that filled out has run, stc_stats.step names the last step
 * that ran, and the meetings that did not fit stay pending for
 * stc_drain_meetings. Phase times of the window's steps are not recorded
 * (stc_stats.step_ms is). */
stc_status stc_step_window(stc_ctx *ctx, const double *xy, int on_device, uint32_t steps, uint32_t t0,
                           stc_meeting *out, size_t cap, size_t *n_out);

/* Copies up to cap emitted meetings (in emission order) into out, removes
 * them from the context and stores how many were copied in *n. */
stc_status stc_drain_meetings(stc_ctx *ctx, stc_meeting *out, size_t cap, size_t *n);

stc_status stc_get_stats(stc_ctx *ctx, stc_stats *stats);

/* ---- Memtable flush: contact tracing blocks (CTBs) ----------------------
 *
 * With kv_restriction > 0 every emitted meeting also enters the memtable as
 * two directed keys (pid, target, duration = end - start, end - end_time_min)
 * with its float box, as cuda_identify_meetings does (cuda/geometry.cu:
 * 701-737). After a step that leaves more than kv_restriction keys, stc_step
 * flushes the memtable into a block, the reference's flush sequence
 * (cuda/geometry.cu:1752-2138):
 *   - objects whose box over all their keys is larger than area_restriction,
 *     and both objects of a meeting longer than max_meet_time, get sid 1; their
 *     keys go to the oversize buffer, sorted by key, with a 256 x 256 bitmap of
 *     their boxes over the map;
 *   - the other objects are ordered by the midpoint of their box (x, then y
 *     within ctf_count^(1/2) slabs) and cut into ctf_count sids (2..);
 *   - their keys, sorted by (sid, pid, target, duration, end), form the CTFs:
 *     per CTF the box, time limits, bit widths (CTF::get_ctf_bits,
 *     tracing/step_merge.cpp:140-186), an x_grid * y_grid bitmap of the key
 *     boxes, and the keys packed into key_bit/8 bytes each (write_key_and_mbr).
 * The block stays readable until the next flush. end_time_min of the next
 * block is the flush step (process.cpp:271). */

/* One CTF (an SSTable) of a block: the reference CTF's fields
 * (tracing/step_merge.h:64-87) plus where its keys are. */
typedef struct stc_ctf {
  float mbr[4];                  /* ctf_mbr: box of its key boxes (low x, low y, high x, high y) */
  uint32_t kv_count;             /* CTF_kv_capacity */
  uint32_t start_time_min, start_time_max, end_time_min, end_time_max;
  uint32_t bitmap_bytes;         /* ctf_bitmap_size: (x_grid * y_grid + 7) / 8 */
  uint16_t key_bit, id_bit, duration_bit, end_bit, low_x_bit, low_y_bit, edge_bit, mbr_bit, x_grid, y_grid;
  uint32_t pad;
  uint64_t first_key;            /* index of its first key in the block's sorted keys */
  uint64_t key_offset;           /* byte offset of its packed keys in the block's key bytes */
} stc_ctf;

typedef struct stc_ctb_info {
  uint32_t index;                /* block number: flushes and compactions number their
                                    blocks 0, 1, 2, ... in the order they make them */
  uint32_t ctf_count;
  uint32_t flush_time;           /* step after which it was flushed (end_time_max) */
  uint32_t end_time_min;         /* base of the keys' end field */
  uint64_t kv_count;             /* directed keys flushed (two per meeting) */
  uint64_t ctf_kv_count;         /* keys in the CTFs */
  uint64_t oversize_kv_count;    /* keys in the oversize buffer */
  uint64_t key_bytes;            /* total bytes of packed CTF keys */
  uint32_t sid_count;            /* objects with at least one key */
  uint32_t oversize_oid_count;   /* the reference's counter: oversize objects plus meetings
                                    longer than max_meet_time */
  uint32_t o_start_time_min, o_start_time_max, o_end_time_min, o_end_time_max;  /* oversize buffer */
  uint32_t bitmap_edge;          /* edge of its map bitmap (stc_config.bitmap_edge) */
  uint32_t pad;
} stc_ctb_info;

/* Bytes of one CTF bitmap slot: 256 x 256 bits, room for the largest CTF
 * grid (x_grid, y_grid <= 255, tracing/step_merge.cpp:175-181). CTF i's
 * bitmap is slot i; its first bitmap_bytes bytes are used. */
#define STC_BITMAP_BYTES 8192u
/* Bytes of a block's map bitmap (the oversize buffer's, cells of the map box
 * on an edge x edge grid, bit i + j * edge; tracing/step_merge.cpp:52-59):
 * 8192 at the default edge of 256. */
#define STC_MAP_BITMAP_BYTES(edge) ((size_t)(edge) * (size_t)(edge) / 8u)

/* Flushes the memtable now if it holds any key (*flushed = 1) -- the
 * reference flushes only past kv_restriction; this also ends a run. */
stc_status stc_flush(stc_ctx *ctx, int *flushed);

/* Describes the last flushed block; STC_ERR_STATE if none yet. */
stc_status stc_get_ctb(stc_ctx *ctx, stc_ctb_info *info);

/* Copies parts of the last flushed block to host memory; any pointer may be
 * NULL. Sizes: ctfs[ctf_count]; bitmaps[ctf_count * STC_BITMAP_BYTES];
 * keys[key_bytes] (CTF i's keys at ctfs[i].key_offset, key_bit/8 bytes each,
 * little-endian); sids[num_objects] (0 no key, 1 oversize, 2.. CTF + 2);
 * oversize_keys[2 * oversize_kv_count] (128-bit keys pid:26 | target:26 |
 * duration:32 | end:32 as (low, high) 64-bit halves, util.h:47-52);
 * oversize_boxes[4 * oversize_kv_count]; oversize_bitmap[STC_MAP_BITMAP_BYTES(bitmap_edge)]. */
stc_status stc_read_ctb(stc_ctx *ctx, stc_ctf *ctfs, uint8_t *bitmaps, uint8_t *keys, uint16_t *sids,
                        uint64_t *oversize_keys, float *oversize_boxes, uint8_t *oversize_bitmap);

/* ---- Queries over the flushed blocks -----------------------------------
 *
 * The reference's disk searches (workbench::id_search_in_CTB,
 * CTF::search_SSTable, oversize_buffer::search_buffer, mbr_search_in_disk;
 * tracing/workbench.cpp:413-460, 495-572, tracing/step_merge.cpp:65-110,
 * 518-570) over the blocks this context keeps (ctb_retain), with the time
 * window applied as the reference's time_query states (a key matches when
 * its start < t_end and t_start < its end, util/query_context.h:95-105) and
 * without the fixed test box of CTF::search_SSTable (step_merge.cpp:549).
 *   object: per block, the object's sid picks the oversize buffer or one CTF,
 *           a binary search finds its first key, the scan runs while the pid
 *           matches (keys are directed: pid is the object queried);
 *   box:    every key whose box intersects the query box (closed intervals,
 *           geometry/geometry.h:128-133): CTF keys by their decoded box
 *           (CTF::new_parse_mbr, step_merge.cpp:362-379), oversize keys by
 *           their float box.
 * *n receives the number of matches; the first cap are written to out.
 * Queries read only flushed blocks, so one host thread may query while
 * another runs stc_step on the same context; queries are serialised among
 * themselves and run on their own high-priority stream. Their errors are
 * reported by stc_last_error(NULL) on the calling thread. */
typedef struct stc_contact {
  uint32_t pid, target, start, end;
  double mbr[4];                 /* decoded key box, or the float box of an oversize key */
  uint32_t block;                /* stc_ctb_info.index of its block */
  uint32_t ctf;                  /* its CTF, or ctf_count for the oversize buffer */
} stc_contact;

stc_status stc_query_object(stc_ctx *ctx, uint32_t pid, uint32_t t_start, uint32_t t_end, stc_contact *out,
                            size_t cap, size_t *n);
stc_status stc_query_box(stc_ctx *ctx, const double box[4], uint32_t t_start, uint32_t t_end, stc_contact *out,
                         size_t cap, size_t *n);

/* A batch of queries in one device pass (the serving path: queries that
 * arrive while a batch runs form the next one). offsets[nq + 1]: the matches
 * of query i are out[offsets[i] .. offsets[i + 1]) when offsets[nq] <= cap;
 * otherwise only offsets and counts are meaningful and out's contents are
 * unspecified. counts[nq] (may be NULL): the number of matches of each
 * query. A query whose kind carries STC_QUERY_COUNT_ONLY is only counted, as
 * the reference's searches do (search_count): it writes no contacts. Up to
 * two batches (from different threads) run on the GPU at the same time, each
 * on its own stream and buffers; a batch larger than 65535 / ctb_retain
 * queries runs as several device passes. */
#define STC_QUERY_OBJECT 0u
#define STC_QUERY_BOX 1u
#define STC_QUERY_COUNT_ONLY 0x100u
typedef struct stc_query {
  uint32_t kind;                 /* STC_QUERY_OBJECT or STC_QUERY_BOX, optionally | STC_QUERY_COUNT_ONLY */
  uint32_t pid;                  /* object queries */
  uint32_t t_start, t_end;
  double box[4];                 /* box queries: low x, low y, high x, high y */
} stc_query;

stc_status stc_query_batch(stc_ctx *ctx, const stc_query *queries, size_t nq, stc_contact *out, size_t cap,
                           uint64_t *offsets, uint64_t *counts);

/* ---- Serving: a request loop over stc_query_batch --------------------------
 *
 * A server owns two worker threads that answer submitted queries by
 * continuous batching: an idle worker takes what has arrived, in arrival
 * order, as its batch and runs it on its own query stream, so queries that
 * arrive while a batch is on the GPU start at once beside it instead of
 * waiting for it to end. Admission is by device footprint: every query takes
 * its record and counters, a query that returns contacts (no
 * STC_QUERY_COUNT_ONLY) also reserves result_cap contacts of device output,
 * and a batch is admitted while the footprint of all batches in flight stays
 * within hbm_budget (a batch's first query is always admitted when nothing
 * else is in flight; otherwise it waits until memory frees). A query with
 * more than result_cap contacts is answered with its count, no contacts and
 * STC_ERR_CAPACITY, whatever else its batch holds. The context keeps
 * stepping meanwhile on other threads (stc_query_batch may run beside
 * stc_step). */
typedef struct stc_server_config {
  uint32_t max_batch;            /* queries per batch; 0 = 4096 */
  uint32_t result_cap;           /* contacts reserved per non-counting query; 0 = 1024 */
  uint64_t hbm_budget;           /* device bytes of one batch's queries and output; 0 = 64 MB */
} stc_server_config;

typedef struct stc_answer {
  uint64_t ticket;               /* from stc_server_submit */
  uint64_t count;                /* matches of the query */
  uint64_t contact_offset;       /* its contacts in the poll's contacts array */
  uint32_t stored;               /* contacts written there */
  uint32_t status;               /* STC_OK, or the error of its batch / STC_ERR_CAPACITY */
  double latency_ms;             /* from its arrival time to its answer */
  uint32_t batch;                /* sequence number of the batch that answered it */
  uint32_t batch_size;           /* queries in that batch */
} stc_answer;

typedef struct stc_server_stats {
  uint64_t submitted, answered, batches;
  uint64_t max_batch_queries;    /* largest batch */
  uint64_t max_batch_bytes;      /* largest admitted footprint */
  uint64_t budget_cuts;          /* batches closed by the budget before max_batch */
  uint64_t overlapped_batches;   /* batches that started while another batch was on the GPU */
  uint64_t slowest_batch_wall_us;  /* the longest batch from its worker's start to its answers */
  uint64_t slowest_batch_gpu_us;   /* that batch's span on its query stream (from its first copy to
                                      the read-back of its counts, waits for SMs included) */
} stc_server_stats;

typedef struct stc_server stc_server;

stc_status stc_server_start(stc_ctx *ctx, const stc_server_config *cfg, stc_server **out);
/* Queues nq queries that arrived at arrival_s (seconds on the host's
 * monotonic clock, as CLOCK_MONOTONIC; <= 0: now); *first_ticket receives the
 * ticket of the first, the others follow in order. */
stc_status stc_server_submit(stc_server *srv, const stc_query *queries, size_t nq, double arrival_s,
                             uint64_t *first_ticket);
/* Moves up to cap answers (and their contacts, up to contacts_cap) completed
 * since the last poll into out / contacts; waits up to wait_ms for the first
 * when none is ready. An answer holds at most result_cap contacts; when the
 * first ready answer alone does not fit contacts_cap, the poll returns
 * STC_ERR_CAPACITY with *n = 0 and the answer stays queued. */
stc_status stc_server_poll(stc_server *srv, stc_answer *out, size_t cap, stc_contact *contacts,
                           size_t contacts_cap, size_t *n, int wait_ms);
stc_status stc_server_get_stats(const stc_server *srv, stc_server_stats *out);
/* Answers everything queued, stops the thread and frees the server. A
 * server must be stopped before its context is destroyed. */
stc_status stc_server_stop(stc_server *srv);

/* ---- Block files ---------------------------------------------------------
 *
 * stc_write_ctb writes retained block `index` (stc_ctb_info.index) as the
 * reference's files (straight_dump, tracing/process.cpp:254-348) in dir:
 *   <prefix>_SSTable_<index>-<c>  packed keys of CTF c,
 *   <prefix>_STcL<index>-<c>      the CTF object (80 bytes) and its bitmap
 *                                 (CTF::dump_meta, step_merge.cpp:644-650),
 *   <prefix>_CTB<index>           the CTB object (128 bytes), sids, oversize keys
 *                                 (128-bit), boxes, map bitmap (dump_CTB_meta,
 *                                 workbench.cpp:597-614),
 * objects in the reference's LP64 byte layout with pointers and padding 0, so
 * the reference's loaders (workbench::load_CTB_meta, load_CTF_keys) read them.
 * stc_load_ctb reads such files (written here or by the reference; its key
 * files must be gathered into dir) into a retained block for queries, as
 * block `index`; the block has as many CTFs as consecutive <prefix>_STcL
 * files exist from CTF 0 (a compacted block may have more or fewer than
 * ctf_count). Like stc_step, neither may run concurrently with stc_step on
 * the same context. Errors: stc_last_error(ctx). */
stc_status stc_write_ctb(stc_ctx *ctx, uint32_t index, const char *dir, const char *prefix);
stc_status stc_load_ctb(stc_ctx *ctx, uint32_t index, const char *dir, const char *prefix);

/* ---- Any retained block --------------------------------------------------
 *
 * stc_get_block / stc_read_block: stc_get_ctb / stc_read_ctb for retained
 * block `index` (a flushed, loaded or compacted one), same layout. */
stc_status stc_get_block(stc_ctx *ctx, uint32_t index, stc_ctb_info *info);
stc_status stc_read_block(stc_ctx *ctx, uint32_t index, stc_ctf *ctfs, uint8_t *bitmaps, uint8_t *keys,
                          uint16_t *sids, uint64_t *oversize_keys, float *oversize_boxes, uint8_t *oversize_bitmap);

/* ---- Compaction ------------------------------------------------------------
 *
 * Merges retained block first_index and the count - 1 blocks retained after it
 * (oldest first) into one block of split * split CTFs (1 <= split <= 63),
 * which replaces them in the retained list under a new index (*new_index);
 * queries then search the merged block. This is the reference's merge_dump
 * (tools/compaction.cpp:729-1206): every CTF key is decoded (CTF::parse_key,
 * CTF::new_parse_mbr_f_box), each object's keys are sorted by target, the
 * objects are re-partitioned by STR over the midpoints of their key boxes
 * into split x split sids, every CTF gets its box, time limits, bit widths
 * (CTF::get_ctf_bits), bitmap and re-packed keys, and the oversize buffers are
 * merged in key order with one map bitmap. Where merge_dump loses or corrupts
 * keys this does not: every key of the inputs is in the result (the STR
 * object merge_dump leaves without a CTF, :931-942, gets one; no CTF is padded
 * with object 0's keys, :925-929; decoded oids are masked to id_bit, as
 * CTF::ctf_get_key_oid does), an object oversize in any input stays oversize,
 * CTF end times are the merged blocks' with key ends stored relative to
 * end_time_min (end_bit grows when the merged span needs it), and oversize
 * ends are re-based to the merged buffer's end_time_min. Objects with equal
 * midpoints are ordered by pid and one object's keys by (target, duration,
 * end), orders merge_dump leaves unspecified. The merge allocates its own
 * scratch (about 100 bytes per merged key). *device_ms (may be NULL): device
 * time of the merge. Call between steps; queries may run meanwhile on other
 * threads. Errors: stc_last_error(ctx). */
stc_status stc_compact(stc_ctx *ctx, uint32_t first_index, uint32_t count, uint32_t split, uint32_t *new_index,
                       float *device_ms);

/* ---- Checkpoint / restore ------------------------------------------------
 *
 * stc_checkpoint writes everything a context carries from one step to the
 * next -- configuration, quadtree schema, meeting table, undrained emitted
 * meetings, memtable, counters -- to one versioned file (a replacement for
 * the reference's raw workbench dumps, tracing/workbench.cpp:574-694);
 * stc_restore creates a context on `device` from it, and the next stc_step
 * continues as the checkpointed context would have. Retained flushed blocks
 * are not in the file (write them with stc_write_ctb); after a restore
 * stc_get_ctb reports none until the next flush, and block indices continue.
 * The file is tied to this library version (struct sizes are checked) and
 * carries a checksum. Call between steps. Errors: stc_last_error(ctx), or
 * stc_last_error(NULL) for stc_restore. */
stc_status stc_checkpoint(stc_ctx *ctx, const char *path);
/* The configuration a context runs with (a restored one's comes from its file). */
stc_status stc_get_config(const stc_ctx *ctx, stc_config *cfg);
stc_status stc_restore(const char *path, uint32_t device, stc_ctx **out);

/* Changes stc_config.step_slices of a running context (between steps): a
 * server slices its steps while it answers queries, so that query kernels
 * start between the slices, and runs whole steps otherwise. */
stc_status stc_set_step_slices(stc_ctx *ctx, uint32_t slices);

/* Last error message of ctx (or, when ctx is NULL, of the last failed
 * stc_create or context-free call on this thread). Never NULL. */
const char *stc_last_error(const stc_ctx *ctx);

void stc_destroy(stc_ctx *ctx);

/* Stable LSD radix sort of n (key, value) uint32 pairs on the low key_bits
 * bits of the key (1..32), on CUDA device `device`. All four pointers are
 * device memory; outputs must not alias inputs. Scratch (2n words plus
 * histograms) is allocated and freed inside the call; the call returns when
 * the sort is done. This is the sort the pipeline uses to group objects by
 * quadtree leaf in pid order; it replaces thrust::sort_by_key in the
 * reference's flush (cuda/geometry.cu:1860-1907) for 32-bit keys. Errors:
 * stc_last_error(NULL). */
stc_status stc_sort_pairs_u32(const uint32_t *keys, const uint32_t *values, uint32_t *keys_out,
                              uint32_t *values_out, size_t n, uint32_t key_bits, uint32_t device);

/* Same sort and arguments as stc_sort_pairs_u32, for callers that cannot
 * have device memory allocated on their behalf: code that owns all device
 * memory through its own allocator or a fixed budget, and code on a
 * latency-critical path where cudaMalloc/cudaFree (which can take driver
 * locks and synchronise the device) are not allowed. It allocates nothing:
 * its scratch is a fixed array inside the library (about 8.7 MB, kept on
 * every device that uses it until the process exits), so n is limited to
 * STC_SORT_NOALLOC_MAX_PAIRS; larger n returns STC_ERR_CAPACITY.
 * The first call on a device looks up the array's device address (a one-time
 * set-up per device); make that first call before any stream capture.
 * All calls share the one array: calls that overlap on the GPU (from several
 * host threads, or launched while another is still running) race and corrupt
 * each other's results. The array's device address is kept per device for
 * the life of the process, so a device reset (cudaDeviceReset) while the
 * library is loaded is not supported by this call. The call returns when the
 * sort is done.
 * No counterpart in the reference. Errors: stc_last_error(NULL). */
#define STC_SORT_NOALLOC_MAX_PAIRS (1u << 20)
stc_status stc_sort_pairs_u32_noalloc(const uint32_t *keys, const uint32_t *values, uint32_t *keys_out,
                                      uint32_t *values_out, size_t n, uint32_t key_bits, uint32_t device);

/* Device time in milliseconds of the sort passes of the last successful
 * stc_sort_pairs_u32 call on this thread (scratch allocation excluded). Only
 * stc_sort_pairs_u32 sets it; stc_sort_pairs_u32_noalloc leaves it as it is. */
float stc_last_sort_ms(void);

/* Random-access ceiling of the meeting-table update on CUDA device
 * `device`: `accesses` reads of the first 16 bytes of random slots of a table
 * of 2^table_log2 32-byte slots (10..32; the slot of access i is a hash of
 * i), each followed by a store of the slot's end word -- the pattern of the
 * table update, where a hit reads its home slot and writes it. The table
 * (32 << table_log2 bytes) is allocated, filled and freed inside the call.
 * *ms = the best device time of three timed runs after one warm-up run.
 * A bench utility for the table update's roofline; no counterpart in the
 * reference. Errors: stc_last_error(NULL). */
stc_status stc_measure_random_access(uint32_t table_log2, unsigned long long accesses, uint32_t device,
                                     float *ms);

#ifdef __cplusplus
}
#endif
#endif /* STC_H */
