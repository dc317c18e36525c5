// Memtable and flush into contact tracing blocks (the LSM layer).
//
// The reference keeps its memtable in the GPU workbench (d_keys / kv_boxs,
// filled by cuda_identify_meetings, cuda/geometry.cu:701-737) and flushes it
// in process_with_gpu (cuda/geometry.cu:1752-2138). Here the memtable is a
// pair of device arrays appended to after every step's sweep, and a flush is
// a short host-driven sequence of device sorts and per-key kernels:
//
//   memtable   rec[i] = (pid, target, duration, end - end_time_min)   uint4
//              box[i] = float box of the meeting                     float4
//   per object cnt (keys), obox (uint_box of all its key boxes), sid
//   block      brec/bbox: CTF keys sorted by (sid, pid, target, duration,
//              end), then the oversize keys sorted by (pid, target, ...);
//              kbytes: packed CTF keys; bitmaps; ctfs; bsid.
#pragma once
#include <deque>
#include <mutex>
#include <shared_mutex>
#include <string>
#include <vector>

#include "stc_pipeline.cuh"

namespace stc {

struct LsmDev {
  uint32_t N, max_meet, F, split;
  uint32_t end_time_min;
  uint32_t edge;                   // map bitmap edge (bitmap_edge)
  double area;
  double map[4];
  unsigned long long cap;          // memtable capacity (directed keys)
  DevState *st;
  uint4 *rec;                      // memtable keys
  float4 *box;                     // memtable boxes
  uint4 *brec;                     // block: sorted keys
  float4 *bbox;
  uint8_t *over;                   // per memtable key: oversize at partition time
  uint32_t *sk[7];                 // sort scratch, max(cap, N) words each
  uint32_t *hist, *scan;           // radix-sort histograms and scan blocks
  unsigned long long *n_dev;       // [6] item counts read by the sorts; [4] the index's largest end offset
  uint32_t *cnt;                   // per object: keys (same_pid_count)
  uint4 *obox;                     // per object: low0, low1, high0, high1 (float_to_uint)
  uint16_t *sid;                   // per object: working sid
  uint16_t *bsid;                  // per object: sids of the last block
  uint32_t *mid_lo, *mid_hi;       // per object: STR midpoint (y, x)
  uint32_t *ctf_cap;               // [F]
  unsigned long long *ctf_first;   // [F + 1]
  stc_ctf *ctfs;                   // [F]
  float4 *lim_box;                 // [F] per-CTF box
  uint2 *lim_time;                 // [F] per-CTF start min, max
  uint32_t *bitmaps;               // [F * 2048]
  uint32_t *obitmap;               // [edge * edge / 32]
  uint8_t *kbytes;                 // packed CTF keys (16 * cap bytes)
};

// Spatial index of a block's CTF keys (query pruning; not part of the
// reference's format). Each CTF gets a loose multi-level grid over its box:
// level 0 has g x g cells, g a power of two near sqrt(keys /
// LSM_INDEX_KEYS_PER_CELL) in [LSM_INDEX_MIN_GRID, LSM_INDEX_MAX_GRID], and
// level k has cells 2^k times larger. A key is filed at the first level
// whose cells are at least as large as its decoded box's extent in level-0
// cells, under the cell of the box's low corner; so at its level the box
// ends at most one cell right of / above that cell, and a query widens its
// window by one cell per level. Keys whose corner falls outside the grid go
// to the CTF's wide list. Within a cell keys go by end time.
constexpr uint32_t LSM_INDEX_KEYS_PER_CELL = 8;
constexpr uint32_t LSM_INDEX_MIN_GRID = 16;
constexpr uint32_t LSM_INDEX_MAX_GRID = 256;

// Cells of one level of the index: (g >> k) + 1 per side (the last holds
// corners exactly on the CTF box's high edge).
__host__ __device__ inline uint32_t index_level_side(uint32_t g, uint32_t k) { return (g >> k) + 1u; }

// Device copy of one flushed block, kept for queries.
struct CtbBlock {
  stc_ctb_info info{};
  std::vector<stc_ctf> ctfs;       // host copy
  uint8_t *keys = nullptr;         // packed CTF keys (+32 bytes of padding for word loads)
  stc_ctf *d_ctfs = nullptr;
  uint32_t *bitmaps = nullptr;     // [F * 2048]
  uint16_t *sids = nullptr;        // [N]
  uint4 *orec = nullptr;           // oversize keys (pid, target, duration, end offset), sorted
  float4 *obox = nullptr;
  uint32_t *obitmap = nullptr;     // [edge * edge / 32]: map bitmap
  // spatial index of the CTF keys: per CTF, dense cells (gx + 1) x (gy + 1)
  // of the low corner of each key's box, then one wide slot
  uint32_t *perm = nullptr;        // block key positions sorted by dense cell id
  uint32_t *cstart = nullptr;      // [ncells + 1] first position of each cell in perm
  uint32_t *cbase = nullptr;       // [F + 1] first dense cell id of each CTF
  uint4 *ixg = nullptr;            // [F] (g, levels, 0, 0) of each CTF's index
  double2 *ixs = nullptr;          // [F] level-0 cells per degree in x and y (g / CTF box side)
  float4 *ixf = nullptr;           // [2F] float filing of keys: per axis (cells per low unit, cells per
                                   // edge unit, error margin, 1 if usable)
  uint16_t *pend = nullptr;       // [keys] end offset of the key at each perm position, saturated at
                                   // 65535; within a cell the keys go by increasing end
};

// A retained block as the query kernels see it.
struct QBlock {
  const uint8_t *keys;
  const stc_ctf *ctfs;
  const uint16_t *sids;
  const uint4 *orec;
  const float4 *obox;
  const uint32_t *bitmaps;
  const uint32_t *obitmap;
  const uint32_t *perm;
  const uint32_t *cstart;
  const uint32_t *cbase;
  const uint4 *ixg;
  const double2 *ixs;
  const uint16_t *pend;
  unsigned long long n_over;
  uint32_t F, index, o_end_time_min, edge;  // edge: of the map bitmap
};

// One match on the device: the contact and the query it answers.
struct QueryRec {
  stc_contact c;
  uint32_t q, pad;
};

// The device and pinned buffers and the stream of one query batch in
// flight. A context keeps QUERY_LANES of them, so that that many batches
// (the serving loop's workers, direct stc_query_batch calls) run on the GPU
// at the same time.
struct QueryLane {
  std::mutex mu;                   // held by the batch using the lane
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // a batch's span on the stream
  QBlock *d_qb = nullptr;          // [retain]
  stc_query *d_q = nullptr;
  size_t q_cap = 0;
  QueryRec *d_out = nullptr;
  size_t out_cap = 0;
  unsigned long long *d_count = nullptr;
  unsigned long long *d_qcounts = nullptr;  // per-query match counts
  size_t qc_cap = 0;
  uint32_t *d_items = nullptr;     // box-query plan: work items per (query, block, CTF), then their scan
  size_t items_cap = 0;
  uint32_t *d_iscan = nullptr;     // scan scratch
  size_t iscan_cap = 0;
  // Mapped pinned host buffers of a batch's inputs and results. Kernels on
  // the lane's stream read and write them over the host link directly, so a
  // batch never queues on a copy engine behind a step's position copy (tens
  // to hundreds of MB) or a drain. m_* are their device-side addresses.
  QBlock *h_qb = nullptr, *m_qb = nullptr;                // [retain]
  stc_query *h_q = nullptr, *m_q = nullptr;
  size_t hq_cap = 0;
  unsigned long long *h_counts = nullptr, *m_counts = nullptr;  // [hq_cap + 1]: per-query counts, then the total
  QueryRec *h_recs = nullptr, *m_recs = nullptr;
  size_t hrecs_cap = 0;
};

constexpr int QUERY_LANES = 2;

struct LsmHost {
  bool has_block = false;
  uint32_t flushes = 0;
  uint32_t next_index = 0;         // index of the next block a flush or compaction makes
  stc_ctb_info info{};
  std::vector<stc_ctf> ctfs;
  // retained blocks (oldest first) and the query state
  uint32_t retain = 8;
  uint32_t edge = 256;             // map bitmap edge of every block (bitmap_edge)
  std::deque<CtbBlock> blocks;
  std::shared_mutex blocks_mu;     // exclusive while the list changes
  QueryLane lanes[QUERY_LANES];
  double map[4] = {0, 0, 0, 0};
};

// Words of sort scratch per array and radix histogram words for the flush.
size_t lsm_sort_words(const LsmDev &L);

// Initial memtable state (empty, object boxes at their initial values).
void lsm_init(LsmDev &L, cudaStream_t s);

// Appends the step's emitted meetings (the last step_emitted records of the
// emit buffer) as two directed keys each.
void lsm_append(const PipeDev &p, const LsmDev &L, cudaStream_t s);

// Flushes the memtable at step t into a block. st_host is a pinned DevState
// mirror used for read-backs. On failure returns a status and sets err.
// marks (optional): four events recorded on s after the object order (STR
// sort, slabs, sids), the key sort, the CTF limits and metadata, and the key
// encoding.
stc_status lsm_flush(LsmDev &L, LsmHost &H, uint32_t t, cudaStream_t s, DevState *st_host, std::string &err,
                     const cudaEvent_t *marks = nullptr);

// Copies the block just flushed into its own allocations, builds its cell
// index and appends it to the retained blocks, dropping the oldest beyond
// H.retain. L's sort scratch is used for the index.
stc_status lsm_store_block(const LsmDev &L, LsmHost &H, cudaStream_t s, std::string &err);

// Writes retained block `index` as the reference's files, and reads such
// files back into a retained block (stc_write_ctb / stc_load_ctb).
stc_status lsm_write_block(LsmHost &H, uint32_t index, uint32_t num_objects, const std::string &dir,
                           const std::string &prefix, std::string &err);
stc_status lsm_load_block(const LsmDev &L, LsmHost &H, uint32_t index, const std::string &dir,
                          const std::string &prefix, cudaStream_t s, std::string &err);

// Retained block `index`: its description, and copies of its arrays in the
// layout of stc_read_ctb (any pointer may be null).
stc_status lsm_block_info(LsmHost &H, uint32_t index, stc_ctb_info *info, std::string &err);
stc_status lsm_read_block(LsmHost &H, uint32_t index, uint32_t num_objects, stc_ctf *ctfs, uint8_t *bitmaps,
                          uint8_t *keys, uint16_t *sids, uint64_t *okeys, float *oboxes, uint8_t *obitmap,
                          std::string &err);

// Frees the retained blocks and the query buffers.
void lsm_release(LsmHost &H);

// Frees the device arrays of one block.
void free_block(CtbBlock &B);

// Builds the cell index of block B (its keys, device CTF records and host CTF
// copies must be in place), sorting with L's radix-sort scratch.
cudaError_t build_index(const LsmDev &L, CtbBlock &B, cudaStream_t s);

// Merges the retained block `first_index` and the count - 1 blocks retained
// after it into one block of split x split CTFs (the reference's merge_dump,
// tools/compaction.cpp:729-1206), which takes their place in the retained
// list under index new_index. L supplies the configuration (objects,
// max_meet_time, map); the merge allocates its own scratch. ms: device time.
// stages (optional, COMPACT_STAGES floats): the device time of the scratch
// allocation, the inputs' decode, the STR order, the key sort, the CTF
// limits and metadata with the new block's allocation, the key encoding and
// the query index.
constexpr int COMPACT_STAGES = 7;
stc_status lsm_compact(const LsmDev &L, LsmHost &H, uint32_t first_index, uint32_t count, uint32_t split,
                       uint32_t new_index, cudaStream_t s, float *ms, std::string &err, float *stages = nullptr);

// Creates the query lanes' streams (priority `priority`) and allocates their
// buffers for batches of up to nq queries over blocks of up to F CTFs (later
// batches then allocate nothing unless they need more).
stc_status lsm_query_reserve(LsmHost &H, size_t nq, uint32_t F, int priority, std::string &err);

// Queries one batch may hold (the plan grid and the per-(query, block) work
// of the object kernel are bounded by queries x retained blocks <= 65535).
size_t lsm_query_chunk(const LsmHost &H);

// Runs a batch of at most lsm_query_chunk(H) queries over the retained blocks
// on query lane `lane` (-1: the first free lane, else lane 0 once it frees)
// (see stc_query_batch in include/stc.h). device_limit (0 = none) bounds the
// match records the device output may hold: a batch with more matches is
// only counted (offsets and counts filled, out untouched). gpu_ms (optional)
// receives the batch's span on its lane's stream, from its first copy to its
// last (waits for SMs included).
stc_status lsm_query(LsmHost &H, int lane, const stc_query *q, size_t nq, stc_contact *out, size_t cap,
                     uint64_t *offsets, uint64_t *counts, std::string &err, size_t device_limit = 0,
                     float *gpu_ms = nullptr);

// Host restatement of CTF::get_ctf_bits (tracing/step_merge.cpp:140-186);
// returns false when the key would exceed 64 box bits or 128 key bits.
bool ctf_bits(const float mbr[4], const double map[4], uint32_t num_objects, uint32_t max_meet_time,
              stc_ctf *c);

}  // namespace stc
