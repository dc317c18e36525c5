// Device buffers of one pipeline context and the per-step launchers.
#pragma once
#include "stc_common.cuh"
#include "stc_schema.cuh"

namespace stc {

// sorig flag: the member's strip is ordered by longitude offset
#define STRIP_XSORTED (1u << 22)
// Candidate positions per refinement job and lane: a row block's candidate
// ranges are cut into chunks of this many, so that the n^2 / 2 pair tests of
// a dense leaf spread over many warps.
constexpr uint32_t REFINE_CHUNK_DEFAULT = 256;  // tile length before the first step's density is known

struct PipeDev {
  // sizes
  uint32_t N, leaf_cap, G, S;
  unsigned long long B;            // meeting table slots
  unsigned long long B_magic;      // ceil(2^64 / B) for fast_mod
  unsigned long long C;            // candidate set slots (power of two)
  unsigned long long cand_cap;     // candidate list capacity
  unsigned long long E;            // emit buffer capacity
  unsigned long long U_cap;        // border units (refine_size*N - N - 1)
  // parameters
  double reach, x_buffer, y_buffer;
  double map_lo_x, map_lo_y, map_hi_x, map_hi_y;
  float fmap_lo_x, fmap_lo_y, fmap_hi_x, fmap_hi_y;  // float f: f >= map_lo <=> f >= fmap_lo, etc.
  uint32_t min_meet_time, grid_capacity, delay;
  int mbr_filter;
  uint32_t slices;                 // launches per long step kernel (stc_config.step_slices)
  uint32_t job_chunk;              // refinement jobs a warp takes at a time (stc_config.job_chunk)
  uint32_t direct_hits;            // pair tests write hit records directly (dense steps), not via a queue
  uint32_t refine_chunk;               // candidate positions per refinement job (a multiple of 32)
  uint32_t refine_bps, hits_bps;   // blocks per SM of the pair tests and of the table update
  // state
  DevState *st;
  SchemaDev sd;
  SchemaWork sw;
  const double2 *xy;               // positions of the current step
  const double2 *xy_in = nullptr;  // when set: page-locked host positions the descent reads and
                                   // copies to xy (a buffer of the context's own)
  // partition
  uint32_t *leaf_gid, *lastvalid, *iota, *sorted_gid, *sorted_pid, *sort_ktmp, *sort_vtmp, *sort_hist;
  uint32_t *grid_count, *grid_start;   // G, G+1
  float4 *pts;                          // N sorted: lx, ly, metres/deg lon, pid bits
  float2 *fxy;                          // N by pid: float lon, lat (MBR of new meetings)
  float2 *gfxy;                         // N in leaf order (pid order within a leaf): fxy of each member
  float2 *sfxy;                         // N in strip order (as spts): fxy of each member
  // each leaf's kept members again, ordered by horizontal strip (strips at
  // least reach tall) and, within a small strip, by longitude: spts as pts;
  // sorig = member index in pid order | strip << 16 | STRIP_XSORTED;
  // scand = the member's candidate ranges within the leaf: [i + 1, x & 0xFFFF)
  // in its strip and [x >> 16, y) in the next; lstrip[g] = (strips per degree
  // of latitude from the leaf's low corner, strip count, longitude window wx
  // in degrees, 0)
  float4 *spts;
  uint32_t *sorig;
  uint2 *scand;
  float4 *lstrip;
  uint32_t *cchunks;                    // G: candidate chunks of refine_chunk per own row block
  // border units
  uint32_t *bcount, *boff;              // N+1 (border units per pid, exclusive offsets)
  uint32_t *blist;                      // N: pids of border points (any order)
  uint32_t *bres;                       // 4N: first four lookup results per border point
  float border_delta;                   // fp32 band (metres) of the border lookup pre-filter
  uint32_t *bu_gid, *bu_pid;            // U_cap (rank order)
  uint32_t *bu_sorted_gid, *bu_sorted_pos;  // U_cap grouped by leaf
  uint32_t *bu_cnt, *bu_start;          // G+1
  uint32_t *job_cnt, *job_start;        // G+1
  // meetings
  Slot *slots;                          // B
  HitRec *hits;                         // hit_cap: hits of the step, applied by k_hits
  unsigned long long hit_cap;
  unsigned long long *hit_bounds;       // [MAX_PARTS + 1]: hit buffer end after each part of the pair tests
  Cand *cset;                           // C
  uint32_t *cand_list;                  // cand_cap
  stc_meeting *emit;                    // E
  uint32_t *scan_tmp;
  // scratch of the border units' scan and sort, which run on the side
  // stream beside the leaf-order sort
  uint32_t *scan_tmp2, *sort_ktmp2, *sort_vtmp2, *sort_hist2;
  unsigned long long *n_dev;            // device copy of N (for radix sort)
};

// stc_partition.cu
// partition in two parts: the descent (leaf of every object, border
// candidates), then the leaf-order sort, leaf starts and gathered points
void step_descend(PipeDev &p, cudaStream_t s);
void step_leaf_order(PipeDev &p, cudaStream_t s);
// each leaf's members in strip order (after step_leaf_order)
void step_strips(PipeDev &p, cudaStream_t s);
void step_border(PipeDev &p, cudaStream_t s);
void step_jobs(PipeDev &p, cudaStream_t s);
// stc_refine.cu
// refinement in two parts: the pair tests (which read the leaves' node
// boxes) and the table update of their hits
// Part `part` of `parts` of the pair tests, then the mark of its hit range;
// the table update of that range (k_hits) may run beside the next part.
constexpr uint32_t STC_MAX_PARTS = 64;
void step_pairs_part(PipeDev &p, uint32_t part, uint32_t parts, cudaStream_t s);
void step_hits_part(PipeDev &p, uint32_t part, uint32_t parts, cudaStream_t s);
// stc_meetings.cu
void step_insert(PipeDev &p, cudaStream_t s);
void step_sweep(PipeDev &p, cudaStream_t s);
void init_tables(PipeDev &p, cudaStream_t s);
void step_begin(PipeDev &p, const uint32_t *t_pinned, cudaStream_t s);

}  // namespace stc
