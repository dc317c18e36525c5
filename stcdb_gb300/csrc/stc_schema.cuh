// Quadtree schema on the device: build at create, dynamic update per step.
#pragma once
#include "stc_common.cuh"

namespace stc {

struct SchemaDev {
  Node *nodes;            // S
  NodeMeta *meta;         // S
  uint32_t *schema_stack; // S
  uint32_t *grids_stack;  // G
  uint32_t *gid_node;     // G: leaf grid id -> node index
  float4 *fbox;           // S: node box in fp32 degrees relative to (ox, oy)
  double ox, oy;          // map origin for fbox
  uint32_t S, G;
};

struct SchemaWork {
  // build temporaries
  Node *bnodes;
  NodeMeta *bmeta;
  uint32_t *bcount, *bsub_nodes, *bsub_leaves, *bpre, *bleafbase;
  uint32_t *node_of;      // N
  uint32_t *level_start;  // host mirror kept in SchemaBuilder
  // update temporaries
  uint32_t *ev_flag;      // S (0 none, 1 split, 2 merge)
  uint32_t *ev_pos;       // S
  uint32_t *ev_list;      // S
  int16_t *old_under;     // S
  uint32_t *heap;         // S
  unsigned long long *ev_total;
  uint8_t *queued;        // S
  uint32_t *scan_tmp;
  uint32_t *par_scratch;  // 9 * 4096 words for the block replay
};

// Builds the schema from step-0 positions (index/QTree.h:157-311 semantics:
// a node splits iff at least grid_capacity points descend into it and its
// geographic width / 2 exceeds reach). Returns cudaSuccess or an error; on a
// capacity problem sets st->error = ERR_BUILD.
cudaError_t build_schema(const double2 *xy, uint32_t n, const double mbr[4], double reach,
                         uint32_t grid_capacity, SchemaDev sd, SchemaWork w, DevState *st, DevState *st_host,
                         cudaStream_t s);

// Dynamic update after a step (tracing/filter.cpp:377-449).
// serial_only forces the one-thread replay (the parallel one is used when it applies).
// Kernel attributes the schema update needs, set once per device before any
// step is issued (outside a stream capture).
cudaError_t schema_prepare();
void update_schema(SchemaDev sd, SchemaWork w, uint32_t *grid_count, double reach, uint32_t grid_capacity,
                   uint32_t delay, int serial_only, DevState *st, cudaStream_t s);

}  // namespace stc
