// Quadtree schema: GPU build and per-step dynamic update.
//
// Build (index/QTree.h:157-311, tracing/filter.cpp:27-93): the reference
// inserts points one by one and splits a leaf as soon as it holds
// grid_capacity objects and width(true)/2 > reach. Objects only ever get
// added, so the final tree does not depend on insertion order: a node is
// split iff the number of step-0 points that descend into it is at least
// grid_capacity and the width condition holds. The build therefore runs level
// by level (count points per node of the level, decide splits, move points
// to children), then numbers nodes in preorder with children 0..3
// (QTNode::create_schema) and leaves in depth-first order (QTNode::set_id).
//
// Update (tracing/filter.cpp:316-449): the reference visits nodes 0..S-1 in
// order. Phase 1 evaluates every node in parallel against the pre-sweep
// state; the only way an earlier visit changes a later decision is a merge
// that turns a branch into a leaf before its parent (higher index) is
// visited, so phase 2 replays the flagged events in index order on one
// thread, with those parents queued for re-evaluation at their own index.
// Stack pops and pushes happen in exactly the reference's order.
#include <vector>

#include "stc_schema.cuh"

namespace stc {

__device__ __forceinline__ double dpml_fast(double lat) {
  double absla = fabs(lat);
  if (absla == 90) absla = 89;
  double arg = RN_DIV(RN_MUL(RN_SUB(90.0, absla), STC_REF_PI), 180.0);
  return RN_DIV(360.0, RN_MUL(RN_MUL(sin(arg), 40076.0), 1000.0));
}

// Geographic width of a box (geometry/geometry.h:166-172), returning the
// value computed with the correctly rounded sine whenever the comparison
// against thr could depend on the last bits of the fast one.
__device__ double width_geo(double lx, double ly, double hx, double thr) {
  double w = RN_DIV(RN_SUB(hx, lx), dpml_fast(ly));
  if (fabs(w - thr) > 1e-12 * fabs(thr)) return w;
  return RN_DIV(RN_SUB(hx, lx), stc_dpml_ref(ly));
}

__device__ __forceinline__ void set_child_box(Node &c, const Node &p, int i) {
  // QTNode::split children (index/QTree.h:163-166)
  double lx = (i & 1) ? p.mid_x : p.lo_x;
  double hx = (i & 1) ? p.hi_x : p.mid_x;
  double ly = (i & 2) ? p.mid_y : p.lo_y;
  double hy = (i & 2) ? p.hi_y : p.mid_y;
  c.lo_x = lx; c.lo_y = ly; c.hi_x = hx; c.hi_y = hy;
  c.mid_x = RN_DIV(RN_ADD(hx, lx), 2.0);
  c.mid_y = RN_DIV(RN_ADD(hy, ly), 2.0);
  c.child[0] = c.child[1] = c.child[2] = c.child[3] = STC_NONE;
}

__global__ void k_build_root(Node *bn, NodeMeta *bm, double lx, double ly, double hx, double hy, uint32_t *node_of,
                             uint32_t n, DevState *st) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    Node r;
    r.lo_x = lx; r.lo_y = ly; r.hi_x = hx; r.hi_y = hy;
    r.mid_x = RN_DIV(RN_ADD(hx, lx), 2.0);
    r.mid_y = RN_DIV(RN_ADD(hy, ly), 2.0);
    r.child[0] = r.child[1] = r.child[2] = r.child[3] = STC_NONE;
    bn[0] = r;
    NodeMeta m;
    m.type = NODE_LEAF; m.level = 0; m.overflow = 0; m.underflow = 0; m.grid_id = 0; m.parent = STC_NONE;
    bm[0] = m;
    st->build_nodes = 1;
  }
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) node_of[i] = 0;
}

__global__ void k_build_count(const uint32_t *node_of, uint32_t n, uint32_t a, uint32_t *bcount) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t nid = node_of[i];
  if (nid >= a) atomicAdd(&bcount[nid], 1u);
}

__global__ void k_build_decide(Node *bn, NodeMeta *bm, const uint32_t *bcount, uint32_t a, uint32_t b,
                               uint32_t cap, double reach, uint32_t S, DevState *st) {
  uint32_t nid = a + blockIdx.x * blockDim.x + threadIdx.x;
  if (nid >= b) return;
  Node p = bn[nid];
  bool split = false;
  if (bcount[nid] >= cap) {
    double w = width_geo(p.lo_x, p.lo_y, p.hi_x, RN_MUL(reach, 2.0));
    split = RN_DIV(w, 2.0) > reach;
  }
  if (!split) {
    bm[nid].type = NODE_LEAF;
    return;
  }
  uint32_t c = atomicAdd(&st->build_nodes, 4u);
  if (c + 4 > S) {
    stc_set_error(st, ERR_BUILD, c);
    bm[nid].type = NODE_LEAF;
    return;
  }
  NodeMeta pm = bm[nid];
  for (int i = 0; i < 4; i++) {
    Node ch;
    set_child_box(ch, p, i);
    bn[c + i] = ch;
    NodeMeta m;
    m.type = NODE_LEAF; m.level = (int16_t)(pm.level + 1); m.overflow = 0; m.underflow = 0;
    m.grid_id = 0; m.parent = nid;
    bm[c + i] = m;
    p.child[i] = c + i;
  }
  bn[nid] = p;
  bm[nid].type = NODE_BRANCH;
}

__global__ void k_build_move(const double2 *xy, uint32_t *node_of, uint32_t n, uint32_t a, const Node *bn,
                             const NodeMeta *bm) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t nid = node_of[i];
  if (nid < a || bm[nid].type != NODE_BRANCH) return;
  double2 p = xy[i];
  const Node &q = bn[nid];
  int loc = (p.y > q.mid_y) * 2 + (p.x > q.mid_x);  // QTree.h:191
  node_of[i] = q.child[loc];
}

__global__ void k_build_sub(const Node *bn, const NodeMeta *bm, uint32_t a, uint32_t b, uint32_t *sub_nodes,
                            uint32_t *sub_leaves) {
  uint32_t nid = a + blockIdx.x * blockDim.x + threadIdx.x;
  if (nid >= b) return;
  if (bm[nid].type == NODE_LEAF) {
    sub_nodes[nid] = 1;
    sub_leaves[nid] = 1;
    return;
  }
  uint32_t sn = 1, sl = 0;
  for (int i = 0; i < 4; i++) {
    uint32_t c = bn[nid].child[i];
    sn += sub_nodes[c];
    sl += sub_leaves[c];
  }
  sub_nodes[nid] = sn;
  sub_leaves[nid] = sl;
}

__global__ void k_build_pre_children(const Node *bn, const NodeMeta *bm, uint32_t a, uint32_t b,
                                     const uint32_t *sub_nodes, const uint32_t *sub_leaves, uint32_t *pre,
                                     uint32_t *leafbase) {
  uint32_t nid = a + blockIdx.x * blockDim.x + threadIdx.x;
  if (nid >= b || bm[nid].type != NODE_BRANCH) return;
  uint32_t run = pre[nid] + 1, lb = leafbase[nid];
  for (int i = 0; i < 4; i++) {
    uint32_t c = bn[nid].child[i];
    pre[c] = run;
    leafbase[c] = lb;
    run += sub_nodes[c];
    lb += sub_leaves[c];
  }
}

__global__ void k_build_write(const Node *bn, const NodeMeta *bm, uint32_t total, const uint32_t *pre,
                              const uint32_t *leafbase, SchemaDev sd) {
  uint32_t nid = blockIdx.x * blockDim.x + threadIdx.x;
  if (nid >= total) return;
  uint32_t p = pre[nid];
  Node q = bn[nid];
  NodeMeta m = bm[nid];
  if (m.type == NODE_BRANCH) {
    for (int i = 0; i < 4; i++) q.child[i] = pre[q.child[i]];
    m.grid_id = 0;  // QTNode::node_id of a branch keeps its default 0
  } else {
    m.grid_id = leafbase[nid];
    if (m.grid_id < sd.G) sd.gid_node[m.grid_id] = p;  // overflow is reported by k_build_finish
  }
  m.parent = m.parent == STC_NONE ? STC_NONE : pre[m.parent];
  m.overflow = 0;
  m.underflow = 0;
  sd.nodes[p] = q;
  sd.meta[p] = m;
  sd.fbox[p] = make_float4(__double2float_rn(RN_SUB(q.lo_x, sd.ox)), __double2float_rn(RN_SUB(q.lo_y, sd.oy)),
                           __double2float_rn(RN_SUB(q.hi_x, sd.ox)), __double2float_rn(RN_SUB(q.hi_y, sd.oy)));
}

__global__ void k_build_finish(const uint32_t *sub_nodes, const uint32_t *sub_leaves, uint32_t S, uint32_t G,
                               DevState *st) {
  uint32_t nodes = sub_nodes[0], leaves = sub_leaves[0];
  // tracing/filter.cpp:82-85 asserts strict inequality
  if (nodes >= S || leaves >= G) stc_set_error(st, ERR_BUILD, nodes);
  st->schema_stack_index = nodes;
  st->grids_stack_index = leaves;
}

static inline unsigned nblk(size_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

cudaError_t build_schema(const double2 *xy, uint32_t n, const double mbr[4], double reach, uint32_t grid_capacity,
                         SchemaDev sd, SchemaWork w, DevState *st, DevState *st_host, cudaStream_t s) {
  cudaMemsetAsync(sd.meta, 0, (size_t)sd.S * sizeof(NodeMeta), s);
  iota_u32(sd.schema_stack, sd.S, s);
  iota_u32(sd.grids_stack, sd.G, s);
  STC_KL k_build_root<<<nblk(n > 0 ? n : 1), 256, 0, s>>>(w.bnodes, w.bmeta, mbr[0], mbr[1], mbr[2], mbr[3], w.node_of, n,
                                                   st);
  std::vector<uint32_t> ls = {0, 1};
  for (int level = 0; level < STC_MAX_DEPTH; level++) {
    uint32_t a = ls[ls.size() - 2], b = ls.back();
    cudaMemsetAsync(w.bcount + a, 0, (size_t)(b - a) * sizeof(uint32_t), s);
    if (n) STC_KL k_build_count<<<nblk(n), 256, 0, s>>>(w.node_of, n, a, w.bcount);
    STC_KL k_build_decide<<<nblk(b - a), 256, 0, s>>>(w.bnodes, w.bmeta, w.bcount, a, b, grid_capacity, reach, sd.S, st);
    if (n) STC_KL k_build_move<<<nblk(n), 256, 0, s>>>(xy, w.node_of, n, a, w.bnodes, w.bmeta);
    cudaError_t e = cudaMemcpyAsync(st_host, st, sizeof(DevState), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    if (st_host->error) return cudaSuccess;
    uint32_t total = st_host->build_nodes;
    if (total == b) break;
    ls.push_back(total);
  }
  uint32_t total = ls.back();
  int nlev = (int)ls.size() - 1;
  for (int L = nlev - 1; L >= 0; L--) {
    uint32_t a = ls[L], b = ls[L + 1];
    STC_KL k_build_sub<<<nblk(b - a), 256, 0, s>>>(w.bnodes, w.bmeta, a, b, w.bsub_nodes, w.bsub_leaves);
  }
  cudaMemsetAsync(w.bpre, 0, sizeof(uint32_t), s);  // root: preorder 0, first leaf id 0
  cudaMemsetAsync(w.bleafbase, 0, sizeof(uint32_t), s);
  for (int L = 0; L < nlev; L++) {
    uint32_t a = ls[L], b = ls[L + 1];
    STC_KL k_build_pre_children<<<nblk(b - a), 256, 0, s>>>(w.bnodes, w.bmeta, a, b, w.bsub_nodes, w.bsub_leaves, w.bpre,
                                                     w.bleafbase);
  }
  STC_KL k_build_write<<<nblk(total), 256, 0, s>>>(w.bnodes, w.bmeta, total, w.bpre, w.bleafbase, sd);
  STC_KL k_build_finish<<<1, 1, 0, s>>>(w.bsub_nodes, w.bsub_leaves, sd.S, sd.G, st);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Dynamic update.

enum { EV_NONE = 0, EV_SPLIT = 1, EV_MERGE = 2 };

__global__ void k_flags_to_bits(const uint32_t *flag, uint32_t *bits, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) bits[i] = flag[i] ? 1u : 0u;
}

__global__ void k_schema_phase1(SchemaDev sd, const uint32_t *grid_count, double reach, uint32_t cap, uint32_t delay,
                                uint32_t *ev_flag, int16_t *old_under) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sd.S) return;
  NodeMeta m = sd.meta[i];
  uint32_t flag = EV_NONE;
  old_under[i] = m.underflow;
  if (m.type == NODE_LEAF) {
    bool cond = false;
    if (grid_count[m.grid_id] > cap) {
      const Node &q = sd.nodes[i];
      double thr = RN_MUL(reach, 2.0);
      cond = width_geo(q.lo_x, q.lo_y, q.hi_x, thr) > thr;
    }
    int16_t nv = cond ? (int16_t)(m.overflow + 1) : (int16_t)0;
    if (cond && (uint32_t)nv >= delay) flag = EV_SPLIT;
    else sd.meta[i].overflow = nv;
  } else if (m.type == NODE_BRANCH) {
    const Node &q = sd.nodes[i];
    int leafchild = 0;
    int ncounter = 0;
    for (int k = 0; k < 4; k++) {
      NodeMeta cm = sd.meta[q.child[k]];
      if (cm.type == NODE_LEAF) {
        leafchild++;
        ncounter += (int)grid_count[cm.grid_id];
      }
    }
    bool cond = leafchild == 4 && (uint32_t)ncounter < cap;
    int16_t nv = cond ? (int16_t)(m.underflow + 1) : (int16_t)0;
    if (cond && (uint32_t)nv >= delay) flag = EV_MERGE;
    else sd.meta[i].underflow = nv;
  }
  ev_flag[i] = flag;
}

__global__ void k_schema_compact(const uint32_t *ev_flag, const uint32_t *ev_pos, uint32_t S, uint32_t *ev_list) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S) return;
  if (ev_flag[i]) ev_list[ev_pos[i]] = (i << 2) | ev_flag[i];
}

__device__ bool split_node(SchemaDev sd, uint32_t cur, uint32_t *grid_count, DevState *st) {
  // tracing/filter.cpp:338-375
  NodeMeta cm = sd.meta[cur];
  cm.type = NODE_BRANCH;
  if (st->grids_stack_index == 0) return false;
  sd.grids_stack[--st->grids_stack_index] = cm.grid_id;
  Node q = sd.nodes[cur];
  double xhalf = RN_SUB(q.mid_x, q.lo_x);
  double yhalf = RN_SUB(q.mid_y, q.lo_y);
  for (int i = 0; i < 4; i++) {
    if (st->schema_stack_index >= sd.S || st->grids_stack_index >= sd.G) return false;
    uint32_t child = sd.schema_stack[st->schema_stack_index++];
    q.child[i] = child;
    uint32_t g = sd.grids_stack[st->grids_stack_index++];
    grid_count[g] = 0;
    sd.gid_node[g] = child;
    Node c;
    c.lo_x = RN_ADD(q.lo_x, (i % 2 == 1) ? xhalf : 0.0);
    c.lo_y = RN_ADD(q.lo_y, (i / 2 == 1) ? yhalf : 0.0);
    c.hi_x = RN_ADD(q.mid_x, (i % 2 == 1) ? xhalf : 0.0);
    c.hi_y = RN_ADD(q.mid_y, (i / 2 == 1) ? yhalf : 0.0);
    c.mid_x = RN_DIV(RN_ADD(c.lo_x, c.hi_x), 2.0);
    c.mid_y = RN_DIV(RN_ADD(c.lo_y, c.hi_y), 2.0);
    c.child[0] = c.child[1] = c.child[2] = c.child[3] = STC_NONE;
    sd.nodes[child] = c;
    sd.fbox[child] = make_float4(__double2float_rn(RN_SUB(c.lo_x, sd.ox)), __double2float_rn(RN_SUB(c.lo_y, sd.oy)),
                                 __double2float_rn(RN_SUB(c.hi_x, sd.ox)), __double2float_rn(RN_SUB(c.hi_y, sd.oy)));
    NodeMeta m;
    m.type = NODE_LEAF; m.level = (int16_t)(cm.level + 1); m.overflow = 0; m.underflow = 0;
    m.grid_id = g; m.parent = cur;
    sd.meta[child] = m;
  }
  sd.nodes[cur] = q;
  cm.overflow = 0;
  sd.meta[cur] = cm;
  return true;
}

__device__ bool merge_node(SchemaDev sd, uint32_t cur, uint32_t *grid_count, DevState *st) {
  // tracing/filter.cpp:316-336
  Node q = sd.nodes[cur];
  for (int i = 0; i < 4; i++) {
    uint32_t ch = q.child[i];
    NodeMeta m = sd.meta[ch];
    sd.meta[ch].type = NODE_INVALID;
    if (st->schema_stack_index == 0 || st->grids_stack_index == 0) return false;
    sd.schema_stack[--st->schema_stack_index] = ch;
    sd.grids_stack[--st->grids_stack_index] = m.grid_id;
    grid_count[m.grid_id] = 0;
  }
  NodeMeta cm = sd.meta[cur];
  cm.type = NODE_LEAF;
  cm.grid_id = sd.grids_stack[st->grids_stack_index++];
  cm.underflow = 0;
  sd.gid_node[cm.grid_id] = cur;
  sd.meta[cur] = cm;
  return true;
}

// binary min-heap of node indices in global memory (single thread)
__device__ void heap_push(uint32_t *h, uint32_t &n, uint32_t v) {
  uint32_t i = n++;
  h[i] = v;
  while (i > 0) {
    uint32_t p = (i - 1) / 2;
    if (h[p] <= h[i]) break;
    uint32_t t = h[p]; h[p] = h[i]; h[i] = t;
    i = p;
  }
}

__device__ uint32_t heap_pop(uint32_t *h, uint32_t &n) {
  uint32_t top = h[0];
  h[0] = h[--n];
  uint32_t i = 0;
  while (true) {
    uint32_t l = 2 * i + 1, r = l + 1, m = i;
    if (l < n && h[l] < h[m]) m = l;
    if (r < n && h[r] < h[m]) m = r;
    if (m == i) break;
    uint32_t t = h[m]; h[m] = h[i]; h[i] = t;
    i = m;
  }
  return top;
}


// Block replay of the flagged events for the common case: at most
// PAR_MAX_EVENTS events and no merge whose parent has a higher index (the
// only source of a cascade). Without cascades every event's decision is fixed
// by phase 1, and the sequential replay's only coupling is through the two
// free stacks: a split pushes its own grid id, then pops 4 node slots and 4
// grid ids; a merge pushes its 4 children and their grid ids and pops the last
// one back. The events touch at most 4 stack positions each side of where the
// step starts, so one thread replays just the stack operations, in event
// order, on windows of both stacks held in shared memory; all node and grid
// bookkeeping is then written in parallel, merges before splits (a node or
// grid id freed by a merge can only be reused by a later split). The per-step
// grid counts are not reset: nothing reads them before the next step
// recounts. Sets *done; k_schema_phase2 then does nothing.
static constexpr uint32_t PAR_MAX_EVENTS = 4096;
static constexpr uint32_t PAR_WIN = 4 * PAR_MAX_EVENTS + 8;  // stack positions one step can touch
static constexpr size_t PAR_SMEM = (size_t)PAR_MAX_EVENTS * 5 + (size_t)2 * PAR_WIN * 4;  // 148 KB

// Per-event scratch in global memory: popped / pushed values.
struct ParScratch {
  uint32_t *node;
  uint32_t *val;  // 8 per event: split -> 4 children, 4 grid ids; merge -> 4 children, 4 grid ids
};

__device__ __forceinline__ ParScratch par_scratch(uint32_t *base, uint32_t cap) {
  ParScratch ps;
  ps.node = base;
  ps.val = base + cap;
  return ps;
}

__global__ void __launch_bounds__(1024) k_schema_phase2_par(SchemaDev sd, const uint32_t *ev_list,
                                                            const unsigned long long *ev_total, unsigned int *done,
                                                            int serial_only, uint32_t *scratch, DevState *st) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t *sh_node = (uint32_t *)smem;                              // PAR_MAX_EVENTS
  uint32_t *swin = sh_node + PAR_MAX_EVENTS;                          // PAR_WIN: schema stack window
  uint32_t *gwin = swin + PAR_WIN;                                    // PAR_WIN: grid stack window
  uint8_t *sh_kind = (uint8_t *)(gwin + PAR_WIN);                    // PAR_MAX_EVENTS
  __shared__ int cascade;
  __shared__ uint32_t n_merges;
  const uint32_t tid = threadIdx.x;
  uint32_t nev = (uint32_t)*ev_total;
  if (tid == 0) {
    *done = 0;
    cascade = 0;
    n_merges = 0;
    st->schema_path = 0;
  }
  if (nev > PAR_MAX_EVENTS || serial_only) return;
  ParScratch ps = par_scratch(scratch, PAR_MAX_EVENTS);
  const int ssi0 = (int)st->schema_stack_index, gsi0 = (int)st->grids_stack_index;
  __syncthreads();
  for (uint32_t e = tid; e < nev; e += blockDim.x) {
    uint32_t v = ev_list[e];
    uint32_t node = v >> 2, kind = v & 3u;
    sh_node[e] = node;
    sh_kind[e] = (uint8_t)kind;
    if (kind == EV_MERGE) {
      atomicAdd(&n_merges, 1u);
      uint32_t par = sd.meta[node].parent;
      if (node != 0 && par != STC_NONE && par > node) cascade = 1;
      Node q = sd.nodes[node];
      for (int i = 0; i < 4; i++) {
        ps.val[8 * e + i] = q.child[i];
        ps.val[8 * e + 4 + i] = sd.meta[q.child[i]].grid_id;
      }
    } else {
      ps.val[8 * e + 4] = sd.meta[node].grid_id;  // the split pushes this first
    }
  }
  __syncthreads();
  // merges move the stack indices down by 4 each, splits up by 4 (schema) and
  // at most 4 (grid): the window [idx0 - 4 merges - 4, +PAR_WIN) holds every
  // position the step touches
  const int sbase = ssi0 - 4 * (int)n_merges - 4, gbase = gsi0 - 4 * (int)n_merges - 4;
  for (uint32_t k = tid; k < PAR_WIN; k += blockDim.x) {
    int qs = sbase + (int)k, qg = gbase + (int)k;
    swin[k] = (qs >= 0 && qs < (int)sd.S) ? sd.schema_stack[qs] : STC_NONE;
    gwin[k] = (qg >= 0 && qg < (int)sd.G) ? sd.grids_stack[qg] : STC_NONE;
  }
  __syncthreads();
  if (cascade) {
    if (tid == 0) st->schema_path = 2;
    return;
  }
  if (tid == 0) {
    // the stack operations of tracing/filter.cpp:316-375, in event order
    int si = ssi0 - sbase, gi = gsi0 - gbase;
    bool bad = false;
    for (uint32_t e = 0; e < nev && !bad; e++) {
      uint32_t *v = ps.val + 8 * e;
      if (sh_kind[e] == EV_SPLIT) {
        if (si + 4 + sbase > (int)sd.S || gi - 1 + gbase < 0 || gi + 3 + gbase > (int)sd.G) { bad = true; break; }
        gwin[--gi] = v[4];
        for (int i = 0; i < 4; i++) {
          v[i] = swin[si++];
          v[4 + i] = gwin[gi++];
        }
      } else {
        if (si - 4 + sbase < 0 || gi - 4 + gbase < 0) { bad = true; break; }
        for (int i = 0; i < 4; i++) {
          swin[--si] = v[i];
          gwin[--gi] = v[4 + i];
        }
        gi++;  // pops the last pushed grid id back for the merged node (v[7])
      }
    }
    if (bad) stc_set_error(st, ERR_SCHEMA, 0u);
    st->schema_stack_index = (uint32_t)(si + sbase);
    st->grids_stack_index = (uint32_t)(gi + gbase);
  }
  __syncthreads();
  if (st->error) return;
  // stack windows back to global memory
  for (uint32_t k = tid; k < PAR_WIN; k += blockDim.x) {
    int qs = sbase + (int)k, qg = gbase + (int)k;
    if (qs >= 0 && qs < (int)sd.S) sd.schema_stack[qs] = swin[k];
    if (qg >= 0 && qg < (int)sd.G) sd.grids_stack[qg] = gwin[k];
  }
  // merges (tracing/filter.cpp:316-336)
  for (uint32_t e = tid; e < nev; e += blockDim.x) {
    if (sh_kind[e] != EV_MERGE) continue;
    uint32_t cur = sh_node[e];
    const uint32_t *v = ps.val + 8 * e;
    for (int i = 0; i < 4; i++) sd.meta[v[i]].type = NODE_INVALID;
    NodeMeta cm = sd.meta[cur];
    cm.type = NODE_LEAF;
    cm.grid_id = v[7];  // the pop returns the last pushed grid id
    cm.underflow = 0;
    sd.meta[cur] = cm;
    sd.gid_node[v[7]] = cur;
  }
  __syncthreads();
  // splits (tracing/filter.cpp:338-375)
  for (uint32_t e = tid; e < nev; e += blockDim.x) {
    if (sh_kind[e] != EV_SPLIT) continue;
    uint32_t cur = sh_node[e];
    const uint32_t *v = ps.val + 8 * e;
    Node q = sd.nodes[cur];
    NodeMeta cm = sd.meta[cur];
    double xhalf = RN_SUB(q.mid_x, q.lo_x);
    double yhalf = RN_SUB(q.mid_y, q.lo_y);
    for (int i = 0; i < 4; i++) {
      uint32_t child = v[i], gid = v[4 + i];
      Node c;
      c.lo_x = RN_ADD(q.lo_x, (i % 2 == 1) ? xhalf : 0.0);
      c.lo_y = RN_ADD(q.lo_y, (i / 2 == 1) ? yhalf : 0.0);
      c.hi_x = RN_ADD(q.mid_x, (i % 2 == 1) ? xhalf : 0.0);
      c.hi_y = RN_ADD(q.mid_y, (i / 2 == 1) ? yhalf : 0.0);
      c.mid_x = RN_DIV(RN_ADD(c.lo_x, c.hi_x), 2.0);
      c.mid_y = RN_DIV(RN_ADD(c.lo_y, c.hi_y), 2.0);
      c.child[0] = c.child[1] = c.child[2] = c.child[3] = STC_NONE;
      sd.nodes[child] = c;
      sd.fbox[child] = make_float4(__double2float_rn(RN_SUB(c.lo_x, sd.ox)), __double2float_rn(RN_SUB(c.lo_y, sd.oy)),
                                   __double2float_rn(RN_SUB(c.hi_x, sd.ox)), __double2float_rn(RN_SUB(c.hi_y, sd.oy)));
      NodeMeta m;
      m.type = NODE_LEAF; m.level = (int16_t)(cm.level + 1); m.overflow = 0; m.underflow = 0;
      m.grid_id = gid; m.parent = cur;
      sd.meta[child] = m;
      sd.gid_node[gid] = child;
      q.child[i] = child;
    }
    sd.nodes[cur] = q;
    cm.type = NODE_BRANCH;
    cm.overflow = 0;
    sd.meta[cur] = cm;
  }
  __syncthreads();
  if (tid == 0) {
    uint32_t splits = 0, merges = 0;
    for (uint32_t e = 0; e < nev; e++) (sh_kind[e] == EV_SPLIT ? splits : merges)++;
    st->splits = splits;
    st->merges = merges;
    st->events = nev;
    st->schema_path = 1;
    *done = 1;
  }
}

__global__ void k_schema_phase2(SchemaDev sd, uint32_t *grid_count, const uint32_t *ev_list,
                                const unsigned long long *ev_total, const int16_t *old_under, uint32_t *heap,
                                uint8_t *queued, uint32_t cap, uint32_t delay, const unsigned int *done,
                                DevState *st) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (*done) return;  // handled by k_schema_phase2_par
  uint32_t nev = (uint32_t)*ev_total;
  uint32_t hn = 0, ei = 0;
  uint32_t splits = 0, merges = 0;
  while (ei < nev || hn > 0) {
    uint32_t ev_node = ei < nev ? (ev_list[ei] >> 2) : 0xFFFFFFFFu;
    uint32_t h_node = hn > 0 ? heap[0] : 0xFFFFFFFFu;
    if (h_node < ev_node) {
      uint32_t p = heap_pop(heap, hn);
      queued[p] = 0;
      // re-evaluate the branch rule at p's own visit (filter.cpp:399-420)
      NodeMeta pm = sd.meta[p];
      if (pm.type != NODE_BRANCH) continue;
      const Node &q = sd.nodes[p];
      int leafchild = 0, ncounter = 0;
      for (int k = 0; k < 4; k++) {
        NodeMeta cm = sd.meta[q.child[k]];
        if (cm.type == NODE_LEAF) {
          leafchild++;
          ncounter += (int)grid_count[cm.grid_id];
        }
      }
      bool cond = leafchild == 4 && (uint32_t)ncounter < cap;
      int16_t nv = cond ? (int16_t)(old_under[p] + 1) : (int16_t)0;
      if (cond && (uint32_t)nv >= delay) {
        if (!merge_node(sd, p, grid_count, st)) { stc_set_error(st, ERR_SCHEMA, p); return; }
        merges++;
        uint32_t pp = sd.meta[p].parent;
        if (p != 0 && pp != STC_NONE && pp > p && !queued[pp]) { queued[pp] = 1; heap_push(heap, hn, pp); }
      } else {
        sd.meta[p].underflow = nv;
      }
      continue;
    }
    if (h_node == ev_node) {  // an event node is never a pending parent; drop the duplicate
      heap_pop(heap, hn);
      queued[h_node] = 0;
    }
    uint32_t e = ev_list[ei++];
    uint32_t node = e >> 2, kind = e & 3u;
    if (kind == EV_SPLIT) {
      if (!split_node(sd, node, grid_count, st)) { stc_set_error(st, ERR_SCHEMA, node); return; }
      splits++;
    } else {
      if (!merge_node(sd, node, grid_count, st)) { stc_set_error(st, ERR_SCHEMA, node); return; }
      merges++;
      uint32_t pp = sd.meta[node].parent;
      if (node != 0 && pp != STC_NONE && pp > node && !queued[pp]) { queued[pp] = 1; heap_push(heap, hn, pp); }
    }
  }
  st->splits = splits;
  st->merges = merges;
  st->events = nev;
}

cudaError_t schema_prepare() {
  return cudaFuncSetAttribute(k_schema_phase2_par, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PAR_SMEM);
}

void update_schema(SchemaDev sd, SchemaWork w, uint32_t *grid_count, double reach, uint32_t grid_capacity,
                   uint32_t delay, int serial_only, DevState *st, cudaStream_t s) {
  STC_KL k_schema_phase1<<<nblk(sd.S), 256, 0, s>>>(sd, grid_count, reach, grid_capacity, delay, w.ev_flag, w.old_under);
  // ordered compaction of the flagged node indices: ev_pos = exclusive scan of (flag != 0)
  STC_KL k_flags_to_bits<<<nblk(sd.S), 256, 0, s>>>(w.ev_flag, w.ev_pos, sd.S);
  exclusive_scan_u32(w.ev_pos, w.ev_pos, sd.S, w.ev_total, w.scan_tmp, s);
  STC_KL k_schema_compact<<<nblk(sd.S), 256, 0, s>>>(w.ev_flag, w.ev_pos, sd.S, w.ev_list);
  unsigned int *done = (unsigned int *)(w.ev_total + 1);
  STC_KL k_schema_phase2_par<<<1, 1024, PAR_SMEM, s>>>(sd, w.ev_list, w.ev_total, done, serial_only, w.par_scratch,
                                                      st);
  STC_KL k_schema_phase2<<<1, 32, 0, s>>>(sd, grid_count, w.ev_list, w.ev_total, w.old_under, w.heap, w.queued,
                                   grid_capacity, delay, done, st);
}

}  // namespace stc
