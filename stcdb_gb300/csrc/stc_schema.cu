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


// Parallel replay of the flagged events for the common case: at most
// PAR_MAX_EVENTS events and no merge whose parent has a higher index (the
// only source of a cascade). Without cascades every event's decision is fixed
// by phase 1, and the sequential replay's only coupling is through the two
// free stacks: a split pops 4 node slots and, after pushing its own grid id,
// 4 grid ids (net +4 / +3); a merge pushes its 4 children and their grid ids
// and pops the last one back (net -4 / -3). Prefix sums give every event its
// stack positions; a pop reads the most recent earlier push to its position
// (or the stack's old content); merges are applied before splits because a
// node or grid id freed by a merge can only be reused by a later split. The
// per-step grid counts are not reset: nothing reads them before the next
// step recounts. Sets *done; k_schema_phase2 then does nothing.
static constexpr uint32_t PAR_MAX_EVENTS = 4096;  // event table in shared memory (36 KB)

// Per-event scratch of the parallel replay (global memory, 10 words per event).
struct ParScratch {
  uint32_t *node;
  int32_t *s0, *g0;
  uint32_t *kind, *spush, *gpush;  // spush/gpush: 4 per event
};

__device__ __forceinline__ ParScratch par_scratch(uint32_t *base, uint32_t cap) {
  ParScratch ps;
  ps.node = base;
  ps.s0 = (int32_t *)(base + cap);
  ps.g0 = (int32_t *)(base + 2 * (size_t)cap);
  ps.kind = base + 3 * (size_t)cap;
  ps.spush = base + 4 * (size_t)cap;
  ps.gpush = base + 8 * (size_t)cap;
  return ps;
}

__global__ void __launch_bounds__(1024) k_schema_phase2_par(SchemaDev sd, const uint32_t *ev_list,
                                                            const unsigned long long *ev_total, unsigned int *done,
                                                            int serial_only, uint32_t *scratch, DevState *st) {
  __shared__ int cascade;
  __shared__ uint32_t warp_s[32], warp_g[32];
  // stack positions and kinds of all events, scanned by the last-push searches
  __shared__ int32_t sh_s0[PAR_MAX_EVENTS], sh_g0[PAR_MAX_EVENTS];
  __shared__ uint8_t sh_kind[PAR_MAX_EVENTS];
  const uint32_t tid = threadIdx.x;
  uint32_t nev = (uint32_t)*ev_total;
  if (tid == 0) {
    *done = 0;
    cascade = 0;
    st->schema_path = 0;
  }
  if (nev > PAR_MAX_EVENTS || serial_only) return;
  ParScratch ps = par_scratch(scratch, PAR_MAX_EVENTS);
  __syncthreads();
  for (uint32_t e = tid; e < nev; e += blockDim.x) {
    uint32_t v = ev_list[e];
    uint32_t node = v >> 2, kind = v & 3u;
    ps.node[e] = node;
    ps.kind[e] = kind;
    sh_kind[e] = (uint8_t)kind;
    if (kind == EV_MERGE) {
      uint32_t par = sd.meta[node].parent;
      if (node != 0 && par != STC_NONE && par > node) cascade = 1;
    }
  }
  __syncthreads();
  if (cascade) {
    if (tid == 0) st->schema_path = 2;
    return;
  }
  // exclusive scan of the stack deltas (each thread owns a contiguous chunk)
  uint32_t per = (nev + blockDim.x - 1) / blockDim.x;
  uint32_t e0 = tid * per, e1 = min(nev, e0 + per);
  int ds = 0, dg = 0;
  for (uint32_t e = e0; e < e1; e++) {
    ds += sh_kind[e] == EV_SPLIT ? 4 : -4;
    dg += sh_kind[e] == EV_SPLIT ? 3 : -3;
  }
  uint32_t lane = tid & 31u, warp = tid >> 5;
  int is = ds, ig = dg;
  for (int o = 1; o < 32; o <<= 1) {
    int a = __shfl_up_sync(0xffffffffu, is, o), b = __shfl_up_sync(0xffffffffu, ig, o);
    if ((int)lane >= o) { is += a; ig += b; }
  }
  if (lane == 31) { warp_s[warp] = (uint32_t)is; warp_g[warp] = (uint32_t)ig; }
  __syncthreads();
  if (warp == 0) {
    int a = (int)warp_s[lane], b = (int)warp_g[lane];
    int ia = a, ib = b;
    for (int o = 1; o < 32; o <<= 1) {
      int x = __shfl_up_sync(0xffffffffu, ia, o), y = __shfl_up_sync(0xffffffffu, ib, o);
      if ((int)lane >= o) { ia += x; ib += y; }
    }
    warp_s[lane] = (uint32_t)(ia - a);
    warp_g[lane] = (uint32_t)(ib - b);
  }
  __syncthreads();
  int bs = (int)st->schema_stack_index + (int)warp_s[warp] + is - ds;
  int bg = (int)st->grids_stack_index + (int)warp_g[warp] + ig - dg;
  for (uint32_t e = e0; e < e1; e++) {
    ps.s0[e] = bs;
    ps.g0[e] = bg;
    sh_s0[e] = bs;
    sh_g0[e] = bg;
    bs += sh_kind[e] == EV_SPLIT ? 4 : -4;
    bg += sh_kind[e] == EV_SPLIT ? 3 : -3;
  }
  __syncthreads();
  // merges (tracing/filter.cpp:316-336); record every push
  for (uint32_t e = tid; e < nev; e += blockDim.x) {
    uint32_t cur = ps.node[e];
    int s0 = ps.s0[e], g0 = ps.g0[e];
    if (ps.kind[e] == EV_SPLIT) {
      ps.gpush[4 * e] = sd.meta[cur].grid_id;
      if (s0 + 4 > (int)sd.S || g0 < 1 || g0 + 3 > (int)sd.G) stc_set_error(st, ERR_SCHEMA, cur);
      continue;
    }
    if (s0 < 4 || g0 < 4) stc_set_error(st, ERR_SCHEMA, cur);
    Node q = sd.nodes[cur];
    uint32_t last_gid = 0;
    for (int i = 0; i < 4; i++) {
      uint32_t ch = q.child[i];
      uint32_t gid = sd.meta[ch].grid_id;
      sd.meta[ch].type = NODE_INVALID;
      ps.spush[4 * e + i] = ch;   // schema_stack[s0 - 1 - i]
      ps.gpush[4 * e + i] = gid;  // grids_stack[g0 - 1 - i]
      last_gid = gid;
    }
    NodeMeta cm = sd.meta[cur];
    cm.type = NODE_LEAF;
    cm.grid_id = last_gid;  // the pop returns the last pushed grid id
    cm.underflow = 0;
    sd.meta[cur] = cm;
    sd.gid_node[last_gid] = cur;
  }
  __syncthreads();
  if (!st->error) {
    // splits (tracing/filter.cpp:338-375)
    for (uint32_t e = tid; e < nev; e += blockDim.x) {
      if (ps.kind[e] != EV_SPLIT) continue;
      uint32_t cur = ps.node[e];
      int s0 = ps.s0[e], g0 = ps.g0[e];
      uint32_t child[4], gid[4];
      for (int i = 0; i < 4; i++) {
        // node slot popped at schema position s0 + i: the latest earlier push there, else the old content
        int qs = s0 + i;
        uint32_t v = sd.schema_stack[qs];
        for (int f = (int)e - 1; f >= 0; f--)
          if (sh_kind[f] == EV_MERGE && qs >= sh_s0[f] - 4 && qs <= sh_s0[f] - 1) {
            v = ps.spush[4 * f + (sh_s0[f] - 1 - qs)];
            break;
          }
        child[i] = v;
        // grid id popped at grid position g0 - 1 + i (the first is this split's own push)
        int qg = g0 - 1 + i;
        uint32_t w = i == 0 ? ps.gpush[4 * e] : sd.grids_stack[qg];
        if (i > 0) {
          for (int f = (int)e - 1; f >= 0; f--) {
            if (sh_kind[f] == EV_MERGE && qg >= sh_g0[f] - 4 && qg <= sh_g0[f] - 1) {
              w = ps.gpush[4 * f + (sh_g0[f] - 1 - qg)];
              break;
            }
            if (sh_kind[f] == EV_SPLIT && qg == sh_g0[f] - 1) {
              w = ps.gpush[4 * f];
              break;
            }
          }
        }
        gid[i] = w;
      }
      Node q = sd.nodes[cur];
      NodeMeta cm = sd.meta[cur];
      double xhalf = RN_SUB(q.mid_x, q.lo_x);
      double yhalf = RN_SUB(q.mid_y, q.lo_y);
      for (int i = 0; i < 4; i++) {
        Node c;
        c.lo_x = RN_ADD(q.lo_x, (i % 2 == 1) ? xhalf : 0.0);
        c.lo_y = RN_ADD(q.lo_y, (i / 2 == 1) ? yhalf : 0.0);
        c.hi_x = RN_ADD(q.mid_x, (i % 2 == 1) ? xhalf : 0.0);
        c.hi_y = RN_ADD(q.mid_y, (i / 2 == 1) ? yhalf : 0.0);
        c.mid_x = RN_DIV(RN_ADD(c.lo_x, c.hi_x), 2.0);
        c.mid_y = RN_DIV(RN_ADD(c.lo_y, c.hi_y), 2.0);
        c.child[0] = c.child[1] = c.child[2] = c.child[3] = STC_NONE;
        sd.nodes[child[i]] = c;
        sd.fbox[child[i]] = make_float4(__double2float_rn(RN_SUB(c.lo_x, sd.ox)), __double2float_rn(RN_SUB(c.lo_y, sd.oy)),
                                        __double2float_rn(RN_SUB(c.hi_x, sd.ox)), __double2float_rn(RN_SUB(c.hi_y, sd.oy)));
        NodeMeta m;
        m.type = NODE_LEAF; m.level = (int16_t)(cm.level + 1); m.overflow = 0; m.underflow = 0;
        m.grid_id = gid[i]; m.parent = cur;
        sd.meta[child[i]] = m;
        sd.gid_node[gid[i]] = child[i];
        q.child[i] = child[i];
      }
      sd.nodes[cur] = q;
      cm.type = NODE_BRANCH;
      cm.overflow = 0;
      sd.meta[cur] = cm;
    }
    __syncthreads();
    // final stack contents: the last push to each position wins
    for (uint32_t e = tid; e < nev; e += blockDim.x) {
      int s0 = ps.s0[e], g0 = ps.g0[e];
      if (ps.kind[e] == EV_MERGE) {
        for (int i = 0; i < 4; i++) {
          int qs = s0 - 1 - i, qg = g0 - 1 - i;
          bool last_s = true, last_g = true;
          for (uint32_t f = e + 1; f < nev; f++) {
            if (sh_kind[f] == EV_MERGE) {
              if (qs >= sh_s0[f] - 4 && qs <= sh_s0[f] - 1) last_s = false;
              if (qg >= sh_g0[f] - 4 && qg <= sh_g0[f] - 1) last_g = false;
            } else if (qg == sh_g0[f] - 1) {
              last_g = false;
            }
          }
          if (last_s) sd.schema_stack[qs] = ps.spush[4 * e + i];
          if (last_g) sd.grids_stack[qg] = ps.gpush[4 * e + i];
        }
      } else {
        int qg = g0 - 1;
        bool last_g = true;
        for (uint32_t f = e + 1; f < nev; f++) {
          if (sh_kind[f] == EV_MERGE) {
            if (qg >= sh_g0[f] - 4 && qg <= sh_g0[f] - 1) last_g = false;
          } else if (qg == sh_g0[f] - 1) {
            last_g = false;
          }
        }
        if (last_g) sd.grids_stack[qg] = ps.gpush[4 * e];
      }
    }
  }
  __syncthreads();
  if (tid == 0) {
    uint32_t splits = 0, merges = 0;
    for (uint32_t e = 0; e < nev; e++) (ps.kind[e] == EV_SPLIT ? splits : merges)++;
    if (nev) {
      uint32_t l = nev - 1;
      st->schema_stack_index = (uint32_t)(ps.s0[l] + (ps.kind[l] == EV_SPLIT ? 4 : -4));
      st->grids_stack_index = (uint32_t)(ps.g0[l] + (ps.kind[l] == EV_SPLIT ? 3 : -3));
    }
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

void update_schema(SchemaDev sd, SchemaWork w, uint32_t *grid_count, double reach, uint32_t grid_capacity,
                   uint32_t delay, int serial_only, DevState *st, cudaStream_t s) {
  STC_KL k_schema_phase1<<<nblk(sd.S), 256, 0, s>>>(sd, grid_count, reach, grid_capacity, delay, w.ev_flag, w.old_under);
  // ordered compaction of the flagged node indices: ev_pos = exclusive scan of (flag != 0)
  STC_KL k_flags_to_bits<<<nblk(sd.S), 256, 0, s>>>(w.ev_flag, w.ev_pos, sd.S);
  exclusive_scan_u32(w.ev_pos, w.ev_pos, sd.S, w.ev_total, w.scan_tmp, s);
  STC_KL k_schema_compact<<<nblk(sd.S), 256, 0, s>>>(w.ev_flag, w.ev_pos, sd.S, w.ev_list);
  unsigned int *done = (unsigned int *)(w.ev_total + 1);
  STC_KL k_schema_phase2_par<<<1, 1024, 0, s>>>(sd, w.ev_list, w.ev_total, done, serial_only, w.par_scratch, st);
  STC_KL k_schema_phase2<<<1, 32, 0, s>>>(sd, grid_count, w.ev_list, w.ev_total, w.old_under, w.heap, w.queued,
                                   grid_capacity, delay, done, st);
}

}  // namespace stc
