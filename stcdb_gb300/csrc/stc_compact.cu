// Compaction of flushed blocks on the GPU: the reference's merge_dump
// (tools/compaction.cpp:729-1206), which merges m contact tracing blocks into
// one block of split x split CTFs.
//
// The reference decodes every CTF key on the host, groups the keys of each
// object in per-object vectors, sorts each vector by target, re-partitions
// the objects by STR over the midpoints of their key boxes, and re-encodes.
// Here the same result comes from whole-array passes over device memory:
//
//   decode    one thread per input CTF key: fields, absolute end, the key box
//             (CTF::new_parse_mbr_f_box), per-object key count and box
//   STR       objects by x midpoint (stable radix sort over ordered float
//             bits, ties by oid), x slabs by y midpoint, sids
//             (the flush's slab and make_sid kernels)
//   key sort  one stable LSD radix sort of all records by (oversize, sid,
//             oid, target, duration, end) on packed 32-bit words (the flush's
//             word kernels): the CTF keys in CTF order, each object's keys by
//             (target, duration, end), then the merged oversize buffer
//   limits    the flush's per-CTF box and start-time reductions, the
//             oversize start times and map bitmap
//   encode    bitmaps (compaction's per-axis clamped cell rule) and packed keys
//             written straight into the new block's arrays
//
// Departures from merge_dump (each a defect that loses or corrupts keys
// there; the oracle's normal mode, oracle/stc_compact.cpp, states them with
// line references): oids masked to id_bit; an object oversize in any input
// stays oversize; every STR object gets its CTF; no object-0 padding; CTF end
// times from the merged blocks with ends stored relative to end_time_min (and
// end_bit widened when the span needs it); oversize ends re-based to the
// merged buffer's end_time_min and their cells added to its bitmap.
//
// Bytes per merged key (algorithmic): read the packed key (<= 16) and write
// the new one (<= 16) plus the 32-byte record and box once each way for the
// sort gather: 2 * 32 per key, as for the flush.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "stc_lsm_kernels.cuh"

namespace stc {

namespace {

using namespace lsmk;

// One CTF of an input block, in decode order.
struct InCtf {
  unsigned long long first;  // first key of this CTF among all decoded CTF keys
  const uint8_t *keys;       // its packed keys (block buffer padded by 32 bytes)
  stc_ctf ctf;
  double rx, ry, re;         // 1 / the largest low-x, low-y and edge field
  double dx, dy, de;         // bounds on the reciprocal decode's error (parse_coord)
};

// One box coordinate as CTF::new_parse_mbr_f_box computes it: the float
// nearest to base + (q / qmax) * w evaluated in double. The correctly rounded
// division costs many FP64 instructions, so q * (1 / qmax) is tried first: it
// differs from the exact double by at most d, and when both ends of
// [v - d, v + d] round to the same float that float is the result.
__device__ __forceinline__ float parse_coord(double base, unsigned long long q, unsigned long long qmax, double rq,
                                            double w, double d) {
  const double qd = __ull2double_rn(q);
  const double v = base + qd * rq * w;
  const float lo = __double2float_rn(v - d), hi = __double2float_rn(v + d);
  if (lo == hi) return lo;
  return __double2float_rn(__dadd_rn(base, __dmul_rn(__ddiv_rn(qd, __ull2double_rn(qmax)), w)));
}

__host__ __device__ __forceinline__ unsigned long long mask64(uint32_t bits) {
  return bits >= 64 ? ~0ull : ((1ull << bits) - 1ull);
}

__device__ __forceinline__ unsigned __int128 load_packed(const uint8_t *p, uint32_t kb) {
  uintptr_t a = (uintptr_t)p;
  const unsigned long long *w = (const unsigned long long *)(a & ~(uintptr_t)7);
  uint32_t sh = (uint32_t)(a & 7) * 8;
  unsigned __int128 k = (((unsigned __int128)__ldg(w + 1) << 64) | __ldg(w)) >> sh;
  if (sh) k |= (unsigned __int128)__ldg(w + 2) << (128 - sh);
  if (kb < 16) k &= (((unsigned __int128)1) << (8 * kb)) - 1;
  return k;
}

// Sortable bits of a float (no NaN); -0 sorts with +0.
__device__ __forceinline__ uint32_t ordered(float f) {
  uint32_t u = __float_as_uint(f == 0.0f ? 0.0f : f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

struct Objs {
  uint16_t *csid;
  uint32_t *cnt;
  float4 *box;
};

// merge_dump's sids (tools/compaction.cpp:740-747): an object oversize in any
// input is oversize (1); the per-object key counts and boxes start empty.
__global__ void k_cmp_init(const uint16_t *const *in_sids, uint32_t m, uint32_t N, Objs o) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  uint16_t s = 0;
  for (uint32_t i = 0; i < m; i++)
    if (in_sids[i][j] == 1) s = 1;
  o.csid[j] = s;
  o.cnt[j] = 0;
  o.box[j] = make_float4(100000.0f, 100000.0f, -100000.0f, -100000.0f);
}

// Decode of every input CTF key (:792-818 with CTF::parse_key and
// CTF::new_parse_mbr_f_box, tracing/step_merge.cpp:347-400): record `base +
// kid` gets (oid, target, duration, end offset) and the float box; keys of
// oversize objects go to the oversize buffer (end relative to o_etm), the
// others mark their object (sid 2), count and box it (end relative to etm).
__global__ void k_cmp_decode(const InCtf *ic, uint32_t nc, unsigned long long nk, unsigned long long base,
                             uint32_t N, uint32_t etm, uint32_t o_etm, Objs o, uint4 *rec, float4 *box,
                             uint8_t *over, DevState *st) {
  uint32_t md = 0, me = 0;
  for (unsigned long long kid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; kid < nk;
       kid += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = nc - 1;  // largest c with first <= kid
    while (lo < hi) {
      uint32_t mid = (lo + hi + 1) >> 1;
      if (ic[mid].first <= kid) lo = mid;
      else hi = mid - 1;
    }
    const stc_ctf &t = ic[lo].ctf;
    const uint32_t kb = t.key_bit / 8u;
    if (kid - ic[lo].first >= t.kv_count) {  // outside every CTF: never read past its keys
      stc_set_error(st, ERR_COMPACT, lo);
      continue;
    }
    unsigned __int128 k = load_packed(ic[lo].keys + (kid - ic[lo].first) * kb, kb);
    unsigned long long vm = (unsigned long long)(k & (unsigned __int128)mask64(t.mbr_bit));
    k >>= t.mbr_bit;
    uint32_t end = (uint32_t)(k & mask64(t.end_bit));
    k >>= t.end_bit;
    uint32_t dur = (uint32_t)(k & mask64(t.duration_bit));
    k >>= t.duration_bit;
    uint32_t target = (uint32_t)(k & mask64(t.id_bit));
    k >>= t.id_bit;
    uint32_t oid = (uint32_t)(k & mask64(t.id_bit));
    if (oid >= N || target >= N) {
      stc_set_error(st, ERR_COMPACT, oid);
      continue;
    }
    const uint32_t real_end = end + t.end_time_min;
    // CTF::new_parse_mbr_f_box: double arithmetic, stored as float
    const InCtf &x = ic[lo];
    unsigned long long me_ = mask64(t.edge_bit), my = mask64(t.low_y_bit), mx = mask64(t.low_x_bit);
    unsigned long long ey = vm & me_;
    vm >>= t.edge_bit;
    unsigned long long ex = vm & me_;
    vm >>= t.edge_bit;
    unsigned long long low1 = vm & my;
    vm >>= t.low_y_bit;
    unsigned long long low0 = vm & mx;
    float wx = __fsub_rn(t.mbr[2], t.mbr[0]), wy = __fsub_rn(t.mbr[3], t.mbr[1]);
    float le = fmaxf(wx, wy);
    float4 b;
    b.x = parse_coord((double)t.mbr[0], low0, mx, x.rx, (double)wx, x.dx);
    b.y = parse_coord((double)t.mbr[1], low1, my, x.ry, (double)wy, x.dy);
    b.z = parse_coord((double)b.x, ex, me_, x.re, (double)le, x.de);
    b.w = parse_coord((double)b.y, ey, me_, x.re, (double)le, x.de);
    const bool ov = o.csid[oid] == 1;
    const uint32_t off = real_end - (ov ? o_etm : etm);
    rec[base + kid] = make_uint4(oid, target, dur, off);
    box[base + kid] = b;
    over[base + kid] = ov;
    md = max(md, dur);
    me = max(me, off);
    if (ov) {
      agg_inc(&st->lsm_over_keys);
    } else {
      o.csid[oid] = 2;  // every writer stores the same value
      atomicAdd(&o.cnt[oid], 1u);
      atomic_min_f(&o.box[oid].x, b.x);
      atomic_min_f(&o.box[oid].y, b.y);
      atomic_max_f(&o.box[oid].z, b.z);
      atomic_max_f(&o.box[oid].w, b.w);
    }
  }
  md = warp_max_u32(md);
  me = warp_max_u32(me);
  if ((threadIdx.x & 31u) == 0) {
    atomicMax(&st->lsm_max_dur, md);
    atomicMax(&st->lsm_max_end, me);
  }
}

// The oversize keys of one input block, re-based to o_etm, at records
// [at, at + n).
__global__ void k_cmp_copy_over(const uint4 *orec, const float4 *obox, unsigned long long n, unsigned long long at,
                                uint32_t add, uint4 *rec, float4 *box, uint8_t *over, DevState *st) {
  uint32_t md = 0, me = 0;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    uint4 r = orec[i];
    r.w += add;
    rec[at + i] = r;
    box[at + i] = obox[i];
    over[at + i] = 1;
    md = max(md, r.z);
    me = max(me, r.w);
    agg_inc(&st->lsm_over_keys);
  }
  md = warp_max_u32(md);
  me = warp_max_u32(me);
  if ((threadIdx.x & 31u) == 0) {
    atomicMax(&st->lsm_max_dur, md);
    atomicMax(&st->lsm_max_end, me);
  }
}

// STR keys (:830-842): the midpoint of each object's box in float, as
// object_info::ave_loc; objects without a CTF sort last. Counts the objects
// with keys and the oversize ones.
__global__ void k_cmp_mid(Objs o, uint32_t N, uint32_t *xkey, uint32_t *ykey, uint32_t *ids, DevState *st) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  uint16_t s = o.csid[j];
  uint32_t kx = 0xFFFFFFFFu, ky = 0;
  if (s == 2) {
    float4 b = o.box[j];
    kx = ordered(__fadd_rn(__fdiv_rn(b.x, 2.0f), __fdiv_rn(b.z, 2.0f)));
    ky = ordered(__fadd_rn(__fdiv_rn(b.y, 2.0f), __fdiv_rn(b.w, 2.0f)));
    atomicAdd(&st->work_next, 1u);
  }
  if (s != 0) atomicAdd(&st->lsm_sid_count, 1u);
  if (s == 1) atomicAdd(&st->lsm_over_count, 1u);
  xkey[j] = kx;
  ykey[j] = ky;
  ids[j] = j;
}

__global__ void k_cmp_limits_init(float4 *lim_box, uint2 *lim_time, uint32_t F) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= F) return;
  lim_box[c] = make_float4(100000.0f, 100000.0f, -100000.0f, -100000.0f);
  lim_time[c] = make_uint2(1u << 30, 1u);  // merge_dump starts the start-time maximum at 1 (:989)
}

__global__ void k_cmp_or_bitmap(const uint32_t *in, uint32_t *out, uint32_t words) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < words) out[i] |= in[i];
}

__global__ void k_cmp_state_init(DevState *st) {
  memset(st, 0, sizeof(DevState));
  st->lsm_os_min = 1u << 30;
  st->lsm_os_max = 0;
}

// Device scratch of one compaction, freed when it ends.
struct Scratch {
  std::vector<void *> ptrs;
  bool ok = true;
  template <typename T>
  T *get(size_t n) {
    void *p = nullptr;
    if (ok && cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
      ok = false;
      p = nullptr;
    }
    if (p) ptrs.push_back(p);
    return (T *)p;
  }
  ~Scratch() {
    for (void *p : ptrs) cudaFree(p);
  }
};

}  // namespace

stc_status lsm_compact(const LsmDev &L, LsmHost &H, uint32_t first_index, uint32_t count, uint32_t split,
                       uint32_t new_index, cudaStream_t s, float *ms, std::string &err, float *stages) {
  const uint32_t N = L.N, S = split, F2 = split * split;
  if (count == 0 || split == 0 || F2 > MAX_CTF) {
    err = "compact: count must be >= 1 and split in 1..63";
    return STC_ERR_INVALID_ARG;
  }
  // the inputs: the block first_index and the count - 1 retained after it;
  // only this thread changes the retained list, so positions stay valid
  size_t pos = 0;
  std::vector<const CtbBlock *> in;
  {
    std::shared_lock<std::shared_mutex> lock(H.blocks_mu);
    while (pos < H.blocks.size() && H.blocks[pos].info.index != first_index) pos++;
    if (pos + count > H.blocks.size()) {
      err = "compact: blocks not retained";
      return STC_ERR_INVALID_ARG;
    }
    for (uint32_t i = 0; i < count; i++) in.push_back(&H.blocks[pos + i]);
  }
  unsigned long long nk = 0, no = 0;
  uint32_t etm = 0xFFFFFFFFu, etmax = 0, o_etm = 0xFFFFFFFFu, o_etmax = 0, flush_max = 0, nc = 0;
  for (const CtbBlock *b : in) {
    // the keys of the CTF files: the flush's CTF ranges can differ from its
    // count of CTF keys (they reach into the oversize keys, as the
    // reference's do), and merge_dump reads each CTF's kv_count keys (:796)
    for (const stc_ctf &t : b->ctfs) nk += t.kv_count;
    no += b->info.oversize_kv_count;
    etm = std::min(etm, b->info.end_time_min);
    etmax = std::max(etmax, b->info.flush_time);
    flush_max = std::max(flush_max, b->info.flush_time);
    o_etm = std::min(o_etm, b->info.o_end_time_min);
    o_etmax = std::max(o_etmax, b->info.o_end_time_max);
    nc += b->info.ctf_count;
  }
  const unsigned long long T = nk + no;
  if (T >= 0xFFFFFFFFull) {
    err = "compact: more than 2^32 - 1 keys";
    return STC_ERR_CAPACITY;
  }
  const size_t W = std::max<size_t>((size_t)T, (size_t)N);
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  cudaEventRecord(ev0, s);
  // stage marks: the ends of the first COMPACT_STAGES - 1 stages (ev1 ends the last)
  struct Marks {
    cudaEvent_t ev[COMPACT_STAGES - 1] = {};
    Marks() {
      for (cudaEvent_t &x : ev) cudaEventCreate(&x);
    }
    ~Marks() {
      for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    }
  } marks;
  auto mark = [&](int i) { cudaEventRecord(marks.ev[i], s); };
  Scratch sc;
  LsmDev C = L;  // configuration; every array below is the compaction's own
  C.F = F2;
  C.split = S;
  C.cap = W;
  C.end_time_min = etm;
  C.rec = sc.get<uint4>(T);
  C.box = sc.get<float4>(T);
  C.brec = sc.get<uint4>(T);
  C.bbox = sc.get<float4>(T);
  C.over = sc.get<uint8_t>(T);
  for (int i = 0; i < 7; i++) C.sk[i] = sc.get<uint32_t>(W);
  const size_t hw = radix_hist_words(W);
  C.hist = sc.get<uint32_t>(hw);
  C.scan = sc.get<uint32_t>(scan_tmp_words(hw));
  C.n_dev = sc.get<unsigned long long>(6);
  C.cnt = sc.get<uint32_t>(N);
  C.sid = sc.get<uint16_t>(N);
  C.mid_lo = sc.get<uint32_t>(N);
  C.mid_hi = sc.get<uint32_t>(N);
  C.ctf_cap = sc.get<uint32_t>(F2);
  C.ctf_first = sc.get<unsigned long long>(F2 + 1);
  C.lim_box = sc.get<float4>(F2);
  C.lim_time = sc.get<uint2>(F2);
  C.st = sc.get<DevState>(1);
  float4 *objbox = sc.get<float4>(N);
  InCtf *d_ic = sc.get<InCtf>(nc);
  const uint16_t **d_sids = sc.get<const uint16_t *>(count);
  if (!sc.ok) {
    err = "compact: device memory for the merge scratch";
    return STC_ERR_CAPACITY;
  }
  mark(0);
  // 1. sids, oversize records of the inputs, decode of the CTF keys
  std::vector<InCtf> ic;
  std::vector<const uint16_t *> sid_ptrs;
  unsigned long long first = 0;
  for (const CtbBlock *b : in) {
    sid_ptrs.push_back(b->sids);
    for (const stc_ctf &t : b->ctfs) {
      InCtf x;
      x.first = first;
      x.keys = b->keys + t.key_offset;
      x.ctf = t;
      // each of the exact decode's five roundings (and the reciprocal
      // decode's) is within 2^-53 of a value below |base| + 2|w| in size; the
      // bound used is 2^7 times their sum
      const double mx = (double)mask64(t.low_x_bit), my = (double)mask64(t.low_y_bit), me = (double)mask64(t.edge_bit);
      const float wx = t.mbr[2] - t.mbr[0], wy = t.mbr[3] - t.mbr[1], le = std::max(wx, wy);
      double m = 0.0;
      for (int i = 0; i < 4; i++) m = std::max(m, std::fabs((double)t.mbr[i]));
      const bool ok = mx > 0 && my > 0 && me > 0 && std::isfinite(m) && std::isfinite((double)le);
      x.rx = ok ? 1.0 / mx : 0.0;
      x.ry = ok ? 1.0 / my : 0.0;
      x.re = ok ? 1.0 / me : 0.0;
      const double u = std::ldexp(1.0, -46);
      x.dx = ok ? (std::fabs((double)t.mbr[0]) + 2.0 * std::fabs((double)wx) + 1.0) * u : INFINITY;
      x.dy = ok ? (std::fabs((double)t.mbr[1]) + 2.0 * std::fabs((double)wy) + 1.0) * u : INFINITY;
      x.de = ok ? (m + std::fabs((double)wx) + std::fabs((double)wy) + 2.0 * std::fabs((double)le) + 1.0) * u : INFINITY;
      ic.push_back(x);
      first += t.kv_count;
    }
  }
  cudaError_t e = cudaMemcpyAsync(d_ic, ic.data(), nc * sizeof(InCtf), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_sids, sid_ptrs.data(), count * sizeof(void *), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) {
    err = std::string("compact: ") + cudaGetErrorString(e);
    return STC_ERR_CUDA;
  }
  Objs ob{C.sid, C.cnt, objbox};
  STC_KL k_cmp_state_init<<<1, 1, 0, s>>>(C.st);
  STC_KL k_cmp_init<<<nblk(N), 256, 0, s>>>(d_sids, count, N, ob);
  unsigned long long at = 0;
  for (const CtbBlock *b : in) {
    const unsigned long long n = b->info.oversize_kv_count;
    if (n)
      STC_KL k_cmp_copy_over<<<lsm_grid(), 256, 0, s>>>(b->orec, b->obox, n, at, b->info.o_end_time_min - o_etm, C.rec,
                                                  C.box, C.over, C.st);
    at += n;
  }
  if (nk)
    STC_KL k_cmp_decode<<<lsm_grid(), 256, 0, s>>>(d_ic, nc, nk, no, N, etm, o_etm, ob, C.rec, C.box, C.over, C.st);
  mark(1);
  // 2. STR: objects by x midpoint, x slabs by y midpoint (:843-942)
  uint32_t **sk = C.sk;
  STC_KL k_cmp_mid<<<nblk(N), 256, 0, s>>>(ob, N, sk[5], C.mid_lo, sk[0], C.st);
  STC_KL k_lsm_set_counts<<<1, 1, 0, s>>>(C.n_dev, N, 0, T);
  sort_words(C, sk[5], sk[0], sk[1], sk[6], sk[3], sk[4], 0, N, 32, s);  // sk[6]: objects in x order
  DevState st{};
  e = cudaMemcpyAsync(&st, C.st, sizeof(DevState), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    err = std::string("compact: ") + cudaGetErrorString(e);
    return STC_ERR_CUDA;
  }
  if (st.error) {
    err = "compact: a key to merge is outside its CTF or names an object outside the configuration";
    return STC_ERR_INVALID_ARG;
  }
  const uint32_t n_str = st.work_next;
  const unsigned long long n_over = st.lsm_over_keys, slim = T - n_over;
  cudaMemsetAsync(C.ctf_cap, 0, F2 * sizeof(uint32_t), s);
  if (n_str) {
    const uint32_t xcap = (n_str - 1) / S + 1, ycap = xcap / S + 1;
    STC_KL k_lsm_set_counts<<<1, 1, 0, s>>>(C.n_dev, N, n_str, T);
    STC_KL k_slab_keys<<<nblk(n_str), 256, 0, s>>>(C.mid_lo, sk[6], 0, n_str, sk[0], sk[2]);
    sort_words(C, sk[0], sk[2], sk[1], sk[5], sk[3], sk[4], 1, n_str, 32, s);
    STC_KL k_slab_of<<<nblk(n_str), 256, 0, s>>>(sk[5], n_str, xcap, S, sk[0]);
    sort_words(C, sk[0], sk[5], sk[1], sk[2], sk[3], sk[4], 1, n_str, bits_for(S - 1), s);
    STC_KL k_make_sid<<<num_sms(), 512, F2 * sizeof(uint32_t), s>>>(C, sk[6], sk[2], 0, n_str, xcap, ycap);
  }
  mark(2);
  // 3. all records by (oversize, sid, oid, target, duration, end), stable
  sort_keys(C, T, N, st.lsm_max_end, st.lsm_max_dur, bits_for(F2 + 1), s);
  mark(3);
  // 4. CTF ranges and limits (:944-1004), oversize times and bitmap
  std::vector<uint32_t> cap(F2);
  e = cudaMemcpyAsync(cap.data(), C.ctf_cap, F2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    err = std::string("compact: ") + cudaGetErrorString(e);
    return STC_ERR_CUDA;
  }
  std::vector<unsigned long long> cfirst(F2 + 1, 0);
  for (uint32_t c = 0; c < F2; c++) cfirst[c + 1] = cfirst[c] + cap[c];
  if (cfirst[F2] != slim) {
    err = "compact: CTF capacities do not add up to the CTF keys";
    return STC_ERR_STATE;
  }
  CtbBlock B;
  const size_t no_out = (size_t)n_over;
  const size_t obm_bytes = STC_MAP_BITMAP_BYTES(L.edge);
  e = cudaMalloc(&B.obitmap, obm_bytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(B.obitmap, 0, obm_bytes, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(C.ctf_first, cfirst.data(), (F2 + 1) * sizeof(unsigned long long),
                                            cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) {
    free_block(B);
    err = std::string("compact: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? STC_ERR_CAPACITY : STC_ERR_CUDA;
  }
  STC_KL k_cmp_limits_init<<<nblk(F2), 256, 0, s>>>(C.lim_box, C.lim_time, F2);
  if (slim) STC_KL k_lsm_limits<<<dim3(F2, LIM_PARTS), 256, 0, s>>>(C, slim);
  for (const CtbBlock *b : in)
    STC_KL k_cmp_or_bitmap<<<nblk(obm_bytes / 4), 256, 0, s>>>(b->obitmap, B.obitmap, (uint32_t)(obm_bytes / 4));
  if (T > slim) {
    LsmDev O = C;
    O.end_time_min = o_etm;
    O.obitmap = B.obitmap;
    STC_KL k_lsm_oversize<<<lsm_grid(), 256, 0, s>>>(O, slim, T);
  }
  std::vector<float4> lb(F2);
  std::vector<uint2> lt(F2);
  e = cudaMemcpyAsync(lb.data(), C.lim_box, F2 * sizeof(float4), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lt.data(), C.lim_time, F2 * sizeof(uint2), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&st, C.st, sizeof(DevState), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    free_block(B);
    err = std::string("compact: ") + cudaGetErrorString(e);
    return STC_ERR_CUDA;
  }
  // 5. per-CTF metadata (CTF::get_ctf_bits, :1003), end_bit widened to the span
  B.ctfs.assign(F2, stc_ctf{});
  unsigned long long off = 0;
  for (uint32_t c = 0; c < F2; c++) {
    stc_ctf &x = B.ctfs[c];
    x.mbr[0] = lb[c].x; x.mbr[1] = lb[c].y; x.mbr[2] = lb[c].z; x.mbr[3] = lb[c].w;
    x.kv_count = cap[c];
    x.start_time_min = lt[c].x;
    x.start_time_max = lt[c].y;
    x.end_time_min = etm;
    x.end_time_max = etmax;
    bool fits = ctf_bits(x.mbr, L.map, N, L.max_meet, &x);
    if (fits && etmax > etm) {
      uint32_t need = bits_for(etmax - etm);
      if (need > x.end_bit) {
        x.end_bit = (uint16_t)need;
        uint32_t temp = 2u * x.id_bit + x.duration_bit + x.end_bit + x.mbr_bit;
        fits = temp <= 128;
        x.key_bit = (uint16_t)((temp + 7) / 8 * 8);
      }
    }
    if (!fits) {
      free_block(B);
      err = "compact: a CTF key needs more than 64 box bits or 128 bits in all";
      return STC_ERR_CAPACITY;
    }
    x.first_key = cfirst[c];
    x.key_offset = off;
    off += (unsigned long long)cap[c] * (x.key_bit / 8u);
  }
  // 6. the new block's arrays; bitmaps and packed keys written in place
  B.info.index = new_index;
  B.info.ctf_count = F2;
  B.info.flush_time = flush_max;
  B.info.end_time_min = etm;
  B.info.kv_count = T;
  B.info.ctf_kv_count = slim;
  B.info.oversize_kv_count = n_over;
  B.info.key_bytes = off;
  B.info.sid_count = st.lsm_sid_count;
  B.info.oversize_oid_count = st.lsm_over_count;
  B.info.o_start_time_min = st.lsm_os_min;
  B.info.o_start_time_max = st.lsm_os_max;
  B.info.o_end_time_min = o_etm;
  B.info.o_end_time_max = o_etmax;
  B.info.bitmap_edge = L.edge;
  e = cudaMalloc(&B.keys, off + 32);
  if (e == cudaSuccess) e = cudaMalloc(&B.d_ctfs, F2 * sizeof(stc_ctf));
  if (e == cudaSuccess) e = cudaMalloc(&B.bitmaps, (size_t)F2 * STC_BITMAP_BYTES);
  if (e == cudaSuccess) e = cudaMalloc(&B.sids, (size_t)N * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc(&B.orec, std::max<size_t>(no_out, 1) * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&B.obox, std::max<size_t>(no_out, 1) * sizeof(float4));
  if (e == cudaSuccess) e = cudaMemsetAsync(B.keys, 0, off + 32, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(B.bitmaps, 0, (size_t)F2 * STC_BITMAP_BYTES, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.d_ctfs, B.ctfs.data(), F2 * sizeof(stc_ctf), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.sids, C.sid, (size_t)N * sizeof(uint16_t), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && no_out)
    e = cudaMemcpyAsync(B.orec, C.brec + slim, no_out * sizeof(uint4), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && no_out)
    e = cudaMemcpyAsync(B.obox, C.bbox + slim, no_out * sizeof(float4), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) mark(4);
  if (e == cudaSuccess && slim)
    // bitmaps (:1015-1035: cells clamped to the grid on each axis) and packed
    // keys (:1048-1060: oid, target, duration, end offset, box; fields added)
    STC_KL k_encode_keys<<<lsm_grid(), ENC_GROUP, 0, s>>>(
        EncodeArgs{C.brec, C.bbox, B.d_ctfs, C.ctf_first, nullptr, B.bitmaps, B.keys, slim, slim, F2, true});
  if (e == cudaSuccess) mark(5);
  if (e == cudaSuccess) e = build_index(C, B, s);
  if (e == cudaSuccess) e = cudaEventRecord(ev1, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    free_block(B);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    err = std::string("compact: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? STC_ERR_CAPACITY : STC_ERR_CUDA;
  }
  if (ms) cudaEventElapsedTime(ms, ev0, ev1);
  if (stages) {
    cudaEvent_t b[COMPACT_STAGES + 1] = {ev0};
    for (int i = 0; i < COMPACT_STAGES - 1; i++) b[i + 1] = marks.ev[i];
    b[COMPACT_STAGES] = ev1;
    for (int i = 0; i < COMPACT_STAGES; i++) {
      stages[i] = 0.0f;
      cudaEventElapsedTime(&stages[i], b[i], b[i + 1]);
    }
    cudaGetLastError();
  }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  // 7. the merged block takes the place of its inputs
  {
    std::unique_lock<std::shared_mutex> lock(H.blocks_mu);
    for (uint32_t i = 0; i < count; i++) free_block(H.blocks[pos + i]);
    H.blocks.erase(H.blocks.begin() + pos, H.blocks.begin() + pos + count);
    H.blocks.insert(H.blocks.begin() + pos, std::move(B));
  }
  return STC_OK;
}

}  // namespace stc
