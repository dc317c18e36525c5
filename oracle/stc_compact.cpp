// CPU restatement of the reference's compaction of contact tracing blocks
// (merge_dump, tools/compaction.cpp:729-1206) -- TEST INFRASTRUCTURE ONLY:
// the checker for the GPU compaction in stcdb_gb300/csrc/stc_compact.cu,
// never linked into the product.
//
// The reference merges m blocks into one: it decodes every CTF key, groups
// the keys by object, sorts each object's keys by target, re-partitions the
// objects into split x split CTFs by STR over the midpoints of their key
// boxes, recomputes each CTF's box, time limits, bit widths
// (CTF::get_ctf_bits) and bitmap, re-encodes the keys, and k-way merges the
// oversize buffers.
//
// reference_mode != 0 follows merge_dump literally where a test can pin it
// against the reference itself (oracle/ref_compact.cpp runs merge_dump on
// block files; tests/golden/compact_pin.npz): the same std::sort calls on
// the same sequences (so equal keys keep the reference's order), the last
// STR object left without a CTF, the CTF end times taken from the blocks'
// CTB objects (0 in the files the flush writes). Its oversize merge is the
// normal one below (the pin's blocks have no oversize keys).
//
// reference_mode == 0 is the compaction the GPU implements: the reference's
// algorithm with these departures, each a defect that loses or corrupts
// keys in merge_dump:
//  D1 the oid of a decoded key is masked to id_bit (CTF::ctf_get_key_oid,
//     tracing/step_merge.cpp:330-332); CTF::parse_key (:335-345) keeps the
//     sid bits the flush stores above it, and merge_dump indexes its
//     per-object arrays with that value (tools/compaction.cpp:797-812);
//  D2 an object that is oversize in any input block is oversize in the
//     result, all its keys in the oversize buffer (merge_dump gives it a CTF
//     when another block has CTF keys of it, :741-747 and :804-812, and its
//     oversize keys become unreachable by object queries);
//  D3 every STR object gets its CTF (merge_dump stops at the last one,
//     :931-942, and its keys are written to no CTF);
//  D4 a CTF holds exactly its objects (merge_dump sizes every list to the
//     y capacity and leaves unfilled places as object 0, :925-929, which
//     copies object 0's keys into those CTFs);
//  D5 the CTF end times are the merged blocks' (min end_time_min, max
//     end_time_max) and key ends are stored relative to end_time_min;
//     merge_dump takes them from the CTB objects, whose times are 0
//     (:979-985, :1001-1002), and adds end_time_min to the absolute end
//     once more (:1056);
//  D6 end_bit grows to hold the largest end offset when the merged span
//     needs more than bits(max_meet_time - 1);
//  D7 oversize keys of every input are stored relative to the merged
//     buffer's end_time_min (merge_dump merges each block's offsets, relative
//     to different times, with absolute ends, :1088-1095, :1118-1133), its
//     times are the true min/max (merge_dump starts its minima at 0,
//     step_merge.h:50-53), and the bitmap also covers the oversize keys taken
//     from CTFs (:1097 leaves them out).
// Equal keys: objects with equal midpoints are ordered by oid, keys of one
// object by (target, duration, end) and then input order; the reference's
// std::sort leaves both orders unspecified.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "stc_oracle.h"

namespace {

typedef unsigned __int128 u128;

uint64_t mask64(uint32_t bits) { return bits >= 64 ? ~0ull : ((1ull << bits) - 1); }

uint32_t f2u32(float x) {  // cvt.rzi.u32.f32: NaN and negatives to 0, saturating
  if (!(x > 0.0f)) return 0;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)x;
}

uint32_t min_bits_to_store(uint32_t v) {  // util/util.h:528-533
  uint32_t b = 1;
  while (b < 32 && (v >> b)) b++;
  return v == 0 ? 1 : b;
}

struct Rec {
  uint32_t oid, target, dur, end;  // end: absolute step
  float box[4];
};

// CTF::new_parse_mbr_f_box (tracing/step_merge.cpp:381-400): the box of a
// packed key, computed in double and stored as float.
void parse_mbr_f_box(uint64_t vm, const stc_ctf &c, float b[4]) {
  uint64_t me = mask64(c.edge_bit), my = mask64(c.low_y_bit), mx = mask64(c.low_x_bit);
  uint64_t y = vm & me;
  vm >>= c.edge_bit;
  uint64_t x = vm & me;
  vm >>= c.edge_bit;
  uint64_t low1 = vm & my;
  vm >>= c.low_y_bit;
  uint64_t low0 = vm & mx;
  float wx = c.mbr[2] - c.mbr[0], wy = c.mbr[3] - c.mbr[1];
  float longer_edge = wx > wy ? wx : wy;
  b[0] = (float)(c.mbr[0] + (double)low0 / (double)mx * wx);
  b[1] = (float)(c.mbr[1] + (double)low1 / (double)my * wy);
  b[2] = (float)(b[0] + (double)x / (double)me * longer_edge);
  b[3] = (float)(b[1] + (double)y / (double)me * longer_edge);
}

// CTF::parse_key (tracing/step_merge.cpp:347-357) with the oid masked (D1).
void parse_key(const uint8_t *p, const stc_ctf &c, Rec &r, uint64_t &vm) {
  u128 k = 0;
  const uint32_t kb = c.key_bit / 8u;
  for (uint32_t i = 0; i < kb; i++) k |= (u128)p[i] << (8 * i);
  vm = (uint64_t)(k & (u128)mask64(c.mbr_bit));
  k >>= c.mbr_bit;
  r.end = (uint32_t)(k & mask64(c.end_bit));
  k >>= c.end_bit;
  r.dur = (uint32_t)(k & mask64(c.duration_bit));
  k >>= c.duration_bit;
  r.target = (uint32_t)(k & mask64(c.id_bit));
  k >>= c.id_bit;
  r.oid = (uint32_t)(k & mask64(c.id_bit));
}

struct ObjInfo {  // object_info (tracing/step_merge.h:27-31)
  double x, y;
  uint32_t oid;
};

}  // namespace

struct cmp_result {
  stc_ctb_info info;
  std::vector<stc_ctf> ctfs;
  std::vector<uint8_t> bitmaps, keys, obitmap;
  std::vector<uint16_t> sids;
  std::vector<uint64_t> okeys;
  std::vector<float> oboxes;
};

extern "C" cmp_result *cmp_compact(const cmp_block *blocks, uint32_t m, uint32_t N, uint32_t S,
                                   uint32_t max_meet_time, const double map[4], uint32_t new_index,
                                   int reference_mode, char *err, size_t errlen) {
  auto fail = [&](const char *msg) -> cmp_result * {
    if (err && errlen) snprintf(err, errlen, "%s", msg);
    return nullptr;
  };
  if (m == 0 || S == 0 || N == 0) return fail("empty compaction");
  const bool ref = reference_mode != 0;
  const uint32_t F2 = S * S;
  // 1. sids (tools/compaction.cpp:740-747): oversize in any block
  std::vector<uint16_t> csid(N, 0);
  for (uint32_t i = 0; i < m; i++)
    for (uint32_t j = 0; j < N; j++)
      if (blocks[i].sids[j] == 1) csid[j] = 1;
  // 2. decode the CTF keys (:792-818)
  std::vector<std::vector<Rec>> obj(N);
  std::vector<Rec> another;
  std::vector<float> obox((size_t)N * 4);
  for (uint32_t j = 0; j < N; j++) {
    obox[4 * j] = obox[4 * j + 1] = 100000.0f;
    obox[4 * j + 2] = obox[4 * j + 3] = -100000.0f;
  }
  for (uint32_t i = 0; i < m; i++) {
    const cmp_block &B = blocks[i];
    for (uint32_t c = 0; c < B.info.ctf_count; c++) {
      const stc_ctf &t = B.ctfs[c];
      const uint32_t kb = t.key_bit / 8u;
      for (uint32_t k = 0; k < t.kv_count; k++) {
        Rec r;
        uint64_t vm;
        parse_key(B.keys + t.key_offset + (uint64_t)k * kb, t, r, vm);
        if (r.oid >= N) return fail("decoded oid out of range");
        r.end += t.end_time_min;
        parse_mbr_f_box(vm, t, r.box);
        bool over = ref ? B.sids[r.oid] == 1 : csid[r.oid] == 1;
        if (over) {
          another.push_back(r);
        } else {
          csid[r.oid] = 2;
          float *ob = &obox[4 * (size_t)r.oid];  // f_box::update (geometry/geometry.h:299-311)
          if (ob[0] > r.box[0]) ob[0] = r.box[0];
          if (ob[2] < r.box[2]) ob[2] = r.box[2];
          if (ob[1] > r.box[1]) ob[1] = r.box[1];
          if (ob[3] < r.box[3]) ob[3] = r.box[3];
          obj[r.oid].push_back(r);
        }
      }
    }
  }
  // 3. each object's keys by target (cpu_sort_by_key, :96-111 and :821-826)
  for (uint32_t j = 0; j < N; j++) {
    std::vector<Rec> &v = obj[j];
    if (v.empty()) continue;
    if (ref)
      std::sort(v.begin(), v.end(), [](const Rec &a, const Rec &b) {
        return a.oid == b.oid ? a.target < b.target : a.oid < b.oid;
      });
    else
      std::stable_sort(v.begin(), v.end(), [](const Rec &a, const Rec &b) {
        if (a.target != b.target) return a.target < b.target;
        if (a.dur != b.dur) return a.dur < b.dur;
        return a.end < b.end;
      });
  }
  // 4. STR over the midpoints of the object boxes (:830-942)
  std::vector<ObjInfo> str(N);
  for (uint32_t j = 0; j < N; j++) {
    str[j].oid = j;
    str[j].x = str[j].y = 0.0;
    if (csid[j] == 2) {
      const float *ob = &obox[4 * (size_t)j];
      float ax = ob[0] / 2 + ob[2] / 2, ay = ob[1] / 2 + ob[3] / 2;
      str[j].x = ax;
      str[j].y = ay;
    }
  }
  std::vector<std::vector<uint32_t>> members(F2);
  uint64_t n_str = 0;
  for (uint32_t j = 0; j < N; j++) n_str += csid[j] == 2;
  if (ref) {
    if (n_str == 0) return fail("reference mode needs at least one STR object");
    const uint16_t *cs = csid.data();
    std::sort(str.begin(), str.end(), [cs](const ObjInfo &a, const ObjInfo &b) {  // compare_two_level (:139-155)
      bool al = cs[a.oid] <= 1, bl = cs[b.oid] <= 1;
      if (al != bl) return bl;
      if (!al) return a.x < b.x;
      return false;
    });
    uint32_t split_index = 0;
    for (uint32_t i = N; i-- > 0;)
      if (cs[str[i].oid] > 1) { split_index = i; break; }
    const uint32_t xcap = split_index / S + 1, ycap = xcap / S + 1;
    // the reference's sizes of the last slab and CTF; negative ones make it
    // sort a reversed range and resize a vector to ~4G entries
    const int64_t last = (int64_t)split_index - (int64_t)xcap * (S - 1) - (int64_t)ycap * (S - 1);
    if (last < 0) return fail("reference mode: the last CTF would have a negative size");
    auto cy = [](const ObjInfo &a, const ObjInfo &b) { return a.y < b.y; };  // compare_y (:157-159)
    for (uint32_t s = 0; s + 1 < S; s++) std::sort(str.begin() + xcap * s, str.begin() + xcap * (s + 1), cy);
    std::sort(str.begin() + xcap * (S - 1), str.begin() + split_index, cy);
    // invert_index (:921-943): every list ycap places, unfilled ones object 0
    for (uint32_t c = 0; c < F2; c++) members[c].assign(c + 1 < F2 ? ycap : (size_t)last, 0u);
    for (uint32_t i = 0; i < split_index; i++) {
      uint32_t x = i / xcap, y = (i % xcap) / ycap, sid = x * S + y + 2;
      csid[str[i].oid] = (uint16_t)sid;
      members[sid - 2][i - x * xcap - y * ycap] = str[i].oid;
    }
    for (uint32_t c = 0; c < F2; c++) std::sort(members[c].begin(), members[c].end());
  } else if (n_str) {
    std::vector<ObjInfo> v;
    v.reserve(n_str);
    for (uint32_t j = 0; j < N; j++)
      if (csid[j] == 2) v.push_back(str[j]);
    std::stable_sort(v.begin(), v.end(), [](const ObjInfo &a, const ObjInfo &b) { return a.x < b.x; });
    const uint32_t split_index = (uint32_t)n_str - 1;
    const uint32_t xcap = split_index / S + 1, ycap = xcap / S + 1;
    for (uint32_t s = 0; s < S; s++) {
      uint64_t lo = std::min<uint64_t>((uint64_t)xcap * s, n_str), hi = std::min<uint64_t>((uint64_t)xcap * (s + 1), n_str);
      std::stable_sort(v.begin() + lo, v.begin() + hi, [](const ObjInfo &a, const ObjInfo &b) { return a.y < b.y; });
    }
    for (uint32_t i = 0; i < (uint32_t)n_str; i++) {
      uint32_t x = i / xcap, y = (i % xcap) / ycap, sid = x * S + y + 2;
      csid[v[i].oid] = (uint16_t)sid;
      members[sid - 2].push_back(v[i].oid);
    }
    for (uint32_t c = 0; c < F2; c++) std::sort(members[c].begin(), members[c].end());
  }
  // 5. per-CTF limits and bit widths (:975-1004)
  uint32_t etm = 0xFFFFFFFFu, etmax = 0, flush_max = 0;
  for (uint32_t i = 0; i < m; i++) {
    etm = std::min(etm, blocks[i].info.end_time_min);
    etmax = std::max(etmax, blocks[i].info.flush_time);
    flush_max = std::max(flush_max, blocks[i].info.flush_time);
  }
  if (ref) etm = etmax = 0;  // the CTB objects' times
  cmp_result *R = new cmp_result();
  R->ctfs.assign(F2, stc_ctf{});
  R->bitmaps.assign((size_t)F2 * 8192, 0);
  uint64_t key_off = 0, first = 0;
  for (uint32_t c = 0; c < F2; c++) {
    stc_ctf &t = R->ctfs[c];
    float lo0 = 100000.0f, lo1 = 100000.0f, hi0 = -100000.0f, hi1 = -100000.0f;
    uint32_t smin = 1u << 30, smax = 1;
    uint64_t kv = 0;
    for (uint32_t oid : members[c])
      for (const Rec &r : obj[oid]) {
        lo0 = std::min(lo0, r.box[0]);
        lo1 = std::min(lo1, r.box[1]);
        hi0 = std::max(hi0, r.box[2]);
        hi1 = std::max(hi1, r.box[3]);
        uint32_t st = r.end - r.dur;
        smin = std::min(smin, st);
        smax = std::max(smax, st);
        kv++;
      }
    t.mbr[0] = lo0; t.mbr[1] = lo1; t.mbr[2] = hi0; t.mbr[3] = hi1;
    t.kv_count = (uint32_t)kv;
    t.start_time_min = smin;
    t.start_time_max = smax;
    t.end_time_min = etm;
    t.end_time_max = etmax;
    if (lsm_ctf_bits(t.mbr, map, N, max_meet_time, &t) != 0) {
      delete R;
      return fail("a CTF key needs more than 64 box bits or 128 bits");
    }
    if (!ref && etmax > etm) {  // D6
      uint32_t need = min_bits_to_store(etmax - etm);
      if (need > t.end_bit) {
        t.end_bit = (uint16_t)need;
        uint32_t temp = 2u * t.id_bit + t.duration_bit + t.end_bit + t.mbr_bit;
        if (temp > 128) {
          delete R;
          return fail("the merged time span needs more than 128 key bits");
        }
        t.key_bit = (uint16_t)((temp + 7) / 8 * 8);
      }
    }
    t.first_key = first;
    t.key_offset = key_off;
    first += kv;
    key_off += kv * (t.key_bit / 8u);
  }
  // 6. bitmaps and packed keys (:1015-1060)
  R->keys.assign(key_off, 0);
  for (uint32_t c = 0; c < F2; c++) {
    const stc_ctf &t = R->ctfs[c];
    uint8_t *bm = R->bitmaps.data() + (size_t)c * 8192;
    const uint32_t kb = t.key_bit / 8u;
    uint64_t k = 0;
    for (uint32_t oid : members[c])
      for (const Rec &r : obj[oid]) {
        float wx = t.mbr[2] - t.mbr[0], wy = t.mbr[3] - t.mbr[1];
        uint32_t l0 = f2u32((r.box[0] - t.mbr[0]) / wx * (float)t.x_grid);
        uint32_t l1 = f2u32((r.box[1] - t.mbr[1]) / wy * (float)t.y_grid);
        uint32_t h0 = f2u32((r.box[2] - t.mbr[0]) / wx * (float)t.x_grid);
        uint32_t h1 = f2u32((r.box[3] - t.mbr[1]) / wy * (float)t.y_grid);
        for (uint32_t a = l0; a <= h0 && a < t.x_grid; a++)
          for (uint32_t b = l1; b <= h1 && b < t.y_grid; b++) {
            uint32_t bit = a + b * t.x_grid;
            bm[bit / 8] |= (uint8_t)(1u << (bit % 8));
          }
        uint64_t vm = lsm_serialize_mbr(r.box, &t);
        uint64_t endf = ref ? (uint64_t)r.end + etm : (uint64_t)(r.end - etm);
        lsm_pack_key(r.oid, r.target, r.dur, endf, vm, &t, R->keys.data() + t.key_offset + k * kb);
        k++;
      }
  }
  // 7. oversize buffers (:1062-1135, with D7): every input's keys relative
  // to the merged end_time_min, then the oversize keys taken from CTFs; one
  // order by (pid, target, duration, end), ties in that input order
  uint32_t o_etm = 0xFFFFFFFFu, o_etmax = 0;
  for (uint32_t i = 0; i < m; i++) {
    o_etm = std::min(o_etm, blocks[i].info.o_end_time_min);
    o_etmax = std::max(o_etmax, blocks[i].info.o_end_time_max);
  }
  std::vector<Rec> ov;
  for (uint32_t i = 0; i < m; i++) {
    const cmp_block &B = blocks[i];
    for (uint64_t k = 0; k < B.info.oversize_kv_count; k++) {
      Rec r;
      uint64_t lo = B.okeys[2 * k], hi = B.okeys[2 * k + 1];
      r.oid = (uint32_t)(hi >> 26);
      r.target = (uint32_t)(hi & ((1ull << 26) - 1));
      r.dur = (uint32_t)(lo >> 32);
      r.end = (uint32_t)lo + B.info.o_end_time_min;
      memcpy(r.box, B.oboxes + 4 * k, sizeof(r.box));
      ov.push_back(r);
    }
  }
  ov.insert(ov.end(), another.begin(), another.end());
  std::stable_sort(ov.begin(), ov.end(), [](const Rec &a, const Rec &b) {
    if (a.oid != b.oid) return a.oid < b.oid;
    if (a.target != b.target) return a.target < b.target;
    if (a.dur != b.dur) return a.dur < b.dur;
    return a.end < b.end;
  });
  // the map bitmap: every input block's (all of one edge), then the merged
  // oversize keys' cells
  const uint32_t edge = blocks[0].info.bitmap_edge ? blocks[0].info.bitmap_edge : 256;
  const size_t obm_bytes = (size_t)edge * edge / 8;
  R->obitmap.assign(obm_bytes, 0);
  for (uint32_t i = 0; i < m; i++)
    for (size_t b = 0; b < obm_bytes; b++) R->obitmap[b] |= blocks[i].obitmap[b];
  uint32_t osmin = 1u << 30, osmax = 0;
  R->okeys.resize(2 * ov.size());
  R->oboxes.resize(4 * ov.size());
  for (size_t k = 0; k < ov.size(); k++) {
    const Rec &r = ov[k];
    uint32_t st = r.end - r.dur;
    osmin = std::min(osmin, st);
    osmax = std::max(osmax, st);
    lsm_o_bitmap_edge(r.box, map, edge, R->obitmap.data());
    R->okeys[2 * k] = ((uint64_t)r.dur << 32) | (uint32_t)(r.end - o_etm);
    R->okeys[2 * k + 1] = ((uint64_t)r.oid << 26) | r.target;
    memcpy(&R->oboxes[4 * k], r.box, sizeof(r.box));
  }
  // 8. the block
  R->sids = csid;
  stc_ctb_info &in = R->info;
  memset(&in, 0, sizeof(in));
  in.index = new_index;
  in.ctf_count = F2;
  in.flush_time = flush_max;
  in.end_time_min = etm;
  in.ctf_kv_count = first;
  in.oversize_kv_count = ov.size();
  in.kv_count = first + ov.size();
  in.key_bytes = key_off;
  uint32_t with_keys = 0, over_objs = 0;
  for (uint32_t j = 0; j < N; j++) {
    with_keys += csid[j] != 0;
    over_objs += csid[j] == 1;
  }
  in.sid_count = with_keys;
  in.oversize_oid_count = over_objs;
  in.o_start_time_min = osmin;
  in.o_start_time_max = osmax;
  in.o_end_time_min = o_etm;
  in.o_end_time_max = o_etmax;
  in.bitmap_edge = edge;
  return R;
}

extern "C" int cmp_get(const cmp_result *r, stc_ctb_info *info) {
  if (!r) return -1;
  *info = r->info;
  return 0;
}

extern "C" int cmp_read(const cmp_result *r, stc_ctf *ctfs, uint8_t *bitmaps, uint8_t *keys, uint16_t *sids,
                        uint64_t *okeys, float *oboxes, uint8_t *obitmap) {
  if (!r) return -1;
  if (ctfs) memcpy(ctfs, r->ctfs.data(), r->ctfs.size() * sizeof(stc_ctf));
  if (bitmaps) memcpy(bitmaps, r->bitmaps.data(), r->bitmaps.size());
  if (keys && !r->keys.empty()) memcpy(keys, r->keys.data(), r->keys.size());
  if (sids) memcpy(sids, r->sids.data(), r->sids.size() * sizeof(uint16_t));
  if (okeys && !r->okeys.empty()) memcpy(okeys, r->okeys.data(), r->okeys.size() * sizeof(uint64_t));
  if (oboxes && !r->oboxes.empty()) memcpy(oboxes, r->oboxes.data(), r->oboxes.size() * sizeof(float));
  if (obitmap) memcpy(obitmap, r->obitmap.data(), r->obitmap.size());
  return 0;
}

extern "C" void cmp_free(cmp_result *r) { delete r; }
