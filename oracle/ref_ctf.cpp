// Harness that runs the reference's own host code for the CTF encoding of a
// flushed block, to pin the oracle's restatement (oracle/stc_lsm.c).
//
// Written for this project; links against the reference's unmodified
// tracing/step_merge.cpp (compiled in place by oracle/build_ref.sh) and calls
//   CTF::get_ctf_bits (tracing/step_merge.cpp:140-186),
//   CTF::serial_mbr   (:290-310; the host twin of serialize_mbr,
//                      cuda/geometry.cu:161-171),
//   CTF::serial_key   (:284-288),
//   oversize_buffer::write_o_buffer (:41-63),
//   CTF::parse_key, CTF::new_parse_mbr, CTF::ctf_get_key_oid (:329-379).
//
// Usage: ref_ctf <in.bin> <out.bin>
//        ref_ctf layout      (offsets and sizes of CTF, CTB, oversize_buffer)
// in.bin:  f64 map[4], u32 num_objects, u32 max_meet_time, u32 n_cases,
//          n_cases x { f32 ctf_mbr[4], f32 box[4], u64 pid_field, u32 target,
//                      u32 duration, u32 end },
//          u32 end_time_min, u32 n_boxes, n_boxes x { f32 box[4], u32 duration, u32 end }
// out.bin: n_cases x { u16 key_bit, id_bit, duration_bit, end_bit, low_x_bit,
//                      low_y_bit, edge_bit, mbr_bit, x_grid, y_grid; u32 bitmap_size;
//                      u64 value_mbr; u64 key_lo, key_hi; u32 oid, target, duration,
//                      end; u64 value_mbr; f64 box[4] (the stored key decoded) },
//          u8 o_bitmap[8192], u32 o_start_time_min, o_start_time_max
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "tracing/step_merge.h"

template <typename T>
static bool rd(FILE *f, T *v, size_t n = 1) { return fread(v, sizeof(T), n, f) == n; }

// Byte layout of the reference's on-disk structs (CTF::dump_meta and
// workbench::dump_CTB_meta write them raw): "name offset size" lines.
#define FIELD(T, f) printf("%s.%s %zu %zu\n", #T, #f, offsetof(T, f), sizeof(((T *)nullptr)->f))
static int print_layout() {
  printf("CTF %zu %zu\n", sizeof(CTF), alignof(CTF));
  FIELD(CTF, ctf_mbr); FIELD(CTF, keys); FIELD(CTF, bitmap); FIELD(CTF, CTF_kv_capacity);
  FIELD(CTF, start_time_min); FIELD(CTF, start_time_max); FIELD(CTF, end_time_min); FIELD(CTF, end_time_max);
  FIELD(CTF, ctf_bitmap_size); FIELD(CTF, key_bit); FIELD(CTF, id_bit); FIELD(CTF, duration_bit);
  FIELD(CTF, end_bit); FIELD(CTF, low_x_bit); FIELD(CTF, low_y_bit); FIELD(CTF, edge_bit); FIELD(CTF, mbr_bit);
  FIELD(CTF, x_grid); FIELD(CTF, y_grid);
  printf("CTB %zu %zu\n", sizeof(CTB), alignof(CTB));
  FIELD(CTB, ctfs); FIELD(CTB, CTF_count); FIELD(CTB, start_time_min); FIELD(CTB, start_time_max);
  FIELD(CTB, end_time_min); FIELD(CTB, end_time_max); FIELD(CTB, first_widpid); FIELD(CTB, sids);
  FIELD(CTB, bitmaps); FIELD(CTB, bitmap_mbrs); FIELD(CTB, CTF_capacity); FIELD(CTB, o_buffer);
  FIELD(CTB, box_rtree);
  printf("oversize_buffer %zu %zu\n", sizeof(oversize_buffer), alignof(oversize_buffer));
  FIELD(oversize_buffer, oversize_kv_count); FIELD(oversize_buffer, keys); FIELD(oversize_buffer, boxes);
  FIELD(oversize_buffer, o_bitmaps); FIELD(oversize_buffer, start_time_min); FIELD(oversize_buffer, start_time_max);
  FIELD(oversize_buffer, end_time_min); FIELD(oversize_buffer, end_time_max);
  printf("f_box %zu %zu\n", sizeof(f_box), alignof(f_box));
  return 0;
}

int main(int argc, char **argv) {
  if (argc == 2 && strcmp(argv[1], "layout") == 0) return print_layout();
  if (argc < 3) {
    fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) { perror("in"); return 2; }
  double mp[4];
  uint32_t num_objects = 0, max_meet = 0, n = 0;
  if (!rd(f, mp, 4) || !rd(f, &num_objects) || !rd(f, &max_meet) || !rd(f, &n)) return 2;
  box map_mbr(mp[0], mp[1], mp[2], mp[3]);
  configuration config;
  config.num_objects = num_objects;
  config.max_meet_time = max_meet;
  FILE *o = fopen(argv[2], "wb");
  if (!o) { perror("out"); return 2; }
  for (uint32_t i = 0; i < n; i++) {
    float cm[4], b[4];
    uint64_t pid_field = 0;
    uint32_t target = 0, duration = 0, end = 0;
    if (!rd(f, cm, 4) || !rd(f, b, 4) || !rd(f, &pid_field) || !rd(f, &target) || !rd(f, &duration) ||
        !rd(f, &end))
      return 2;
    CTF ctf;
    ctf.ctf_mbr.low[0] = cm[0]; ctf.ctf_mbr.low[1] = cm[1];
    ctf.ctf_mbr.high[0] = cm[2]; ctf.ctf_mbr.high[1] = cm[3];
    ctf.get_ctf_bits(map_mbr, &config);
    f_box fb;
    fb.low[0] = b[0]; fb.low[1] = b[1]; fb.high[0] = b[2]; fb.high[1] = b[3];
    uint64_t value_mbr = ctf.serial_mbr(&fb);
    __uint128_t key = ctf.serial_key(pid_field, target, duration, end, value_mbr);
    uint16_t bits[10] = {ctf.key_bit, ctf.id_bit, ctf.duration_bit, ctf.end_bit, ctf.low_x_bit,
                         ctf.low_y_bit, ctf.edge_bit, ctf.mbr_bit, ctf.x_grid, ctf.y_grid};
    uint32_t bsize = ctf.ctf_bitmap_size;
    uint64_t klo = (uint64_t)key, khi = (uint64_t)(key >> 64);
    fwrite(bits, 2, 10, o);
    fwrite(&bsize, 4, 1, o);
    fwrite(&value_mbr, 8, 1, o);
    fwrite(&klo, 8, 1, o);
    fwrite(&khi, 8, 1, o);
    // decode the key as stored: its low key_bit/8 bytes (CTF::parse_key,
    // CTF::new_parse_mbr, CTF::ctf_get_key_oid)
    __uint128_t stored = 0;
    memcpy(&stored, &key, ctf.key_bit / 8);
    key_info ki;
    uint64_t vm2 = 0;
    ctf.parse_key(stored, ki, vm2);
    box db = ctf.new_parse_mbr(vm2);
    uint32_t dec[4] = {ctf.ctf_get_key_oid(stored), ki.target, ki.duration, ki.end};
    fwrite(dec, 4, 4, o);
    fwrite(&vm2, 8, 1, o);
    double dbx[4] = {db.low[0], db.low[1], db.high[0], db.high[1]};
    fwrite(dbx, 8, 4, o);
  }
  uint32_t end_time_min = 0, nb = 0;
  if (!rd(f, &end_time_min) || !rd(f, &nb)) return 2;
  oversize_buffer ob;
  std::vector<__uint128_t> keys(nb ? nb : 1);
  std::vector<f_box> boxes(nb ? nb : 1);
  for (uint32_t i = 0; i < nb; i++) {
    float b[4];
    uint32_t duration = 0, end = 0;
    if (!rd(f, b, 4) || !rd(f, &duration) || !rd(f, &end)) return 2;
    boxes[i].low[0] = b[0]; boxes[i].low[1] = b[1]; boxes[i].high[0] = b[2]; boxes[i].high[1] = b[3];
    keys[i] = ((__uint128_t)duration << 32) + end;  // END_BIT = 32 (util/util.h:52)
  }
  fclose(f);
  std::vector<unsigned char> bitmap(8192, 0);
  ob.oversize_kv_count = nb;
  ob.keys = keys.data();
  ob.boxes = boxes.data();
  ob.o_bitmaps = bitmap.data();
  ob.end_time_min = end_time_min;
  ob.start_time_min = 1u << 30;  // get_o_limit's initial values (cuda/geometry.cu:966)
  ob.start_time_max = 0;
  ob.write_o_buffer(map_mbr, 65536);
  fwrite(bitmap.data(), 1, 8192, o);
  fwrite(&ob.start_time_min, 4, 1, o);
  fwrite(&ob.start_time_max, 4, 1, o);
  ob.keys = nullptr;  // owned by the vectors
  ob.boxes = nullptr;
  ob.o_bitmaps = nullptr;
  fclose(o);
  return 0;
}
