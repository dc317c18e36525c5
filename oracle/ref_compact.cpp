// Harness that runs the reference's own compaction (merge_dump,
// tools/compaction.cpp:729-1206) on block files, to pin the oracle's
// restatement (oracle/stc_compact.cpp, reference mode).
//
// Written for this project; links against the reference's unmodified
// tools/compaction.cpp (its `main` renamed at compile time, never called) and
// tracing/{workbench,step_merge,...}.cpp, compiled in place by
// oracle/build_ref.sh. The reference loads the input blocks with its own
// workbench::load_CTB_meta / load_CTF_keys and writes the compacted block with
// workbench::dump_CTB_meta, CTF::dump_meta and CTF::dump_keys.
//
// Usage (run inside <dir>):
//   ref_compact <num_objects> <ctf_count> <split> <blocks> <max_meet_time> <x0> <y0> <x1> <y1>
// Inputs:  m/N_CTB<i>, m/N_STcL<i>-<j>, r<j%2>/N_SSTable_<i>-<j>   (i < blocks, j < ctf_count)
// Outputs: m/2G_CTB0, m/2G_STcL0-<c>, r<c%2>/2G_SSTable_0-<c>     (c < split^2)
//
// Two settings differ from the reference's experiment driver (main at
// tools/compaction.cpp:1352-1448), both without effect on the written bytes:
// bitmaps_size is the size of one oversize bitmap (the driver's value, one
// bitmap per CTF, makes merge_dump read past the 8 KB bitmaps it ORs,
// tools/compaction.cpp:1110-1112, while only the first 8 KB are written),
// and the reference's serialize_mbr (cuda/geometry.cu:161-171, a CUDA file)
// is supplied by its host twin CTF::serial_mbr (tracing/step_merge.cpp:290-310),
// which has the same arithmetic.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "tracing/workbench.h"

using namespace std;

void *merge_dump(workbench *bench, uint start_ctb, uint merge_ctb_count, vector<vector<key_info> > &keys_with_sid,
                 vector<vector<f_box> > &mbrs_with_sid, vector<vector<uint> > &invert_index,
                 vector<pair<vector<key_info>, vector<f_box> > > &objects_map, vector<object_info> &str_list);

uint64_t serialize_mbr(f_box *b, f_box *bitmap_mbr, CTF *ctf) {
  if (bitmap_mbr != &ctf->ctf_mbr) {
    fprintf(stderr, "serialize_mbr: box not the CTF's own\n");
    exit(3);
  }
  return ctf->serial_mbr(b);
}

// Referenced only by the renamed driver, which is never called.
workbench *load_meta(const char *, uint, uint) {
  fprintf(stderr, "load_meta is not available in the harness\n");
  exit(3);
}

int main(int argc, char **argv) {
  if (argc != 10) {
    fprintf(stderr, "usage: %s num_objects ctf_count split blocks max_meet_time x0 y0 x1 y1\n", argv[0]);
    return 2;
  }
  configuration config;
  config.num_objects = (uint)strtoul(argv[1], nullptr, 10);
  config.CTF_count = (uint)strtoul(argv[2], nullptr, 10);
  config.split_num = (uint)strtoul(argv[3], nullptr, 10);
  const uint blocks = (uint)strtoul(argv[4], nullptr, 10);
  config.max_meet_time = (uint)strtoul(argv[5], nullptr, 10);
  config.num_threads = 1;
  config.G_bytes = 2;
  strcpy(config.CTB_meta_path, "m/");
  strcpy(config.raid_path, "r");
  box map(strtod(argv[6], nullptr), strtod(argv[7], nullptr), strtod(argv[8], nullptr), strtod(argv[9], nullptr));

  workbench *bench = new workbench(&config);
  bench->mbr = map;
  bench->bit_count = 256 * 256;
  bench->bitmaps_size = bench->bit_count / 8;
  bench->ctbs = new CTB[blocks];
  for (uint i = 0; i < blocks; i++) bench->load_CTB_meta("m/N", (int)i);

  const uint F2 = config.split_num * config.split_num;
  vector<object_info> str_list(config.num_objects);
  vector<vector<key_info> > keys_with_sid(F2);
  vector<vector<f_box> > mbrs_with_sid(F2);
  vector<vector<uint> > invert_index(F2);
  vector<pair<vector<key_info>, vector<f_box> > > objects_map(config.num_objects);
  merge_dump(bench, 0, blocks, keys_with_sid, mbrs_with_sid, invert_index, objects_map, str_list);
  return 0;
}
