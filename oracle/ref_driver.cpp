// Harness that runs the reference's own CPU co-occurrence path, single
// threaded, on a trace file and writes every emitted meeting per step.
//
// This file is written for this project; it links against the reference's
// unmodified sources (compiled in place by oracle/build_ref.sh) and drives
// them the way the reference's tracer::process does for its CPU branch
// (tracing/process.cpp:401-459 and :608-612):
//   partitioner::build_schema on the step-0 positions (tracing/filter.cpp:27),
//   then per step reset, filter, reachability, update_meetings
//   (tracing/workbench.h:323, tracing/filter.cpp:290,
//    tracing/refinement.cpp:66, tracing/meeting.cpp:78),
//   read h_meetings_ps[0..kv_count) (tracing/meeting.cpp:11-24),
//   then update_schema (tracing/filter.cpp:428).
// tracer::process itself cannot be reused: it generates positions internally
// with an unseeded generator and returns after its first memtable dump.
//
// Usage:
//   ref_driver <trace.bin> <out.bin> reach min_meet grid_capacity grid_amplify
//              num_buckets refine_size threads dynamic_schema
// trace.bin: u32 N, u32 T, f64 mbr[4] (low x, low y, high x, high y), then
//            T*N (x, y) f64 pairs, layout [t][oid].
// out.bin:   per step: u32 t, u32 count, u32 units, u32 leaves, then count
//            records of u32 (pid_lo, pid_hi, start, end).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>

#include "tracing/partitioner.h"
#include "tracing/workbench.h"

static uint64_t isqrt_u64(uint64_t v) {
  uint64_t r = (uint64_t)sqrtl((long double)v);
  while (r * r > v) r--;
  while ((r + 1) * (r + 1) <= v) r++;
  return r;
}

// Exact integer inverse of the Cantor pairing (util/util.h:68-70).
static void cantor_decode(uint64_t z, uint32_t *a, uint32_t *b) {
  uint64_t w = (isqrt_u64(8 * z + 1) - 1) / 2;
  uint64_t t = (w * w + w) / 2;
  uint64_t y = z - t;
  *b = (uint32_t)y;
  *a = (uint32_t)(w - y);
}

int main(int argc, char **argv) {
  if (argc < 11) {
    fprintf(stderr, "usage: %s trace.bin out.bin reach min_meet grid_capacity grid_amplify "
                    "num_buckets refine_size threads dynamic_schema\n", argv[0]);
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) { perror("trace"); return 2; }
  uint32_t N = 0, T = 0;
  double mb[4];
  if (fread(&N, 4, 1, f) != 1 || fread(&T, 4, 1, f) != 1 || fread(mb, 8, 4, f) != 4) return 2;
  std::vector<Point> trace((size_t)N * T);
  std::vector<double> buf((size_t)N * 2);
  for (uint32_t t = 0; t < T; t++) {
    if (fread(buf.data(), 16, N, f) != N) { fprintf(stderr, "short trace\n"); return 2; }
    for (uint32_t i = 0; i < N; i++) {
      trace[(size_t)t * N + i].x = buf[2 * i];
      trace[(size_t)t * N + i].y = buf[2 * i + 1];
    }
  }
  fclose(f);

  generator_configuration *cfg = new generator_configuration();
  cfg->num_objects = N;
  cfg->duration = T;
  cfg->reach_distance = atof(argv[3]);
  cfg->min_meet_time = (uint)atoi(argv[4]);
  cfg->grid_capacity = (uint)atoi(argv[5]);
  cfg->grid_amplify = atof(argv[6]);
  cfg->num_meeting_buckets = (size_t)strtoull(argv[7], nullptr, 10);
  cfg->refine_size = (uint)atoi(argv[8]);
  cfg->num_threads = (uint)atoi(argv[9]);
  cfg->dynamic_schema = atoi(argv[10]) != 0;
  cfg->gpu = false;
  cfg->phased_lookup = true;
  cfg->zone_capacity = cfg->grid_capacity;

  box mbr(mb[0], mb[1], mb[2], mb[3]);
  partitioner part(mbr, cfg);
  workbench *bench = part.build_schema(trace.data(), N);
  bench->mbr = mbr;

  FILE *o = fopen(argv[2], "wb");
  if (!o) { perror("out"); return 2; }
  for (uint32_t t = 0; t < T; t++) {
    bench->reset();
    bench->points = trace.data() + (size_t)t * N;
    bench->cur_time = t;
    bench->filter();
    bench->reachability();
    bench->update_meetings();
    uint32_t cnt = bench->kv_count;
    uint32_t units = bench->grid_check_counter;
    uint32_t leaves = bench->grids_stack_index;
    fwrite(&t, 4, 1, o);
    fwrite(&cnt, 4, 1, o);
    fwrite(&units, 4, 1, o);
    fwrite(&leaves, 4, 1, o);
    for (uint32_t i = 0; i < cnt; i++) {
      meeting_unit &m = bench->h_meetings_ps[i];
      uint32_t rec[4];
      cantor_decode((uint64_t)m.key, &rec[0], &rec[1]);
      rec[2] = m.start;
      rec[3] = m.end;
      fwrite(rec, 4, 4, o);
    }
    if (cfg->dynamic_schema) bench->update_schema();
  }
  fclose(o);
  return 0;
}
