// Autotuner: picks the layer-kernel tile (rows per CTA, threads per CTA) and,
// in SNICIT mode, the threshold layer and centroid-candidate count by timing
// full inferences on a caller-supplied sample of rows.  Every trial is
// appended as one JSON line to the record file, with the survivor count so a
// reader can check that all settings returned the same category set.
//
// The reference hard-codes these choices (threshold default 30,
// main/SDGC.cu:38-42; 32 candidates, src/SDGC/SNICIT/SNICIT.hpp:228-229;
// fixed launch shapes, SNICIT.hpp:364-536).
#include <cstdio>
#include <string>
#include <vector>

#include "snicit_gb300.h"

namespace sdnn {
int engine_set_tile(sdnn_engine* e, int tile_rows, int threads);
void engine_set_snicit(sdnn_engine* e, int threshold, int centroids);
sdnn_config engine_config(const sdnn_engine* e);
}  // namespace sdnn

namespace {

struct Trial {
  int tile, threads, threshold, centroids;
  float ms;
  int64_t survivors;
  int status;
};

// Times one setting: best of two runs after a warm-up (which captures the
// graph).  stage < 0 times the whole inference, else that stage only (the
// tile sweep times the plain layers, stage 0, where the tile shape matters).
int time_setting(sdnn_engine* e, const float* Y0, int64_t rows, int stage, float& ms,
                 int64_t& survivors) {
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    int64_t count = 0;
    int rc = sdnn_infer_host(e, Y0, rows, nullptr, nullptr, &count);
    if (rc) return rc;
    sdnn_stats st{};
    rc = sdnn_get_stats(e, &st);
    if (rc) return rc;
    const float t = stage < 0 ? st.total_ms : st.stage_ms[stage];
    if (rep > 0 && t < best) best = t;
    survivors = count;
  }
  ms = best;
  return SDNN_OK;
}

void record(FILE* f, const char* phase, const Trial& t, int64_t rows) {
  if (!f) return;
  std::fprintf(f,
               "{\"phase\": \"%s\", \"tile_rows\": %d, \"threads\": %d, \"threshold\": %d, "
               "\"centroids\": %d, \"rows\": %lld, \"ms\": %.4f, \"survivors\": %lld, "
               "\"status\": %d}\n",
               phase, t.tile, t.threads, t.threshold, t.centroids, (long long)rows, t.ms,
               (long long)t.survivors, t.status);
  std::fflush(f);
}

}  // namespace

extern "C" int sdnn_autotune(sdnn_engine* e, const float* Y0, int64_t rows,
                             const char* record_path) {
  if (!e || !Y0 || rows <= 0) return SDNN_ERR_INVALID;
  FILE* f = record_path ? std::fopen(record_path, "ab") : nullptr;
  const sdnn_config cfg0 = sdnn::engine_config(e);
  const int N = cfg0.num_neurons;
  std::vector<int> tiles;
  if (N == 1024) tiles = {24, 16, 12, 8};
  else if (N == 4096) tiles = {6, 5, 4, 3, 2};
  else if (N == 16384) tiles = {3, 2, 1};
  else if (N > 32768) tiles = {3, 2, 1};
  else tiles = {8, 4, 2, 1};
  Trial best{0, 0, cfg0.threshold, cfg0.num_centroids, 1e30f, -1, 0};
  // the plain layers (stage 0) are where the tile shape matters; in SNICIT mode
  // the post layers run a handful of rows whatever the tile
  const int tile_stage =
      (cfg0.mode == SDNN_MODE_SNICIT && cfg0.threshold > 0 && cfg0.threshold < cfg0.num_layers) ? 0 : -1;
  int64_t ref_survivors = -1;
  for (int tile : tiles) {
    for (int threads : {256, 512}) {
      Trial t{tile, threads, cfg0.threshold, cfg0.num_centroids, 0.f, 0, 0};
      t.status = sdnn::engine_set_tile(e, tile, threads);
      if (t.status == SDNN_OK) t.status = time_setting(e, Y0, rows, tile_stage, t.ms, t.survivors);
      record(f, "tile", t, rows);
      if (t.status != SDNN_OK) continue;
      if (ref_survivors < 0) ref_survivors = t.survivors;
      if (t.ms < best.ms) best = t;
    }
  }
  if (best.ms >= 1e30f) {
    if (f) std::fclose(f);
    sdnn::engine_set_tile(e, cfg0.tile_rows, cfg0.threads);
    return SDNN_ERR_UNSUPPORTED;
  }
  sdnn::engine_set_tile(e, best.tile, best.threads);
  if (cfg0.mode == SDNN_MODE_SNICIT) {
    Trial bs = best;
    bs.ms = 1e30f;
    for (int th : {30, 60, 120, 240}) {
      if (th >= cfg0.num_layers) continue;
      for (int k : {50, 100, 200}) {
        sdnn::engine_set_snicit(e, th, k);
        Trial t{best.tile, best.threads, th, k, 0.f, 0, 0};
        t.status = time_setting(e, Y0, rows, -1, t.ms, t.survivors);
        record(f, "snicit", t, rows);
        if (t.status != SDNN_OK) continue;
        if (t.ms < bs.ms) bs = t;
      }
    }
    if (bs.ms < 1e30f) sdnn::engine_set_snicit(e, bs.threshold, bs.centroids);
    else sdnn::engine_set_snicit(e, cfg0.threshold, cfg0.num_centroids);
  }
  if (f) std::fclose(f);
  return SDNN_OK;
}
