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

#include <cuda_runtime.h>

#include "snicit_gb300.h"

namespace sdnn {
int engine_set_tile(sdnn_engine* e, int tile_rows, int threads);
void engine_set_snicit(sdnn_engine* e, int threshold, int centroids);
void engine_set_merge(sdnn_engine* e, int start, int every, bool on);
bool engine_set_sparse(sdnn_engine* e, bool on);
sdnn_config engine_config(const sdnn_engine* e);
}  // namespace sdnn

namespace {

struct Trial {
  int tile, threads, threshold, centroids, merge_start;
  float ms;
  int64_t survivors;
  int status;
};

// One inference of the sample: host rows (copied in) or device rows.
struct Sample {
  const float* host = nullptr;
  const float* dev = nullptr;
  int64_t rows = 0;
  int32_t* d_flags = nullptr;  // device path: flags buffer
};

int run_once(sdnn_engine* e, const Sample& smp, int64_t& survivors) {
  if (smp.host) return sdnn_infer_host(e, smp.host, smp.rows, nullptr, nullptr, &survivors);
  int rc = sdnn_infer_device(e, smp.dev, smp.rows, smp.d_flags, nullptr);
  if (rc) return rc;
  std::vector<int32_t> flags((size_t)smp.rows);
  if (cudaDeviceSynchronize() != cudaSuccess ||
      cudaMemcpy(flags.data(), smp.d_flags, flags.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return SDNN_ERR_CUDA;
  survivors = 0;
  for (int32_t v : flags) survivors += v != 0;
  return SDNN_OK;
}

// Times one setting: best of two runs after a warm-up (which captures the
// graph).  stage < 0 times the whole inference, else that stage only (the
// tile sweep times the plain layers, stage 0, where the tile shape matters).
int time_setting(sdnn_engine* e, const Sample& smp, int stage, float& ms, int64_t& survivors) {
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    int64_t count = 0;
    int rc = run_once(e, smp, count);
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
               "\"centroids\": %d, \"merge_start\": %d, \"rows\": %lld, \"ms\": %.4f, "
               "\"survivors\": %lld, \"status\": %d}\n",
               phase, t.tile, t.threads, t.threshold, t.centroids, t.merge_start, (long long)rows,
               t.ms, (long long)t.survivors, t.status);
  std::fflush(f);
}

int tune(sdnn_engine* e, const Sample& smp, const char* record_path) {
  FILE* f = record_path ? std::fopen(record_path, "ab") : nullptr;
  const sdnn_config cfg0 = sdnn::engine_config(e);
  const int N = cfg0.num_neurons;
  std::vector<int> tiles;
  if (N == 1024) tiles = {24, 16, 12, 8};
  else if (N == 4096) tiles = {6, 5, 4, 3, 2};
  else if (N == 16384) tiles = {3, 2, 1};
  else if (N > 32768) tiles = {3, 2, 1};
  else tiles = {8, 4, 2, 1};
  const bool merge_on = !(cfg0.flags & SDNN_FLAG_NO_MERGE);
  Trial best{0, 0, cfg0.threshold, cfg0.num_centroids, cfg0.merge_start, 1e30f, -1, 0};
  // the plain layers (stage 0) are where the tile shape matters; in SNICIT mode
  // the post layers run a handful of rows whatever the tile
  const int tile_stage =
      (cfg0.mode == SDNN_MODE_SNICIT && cfg0.threshold > 0 && cfg0.threshold < cfg0.num_layers) ? 0 : -1;
  for (int tile : tiles) {
    for (int threads : {256, 512, 1024}) {
      Trial t{tile, threads, cfg0.threshold, cfg0.num_centroids, cfg0.merge_start, 0.f, 0, 0};
      t.status = sdnn::engine_set_tile(e, tile, threads);
      if (t.status == SDNN_OK) t.status = time_setting(e, smp, tile_stage, t.ms, t.survivors);
      record(f, "tile", t, smp.rows);
      if (t.status != SDNN_OK) continue;
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
    // thresholds {30, 60, 120, 240} x centroid counts {50, 100, 200}, and no
    // clustering at all (threshold = L: the plain path with merging), so the
    // chosen setting is never slower than plain on the sample
    std::vector<int> ths;
    for (int th : {30, 60, 120, 240})
      if (th < cfg0.num_layers) ths.push_back(th);
    ths.push_back(cfg0.num_layers);
    for (int th : ths) {
      for (int k : {50, 100, 200}) {
        if (th == cfg0.num_layers && k != 50) continue;  // no clustering: one trial
        sdnn::engine_set_snicit(e, th, k);
        Trial t{best.tile, best.threads, th, k, cfg0.merge_start, 0.f, 0, 0};
        t.status = time_setting(e, smp, -1, t.ms, t.survivors);
        record(f, "snicit", t, smp.rows);
        if (t.status != SDNN_OK) continue;
        if (t.ms < bs.ms) bs = t;
      }
    }
    if (bs.ms < 1e30f) sdnn::engine_set_snicit(e, bs.threshold, bs.centroids);
    else sdnn::engine_set_snicit(e, cfg0.threshold, cfg0.num_centroids);
    // residue rows at the chosen threshold: sparse residue lists or dense rows
    // only, whichever is faster on the sample
    if (bs.ms < 1e30f && bs.threshold < cfg0.num_layers) {
      const bool sparse0 = !(cfg0.flags & SDNN_FLAG_DENSE_RESIDUE);
      if (sdnn::engine_set_sparse(e, !sparse0) != sparse0) {
        Trial t = bs;
        t.status = time_setting(e, smp, -1, t.ms, t.survivors);
        record(f, sparse0 ? "dense_residue" : "sparse_residue", t, smp.rows);
        if (t.status == SDNN_OK && t.ms < bs.ms) bs = t;
        else sdnn::engine_set_sparse(e, sparse0);
      }
    }
    if (merge_on && bs.ms < 1e30f) {
      // first layer after which identical rows are merged: early merging finds
      // duplicates sooner, late merging skips hashing rows that are all distinct;
      // and the spacing of the later merge steps (each costs three launches)
      Trial bm = bs;
      int best_every = cfg0.merge_every;
      for (int every : {1, 2, 4, 8}) {
        for (int ms : {2, 4, 6, 8, 10, 12, 16}) {
          if (ms >= bs.threshold) continue;  // no merge below the threshold
          sdnn::engine_set_merge(e, ms, every, true);
          Trial t{bs.tile, bs.threads, bs.threshold, bs.centroids, ms, 0.f, 0, 0};
          t.status = time_setting(e, smp, -1, t.ms, t.survivors);
          char phase[24];
          std::snprintf(phase, sizeof phase, "merge_every%d", every);
          record(f, phase, t, smp.rows);
          if (t.status == SDNN_OK && t.ms < bm.ms) {
            bm = t;
            best_every = every;
          }
        }
      }
      sdnn::engine_set_merge(e, bm.merge_start, best_every, true);
      // with merging on, clustering earlier than the sweep's thresholds can
      // pay (the merged rows may be down to a few centroids sooner): thresholds
      // below the chosen one and above the first merge, with that merge setting
      if (bs.threshold < cfg0.num_layers) {
        Trial bt = bm;
        for (int th : {12, 16, 20, 24}) {
          if (th >= bm.threshold || th <= bm.merge_start) continue;
          sdnn::engine_set_snicit(e, th, bm.centroids);
          Trial t{bm.tile, bm.threads, th, bm.centroids, bm.merge_start, 0.f, 0, 0};
          t.status = time_setting(e, smp, -1, t.ms, t.survivors);
          record(f, "snicit_merged", t, smp.rows);
          if (t.status == SDNN_OK && t.ms < bt.ms) bt = t;
        }
        sdnn::engine_set_snicit(e, bt.threshold, bt.centroids);
      }
    }
  }
  if (f) std::fclose(f);
  return SDNN_OK;
}

}  // namespace

extern "C" int sdnn_autotune(sdnn_engine* e, const float* Y0, int64_t rows,
                             const char* record_path) {
  if (!e || !Y0 || rows <= 0) return SDNN_ERR_INVALID;
  Sample smp;
  smp.host = Y0;
  smp.rows = rows;
  return tune(e, smp, record_path);
}

extern "C" int sdnn_autotune_device(sdnn_engine* e, const float* d_Y0, int64_t rows,
                                    const char* record_path) {
  if (!e || !d_Y0 || rows <= 0) return SDNN_ERR_INVALID;
  Sample smp;
  smp.dev = d_Y0;
  smp.rows = rows;
  if (cudaMalloc((void**)&smp.d_flags, (size_t)rows * 4) != cudaSuccess) {
    cudaGetLastError();
    return SDNN_ERR_OOM;
  }
  const int rc = tune(e, smp, record_path);
  cudaFree(smp.d_flags);
  return rc;
}
