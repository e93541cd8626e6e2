// SDGC command-line driver: the reference's flags, data paths and stdout
// grammar (main/SDGC.cu:13-110) on top of the C ABI.
//
//   SDGC -m {SNICIT,BF,SNIG,XY} -n N -l L -t threshold -b batch
//
// Reads ../dataset/SDGC/tsv_weights/neuron{N}/n{N}-l{l}.tsv,
// ../dataset/SDGC/MNIST/sparse-images-{N}.tsv and checks against
// ../dataset/SDGC/MNIST/neuron{N}-l{L}-categories.tsv, like the reference.
// Extra flags (not in the reference): --data DIR replaces ../dataset/SDGC;
// --synthetic SEED generates the weights and inputs in memory instead of
// reading TSV files; --num-inputs K (default 60000); --write-data writes the
// synthetic set in the reference layout under --data; --write-golden writes
// the category file; --centroids K; --autotune.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "snicit_gb300.h"

static bool exists(const std::string& p) {
  struct stat st;
  return ::stat(p.c_str(), &st) == 0;
}

// mkdir -p
static void make_dirs(const std::string& path) {
  for (size_t i = 1; i <= path.size(); ++i)
    if (i == path.size() || path[i] == '/') ::mkdir(path.substr(0, i).c_str(), 0755);
}

static int die(sdnn_engine* e, int rc, const char* what) {
  std::fprintf(stderr, "%s failed: %s (%s)\n", what, sdnn_status_string(rc),
               e ? sdnn_last_error(e) : "");
  return 1;
}

int main(int argc, char** argv) {
  std::string mode = "SNICIT";
  long num_neurons = 1024, num_layers = 120, batch = 60000, num_inputs = 60000;
  int threshold = 30, centroids = 32;
  std::string data = "../dataset/SDGC";
  bool synthetic = false, write_data = false, write_golden = false, autotune = false;
  unsigned long long seed = 20260101ull;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&](const char* flag) -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "%s needs a value\n", flag);
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "-m" || a == "--mode") mode = next("-m");
    else if (a == "-n" || a == "--num_neurons") num_neurons = std::atol(next("-n"));
    else if (a == "-l" || a == "--num_layers") num_layers = std::atol(next("-l"));
    else if (a == "-t" || a == "--threshold") threshold = std::atoi(next("-t"));
    else if (a == "-b" || a == "--input_batch_size") batch = std::atol(next("-b"));
    else if (a == "--data") data = next("--data");
    else if (a == "--synthetic") { synthetic = true; seed = std::strtoull(next("--synthetic"), nullptr, 10); }
    else if (a == "--num-inputs") num_inputs = std::atol(next("--num-inputs"));
    else if (a == "--write-data") write_data = true;
    else if (a == "--write-golden") write_golden = true;
    else if (a == "--centroids") centroids = std::atoi(next("--centroids"));
    else if (a == "--autotune") autotune = true;
    else if (a == "-h" || a == "--help") {
      std::printf("SNICIT-SDGC (GB300)\n  -m,--mode SNICIT|BF|SNIG|XY\n  -n,--num_neurons N\n"
                  "  -l,--num_layers L\n  -t,--threshold T\n  -b,--input_batch_size B\n");
      return 0;
    } else {
      std::fprintf(stderr, "unknown option %s\n", a.c_str());
      return 2;
    }
  }
  std::map<std::string, int> modes = {{"BF", SDNN_MODE_BF}, {"SNIG", SDNN_MODE_SNIG},
                                      {"XY", SDNN_MODE_XY}, {"SNICIT", SDNN_MODE_SNICIT}};
  if (!modes.count(mode)) {
    std::fprintf(stderr, "Error mode. Please correct your mode name\n");
    return 1;
  }
  const std::string weight_path = data + "/tsv_weights/neuron" + std::to_string(num_neurons);
  const std::string input_path = data + "/MNIST/sparse-images-" + std::to_string(num_neurons) + ".tsv";
  const std::string golden_path = data + "/MNIST/neuron" + std::to_string(num_neurons) + "-l" +
                                  std::to_string(num_layers) + "-categories.tsv";
  std::cout << "Current mode: " << mode << std::endl;

  sdnn_config cfg;
  sdnn_config_default(&cfg);
  cfg.num_neurons = (int32_t)num_neurons;
  cfg.num_layers = (int32_t)num_layers;
  cfg.mode = modes[mode];
  cfg.threshold = threshold;
  cfg.batch = std::min(batch, num_inputs);
  cfg.bias = sdnn_reference_bias((int32_t)num_neurons);
  cfg.num_centroids = centroids;
  cfg.seed = seed;
  sdnn_engine* e = nullptr;
  int rc = sdnn_create(&cfg, &e);
  if (rc) return die(e, rc, "sdnn_create");

  std::vector<float> Y0((size_t)num_inputs * num_neurons);
  if (synthetic) {
    rc = sdnn_generate_weights(e, seed, 32, 0.0625f);
    if (rc) return die(e, rc, "sdnn_generate_weights");
    rc = sdnn_generate_inputs((int32_t)num_neurons, seed, 0, num_inputs, Y0.data());
    if (rc) return die(e, rc, "sdnn_generate_inputs");
    if (write_data) {
      make_dirs(weight_path);
      make_dirs(data + "/MNIST");
      if ((rc = sdnn_write_weights_tsv(e, weight_path.c_str()))) return die(e, rc, "write weights");
      if ((rc = sdnn_write_inputs_tsv(input_path.c_str(), Y0.data(), num_inputs, (int32_t)num_neurons)))
        return die(e, rc, "write inputs");
    }
  } else {
    std::cout << "Loading the weight......" << std::endl;
    rc = sdnn_load_weights_tsv(e, weight_path.c_str());
    if (rc) return die(e, rc, "sdnn_load_weights_tsv");
    rc = sdnn_read_inputs_tsv(input_path.c_str(), (int32_t)num_neurons, 0, num_inputs, Y0.data());
    if (rc) return die(e, rc, "sdnn_read_inputs_tsv");
  }
  rc = sdnn_finalize_weights(e);
  if (rc) return die(e, rc, "sdnn_finalize_weights");
  if (autotune) {
    const long sample = std::min<long>(num_inputs, 8192);
    rc = sdnn_autotune(e, Y0.data(), sample, "autotune_record.jsonl");
    if (rc) return die(e, rc, "sdnn_autotune");
  }
  std::vector<int32_t> flags(num_inputs), ids(num_inputs);
  int64_t count = 0;
  // warm-up (graph capture and allocation are not part of the reference's timed region)
  rc = sdnn_infer_host(e, Y0.data(), num_inputs, flags.data(), ids.data(), &count);
  if (rc) return die(e, rc, "sdnn_infer_host");
  rc = sdnn_infer_host(e, Y0.data(), num_inputs, flags.data(), ids.data(), &count);
  if (rc) return die(e, rc, "sdnn_infer_host");
  sdnn_stats st;
  sdnn_get_stats(e, &st);
  const int post_layers = std::max(1, (int)num_layers - std::min(threshold, (int)num_layers));
  if (mode == "SNICIT") {
    std::cout << "pre-conv Time [SNICIT] = " << st.stage_ms[0] << "ms" << std::endl;
    std::cout << "cluster-based conversion Time [overhead] = " << st.stage_ms[1] << "ms" << std::endl;
    std::cout << "post-conv Time [SNICIT] = " << st.stage_ms[2] << "ms" << std::endl;
    std::cout << "recover Time [SNICIT] = " << st.stage_ms[3] << "ms" << std::endl;
    std::cout << "SNICIT info: runtime " << st.total_ms << "ms avgpost "
              << st.stage_ms[2] / post_layers << "ms" << std::endl;
  } else if (mode == "XY") {
    std::cout << "XY info: runtime " << st.total_ms << "ms avgpost " << st.stage_ms[2] / post_layers
              << "ms" << std::endl;
  } else {
    std::cout << mode << " info: runtime " << st.total_ms << " ms" << std::endl;
  }
  if (write_golden) {
    rc = sdnn_write_categories_tsv(golden_path.c_str(), ids.data(), count);
    if (rc) return die(e, rc, "write golden");
  } else if (exists(golden_path)) {
    std::vector<int32_t> golden(num_inputs, 0);
    std::ifstream g(golden_path);
    std::string line;
    while (std::getline(g, line)) {
      if (line.empty()) continue;
      const long id = std::atol(line.c_str());
      if (id >= 1 && id <= num_inputs) golden[id - 1] = 1;
    }
    long diff = 0;
    for (long i = 0; i < num_inputs; ++i) diff += (golden[i] != (flags[i] ? 1 : 0));
    std::cout << "\nNumber of different categories: " << diff << std::endl;
    std::cout << (diff == 0 ? "CHALLENGE PASSED" : "CHALLENGE FAILED") << std::endl;
  } else {
    std::cout << "golden file not found: " << golden_path << std::endl;
  }
  sdnn_destroy(e);
  return 0;
}
