// wlg_prerun: the reference's `prerun` program (prerun.cu:36-166) on the
// engine's C ABI.  Same flags (program_options.cpp:37-71), same output path
// (utils.cpp:88-100) and file layout (file_io.cpp:23-214):
//   init/task_id_<d>/seed_<s>/<boundary>/prob_<p>/X_<x>_Y_<y>/error_class_<e>/prerun_results.h5
// with /Histogram/<k>/Histogram (uint64 0/1, 4N+1), /Interaction/<k>/Interaction
// (int8, 2N) and /Lattice/<k>/<E>/Lattice (int8, N) per stored lattice.
// Exit status: success for a run, a help or version request, or missing
// required options (usage printed); failure on errors.

#include <cstdio>
#include <cstdlib>
#include <exception>
#include <filesystem>
#include <string>
#include <vector>

#include "../../include/wlg.h"
#include "../csrc/wlg_h5.h"
#include "cli_common.h"

int main(int argc, char** argv)
{
  using wlg::cli::Opt;
  wlg::cli::Options o({
    {"help", 'h', false, false, "", "Help"},
    {"X", 'x', true, true, "", "Ising lattice, horizontal dimension"},
    {"Y", 'y', true, true, "", "Ising lattice, vertical dimension"},
    {"prob", 'p', true, false, "", "Bit-flip error probablities"},
    {"nit", 'n', true, true, "", "Number of WL iterations"},
    {"nw", 'w', true, true, "", "Number of walkers per disorder sample"},
    {"seed", 's', true, false, "", "Random seed"},
    {"num-intervals", 'i', true, true, "", "Number of intervals in the energy spectrum"},
    {"logical-error", 'e', true, false, "i", "type of logical error coset representative"},
    {"disorder-samples", 'r', true, true, "", "Number of disorder samples"},
    {"boundary", 0, true, false, "0", "Boundary condition"},
    {"task_id", 'd', true, true, "", "Task ID"},
    {"skip-output", 0, false, false, "", "Skip writing results to the filesystem"},
    {"version", 'v', false, false, "", "Show version"},
  });
  try {
    const std::string err = o.parse(argc, argv);
    if (!err.empty()) {
      std::fprintf(stderr, "%s\n", err.c_str());
      return EXIT_FAILURE;
    }
    if (o.has("help")) {
      o.usage(argv[0], "WL pre-run usage");
      return EXIT_SUCCESS;
    }
    if (o.has("version")) {
      std::printf("WL prerun version: %s\n", wlg_version());
      return EXIT_SUCCESS;
    }
    if (const std::string m = o.missing(); !m.empty()) {
      std::fprintf(stderr, "the option '--%s' is required but missing\n", m.c_str());
      o.usage(argv[0], "WL pre-run usage");
      return EXIT_SUCCESS;
    }
    const int X = std::stoi(o.str("X")), Y = std::stoi(o.str("Y"));
    const float prob = o.has("prob") ? std::stof(o.str("prob")) : 0.0f;
    const int n_iter = std::stoi(o.str("nit")), walkers = std::stoi(o.str("nw"));
    const int seed = o.has("seed") ? std::stoi(o.str("seed")) : wlg::cli::seed_from_os();
    const int bins = std::stoi(o.str("num-intervals"));
    const std::string e = o.str("logical-error");
    const int R = std::stoi(o.str("disorder-samples"));
    const int boundary = std::stoi(o.str("boundary"));
    const int task = std::stoi(o.str("task_id"));
    if (boundary != 0 && boundary != 1) {
      std::fprintf(stderr, "Unsupported boundary condition %d\n", boundary);
      return EXIT_FAILURE;
    }
    if (e.size() != 1 || R <= 0) {
      std::fprintf(stderr, "invalid logical error type or sample count\n");
      return EXIT_FAILURE;
    }
    std::vector<wlg_problem> probs(static_cast<size_t>(R));
    for (int k = 0; k < R; ++k) {
      wlg_problem& q = probs[k];
      q = wlg_problem{};
      q.X = X;
      q.Y = Y;
      q.boundary = boundary;
      q.prob = prob;
      q.error_class = e[0];
      q.seed = seed;
      q.sample = k;
      q.pre_walkers = walkers;
      q.pre_intervals = bins;
      q.pre_iterations = n_iter;
      // main-run fields are not used by the pre-run; valid placeholders
      q.intervals = 1;
      q.walkers_per_interval = 1;
      q.overlap = 0.25f;
      q.alpha = 0.8;
      q.beta = 1e-3;
      q.iterations = 1;
      q.exchange_every = 1;
    }
    const int N = X * Y;
    std::vector<unsigned char> seen(static_cast<size_t>(R) * (4 * N + 1));
    std::vector<signed char> J(static_cast<size_t>(R) * 2 * N), lat(static_cast<size_t>(R) * bins * N);
    std::vector<int> found(static_cast<size_t>(R) * bins), energy(found.size());
    wlg_context* ctx = nullptr;
    wlg_status st = wlg_context_create(0, 0, &ctx);
    if (st == WLG_OK)
      st = wlg_prerun(ctx, probs.data(), R, seen.data(), J.data(), found.data(), energy.data(), lat.data());
    if (st != WLG_OK) {
      std::fprintf(stderr, "pre-run failed: %s %s\n", wlg_status_string(st), ctx ? wlg_context_last_error(ctx) : "");
      if (ctx) wlg_context_destroy(ctx);
      return EXIT_FAILURE;
    }
    wlg_context_destroy(ctx);
    if (o.has("skip-output")) return EXIT_SUCCESS;

    const std::string dir = wlg::cli::run_path("init", task, seed, boundary, prob, X, Y, e[0]);
    std::filesystem::create_directories(dir);
    const std::string path = dir + "/prerun_results.h5";
    if (std::filesystem::exists(path)) {
      std::fprintf(stderr, "Prerun result file %s already exists, aborting.\n", path.c_str());
      return EXIT_FAILURE;
    }
    wlg::h5::Group root;
    for (int k = 0; k < R; ++k) {
      const std::string key = std::to_string(k);
      std::vector<uint64_t> h(seen.begin() + static_cast<long>(k) * (4 * N + 1),
                              seen.begin() + static_cast<long>(k + 1) * (4 * N + 1));
      root.group("Histogram").group(key).datasets["Histogram"] = wlg::h5::make_u64(h);
      std::vector<int8_t> jk(J.begin() + static_cast<long>(k) * 2 * N, J.begin() + static_cast<long>(k + 1) * 2 * N);
      root.group("Interaction").group(key).datasets["Interaction"] = wlg::h5::make_i8(jk);
      wlg::h5::Group& lg = root.group("Lattice").group(key);
      for (int b = 0; b < bins; ++b) {
        if (!found[static_cast<size_t>(k) * bins + b]) continue;
        const std::string ename = std::to_string(energy[static_cast<size_t>(k) * bins + b]);
        if (lg.groups.count(ename)) {  // the reference's group creation fails on a duplicate name
          std::fprintf(stderr, "Failed to create h5 interval group for lattice write\n");
          return EXIT_FAILURE;
        }
        const auto at = lat.begin() + (static_cast<long>(k) * bins + b) * N;
        lg.group(ename).datasets["Lattice"] = wlg::h5::make_i8(std::vector<int8_t>(at, at + N));
      }
    }
    const std::string werr = wlg::h5::write_file(path, root);
    if (!werr.empty()) {
      std::fprintf(stderr, "Failed to write %s: %s\n", path.c_str(), werr.c_str());
      return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
  } catch (const std::exception& ex) {
    std::fprintf(stderr, "%s\n", ex.what());
    return EXIT_FAILURE;
  }
}
