// wlg_mainrun: the reference's `mainrun` program (mainrun.cu:36-421) on the
// engine's C ABI.  Same flags (program_options.cpp:110-157), reads the
// pre-run file at the path prerun writes (utils.cpp:102-114) and writes
// mainrun_results.h5 under results/... (utils.cpp:116-128, :137-236): for each
// converged disorder sample k the group /<k>/<seed>/<ctime>/ holds log_g, a
// 1-D compound {Key: int32, Value: float64} of the stitched, normalised
// (E, log g) pairs, with a 256-byte string attribute CodeVersion.  An
// existing result file is extended (it must have been written by this
// program).  The reference's exchange counter never advances
// (mainrun.cu:241,346), so by default exchange happens only with -c 1;
// --exchange-mode 1 exchanges every c iterations; --stitching 1 skips
// energies without a successor where the reference reads past a map's end.  Exit status: failure when
// a walker finds an energy the pre-run did not (nothing written, as the
// reference), or on errors.

#include <algorithm>
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
  wlg::cli::Options o({
    {"help", 0, false, false, "", "Help"},
    {"X", 'x', true, true, "", "X"},
    {"Y", 'y', true, true, "", "Y"},
    {"num_iterations", 'n', true, true, "", "Number of iterations"},
    {"prob_interactions", 'p', true, true, "", "Interaction probabilities"},
    {"alpha", 'a', true, true, "", "Alpha"},
    {"beta", 'b', true, true, "", "Beta"},
    {"num_intervals", 'i', true, true, "", "Number of intervals"},
    {"walker_per_interval", 'w', true, true, "", "Number of walkers per interval"},
    {"overlap_decimal", 'o', true, true, "", "Overlap of neighbouring intervals"},
    {"seed", 's', true, false, "", "Random seed (Run)"},
    {"logical_error", 'e', true, false, "I", "Type of logical error"},
    {"repetitions_interactions", 'r', true, true, "", "Repetitions interactions"},
    {"replica_exchange_offsets", 'c', true, true, "", "Outer iterations between replica exchanges"},
    {"boundary", 0, true, false, "0", "Boundary condition"},
    {"task_id", 'd', true, true, "", "Task ID"},
    {"time_limit", 'f', true, true, "", "Time Limit"},
    {"exchange-mode", 0, true, false, "0", "0: as the reference (exchange only with -c 1); 1: every c iterations"},
    {"stitching", 0, true, false, "0", "0: the reference's output bins; 1: energies without a successor skipped"},
    {"version", 'v', false, false, "", "Show version"},
  });
  try {
    const std::string err = o.parse(argc, argv);
    if (!err.empty()) {
      std::fprintf(stderr, "%s\n", err.c_str());
      return EXIT_FAILURE;
    }
    if (o.has("help")) {
      o.usage(argv[0], "WL main usage");
      return EXIT_SUCCESS;
    }
    if (o.has("version")) {
      std::printf("WL mainrun version: %s\n", wlg_version());
      return EXIT_SUCCESS;
    }
    if (const std::string m = o.missing(); !m.empty()) {
      std::fprintf(stderr, "the option '--%s' is required but missing\n", m.c_str());
      o.usage(argv[0], "WL main usage");
      return EXIT_SUCCESS;
    }
    const int X = std::stoi(o.str("X")), Y = std::stoi(o.str("Y")), N = X * Y;
    const int n_iter = std::stoi(o.str("num_iterations"));
    const float prob = std::stof(o.str("prob_interactions"));
    const double alpha = std::stod(o.str("alpha")), beta = std::stod(o.str("beta"));
    const int I = std::stoi(o.str("num_intervals")), W = std::stoi(o.str("walker_per_interval"));
    const float overlap = std::stof(o.str("overlap_decimal"));
    const int seed = o.has("seed") ? std::stoi(o.str("seed")) : wlg::cli::seed_from_os();
    const std::string e = o.str("logical_error");
    const int R = std::stoi(o.str("repetitions_interactions"));
    const int c = std::stoi(o.str("replica_exchange_offsets"));
    const int boundary = std::stoi(o.str("boundary"));
    const int task = std::stoi(o.str("task_id"));
    const int time_limit = std::stoi(o.str("time_limit"));
    const int xmode = std::stoi(o.str("exchange-mode"));
    const int stitching = std::stoi(o.str("stitching"));
    if (boundary != 0 && boundary != 1) {
      std::fprintf(stderr, "Unsupported boundary condition %d\n", boundary);
      return EXIT_FAILURE;
    }
    if (e.size() != 1 || R <= 0 || (xmode != 0 && xmode != 1)) {
      std::fprintf(stderr, "invalid logical error type, sample count or exchange mode\n");
      return EXIT_FAILURE;
    }

    // ---- pre-run results (file_io.cpp:217-556)
    const std::string init = wlg::cli::run_path("init", task, seed, boundary, prob, X, Y, e[0]) + "/prerun_results.h5";
    wlg::h5::Group pre;
    if (const std::string rerr = wlg::h5::read_file(init, pre); !rerr.empty()) {
      std::fprintf(stderr, "Error: Could not open HDF5 file:%s (%s)\n", init.c_str(), rerr.c_str());
      return EXIT_FAILURE;
    }
    std::vector<unsigned char> seen;
    std::vector<signed char> J, lat;
    std::vector<int> found, energy;
    std::vector<wlg_problem> probs(static_cast<size_t>(R));
    for (int k = 0; k < R; ++k) {
      const std::string key = std::to_string(k);
      auto need = [&](const char* top, const char* name) -> const wlg::h5::Dataset& {
        auto g = pre.groups.find(top);
        if (g == pre.groups.end() || !g->second->groups.count(key) || !g->second->groups.at(key)->datasets.count(name))
          throw std::runtime_error(std::string("missing /") + top + "/" + key + "/" + name);
        return g->second->groups.at(key)->datasets.at(name);
      };
      const wlg::h5::Dataset& h = need("Histogram", "Histogram");
      if (h.count != static_cast<uint64_t>(4 * N + 1) || h.type != wlg::h5::Type::u64)
        throw std::runtime_error("Histogram length does not coincide with length of histogram written to file");
      for (uint64_t i = 0; i < h.count; ++i) seen.push_back(h.bytes[8 * i] != 0 ? 1 : 0);
      const wlg::h5::Dataset& jd = need("Interaction", "Interaction");
      if (jd.count != static_cast<uint64_t>(2 * N) || jd.type != wlg::h5::Type::i8)
        throw std::runtime_error("Interaction length does not coincide with length of interaction written to file");
      auto pm1 = [](const std::vector<uint8_t>& v) {
        return std::all_of(v.begin(), v.end(), [](uint8_t x) { return x == 0x01 || x == 0xFF; });
      };
      if (!pm1(jd.bytes)) throw std::runtime_error("Interaction values other than +-1");
      J.insert(J.end(), jd.bytes.begin(), jd.bytes.end());
      int stored = 0;
      auto lg = pre.groups.find("Lattice");
      if (lg != pre.groups.end() && lg->second->groups.count(key)) {
        for (const auto& [ename, eg] : lg->second->groups.at(key)->groups) {
          auto ds = eg->datasets.find("Lattice");
          if (ds == eg->datasets.end() || ds->second.count != static_cast<uint64_t>(N) ||
              ds->second.type != wlg::h5::Type::i8)
            continue;
          if (!pm1(ds->second.bytes)) throw std::runtime_error("Lattice values other than +-1");
          found.push_back(1);
          energy.push_back(std::stoi(ename));
          lat.insert(lat.end(), ds->second.bytes.begin(), ds->second.bytes.end());
          ++stored;
        }
      }
      if (stored == 0) {  // no start lattice at all: the hand-off reports it
        found.push_back(0);
        energy.push_back(0);
        lat.insert(lat.end(), static_cast<size_t>(N), 0);
        stored = 1;
      }
      wlg_problem& q = probs[k];
      q = wlg_problem{};
      q.X = X;
      q.Y = Y;
      q.boundary = boundary;
      q.prob = prob;
      q.error_class = e[0];
      q.seed = seed;
      q.sample = k;
      q.pre_walkers = 1;  // the pre-run is not run again
      q.pre_intervals = stored;
      q.pre_iterations = 0;
      q.intervals = I;
      q.walkers_per_interval = W;
      q.overlap = overlap;
      q.alpha = alpha;
      q.beta = beta;
      q.iterations = n_iter;
      q.exchange_every = c;
      q.exchange_mode = xmode;
      q.global_parity = 1;  // the reference's exchange parity (global block index)
    }

    // ---- main run
    std::vector<wlg_result> res(static_cast<size_t>(R));
    const long long cap = static_cast<long long>(R) * (4 * N + 1);
    std::vector<int> E(static_cast<size_t>(cap));
    std::vector<double> G(static_cast<size_t>(cap));
    wlg_context* ctx = nullptr;
    wlg_status st = wlg_context_create(0, 0, &ctx);
    if (st == WLG_OK) st = wlg_context_set_stitching(ctx, stitching);
    if (st == WLG_OK)
      st = wlg_mainrun(ctx, probs.data(), R, seen.data(), J.data(), found.data(), energy.data(), lat.data(),
                       static_cast<double>(std::max(time_limit, 0)) + 1e-9,  // -f 0: stop at the first check
                       res.data(), E.data(), G.data(), cap);
    if (st != WLG_OK) {
      std::fprintf(stderr, "main run failed: %s %s\n", wlg_status_string(st), ctx ? wlg_context_last_error(ctx) : "");
      if (ctx) wlg_context_destroy(ctx);
      return EXIT_FAILURE;
    }
    wlg_context_destroy(ctx);
    for (int k = 0; k < R; ++k)
      if (res[k].status == WLG_ERR_NEW_ENERGY) {
        std::fprintf(stderr, "Error: Found new energy %d in sample %d\n", res[k].new_energy, k);
        return EXIT_FAILURE;
      }
    for (int k = 0; k < R; ++k)
      if (res[k].status == WLG_ERR_TIMEOUT) std::fprintf(stderr, "Time limit reached for sample %d\n", k);

    // ---- results (utils.cpp:137-236)
    int converged = 0;
    for (int k = 0; k < R; ++k) converged += res[k].status == WLG_OK ? 1 : 0;
    const std::string dir = wlg::cli::run_path("results", task, seed, boundary, prob, X, Y, e[0]);
    std::filesystem::create_directories(dir);
    const std::string path = dir + "/mainrun_results.h5";
    if (converged == 0) return EXIT_SUCCESS;  // nothing to write (no file is created)
    wlg::h5::Group root;
    if (std::filesystem::exists(path)) {
      if (const std::string rerr = wlg::h5::read_file(path, root); !rerr.empty()) {
        std::fprintf(stderr, "Error: cannot extend %s (%s)\n", path.c_str(), rerr.c_str());
        return EXIT_FAILURE;
      }
    }
    const std::string stamp = wlg::cli::timestamp_group_name();
    for (int k = 0; k < R; ++k) {
      if (res[k].status != WLG_OK) continue;
      std::vector<std::pair<int32_t, double>> kv;
      for (int i = 0; i < res[k].n_energies; ++i)
        kv.emplace_back(E[res[k].offset + i], G[res[k].offset + i]);
      wlg::h5::Dataset d = wlg::h5::make_key_value(kv);
      d.string_attrs["CodeVersion"] = wlg_version();
      root.group(std::to_string(k)).group(std::to_string(seed)).group(stamp).datasets["log_g"] = std::move(d);
    }
    if (const std::string werr = wlg::h5::write_file(path, root); !werr.empty()) {
      std::fprintf(stderr, "Failed to write %s: %s\n", path.c_str(), werr.c_str());
      return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
  } catch (const std::exception& ex) {
    std::fprintf(stderr, "%s\n", ex.what());
    return EXIT_FAILURE;
  }
}
