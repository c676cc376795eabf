// wlg_decode: the decoding front-end on the serving API (no counterpart in
// the reference, whose programs simulate drawn disorder; the class
// probabilities follow the paper behind it, README.md:196-200).
//
// Reads syndromes, one per line (plaquette flags as '0'/'1' characters,
// row-major; X*Y plaquettes for periodic lattices, (X-1)*(Y-1) for open
// ones; blank lines and lines starting with '#' are skipped), builds for each
// a bond pattern with exactly those frustrated plaquettes
// (wlg_couplings_from_syndrome), submits all of them to a continuous-batching
// server (wlg_server_submit_couplings: the pattern's four error classes
// i, v, h, c) and prints one line per syndrome, in input order:
//
//   <index> <status> <log p_i> <log p_v> <log p_h> <log p_c> <most likely class>
//
// log p_c is the Nishimori-temperature log-probability that the error is the
// pattern times class c's logical chain.  The Wang-Landau flags are the
// reference's (prerun.cu / mainrun.cu names, program_options.cpp:37-157).
// Exit status: failure on unreadable input, an invalid syndrome or a device
// error; requests that fail individually report their status on their line.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "../../include/wlg.h"
#include "cli_common.h"

int main(int argc, char** argv)
{
  wlg::cli::Options o({
    {"help", 0, false, false, "", "Help"},
    {"X", 'x', true, true, "", "X"},
    {"Y", 'y', true, true, "", "Y"},
    {"prob_interactions", 'p', true, true, "", "Bond flip probability (sets the Nishimori temperature)"},
    {"boundary", 0, true, false, "0", "Boundary condition (0 periodic, 1 open)"},
    {"input", 'f', true, false, "-", "Syndrome file ('-': standard input)"},
    {"seed", 's', true, false, "1", "Random seed of the walks"},
    {"prerun_walkers", 0, true, false, "128", "Pre-run walkers"},
    {"prerun_intervals", 0, true, false, "32", "Pre-run intervals"},
    {"prerun_iterations", 0, true, false, "", "Pre-run iterations (default 100*X*Y)"},
    {"num_iterations", 'n', true, false, "1000", "WL steps per walker between flatness checks"},
    {"alpha", 'a', true, false, "0.8", "Flatness"},
    {"beta", 'b', true, false, "1e-6", "Final ln f"},
    {"num_intervals", 'i', true, false, "", "Windows (default X*Y/16, at least 4)"},
    {"walker_per_interval", 'w', true, false, "4", "Walkers per window"},
    {"overlap_decimal", 'o', true, false, "0.25", "Window overlap"},
    {"replica_exchange_offsets", 'c', true, false, "10", "Outer iterations between replica exchanges"},
    {"memory", 0, true, false, "0", "Device memory budget of the server in bytes (0: 1 GiB)"},
    {"max_outer", 0, true, false, "0", "Cap on outer iterations per class (0: none); capped requests report status 7"},
    {"version", 'v', false, false, "", "Show version"},
  });
  try {
    const std::string err = o.parse(argc, argv);
    if (!err.empty()) {
      std::fprintf(stderr, "%s\n", err.c_str());
      return EXIT_FAILURE;
    }
    if (o.has("help")) {
      o.usage(argv[0], "WL decode usage");
      return EXIT_SUCCESS;
    }
    if (o.has("version")) {
      std::printf("WL decode version: %s\n", wlg_version());
      return EXIT_SUCCESS;
    }
    if (const std::string m = o.missing(); !m.empty()) {
      std::fprintf(stderr, "the option '--%s' is required but missing\n", m.c_str());
      return EXIT_FAILURE;
    }
    const int X = std::stoi(o.str("X")), Y = std::stoi(o.str("Y")), N = X * Y;
    const int boundary = std::stoi(o.str("boundary"));
    const float prob = std::stof(o.str("prob_interactions"));
    const int plaquettes = boundary == 0 ? X * Y : (X - 1) * (Y - 1);
    if ((boundary != 0 && boundary != 1) || prob <= 0.0f || prob >= 1.0f || X < 2 || Y < 2) {
      std::fprintf(stderr, "invalid lattice, boundary or probability\n");
      return EXIT_FAILURE;
    }
    wlg_problem q{};
    q.X = X;
    q.Y = Y;
    q.boundary = boundary;
    q.prob = prob;
    q.error_class = 'i';
    q.seed = std::stoi(o.str("seed"));
    q.pre_walkers = std::stoi(o.str("prerun_walkers"));
    q.pre_intervals = std::stoi(o.str("prerun_intervals"));
    q.pre_iterations = o.str("prerun_iterations").empty() ? 100 * N : std::stoi(o.str("prerun_iterations"));
    q.intervals = o.str("num_intervals").empty() ? std::max(4, N / 16) : std::stoi(o.str("num_intervals"));
    q.walkers_per_interval = std::stoi(o.str("walker_per_interval"));
    q.overlap = std::stof(o.str("overlap_decimal"));
    q.alpha = std::stod(o.str("alpha"));
    q.beta = std::stod(o.str("beta"));
    q.iterations = std::stoi(o.str("num_iterations"));
    q.exchange_every = std::stoi(o.str("replica_exchange_offsets"));
    q.exchange_mode = 1;
    q.global_parity = 0;
    q.max_outer = std::stoll(o.str("max_outer"));

    // ---- syndromes -> bond patterns
    std::ifstream file;
    const std::string in = o.str("input");
    if (in != "-") {
      file.open(in);
      if (!file) {
        std::fprintf(stderr, "cannot read %s\n", in.c_str());
        return EXIT_FAILURE;
      }
    }
    std::istream& src = in == "-" ? std::cin : file;
    std::vector<wlg_problem> reqs;
    std::vector<signed char> J;
    std::string line;
    int lineno = 0;
    while (std::getline(src, line)) {
      ++lineno;
      std::string bits;
      for (char ch : line)
        if (ch != ' ' && ch != '\t' && ch != '\r') bits += ch;
      if (bits.empty() || bits[0] == '#') continue;
      if (static_cast<int>(bits.size()) != plaquettes || bits.find_first_not_of("01") != std::string::npos) {
        std::fprintf(stderr, "line %d: expected %d characters 0/1\n", lineno, plaquettes);
        return EXIT_FAILURE;
      }
      std::vector<unsigned char> s(bits.size());
      for (size_t k = 0; k < bits.size(); ++k) s[k] = bits[k] == '1' ? 1 : 0;
      std::vector<signed char> pattern(static_cast<size_t>(2 * N));
      if (wlg_couplings_from_syndrome(X, Y, boundary, s.data(), pattern.data()) != WLG_OK) {
        std::fprintf(stderr, "line %d: no bond pattern has this syndrome (a torus needs an even number)\n", lineno);
        return EXIT_FAILURE;
      }
      wlg_problem r = q;
      r.sample = static_cast<int>(reqs.size());
      reqs.push_back(r);
      J.insert(J.end(), pattern.begin(), pattern.end());
    }
    if (reqs.empty()) return EXIT_SUCCESS;

    // ---- serve
    wlg_server_config cfg{};
    cfg.mem_budget_bytes = static_cast<size_t>(std::stoull(o.str("memory")));
    wlg_server* srv = nullptr;
    if (wlg_server_create(0, &cfg, &srv) != WLG_OK) {
      std::fprintf(stderr, "cannot start the server on device 0\n");
      return EXIT_FAILURE;
    }
    const int n = static_cast<int>(reqs.size());
    std::vector<unsigned long long> ids(static_cast<size_t>(n));
    wlg_status st = wlg_server_submit_couplings(srv, reqs.data(), n, J.data(), ids.data());
    std::map<unsigned long long, wlg_decoded> done;
    std::vector<wlg_decoded> buf(256);
    while (st == WLG_OK && static_cast<int>(done.size()) < n) {
      int k = 0;
      st = wlg_server_poll(srv, buf.data(), static_cast<int>(buf.size()), &k, 1000);
      for (int i = 0; i < k; ++i) done[buf[i].id] = buf[i];
    }
    const std::string why = wlg_server_last_error(srv);
    wlg_server_destroy(srv);
    if (st != WLG_OK) {
      std::fprintf(stderr, "serving failed: %s %s\n", wlg_status_string(st), why.c_str());
      return EXIT_FAILURE;
    }
    static const char kClass[4] = {'i', 'v', 'h', 'c'};
    for (int k = 0; k < n; ++k) {
      const wlg_decoded& d = done[ids[k]];
      int best = 0;
      for (int c = 1; c < 4; ++c)
        if (d.log_probs[c] > d.log_probs[best]) best = c;
      std::printf("%d %d %.10g %.10g %.10g %.10g %c\n", k, d.status, d.log_probs[0], d.log_probs[1], d.log_probs[2],
                  d.log_probs[3], d.status == WLG_OK ? kClass[best] : '-');
    }
    return EXIT_SUCCESS;
  } catch (const std::exception& ex) {
    std::fprintf(stderr, "%s\n", ex.what());
    return EXIT_FAILURE;
  }
}
