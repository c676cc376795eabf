// Test-only: writes a small file in both result layouts with the engine's
// HDF5 writer (the prerun/mainrun programs need a GPU to produce data).
#include <cstdio>
#include <string>
#include <vector>

#include "../../qec_pf_wang_landau_gb300/csrc/wlg_h5.h"

int main(int argc, char** argv)
{
  if (argc != 2) return 2;
  wlg::h5::Group root;
  root.group("Histogram").group("0").datasets["Histogram"] = wlg::h5::make_u64({0, 1, 1, 0, 1});
  root.group("Histogram").group("1").datasets["Histogram"] = wlg::h5::make_u64({1, 0, 0, 0, 1});
  root.group("Interaction").group("0").datasets["Interaction"] = wlg::h5::make_i8({1, -1, 1, 1, -1, 1, 1, 1});
  root.group("Lattice").group("0").group("-8").datasets["Lattice"] = wlg::h5::make_i8({1, 1, -1, 1});
  root.group("Lattice").group("0").group("12").datasets["Lattice"] = wlg::h5::make_i8({-1, 1, -1, 1});
  wlg::h5::Dataset d = wlg::h5::make_key_value({{-8, 0.5}, {-4, 1.25}, {0, 2.75}});
  d.string_attrs["CodeVersion"] = "wlg test 1";
  root.group("0").group("12345").group("Thu_Dec__3_18:00:00_2026").datasets["log_g"] = d;
  const std::string err = wlg::h5::write_file(argv[1], root);
  if (!err.empty()) {
    std::fprintf(stderr, "%s\n", err.c_str());
    return 1;
  }
  return 0;
}
