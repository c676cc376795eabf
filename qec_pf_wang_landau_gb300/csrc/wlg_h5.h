// Minimal HDF5 files for the reference's result layouts, without libhdf5.
//
// The reference writes prerun_results.h5 (file_io.cpp:23-192: groups
// /Histogram/<k>, /Interaction/<k>, /Lattice/<k>/<E>, each holding one 1-D
// dataset) and mainrun_results.h5 (utils.cpp:137-236: /<k>/<seed>/<time>/log_g,
// a 1-D dataset of compound {Key: int32, Value: float64} with a 256-byte
// string attribute CodeVersion).  It does not depend on libhdf5: this module
// writes and reads exactly those shapes itself, following the
// public HDF5 File Format Specification (version 3.0): a version-2
// superblock, version-2 object headers, groups with compact link storage
// (Link Info, Group Info and Link messages), contiguous dataset storage, and
// Jenkins' lookup3 checksums.  The reader accepts those files and the
// structure libhdf5 writes by default for the same layouts (superblock 0,
// version-1 object headers with continuation blocks, symbol-table groups
// through version-1 B-trees and a local heap, version-1 dataspaces and
// attributes, compact or contiguous storage); it is not a general HDF5
// reader (no chunked storage, no dense link storage, no other types).
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace wlg::h5 {

// lookup3 hashlittle (Bob Jenkins, public domain) as the format's checksum.
uint32_t lookup3(const uint8_t* data, size_t n, uint32_t init = 0);

enum class Type { u8, i8, i32, u64, f64, key_value };  // key_value: compound {Key int32, Value float64}

struct Dataset {
  Type type = Type::u8;
  uint64_t count = 0;              // elements (1-D)
  std::vector<uint8_t> bytes;      // little-endian elements (key_value: 16 bytes each, Key at 0, Value at 8)
  std::map<std::string, std::string> string_attrs;  // fixed 256-byte null-terminated strings
};

struct Group {
  std::map<std::string, std::unique_ptr<Group>> groups;
  std::map<std::string, Dataset> datasets;
  Group& group(const std::string& name);  // child group, created if missing
};

// Whole-file write and read of a group tree.  Return "" or an error text.
std::string write_file(const std::string& path, const Group& root);
std::string read_file(const std::string& path, Group& root);

// Helpers for typed datasets.
Dataset make_u64(const std::vector<uint64_t>& v);
Dataset make_i8(const std::vector<int8_t>& v);
Dataset make_key_value(const std::vector<std::pair<int32_t, double>>& v);

}  // namespace wlg::h5
