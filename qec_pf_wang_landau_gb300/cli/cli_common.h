// Shared pieces of the prerun/mainrun command-line programs: option parsing
// in the style the reference's Boost.Program_options setup accepts
// (program_options.cpp:37-71, :110-157: "--name value", "--name=value",
// "-c value", "-cvalue"), the output paths (utils.cpp:88-128) and the
// timestamp group name (utils.cpp:238-250).
#pragma once

#include <chrono>
#include <cstdio>
#include <ctime>
#include <iomanip>
#include <map>
#include <optional>
#include <random>
#include <sstream>
#include <string>
#include <vector>

namespace wlg::cli {

struct Opt {
  std::string name;        // long name
  char shorthand = 0;      // 0: long only
  bool value = true;       // takes a value
  bool required = false;
  std::string def;         // default value ("" = none)
  std::string help;
};

class Options {
 public:
  explicit Options(std::vector<Opt> opts) : opts_(std::move(opts)) {}

  // "" on success, else the error text.
  std::string parse(int argc, char** argv)
  {
    for (int i = 1; i < argc; ++i) {
      std::string a = argv[i];
      const Opt* o = nullptr;
      std::optional<std::string> val;
      if (a.rfind("--", 0) == 0) {
        std::string name = a.substr(2);
        const size_t eq = name.find('=');
        if (eq != std::string::npos) {
          val = name.substr(eq + 1);
          name = name.substr(0, eq);
        }
        for (const Opt& c : opts_)
          if (c.name == name) o = &c;
        if (o == nullptr) return "unrecognised option '--" + name + "'";
      } else if (a.size() >= 2 && a[0] == '-') {
        for (const Opt& c : opts_)
          if (c.shorthand != 0 && c.shorthand == a[1]) o = &c;
        if (o == nullptr) return "unrecognised option '" + a + "'";
        if (a.size() > 2) val = a.substr(2);
      } else {
        return "unexpected argument '" + a + "'";
      }
      if (o->value && !val) {
        if (i + 1 >= argc) return "the required argument for option '--" + o->name + "' is missing";
        val = argv[++i];
      }
      if (!o->value && val) return "option '--" + o->name + "' does not take a value";
      values_[o->name] = val.value_or("");
    }
    return "";
  }

  bool has(const std::string& name) const { return values_.count(name) > 0; }

  // the first required option that is missing, or ""
  std::string missing() const
  {
    for (const Opt& o : opts_)
      if (o.required && !has(o.name)) return o.name;
    return "";
  }

  std::string str(const std::string& name) const
  {
    auto it = values_.find(name);
    if (it != values_.end()) return it->second;
    for (const Opt& o : opts_)
      if (o.name == name) return o.def;
    return "";
  }

  void usage(const char* prog, const char* title) const
  {
    std::printf("%s\n\n%s:\n", prog, title);
    for (const Opt& o : opts_) {
      std::string flag = o.shorthand ? std::string("  -") + o.shorthand + " [ --" + o.name + " ]"
                                     : std::string("  --") + o.name;
      if (o.value) flag += " arg";
      if (!o.def.empty()) flag += " (=" + o.def + ")";
      std::printf("%-44s %s\n", flag.c_str(), o.help.c_str());
    }
  }

 private:
  std::vector<Opt> opts_;
  std::map<std::string, std::string> values_;
};

inline int seed_from_os()
{
  std::random_device dev;
  return static_cast<int>(dev());
}

inline std::string boundary_name(int b) { return b == 0 ? "periodic" : "open"; }

// <root>/task_id_<d>/seed_<s>/<boundary>/prob_<p:.6f>/X_<x>_Y_<y>/error_class_<e>
inline std::string run_path(const char* root, int task_id, int seed, int boundary, float prob, int X, int Y, char e)
{
  std::ostringstream s;
  s << root << "/task_id_" << task_id << "/seed_" << seed << "/" << boundary_name(boundary) << "/prob_" << std::fixed
    << std::setprecision(6) << prob << "/X_" << X << "_Y_" << Y << "/error_class_" << e;
  return s.str();
}

// ctime() of now without the newline, spaces replaced by '_'
inline std::string timestamp_group_name()
{
  const std::time_t t = std::chrono::system_clock::to_time_t(std::chrono::system_clock::now());
  char buf[64] = {};
  std::string s = ctime_r(&t, buf) != nullptr ? std::string(buf) : std::string("unknown time");
  while (!s.empty() && s.back() == '\n') s.pop_back();
  for (char& c : s)
    if (c == ' ') c = '_';
  return s;
}

}  // namespace wlg::cli
