// scamp_main.cpp -- the reference's command-line program (src/main.cpp) as
// a native binary over the C++ do_SCAMP shim and scamp_utils.h: the same
// gflags-style flags, checks, messages and output files as
// `python -m scamp_gb300`.  Exit status 0 on success, 1 on any error (the
// message is printed to standard output, as the reference does).
#include <cctype>
#include <cstdlib>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "scamp/SCAMP.h"
#include "scamp/scamp_utils.h"

namespace {

enum Kind { K_INT, K_FLOAT, K_STR, K_BOOL };

struct Flag {
  Kind kind;
  std::string value;
};

struct UsageError {
  std::string msg;
};

std::map<std::string, Flag> default_flags() {
  return {
      {"window", {K_INT, "-1"}},
      {"max_tile_size", {K_INT, "131072"}},
      {"threshold", {K_FLOAT, "0"}},
      {"profile_type", {K_STR, "1NN_INDEX"}},
      {"ultra_precision", {K_BOOL, "false"}},
      {"double_precision", {K_BOOL, "false"}},
      {"mixed_precision", {K_BOOL, "false"}},
      {"single_precision", {K_BOOL, "false"}},
      {"keep_rows", {K_BOOL, "false"}},
      {"aligned", {K_BOOL, "false"}},
      {"global_row", {K_INT, "-1"}},
      {"global_col", {K_INT, "-1"}},
      {"input_a_file_name", {K_STR, ""}},
      {"input_b_file_name", {K_STR, ""}},
      {"output_a_file_name", {K_STR, "mp_columns_out"}},
      {"output_a_index_file_name", {K_STR, "mp_columns_out_index"}},
      {"output_b_file_name", {K_STR, "mp_rows_out"}},
      {"output_b_index_file_name", {K_STR, "mp_rows_out_index"}},
      {"output_pearson", {K_BOOL, "false"}},
      {"gpus", {K_STR, ""}},
      {"print_debug_info", {K_BOOL, "false"}},
      {"no_gpu", {K_BOOL, "false"}},
      {"max_matches_per_column", {K_INT, "5"}},
      {"reduced_height", {K_INT, "50"}},
      {"reduced_width", {K_INT, "50"}},
      // accepted, no effect here
      {"num_cpu_workers", {K_INT, "0"}},
      {"distributed_tile_size", {K_INT, "4000000"}},
      {"hostname_port", {K_STR, "localhost:30078"}},
  };
}

std::string trim(const std::string& s) {
  size_t b = 0, e = s.size();
  while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
  while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
  return s.substr(b, e - b);
}

bool parse_int(const std::string& text, long long* out) {
  const std::string s = trim(text);
  if (s.empty()) return false;
  size_t i = (s[0] == '+' || s[0] == '-') ? 1 : 0;
  if (i == s.size()) return false;
  for (size_t j = i; j < s.size(); ++j)
    if (!std::isdigit(static_cast<unsigned char>(s[j]))) return false;
  try {
    *out = std::stoll(s);
  } catch (...) {
    return false;
  }
  return true;
}

bool parse_float(const std::string& text, double* out) {
  const std::string s = trim(text);
  if (s.empty()) return false;
  size_t used = 0;
  try {
    *out = std::stod(s, &used);
  } catch (...) {
    return false;
  }
  return used == s.size();
}

std::string lower(std::string s) {
  for (char& c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
  return s;
}

// --name=value, --name value, --bool, --bool=value, --nobool.
std::map<std::string, Flag> parse_flags(int argc, char** argv) {
  std::map<std::string, Flag> fl = default_flags();
  for (int i = 1; i < argc; ++i) {
    std::string tok = argv[i];
    if (tok.empty() || tok[0] != '-') throw UsageError{"Error: unexpected argument " + tok};
    tok = tok.substr(tok.find_first_not_of('-') == std::string::npos ? tok.size()
                                                                      : tok.find_first_not_of('-'));
    const size_t eq = tok.find('=');
    const std::string name = tok.substr(0, eq);
    auto it = fl.find(name);
    if (it == fl.end() && name.compare(0, 2, "no") == 0) {
      auto b = fl.find(name.substr(2));
      if (b != fl.end() && b->second.kind == K_BOOL) {
        b->second.value = "false";
        continue;
      }
    }
    if (it == fl.end()) throw UsageError{"ERROR: unknown command line flag '" + name + "'"};
    Flag& f = it->second;
    if (f.kind == K_BOOL) {
      if (eq == std::string::npos) {
        f.value = "true";
      } else {
        const std::string v = lower(tok.substr(eq + 1));
        f.value = (v == "false" || v == "0" || v == "no") ? "false" : "true";
      }
      continue;
    }
    std::string value;
    if (eq == std::string::npos) {
      if (i + 1 >= argc) throw UsageError{"ERROR: flag '--" + name + "' is missing its argument"};
      value = argv[++i];
    } else {
      value = tok.substr(eq + 1);
    }
    long long iv;
    double dv;
    if ((f.kind == K_INT && !parse_int(value, &iv)) || (f.kind == K_FLOAT && !parse_float(value, &dv)))
      throw UsageError{"ERROR: illegal value '" + value + "' specified for " +
                       (f.kind == K_INT ? "int" : "float") + " flag '" + name + "'"};
    f.value = value;
  }
  return fl;
}

long long as_int(const std::map<std::string, Flag>& fl, const char* name) {
  long long v = 0;
  parse_int(fl.at(name).value, &v);
  return v;
}

bool as_bool(const std::map<std::string, Flag>& fl, const char* name) {
  return fl.at(name).value == "true";
}

int run(int argc, char** argv) {
  const std::map<std::string, Flag> fl = parse_flags(argc, argv);
  const char* precisions[] = {"ultra", "double", "mixed", "single"};
  int n_prec = 0;
  bool prec[4];
  for (int p = 0; p < 4; ++p) {
    prec[p] = as_bool(fl, (std::string(precisions[p]) + "_precision").c_str());
    n_prec += prec[p] ? 1 : 0;
  }
  if (n_prec == 0) prec[1] = true, n_prec = 1;
  if (n_prec != 1) throw UsageError{"Error: only one precision flag can be enabled at a time"};
  const long long window = as_int(fl, "window");
  const long long max_tile = as_int(fl, "max_tile_size");
  if (window < 3)
    throw UsageError{"Error: Subsequence length must be at least 3, please use "
                     "--window=<window_size> to specify your subsequence length."};
  if (max_tile < 1024) throw UsageError{"Error: max tile size must be at least 1024"};
  if (max_tile / 2 < window)
    throw UsageError{"Error: Tile length and width must be at least 2x larger than the "
                     "window size. Please set a larger --max_tile_size=<max_tile_size>"};
  const std::string in_a = fl.at("input_a_file_name").value;
  const std::string in_b = fl.at("input_b_file_name").value;
  if (in_a.empty())
    throw UsageError{"Error: primary input filename must be specified using --input_a_file_name"};
  if (as_bool(fl, "no_gpu"))
    throw UsageError{"Error: this engine runs on the GPU only (--no_gpu is not supported)"};
  const std::string ptype = fl.at("profile_type").value;
  const SCAMP::SCAMPProfileType profile_type = ParseProfileType(ptype);
  if (profile_type == SCAMP::PROFILE_TYPE_INVALID)
    throw UsageError{"Error: profile type " + ptype + " is not supported by this engine"};
  const bool self_join = in_b.empty();
  std::vector<double> ta, tb;
  readFile(in_a, ta);
  if (!self_join) readFile(in_b, tb);
  const long long n_x = static_cast<long long>(ta.size()) - window + 1;
  const long long n_y = self_join ? n_x : static_cast<long long>(tb.size()) - window + 1;
  if (n_x < 1 || n_y < 1)
    throw UsageError{"Error: window size must be smaller than the timeseries length"};
  const std::vector<int> devices = ParseIntList(fl.at("gpus").value);
  const bool keep = as_bool(fl, "keep_rows");
  SCAMP::SCAMPArgs args;
  args.window = static_cast<uint64_t>(window);
  args.max_tile_size = static_cast<uint64_t>(max_tile);
  args.has_b = !self_join;
  args.distributed_start_row = as_int(fl, "global_row");
  args.distributed_start_col = as_int(fl, "global_col");
  double thr = 0;
  parse_float(fl.at("threshold").value, &thr);
  args.distance_threshold = thr;
  args.computing_columns = true;
  args.computing_rows = self_join ? true : keep;
  args.precision_type = GetPrecisionType(prec[0], prec[1], prec[2], prec[3]);
  args.profile_type = profile_type;
  args.keep_rows_separate = keep;
  args.is_aligned = as_bool(fl, "aligned");
  args.timeseries_a = std::move(ta);
  args.timeseries_b = std::move(tb);
  args.silent_mode = !as_bool(fl, "print_debug_info");
  args.max_matches_per_column = as_int(fl, "max_matches_per_column");
  args.matrix_height = as_int(fl, "reduced_height");
  args.matrix_width = as_int(fl, "reduced_width");
  InitProfileMemory(&args);
  SCAMP::do_SCAMP(&args, devices.empty() ? std::vector<int>{0} : devices, 0);
  const bool pearson = as_bool(fl, "output_pearson");
  const int w = static_cast<int>(args.matrix_width), h = static_cast<int>(args.matrix_height);
  WriteProfileToFile(fl.at("output_a_file_name").value, fl.at("output_a_index_file_name").value,
                     args.profile_a, pearson, static_cast<int>(window), w, h);
  if (keep && profile_type != SCAMP::PROFILE_TYPE_MATRIX_SUMMARY)
    WriteProfileToFile(fl.at("output_b_file_name").value, fl.at("output_b_index_file_name").value,
                       args.profile_b, pearson, static_cast<int>(window), w, h);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return run(argc, argv);
  } catch (const UsageError& e) {
    std::cout << e.msg << std::endl;
  } catch (const SCAMPException& e) {
    std::cout << e.what() << std::endl;
  }
  return 1;
}
