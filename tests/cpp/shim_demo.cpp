// Drives the C++ do_SCAMP shim (include/scamp/SCAMP.h) the way a reference
// user would.  Modes:
//   errors            argument errors and the no-device case must throw
//                     SCAMPException (needs no GPU)
//   join <in> <out>   self-join (1NN_INDEX, DOUBLE, m from argv[4]) of the
//                     float64 series in <in>; writes profile_a (uint64) to <out>
//   utils <dir>       scamp_utils.h without a GPU: readFile of <dir>/in.txt
//                     into <dir>/read.bin, WriteProfileToFile of the raw
//                     profiles <dir>/{nn_index,nn,sum,knn,matrix}.bin into
//                     <dir>/out_*.txt, and the option parsers
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "scamp/SCAMP.h"
#include "scamp/scamp_utils.h"

template <typename T>
static std::vector<T> read_raw(const std::string& path) {
  std::ifstream in(path, std::ios::binary | std::ios::ate);
  const size_t n = static_cast<size_t>(in.tellg()) / sizeof(T);
  in.seekg(0);
  std::vector<T> v(n);
  in.read(reinterpret_cast<char*>(v.data()), n * sizeof(T));
  return v;
}

static int utils_mode(const std::string& dir) {
  int bad = 0;
  std::vector<double> v;
  readFile(dir + "/in.txt", v);
  std::ofstream(dir + "/read.bin", std::ios::binary)
      .write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(double));
  const int m = 16, k = 3, h = 4, w = 5;
  SCAMP::Profile p1(SCAMP::PROFILE_TYPE_1NN_INDEX, 0);
  p1.data[0].uint64_value = read_raw<uint64_t>(dir + "/nn_index.bin");
  SCAMP::Profile p2(SCAMP::PROFILE_TYPE_1NN, 0);
  p2.data[0].float_value = read_raw<float>(dir + "/nn.bin");
  SCAMP::Profile p3(SCAMP::PROFILE_TYPE_SUM_THRESH, 0);
  p3.data[0].double_value = read_raw<double>(dir + "/sum.bin");
  SCAMP::Profile p4(SCAMP::PROFILE_TYPE_APPROX_ALL_NEIGHBORS, 0);
  p4.data[0].uint64_value = read_raw<uint64_t>(dir + "/knn.bin");
  p4.matches_per_window = k;
  SCAMP::Profile p5(SCAMP::PROFILE_TYPE_MATRIX_SUMMARY, 0);
  p5.data[0].float_value = read_raw<float>(dir + "/matrix.bin");
  for (int pearson = 0; pearson < 2; ++pearson) {
    const std::string s = pearson ? "_pearson" : "";
    WriteProfileToFile(dir + "/out_nn_index" + s + ".txt", dir + "/out_nn_index_i" + s + ".txt", p1,
                       pearson, m, w, h);
    WriteProfileToFile(dir + "/out_nn" + s + ".txt", "", p2, pearson, m, w, h);
    WriteProfileToFile(dir + "/out_knn" + s + ".txt", "", p4, pearson, m, w, h);
    WriteProfileToFile(dir + "/out_matrix" + s + ".txt", "", p5, pearson, m, w, h);
  }
  WriteProfileToFile(dir + "/out_sum.txt", "", p3, false, m, w, h);
  const std::vector<int> ints = ParseIntList("0,3,12");
  bad += !(ints.size() == 3 && ints[1] == 3 && ints[2] == 12) + !ParseIntList("").empty();
  bad += GetPrecisionType(false, true, true, false) != SCAMP::PRECISION_DOUBLE;
  bad += GetPrecisionType(false, false, false, false) != SCAMP::PRECISION_INVALID;
  bad += ParseProfileType("ALL_NEIGHBORS") != SCAMP::PROFILE_TYPE_APPROX_ALL_NEIGHBORS;
  bad += ParseProfileType("FREQUENCY_THRESH") != SCAMP::PROFILE_TYPE_INVALID;
  bad += !std::isnan(ConvertToEuclidean(-2.0, 10)) + (ConvertToEuclidean(1.5, 10) != 0.0);
  bad += !std::isnan(CleanupPearson(-3.0)) + (CleanupPearson(0.25) != 0.25);
  SCAMP::SCAMPArgs a;  // the reference's global InitProfileMemory
  a.timeseries_a.assign(50, 0.0);
  a.window = 10;
  a.profile_type = SCAMP::PROFILE_TYPE_APPROX_ALL_NEIGHBORS;
  a.max_matches_per_column = k;
  bad += !::InitProfileMemory(&a) + (a.profile_a.data[0].uint64_value.size() != 41u * k);
  std::cout << (bad ? "FAIL" : "OK") << " " << v.size() << "\n";
  return bad;
}

static int expect_throw(SCAMP::SCAMPArgs& a, const char* what) {
  try {
    SCAMP::do_SCAMP(&a);
  } catch (const SCAMPException& e) {
    std::cout << what << ": " << e.what() << "\n";
    return 0;
  }
  std::cout << what << ": no exception\n";
  return 1;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string mode = argv[1];
  if (mode == "errors") {
    int bad = 0;
    SCAMP::SCAMPArgs a;
    a.timeseries_a.assign(100, 1.0);
    a.window = 200;  // longer than the series
    bad += expect_throw(a, "window");
    // SCAMPArgs::validate checks without running anything
    try {
      a.validate();
      std::cout << "validate: no exception\n";
      bad += 1;
    } catch (const SCAMPException& e) {
      std::cout << "validate: " << e.what() << "\n";
    }
    a.window = 2;
    try {
      a.validate();
      bad += 1;
    } catch (const SCAMPException& e) {
      std::cout << "validate: " << e.what() << "\n";
    }
    a.window = 200;
    a.print();
    if (SCAMP::InitProfileMemory(&a)) bad += 1;  // must refuse
    a.window = 10;
    a.precision_type = SCAMP::PRECISION_INVALID;
    SCAMP::InitProfileMemory(&a);
    bad += expect_throw(a, "precision");
    a.precision_type = SCAMP::PRECISION_DOUBLE;
    a.profile_a = SCAMP::Profile();  // not initialised
    bad += expect_throw(a, "profile");
    if (!scamp_gb300_gpu_supported()) {
      SCAMP::InitProfileMemory(&a);
      bad += expect_throw(a, "device");
    }
    std::cout << (bad ? "FAIL" : "OK") << "\n";
    return bad;
  }
  if (mode == "utils" && argc >= 3) return utils_mode(argv[2]);
  if (mode == "join" && argc >= 5) {
    std::ifstream in(argv[2], std::ios::binary | std::ios::ate);
    const size_t n = static_cast<size_t>(in.tellg()) / sizeof(double);
    in.seekg(0);
    std::vector<double> series(n);
    in.read(reinterpret_cast<char*>(series.data()), n * sizeof(double));
    SCAMP::SCAMPArgs a;
    a.timeseries_a = series;
    a.window = std::stoull(argv[4]);
    a.precision_type = SCAMP::PRECISION_DOUBLE;
    a.profile_type = SCAMP::PROFILE_TYPE_1NN_INDEX;
    if (!SCAMP::InitProfileMemory(&a)) return 3;
    SCAMP::do_SCAMP(&a);
    const auto& p = a.profile_a.data[0].uint64_value;
    std::ofstream out(argv[3], std::ios::binary);
    out.write(reinterpret_cast<const char*>(p.data()), p.size() * sizeof(uint64_t));
    std::cout << "OK " << p.size() << "\n";
    return 0;
  }
  return 2;
}
