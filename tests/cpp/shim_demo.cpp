// Drives the C++ do_SCAMP shim (include/scamp/SCAMP.h) the way a reference
// user would.  Modes:
//   errors            argument errors and the no-device case must throw
//                     SCAMPException (needs no GPU)
//   join <in> <out>   self-join (1NN_INDEX, DOUBLE, m from argv[4]) of the
//                     float64 series in <in>; writes profile_a (uint64) to <out>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "scamp/SCAMP.h"

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
