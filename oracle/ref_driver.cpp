// ref_driver.cpp -- C entry point over the reference's own CPU path.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference's CPU sources where they lie (src/{common,cpu_stats,
// cpu_kernels,kernel_common,qt_helper,tile,SCAMP,scamp_utils}.cpp of
// zpzim/GPU-SCRIMP-LARGE) into oracle/_ref/libscampref.so.  Nothing from the
// reference is copied into this repository; this file only builds a
// SCAMP::SCAMPArgs the way python/SCAMP_python.cpp:67-89,179-236 does and calls
// SCAMP::do_SCAMP(args, {}, threads) (src/SCAMP.cpp:279-334) on CPU workers.
#include <cstdint>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "SCAMP.h"
#include "common.h"
#include "scamp_utils.h"

extern "C" int ref_scamp_join(const double* a, uint64_t na, const double* b,
                              uint64_t nb, int has_b, uint64_t window,
                              uint64_t max_tile_size, int profile_type,
                              int precision, int computing_rows,
                              int computing_cols, int keep_rows, int aligned,
                              int64_t start_row, int64_t start_col,
                              double threshold, int threads, uint64_t* prof_a,
                              uint64_t* prof_b, double* sum_a, double* sum_b,
                              char* err, uint64_t errlen) {
  try {
    SCAMP::SCAMPArgs args;
    args.timeseries_a.assign(a, a + na);
    if (has_b) {
      args.timeseries_b.assign(b, b + nb);
    } else {
      args.timeseries_b = args.timeseries_a;
    }
    args.has_b = has_b != 0;
    args.window = window;
    args.max_tile_size = max_tile_size;
    args.distributed_start_row = start_row;
    args.distributed_start_col = start_col;
    args.distance_threshold = threshold;
    args.precision_type = static_cast<SCAMP::SCAMPPrecisionType>(precision);
    args.profile_type = static_cast<SCAMP::SCAMPProfileType>(profile_type);
    args.computing_rows = computing_rows != 0;
    args.computing_columns = computing_cols != 0;
    args.keep_rows_separate = keep_rows != 0;
    args.is_aligned = aligned != 0;
    args.silent_mode = true;
    args.max_matches_per_column = 5;
    args.matrix_height = 50;
    args.matrix_width = 50;
    args.profile_a.type = args.profile_type;
    args.profile_b.type = args.profile_type;
    if (!InitProfileMemory(&args)) {
      std::strncpy(err, "InitProfileMemory failed", errlen);
      return 2;
    }
    std::vector<int> devices;
    SCAMP::do_SCAMP(&args, devices, threads);
    if (args.profile_type == SCAMP::PROFILE_TYPE_1NN_INDEX) {
      const auto& pa = args.profile_a.data[0].uint64_value;
      std::memcpy(prof_a, pa.data(), pa.size() * sizeof(uint64_t));
      if (keep_rows && prof_b) {
        const auto& pb = args.profile_b.data[0].uint64_value;
        std::memcpy(prof_b, pb.data(), pb.size() * sizeof(uint64_t));
      }
    } else if (args.profile_type == SCAMP::PROFILE_TYPE_SUM_THRESH) {
      const auto& pa = args.profile_a.data[0].double_value;
      std::memcpy(sum_a, pa.data(), pa.size() * sizeof(double));
      if (keep_rows && sum_b) {
        const auto& pb = args.profile_b.data[0].double_value;
        std::memcpy(sum_b, pb.data(), pb.size() * sizeof(double));
      }
    } else if (args.profile_type == SCAMP::PROFILE_TYPE_1NN) {
      // float profile, returned widened to double in sum_a / sum_b
      const auto& pa = args.profile_a.data[0].float_value;
      for (size_t i = 0; i < pa.size(); ++i) sum_a[i] = pa[i];
      if (keep_rows && sum_b) {
        const auto& pb = args.profile_b.data[0].float_value;
        for (size_t i = 0; i < pb.size(); ++i) sum_b[i] = pb[i];
      }
    }
  } catch (const std::exception& e) {
    std::strncpy(err, e.what(), errlen);
    return 1;
  }
  return 0;
}
