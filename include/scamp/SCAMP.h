// SCAMP.h -- C++ drop-in for SCAMP::do_SCAMP on the GB300 engine.
//
// Header-only host code over the C ABI (scamp_gb300.h).  It keeps the
// reference's interface for the join path: namespace SCAMP, the SCAMPArgs
// fields and meaning (zpzim/GPU-SCRIMP-LARGE src/common.h:164-188), the
// profile enums (src/common.h:34-58), Profile/ProfileData storage of the
// results (src/common.h:96-150, 1NN_INDEX in data[0].uint64_value with the
// mp_entry layout, SUM_THRESH in data[0].double_value, 1NN in
// data[0].float_value, APPROX_ALL_NEIGHBORS as max_matches_per_column
// entries per window in data[0].uint64_value, MATRIX_SUMMARY as the grid in
// data[0].float_value), SCAMPArgs::validate / print
// (src/common.cpp:417-436, 495-515), InitProfileMemory
// (src/scamp_utils.cpp:226-245), do_SCAMP (src/SCAMP.h:15-18) and
// SCAMPException for every failure (src/scamp_exception.h:7-22).  Link with
// libscamp_gb300.so.
//
// FREQUENCY_THRESH and 1NN_MULTIDIM, which the reference declares but does
// not implement, are absent.
#ifndef SCAMP_GB300_SCAMP_H
#define SCAMP_GB300_SCAMP_H

#include <cstdint>
#include <cstring>
#include <exception>
#include <iostream>
#include <string>
#include <vector>

#include "scamp_gb300.h"

class SCAMPException : public std::exception {
 public:
  explicit SCAMPException(std::string message) : msg_(std::move(message)) {}
  const char* what() const noexcept override { return msg_.c_str(); }

 private:
  std::string msg_;
};

namespace SCAMP {

enum SCAMPProfileType {
  PROFILE_TYPE_INVALID = 0,
  PROFILE_TYPE_1NN_INDEX = SCAMP_PROFILE_1NN_INDEX,
  PROFILE_TYPE_SUM_THRESH = SCAMP_PROFILE_SUM_THRESH,
  PROFILE_TYPE_1NN = SCAMP_PROFILE_1NN,
  PROFILE_TYPE_APPROX_ALL_NEIGHBORS = SCAMP_PROFILE_APPROX_ALL_NEIGHBORS,
  PROFILE_TYPE_MATRIX_SUMMARY = SCAMP_PROFILE_MATRIX_SUMMARY,
};

enum SCAMPPrecisionType {
  PRECISION_INVALID = 0,
  PRECISION_SINGLE = SCAMP_PRECISION_SINGLE,
  PRECISION_MIXED = SCAMP_PRECISION_MIXED,
  PRECISION_DOUBLE = SCAMP_PRECISION_DOUBLE,
  PRECISION_ULTRA = SCAMP_PRECISION_ULTRA,
};

struct ProfileData {
  // 1NN_INDEX: low word float r, high word index; APPROX_ALL_NEIGHBORS:
  // max_matches_per_column such entries per window, best first
  std::vector<uint64_t> uint64_value;
  std::vector<double> double_value;    // SUM_THRESH
  std::vector<float> float_value;      // 1NN: best correlation; MATRIX_SUMMARY: the grid
};

struct Profile {
  Profile() : type(PROFILE_TYPE_INVALID) {}
  Profile(SCAMPProfileType t, size_t size) : type(t) { Alloc(size); }

  // Best-so-far initial values: {r = -2.0f, index = 0xFFFFFFFF} per 1NN_INDEX
  // (and APPROX_ALL_NEIGHBORS) entry, -2.0f per 1NN (and MATRIX_SUMMARY)
  // entry, 0 per SUM_THRESH entry.  `size` counts entries.
  void Alloc(size_t size) {
    data.assign(1, ProfileData());
    if (type == PROFILE_TYPE_1NN_INDEX || type == PROFILE_TYPE_APPROX_ALL_NEIGHBORS) {
      const float minus_two = -2.0f;
      uint32_t bits;
      static_assert(sizeof bits == sizeof minus_two, "float is 32 bits");
      std::memcpy(&bits, &minus_two, sizeof bits);
      data[0].uint64_value.assign(size, (uint64_t{0xFFFFFFFFu} << 32) | bits);
    } else if (type == PROFILE_TYPE_SUM_THRESH) {
      data[0].double_value.assign(size, 0.0);
    } else if (type == PROFILE_TYPE_1NN || type == PROFILE_TYPE_MATRIX_SUMMARY) {
      data[0].float_value.assign(size, -2.0f);
    }
  }

  std::vector<ProfileData> data;
  SCAMPProfileType type;
  // APPROX_ALL_NEIGHBORS: entries per window (max_matches_per_column)
  int64_t matches_per_window = 1;
};

struct SCAMPArgs {
  // Throws SCAMPException for arguments the join rejects (the reference's
  // checks, src/common.cpp:417-436, and this engine's own).
  void validate() const;
  // The fields, one per line (src/common.cpp:495-515).
  void print() const;

  std::vector<double> timeseries_a;
  std::vector<double> timeseries_b;
  Profile profile_a;
  Profile profile_b;
  bool has_b = false;
  uint64_t window = 0;
  uint64_t max_tile_size = 1 << 17;
  int64_t distributed_start_row = -1;
  int64_t distributed_start_col = -1;
  double distance_threshold = 0.0;
  SCAMPPrecisionType precision_type = PRECISION_DOUBLE;
  SCAMPProfileType profile_type = PROFILE_TYPE_1NN_INDEX;
  bool computing_rows = true;
  bool computing_columns = true;
  bool keep_rows_separate = false;
  bool is_aligned = false;
  bool silent_mode = true;
  int64_t max_matches_per_column = 5;  // APPROX_ALL_NEIGHBORS
  int64_t matrix_height = 50;          // MATRIX_SUMMARY
  int64_t matrix_width = 50;
  // Filled by do_SCAMP (no counterpart in the reference's SCAMPArgs): the
  // accuracy statement of the last join, scamp_c_result's max_abs_r_err
  // and max_tie_margin (-1 where not tracked).
  double max_abs_r_err = -1.0;
  double max_tie_margin = -1.0;
};

namespace detail {

inline scamp_c_args to_c(const SCAMPArgs& a) {
  scamp_c_args c{};
  c.timeseries_a = a.timeseries_a.data();
  c.len_a = a.timeseries_a.size();
  c.timeseries_b = a.has_b ? a.timeseries_b.data() : nullptr;
  c.len_b = a.has_b ? a.timeseries_b.size() : 0;
  c.has_b = a.has_b ? 1 : 0;
  c.window = a.window;
  c.max_tile_size = a.max_tile_size;
  c.distributed_start_row = a.distributed_start_row;
  c.distributed_start_col = a.distributed_start_col;
  c.distance_threshold = a.distance_threshold;
  c.precision_type = static_cast<int32_t>(a.precision_type);
  c.profile_type = static_cast<int32_t>(a.profile_type);
  c.computing_rows = a.computing_rows ? 1 : 0;
  c.computing_columns = a.computing_columns ? 1 : 0;
  c.keep_rows_separate = a.keep_rows_separate ? 1 : 0;
  c.is_aligned = a.is_aligned ? 1 : 0;
  c.silent_mode = a.silent_mode ? 1 : 0;
  c.max_matches_per_column = static_cast<int32_t>(a.max_matches_per_column);
  c.matrix_height = static_cast<int32_t>(a.matrix_height);
  c.matrix_width = static_cast<int32_t>(a.matrix_width);
  return c;
}

inline void check(int rc, const char* msg) {
  if (rc != SCAMP_OK) throw SCAMPException(msg[0] ? std::string(msg) : "SCAMP error " + std::to_string(rc));
}

}  // namespace detail

inline std::string GetProfileTypeString(SCAMPProfileType t) {
  switch (t) {
    case PROFILE_TYPE_1NN_INDEX: return "PROFILE_TYPE_1NN_INDEX";
    case PROFILE_TYPE_SUM_THRESH: return "PROFILE_TYPE_SUM_THRESH";
    case PROFILE_TYPE_1NN: return "PROFILE_TYPE_1NN";
    case PROFILE_TYPE_APPROX_ALL_NEIGHBORS: return "PROFILE_TYPE_APPROX_ALL_NEIGHBORS";
    case PROFILE_TYPE_MATRIX_SUMMARY: return "PROFILE_TYPE_MATRIX_SUMMARY";
    default: return "PROFILE_TYPE_INVALID";
  }
}

inline std::string GetPrecisionTypeString(SCAMPPrecisionType t) {
  switch (t) {
    case PRECISION_SINGLE: return "PRECISION_SINGLE";
    case PRECISION_MIXED: return "PRECISION_MIXED";
    case PRECISION_DOUBLE: return "PRECISION_DOUBLE";
    case PRECISION_ULTRA: return "PRECISION_ULTRA";
    default: return "PRECISION_INVALID";
  }
}

inline void SCAMPArgs::validate() const {
  char msg[512] = {0};
  const scamp_c_args c = detail::to_c(*this);
  detail::check(scamp_gb300_validate(&c, msg, sizeof msg), msg);
}

inline void SCAMPArgs::print() const {
  std::cout << "window: " << window << std::endl;
  std::cout << "max_tile_size: " << max_tile_size << std::endl;
  std::cout << "has_b: " << has_b << std::endl;
  std::cout << "keep_rows_separate: " << keep_rows_separate << std::endl;
  std::cout << "distributed_start_row: " << distributed_start_row << std::endl;
  std::cout << "distributed_start_col: " << distributed_start_col << std::endl;
  std::cout << "computing_rows: " << computing_rows << std::endl;
  std::cout << "computing_columns: " << computing_columns << std::endl;
  std::cout << "is_aligned: " << is_aligned << std::endl;
  std::cout << "profile_type: " << GetProfileTypeString(profile_type) << std::endl;
  std::cout << "precision_type: " << GetPrecisionTypeString(precision_type) << std::endl;
  std::cout << "distance_threshold: " << distance_threshold << std::endl;
  std::cout << "silent_mode: " << silent_mode << std::endl;
  std::cout << "max_matches_per_column: " << max_matches_per_column << std::endl;
  std::cout << "timeseries_a size: " << timeseries_a.size() << std::endl;
  std::cout << "timeseries_b size: " << timeseries_b.size() << std::endl;
}

// Allocates and initialises the profiles the join writes (the caller calls it
// before do_SCAMP, as with the reference).  Returns false for a window longer
// than a series.
inline bool InitProfileMemory(SCAMPArgs* args) {
  const int64_t na = static_cast<int64_t>(args->timeseries_a.size()) - static_cast<int64_t>(args->window) + 1;
  const int64_t nb = args->has_b
                         ? static_cast<int64_t>(args->timeseries_b.size()) - static_cast<int64_t>(args->window) + 1
                         : na;
  if (na <= 0 || (args->keep_rows_separate && nb <= 0)) return false;
  int64_t per = 1;
  if (args->profile_type == PROFILE_TYPE_APPROX_ALL_NEIGHBORS) per = args->max_matches_per_column;
  if (args->profile_type == PROFILE_TYPE_MATRIX_SUMMARY) {
    args->profile_a = Profile(args->profile_type,
                              static_cast<size_t>(args->matrix_height * args->matrix_width));
    return true;
  }
  args->profile_a = Profile(args->profile_type, static_cast<size_t>(na * per));
  args->profile_a.matches_per_window = per;
  if (args->keep_rows_separate) {
    args->profile_b = Profile(args->profile_type, static_cast<size_t>(nb * per));
    args->profile_b.matches_per_window = per;
  }
  return true;
}

// Runs the join on the first device of `devices` (default 0); the results are
// merged into args->profile_a (and profile_b when keep_rows_separate).
// `num_threads` (CPU workers in the reference) is accepted and unused: this
// engine has no CPU path.  Throws SCAMPException on any error.
inline void do_SCAMP(SCAMPArgs* args, const std::vector<int>& devices, int num_threads) {
  (void)num_threads;
  char msg[512] = {0};
  scamp_c_args c = detail::to_c(*args);
  c.device = devices.empty() ? 0 : devices[0];
  detail::check(scamp_gb300_validate(&c, msg, sizeof msg), msg);
  const bool knn = args->profile_type == PROFILE_TYPE_APPROX_ALL_NEIGHBORS;
  const bool mat = args->profile_type == PROFILE_TYPE_MATRIX_SUMMARY;
  const bool nn = args->profile_type == PROFILE_TYPE_1NN_INDEX || knn;
  const bool nn_max = args->profile_type == PROFILE_TYPE_1NN || mat;
  const size_t per = knn ? static_cast<size_t>(args->max_matches_per_column) : 1;
  const size_t na = mat ? static_cast<size_t>(args->matrix_height * args->matrix_width)
                        : (args->timeseries_a.size() - args->window + 1) * per;
  const size_t nb = (args->has_b ? args->timeseries_b.size() - args->window + 1
                                 : args->timeseries_a.size() - args->window + 1) * per;
  auto sized = [&](Profile& p, size_t n) {
    if (p.type != args->profile_type || p.data.empty() ||
        (nn ? p.data[0].uint64_value.size()
            : nn_max ? p.data[0].float_value.size() : p.data[0].double_value.size()) != n)
      throw SCAMPException("Error: profile memory not initialised (call InitProfileMemory)");
  };
  sized(args->profile_a, na);
  if (args->keep_rows_separate && !mat) sized(args->profile_b, nb);
  scamp_c_result r{};
  if (knn) {
    r.knn_a = args->profile_a.data[0].uint64_value.data();
    if (args->keep_rows_separate) r.knn_b = args->profile_b.data[0].uint64_value.data();
  } else if (mat) {
    r.matrix = args->profile_a.data[0].float_value.data();
  } else if (nn) {
    r.profile_a = args->profile_a.data[0].uint64_value.data();
    if (args->keep_rows_separate) r.profile_b = args->profile_b.data[0].uint64_value.data();
  } else if (nn_max) {
    r.max_a = args->profile_a.data[0].float_value.data();
    if (args->keep_rows_separate) r.max_b = args->profile_b.data[0].float_value.data();
  } else {
    r.sum_a = args->profile_a.data[0].double_value.data();
    if (args->keep_rows_separate) r.sum_b = args->profile_b.data[0].double_value.data();
  }
  detail::check(scamp_gb300_join(&c, &r, msg, sizeof msg), msg);
  args->max_abs_r_err = r.max_abs_r_err;
  args->max_tie_margin = r.max_tie_margin;
}

inline void do_SCAMP(SCAMPArgs* args) { do_SCAMP(args, std::vector<int>{0}, 0); }

}  // namespace SCAMP

#endif  // SCAMP_GB300_SCAMP_H
