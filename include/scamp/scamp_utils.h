// scamp_utils.h -- the utility functions that callers of do_SCAMP use around
// the join (zpzim/GPU-SCRIMP-LARGE src/scamp_utils.h, src/scamp_utils.cpp),
// header-only and in the global namespace as there: reading a series,
// parsing precision and profile-type options, converting correlations to
// distances, writing profiles to text files, and InitProfileMemory.
//
// Output files match the reference's byte for byte for the same profile
// values (numbers as printed by an ostream at precision 10).  The k-best
// lists (APPROX_ALL_NEIGHBORS) are written from this engine's layout (k
// entries per window in data[0].uint64_value, best first): one
// "column row value" line per match, columns in order, best match first.
#ifndef SCAMP_GB300_SCAMP_UTILS_H
#define SCAMP_GB300_SCAMP_UTILS_H

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "scamp/SCAMP.h"

// The reference declares InitProfileMemory here, outside namespace SCAMP.
using SCAMP::InitProfileMemory;

// sqrt(2 m (1 - r)), clamped at 0; NaN where there was no match (r < -1)
// (src/scamp_utils.cpp:127-133).
inline double ConvertToEuclidean(double val, int window) {
  if (val < -1) return NAN;
  return std::sqrt(std::max(2.0 * window * (1.0 - val), 0.0));
}

// r itself, NaN where there was no match (src/scamp_utils.cpp:135-141).
inline double CleanupPearson(double val) { return val < -1 ? NAN : val; }

// "1,2,3" -> {1, 2, 3}; "" -> {} (src/scamp_utils.cpp:74-88).
inline std::vector<int> ParseIntList(const std::string& s) {
  std::vector<int> out;
  if (s.empty()) return out;
  std::stringstream ss(s);
  std::string item;
  while (ss.good()) {
    std::getline(ss, item, ',');
    out.push_back(std::stoi(item));
  }
  return out;
}

// The first of ultra, double, mixed, single that is set
// (src/scamp_utils.cpp:90-105).
inline SCAMP::SCAMPPrecisionType GetPrecisionType(bool ultrap, bool doublep, bool mixedp,
                                                  bool singlep) {
  if (ultrap) return SCAMP::PRECISION_ULTRA;
  if (doublep) return SCAMP::PRECISION_DOUBLE;
  if (mixedp) return SCAMP::PRECISION_MIXED;
  if (singlep) return SCAMP::PRECISION_SINGLE;
  return SCAMP::PRECISION_INVALID;
}

// Profile type from its command-line name (src/scamp_utils.cpp:107-125).
inline SCAMP::SCAMPProfileType ParseProfileType(const std::string& s) {
  if (s == "1NN_INDEX") return SCAMP::PROFILE_TYPE_1NN_INDEX;
  if (s == "SUM_THRESH") return SCAMP::PROFILE_TYPE_SUM_THRESH;
  if (s == "1NN") return SCAMP::PROFILE_TYPE_1NN;
  if (s == "ALL_NEIGHBORS") return SCAMP::PROFILE_TYPE_APPROX_ALL_NEIGHBORS;
  if (s == "MATRIX_SUMMARY") return SCAMP::PROFILE_TYPE_MATRIX_SUMMARY;
  return SCAMP::PROFILE_TYPE_INVALID;
}

// Appends the whitespace-separated numbers of `filename` to `v`
// (src/scamp_utils.cpp:30-72).  As in the reference: a value is kept only
// when more input follows it (a last value without a trailing newline is
// dropped), and a missing file or a token that does not parse prints a
// message and ends the program with status 1.
inline void readFile(const std::string& filename, std::vector<double>& v) {
  std::ifstream f(filename);
  if (f.fail()) {
    std::cout << "Unable to open" << filename << "for reading, please make sure it exists"
              << std::endl;
    std::exit(1);
  }
  for (;;) {
    std::string token;
    if (!(f >> token)) break;  // only whitespace left
    double value;
    try {
      value = std::stod(token);
    } catch (const std::invalid_argument&) {
      std::cout << token[0] << std::endl;
      std::cout << "FATAL ERROR: invalid argument: Could not parse line number " << v.size() + 1
                << " from input file.\n";
      std::exit(1);
    } catch (const std::out_of_range&) {
      std::cout << token[0] << std::endl;
      std::cout << "FATAL ERROR: out of range: Could not parse line number " << v.size() + 1
                << " from input file.\n";
      std::exit(1);
    }
    if (f.peek() == EOF) break;
    v.push_back(value);
  }
}

// A matrix summary, `matrix_width` values per line, each followed by a space
// (src/scamp_utils.cpp:9-28).
inline void write_matrix(const std::string& mp, bool output_pearson,
                         const std::vector<float>& matrix, int window, int matrix_width,
                         int matrix_height) {
  (void)matrix_height;
  std::ofstream out(mp);
  out << std::setprecision(10);
  for (size_t i = 0; i < matrix.size(); ++i) {
    if (i > 0 && matrix_width > 0 && i % static_cast<size_t>(matrix_width) == 0) out << std::endl;
    out << (output_pearson ? CleanupPearson(matrix[i]) : ConvertToEuclidean(matrix[i], window))
        << " ";
  }
  out << std::endl;
}

// Writes a profile as the reference's command line does
// (src/scamp_utils.cpp:143-224): 1NN_INDEX to `mp` (distances, or
// correlations with output_pearson) and `mpi` (indices, -1 where there was
// no match); 1NN and SUM_THRESH to `mp`; APPROX_ALL_NEIGHBORS as
// "column row value" lines; MATRIX_SUMMARY through write_matrix.
inline bool WriteProfileToFile(const std::string& mp, const std::string& mpi, SCAMP::Profile& p,
                               bool output_pearson, int window, int matrix_width,
                               int matrix_height) {
  auto value = [&](double r) {
    return output_pearson ? CleanupPearson(r) : ConvertToEuclidean(r, window);
  };
  auto unpack = [](uint64_t e, float* r, int64_t* idx) {
    const uint32_t lo = static_cast<uint32_t>(e & 0xFFFFFFFFu);
    std::memcpy(r, &lo, sizeof lo);
    *idx = *r < -1 ? -1 : static_cast<int64_t>(e >> 32);
  };
  if (p.data.empty()) return false;
  switch (p.type) {
    case SCAMP::PROFILE_TYPE_1NN_INDEX: {
      std::ofstream out(mp), outi(mpi);
      out << std::setprecision(10);
      for (const uint64_t e : p.data[0].uint64_value) {
        float r;
        int64_t idx;
        unpack(e, &r, &idx);
        out << value(r) << std::endl;
        outi << idx << std::endl;
      }
      break;
    }
    case SCAMP::PROFILE_TYPE_1NN: {
      std::ofstream out(mp);
      out << std::setprecision(10);
      for (const float r : p.data[0].float_value) out << value(r) << std::endl;
      break;
    }
    case SCAMP::PROFILE_TYPE_SUM_THRESH: {
      std::ofstream out(mp);
      out << std::setprecision(10);
      for (const double s : p.data[0].double_value) out << s << std::endl;
      break;
    }
    case SCAMP::PROFILE_TYPE_APPROX_ALL_NEIGHBORS: {
      std::ofstream out(mp);
      out << std::setprecision(10);
      const std::vector<uint64_t>& e = p.data[0].uint64_value;
      const size_t k = p.matches_per_window > 0 ? static_cast<size_t>(p.matches_per_window) : 1;
      for (size_t i = 0; i < e.size(); ++i) {
        float r;
        int64_t idx;
        unpack(e[i], &r, &idx);
        if (idx < 0) continue;
        out << i / k << " " << idx << " " << value(r) << std::endl;
      }
      break;
    }
    case SCAMP::PROFILE_TYPE_MATRIX_SUMMARY:
      write_matrix(mp, output_pearson, p.data[0].float_value, window, matrix_width,
                   matrix_height);
      break;
    default:
      break;
  }
  return true;
}

#endif  // SCAMP_GB300_SCAMP_UTILS_H
