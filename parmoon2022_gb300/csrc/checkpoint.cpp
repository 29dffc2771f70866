// checkpoint.cpp -- solution vectors to and from files in the reference's
// checkpoint format, and the CheckpointIO naming / interval rules.
//
// Format (BlockVector::write_to_stream / read_from_stream,
// src/Matrix/BlockVector.C:1064-1139): a text line holding only the number
// of entries, then the entries as raw native doubles.  CheckpointIO
// (src/FE/CheckpointIO.C:68-130): a time-dependent run writes after every
// n-th completed step (never at step 0) into `base` or, unless overwriting,
// `base + "." + std::to_string(time)`.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "parmoon_cd.h"

namespace cdg {
void set_error(const char* fmt, ...);
}

using cdg::set_error;

namespace {

int write_vector(const char* filename, const double* v, long long n) {
  if (!filename || (!v && n > 0) || n < 0) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  std::ofstream dat(filename, std::ios::binary);
  if (!dat) {
    // the reference warns and returns (BlockVector::write_to_file)
    set_error("cannot open file '%s' to save data", filename);
    return CDG_ERR_ARG;
  }
  dat << n << '\n';
  dat.write(reinterpret_cast<const char*>(v), (std::streamsize)(sizeof(double) * n));
  if (!dat) {
    set_error("writing '%s' failed", filename);
    return CDG_ERR_ARG;
  }
  return CDG_OK;
}

// n_expected > 0: the file must hold exactly that many entries; 0: any count
// up to capacity (the reference resizes an empty vector to the file's size)
int read_vector(const char* filename, double* v, long long capacity, long long n_expected,
                long long* n_read) {
  if (!filename || !n_read || capacity < 0 || n_expected < 0) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  std::ifstream dat(filename, std::ios::binary);
  if (!dat) {
    set_error("cannot open file '%s' to read data", filename);
    return CDG_ERR_ARG;
  }
  std::string line;
  std::getline(dat, line);
  std::istringstream parser(line);
  unsigned long long len = 0;
  parser >> len >> std::ws;   // a failed parse leaves 0, as the reference's read does
  if (parser.good()) {
    set_error("formatting error, the first line in the file should contain only a number "
              "indicating the number of entries to be read");
    return CDG_ERR_ARG;
  }
  *n_read = (long long)len;
  if (n_expected > 0 && (long long)len != n_expected) {
    set_error("unexpected size to be read. Expected: %lld\tin file: %llu", n_expected, len);
    return CDG_ERR_ARG;
  }
  if ((long long)len > capacity || (!v && len > 0)) {
    set_error("file holds %llu entries, buffer %lld", len, capacity);
    return CDG_ERR_LIMIT;
  }
  dat.read(reinterpret_cast<char*>(v), (std::streamsize)(sizeof(double) * len));
  if ((unsigned long long)dat.gcount() != sizeof(double) * len) {
    set_error("'%s' ends after %lld of %llu bytes", filename, (long long)dat.gcount(),
              (unsigned long long)(sizeof(double) * len));
    return CDG_ERR_ARG;
  }
  return CDG_OK;
}

std::string checkpoint_name(const char* base, double time, int overwrite) {
  std::string name = base;
  if (!overwrite) name += "." + std::to_string(time);
  return name;
}

}  // namespace

extern "C" {

int cdg_vector_write_file(const char* filename, const double* v, long long n) {
  return write_vector(filename, v, n);
}

int cdg_vector_read_file(const char* filename, double* v, long long capacity,
                         long long n_expected, long long* n_read) {
  return read_vector(filename, v, capacity, n_expected, n_read);
}

int cdg_checkpoint_file_name(const char* base, double time, int overwrite, char* out,
                             long long capacity) {
  if (!base || !out || capacity < 1) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  const std::string name = checkpoint_name(base, time, overwrite);
  if ((long long)name.size() + 1 > capacity) {
    set_error("file name of %zu characters, buffer %lld", name.size(), capacity);
    return CDG_ERR_LIMIT;
  }
  std::memcpy(out, name.c_str(), name.size() + 1);
  return CDG_OK;
}

int cdg_problem_write_solution(cdg_problem* p, const char* filename) {
  int info[6];
  int rc = cdg_problem_level_info(p, 0, info);
  if (rc != CDG_OK) return rc;
  std::vector<double> sol((size_t)info[2]);
  rc = cdg_problem_get_solution(p, sol.data());
  if (rc != CDG_OK) return rc;
  return write_vector(filename, sol.data(), (long long)sol.size());
}

int cdg_problem_read_solution(cdg_problem* p, const char* filename) {
  int info[6];
  int rc = cdg_problem_level_info(p, 0, info);
  if (rc != CDG_OK) return rc;
  std::vector<double> sol((size_t)info[2]);
  long long n = 0;
  rc = read_vector(filename, sol.data(), (long long)sol.size(), (long long)sol.size(), &n);
  if (rc != CDG_OK) return rc;
  return cdg_problem_set_solution(p, sol.data());
}

int cdg_problem_checkpoint(cdg_problem* p, const char* base, int step, double time,
                           int every_n_steps, int overwrite, int* written) {
  if (!p || !base || !written || every_n_steps < 1 || step < 0) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  *written = 0;
  if (step == 0 || step % every_n_steps != 0) return CDG_OK;   // skip the initial time
  const std::string name = checkpoint_name(base, time, overwrite);
  const int rc = cdg_problem_write_solution(p, name.c_str());
  if (rc == CDG_OK) *written = 1;
  return rc;
}

}  // extern "C"
