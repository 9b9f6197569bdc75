// Amber NetCDF trajectory writer: the file that mme_init_sff(..., ncname)
// creates and md() appends a frame to every ntwx steps (the reference's
// src/sff/AmberNetcdf.c:595-740 over the netCDF library,
// sff.c:1164-1168 and 2341-2342).
//
// Written directly in the netCDF classic format with 64-bit offsets
// ("CDF\x02", the format the reference asks the library for): a big-endian
// header of dimensions, attributes and variables, the fixed-size variables,
// then one record per frame.  The layout follows the published netCDF
// classic format specification; the names, dimensions and attributes are
// the AMBER trajectory convention the reference defines (dimensions frame
// (unlimited), spatial 3, atom N, cell_spatial 3, label 5, cell_angular 3;
// variables time(frame) float "picosecond", spatial(spatial) char,
// coordinates(frame, atom, spatial) float "angstrom", cell_spatial char,
// cell_angular char; global title, application, program, programVersion,
// Conventions, ConventionVersion), so readers of Amber trajectories (cpptraj,
// MDAnalysis, scipy.io.netcdf_file) open it.
//
// The record count in the header is rewritten and the stream flushed after
// every frame, as the reference syncs after each write, so a file is
// readable while md() runs.  One difference: the time of each frame is
// written (md's time in ps); the reference defines the variable but leaves
// it unwritten.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sffg_internal.h"

namespace sffg {
namespace {

constexpr uint32_t kNcChar = 2, kNcFloat = 5;
constexpr uint32_t kNcDimension = 0x0A, kNcVariable = 0x0B, kNcAttribute = 0x0C;

struct Out {
  std::vector<unsigned char> b;
  void u32(uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) b.push_back(static_cast<unsigned char>(v >> s));
  }
  void u64(uint64_t v) {
    for (int s = 56; s >= 0; s -= 8) b.push_back(static_cast<unsigned char>(v >> s));
  }
  void pad() {
    while (b.size() % 4) b.push_back(0);
  }
  void name(const std::string &s) {
    u32(static_cast<uint32_t>(s.size()));
    b.insert(b.end(), s.begin(), s.end());
    pad();
  }
  void text_attr(const std::string &n, const std::string &v) {
    name(n);
    u32(kNcChar);
    u32(static_cast<uint32_t>(v.size()));
    b.insert(b.end(), v.begin(), v.end());
    pad();
  }
};

inline uint32_t round4(uint64_t n) { return static_cast<uint32_t>((n + 3) / 4 * 4); }

}  // namespace

bool NcTrajectory::create(const char *path, int natom) {
  close();
  natom_ = natom;
  fp_ = std::fopen(path, "wb+");
  if (!fp_) return false;
  // dimension ids: 0 frame, 1 spatial, 2 atom, 3 cell_spatial, 4 label, 5 cell_angular
  struct Var {
    const char *name;
    std::vector<uint32_t> dims;
    uint32_t type;
    const char *units;
    uint64_t bytes;  // per record for record variables
    bool record;
  };
  const uint64_t coord_bytes = 12ull * static_cast<uint64_t>(natom);
  const Var vars[] = {{"time", {0}, kNcFloat, "picosecond", 4, true},
                      {"spatial", {1}, kNcChar, nullptr, 3, false},
                      {"coordinates", {0, 2, 1}, kNcFloat, "angstrom", coord_bytes, true},
                      {"cell_spatial", {3}, kNcChar, nullptr, 3, false},
                      {"cell_angular", {5, 4}, kNcChar, nullptr, 15, false}};
  // header with placeholder offsets, sized first, then written for real
  auto header = [&](const std::vector<uint64_t> &begin) {
    Out h;
    h.b = {'C', 'D', 'F', 2};
    h.u32(0);  // numrecs
    h.u32(kNcDimension);
    h.u32(6);
    const std::pair<const char *, uint32_t> dims[] = {{"frame", 0},        {"spatial", 3}, {"atom", uint32_t(natom)},
                                                      {"cell_spatial", 3}, {"label", 5},   {"cell_angular", 3}};
    for (const auto &d : dims) {
      h.name(d.first);
      h.u32(d.second);
    }
    h.u32(kNcAttribute);
    h.u32(6);
    h.text_attr("title", "AmberNetcdf trajectory");
    h.text_attr("application", "AMBER");
    h.text_attr("program", "AmberNetcdf");
    h.text_attr("programVersion", "1.0");
    h.text_attr("Conventions", "AMBER");
    h.text_attr("ConventionVersion", "1.0");
    h.u32(kNcVariable);
    h.u32(5);
    for (int k = 0; k < 5; k++) {
      const Var &v = vars[k];
      h.name(v.name);
      h.u32(static_cast<uint32_t>(v.dims.size()));
      for (uint32_t d : v.dims) h.u32(d);
      if (v.units) {
        h.u32(kNcAttribute);
        h.u32(1);
        h.text_attr("units", v.units);
      } else {
        h.u32(0);
        h.u32(0);
      }
      h.u32(v.type);
      h.u32(round4(v.bytes));
      h.u64(begin[k]);
    }
    return h;
  };
  std::vector<uint64_t> begin(5, 0);
  const uint64_t hsize = header(begin).b.size();
  // fixed-size variables in order, then the records (time, coordinates)
  uint64_t off = hsize;
  for (int k = 0; k < 5; k++)
    if (!vars[k].record) {
      begin[k] = off;
      off += round4(vars[k].bytes);
    }
  data_begin_ = off;
  begin[0] = off;
  begin[2] = off + 4;
  record_bytes_ = 4 + round4(coord_bytes);
  Out h = header(begin);
  // fixed data: spatial "xyz", cell_spatial "abc", cell_angular labels
  const char xyz[4] = {'x', 'y', 'z', 0}, abc[4] = {'a', 'b', 'c', 0};
  const char angular[16] = "alphabeta gamma";
  h.b.insert(h.b.end(), xyz, xyz + 4);
  h.b.insert(h.b.end(), abc, abc + 4);
  h.b.insert(h.b.end(), angular, angular + 15);
  h.b.push_back(0);
  frames_ = 0;
  const bool ok = std::fwrite(h.b.data(), 1, h.b.size(), fp_) == h.b.size() && std::fflush(fp_) == 0;
  if (!ok) close();
  return ok;
}

bool NcTrajectory::write_frame(const double *x, double time_ps) {
  if (!fp_) return false;
  Out r;
  r.b.reserve(record_bytes_);
  auto put_float = [&](float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    r.u32(u);
  };
  put_float(static_cast<float>(time_ps));
  for (int i = 0; i < 3 * natom_; i++) put_float(static_cast<float>(x[i]));
  r.pad();
  const uint64_t at = data_begin_ + static_cast<uint64_t>(frames_) * record_bytes_;
  bool ok = std::fseek(fp_, static_cast<long>(at), SEEK_SET) == 0 &&
            std::fwrite(r.b.data(), 1, r.b.size(), fp_) == r.b.size();
  frames_++;
  Out n;
  n.u32(static_cast<uint32_t>(frames_));
  ok = ok && std::fseek(fp_, 4, SEEK_SET) == 0 && std::fwrite(n.b.data(), 1, 4, fp_) == 4 && std::fflush(fp_) == 0;
  return ok;
}

void NcTrajectory::close() {
  if (fp_) std::fclose(fp_);
  fp_ = nullptr;
}

}  // namespace sffg
