// Host-side files of the reference shared by the driver and the exporter:
// dns.in (read_dnsin, dnsdata.f90:98-125) and the restart file
// (read_restart_file / save_restart_file, dnsdata.f90:677-720, 821-848):
// a 68-byte header (nx, ny, nz as int32; alfa0, beta0, ni, a, ymin, ymax,
// time as float64) then V(-1:ny+1, -nz:nz, 0:nx, 1:3) complex128 in Fortran
// order.
#pragma once

#include <chgpu.h>

#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace hostio {

struct DnsIn {
  chgpu_params p{};
  double re = 0;
};

inline std::string strip_comment(const std::string& s) {
  size_t k = s.find('!');
  return k == std::string::npos ? s : s.substr(0, k);
}

inline double fortran_real(std::string t) {
  for (char& c : t)
    if (c == 'd' || c == 'D') c = 'e';
  return std::strtod(t.c_str(), nullptr);
}

inline bool fortran_logical(std::string t) {
  size_t i = 0;
  while (i < t.size() && t[i] == '.') ++i;
  char c = i < t.size() ? (char)std::toupper((unsigned char)t[i]) : 'F';
  return c == 'T';
}

// list-directed reads: each READ takes the values it needs from the next
// record(s); the rest of the record (the comment) is skipped
inline bool read_dnsin(const char* path, DnsIn& d) {
  std::ifstream f(path);
  if (!f) return false;
  const int need[12] = {3, 2, 1, 3, 3, 2, 2, 2, 3, 4, 1, 1};
  std::vector<std::vector<std::string>> v(12);
  std::string line;
  for (int k = 0; k < 12; ++k) {
    while ((int)v[k].size() < need[k]) {
      if (!std::getline(f, line)) return false;
      std::string s = strip_comment(line);
      for (char& c : s)
        if (c == ',') c = ' ';
      std::istringstream is(s);
      std::string tok;
      while (is >> tok) v[k].push_back(tok);
    }
    v[k].resize(need[k]);
  }
  chgpu_params& p = d.p;
  p.nx = std::atoi(v[0][0].c_str()); p.ny = std::atoi(v[0][1].c_str()); p.nz = std::atoi(v[0][2].c_str());
  p.alfa0 = fortran_real(v[1][0]); p.beta0 = fortran_real(v[1][1]);
  d.re = fortran_real(v[2][0]);
  p.ni = 1 / d.re;  // ni=1/ni (dnsdata.f90:115)
  p.a = fortran_real(v[3][0]); p.ymin = fortran_real(v[3][1]); p.ymax = fortran_real(v[3][2]);
  p.cpi = fortran_logical(v[4][0]); p.cpi_type = std::atoi(v[4][1].c_str()); p.gamma = fortran_real(v[4][2]);
  p.meanpx = fortran_real(v[5][0]); p.meanpz = fortran_real(v[5][1]);
  p.meanflowx = fortran_real(v[6][0]); p.meanflowz = fortran_real(v[6][1]);
  p.u0 = fortran_real(v[7][0]); p.uN = fortran_real(v[7][1]);
  p.deltat = fortran_real(v[8][0]); p.cflmax = fortran_real(v[8][1]); p.time = fortran_real(v[8][2]);
  p.dt_field = fortran_real(v[9][0]); p.dt_save = fortran_real(v[9][1]); p.t_max = fortran_real(v[9][2]);
  p.time_from_restart = fortran_logical(v[9][3]);
  p.nstep = std::atoll(v[10][0].c_str());
  p.npy = std::atoi(v[11][0].c_str());
  return true;
}

#pragma pack(push, 1)
struct Header {
  int32_t nx, ny, nz;
  double alfa0, beta0, ni, a, ymin, ymax, time;
};
#pragma pack(pop)
static_assert(sizeof(Header) == 68, "restart header is 68 bytes");

inline size_t field_count(const chgpu_params& p) { return (size_t)3 * (p.nx + 1) * (2 * p.nz + 1) * (p.ny + 3); }

inline bool write_restart(const std::string& path, const chgpu_params& p, double time, const double* V, size_t n) {
  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  Header h{p.nx, p.ny, p.nz, p.alfa0, p.beta0, p.ni, p.a, p.ymin, p.ymax, time};
  bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 && std::fwrite(V, sizeof(double), n, f) == n;
  return std::fclose(f) == 0 && ok;
}

// 0: read; 1: absent; -1: unreadable; -2: metadata mismatch
inline int read_restart(const std::string& path, const chgpu_params& p, std::vector<double>& V, double& time) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return 1;
  Header h{};
  if (std::fread(&h, sizeof h, 1, f) != 1) { std::fclose(f); return -1; }
  if (h.nx != p.nx || h.ny != p.ny || h.nz != p.nz || h.alfa0 != p.alfa0 || h.beta0 != p.beta0 || h.ni != p.ni ||
      h.a != p.a || h.ymin != p.ymin || h.ymax != p.ymax) {
    std::fprintf(stderr, "ERROR: mismatch in metadata between restart file and dns.in. Stopping.\n"
                         "From .out file:\n %d %d %d %.17g %.17g %.17g %.17g %.17g %.17g\nFrom dns.in:\n"
                         " %d %d %d %.17g %.17g %.17g %.17g %.17g %.17g\n",
                 h.nx, h.ny, h.nz, h.alfa0, h.beta0, h.ni, h.a, h.ymin, h.ymax, p.nx, p.ny, p.nz, p.alfa0, p.beta0,
                 p.ni, p.a, p.ymin, p.ymax);
    std::fclose(f);
    return -2;
  }
  V.assign(2 * field_count(p), 0.0);
  size_t got = std::fread(V.data(), sizeof(double), V.size(), f);
  std::fclose(f);
  if (got != V.size()) return -1;
  time = h.time;
  return 0;
}

// the laminar start of read_restart_file when no file exists (dnsdata.f90:704-718)
inline void laminar_start(const chgpu_params& p, std::vector<double>& V) {
  V.assign(2 * field_count(p), 0.0);
  const int nyt = p.ny + 3, nzt = 2 * p.nz + 1;
  for (int iy = -1; iy <= p.ny + 1; ++iy) {
    double y = p.ymin + 0.5 * (p.ymax - p.ymin) * (std::tanh(p.a * (2.0 * iy / (double)p.ny - 1)) / std::tanh(p.a) + 1);
    size_t idx = (size_t)(iy + 1) + (size_t)nyt * (size_t)p.nz;  // iz=0, ix=0, ic=1
    V[2 * idx] = 3 * 0.5 * y * (2 - y);
  }
  (void)nzt;
}

}  // namespace hostio
