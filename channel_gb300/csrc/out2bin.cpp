// out2bin -- the reference's field exporter (out_exporter/out2bin.f90) over
// the C ABI: each restart file named on the command line becomes the raw
// velocity array of its physical-space field, vec(3, nxtot, 0:ny, nztot) of
// float64 in Fortran order, written to <name up to the last dot>.bin
// (write_brutal_bin, :207-232); spatial_grid.nfo gets the grid sizes and
// spacings (write_metadata, :303-323).  dns.in is read from the working
// directory as the reference does.
//
// Usage: out2bin [-h] [-f] [-l | -s | -ls] [-u factor] file.out [file.out ...]
//   -f, --fluctuation   remove the mean mode before transforming
//   -l, --large         also write <name>.large.bin: modes |beta0 kz| <= z_threshold
//   -s, --small         also write <name>.small.bin: modes |beta0 kz| >  z_threshold
//   -ls, -sl, --largesmall, --smalllarge   both
//   -u, --undersample x sample on nint(x (2n+1)) points in x and z
// z_threshold is the first integer of largesmall_settings.in (:327-334).
// Errors (no input, unreadable or mismatching restart file, a failing call)
// exit with status 1; a missing file gives the laminar field of
// read_restart_file (dnsdata.f90:704-718), as in the reference.
#include <chgpu.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hostio.h"

namespace {

using namespace hostio;

constexpr double PI = 3.1415926535897932384626433832795028841971;

void print_help() {
  std::printf(
      " Converts a given .out file from channel into a pure binary velocity array.\n"
      " The binary array is Fourier-antitransformed with respect to the .out file,\n"
      " so that it represents a velocity field in space (and not in the Fourier domain).\n"
      " Syntax:\n"
      "    out2bin [-h] [-f] [-l -s -ls -sl] [-u undersample_xcent] file.name\n"
      " Flag -f (--fluctuation) subtracts the (spatial) average before converting.\n"
      " Flags -l, -s, -ls read the filtering threshold from largesmall_settings.in\n"
      " and write the large- or small-scale field as well.\n"
      " Flag -u undersamples the field: n_new = undersample_xcent * n_old points in x and z.\n");
}

// undersampled_to_fullindex (out2bin.f90:296), the ratio in real*4
double fullindex(int n_full, int n_tot, int i) {
  volatile float s = (float)n_full / (float)n_tot;
  volatile float t = s * ((float)i - 1.0f);
  volatile float r = t + 1.0f;
  return (double)r;
}

std::string bin_name(const std::string& fname, int part) {
  const char* mid = part == CHGPU_EXPORT_LARGE ? "large." : part == CHGPU_EXPORT_SMALL ? "small." : "";
  const size_t k = fname.rfind('.');
  return (k == std::string::npos ? fname + "." : fname.substr(0, k + 1)) + mid + "bin";
}

int fail(chgpu_handle* h, int rc, const char* what) {
  std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, chgpu_last_error(h));
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  bool fluct = false, large = false, small = false;
  float xcent = 1.0f;
  std::vector<std::string> files;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "-f" || a == "--fluctuation") fluct = true;
    else if (a == "-l" || a == "--large") large = true;
    else if (a == "-s" || a == "--small") small = true;
    else if (a == "-ls" || a == "-sl" || a == "--largesmall" || a == "--smalllarge") large = small = true;
    else if (a == "-u" || a == "--undersample") {
      if (++i >= argc) {
        std::fprintf(stderr, "ERROR: -u needs a factor\n");
        return 1;
      }
      xcent = std::strtof(argv[i], nullptr);
    } else if (a == "-h" || a == "--help") {
      print_help();
      return 0;
    } else files.push_back(a);
  }
  if (files.empty()) {
    std::printf(" ERROR: please provide one input file as command line argument.\n");
    return 1;
  }
  int z_threshold = 0;
  if (large || small) {
    std::FILE* f = std::fopen("largesmall_settings.in", "r");
    if (!f || std::fscanf(f, "%d", &z_threshold) != 1) {
      std::fprintf(stderr, "ERROR: cannot read z_threshold from largesmall_settings.in\n");
      if (f) std::fclose(f);
      return 1;
    }
    std::fclose(f);
    std::printf("   z_threshold =%5d\n", z_threshold);
  }
  DnsIn d;
  if (!read_dnsin("dns.in", d)) {
    std::fprintf(stderr, "ERROR: cannot read dns.in\n");
    return 1;
  }
  const chgpu_params& p = d.p;
  chgpu_handle* h = nullptr;
  if (int rc = chgpu_create(&p, &h)) return fail(nullptr, rc, "chgpu_create");
  int dims[3];
  if (int rc = chgpu_export_dims(h, xcent, dims)) return fail(h, rc, "chgpu_export_dims");
  const int nxtot = dims[0], nytot = dims[1], nztot = dims[2];
  std::vector<double> vec((size_t)3 * nxtot * nytot * nztot);
  std::vector<double> V;
  for (const std::string& name : files) {
    double time = 0;
    const int r = read_restart(name, p, V, time);
    if (r == 1) {
      std::printf(" Generating initial field...\n");
      laminar_start(p, V);
    } else if (r == -1) {
      std::fprintf(stderr, "ERROR: cannot read %s\n", name.c_str());
      return 1;
    } else if (r == -2) {
      return 1;
    } else {
      std::printf(" Reading from file %s\n", name.c_str());
    }
    if (int rc = chgpu_upload_field(h, V.data())) return fail(h, rc, "chgpu_upload_field");
    const int parts[3] = {CHGPU_EXPORT_ALL, large ? CHGPU_EXPORT_LARGE : -1, small ? CHGPU_EXPORT_SMALL : -1};
    for (int part : parts) {
      if (part < 0) continue;
      chgpu_export_opts o{fluct ? 1 : 0, part, z_threshold, xcent};
      if (int rc = chgpu_export_physical(h, &o, vec.data())) return fail(h, rc, "chgpu_export_physical");
      const std::string out = bin_name(name, part);
      std::printf(" Writing %s\n", out.c_str());
      std::FILE* f = std::fopen(out.c_str(), "wb");
      if (!f || std::fwrite(vec.data(), sizeof(double), vec.size(), f) != vec.size()) {
        std::fprintf(stderr, "ERROR: cannot write %s\n", out.c_str());
        if (f) std::fclose(f);
        return 1;
      }
      if (std::fclose(f) != 0) return 1;
    }
  }
  // write_metadata (out2bin.f90:303-323)
  const int Nx = 2 * p.nx + 1, Nz = 2 * p.nz + 1;
  const double dx = std::fabs(fullindex(Nx, nxtot, 2) - fullindex(Nx, nxtot, 1)) * 2 * PI / p.alfa0 / Nx;
  const double dz = std::fabs(fullindex(Nz, nztot, 2) - fullindex(Nz, nztot, 1)) * 2 * PI / p.beta0 / Nz;
  std::FILE* f = std::fopen("spatial_grid.nfo", "w");
  if (!f) return 1;
  std::fprintf(f, " %11d %11d %25.17E %25.17E\n", nxtot, nztot, dx, dz);
  std::fprintf(f, " %11d %11d %25.17E %25.17E %25.17E\n", p.ny, p.ny + 1, p.a, p.ymin, p.ymax);
  std::fprintf(f, " # * ~ - ~ * # LEGEND # * ~ - ~ * #\n");
  std::fprintf(f, " nxtot, nztot, dx, dz\n");
  std::fprintf(f, " ny (see dns.in), nytot, a, ymin, ymax, nztot, dx, dz\n");
  std::fclose(f);
  chgpu_destroy(h);
  return 0;
}
