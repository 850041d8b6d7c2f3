// channel_gb300 -- the channel DNS driver on top of libchgpu.so.
//
// Restates the program flow of channel.f90 (the reference's Fortran driver,
// which needs gfortran + MPI to build) in C++ over the C ABI of
// include/chgpu.h, keeping its files:
//   dns.in        read as read_dnsin does (dnsdata.f90:98-125)
//   Dati.cart.out read (header check, dnsdata.f90:677-720) or, when absent,
//                 the laminar start of dnsdata.f90:704-718; rewritten at the
//                 end (channel.f90:181) and every dt_save (dnsdata.f90:882-886)
//   Dati.cart.<n>.out  snapshots every dt_field (dnsdata.f90:895-918)
//   Runtimedata   one line per step (dnsdata.f90:878), rewound to the restart
//                 time when time_from_restart (get_record, dnsdata.f90:181-218)
// Usage: channel_gb300 [--mixed | --fp64dd] [--quiet] [--no-tune]   (in the run
// directory; --no-tune keeps the default transform tiles instead of timing them)
#include <chgpu.h>

#include "hostio.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace {

using namespace hostio;

std::string fmt_line(const double* v) {  // one Runtimedata record
  std::string s;
  char buf[40];
  for (int i = 0; i < 11; ++i) {
    std::snprintf(buf, sizeof buf, " %25.16E", v[i]);
    s += buf;
  }
  return s + "\n";
}

void echo_line(const double* v) {  // dnsdata.f90:876
  std::printf("%10.4f   ", v[0]);
  for (int i = 1; i <= 4; ++i) std::printf("%11.6f   ", v[i]);
  for (int i = 5; i <= 8; ++i) std::printf("%9.4f   ", v[i]);
  for (int i = 9; i <= 10; ++i) std::printf("%9.6f   ", v[i]);
  std::printf("\n");
  std::fflush(stdout);
}

// get_record (dnsdata.f90:181-218): keep the records before the one whose
// time matches the restart time; returns that record's deltat (or 0).
double rewind_runtimedata(const char* path, double threshold, bool& found) {
  found = false;
  std::ifstream f(path);
  if (!f) return 0.0;
  std::vector<std::string> keep;
  std::string line;
  double dt = 0.0;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    double v[11];
    int n = 0;
    while (n < 11 && (is >> v[n])) ++n;
    if (n == 11 && std::fabs(v[0] - threshold) < 0.5 * v[10]) {
      found = true;
      dt = v[10];
      break;
    }
    keep.push_back(line);
  }
  f.close();
  std::ofstream o(path, std::ios::trunc);
  for (auto& l : keep) o << l << "\n";
  if (!found) o << "\n";  // "Skipping one line and appending."
  return dt;
}

int check(int rc, chgpu_handle* h, const char* what) {
  if (rc != 0) {
    std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, chgpu_last_error(h));
    std::exit(1);
  }
  return rc;
}

}  // namespace

int main(int argc, char** argv) {
  bool quiet = false, tune = true;
  int precision = CHGPU_FP64;
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--mixed")) precision = CHGPU_MIXED;
    else if (!std::strcmp(argv[i], "--fp64dd")) precision = CHGPU_FP64DD;
    else if (!std::strcmp(argv[i], "--quiet")) quiet = true;
    else if (!std::strcmp(argv[i], "--no-tune")) tune = false;
    else {
      std::fprintf(stderr, "usage: %s [--mixed | --fp64dd] [--quiet] [--no-tune]\n", argv[0]);
      return 2;
    }
  }
  const bool mixed = precision == CHGPU_MIXED;
  DnsIn d;
  if (!read_dnsin("dns.in", d)) {
    std::fprintf(stderr, "cannot read dns.in\n");
    return 1;
  }
  const double deltat_from_dnsin = d.p.deltat;
  d.p.precision = precision;
  chgpu_handle* h = nullptr;
  check(chgpu_create(&d.p, &h), nullptr, "chgpu_create");
  if (tune) check(chgpu_autotune(h), h, "chgpu_autotune");  // transform tiles; results do not depend on them
  chgpu_params& p = d.p;
  std::vector<double> V;
  double time = p.time;
  int rr = read_restart("Dati.cart.out", p, V, time);
  if (rr == -2) return 1;
  if (rr == -1) {
    std::fprintf(stderr, "Dati.cart.out is truncated or unreadable\n");
    return 1;
  }
  if (rr == 1) {
    std::printf(" Generating initial field...\n");
    laminar_start(p, V);
    time = p.time;
  } else {
    std::printf(" Reading from file Dati.cart.out\n");
  }
  bool have_rtd = std::ifstream("Runtimedata").good();
  double deltat = p.deltat;
  if (p.time_from_restart && have_rtd) {
    bool found = false;
    double dt = rewind_runtimedata("Runtimedata", time, found);
    if (found) {
      std::printf(" In Runtimedata: starting from time %g\n", time);
      deltat = dt;
    } else {
      std::printf(" WARNING: No instant of time matching restart file has been found in Runtimedata.\n"
                  " Skipping one line and appending.\n");
    }
  } else if (!p.time_from_restart) {
    time = p.time;  // read_dnsin again (channel.f90:57)
    deltat = p.deltat;
  }
  std::ofstream rtd("Runtimedata", (p.time_from_restart && have_rtd) ? std::ios::app : std::ios::trunc);
  long long ifield = (long long)std::floor((time + 0.5 * deltat) / p.dt_field);
  const double time0 = time;
  if (p.cflmax == 0) deltat = deltat_from_dnsin;
  int nxd = 3 * (p.nx + 1) / 2, nzd = 3 * p.nz;
  auto fit = [](int n) { while (n % 2 == 0) n >>= 1; return n == 1 || n == 3; };
  while (!fit(nxd)) ++nxd;
  while (!fit(nzd)) ++nzd;
  if (!quiet) {
    std::printf("\n !====================================================!\n"
                " !                     D   N   S                      !\n"
                " !====================================================!\n\n");
    std::printf("   nx =%5d   ny =%5d   nz =%5d\n   nxd =%5d  nzd =%5d\n", p.nx, p.ny, p.nz, nxd, nzd);
    std::printf("   alfa0 =%11.6f       beta0 =%11.6f   ni =%8.6f\n", p.alfa0, p.beta0, p.ni);
    std::printf("   meanpx =%11.6f      meanpz =%11.6f\n", p.meanpx, p.meanpz);
    std::printf("   meanflowx =%11.6f   meanflowz =%11.6f\n", p.meanflowx, p.meanflowz);
    std::printf("   nsteps =%6lld   time_from_restart =%c   precision = %s\n\n", p.nstep,
                p.time_from_restart ? 'T' : 'F', mixed ? "mixed" : (precision == CHGPU_FP64DD ? "fp64dd" : "fp64"));
  }
  check(chgpu_upload_field(h, V.data()), h, "upload");
  chgpu_stats st{};
  check(chgpu_start(h, time, deltat, &st), h, "start");
  check(chgpu_set_wall_velocity(h, p.u0, p.uN), h, "wall velocity");
  rtd << fmt_line(st.line);
  rtd.flush();
  if (!quiet) echo_line(st.line);
  bool prev_was_close = false;
  long long istep = 0;
  deltat = st.deltat;
  time = st.time;
  // Snapshots leave the device while later steps run: the field is copied
  // to a pinned buffer on a side stream (chgpu_snapshot_async), collected
  // after the next step and written by a thread.
  std::thread writer;
  std::vector<std::string> pend_names;
  double pend_time = 0.0;
  bool pending = false;
  auto collect = [&]() {
    if (!pending) return;
    const double* Vh = nullptr;
    check(chgpu_snapshot_wait(h, &Vh), h, "snapshot");
    if (writer.joinable()) writer.join();
    writer = std::thread([&p, names = pend_names, pend_time, Vh, n = V.size()]() {
      for (const auto& nm : names) write_restart(nm, p, pend_time, Vh, n);
    });
    pending = false;
  };
  while (time < p.t_max - deltat / 2.0 && istep < p.nstep) {
    check(chgpu_step(h, &st), h, "step");
    collect();  // the snapshot of the previous step has arrived by now
    istep = st.istep;
    time = st.time;
    deltat = st.deltat;
    rtd << fmt_line(st.line);
    rtd.flush();
    if (!quiet) echo_line(st.line);
    // restart and snapshot cadence (dnsdata.f90:882-918)
    std::vector<std::string> names;
    if (p.dt_save > 0 && std::floor((time + 0.5 * deltat) / p.dt_save) > std::floor((time - 0.5 * deltat) / p.dt_save) &&
        istep > 1) {
      std::printf(" Writing Dati.cart.out at time %g\n", time);
      names.push_back("Dati.cart.out");
    }
    if (time + deltat >= (ifield + 1) * p.dt_field) {
      if (prev_was_close || (std::floor((time + 0.5 * deltat) / p.dt_field) >
                                 std::floor((time - 0.5 * deltat) / p.dt_field) &&
                             time > time0)) {
        ++ifield;
        std::string name = "Dati.cart." + std::to_string(ifield) + ".out";
        std::printf(" Writing %s at time %g\n", name.c_str(), time);
        names.push_back(name);
        prev_was_close = false;
      } else {
        prev_was_close = true;
      }
    }
    if (!names.empty()) {
      if (writer.joinable()) writer.join();  // the library's snapshot buffer is free again
      check(chgpu_snapshot_async(h), h, "snapshot");
      pend_names = names;
      pend_time = time;
      pending = true;
    }
  }
  collect();
  if (writer.joinable()) writer.join();
  std::printf(" End of time/iterations loop: writing restart file at time %g\n", time);
  check(chgpu_download_field(h, V.data()), h, "download");
  write_restart("Dati.cart.out", p, time, V.data(), V.size());
  chgpu_destroy(h);
  return 0;
}
