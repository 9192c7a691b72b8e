// Host-side case setup for the GB300 SIMPLE-TS step: everything the reference's
// main() does before its time loop that is not array arithmetic (configuration,
// bodies, mesh, obstacle masks, solve ranges, per-cell classes, wall lists).
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "sts_common.cuh"

namespace sts {

// One EnteredData.txt field.  kind: 'd' double, 'u' unsigned, 'i' int, 'b' bool.
struct FieldDef {
  const char* name;
  char kind;
};
extern const FieldDef kEnteredData[126];

struct Config {
  std::map<std::string, double> v;  // every field, as read
  double d(const char* k) const;
  long n(const char* k) const { return (long)d(k); }
  bool b(const char* k) const { return d(k) != 0; }
  void set(const char* k, double x) { v[k] = x; }
};

// Parses EnteredData.txt with the reference's positional rule (SIMPLE_TS_MPI.cpp:5241-5561):
// one extraction per field in order, rest of the line discarded.
bool read_config(const std::string& path, Config& cfg, std::string& err);
bool write_config(const std::string& path, const Config& cfg);

struct HostBody {
  bool circle = false;
  double xc = 1, yc = 1, rc = 1;
  std::vector<double> xs, ys;
  double p1x = 0, p1y = 0, p2x = 1, p2y = 1;
  Body dev{};  // properties used on the device
  double w_slip = 0.1;
  bool drag = false;
};

// Objects_for_Solving::Import_data_for_circles_from_file / _for_polyhedrons_ (Objects_for_Solving.h:101-412)
bool read_bodies(const std::string& path, bool circles, std::vector<HostBody>& out, std::string& err);

// Test of a cell centre against a body (Polyhedrons_Objects.cpp:190-324, Circles_Objects.h:118-126).
bool body_contains(const HostBody& b, double x, double y);

struct Case {
  std::string dir;
  Config cfg;
  int Nx = 0, Ny = 0, Na = 0;
  bool periodic = false, restart = false;
  std::vector<double> hx, hy, x_v, y_v, x_f, y_f;
  std::vector<HostBody> bodies;  // circles first, then polygons: id k+1 is bodies[k]
  int n_circles = 0;
  std::vector<uint32_t> vol_id;  // vol_inf_fb as computed from the bodies
  std::vector<uint8_t> cls;
  int Nx_u[2], Ny_u[2], Nx_v[2], Ny_v[2], Nx_o[2], Ny_o[2];
  // wall lists in the reference's order with the surviving-write flags
  std::vector<int> slip_u, slip_v, tjump;
  std::vector<uint8_t> slip_u_fin, slip_v_fin, tjump_fin, tjump_wr_fin;
  // initial fields (host copies, uploaded once)
  std::vector<double> u, v, p, T, rho;
  std::vector<uint32_t> vol_file;  // vol_inf_fb as read from a restart (what the reference keeps)
  double it_begin = 0;
  // scalars
  double cT = 0, cPch = 0.5, cT1 = 0, cT2 = 0, c_Fr_v = 0, u_given_xb = 0, u_given_xb_in_it = 0;
  double p_BC_xb = 0, p_BC_xe = 0;
  uint64_t bits = 0;
};

// Reads a case directory and builds everything up to the first device operation.
bool load_case(const std::string& dir, bool fixed_sweeps, Case& c, std::string& err);

}  // namespace sts
