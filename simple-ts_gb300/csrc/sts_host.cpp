// Host-side case setup for the GB300 SIMPLE-TS step.  Compiled with
// -ffp-contract=off so the setup arithmetic (mesh, masks) rounds like the
// reference on both x86 and Arm hosts.
#include "sts_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>

namespace sts {

// Field order of EnteredData.txt (SIMPLE_TS_MPI.cpp:5253-5544) with the C++ type each is read into.
const FieldDef kEnteredData[126] = {
    {"u_gas_nd", 'd'}, {"v_gas_nd", 'd'}, {"T_gas_nd", 'd'}, {"p_gas_nd", 'd'}, {"Ma", 'd'}, {"Pr", 'd'},
    {"gamma1", 'd'}, {"c_mu", 'd'}, {"Kn", 'd'}, {"Fr", 'd'}, {"SolveGravityField", 'b'}, {"Re", 'd'},
    {"TypeOfNonDimensiolization", 'u'}, {"Nt", 'd'}, {"Nx", 'u'}, {"Ny", 'u'}, {"N_I", 'u'}, {"N_I_p_c", 'u'},
    {"N_I_T", 'u'}, {"ht", 'd'}, {"x_b", 'd'}, {"x_e", 'd'}, {"y_b", 'd'}, {"y_e", 'd'}, {"kind_of_mesh", 'u'},
    {"hxmin", 'd'}, {"hxmax", 'd'}, {"xfmin", 'd'}, {"xfmax", 'd'}, {"xbmin", 'd'}, {"xbmax", 'd'}, {"xmid", 'd'},
    {"hymin", 'd'}, {"hymax", 'd'}, {"ytmin", 'd'}, {"ytmax", 'd'}, {"ybmin", 'd'}, {"ybmax", 'd'}, {"ymid", 'd'},
    {"MaxError_Velocities", 'd'}, {"MaxError_p_c", 'd'}, {"MaxError_T", 'd'}, {"MaxError_to_stop_program", 'd'},
    {"max_time_for_solve", 'd'}, {"solve_is_finished", 'b'}, {"Nt_save_solved_data", 'i'},
    {"Nt_save_DragCoefficient", 'u'}, {"Nt_save_temp_data", 'i'}, {"N_I_check", 'i'},
    {"WriteDataInShortFormat_kind", 'i'}, {"ToReadSolvedDataFromFile", 'b'}, {"ToReadSolvedDataFromBinaryFile", 'b'},
    {"ToWriteSolvedDataToBinaryFile", 'b'}, {"ToWriteSolvedDataToNewFiles", 'b'}, {"ToContinueFromInterpolation", 'b'},
    {"ToImport_data_for_circles_from_file_b", 'b'}, {"ToImport_data_for_polyhedrons_from_file_b", 'b'},
    {"ToImport_data_for_circles_from_file_p", 'b'}, {"ToImport_data_for_polyhedrons_from_file_p", 'b'},
    {"ToImport_data_for_circles_from_file_V", 'b'}, {"ToImport_data_for_polyhedrons_from_file_V", 'b'},
    {"Given_velocity_on_xb", 'b'}, {"Given_velocity_on_xe", 'b'}, {"Periodic_boundary_conditions_about_OX", 'b'},
    {"Pressure_BC", 'b'}, {"ToStartFromExactSolutionForChannelFlowWithPressureBC", 'b'},
    {"p_BC_xb_correction_method", 'u'}, {"Pressure_ratio_correct", 'b'}, {"GivenReKn", 'b'}, {"correct_p_BC_xb", 'b'},
    {"u_given_xb", 'd'}, {"u_given_xb_error", 'd'}, {"p_correction_auto", 'b'}, {"p_correction_min", 'd'},
    {"p_correction_max", 'd'}, {"p_correction", 'd'}, {"p_BC_xb", 'd'}, {"T_BC_xb", 'd'}, {"p_BC_xe", 'd'},
    {"T_BC_xe", 'd'}, {"dudx_0_BC_xb", 'b'}, {"durhodx_0_BC_xb", 'b'}, {"drhodt_durhodx_dvrhody_0_BC_xb", 'b'},
    {"ToCalculate_ui_1j_from_equation_for_uij_at_x_b", 'b'}, {"dudx_0_BC_xe", 'b'}, {"durhodx_0_BC_xe", 'b'},
    {"drhodt_durhodx_dvrhody_0_BC_xe", 'b'}, {"ToCalculate_ui1j_from_equation_for_uij_at_x_e", 'b'},
    {"u_uMin_Mout_0_BC_xe", 'b'}, {"dudy_0_BC_yb", 'b'}, {"dudy_0_BC_ye", 'b'}, {"dvdx_0_BC_xb", 'b'},
    {"ToCalculate_vi_1j_from_equation_for_vij_at_x_b", 'b'}, {"dvdx_0_BC_xe", 'b'},
    {"ToCalculate_vi1j_from_equation_for_vij_at_x_e", 'b'}, {"dvdy_0_BC_yb", 'b'}, {"dvdy_0_BC_ye", 'b'},
    {"dpdx_0_BC_xb", 'b'}, {"ToCalculate_pi_1j_from_equation_for_pij_at_x_b", 'b'}, {"dpdx_0_BC_xe", 'b'},
    {"ToCalculate_pi1j_from_equation_for_pij_at_x_e", 'b'}, {"dpdy_0_BC_yb", 'b'}, {"dpdy_0_BC_ye", 'b'},
    {"dTdx_0_BC_xb", 'b'}, {"ToCalculate_Temperi_1j_from_equation_for_Temperij_at_x_b", 'b'}, {"dTdx_0_BC_xe", 'b'},
    {"ToCalculate_Temperi1j_from_equation_for_Temperij_at_x_e", 'b'}, {"dTdy_0_BC_yb", 'b'}, {"dTdy_0_BC_ye", 'b'},
    {"To_Use_Kn_local_in_wall_BC", 'b'}, {"ToSolveContinuityEquation", 'b'}, {"use_interpolation_for_u_BC_by_time", 'b'},
    {"t_BC_b", 'd'}, {"t_BC_e", 'd'}, {"u_BC_xb_t_BC_b", 'd'}, {"u_BC_xb_t_BC_e", 'd'}, {"w_u", 'd'}, {"w_v", 'd'},
    {"w_p", 'd'}, {"w_Temper", 'd'}, {"N_SubDomains_x", 'u'}, {"N_SubDomains_y", 'u'},
    {"ToReadSolvedDataFromSeparateFileForEachSubDomain", 'b'},
    {"ToWriteSolvedDataToFileForEntireComputationalDomain", 'b'},
    {"ToWriteSolvedDataToSeparateFileForEachSubDomain", 'b'}, {"ToOnlyWriteDataFor_Nx_Ny_ForAllSubDomains_AndExit", 'b'},
};

double Config::d(const char* k) const {
  auto it = v.find(k);
  return it == v.end() ? 0.0 : it->second;
}

namespace {

void skip_line(std::istream& in) {
  char buf[5000];
  in.getline(buf, sizeof buf, '\n');
  if (in.fail() && !in.bad() && !in.eof()) in.clear();  // over-long comment: keep going like the reference
}

}  // namespace

bool read_config(const std::string& path, Config& cfg, std::string& err) {
  std::ifstream in(path.c_str());
  if (!in.is_open()) {
    err = "cannot open " + path;
    return false;
  }
  for (const FieldDef& f : kEnteredData) {
    double x = 0;
    if (f.kind == 'd') {
      in >> x;
    } else if (f.kind == 'u') {
      unsigned int t = 0;
      in >> t;
      x = t;
    } else if (f.kind == 'i') {
      int t = 0;
      in >> t;
      x = t;
    } else {
      bool t = false;
      in >> t;
      x = t ? 1 : 0;
    }
    if (in.fail()) {
      err = std::string("EnteredData.txt: cannot read field ") + f.name;
      return false;
    }
    cfg.v[f.name] = x;
    skip_line(in);
  }
  return true;
}

bool write_config(const std::string& path, const Config& cfg) {
  std::ofstream o(path.c_str());
  if (!o.is_open()) return false;
  o << std::setprecision(15);
  for (const FieldDef& f : kEnteredData) {
    const double x = cfg.d(f.name);
    if (f.kind == 'd') o << x;
    else if (f.kind == 'i') o << (int)x;
    else o << (unsigned long)x;
    o << "\t//" << f.name << "\n";
  }
  return true;
}

bool read_bodies(const std::string& path, bool circles, std::vector<HostBody>& out, std::string& err) {
  std::ifstream in(path.c_str());
  if (!in.is_open()) {
    err = "cannot open " + path;
    return false;
  }
  unsigned n = 0;
  in >> n;
  skip_line(in);
  for (unsigned k = 0; k < n; k++) {
    HostBody b;
    b.circle = circles;
    // constructor defaults (Polyhedrons_Objects.cpp:39-67, Circles_Objects.cpp:29-50)
    b.dev.u = b.dev.v = b.dev.p = 0;
    b.dev.T = circles ? 1.0 : 0.0;
    b.dev.F_slip = 1.1466;
    b.dev.F_jump = 2.1904;
    b.dev.dTdn0 = 0;
    bool slip = false, jump = false;
    if (circles) {
      in >> b.xc >> b.yc >> b.rc;
      skip_line(in);
    } else {
      unsigned nv = 0;
      in >> nv;
      skip_line(in);
      in >> b.p1x >> b.p1y;
      skip_line(in);
      in >> b.p2x >> b.p2y;
      skip_line(in);
      b.xs.resize(nv);
      b.ys.resize(nv);
    }
    in >> b.dev.u >> b.dev.v;
    skip_line(in);
    in >> b.dev.p; skip_line(in);
    in >> b.dev.T; skip_line(in);
    in >> slip; skip_line(in);
    in >> b.dev.F_slip; skip_line(in);
    in >> b.w_slip; skip_line(in);
    in >> jump; skip_line(in);
    in >> b.dev.F_jump; skip_line(in);
    in >> b.dev.dTdn0; skip_line(in);
    in >> b.drag; skip_line(in);
    for (size_t q = 0; q < b.xs.size(); q++) in >> b.xs[q] >> b.ys[q];
    if (in.fail()) {
      err = "malformed body file " + path;
      return false;
    }
    b.dev.slip = slip;
    b.dev.jump = jump;
    out.push_back(b);
  }
  return true;
}

namespace {

inline double lo(double a, double b) { return a < b ? a : b; }
inline double hi(double a, double b) { return a > b ? a : b; }

// Whether segment (x11,y11)-(x12,y12) meets segment (x21,y21)-(x22,y22); the slope/intercept
// construction and its special cases follow Polyhedrons_Objects.cpp:327-501.
bool segments_meet(double x11, double y11, double x12, double y12, double x21, double y21, double x22, double y22) {
  const double ax0 = lo(x11, x12), ax1 = hi(x11, x12), ay0 = lo(y11, y12), ay1 = hi(y11, y12);
  const double bx0 = lo(x21, x22), bx1 = hi(x21, x22), by0 = lo(y21, y22), by1 = hi(y21, y22);
  const bool a_flat = ay0 == ay1, a_vert = ax0 == ax1, b_flat = by0 == by1, b_vert = bx0 == bx1;
  const bool a_slant = !a_vert && !a_flat, b_slant = !b_vert && !b_flat;
  double xi = 0, yi = 0;
  bool hit = false;
  if (a_slant && b_slant) {
    const double k1 = (y11 - y12) / (x11 - x12), c1 = y11 - k1 * x11;
    const double k2 = (y21 - y22) / (x21 - x22), c2 = y21 - k2 * x21;
    if (k1 != k2) {
      xi = (c1 - c2) / (k2 - k1);
      yi = k1 * xi + c1;
      hit = true;
    }
  } else if (a_flat && b_vert) {
    xi = bx0; yi = ay0; hit = true;
  } else if (a_flat && b_slant) {
    yi = ay0;
    const double k2 = (y21 - y22) / (x21 - x22), c2 = y21 - k2 * x21;
    xi = (yi - c2) / k2;
    hit = true;
  } else if (a_vert && b_flat) {
    xi = ax0; yi = by0; hit = true;
  } else if (a_vert && b_slant) {
    xi = ax0;
    const double k2 = (y21 - y22) / (x21 - x22), c2 = y21 - k2 * x21;
    yi = k2 * xi + c2;
    hit = true;
  } else if (a_slant && b_vert) {
    xi = bx0;
    const double k1 = (y11 - y12) / (x11 - x12), c1 = y11 - k1 * x11;
    yi = k1 * xi + c1;
    hit = true;
  } else if (a_slant && b_flat) {
    yi = by0;
    const double k1 = (y11 - y12) / (x11 - x12), c1 = y11 - k1 * x11;
    xi = (yi - c1) / k1;
    hit = true;
  }
  return hit && ax0 <= xi && xi <= ax1 && bx0 <= xi && xi <= bx1 && ay0 <= yi && yi <= ay1 && by0 <= yi && yi <= by1;
}

// Parity of the crossings between the cell centre and a point inside the polygon
// (Polyhedrons_Objects.cpp:190-324).  The inside point walks along the segment between
// the two given inside points until it is not degenerate with respect to (x, y).
bool polygon_contains(const HostBody& b, double x, double y) {
  const size_t n = b.xs.size();
  const double bx0 = *std::min_element(b.xs.begin(), b.xs.end()), bx1 = *std::max_element(b.xs.begin(), b.xs.end());
  const double by0 = *std::min_element(b.ys.begin(), b.ys.end()), by1 = *std::max_element(b.ys.begin(), b.ys.end());
  if (!(bx0 <= x && x <= bx1 && by0 <= y && y <= by1)) return false;
  const double px0 = lo(b.p1x, b.p2x), px1 = hi(b.p1x, b.p2x), py0 = lo(b.p1y, b.p2y), py1 = hi(b.p1y, b.p2y);
  double k = 0, c = 0;
  if (px0 != px1 && py0 != py1) {
    k = (b.p2y - b.p1y) / (b.p2x - b.p1x);
    c = b.p1y - k * b.p1x;
  }
  double qx = 0, qy = 0;
  bool degenerate = true;
  for (unsigned div = 1; degenerate && div < 5000; div++) {
    if (px0 == px1) {
      qx = px0;
      qy = py0 + (py1 - py0) / div;
    } else if (py0 == py1) {
      qx = px0 + (px1 - px0) / div;
      qy = py0;
    } else {
      qx = px0 + (px1 - px0) / div;
      qy = k * qx + c;
    }
    degenerate = (qx == x && qy == y);
    for (size_t q = 0; !degenerate && q < n; q++) {
      degenerate = (qx == x && x == b.xs[q]) || (qy == y && y == b.ys[q]) ||
                   (b.ys[q] == (qy - y) * (b.xs[q] - qx) / (qx - x) + qy);
    }
  }
  if (degenerate) return true;  // no usable inside point: the reference keeps its bounding-box answer
  double crossings = 0;
  for (size_t q = 0; q < n; q++) {
    const size_t r = (q + 1 < n) ? q + 1 : 0;
    crossings = crossings + segments_meet(qx, qy, x, y, b.xs[q], b.ys[q], b.xs[r], b.ys[r]);
  }
  return (crossings / 2.0) == std::floor(crossings / 2.0);
}

// Mesh step functions (SIMPLE_TS_MPI.cpp:4736-4952) for one axis.
struct Axis {
  int kind;
  double hmin, hmax, fmin, fmax, bmin, bmax, mid, hmid;
  double f0 = 0, f1 = 0, f2 = 0, f3 = 0, b0 = 0, b1 = 0, b2 = 0, b3 = 0;
  bool y_axis;
  double step(double x) const {
    double h;
    // the y axis names its bounds differently (bottom/top) but has the same shape
    const double front = fmax, frontin = fmin, backin = bmin, back = bmax;
    auto poly_f = [&](double t) { return f0 + f1 * t + f2 * t * t; };
    auto poly_f3 = [&](double t) { return f0 + f1 * t + f2 * t * t + f3 * t * t * t; };
    auto poly_b = [&](double t) { return b0 + b1 * t + b2 * t * t + b3 * t * t * t; };
    auto poly_b2 = [&](double t) { return b0 + b1 * t + b2 * t * t; };
    if (x < front) {
      h = hmax;
    } else if (kind == 1) {
      if (x <= frontin) h = ((hmin - hmax) / (frontin - front)) * (x - front) + hmax;
      else if (x <= mid) h = ((hmid - hmin) / (mid - frontin)) * (x - frontin) + hmin;
      else if (x <= backin) h = ((hmin - hmid) / (backin - mid)) * (x - mid) + hmid;
      else if (x <= back) h = ((hmax - hmin) / (back - backin)) * (x - backin) + hmin;
      else h = hmax;
    } else if (kind == 2) {
      if (x <= mid) h = poly_f(x);
      else if (x <= back) h = y_axis ? poly_b2(x) : poly_b(x);
      else h = hmax;
    } else if (kind == 3) {
      if (x <= frontin) h = ((hmin - hmax) / (frontin - front)) * (x - front) + hmax;
      else if (x <= backin) h = hmin;
      else if (x <= back) h = ((hmax - hmin) / (back - backin)) * (x - backin) + hmin;
      else h = hmax;
    } else if (kind == 4) {
      if (x <= frontin) h = poly_f(x);
      else if (x <= backin) h = hmin;
      else if (x <= back) h = y_axis ? poly_b2(x) : poly_b(x);
      else h = hmax;
    } else {
      if (x <= frontin) h = poly_f3(x);
      else if (x <= backin) h = hmin;
      else if (x <= back) h = poly_b(x);
      else h = hmax;
    }
    if (hmax < h) h = hmax;
    else if (h < hmin) h = hmin;
    return h;
  }
};

// Coefficients of the polynomial meshes (SIMPLE_TS_MPI.cpp:2078-2148).  For the y axis the
// "front" side is the bottom and the "back" side the top.  The cubic y coefficients use the
// x step limits, as the reference does.
void axis_coefficients(Axis& a, double hxmin, double hxmax) {
  if (a.kind == 2 || a.kind == 4) {
    a.mid = a.fmin + 0.5 * (a.bmin - a.fmin);
    a.f2 = (a.hmax - a.hmin) / ((a.fmax - a.fmin) * (a.fmax - a.fmin));
    a.f1 = -2.0 * a.f2 * a.fmin;
    a.f0 = a.hmin + a.f2 * a.fmin * a.fmin;
    a.b2 = (a.hmax - a.hmin) / ((a.bmax - a.bmin) * (a.bmax - a.bmin));
    a.b1 = -2.0 * a.b2 * a.bmin;
    a.b0 = a.hmin + a.b2 * a.bmin * a.bmin;
    // hmid from the parabolic branch (the par mesh evaluates it for both kinds)
    const double x = a.mid;
    if (x < a.fmax) a.hmid = a.hmax;
    else if (x <= a.mid) a.hmid = a.f0 + a.f1 * x + a.f2 * x * x;
    else if (x <= a.bmax) a.hmid = a.b0 + a.b1 * x + a.b2 * x * x + (a.y_axis ? 0.0 : a.b3 * x * x * x);
    else a.hmid = a.hmax;
  } else if (a.kind == 5) {
    const double F = a.fmax, f = a.fmin, Bn = a.bmin, Bx = a.bmax;
    const double lo_h = a.y_axis ? hxmin : a.hmin, hi_h = a.y_axis ? hxmax : a.hmax;
    double t = 1.0 / (3.0 * F * std::pow(f, 2) - std::pow(f, 3) - 3.0 * std::pow(F, 2) * f + std::pow(F, 3));
    a.f3 = 2.0 * (lo_h - hi_h) * t;
    a.f2 = -3.0 * (F + f) * (lo_h - hi_h) * t;
    a.f1 = 6.0 * f * F * (lo_h - hi_h) * t;
    a.f0 = (-3.0 * lo_h * std::pow(F, 2) * f + lo_h * std::pow(F, 3) + 3.0 * hi_h * std::pow(f, 2) * F -
            hi_h * std::pow(f, 3)) * t;
    t = 1.0 / (3.0 * Bn * std::pow(Bx, 2) - std::pow(Bx, 3) - 3.0 * std::pow(Bn, 2) * Bx + std::pow(Bn, 3));
    a.b3 = 2.0 * (hi_h - lo_h) * t;
    a.b2 = -3.0 * (Bn + Bx) * (hi_h - lo_h) * t;
    a.b1 = 6.0 * Bx * Bn * (hi_h - lo_h) * t;
    a.b0 = (-3.0 * hi_h * std::pow(Bn, 2) * Bx + hi_h * std::pow(Bn, 3) + 3.0 * lo_h * std::pow(Bx, 2) * Bn -
            lo_h * std::pow(Bx, 3)) * t;
  }
}

// define_Nx_Ny (SIMPLE_TS_MPI.cpp:4955-5041): adjust the cell count until the mesh ends near the domain end.
unsigned fit_count(const Axis& a, unsigned n, double start, double end, double tol) {
  for (int guard = 0; guard < 100000; guard++) {
    double e = start;
    for (unsigned c = 0; c < n; c++) e = e + a.step(e);
    const double d = e - end;
    if (!(std::fabs(d) > tol)) return n;
    const int k = int(std::fabs(d / a.hmax));
    if (d < 0) n = n + k;
    if (d > 0) n = ((n - k) > 2) ? n - k : (unsigned)int(0.75 * n);
  }
  return 0;  // no cell count fits: rejected by the caller
}

// faces, steps and centres (SIMPLE_TS_MPI.cpp:2181-2248)
void build_axis(const Axis& a, unsigned n, double start, unsigned smooth, std::vector<double>& f, std::vector<double>& h,
                std::vector<double>& c) {
  f.assign(n + 1, 0);
  h.assign(n, 0);
  c.assign(n, 0);
  f[0] = start - 0.5 * a.hmax;
  f[1] = start + 0.5 * a.hmax;
  for (unsigned k = 1; k < n; k++) {
    const double t = f[k] + 0.5 * a.step(f[k]);
    f[k + 1] = f[k] + a.step(t);
  }
  for (unsigned k = 0; k < n; k++) {
    h[k] = f[k + 1] - f[k];
    c[k] = f[k] + 0.5 * h[k];
  }
  for (unsigned it = 0; it < smooth; it++) {
    for (unsigned k = 1; k < n; k++) f[k + 1] = f[k] + a.step(c[k]);
    for (unsigned k = 0; k < n; k++) {
      h[k] = f[k + 1] - f[k];
      c[k] = f[k] + 0.5 * h[k];
    }
  }
}

bool read_raw(const std::string& path, void* dst, size_t bytes) {
  FILE* fp = std::fopen(path.c_str(), "rb");
  if (!fp) return false;
  const size_t got = std::fread(dst, 1, bytes, fp);
  std::fclose(fp);
  return got == bytes;
}

bool read_text(const std::string& path, double* dst, int n) {
  std::ifstream in(path.c_str());
  if (!in.is_open()) return false;
  for (int k = 0; k < n; k++) in >> dst[k];
  return !in.fail();
}

// Final-write analysis for an ordered list of updates.  `writes(e)` enumerates the locations
// entry e writes (with a slot number); the returned flags keep, per entry, only the writes that
// are not overwritten by a later entry, so running all entries at once reproduces the
// sequential loop as long as no entry reads a location another entry writes.
template <class F>
std::vector<uint8_t> surviving_writes(size_t n, F writes) {
  std::vector<uint8_t> fin(n, 0);
  std::map<long, std::pair<size_t, int>> last;  // location -> (entry, slot)
  for (size_t e = 0; e < n; e++) {
    std::vector<std::pair<long, int>> w;
    writes(e, w);
    for (auto& x : w) last[x.first] = std::make_pair(e, x.second);
  }
  for (auto& kv : last) fin[kv.second.first] |= (uint8_t)(1u << kv.second.second);
  return fin;
}

}  // namespace

bool body_contains(const HostBody& b, double x, double y) {
  if (b.circle) return ((std::pow((x - b.xc), 2) + std::pow((y - b.yc), 2)) <= std::pow(b.rc, 2));
  return polygon_contains(b, x, y);
}

bool load_case(const std::string& dir, bool fixed_sweeps, Case& c, std::string& err) {
  c.dir = dir;
  Config& cf = c.cfg;
  if (!read_config(dir + "/EnteredData.txt", cf, err)) return false;
  c.restart = cf.b("ToReadSolvedDataFromFile");
  c.periodic = cf.b("Periodic_boundary_conditions_about_OX");
  const unsigned TypeND = (unsigned)cf.n("TypeOfNonDimensiolization");
  if (cf.n("N_I") < 1 || cf.n("N_I") > 64) {
    err = "N_I must be between 1 and 64";
    return false;
  }
  if (cf.n("N_I_p_c") < 1) {
    err = "N_I_p_c must be at least 1";
    return false;
  }

  // nondimensional constants (SIMPLE_TS_MPI.cpp:2013-2071)
  double Ma = cf.d("Ma"), Pr = cf.d("Pr"), gamma1 = cf.d("gamma1"), c_mu = cf.d("c_mu");
  const double Kn = cf.d("Kn"), Re = cf.d("Re"), Fr = cf.d("Fr");
  c.u_given_xb = cf.d("u_given_xb");
  c.p_BC_xb = cf.d("p_BC_xb");
  c.p_BC_xe = cf.d("p_BC_xe");
  if (TypeND == 1 || TypeND == 2) {
    if (cf.b("GivenReKn")) c.u_given_xb = Re * Kn * std::sqrt(15.0 * M_PI / 128.0);
    c.u_given_xb_in_it = c.u_given_xb;
    c.cT = (1.0 / Re) * (c.u_given_xb_in_it * c.p_BC_xb / cf.d("T_BC_xb"));
    c.cPch = (TypeND == 1) ? 0.5 : c.u_given_xb_in_it * c.u_given_xb_in_it / (gamma1 * Ma * Ma);
  } else if (TypeND == 3) {
    Ma = std::sqrt(6.0 / 5.0);
    Pr = 2.0 / 3.0;
    gamma1 = 5.0 / 3.0;
    c_mu = (5.0 / 16.0) * std::sqrt(2.0 * M_PI / gamma1);
    c.cT = Kn * 5.0 * std::sqrt(M_PI) / 16.0;
    c.cPch = 0.5;
  }
  cf.set("Ma", Ma);
  cf.set("Pr", Pr);
  cf.set("gamma1", gamma1);
  cf.set("c_mu", c_mu);
  c.c_Fr_v = cf.b("SolveGravityField") ? 2.0 / (gamma1 * Fr * Ma * Ma) : 0;
  c.cT1 = gamma1 * c_mu * Kn / (Ma * Pr);
  c.cT2 = gamma1 * (gamma1 - 1.0) * c_mu * Kn * Ma;

  // mesh
  Axis ax{(int)cf.n("kind_of_mesh"), cf.d("hxmin"), cf.d("hxmax"), cf.d("xfmin"), cf.d("xfmax"), cf.d("xbmin"),
          cf.d("xbmax"), cf.d("xmid"), 0.0};
  ax.y_axis = false;
  Axis ay{(int)cf.n("kind_of_mesh"), cf.d("hymin"), cf.d("hymax"), cf.d("ybmin"), cf.d("ybmax"), cf.d("ytmin"),
          cf.d("ytmax"), cf.d("ymid"), 0.0};
  ay.y_axis = true;
  axis_coefficients(ax, ax.hmin, ax.hmax);
  axis_coefficients(ay, ax.hmin, ax.hmax);
  unsigned Nx = (unsigned)cf.n("Nx"), Ny = (unsigned)cf.n("Ny");
  if (!c.restart) {
    Nx = fit_count(ax, Nx, cf.d("x_b"), cf.d("x_e"), 5 * ax.hmax);
    Ny = fit_count(ay, Ny, cf.d("y_b"), cf.d("y_e"), 5 * ax.hmax);  // the y tolerance also uses hxmax (:5002)
    cf.set("Nx", Nx);
    cf.set("Ny", Ny);
  }
  if (Nx < 4 || Ny < 4) {
    err = "mesh must have at least 4 cells in each direction";
    return false;
  }
  c.Nx = (int)Nx;
  c.Ny = (int)Ny;
  c.Na = c.Nx * c.Ny;
  const unsigned smooth = (unsigned)cf.n("N_I_T");
  build_axis(ax, Nx, cf.d("x_b"), smooth, c.x_f, c.hx, c.x_v);
  build_axis(ay, Ny, cf.d("y_b"), smooth, c.y_f, c.hy, c.y_v);
  for (int i = 0; i < c.Nx; i++)
    if (!(c.hx[i] > 0)) { err = "zero or negative cell width"; return false; }
  for (int j = 0; j < c.Ny; j++)
    if (!(c.hy[j] > 0)) { err = "zero or negative cell height"; return false; }

  // bodies and the obstacle mask (SIMPLE_TS_MPI.cpp:6306-6360)
  const bool imp_c = cf.b("ToImport_data_for_circles_from_file_b"), imp_p = cf.b("ToImport_data_for_polyhedrons_from_file_b");
  if (imp_c && !read_bodies(dir + "/solve_circles_b.txt", true, c.bodies, err)) return false;
  c.n_circles = (int)c.bodies.size();
  if (imp_p && !read_bodies(dir + "/solve_polyhedrons_b.txt", false, c.bodies, err)) return false;
  for (const HostBody& b : c.bodies)
    if (!b.circle && b.xs.size() < 3) { err = "polygon with fewer than 3 vertices"; return false; }
  c.vol_id.assign(c.Na, 0);
  for (size_t k = 0; k < c.bodies.size(); k++)
    for (int j = 0; j < c.Ny; j++)
      for (int i = 0; i < c.Nx; i++)
        if (body_contains(c.bodies[k], c.x_v[i], c.y_v[j])) c.vol_id[i + j * c.Nx] = (uint32_t)(k + 1);

  // A restart replaces vol_inf_fb by the file's copy after the masks and lists were built
  // (SIMPLE_TS_MPI.cpp:2487 then :5764); body lookups use the file's ids from then on.
  if (c.restart) {
    c.vol_file.assign(c.Na, 0);
    bool ok = true;
    if (cf.b("ToReadSolvedDataFromBinaryFile")) {
      ok = read_raw(dir + "/vol_inf_fb.bin", c.vol_file.data(), sizeof(uint32_t) * c.Na);
    } else {
      std::ifstream in((dir + "/vol_inf_fb.txt").c_str());
      for (int k = 0; k < c.Na && in; k++) in >> c.vol_file[k];
      ok = (bool)in;
    }
    if (!ok) {
      err = "cannot read restart field vol_inf_fb";
      return false;
    }
    for (int k = 0; k < c.Na; k++) {
      if ((c.vol_file[k] == 0) != (c.vol_id[k] == 0) || c.vol_file[k] > c.bodies.size()) {
        err = "restart vol_inf_fb does not match the bodies";
        return false;
      }
    }
  } else {
    c.vol_file = c.vol_id;
  }

  // solve ranges (SIMPLE_TS_MPI.cpp:6009-6191, serial branches)
  const bool pbc = cf.b("Pressure_BC"), gxb = cf.b("Given_velocity_on_xb"), gxe = cf.b("Given_velocity_on_xe");
  const int NX = c.Nx, NY = c.Ny;
  if (c.periodic) { c.Nx_u[0] = c.Nx_v[0] = c.Nx_o[0] = 0; c.Nx_u[1] = c.Nx_v[1] = c.Nx_o[1] = NX; }
  else if (pbc) { c.Nx_u[0] = c.Nx_v[0] = c.Nx_o[0] = 1; c.Nx_u[1] = NX - 1; c.Nx_v[1] = NX - 2; c.Nx_o[1] = NX - 2; }
  else {
    c.Nx_u[0] = gxb ? 2 : 1; c.Nx_v[0] = 1; c.Nx_o[0] = 1;
    c.Nx_u[1] = NX - 1; c.Nx_v[1] = NX - 2; c.Nx_o[1] = gxe ? NX - 1 : NX - 2;
  }
  c.Ny_u[0] = c.Ny_v[0] = c.Ny_o[0] = 1;
  c.Ny_u[1] = NY - 2; c.Ny_v[1] = NY - 1; c.Ny_o[1] = NY - 2;

  // per-cell classes: the reference's interior ("nch") and boundary ("bc") lists
  // (SIMPLE_TS_MPI.cpp:8617-9061) become two bits per variable
  auto F = [&](int k) { return c.vol_id[k] == 0; };
  c.cls.assign(c.Na, 0);
  for (int j = 0; j < NY; j++)
    for (int i = 0; i < NX; i++) {
      const Nb d = neighbours(i, j, NX, NY, c.periodic);
      // the interior test of every variable uses the u ranges (:8639, :8787, :8930)
      const bool inner = (c.Ny_u[0] + 1 < j) && (j < c.Ny_u[1] - 2) && (c.Nx_u[0] + 1 < i) && (i < c.Nx_u[1] - 2);
      uint8_t b = F(d.ij) ? 0x40 : 0;
      if (j >= c.Ny_u[0] && j < c.Ny_u[1] && i >= c.Nx_u[0] && i < c.Nx_u[1] && F(d.i_1j) && F(d.ij)) {
        const bool nb = F(d.i_1j_1) && F(d.ij_1) && F(d.i_1j1) && F(d.ij1) && F(d.i1j) && F(d.i_2j);
        b |= (inner && nb) ? CLS_NCH : CLS_BC;
      }
      if (j >= c.Ny_v[0] && j < c.Ny_v[1] && i >= c.Nx_v[0] && i < c.Nx_v[1] && F(d.ij_1) && F(d.ij)) {
        const int far = d.ij_1 - ((j - 2) >= 0 ? NX : 0);
        const bool nb = F(d.i_1j_1) && F(d.i_1j) && F(d.i1j_1) && F(d.i1j) && F(far) && F(d.ij1);
        b |= (uint8_t)(((inner && nb) ? CLS_NCH : CLS_BC) << 2);
      }
      if (j >= c.Ny_o[0] && j < c.Ny_o[1] && i >= c.Nx_o[0] && i < c.Nx_o[1] && F(d.ij)) {
        const bool nb = F(d.i_1j) && F(d.i1j) && F(d.ij_1) && F(d.ij1) && F(d.i_1j_1) && F(d.i_1j1) && F(d.i1j_1) &&
                        F(d.i1j1);
        b |= (uint8_t)(((inner && nb) ? CLS_NCH : CLS_BC) << 4);
      }
      c.cls[d.ij] = b;
    }

  // wall lists (SIMPLE_TS_MPI.cpp:10158-10379) with their surviving writes
  for (int j = 0; j < NY; j++)
    for (int i = 0; i < NX; i++) {
      const Nb d = neighbours(i, j, NX, NY, c.periodic);
      if (c.vol_id[d.ij] > 0 && (c.vol_id[d.ij_1] == 0 || c.vol_id[d.ij1] == 0) && c.bodies[c.vol_file[d.ij] - 1].dev.slip)
        c.slip_u.push_back(d.ij);
    }
  for (int j = 0; j < NY; j++)
    for (int i = 0; i < NX; i++) {
      const Nb d = neighbours(i, j, NX, NY, c.periodic);
      if (c.vol_id[d.ij] > 0 && (c.vol_id[d.i_1j] == 0 || c.vol_id[d.i1j] == 0) && c.bodies[c.vol_file[d.ij] - 1].dev.slip)
        c.slip_v.push_back(d.ij);
    }
  for (int j = 0; j < NY; j++)
    for (int i = 0; i < NX; i++) {
      const Nb d = neighbours(i, j, NX, NY, c.periodic);
      if (F(d.ij) && (!F(d.i_1j) || !F(d.i1j) || !F(d.ij_1) || !F(d.ij1))) c.tjump.push_back(d.ij);
    }
  auto nb_of = [&](int node) { const int j = node / NX, i = node - j * NX; return neighbours(i, j, NX, NY, c.periodic); };
  c.slip_u_fin = surviving_writes(c.slip_u.size(), [&](size_t e, std::vector<std::pair<long, int>>& w) {
    const Nb d = nb_of(c.slip_u[e]);
    const bool below = c.vol_id[d.ij_1] == 0;
    if (F(below ? d.i_1j_1 : d.i_1j1)) w.push_back({d.ij, 0});
    if (F(below ? d.i1j_1 : d.i1j1)) w.push_back({d.i1j, 1});
  });
  c.slip_v_fin = surviving_writes(c.slip_v.size(), [&](size_t e, std::vector<std::pair<long, int>>& w) {
    const Nb d = nb_of(c.slip_v[e]);
    const bool left = c.vol_id[d.i_1j] == 0;
    if (F(left ? d.i_1j_1 : d.i1j_1)) w.push_back({d.ij, 0});
    if (F(left ? d.i_1j1 : d.i1j1)) w.push_back({d.ij1, 1});
  });
  c.tjump_fin = surviving_writes(c.tjump.size(), [&](size_t e, std::vector<std::pair<long, int>>& w) {
    const Nb d = nb_of(c.tjump[e]);
    if (!F(d.i_1j)) w.push_back({(long)d.ij, 0});
    if (!F(d.i1j)) w.push_back({(long)d.i1j, 1});
    if (!F(d.ij_1)) w.push_back({(long)c.Na + d.ij, 2});
    if (!F(d.ij1)) w.push_back({(long)c.Na + d.ij1, 3});
  });
  c.tjump_wr_fin = surviving_writes(c.tjump.size(), [&](size_t e, std::vector<std::pair<long, int>>& w) {
    const Nb d = nb_of(c.tjump[e]);
    if (!F(d.i_1j)) w.push_back({d.i_1j, 0});
    if (!F(d.i1j)) w.push_back({d.i1j, 1});
    if (!F(d.ij_1)) w.push_back({d.ij_1, 2});
    if (!F(d.ij1)) w.push_back({d.ij1, 3});
  });
  // the parallel wall updates rely on no entry reading a face another entry writes
  {
    std::vector<char> written(c.Na, 0);
    for (size_t e = 0; e < c.slip_u.size(); e++) {
      const Nb d = nb_of(c.slip_u[e]);
      written[d.ij] = written[d.i1j] = 1;
    }
    for (size_t e = 0; e < c.slip_u.size(); e++) {
      const Nb d = nb_of(c.slip_u[e]);
      const bool below = c.vol_id[d.ij_1] == 0;
      const int r0 = below ? d.ij_1 : d.ij1, r1 = below ? d.i1j_1 : d.i1j1;
      const bool w0 = F(below ? d.i_1j_1 : d.i_1j1), w1 = F(below ? d.i1j_1 : d.i1j1);
      if ((w0 && written[r0]) || (w1 && written[r1])) { err = "slip-u wall list reads a face it writes"; return false; }
    }
    std::fill(written.begin(), written.end(), 0);
    for (size_t e = 0; e < c.slip_v.size(); e++) {
      const Nb d = nb_of(c.slip_v[e]);
      written[d.ij] = written[d.ij1] = 1;
    }
    for (size_t e = 0; e < c.slip_v.size(); e++) {
      const Nb d = nb_of(c.slip_v[e]);
      const bool left = c.vol_id[d.i_1j] == 0;
      const int r0 = left ? d.i_1j : d.i1j, r1 = left ? d.i_1j1 : d.i1j1;
      const bool w0 = F(left ? d.i_1j_1 : d.i1j_1), w1 = F(left ? d.i_1j1 : d.i1j1);
      if ((w0 && written[r0]) || (w1 && written[r1])) { err = "slip-v wall list reads a face it writes"; return false; }
    }
  }

  // flags
  uint64_t& bits = c.bits;
  struct { const char* name; uint64_t bit; } fl[] = {
      {"Periodic_boundary_conditions_about_OX", F_PERIODIC}, {"Pressure_BC", F_PRESSURE_BC},
      {"Given_velocity_on_xb", F_GIVEN_U_XB}, {"Given_velocity_on_xe", F_GIVEN_U_XE}, {"dvdx_0_BC_xb", F_DVDX0_XB},
      {"dvdx_0_BC_xe", F_DVDX0_XE}, {"dvdy_0_BC_yb", F_DVDY0_YB}, {"dvdy_0_BC_ye", F_DVDY0_YE},
      {"dudx_0_BC_xb", F_DUDX0_XB}, {"durhodx_0_BC_xb", F_DURHODX0_XB},
      {"drhodt_durhodx_dvrhody_0_BC_xb", F_DRHODT0_XB}, {"dudx_0_BC_xe", F_DUDX0_XE},
      {"durhodx_0_BC_xe", F_DURHODX0_XE}, {"drhodt_durhodx_dvrhody_0_BC_xe", F_DRHODT0_XE},
      {"u_uMin_Mout_0_BC_xe", F_U_MINMOUT_XE}, {"dudy_0_BC_yb", F_DUDY0_YB}, {"dudy_0_BC_ye", F_DUDY0_YE},
      {"dpdx_0_BC_xb", F_DPDX0_XB}, {"dpdx_0_BC_xe", F_DPDX0_XE}, {"dpdy_0_BC_yb", F_DPDY0_YB},
      {"dpdy_0_BC_ye", F_DPDY0_YE}, {"dTdx_0_BC_xb", F_DTDX0_XB}, {"dTdx_0_BC_xe", F_DTDX0_XE},
      {"dTdy_0_BC_yb", F_DTDY0_YB}, {"dTdy_0_BC_ye", F_DTDY0_YE}, {"To_Use_Kn_local_in_wall_BC", F_KN_LOCAL},
      {"GivenReKn", F_GIVEN_REKN}, {"Pressure_ratio_correct", F_RATIO_CORRECT}, {"p_correction_auto", F_P_CORR_AUTO},
      {"correct_p_BC_xb", F_CORRECT_P_XB}, {"use_interpolation_for_u_BC_by_time", F_U_BY_TIME},
  };
  for (auto& f : fl)
    if (cf.b(f.name)) bits |= f.bit;
  if (fixed_sweeps) bits |= F_FIXED_SWEEPS;

  // initial fields (SIMPLE_TS_MPI.cpp:2476-2483 and :2502-2845)
  const int Na = c.Na;
  c.u.assign(Na, cf.d("u_gas_nd"));
  c.v.assign(Na, cf.d("v_gas_nd"));
  c.p.assign(Na, cf.d("p_gas_nd"));
  c.T.assign(Na, cf.d("T_gas_nd"));
  c.rho.assign(Na, cf.d("p_gas_nd") / cf.d("T_gas_nd"));
  if (c.restart) {
    const bool bin = cf.b("ToReadSolvedDataFromBinaryFile");
    const char* names[4] = {"u", "v", "p", "Temper"};
    std::vector<double>* dst[4] = {&c.u, &c.v, &c.p, &c.T};
    for (int k = 0; k < 4; k++) {
      const bool ok = bin ? read_raw(dir + "/" + names[k] + ".bin", dst[k]->data(), sizeof(double) * Na)
                          : read_text(dir + "/" + names[k] + ".txt", dst[k]->data(), Na);
      if (!ok) {
        err = std::string("cannot read restart field ") + names[k];
        return false;
      }
    }
    for (int k = 0; k < Na; k++) {
      if (!std::isfinite(c.u[k]) || !std::isfinite(c.v[k]) || !std::isfinite(c.p[k]) || !std::isfinite(c.T[k])) {
        err = "restart fields hold a non-finite value";
        return false;
      }
      c.rho[k] = F(k) ? c.p[k] / c.T[k] : 0;
    }
    std::ifstream itf((dir + "/it_begin.txt").c_str());
    if (itf.is_open()) itf >> c.it_begin;
  } else {
    auto apply_bodies = [&]() {  // ApplyBodiesConditionsToVariables, SIMPLE_TS_MPI.cpp:6470-6584
      for (int i = 0; i < NX; i++)
        for (int j = 0; j < NY; j++) {
          const Nb d = neighbours(i, j, NX, NY, false);
          if (c.vol_id[d.ij] >= 1) {
            const double ub = c.bodies[c.vol_id[d.ij] - 1].dev.u;
            c.u[d.ij] = ub;
            c.u[d.i1j] = ub;
          }
        }
      for (int i = 0; i < NX; i++)
        for (int j = 0; j < NY; j++) {
          const Nb d = neighbours(i, j, NX, NY, false);
          if (c.vol_id[d.ij] >= 1) {
            const double vb = c.bodies[c.vol_id[d.ij] - 1].dev.v;
            c.v[d.ij] = vb;
            c.v[d.ij1] = vb;
          }
        }
      for (int k = 0; k < Na; k++)
        if (c.vol_id[k] >= 1) {
          const Body& B = c.bodies[c.vol_id[k] - 1].dev;
          c.p[k] = B.p;
          c.T[k] = B.T;
          c.rho[k] = F(k) ? c.p[k] / c.T[k] : 0;
        }
    };
    apply_bodies();
    const double T_BC_xb = cf.d("T_BC_xb"), T_BC_xe = cf.d("T_BC_xe");
    const bool exact = cf.b("ToStartFromExactSolutionForChannelFlowWithPressureBC");
    if (pbc) {
      const double rb = c.p_BC_xb / T_BC_xb, re = c.p_BC_xe / T_BC_xe;
      for (int j = 0; j < NY; j++) {
        for (int i = 0; i < c.Nx_o[0]; i++) {
          const int n = i + j * NX;
          if (F(n)) { c.p[n] = c.p_BC_xb; c.rho[n] = rb; c.T[n] = T_BC_xb; }
        }
        for (int i = c.Nx_o[1]; i < NX; i++) {
          const int n = i + j * NX;
          if (F(n)) { c.p[n] = c.p_BC_xe; c.rho[n] = re; c.T[n] = T_BC_xe; }
        }
      }
      if (exact) {  // analytic slip channel flow start (SIMPLE_TS_MPI.cpp:2566-2688)
        int jb = 0, je = 0;
        for (int j = 1; j < NY; j++) {
          const int n = 1 + j * NX;
          if (!F(n - NX) && F(n)) jb = j - 1;
          if (F(n - NX) && !F(n)) je = j;
        }
        const double hch = c.y_v[je] - c.y_v[jb];
        const double Lch = c.x_v[c.Nx_o[1]] - c.x_v[c.Nx_o[0] - 1];
        if ((int)c.bodies.size() <= c.n_circles) { err = "analytic start needs a polygon body"; return false; }
        const HostBody& B0 = c.bodies[c.n_circles];  // the first polyhedron
        const double sig = B0.dev.slip * B0.dev.F_slip, Px = c.p_BC_xb / c.p_BC_xe;
        std::vector<double> xa(NX), ya(NY);
        for (int i = 0; i < NX; i++) xa[i] = (c.x_v[i] - c.x_v[0]) / Lch;
        for (int j = 0; j < NY; j++)
          ya[j] = (j <= jb) ? -0.5 * hch : ((je <= j) ? 0.5 * hch : c.y_v[j + jb] - (c.y_v[jb] + 0.5 * hch));
        for (int j = 0; j < NY; j++)
          for (int i = c.Nx_o[0]; i < c.Nx_o[1]; i++) {
            const int n = i + j * NX;
            if (F(n))
              c.p[n] = c.p_BC_xe * (-6.0 * sig * Kn + std::sqrt(std::pow((6.0 * sig * Kn), 2) +
                                                                (1.0 + 12.0 * sig * Kn) * xa[i] +
                                                                (Px + 12.0 * sig * Kn) * Px * (1.0 - xa[i])));
          }
        double ND = 0;
        if (TypeND == 1 || TypeND == 2) ND = Re * hch * hch / (4.0 * c.u_given_xb);
        else if (TypeND == 3) ND = hch / (5.0 * std::sqrt(M_PI * T_BC_xb) * Kn * Lch);
        for (int j = 0; j < NY; j++)
          for (int i = 0; i < NX; i++) {
            const int n = i + j * NX;
            if (F(n))
              c.u[n] = -ND *
                       ((c.p_BC_xe * (1.0 - Px * Px + 12.0 * sig * Kn * (1.0 - Px))) /
                        (2.0 * std::sqrt(std::pow((6.0 * sig * Kn), 2) + (1.0 + 12.0 * sig * Kn) * xa[i] +
                                         (Px + 12.0 * sig * Kn) * Px * (1.0 - xa[i])))) *
                       (1.0 - 4.0 * ya[j] * ya[j] / (hch * hch) + 4.0 * sig * Kn / c.p[n]);
          }
      }
    }
    if (gxb && exact) {  // SIMPLE_TS_MPI.cpp:2694-2806
      for (int j = 0; j < NY; j++)
        for (int i = 0; i < c.Nx_o[0] + 1; i++) {
          const int n = i + j * NX;
          if (F(n)) c.p[n] = c.p_BC_xb;
        }
      int jb = 0, je = 0;
      for (int j = 1; j < NY; j++) {
        const int n = 1 + j * NX;
        if (!F(n - NX) && F(n)) jb = j - 1;
        if (F(n - NX) && !F(n)) je = j;
      }
      const double hch = c.y_f[je + 1] - c.y_f[jb];
      const double Lch = c.x_v[c.Nx_o[1]] - c.x_v[c.Nx_o[0] - 1];
      const double yc = c.y_v[jb] + 0.5 * hch;
      const double q = (yc - c.y_v[jb] / hch - (yc - c.y_v[jb] / hch) * (yc - c.y_v[jb] / hch));
      const double ug = c.u_given_xb;
      if (cf.b("correct_p_BC_xb")) c.p_BC_xb = c.p_BC_xe + 4.0 * Lch * ug * ug / (Re * hch * hch * q);
      else c.p_BC_xe = c.p_BC_xb - 4.0 * Lch * ug * ug / (Re * hch * hch * q);
      const double dpdx = (c.p_BC_xe - c.p_BC_xb) / Lch;
      double ND = 0;
      if (TypeND == 1 || TypeND == 2) ND = Re * hch * hch / (4.0 * ug);
      else if (TypeND == 3) ND = 4.0 * hch * hch / (5.0 * std::sqrt(M_PI * T_BC_xb) * Kn);
      if ((int)c.bodies.size() <= c.n_circles) { err = "analytic start needs a polygon body"; return false; }
      const HostBody& B0 = c.bodies[c.n_circles];  // the first polyhedron
      for (int j = 0; j < NY; j++)
        for (int i = 0; i < c.Nx_u[0]; i++) {
          const int n = i + j * NX;
          if (F(n))
            c.u[n] = -ND * dpdx *
                     ((c.y_v[j] - c.y_v[jb]) / hch - ((c.y_v[j] - c.y_v[jb]) / hch) * ((c.y_v[j] - c.y_v[jb]) / hch) +
                      Kn * B0.dev.F_slip * B0.dev.slip / hch);
        }
    }
    if (gxe && exact) {
      for (int j = 0; j < NY; j++)
        for (int i = c.Nx_o[1]; i < NX; i++) {
          const int n = i + j * NX;
          if (F(n)) c.p[n] = c.p_BC_xe;
        }
    }
    apply_bodies();
  }
  // coefficients as refreshed just before the time loop (SIMPLE_TS_MPI.cpp:3043-3057)
  if (TypeND == 1 || TypeND == 2) {
    c.cT = (1.0 / Re) * (c.u_given_xb_in_it * c.p_BC_xb / cf.d("T_BC_xb"));
    c.cPch = (TypeND == 1) ? 0.5 : c.u_given_xb_in_it * c.u_given_xb_in_it / (gamma1 * Ma * Ma);
  }
  return true;
}

}  // namespace sts
