// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// CPU oracle for the SIMPLE-TS time step: a plain C++ restatement of the serial
// (non-MPI) path of the reference solver SIMPLE_TS_MPI.cpp, used only by tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg, always as the checker.
// The GB300 product never links, loads or calls this file.
//
// Every routine names the reference lines it restates.  Arithmetic follows the
// reference expression by expression (same operand order, no reassociation),
// so with -ffp-contract=off it reproduces the reference binary bit for bit; the
// pinning tests compare it with dumps of the reference itself.
//
// Layout: all fields are double[Nx*Ny], ij = i + j*Nx (x fastest), exactly as in
// the reference (SIMPLE_TS_MPI.cpp:2384-2464).

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

namespace {

typedef unsigned int uint;

inline double dmax(double a, double b) { return a > b ? a : b; }   // maximum(), SIMPLE_TS_MPI.cpp:120
inline double dmin(double a, double b) { return a < b ? a : b; }   // minimum(), SIMPLE_TS_MPI.cpp:123
// upwind_rho, SIMPLE_TS_MPI.cpp:129
inline double upwind_rho(double r0, double r1, double v1) {
  return (v1 == 0) ? (0.5 * (r0 + r1)) : ((v1 > 0) ? r0 : r1);
}
// Li / Hi, SIMPLE_TS_MPI.cpp:133-136
inline double Li(double f1, double f2, double h1, double h2) { return (f1 * h2 + f2 * h1) / (h1 + h2); }
inline double Hi(double f1, double f2, double h1, double h2) {
  return (h1 + h2) * f1 * f2 / (h1 * f2 + h2 * f1);
}

struct Body {
  bool circle = false;
  // circle (Circles_Objects.h:47-51)
  double xc = 1, yc = 1, rc = 1;
  // polygon (Polyhedrons_Objects.h)
  std::vector<double> xs, ys;
  double p1x = 0, p1y = 0, p2x = 1, p2y = 1;
  double u = 0, v = 0, p = 0, T = 0;
  bool slip = false;
  double F_slip = 1.1466, w_slip = 0.1;
  bool jump = false;
  double F_jump = 2.1904, dTdn0 = 0;
  bool drag = false;
  // cached state of Polyhedrons_Objects::is_point_inside_polyhedron
  bool rect_defined = false;
  double xrmin = 0, xrmax = 0, yrmin = 0, yrmax = 0;
  double kpi = 0, bpi = 0;
};

// Polyhedrons_Objects::is_two_lines_intersections, Polyhedrons_Objects.cpp:327-501
bool lines_intersect(double x11, double y11, double x12, double y12, double x21, double y21,
                     double x22, double y22) {
  bool hit = false;
  double xi = 0, yi = 0;
  double x1min = dmin(x11, x12), x1max = dmax(x11, x12);
  double y1min = dmin(y11, y12), y1max = dmax(y11, y12);
  double x2min = dmin(x21, x22), x2max = dmax(x21, x22);
  double y2min = dmin(y21, y22), y2max = dmax(y21, y22);
  double k1, b1, k2, b2;
  if ((x1min != x1max) && (y1min != y1max) && (x2min != x2max) && (y2min != y2max)) {
    k1 = (y11 - y12) / (x11 - x12);
    b1 = y11 - k1 * x11;
    k2 = (y21 - y22) / (x21 - x22);
    b2 = y21 - k2 * x21;
    if (k1 != k2) {
      xi = (b1 - b2) / (k2 - k1);
      yi = k1 * xi + b1;
      hit = true;
    }
  } else if (y1min == y1max && x2min == x2max) {
    xi = x2min; yi = y1min; hit = true;
  } else if ((y1min == y1max) && (x2min != x2max) && (y2min != y2max)) {
    yi = y1min;
    k2 = (y21 - y22) / (x21 - x22);
    b2 = y21 - k2 * x21;
    xi = (yi - b2) / k2;
    hit = true;
  } else if (x1min == x1max && y2min == y2max) {
    xi = x1min; yi = y2min; hit = true;
  } else if ((x1min == x1max) && (x2min != x2max) && (y2min != y2max)) {
    xi = x1min;
    k2 = (y21 - y22) / (x21 - x22);
    b2 = y21 - k2 * x21;
    yi = k2 * xi + b2;
    hit = true;
  } else if ((x1min != x1max) && (y1min != y1max) && (x2min == x2max)) {
    xi = x2min;
    k1 = (y11 - y12) / (x11 - x12);
    b1 = y11 - k1 * x11;
    yi = k1 * xi + b1;
    hit = true;
  } else if ((x1min != x1max) && (y1min != y1max) && (y2min == y2max)) {
    yi = y2min;
    k1 = (y11 - y12) / (x11 - x12);
    b1 = y11 - k1 * x11;
    xi = (yi - b1) / k1;
    hit = true;
  } else {
    hit = false;
  }
  if (hit && !(x1min <= xi && xi <= x1max && x2min <= xi && xi <= x2max && y1min <= yi &&
               yi <= y1max && y2min <= yi && yi <= y2max))
    hit = false;
  return hit;
}

// Polyhedrons_Objects::is_point_inside_polyhedron, Polyhedrons_Objects.cpp:190-324
bool point_in_polygon(Body& b, double x, double y) {
  const int N = (int)b.xs.size();
  if (!b.rect_defined) {  // define_rectangular_around_polyhedron, :506-528
    b.xrmin = b.xrmax = b.xs[0];
    b.yrmin = b.yrmax = b.ys[0];
    for (int c = 0; c < N; c++) {
      b.xrmin = dmin(b.xrmin, b.xs[c]); b.xrmax = dmax(b.xrmax, b.xs[c]);
      b.yrmin = dmin(b.yrmin, b.ys[c]); b.yrmax = dmax(b.yrmax, b.ys[c]);
    }
    b.rect_defined = true;
  }
  bool inside = (b.xrmin <= x && x <= b.xrmax && b.yrmin <= y && y <= b.yrmax);
  if (!inside) return false;
  double xpmin = dmin(b.p1x, b.p2x), xpmax = dmax(b.p1x, b.p2x);
  double ypmin = dmin(b.p1y, b.p2y), ypmax = dmax(b.p1y, b.p2y);
  if ((xpmin != xpmax) && (ypmin != ypmax)) {
    b.kpi = (b.p2y - b.p1y) / (b.p2x - b.p1x);
    b.bpi = b.p1y - b.kpi * b.p1x;
  }
  const unsigned N_maximum_divide = 5000;
  bool again;
  unsigned div = 1;
  double px = 0, py = 0;
  do {
    again = false;
    if (xpmin == xpmax) {
      px = xpmin; py = ypmin + (ypmax - ypmin) / div;
    } else if (ypmin == ypmax) {
      px = xpmin + (xpmax - xpmin) / div; py = ypmin;
    } else {
      px = xpmin + (xpmax - xpmin) / div; py = b.kpi * px + b.bpi;
    }
    if (px == x && py == y) again = true;
    if (!again) {
      int c = 0;
      do {
        if (px == x && x == b.xs[c]) again = true;
        else if (py == y && y == b.ys[c]) again = true;
        else if (b.ys[c] == (py - y) * (b.xs[c] - px) / (px - x) + py) again = true;
        c++;
      } while (c < N && !again);
    }
    div++;
  } while (div < N_maximum_divide && again);
  if (again) {
    std::cout << "The check with point inside can NOT be done!" << std::endl;
    return inside;
  }
  double n = 0;
  for (int c = 0; c < N; c++) {
    int c2 = (c < N - 1) ? c + 1 : 0;
    n = n + lines_intersect(px, py, x, y, b.xs[c], b.ys[c], b.xs[c2], b.ys[c2]);
  }
  return ((n / 2.0) == std::floor(n / 2.0));
}

// Circles_Objects.h:118-126
bool point_in_circle(const Body& b, double x, double y) {
  return ((std::pow((x - b.xc), 2) + std::pow((y - b.yc), 2)) <= std::pow(b.rc, 2));
}

struct Oracle {
  std::string dir;
  bool write_files = true;
  bool fixed_sweeps = true;      // FIXED_NUMBER_OF_ITERATIONS_LOOP_3 (SIMPLE_TS_MPI.cpp:56)
  // Warm start of the p-T sweeps (not in the reference; the GB300 library's option of the same
  // name): 1 starts every step's sweeps from the linear extrapolation p_n + (p_n - p_{n-1}) on the
  // solved cells instead of p_n.  The first step, with no history, starts from p_n.
  int warm_start = 0;
  std::vector<double> p_m1, T_m1, p_m2, T_m2;
  int warm_ready = 0;  // steps of history
  // mode 3: x0 = x_n + sum_k w_k D_{n-k} (D_j = x_j - x_{j-1}), k = 0..2, with w fitted by least
  // squares on the last kWin steps of the trajectory (see warm_ar)
  static constexpr int kRing = 9, kWin = 6;
  std::vector<std::vector<double>> Dp, DT;  // ring of differences on the solved cells
  void warm_ar();
  // an initial iterate supplied from outside for the next step only (predictor studies, and
  // replaying a guess the GPU library computed): replaces p and T on the solved cells after the
  // step's previous-value copies, where the warm start acts
  std::vector<double> guess_p, guess_T;
  // mode 4: the convolutional predictor (see warm_conv)
  static constexpr int kCFeat = 36, kCTerms = 36 * 37 / 2 + 36, kCWin = 6, kCRing = 5;
  std::vector<float> cD[2][kCRing];
  std::vector<unsigned char> cact[2], csolved;
  std::vector<float> cgram;
  float conv_w[2][kCFeat] = {};
  bool conv_ok[2] = {false, false};
  void warm_conv();
  void conv_features(int f, unsigned t, int i, int j, float* out) const;
  bool check_wallclock = false;  // honour max_time_for_solve (CLI only)
  bool apply_saves = false;      // periodic WriteSolvedDataToFile inside step() (CLI only)
  bool finished = false;
  std::string err;

  // ---- EnteredData.txt (SIMPLE_TS_MPI.cpp:5253-5544) ----
  double u_gas_nd = 0, v_gas_nd = 0, T_gas_nd = 1, p_gas_nd = 1, Ma = 0, Pr = 0, gamma1 = 0, c_mu = 0,
         Kn = 0, Fr = 0;
  bool SolveGravityField = false;
  double Re = 0;
  uint TypeND = 3;
  double Nt = 0;
  uint Nx = 0, Ny = 0, N_I = 1, N_I_p_c = 2, N_I_T = 0;
  double ht = 0, x_b = 0, x_e = 0, y_b = 0, y_e = 0;
  uint kind_of_mesh = 3;
  double hxmin, hxmax, xfmin, xfmax, xbmin, xbmax, xmid, hymin, hymax, ytmin, ytmax, ybmin, ybmax,
      ymid;
  double MaxError_Velocities, MaxError_p_c, MaxError_T, MaxError_to_stop_program, max_time_for_solve;
  bool solve_is_finished = false;
  int Nt_save_solved_data = 1;
  uint Nt_save_DragCoefficient = 1;
  int Nt_save_temp_data = 1, N_I_check = 1, WriteDataInShortFormat_kind = 0;
  bool ToReadSolvedDataFromFile = false, ToReadSolvedDataFromBinaryFile = true,
       ToWriteSolvedDataToBinaryFile = true, ToWriteSolvedDataToNewFiles = false,
       ToContinueFromInterpolation = false;
  bool imp_circ_b = false, imp_poly_b = false, imp_circ_p = false, imp_poly_p = false,
       imp_circ_V = false, imp_poly_V = false;
  bool Given_velocity_on_xb = false, Given_velocity_on_xe = false, Periodic = false, Pressure_BC = false,
       ToStartFromExactSolution = false;
  uint p_BC_xb_correction_method = 0;
  bool Pressure_ratio_correct = false, GivenReKn = false, correct_p_BC_xb = false;
  double u_given_xb = 0, u_given_xb_error = 0;
  bool p_correction_auto = false;
  double p_correction_min = 0, p_correction_max = 0, p_correction = 0;
  double p_BC_xb = 0, T_BC_xb = 0, p_BC_xe = 0, T_BC_xe = 0;
  bool dudx_0_BC_xb, durhodx_0_BC_xb, drhodt_0_BC_xb, calc_u_xb, dudx_0_BC_xe, durhodx_0_BC_xe,
      drhodt_0_BC_xe, calc_u_xe, u_uMin_Mout_0_BC_xe, dudy_0_BC_yb, dudy_0_BC_ye, dvdx_0_BC_xb, calc_v_xb,
      dvdx_0_BC_xe, calc_v_xe, dvdy_0_BC_yb, dvdy_0_BC_ye, dpdx_0_BC_xb, calc_p_xb, dpdx_0_BC_xe, calc_p_xe,
      dpdy_0_BC_yb, dpdy_0_BC_ye, dTdx_0_BC_xb, calc_T_xb, dTdx_0_BC_xe, calc_T_xe, dTdy_0_BC_yb,
      dTdy_0_BC_ye, To_Use_Kn_local_in_wall_BC, ToSolveContinuityEquation,
      use_interpolation_for_u_BC_by_time;
  double t_BC_b = 0, t_BC_e = 0, u_BC_xb_t_BC_b = 0, u_BC_xb_t_BC_e = 0, w_u, w_v, w_p, w_Temper;
  uint N_SubDomains_x = 1, N_SubDomains_y = 1;
  bool rd_sep, wr_entire, wr_sep, only_nx_ny;

  // ---- derived scalars ----
  double rho_gas_nd = 1, V_gas_nd = 0, cT = 0, cPch = 0.5, c_Fr_v = 0, cT1 = 0, cT2 = 0;
  double u_given_xb_in_it = 0, u_given_xb_in_it_max = 0, u_given_xb_in_it_mean = 0;
  double rho_BC_xb = 0, rho_BC_xe = 0;
  double axf3 = 0, axf2 = 0, axf1 = 0, axf0 = 0, axb3 = 0, axb2 = 0, axb1 = 0, axb0 = 0;
  double ayt3 = 0, ayt2 = 0, ayt1 = 0, ayt0 = 0, ayb3 = 0, ayb2 = 0, ayb1 = 0, ayb0 = 0;
  double hxmid = 0, hymid = 0;
  double it = 0, it_begin = 0;
  uint it_counter = 0, Na = 0, Iter = 0, Iter_pr1 = 0, Iter_pr2 = 0, Iter_p_c = 0, Iter_T = 0;
  bool continue_iter = true, continue_iter_p_c = true, countinue_time_step = true;
  double time_solve_stop = 0;
  long time_solve_start = 0;
  int Nt_save_solved_data_counter = 0, Nt_save_temp_data_counter = 0;
  uint Nt_save_DragCoefficient_counter = 0;
  bool ToCheckForFileIsNow_Tmp = true, ToCheckForFileIsNow_Iterations_in_loops = true;
  bool ToCheckForFileIsNow_CD = true, ToCheckForFileIsNow_p_u_x_b = true;
  std::vector<double> continuity_st, continuity;

  // ---- mesh ----
  std::vector<double> x_f, y_f, hx, hy, x_v, y_v;

  // ---- bodies (index 0 = gb) ----
  std::vector<Body> bodies;  // circles first, then polygons (ids 1..)
  uint N_circles = 0, N_polygons = 0;

  // ---- masks and lists ----
  std::vector<uint> vol_inf_fb;
  std::vector<char> vol;  // vol_inf_fb_bool
  uint Nx_u[2], Ny_u[2], Nx_v[2], Ny_v[2], Nx_o[2], Ny_o[2];
  std::vector<uint> nch_u, bc_u, nch_v, bc_v, nch_o, bc_o;  // node indices (j = node / Nx)
  std::vector<int> slip_u, slip_v, tjump;

  // ---- fields ----
  std::vector<double> Gamma_yf, Gamma_xf, Fx, Fy, st_u0, st_u1, u_pseudo, D_ux, D_uy, st_v0, st_v1,
      v_pseudo, D_vx, D_vy, st_p0, st_p1, st_p2, d_p_c_12, d_p_c_34, apx, apy, bpx, bpy, st_r0, st_r1,
      rho_u, rho_v, st_T0, st_T1, st_T2, Tw_u, Tw_v, sqrt_T, DTx, DTy, ScT1;
  double *u, *u_pr, *v, *v_pr, *p, *p_pr, *p_old, *rho, *rho_pr, *Temper, *Temper_pr, *Temper_old;
  std::vector<double> max_res_p, max_res_T, max_res_p0, max_res_T0;
  std::vector<uint> max_Iter_p_c;
  double max_residual_in_u = 0, max_residual_in_v = 0, max_residual_in_u_Iter_0 = 0,
         max_residual_in_v_Iter_0 = 0;
  // per-step record of the sweep counts (sum over outer iterations)
  std::vector<uint> sweeps_per_step;

  // ---- index helpers: ij_function / ij_function_PeriodicBC, SIMPLE_TS_MPI.cpp:140-232 ----
  struct Idx {
    uint i, j, ij, i_1, i_2, i1, i_1j, i1j, ij_1, ij1, i_1j_1, i_1j1, i1j_1, i1j1, i_2j;
  };
  Idx clamped(uint i, uint j) const {
    Idx d;
    d.i = i; d.j = j;
    d.ij = i + j * Nx;
    d.i_1 = i - 1 * (0 < i);
    d.i_2 = i - 1 * (0 < i) - 1 * (1 < i);
    d.i1 = i + 1 * (i < (Nx - 1));
    d.i_1j = d.ij - 1 * (0 < i);
    d.i1j = d.ij + 1 * (i < (Nx - 1));
    d.ij_1 = d.ij - Nx * (0 < j);
    d.ij1 = d.ij + Nx * (j < (Ny - 1));
    d.i_1j_1 = d.ij - 1 * (0 < i) - Nx * (0 < j);
    d.i_1j1 = d.ij - 1 * (0 < i) + Nx * (j < (Ny - 1));
    d.i1j_1 = d.ij + 1 * (i < (Nx - 1)) - Nx * (0 < j);
    d.i1j1 = d.ij + 1 * (i < (Nx - 1)) + Nx * (j < (Ny - 1));
    d.i_2j = d.i_2 + j * Nx;
    return d;
  }
  Idx periodic(uint i, uint j) const {
    Idx d;
    d.i = i; d.j = j;
    d.i_1 = (i == 0) ? Nx - 1 : i - 1;
    d.i_2 = (i == 1) ? Nx - 1 : ((i == 0) ? Nx - 2 : i - 2);
    d.i1 = (i == Nx - 1) ? 0 : i + 1;
    d.ij = i + j * Nx;
    d.i_1j = d.i_1 + j * Nx;
    d.i1j = d.i1 + j * Nx;
    d.ij_1 = i + (j - 1 * (0 < j)) * Nx;
    d.ij1 = i + (j + 1 * (j < (Ny - 1))) * Nx;
    d.i_1j_1 = d.i_1 + (j - 1 * (0 < j)) * Nx;
    d.i_1j1 = d.i_1 + (j + 1 * (j < (Ny - 1))) * Nx;
    d.i1j_1 = d.i1 + (j - 1 * (0 < j)) * Nx;
    d.i1j1 = d.i1 + (j + 1 * (j < (Ny - 1))) * Nx;
    d.i_2j = d.i_2 + j * Nx;
    return d;
  }
  Idx bc_idx(uint node) const {
    uint j = node / Nx, i = node - j * Nx;
    return Periodic ? periodic(i, j) : clamped(i, j);
  }

  // ======================= input =======================
  bool read_entered_data();
  bool read_bodies(const char* fname, bool circles);
  void build_mesh();
  double hx_all(double x) const;
  double hy_all(double y) const;
  void define_Nx_Ny();
  void define_vol_inf();
  void define_area_for_solving();
  void define_rule_vectors();
  void apply_bodies();
  bool read_restart();
  // ======================= step pieces =======================
  void solve_rho_mid();
  void solve_fluxes();
  void solve_diffusion();
  void bc_velocities();
  void bc_slip_u();
  void bc_slip_v();
  void bc_pressure();
  void bc_pressure_begin_it();
  void bc_temperature();
  void bc_tjump();
  void bc_tjump_write();
  void bc_function_of_time();
  void pt_sweeps();
  void nondim_refresh();
  // ======================= driver =======================
  bool setup();
  void step();
  void write_solved();
  void write_temp();
  void write_drag();
  void solve_continuity();
  void write_iterations();
  void finish();
  std::string path(const std::string& f) const { return dir + "/" + f; }
};

template <class T>
static void rd(std::istream& in, T& v) {
  char buf[5000];
  in >> v;
  in.getline(buf, 5000, '\n');
}

bool Oracle::read_entered_data() {
  std::ifstream in(path("EnteredData.txt").c_str());
  if (!in.is_open()) {
    err = "cannot open EnteredData.txt";
    return false;
  }
  rd(in, u_gas_nd); rd(in, v_gas_nd); rd(in, T_gas_nd); rd(in, p_gas_nd);
  rd(in, Ma); rd(in, Pr); rd(in, gamma1); rd(in, c_mu); rd(in, Kn); rd(in, Fr);
  rd(in, SolveGravityField); rd(in, Re); rd(in, TypeND);
  rd(in, Nt); rd(in, Nx); rd(in, Ny); rd(in, N_I); rd(in, N_I_p_c); rd(in, N_I_T); rd(in, ht);
  rd(in, x_b); rd(in, x_e); rd(in, y_b); rd(in, y_e); rd(in, kind_of_mesh);
  rd(in, hxmin); rd(in, hxmax); rd(in, xfmin); rd(in, xfmax); rd(in, xbmin); rd(in, xbmax); rd(in, xmid);
  rd(in, hymin); rd(in, hymax); rd(in, ytmin); rd(in, ytmax); rd(in, ybmin); rd(in, ybmax); rd(in, ymid);
  rd(in, MaxError_Velocities); rd(in, MaxError_p_c); rd(in, MaxError_T); rd(in, MaxError_to_stop_program);
  rd(in, max_time_for_solve); rd(in, solve_is_finished);
  rd(in, Nt_save_solved_data); rd(in, Nt_save_DragCoefficient); rd(in, Nt_save_temp_data);
  rd(in, N_I_check); rd(in, WriteDataInShortFormat_kind);
  rd(in, ToReadSolvedDataFromFile); rd(in, ToReadSolvedDataFromBinaryFile);
  rd(in, ToWriteSolvedDataToBinaryFile); rd(in, ToWriteSolvedDataToNewFiles); rd(in, ToContinueFromInterpolation);
  rd(in, imp_circ_b); rd(in, imp_poly_b); rd(in, imp_circ_p); rd(in, imp_poly_p); rd(in, imp_circ_V);
  rd(in, imp_poly_V);
  rd(in, Given_velocity_on_xb); rd(in, Given_velocity_on_xe); rd(in, Periodic); rd(in, Pressure_BC);
  rd(in, ToStartFromExactSolution);
  rd(in, p_BC_xb_correction_method); rd(in, Pressure_ratio_correct); rd(in, GivenReKn); rd(in, correct_p_BC_xb);
  rd(in, u_given_xb); rd(in, u_given_xb_error); rd(in, p_correction_auto); rd(in, p_correction_min);
  rd(in, p_correction_max); rd(in, p_correction);
  rd(in, p_BC_xb); rd(in, T_BC_xb); rd(in, p_BC_xe); rd(in, T_BC_xe);
  rd(in, dudx_0_BC_xb); rd(in, durhodx_0_BC_xb); rd(in, drhodt_0_BC_xb); rd(in, calc_u_xb);
  rd(in, dudx_0_BC_xe); rd(in, durhodx_0_BC_xe); rd(in, drhodt_0_BC_xe); rd(in, calc_u_xe);
  rd(in, u_uMin_Mout_0_BC_xe);
  rd(in, dudy_0_BC_yb); rd(in, dudy_0_BC_ye);
  rd(in, dvdx_0_BC_xb); rd(in, calc_v_xb); rd(in, dvdx_0_BC_xe); rd(in, calc_v_xe);
  rd(in, dvdy_0_BC_yb); rd(in, dvdy_0_BC_ye);
  rd(in, dpdx_0_BC_xb); rd(in, calc_p_xb); rd(in, dpdx_0_BC_xe); rd(in, calc_p_xe);
  rd(in, dpdy_0_BC_yb); rd(in, dpdy_0_BC_ye);
  rd(in, dTdx_0_BC_xb); rd(in, calc_T_xb); rd(in, dTdx_0_BC_xe); rd(in, calc_T_xe);
  rd(in, dTdy_0_BC_yb); rd(in, dTdy_0_BC_ye);
  rd(in, To_Use_Kn_local_in_wall_BC); rd(in, ToSolveContinuityEquation);
  rd(in, use_interpolation_for_u_BC_by_time); rd(in, t_BC_b); rd(in, t_BC_e); rd(in, u_BC_xb_t_BC_b);
  rd(in, u_BC_xb_t_BC_e);
  rd(in, w_u); rd(in, w_v); rd(in, w_p); rd(in, w_Temper);
  rd(in, N_SubDomains_x); rd(in, N_SubDomains_y);
  rd(in, rd_sep); rd(in, wr_entire); rd(in, wr_sep); rd(in, only_nx_ny);
  if (!in) {
    err = "EnteredData.txt is truncated or malformed";
    return false;
  }
  return true;
}

// Objects_for_Solving.h:101-150 (circles) and :306-412 (polyhedrons)
bool Oracle::read_bodies(const char* fname, bool circles) {
  std::ifstream in(path(fname).c_str());
  if (!in.is_open()) {
    err = std::string("cannot open ") + fname;
    return false;
  }
  uint n = 0;
  rd(in, n);
  char buf[5000];
  for (uint c = 0; c < n; c++) {
    Body b;
    b.circle = circles;
    if (circles) {
      b.T = 1;
      in >> b.xc >> b.yc >> b.rc; in.getline(buf, 5000, '\n');
      in >> b.u >> b.v; in.getline(buf, 5000, '\n');
      rd(in, b.p); rd(in, b.T); rd(in, b.slip); rd(in, b.F_slip); rd(in, b.w_slip); rd(in, b.jump);
      rd(in, b.F_jump); rd(in, b.dTdn0); rd(in, b.drag);
    } else {
      uint nv = 0;
      rd(in, nv);
      in >> b.p1x >> b.p1y; in.getline(buf, 5000, '\n');
      in >> b.p2x >> b.p2y; in.getline(buf, 5000, '\n');
      in >> b.u >> b.v; in.getline(buf, 5000, '\n');
      rd(in, b.p); rd(in, b.T); rd(in, b.slip); rd(in, b.F_slip); rd(in, b.w_slip); rd(in, b.jump);
      rd(in, b.F_jump); rd(in, b.dTdn0); rd(in, b.drag);
      b.xs.resize(nv); b.ys.resize(nv);
      for (uint k = 0; k < nv; k++) in >> b.xs[k] >> b.ys[k];
    }
    if (!in) {
      err = std::string("truncated body file ") + fname;
      return false;
    }
    bodies.push_back(b);
  }
  if (circles) N_circles = n; else N_polygons = n;
  return true;
}

// hx_all & variants, SIMPLE_TS_MPI.cpp:4736-4842
double Oracle::hx_all(double x) const {
  double h;
  auto front = [&](double x) { return axf0 + axf1 * x + axf2 * x * x; };
  auto back = [&](double x) { return axb0 + axb1 * x + axb2 * x * x + axb3 * x * x * x; };
  auto front3 = [&](double x) { return axf0 + axf1 * x + axf2 * x * x + axf3 * x * x * x; };
  if (kind_of_mesh == 1) {
    if (x < xfmax) h = hxmax;
    else if ((xfmax <= x) && (x <= xfmin)) h = ((hxmin - hxmax) / (xfmin - xfmax)) * (x - xfmax) + hxmax;
    else if ((xfmin < x) && (x <= xmid)) h = ((hxmid - hxmin) / (xmid - xfmin)) * (x - xfmin) + hxmin;
    else if ((xmid < x) && (x <= xbmin)) h = ((hxmin - hxmid) / (xbmin - xmid)) * (x - xmid) + hxmid;
    else if ((xbmin < x) && (x <= xbmax)) h = ((hxmax - hxmin) / (xbmax - xbmin)) * (x - xbmin) + hxmin;
    else h = hxmax;
  } else if (kind_of_mesh == 2) {
    if (x < xfmax) h = hxmax;
    else if ((xfmax <= x) && (x <= xmid)) h = front(x);
    else if ((xmid < x) && (x <= xbmax)) h = back(x);
    else h = hxmax;
  } else if (kind_of_mesh == 3) {
    if (x < xfmax) h = hxmax;
    else if ((xfmax <= x) && (x <= xfmin)) h = ((hxmin - hxmax) / (xfmin - xfmax)) * (x - xfmax) + hxmax;
    else if ((xfmin < x) && (x <= xbmin)) h = hxmin;
    else if ((xbmin < x) && (x <= xbmax)) h = ((hxmax - hxmin) / (xbmax - xbmin)) * (x - xbmin) + hxmin;
    else h = hxmax;
  } else if (kind_of_mesh == 4) {
    if (x < xfmax) h = hxmax;
    else if ((xfmax <= x) && (x <= xfmin)) h = front(x);
    else if ((xfmin < x) && (x <= xbmin)) h = hxmin;
    else if ((xbmin < x) && (x <= xbmax)) h = back(x);
    else h = hxmax;
  } else {
    if (x < xfmax) h = hxmax;
    else if ((xfmax <= x) && (x <= xfmin)) h = front3(x);
    else if ((xfmin < x) && (x <= xbmin)) h = hxmin;
    else if ((xbmin < x) && (x <= xbmax)) h = back(x);
    else h = hxmax;
  }
  if (hxmax < h) h = hxmax;
  else if (h < hxmin) h = hxmin;
  return h;
}

// hy_all & variants, SIMPLE_TS_MPI.cpp:4845-4952
double Oracle::hy_all(double y) const {
  double h;
  auto top = [&](double y) { return ayt0 + ayt1 * y + ayt2 * y * y; };
  auto bottom = [&](double y) { return ayb0 + ayb1 * y + ayb2 * y * y; };
  auto top3 = [&](double y) { return ayt0 + ayt1 * y + ayt2 * y * y + ayt3 * y * y * y; };
  auto bottom3 = [&](double y) { return ayb0 + ayb1 * y + ayb2 * y * y + ayb3 * y * y * y; };
  if (kind_of_mesh == 1) {
    if (y < ybmax) h = hymax;
    else if ((ybmax <= y) && (y <= ybmin)) h = ((hymin - hymax) / (ybmin - ybmax)) * (y - ybmax) + hymax;
    else if ((ybmin < y) && (y <= ymid)) h = ((hymid - hymin) / (ymid - ybmin)) * (y - ybmin) + hymin;
    else if ((ymid < y) && (y <= ytmin)) h = ((hymin - hymid) / (ytmin - ymid)) * (y - ymid) + hymid;
    else if ((ytmin < y) && (y <= ytmax)) h = ((hymax - hymin) / (ytmax - ytmin)) * (y - ytmin) + hymin;
    else h = hymax;
  } else if (kind_of_mesh == 2) {
    if (y < ybmax) h = hymax;
    else if ((ybmax <= y) && (y <= ymid)) h = bottom(y);
    else if ((ymid < y) && (y <= ytmax)) h = top(y);
    else h = hymax;
  } else if (kind_of_mesh == 3) {
    if (y < ybmax) h = hymax;
    else if ((ybmax <= y) && (y <= ybmin)) h = ((hymin - hymax) / (ybmin - ybmax)) * (y - ybmax) + hymax;
    else if ((ybmin < y) && (y <= ytmin)) h = hymin;
    else if ((ytmin < y) && (y <= ytmax)) h = ((hymax - hymin) / (ytmax - ytmin)) * (y - ytmin) + hymin;
    else h = hymax;
  } else if (kind_of_mesh == 4) {
    if (y < ybmax) h = hymax;
    else if ((ybmax <= y) && (y <= ybmin)) h = bottom(y);
    else if ((ybmin < y) && (y <= ytmin)) h = hymin;
    else if ((ytmin < y) && (y <= ytmax)) h = top(y);
    else h = hymax;
  } else {
    if (y < ybmax) h = hymax;
    else if ((ybmax <= y) && (y <= ybmin)) h = bottom3(y);
    else if ((ybmin < y) && (y <= ytmin)) h = hymin;
    else if ((ytmin < y) && (y <= ytmax)) h = top3(y);
    else h = hymax;
  }
  if (hymax < h) h = hymax;
  else if (h < hymin) h = hymin;
  return h;
}

// define_Nx_Ny, SIMPLE_TS_MPI.cpp:4955-5041
void Oracle::define_Nx_Ny() {
  double tol = 5 * hxmax;
  for (;;) {
    double xe = x_b;
    for (uint c = 0; c < Nx; c++) xe = xe + hx_all(xe);
    double d = xe - x_e;
    if (std::fabs(d) > tol) {
      if (d < 0) Nx = Nx + int(std::fabs(d / hxmax));
      if (d > 0) {
        if ((Nx - int(std::fabs(d / hxmax))) > 2) Nx = Nx - int(std::fabs(d / hxmax));
        else Nx = int(0.75 * Nx);
      }
    } else break;
  }
  double toly = 5 * hxmax;  // the reference compares against 5*hxmax for y as well (:5002)
  for (;;) {
    double ye = y_b;
    for (uint c = 0; c < Ny; c++) ye = ye + hy_all(ye);
    double d = ye - y_e;
    if (std::fabs(d) > toly) {
      if (d < 0) Ny = Ny + int(std::fabs(d / hymax));
      if (d > 0) {
        if ((Ny - int(std::fabs(d / hymax))) > 2) Ny = Ny - int(std::fabs(d / hymax));
        else Ny = int(0.75 * Ny);
      }
    } else break;
  }
}

// mesh coefficients SIMPLE_TS_MPI.cpp:2078-2148 and mesh build :2165-2248
void Oracle::build_mesh() {
  if (kind_of_mesh == 2 || kind_of_mesh == 4) {
    xmid = xfmin + 0.5 * (xbmin - xfmin);
    axf2 = (hxmax - hxmin) / ((xfmax - xfmin) * (xfmax - xfmin));
    axf1 = -2.0 * axf2 * xfmin;
    axf0 = hxmin + axf2 * xfmin * xfmin;
    axb2 = (hxmax - hxmin) / ((xbmax - xbmin) * (xbmax - xbmin));
    axb1 = -2.0 * axb2 * xbmin;
    axb0 = hxmin + axb2 * xbmin * xbmin;
    {  // hxmid = hx_all_par(xmid)
      double x = xmid;
      if (x < xfmax) hxmid = hxmax;
      else if ((xfmax <= x) && (x <= xmid)) hxmid = axf0 + axf1 * x + axf2 * x * x;
      else if ((xmid < x) && (x <= xbmax)) hxmid = axb0 + axb1 * x + axb2 * x * x + axb3 * x * x * x;
      else hxmid = hxmax;
    }
    ymid = ybmin + 0.5 * (ytmin - ybmin);
    ayt2 = (hymax - hymin) / ((ytmax - ytmin) * (ytmax - ytmin));
    ayt1 = -2.0 * ayt2 * ytmin;
    ayt0 = hymin + ayt2 * ytmin * ytmin;
    ayb2 = (hymax - hymin) / ((ybmax - ybmin) * (ybmax - ybmin));
    ayb1 = -2.0 * ayb2 * ybmin;
    ayb0 = hymin + ayb2 * ybmin * ybmin;
    {
      double y = ymid;
      if (y < ybmax) hymid = hymax;
      else if ((ybmax <= y) && (y <= ymid)) hymid = ayb0 + ayb1 * y + ayb2 * y * y;
      else if ((ymid < y) && (y <= ytmax)) hymid = ayt0 + ayt1 * y + ayt2 * y * y;
      else hymid = hymax;
    }
  } else if (kind_of_mesh == 5) {
    double t = 1.0 / (3.0 * xfmax * std::pow(xfmin, 2) - std::pow(xfmin, 3) - 3.0 * std::pow(xfmax, 2) * xfmin +
                      std::pow(xfmax, 3));
    axf3 = 2.0 * (hxmin - hxmax) * t;
    axf2 = -3.0 * (xfmax + xfmin) * (hxmin - hxmax) * t;
    axf1 = 6.0 * xfmin * xfmax * (hxmin - hxmax) * t;
    axf0 = (-3.0 * hxmin * std::pow(xfmax, 2) * xfmin + hxmin * std::pow(xfmax, 3) +
            3.0 * hxmax * std::pow(xfmin, 2) * xfmax - hxmax * std::pow(xfmin, 3)) * t;
    t = 1.0 / (3.0 * xbmin * std::pow(xbmax, 2) - std::pow(xbmax, 3) - 3.0 * std::pow(xbmin, 2) * xbmax +
               std::pow(xbmin, 3));
    axb3 = 2.0 * (hxmax - hxmin) * t;
    axb2 = -3.0 * (xbmin + xbmax) * (hxmax - hxmin) * t;
    axb1 = 6.0 * xbmax * xbmin * (hxmax - hxmin) * t;
    axb0 = (-3.0 * hxmax * std::pow(xbmin, 2) * xbmax + hxmax * std::pow(xbmin, 3) +
            3.0 * hxmin * std::pow(xbmax, 2) * xbmin - hxmin * std::pow(xbmax, 3)) * t;
    // the y coefficients reuse hxmin/hxmax exactly as the reference does (:2131-2146)
    t = 1.0 / (3.0 * ybmax * std::pow(ybmin, 2) - std::pow(ybmin, 3) - 3.0 * std::pow(ybmax, 2) * ybmin +
               std::pow(ybmax, 3));
    ayb3 = 2.0 * (hxmin - hxmax) * t;
    ayb2 = -3.0 * (ybmax + ybmin) * (hxmin - hxmax) * t;
    ayb1 = 6.0 * ybmin * ybmax * (hxmin - hxmax) * t;
    ayb0 = (-3.0 * hxmin * std::pow(ybmax, 2) * ybmin + hxmin * std::pow(ybmax, 3) +
            3.0 * hxmax * std::pow(ybmin, 2) * ybmax - hxmax * std::pow(ybmin, 3)) * t;
    t = 1.0 / (3.0 * ytmin * std::pow(ytmax, 2) - std::pow(ytmax, 3) - 3.0 * std::pow(ytmin, 2) * ytmax +
               std::pow(ytmin, 3));
    ayt3 = 2.0 * (hxmax - hxmin) * t;
    ayt2 = -3.0 * (ytmin + ytmax) * (hxmax - hxmin) * t;
    ayt1 = 6.0 * ytmax * ytmin * (hxmax - hxmin) * t;
    ayt0 = (-3.0 * hxmax * std::pow(ytmin, 2) * ytmax + hxmax * std::pow(ytmin, 3) +
            3.0 * hxmin * std::pow(ytmax, 2) * ytmin - hxmin * std::pow(ytmax, 3)) * t;
  }
  if (!ToReadSolvedDataFromFile) define_Nx_Ny();
  Na = Nx * Ny;
  x_f.assign(Nx + 1, 0); y_f.assign(Ny + 1, 0);
  hx.assign(Nx, 0); hy.assign(Ny, 0); x_v.assign(Nx, 0); y_v.assign(Ny, 0);
  x_f[0] = x_b - 0.5 * hxmax;
  x_f[1] = x_b + 0.5 * hxmax;
  for (uint i = 1; i < Nx; i++) {
    double t = x_f[i] + 0.5 * hx_all(x_f[i]);
    x_f[i + 1] = x_f[i] + hx_all(t);
  }
  y_f[0] = y_b - 0.5 * hymax;
  y_f[1] = y_b + 0.5 * hymax;
  for (uint j = 1; j < Ny; j++) {
    double t = y_f[j] + 0.5 * hy_all(y_f[j]);
    y_f[j + 1] = y_f[j] + hy_all(t);
  }
  for (uint i = 0; i < Nx; i++) { hx[i] = x_f[i + 1] - x_f[i]; x_v[i] = x_f[i] + 0.5 * hx[i]; }
  for (uint j = 0; j < Ny; j++) { hy[j] = y_f[j + 1] - y_f[j]; y_v[j] = y_f[j] + 0.5 * hy[j]; }
  if (N_I_T > 0) {
    Iter_T = 0;
    do {
      for (uint i = 1; i < Nx; i++) x_f[i + 1] = x_f[i] + hx_all(x_v[i]);
      for (uint j = 1; j < Ny; j++) y_f[j + 1] = y_f[j] + hy_all(y_v[j]);
      for (uint i = 0; i < Nx; i++) { hx[i] = x_f[i + 1] - x_f[i]; x_v[i] = x_f[i] + 0.5 * hx[i]; }
      for (uint j = 0; j < Ny; j++) { hy[j] = y_f[j + 1] - y_f[j]; y_v[j] = y_f[j] + 0.5 * hy[j]; }
      Iter_T++;
    } while (Iter_T < N_I_T);
  }
}

// define_OforS + define_vol_inf (body part), SIMPLE_TS_MPI.cpp:6269-6360
void Oracle::define_vol_inf() {
  vol_inf_fb.assign(Na, 0);
  if (!(imp_circ_b || imp_poly_b)) return;
  for (uint c = 0; c < N_circles; c++)
    for (uint j = 0; j < Ny; j++)
      for (uint i = 0; i < Nx; i++)
        if (point_in_circle(bodies[c], x_v[i], y_v[j])) vol_inf_fb[i + j * Nx] = 1 + c;
  for (uint c = 0; c < N_polygons; c++)
    for (uint j = 0; j < Ny; j++)
      for (uint i = 0; i < Nx; i++)
        if (point_in_polygon(bodies[N_circles + c], x_v[i], y_v[j])) vol_inf_fb[i + j * Nx] = 1 + N_circles + c;
}

// define_area_for_solving, SIMPLE_TS_MPI.cpp:6009-6191 (serial branches)
void Oracle::define_area_for_solving() {
  if (Periodic) { Nx_u[0] = 0; Nx_v[0] = 0; Nx_o[0] = 0; }
  else if (Pressure_BC) { Nx_u[0] = 1; Nx_v[0] = 1; Nx_o[0] = 1; }
  else if (Given_velocity_on_xb) { Nx_u[0] = 2; Nx_v[0] = 1; Nx_o[0] = 1; }
  else { Nx_u[0] = 1; Nx_v[0] = 1; Nx_o[0] = 1; }
  if (Periodic) { Nx_u[1] = Nx; Nx_v[1] = Nx; Nx_o[1] = Nx; }
  else if (Pressure_BC) { Nx_u[1] = Nx - 1; Nx_v[1] = Nx - 2; Nx_o[1] = Nx - 2; }
  else if (Given_velocity_on_xe) { Nx_u[1] = Nx - 1; Nx_v[1] = Nx - 2; Nx_o[1] = Nx - 1; }
  else { Nx_u[1] = Nx - 1; Nx_v[1] = Nx - 2; Nx_o[1] = Nx - 2; }
  Ny_u[0] = 1; Ny_v[0] = 1; Ny_o[0] = 1;
  Ny_u[1] = Ny - 2; Ny_v[1] = Ny - 1; Ny_o[1] = Ny - 2;
}

// define_rule_vectors, SIMPLE_TS_MPI.cpp:8581-9063 and :10158-10379
void Oracle::define_rule_vectors() {
  vol.assign(Na, 0);
  for (uint c = 0; c < Na; c++) vol[c] = (vol_inf_fb[c] == 0);
  const uint J1 = 1, J_1 = 2, I1 = 1, I_1 = 2;  // BlockLengthSwap_*, SIMPLE_TS_MPI.cpp:1277-1287
  auto idx = [&](uint i, uint j) { return Periodic ? periodic(i, j) : clamped(i, j); };
  auto inner = [&](uint i, uint j) {
    return ((Ny_u[0] + J1) < j) && (j < (Ny_u[1] - J_1)) && ((Nx_u[0] + I1) < i) && (i < (Nx_u[1] - I_1));
  };
  nch_u.clear(); bc_u.clear(); nch_v.clear(); bc_v.clear(); nch_o.clear(); bc_o.clear();
  for (uint j = Ny_u[0]; j < Ny_u[1]; j++)
    for (uint i = Nx_u[0]; i < Nx_u[1]; i++) {
      Idx d = idx(i, j);
      bool nb = vol[d.i_1j_1] && vol[d.ij_1] && vol[d.i_1j1] && vol[d.ij1] && vol[d.i1j] && vol[d.i_2j];
      if (inner(i, j) && vol[d.i_1j] && vol[d.ij] && nb) nch_u.push_back(d.ij);
      if (vol[d.i_1j] && vol[d.ij] && (!inner(i, j) || !nb)) bc_u.push_back(d.ij);
    }
  for (uint j = Ny_v[0]; j < Ny_v[1]; j++)
    for (uint i = Nx_v[0]; i < Nx_v[1]; i++) {
      Idx d = idx(i, j);
      uint far = d.ij_1 - Nx * (0 <= (int)(j - 2));
      bool nb = vol[d.i_1j_1] && vol[d.i_1j] && vol[d.i1j_1] && vol[d.i1j] && vol[far] && vol[d.ij1];
      if (inner(i, j) && vol[d.ij_1] && vol[d.ij] && nb) nch_v.push_back(d.ij);
      if (vol[d.ij_1] && vol[d.ij] && (!inner(i, j) || !nb)) bc_v.push_back(d.ij);
    }
  for (uint j = Ny_o[0]; j < Ny_o[1]; j++)
    for (uint i = Nx_o[0]; i < Nx_o[1]; i++) {
      Idx d = idx(i, j);
      bool nb = vol[d.i_1j] && vol[d.i1j] && vol[d.ij_1] && vol[d.ij1] && vol[d.i_1j_1] && vol[d.i_1j1] &&
                vol[d.i1j_1] && vol[d.i1j1];
      if (inner(i, j) && vol[d.ij] && nb) nch_o.push_back(d.ij);
      if (vol[d.ij] && (!inner(i, j) || !nb)) bc_o.push_back(d.ij);
    }
  slip_u.clear(); slip_v.clear(); tjump.clear();
  for (uint j = 0; j < Ny; j++)
    for (uint i = 0; i < Nx; i++) {
      Idx d = idx(i, j);
      if ((0 < vol_inf_fb[d.ij]) && ((0 == vol_inf_fb[d.ij_1]) || (0 == vol_inf_fb[d.ij1]))) slip_u.push_back(d.ij);
    }
  for (uint j = 0; j < Ny; j++)
    for (uint i = 0; i < Nx; i++) {
      Idx d = idx(i, j);
      if ((0 < vol_inf_fb[d.ij]) && ((0 == vol_inf_fb[d.i_1j]) || (0 == vol_inf_fb[d.i1j]))) slip_v.push_back(d.ij);
    }
  for (uint j = 0; j < Ny; j++)
    for (uint i = 0; i < Nx; i++) {
      Idx d = idx(i, j);
      if (vol[d.ij] && ((!vol[d.i_1j]) || (!vol[d.i1j]) || (!vol[d.ij_1]) || (!vol[d.ij1]))) tjump.push_back(d.ij);
    }
}

// ApplyBodiesConditionsToVariables, SIMPLE_TS_MPI.cpp:6470-6584
void Oracle::apply_bodies() {
  for (uint i = 0; i < Nx; i++)
    for (uint j = 0; j < Ny; j++) {
      Idx d = clamped(i, j);
      if (1 <= vol_inf_fb[d.ij]) {
        const Body& b = bodies[vol_inf_fb[d.ij] - 1];
        u[d.ij] = b.u;
        u[d.i1j] = b.u;
      }
    }
  for (uint i = 0; i < Nx; i++)
    for (uint j = 0; j < Ny; j++) {
      Idx d = clamped(i, j);
      if (1 <= vol_inf_fb[d.ij]) {
        const Body& b = bodies[vol_inf_fb[d.ij] - 1];
        v[d.ij] = b.v;
        v[d.ij1] = b.v;
      }
    }
  for (uint i = 0; i < Nx; i++)
    for (uint j = 0; j < Ny; j++) {
      uint n = i + j * Nx;
      if (1 <= vol_inf_fb[n]) {
        const Body& b = bodies[vol_inf_fb[n] - 1];
        p[n] = b.p;
        Temper[n] = b.T;
        if (vol[n]) rho[n] = p[n] / Temper[n];
        else rho[n] = 0;
      }
    }
}

static bool read_bin(const std::string& f, void* dst, size_t bytes) {
  std::ifstream in(f.c_str(), std::ios::in | std::ios::binary);
  if (!in.is_open()) return false;
  in.read((char*)dst, bytes);
  return true;
}

// ReadSolvedDataFromFile (binary and text), SIMPLE_TS_MPI.cpp:5734-5835; Read_it_FromFile :6762-6787
bool Oracle::read_restart() {
  const char* names[4] = {"u", "v", "p", "Temper"};
  double* dst[4] = {u, v, p, Temper};
  if (ToReadSolvedDataFromBinaryFile) {
    for (int k = 0; k < 4; k++)
      if (!read_bin(path(std::string(names[k]) + ".bin"), dst[k], sizeof(double) * Na)) {
        err = std::string("cannot open ") + names[k] + ".bin";
        return false;
      }
    if (!read_bin(path("vol_inf_fb.bin"), vol_inf_fb.data(), sizeof(uint) * Na)) {
      err = "cannot open vol_inf_fb.bin";
      return false;
    }
  } else {
    for (int k = 0; k < 4; k++) {
      std::ifstream in(path(std::string(names[k]) + ".txt").c_str());
      if (!in.is_open()) { err = std::string("cannot open ") + names[k] + ".txt"; return false; }
      for (uint c = 0; c < Na; c++) in >> dst[k][c];
    }
    std::ifstream in(path("vol_inf_fb.txt").c_str());
    if (!in.is_open()) { err = "cannot open vol_inf_fb.txt"; return false; }
    for (uint c = 0; c < Na; c++) in >> vol_inf_fb[c];
  }
  for (uint c = 0; c < Na; c++) {
    if (vol[c]) rho[c] = p[c] / Temper[c];
    else rho[c] = 0;
  }
  solve_rho_mid();
  std::ifstream in(path("it_begin.txt").c_str());
  if (in.is_open()) { in >> it_begin; it = it_begin; }
  return true;
}

// Solve_rho_in_middle_points, SIMPLE_TS_MPI.cpp:10382-10437
void Oracle::solve_rho_mid() {
  for (uint j = 0; j < Ny; j++)
    for (uint i = 0; i < Nx; i++) {
      Idx d = Periodic ? periodic(i, j) : clamped(i, j);
      if (vol[d.i_1j] && vol[d.ij]) rho_u[d.ij] = upwind_rho(rho[d.i_1j], rho[d.ij], u[d.ij]);
      else if (vol[d.i_1j] != vol[d.ij]) rho_u[d.ij] = (vol[d.i_1j] ? rho[d.i_1j] : rho[d.ij]);
      else rho_u[d.ij] = 0.0;
      if (vol[d.ij_1] && vol[d.ij]) rho_v[d.ij] = upwind_rho(rho[d.ij_1], rho[d.ij], v[d.ij]);
      else if (vol[d.ij_1] != vol[d.ij]) rho_v[d.ij] = (vol[d.ij_1] ? rho[d.ij_1] : rho[d.ij]);
      else rho_v[d.ij] = 0.0;
    }
}

// SolveFluxes, SIMPLE_TS_MPI.cpp:10440-10454
void Oracle::solve_fluxes() {
  for (uint j = 0; j < Ny; j++)
    for (uint i = 0; i < Nx; i++) {
      uint n = i + j * Nx;
      Fx[n] = hy[j] * rho_u[n] * u[n];
      Fy[n] = hx[i] * rho_v[n] * v[n];
    }
}

// SolveDiffisionTerms, SIMPLE_TS_MPI.cpp:10457-10618
void Oracle::solve_diffusion() {
  const std::vector<char>& b = vol;
  for (uint j = 0; j < Ny; j++)
    for (uint i = 0; i < Nx; i++) {
      Idx d = Periodic ? periodic(i, j) : clamped(i, j);
      const uint jm = j - 1 * (0 < j);
      if (b[d.i_1j_1] && b[d.ij_1] && b[d.i_1j] && b[d.ij]) {
        Gamma_yf[d.ij] = 0.5 * (Li(sqrt_T[d.i_1j_1], sqrt_T[d.i_1j], hy[jm], hy[j]) +
                                Li(sqrt_T[d.ij_1], sqrt_T[d.ij], hy[jm], hy[j]));
      } else if (b[d.i_1j_1] || b[d.ij_1] || b[d.i_1j] || b[d.ij]) {
        Gamma_yf[d.ij] =
            0.5 * ((b[d.i_1j_1] && b[d.i_1j]) * Li(sqrt_T[d.i_1j_1], sqrt_T[d.i_1j], hy[jm], hy[j]) +
                   (b[d.i_1j_1] != b[d.i_1j]) * std::sqrt(Tw_v[d.i_1j]) +
                   (b[d.ij_1] && b[d.ij]) * Li(sqrt_T[d.ij_1], sqrt_T[d.ij], hy[jm], hy[j]) +
                   (b[d.ij_1] != b[d.ij]) * std::sqrt(Tw_v[d.ij]) +
                   ((!(b[d.i_1j_1] && b[d.i_1j])) || (!(b[d.ij_1] && b[d.ij]))) *
                       Li(std::sqrt(Tw_u[d.ij_1]), std::sqrt(Tw_u[d.ij]), hy[jm], hy[j]));
      }
      D_ux[d.ij] = cT * sqrt_T[d.i_1j] * (hy[j] / hx[d.i_1]);
      if ((b[d.ij] && b[d.i_1j]) || (b[d.ij_1] && b[d.i_1j_1])) {
        D_uy[d.ij] = cT * Gamma_yf[d.ij] *
                     ((hx[i] + hx[d.i_1]) / (b[d.ij] * b[d.i_1j] * hy[j] + b[d.ij_1] * b[d.i_1j_1] * hy[jm]));
      } else {
        D_uy[d.ij] = 0;
      }
      if (b[d.i_1j_1] && b[d.ij_1] && b[d.i_1j] && b[d.ij]) {
        Gamma_xf[d.ij] = 0.5 * (Li(sqrt_T[d.i_1j_1], sqrt_T[d.ij_1], hx[d.i_1], hx[i]) +
                                Li(sqrt_T[d.i_1j], sqrt_T[d.ij], hx[d.i_1], hx[i]));
      } else if (b[d.i_1j_1] || b[d.ij_1] || b[d.i_1j] || b[d.ij]) {
        Gamma_xf[d.ij] =
            0.5 * ((b[d.i_1j_1] && b[d.ij_1]) * Li(sqrt_T[d.i_1j_1], sqrt_T[d.ij_1], hx[d.i_1], hx[i]) +
                   (b[d.i_1j_1] != b[d.ij_1]) * std::sqrt(Tw_u[d.ij_1]) +
                   (b[d.i_1j] && b[d.ij]) * Li(sqrt_T[d.i_1j], sqrt_T[d.ij], hx[d.i_1], hx[i]) +
                   (b[d.i_1j] != b[d.ij]) * std::sqrt(Tw_u[d.ij]) +
                   ((!(b[d.i_1j_1] && b[d.ij_1])) || (!(b[d.i_1j] && b[d.ij]))) *
                       Li(std::sqrt(Tw_v[d.i_1j]), std::sqrt(Tw_v[d.ij]), hx[d.i_1], hx[i]));
      }
      if ((b[d.ij] && b[d.ij_1]) || (b[d.i_1j] && b[d.i_1j_1])) {
        D_vx[d.ij] = cT * Gamma_xf[d.ij] *
                     ((hy[j] + hy[jm]) / (b[d.ij] * b[d.ij_1] * hx[i] + b[d.i_1j] * b[d.i_1j_1] * hx[d.i_1]));
      } else {
        D_vx[d.ij] = 0;
      }
      D_vy[d.ij] = cT * sqrt_T[d.ij_1] * (hx[i] / hy[jm]);
      if (b[d.ij] || b[d.i_1j]) {
        DTx[d.ij] = cT1 * (hy[j] / (0.5 * (b[d.ij] * hx[i] + b[d.i_1j] * hx[d.i_1]))) *
                    (((!b[d.ij]) || (!b[d.i_1j])) * std::sqrt(Tw_u[d.ij]) +
                     b[d.ij] * b[d.i_1j] * Hi(sqrt_T[d.i_1j], sqrt_T[d.ij], hx[d.i_1], hx[i]));
      } else {
        DTx[d.ij] = 0;
      }
      if (b[d.ij] || b[d.ij_1]) {
        DTy[d.ij] = cT1 * (hx[i] / (0.5 * (b[d.ij] * hy[j] + b[d.ij_1] * hy[jm]))) *
                    (((!b[d.ij]) || (!b[d.ij_1])) * std::sqrt(Tw_v[d.ij]) +
                     b[d.ij] * b[d.ij_1] * Hi(sqrt_T[d.ij_1], sqrt_T[d.ij], hy[jm], hy[j]));
      } else {
        DTy[d.ij] = 0;
      }
    }
}

// BoundaryConditions_Velocities, SIMPLE_TS_MPI.cpp:6790-7096 (serial path)
void Oracle::bc_velocities() {
  if (Periodic) return;
  if (dvdx_0_BC_xb)
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_v[0] + j * Nx;
      for (uint i = 0; i < Nx_v[0]; i++) if (vol[n]) v[i + j * Nx] = v[n];
    }
  if (dvdx_0_BC_xe)
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_v[1] - 1 + j * Nx;
      for (uint i = Nx_v[1]; i < Nx; i++) if (vol[n]) v[i + j * Nx] = v[n];
    }
  if (dvdy_0_BC_yb)
    for (uint i = 0; i < Nx; i++) {
      uint n = i + Ny_v[0] * Nx;
      for (uint j = 0; j < Ny_v[0]; j++) if (vol[n]) v[i + j * Nx] = v[n];
    }
  if (dvdy_0_BC_ye)
    for (uint i = 0; i < Nx; i++) {
      uint n = i + (Ny_v[1] - 1) * Nx;
      for (uint j = Ny_v[1]; j < Ny; j++) if (vol[n]) v[i + j * Nx] = v[n];
    }
  if (dudx_0_BC_xb)
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_u[0] + j * Nx;
      for (uint i = 0; i < Nx_u[0]; i++) if (vol[n]) u[i + j * Nx] = u[n];
    }
  if (durhodx_0_BC_xb)
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_u[0] - 1 + j * Nx;
      if (vol[n]) u[n] = (rho_u[n + 1] * u[n + 1]) / rho_u[n];
    }
  if (drhodt_0_BC_xb) {
    uint i = Nx_u[0] - 1;
    for (uint j = 0; j < Ny; j++) {
      uint n = i + j * Nx;
      if (vol[n])
        u[n] = ((rho[n] - rho_pr[n]) * hx[i] * hy[j] / ht + (rho_v[n + Nx] * v[n + Nx] - rho_v[n] * v[n]) * hx[i] +
                rho_u[n + 1] * u[n + 1] * hy[j]) /
               (rho_u[n] * hy[j]);
    }
  }
  if (dudx_0_BC_xe)
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_u[1] - 1 + j * Nx;
      for (uint i = Nx_u[1]; i < Nx; i++) if (vol[n]) u[i + j * Nx] = u[n];
    }
  if (durhodx_0_BC_xe)
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_u[1] - 1 + j * Nx;
      if (vol[n]) u[n + 1] = (rho_u[n] * u[n]) / rho_u[n + 1];
    }
  if (drhodt_0_BC_xe) {
    uint i = Nx_u[1] - 1;
    for (uint j = 0; j < Ny; j++) {
      uint n = i + j * Nx;
      if (vol[n])
        u[n + 1] = (-(rho[n] - rho_pr[n]) * hx[i] * hy[j] / ht - (rho_v[n + Nx] * v[n + Nx] - rho_v[n] * v[n]) * hx[i] +
                    rho_u[n] * u[n] * hy[j]) /
                   (rho_u[n + 1] * hy[j]);
    }
  }
  if (u_uMin_Mout_0_BC_xe) {  // serial only, :7018-7055 (keeps the last row's value, as written)
    double Min = 0, Mout = 0;
    for (uint j = 0; j < Ny; j++) Min = rho_u[Nx_u[0] + j * Nx];
    for (uint j = 0; j < Ny; j++) Mout = rho_u[Nx_u[1] + j * Nx];
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_u[1] - 1 + j * Nx;
      u[n + 1] = u[n] * Min / Mout;
    }
  }
  if (dudy_0_BC_yb)
    for (uint i = 0; i < Nx; i++) {
      uint n = i + Ny_u[0] * Nx;
      for (uint j = 0; j < Ny_u[0]; j++) if (vol[n]) u[i + j * Nx] = u[n];
    }
  if (dudy_0_BC_ye)
    for (uint i = 0; i < Nx; i++) {
      uint n = i + (Ny_u[1] - 1) * Nx;
      for (uint j = Ny_u[1]; j < Ny; j++) if (vol[n]) u[i + j * Nx] = u[n];
    }
}

// BoundaryConditions_Velocities_SlipBC_u, SIMPLE_TS_MPI.cpp:7098-7213
void Oracle::bc_slip_u() {
  for (size_t c = 0; c < slip_u.size(); c++) {
    Idx d = bc_idx(slip_u[c]);
    uint id = vol_inf_fb[d.ij];
    if (id < 1) continue;
    const Body& B = bodies[id - 1];
    if (!B.slip) continue;
    double a_ij, a_i1j;
    if (0 == vol_inf_fb[d.ij_1]) {
      uint jm = d.j - 1 * (0 < d.j);
      if (To_Use_Kn_local_in_wall_BC) {
        a_ij = (B.F_slip * Kn) / (rho_u[d.ij_1] * 0.5 * hy[jm]);
        a_i1j = (B.F_slip * Kn) / (rho_u[d.i1j_1] * 0.5 * hy[jm]);
      } else {
        a_ij = (B.F_slip * Kn) / (0.5 * hy[jm]);
        a_i1j = (B.F_slip * Kn) / (0.5 * hy[jm]);
      }
      if (vol[d.i_1j_1]) u[d.ij] = (u[d.ij_1] * a_ij + B.u) / (1.0 + a_ij);
      if (vol[d.i1j_1]) u[d.i1j] = (u[d.i1j_1] * a_i1j + B.u) / (1.0 + a_i1j);
    } else {
      uint jp = d.j + 1 * (d.j < (Ny - 1));
      if (To_Use_Kn_local_in_wall_BC) {
        a_ij = (B.F_slip * Kn) / (rho_u[d.ij1] * 0.5 * hy[jp]);
        a_i1j = (B.F_slip * Kn) / (rho_u[d.i1j1] * 0.5 * hy[jp]);
      } else {
        a_ij = (B.F_slip * Kn) / (0.5 * hy[jp]);
        a_i1j = (B.F_slip * Kn) / (0.5 * hy[jp]);
      }
      if (vol[d.i_1j1]) u[d.ij] = (u[d.ij1] * a_ij + B.u) / (1.0 + a_ij);
      if (vol[d.i1j1]) u[d.i1j] = (u[d.i1j1] * a_i1j + B.u) / (1.0 + a_i1j);
    }
  }
}

// BoundaryConditions_Velocities_SlipBC_v, SIMPLE_TS_MPI.cpp:7216-7331
void Oracle::bc_slip_v() {
  for (size_t c = 0; c < slip_v.size(); c++) {
    Idx d = bc_idx(slip_v[c]);
    uint id = vol_inf_fb[d.ij];
    if (id < 1) continue;
    const Body& B = bodies[id - 1];
    if (!B.slip) continue;
    double a_ij, a_ij1;
    if (0 == vol_inf_fb[d.i_1j]) {
      if (To_Use_Kn_local_in_wall_BC) {
        a_ij = (B.F_slip * Kn) / (rho_v[d.i_1j] * 0.5 * hx[d.i_1]);
        a_ij1 = (B.F_slip * Kn) / (rho_v[d.i_1j1] * 0.5 * hx[d.i_1]);
      } else {
        a_ij = (B.F_slip * Kn) / (0.5 * hx[d.i_1]);
        a_ij1 = (B.F_slip * Kn) / (0.5 * hx[d.i_1]);
      }
      if (vol[d.i_1j_1]) v[d.ij] = (v[d.i_1j] * a_ij + B.v) / (1.0 + a_ij);
      if (vol[d.i_1j1]) v[d.ij1] = (v[d.i_1j1] * a_ij1 + B.v) / (1.0 + a_ij1);
    } else {
      if (To_Use_Kn_local_in_wall_BC) {
        a_ij = (B.F_slip * Kn) / (rho_v[d.i1j] * 0.5 * hx[d.i1]);
        a_ij1 = (B.F_slip * Kn) / (rho_v[d.i1j1] * 0.5 * hx[d.i1]);
      } else {
        a_ij = (B.F_slip * Kn) / (0.5 * hx[d.i1]);
        a_ij1 = (B.F_slip * Kn) / (0.5 * hx[d.i1]);
      }
      if (vol[d.i1j_1]) v[d.ij] = (v[d.i1j] * a_ij + B.v) / (1.0 + a_ij);
      if (vol[d.i1j1]) v[d.ij1] = (v[d.i1j1] * a_ij1 + B.v) / (1.0 + a_ij1);
    }
  }
}

// BoundaryConditions_Pressure, SIMPLE_TS_MPI.cpp:7335-7428
void Oracle::bc_pressure() {
  if (Periodic) return;
  if (dpdx_0_BC_xb)
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_o[0] + j * Nx;
      for (uint i = 0; i < Nx_o[0]; i++) if (vol[n]) p[i + j * Nx] = p[n];
    }
  if (dpdx_0_BC_xe)
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_o[1] - 1 + j * Nx;
      for (uint i = Nx_o[1]; i < Nx; i++) if (vol[n]) p[i + j * Nx] = p[n];
    }
  if (dpdy_0_BC_yb)
    for (uint i = 0; i < Nx; i++) {
      uint n = i + Ny_o[0] * Nx;
      for (uint j = 0; j < Ny_o[0]; j++) if (vol[n]) p[i + j * Nx] = p[n];
    }
  if (dpdy_0_BC_ye)
    for (uint i = 0; i < Nx; i++) {
      uint n = i + (Ny_o[1] - 1) * Nx;
      for (uint j = Ny_o[1]; j < Ny; j++) if (vol[n]) p[i + j * Nx] = p[n];
    }
}

// BoundaryConditions_Pressure_begin_iteration_for_it, SIMPLE_TS_MPI.cpp:7430-7647 (serial path)
void Oracle::bc_pressure_begin_it() {
  if (Periodic) return;
  uint i = Nx_u[0];
  u_given_xb_in_it_max = u[0];
  for (uint j = 0; j < Ny; j++) {
    uint n = i + j * Nx;
    if (vol[n]) u_given_xb_in_it_max = dmax(u_given_xb_in_it_max, u[n]);
  }
  double h_in = 0;
  u_given_xb_in_it_mean = 0;
  for (uint j = 0; j < Ny; j++) {
    uint n = i + j * Nx;
    if (vol[n]) { u_given_xb_in_it_mean += u[n] * hy[j]; h_in += hy[j]; }
  }
  u_given_xb_in_it_mean = u_given_xb_in_it_mean / h_in;
  if (GivenReKn) u_given_xb = Re * Kn * std::sqrt(15.0 * M_PI / 128.0);
  if (p_BC_xb_correction_method == 0) {
    u_given_xb_in_it = u_given_xb;
    if (Given_velocity_on_xb) {
      uint ii = Nx_o[0];
      uint jj = int((Ny_o[1] - 1.0) - Ny_o[0]);
      p_BC_xb = p[ii + jj * Nx];
    }
  } else if (p_BC_xb_correction_method == 1) {
    u_given_xb_in_it = u_given_xb_in_it_max;
  } else if (p_BC_xb_correction_method == 2) {
    u_given_xb_in_it = u_given_xb_in_it_mean;
  }
  if (Pressure_BC && Pressure_ratio_correct) {
    if (p_correction_auto) {
      double t;
      double r = std::sqrt(max_residual_in_u * max_residual_in_u + max_residual_in_v * max_residual_in_v);
      if (Iter_pr1 <= Iter_pr2 && Iter_pr1 < (N_I - 1)) t = p_correction * (1.0 + r);
      else t = p_correction * (1.0 - r);
      if (t < p_correction_min) t = p_correction_min;
      else if (p_correction_max < t) t = p_correction_max;
      p_correction = t;
    }
    double du = (u_given_xb - u_given_xb_in_it);
    if (u_given_xb_in_it < (u_given_xb * (1.0 - u_given_xb_error))) {
      if (correct_p_BC_xb) {
        p_BC_xb = p_BC_xb * (1.0 + p_correction * (u_given_xb - u_given_xb_in_it) * (u_given_xb - u_given_xb_in_it));
      } else {
        double t = p_BC_xe * (1.0 - p_correction * (u_given_xb - u_given_xb_in_it) * (u_given_xb - u_given_xb_in_it));
        p_BC_xe = (t < 0.0) ? 0.0 : t;
      }
    } else if ((u_given_xb * (1.0 + u_given_xb_error)) < u_given_xb_in_it) {
      if (correct_p_BC_xb) {
        double t = p_BC_xb * (1.0 - p_correction * (u_given_xb - u_given_xb_in_it) * (u_given_xb - u_given_xb_in_it));
        p_BC_xb = (t > p_BC_xe) ? t : p_BC_xe;
      } else {
        double t = p_BC_xb * (1.0 + p_correction * (u_given_xb - u_given_xb_in_it) * (u_given_xb - u_given_xb_in_it));
        p_BC_xe = (t > p_BC_xb) ? p_BC_xb : t;
      }
    }
    (void)du;
    if (correct_p_BC_xb) {
      for (uint j = 0; j < Ny; j++)
        for (uint ii = 0; ii < Nx_o[0]; ii++) {
          uint n = ii + j * Nx;
          if (vol[n]) { p[n] = p_BC_xb; rho[n] = p_BC_xb / T_BC_xb; }
        }
    } else {
      for (uint j = 0; j < Ny; j++)
        for (uint ii = Nx_o[1]; ii < Nx; ii++) {
          uint n = ii + j * Nx;
          if (vol[n]) { p[n] = p_BC_xe; rho[n] = p_BC_xe / T_BC_xe; }
        }
    }
  }
}

// BoundaryConditions_Temperature, SIMPLE_TS_MPI.cpp:7650-7741
void Oracle::bc_temperature() {
  if (Periodic) return;
  if (dTdx_0_BC_xb)
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_o[0] + j * Nx;
      for (uint i = 0; i < Nx_o[0]; i++) if (vol[n]) Temper[i + j * Nx] = Temper[n];
    }
  if (dTdx_0_BC_xe)
    for (uint j = 0; j < Ny; j++) {
      uint n = Nx_o[1] - 1 + j * Nx;
      for (uint i = Nx_o[1]; i < Nx; i++) if (vol[n]) Temper[i + j * Nx] = Temper[n];
    }
  if (dTdy_0_BC_yb)
    for (uint i = 0; i < Nx; i++) {
      uint n = i + Ny_o[0] * Nx;
      for (uint j = 0; j < Ny_o[0]; j++) if (vol[n]) Temper[i + j * Nx] = Temper[n];
    }
  if (dTdy_0_BC_ye)
    for (uint i = 0; i < Nx; i++) {
      uint n = i + (Ny_o[1] - 1) * Nx;
      for (uint j = Ny_o[1]; j < Ny; j++) if (vol[n]) Temper[i + j * Nx] = Temper[n];
    }
}

// BoundaryConditions_Temperature_TemperatureJumpBC, SIMPLE_TS_MPI.cpp:7744-8045
void Oracle::bc_tjump() {
  for (size_t c = 0; c < tjump.size(); c++) {
    Idx d = bc_idx(tjump[c]);
    // the four neighbours in the order the reference visits them; h = hx for x faces, hy for y faces
    const uint nb[4] = {d.i_1j, d.i1j, d.ij_1, d.ij1};
    const uint dst[4] = {d.ij, d.i1j, d.ij, d.ij1};
    for (int k = 0; k < 4; k++) {
      if (vol[nb[k]]) continue;
      uint id = vol_inf_fb[nb[k]];
      bool jump = false;
      double Tb = 0, dTdn0 = 0, Fj = 0;
      if (id >= 1) {
        const Body& B = bodies[id - 1];
        Tb = B.T; jump = B.jump; dTdn0 = B.dTdn0; Fj = B.F_jump;
      }
      double* out = (k < 2) ? Tw_u.data() : Tw_v.data();
      if (jump) {
        double FK = To_Use_Kn_local_in_wall_BC ? (Fj * Kn) / rho[d.ij] : Fj * Kn;
        double a = FK / (0.5 * ((k < 2) ? hx[d.i] : hy[d.j]));
        out[dst[k]] = (a * Temper[d.ij] + Tb) / (1.0 + a);
      } else if (dTdn0) {
        out[dst[k]] = Temper[d.ij];
      } else {
        out[dst[k]] = Tb;
      }
    }
  }
}

// BoundaryConditions_Temperature_TemperatureJumpBC_WriteToMassiveToWriteDataToFile, :8048-8099
void Oracle::bc_tjump_write() {
  bc_tjump();
  for (size_t c = 0; c < tjump.size(); c++) {
    Idx d = bc_idx(tjump[c]);
    if (!vol[d.i_1j]) Temper[d.i_1j] = Tw_u[d.ij];
    if (!vol[d.i1j]) Temper[d.i1j] = Tw_u[d.i1j];
    if (!vol[d.ij_1]) Temper[d.ij_1] = Tw_v[d.ij];
    if (!vol[d.ij1]) Temper[d.ij1] = Tw_v[d.ij1];
  }
}

// BoundaryConditions_function_of_time, SIMPLE_TS_MPI.cpp:8102-8144
void Oracle::bc_function_of_time() {
  if (Periodic || !use_interpolation_for_u_BC_by_time) return;
  if (it <= t_BC_b) u_gas_nd = u_BC_xb_t_BC_b;
  else if (t_BC_b < it && it <= t_BC_e)
    u_gas_nd = ((u_BC_xb_t_BC_e - u_BC_xb_t_BC_b) / (t_BC_e - t_BC_b)) * (it - t_BC_b) + u_BC_xb_t_BC_b;
  else u_gas_nd = u_BC_xb_t_BC_e;
  u_given_xb = u_gas_nd;
  for (uint j = 0; j < Ny; j++)
    for (uint i = 0; i < Nx_u[0]; i++)
      if (vol[i + j * Nx]) u[i + j * Nx] = u_gas_nd;
}

// cT / cPch refresh, SIMPLE_TS_MPI.cpp:3043-3057 and :4347-4361
void Oracle::nondim_refresh() {
  if (TypeND == 1) {
    cT = (1.0 / Re) * (u_given_xb_in_it * p_BC_xb / T_BC_xb);
    cPch = 0.5;
  } else if (TypeND == 2) {
    cT = (1.0 / Re) * (u_given_xb_in_it * p_BC_xb / T_BC_xb);
    cPch = u_given_xb_in_it * u_given_xb_in_it / (gamma1 * Ma * Ma);
  } else if (TypeND == 3) {
    cT = Kn * 5.0 * std::sqrt(M_PI) / 16.0;
    cPch = 0.5;
  }
}

static void write_txt(const std::string& f, const double* a, uint n) {
  FILE* fp = std::fopen(f.c_str(), "w");
  if (!fp) return;
  for (uint c = 0; c < n; c++) std::fprintf(fp, "%.15e\n", a[c]);
  std::fclose(fp);
}
static void write_txt_u(const std::string& f, const uint* a, uint n) {
  FILE* fp = std::fopen(f.c_str(), "w");
  if (!fp) return;
  for (uint c = 0; c < n; c++) std::fprintf(fp, "%u\n", a[c]);
  std::fclose(fp);
}
static void write_bin(const std::string& f, const void* a, size_t bytes) {
  FILE* fp = std::fopen(f.c_str(), "wb");
  if (!fp) return;
  std::fwrite(a, 1, bytes, fp);
  std::fclose(fp);
}

// WriteSolvedDataToFile, SIMPLE_TS_MPI.cpp:5564-5731 (serial path; EnteredData.txt is not rewritten)
void Oracle::write_solved() {
  bc_tjump();
  bc_tjump_write();
  if (!write_files) return;
  const char* names[4] = {"u", "v", "p", "Temper"};
  const double* src[4] = {u, v, p, Temper};
  std::ostringstream its;
  its << it;
  for (int k = 0; k < 4; k++) {
    if (ToWriteSolvedDataToBinaryFile) {
      write_bin(path(std::string(names[k]) + ".bin"), src[k], sizeof(double) * Na);
      if (ToWriteSolvedDataToNewFiles)
        write_bin(path(std::string(names[k]) + "." + its.str() + ".bin"), src[k], sizeof(double) * Na);
    } else {
      write_txt(path(std::string(names[k]) + ".txt"), src[k], Na);
      if (ToWriteSolvedDataToNewFiles) write_txt(path(std::string(names[k]) + "." + its.str() + ".txt"), src[k], Na);
    }
  }
  // the per-save copy of vol_inf_fb is named vol_inf_fb.<it>.bin, but vol_inf_fb.txt.<it>.txt in
  // text mode (SIMPLE_TS_MPI.cpp:5614, :5668)
  if (ToWriteSolvedDataToBinaryFile) {
    write_bin(path("vol_inf_fb.bin"), vol_inf_fb.data(), sizeof(uint) * Na);
    if (ToWriteSolvedDataToNewFiles)
      write_bin(path("vol_inf_fb." + its.str() + ".bin"), vol_inf_fb.data(), sizeof(uint) * Na);
  } else {
    write_txt_u(path("vol_inf_fb.txt"), vol_inf_fb.data(), Na);
    if (ToWriteSolvedDataToNewFiles) write_txt_u(path("vol_inf_fb.txt." + its.str() + ".txt"), vol_inf_fb.data(), Na);
  }
  std::ofstream o(path("it_begin.txt").c_str());
  o << it << std::endl;
}

// WriteDragCoefficient, SIMPLE_TS_MPI.cpp:8147-8578 (serial path): drag coefficients of the
// flagged bodies (CD.<body>.txt), the short-format summary and the inflow pressure-control log.
void Oracle::write_drag() {
  if (!write_files) return;
  double CD_fr_x = 0, CD_p_x = 0;
  const uint nbodies = (uint)bodies.size();
  for (uint counter = 0; counter < nbodies; counter++) {
    if (!bodies[counter].drag) continue;
    double CD_fr_bottom = 0, CD_p_bottom = 0, S_bottom = 0, CD_fr_front = 0, CD_p_front = 0, S_front = 0;
    double CD_fr_top = 0, CD_p_top = 0, S_top = 0, CD_fr_behind = 0, CD_p_behind = 0, S_behind = 0;
    for (uint i = Nx_o[0]; i < Nx_o[1]; i++)
      for (uint j = Ny_o[0]; j < Ny_o[1]; j++) {
        const uint node = i + j * Nx;
        if (vol_inf_fb[node] - 1 != counter) continue;
        const Idx d = clamped(i, j);  // ij_function_i_and_j_to_the_boundaries, also for periodic cases
        if (vol[d.ij_1]) {
          CD_fr_bottom += hx[i] * std::sqrt(Tw_v[d.ij]) *
                          ((u[d.ij_1] - u[d.ij]) / hy[j - 1 * (j < (Ny - 1))] +
                           (u[d.i1j_1] - u[d.i1j]) / hy[j - 1 * (j < (Ny - 1))]);
          CD_p_bottom += p[d.ij_1] * hx[i];
          S_bottom += hx[i];
        }
        if (vol[d.i_1j]) {
          CD_fr_front += hy[j] * std::sqrt(Tw_u[d.ij]) *
                         ((v[d.i_1j] - v[d.ij]) / hx[d.i_1] + (v[d.i_1j1] - v[d.ij1]) / hx[d.i_1]);
          CD_p_front += p[d.i_1j] * hy[j];
          S_front += hy[j];
        }
        if (vol[d.ij1]) {
          CD_fr_top += hx[i] * std::sqrt(Tw_v[d.ij1]) *
                       ((u[d.ij1] - u[d.ij]) / hy[j + 1 * (0 < j)] + (u[d.i1j1] - u[d.i1j]) / hy[j + 1 * (0 < j)]);
          CD_p_top += p[d.ij1] * hx[i];
          S_top += hx[i];
        }
        if (vol[d.i1j]) {
          CD_fr_behind += hy[j] * std::sqrt(Tw_u[d.i1j]) *
                          ((v[d.i1j] - v[d.ij]) / hx[d.i1] + (v[d.i1j1] - v[d.ij1]) / hx[d.i1]);
          CD_p_behind += p[d.i1j] * hy[j];
          S_behind += hy[j];
        }
      }
    double c_CD_p = 0, c_CD_fr = 0;
    if (TypeND == 1) {
      c_CD_p = 1.0 / (u_given_xb_in_it * u_given_xb_in_it * (p_BC_xb / T_BC_xb));
      c_CD_fr = 2.0 / (Re * u_given_xb_in_it);
    } else if (TypeND == 2) {
      c_CD_p = 2.0 / (gamma1 * Ma * Ma * (p_BC_xb / T_BC_xb));
      c_CD_fr = 2.0 / (Re * u_given_xb_in_it);
    } else if (TypeND == 3) {
      c_CD_p = 1.0 / (u_given_xb_in_it * u_given_xb_in_it * (p_BC_xb / T_BC_xb));
      c_CD_fr = (5.0 / 8.0) * std::sqrt(M_PI) * Kn / (u_given_xb_in_it * u_given_xb_in_it * (p_BC_xb / T_BC_xb));
    }
    CD_fr_bottom = c_CD_fr * CD_fr_bottom;
    CD_p_bottom = c_CD_p * CD_p_bottom;
    CD_fr_front = c_CD_fr * CD_fr_front;
    CD_p_front = c_CD_p * CD_p_front;
    CD_fr_top = c_CD_fr * CD_fr_top;
    CD_p_top = c_CD_p * CD_p_top;
    CD_fr_behind = c_CD_fr * CD_fr_behind;
    CD_p_behind = c_CD_p * CD_p_behind;
    CD_fr_x = (CD_fr_top / S_top) + (CD_fr_bottom / S_bottom);
    CD_p_x = (CD_p_front / S_front) - (CD_p_behind / S_behind);
    std::ostringstream name;
    name << "CD." << counter << ".txt";
    std::ofstream o;
    if (ToCheckForFileIsNow_CD && !ToReadSolvedDataFromFile) o.open(path(name.str()).c_str());
    else o.open(path(name.str()).c_str(), std::ios::out | std::ios::app);
    const int w = 30;
    if (!ToReadSolvedDataFromFile && ToCheckForFileIsNow_CD) {
      const char* hdr[16] = {"//it (number of step by time) 00", "ht (step by time) 01", "CD_fr_x (CD from friction) 02",
                             "CD_p_x (CD from pressure) 03", "S_for_CD_bottom 04", "S_for_CD_front 05",
                             "S_for_CD_top 06", "S_for_CD_behind 07", "CD_fr_bottom 08", "CD_p_bottom 09",
                             "CD_fr_front 10", "CD_p_front 11", "CD_fr_top 12", "CD_p_top 13", "CD_fr_behind 14",
                             "CD_p_behind 15"};
      for (const char* h : hdr) o << std::setw(w) << h;
      o << std::endl;
    }
    o << std::setw(w) << it << std::setiosflags(std::ios::scientific) << std::setprecision(10);
    const double vals[15] = {ht, CD_fr_x, CD_p_x, S_bottom, S_front, S_top, S_behind, CD_fr_bottom,
                             CD_p_bottom, CD_fr_front, CD_p_front, CD_fr_top, CD_p_top, CD_fr_behind, CD_p_behind};
    for (double x : vals) o << std::setw(w) << x;
    o << std::endl;
    ToCheckForFileIsNow_CD = false;
  }
  if (WriteDataInShortFormat_kind == 1) {
    double q_xb = 0, q_xe = 0;
    for (uint j = 0; j < Ny; j++) {
      const uint n = 0 + j * Nx;
      if (vol[n]) q_xb += rho[n] * u[n] * hy[j];
    }
    for (uint j = 0; j < Ny; j++) {
      const uint n = Nx_u[1] + j * Nx;
      if (vol[n]) q_xe += rho[n] * u[n] * hy[j];
    }
    std::ofstream o(path("DataInShortFormat.txt").c_str());
    const int w = 30;
    o << std::setiosflags(std::ios::scientific) << std::setprecision(15) << std::setw(w) << Re << std::setw(w) << Kn
      << std::setw(w) << CD_p_x + CD_fr_x << std::setw(w) << CD_p_x << std::setw(w) << u_gas_nd << std::setw(w) << q_xb
      << std::setw(w) << q_xe << std::setw(w) << p_BC_xb << std::setw(w) << p_BC_xe << std::endl;
  }
  if (Pressure_BC) {
    std::ofstream o;
    if (ToCheckForFileIsNow_p_u_x_b && !ToReadSolvedDataFromFile) o.open(path("p_and_u_xb_it.txt").c_str());
    else o.open(path("p_and_u_xb_it.txt").c_str(), std::ios::out | std::ios::app);
    const int w = 30;
    if (!ToReadSolvedDataFromFile && ToCheckForFileIsNow_p_u_x_b) {
      const char* hdr[7] = {"//it (number of step by time)", "ht (step by time)", "p_BC_xb", "u_given_xb_in_it",
                            "u_given_xb_in_it_max", "u_given_xb_in_it_mean", "p_correction"};
      for (const char* h : hdr) o << std::setw(w) << h;
      o << std::endl;
    }
    o << std::setw(w) << it << std::setiosflags(std::ios::scientific) << std::setprecision(15) << std::setw(w) << ht
      << std::setw(w) << p_BC_xb << std::setw(w) << u_given_xb_in_it << std::setw(w) << u_given_xb_in_it_max
      << std::setw(w) << u_given_xb_in_it_mean << std::setw(w) << p_correction << std::endl;
    ToCheckForFileIsNow_p_u_x_b = false;
  }
}

// SolveContinuityEquation, SIMPLE_TS_MPI.cpp:10621-10714 (serial path): the fluxes again, then the
// steady and unsteady continuity residuals of every cell, written as dumps.
void Oracle::solve_continuity() {
  solve_fluxes();
  continuity_st.assign(Na, 0.0);
  continuity.assign(Na, 0.0);
  for (uint j = 0; j < Ny - 1; j++)
    for (uint i = 0; i < Nx - 1; i++) {
      const Idx d = Periodic ? periodic(i, j) : clamped(i, j);
      continuity_st[d.ij] = Fx[d.i1j] - Fx[d.ij] + Fy[d.ij1] - Fy[d.ij];
      continuity[d.ij] = (rho[d.ij] - rho_pr[d.ij]) * hx[i] * hy[j] / ht + continuity_st[d.ij];
    }
  if (!write_files) return;
  std::ostringstream its;
  its << it;
  if (ToWriteSolvedDataToBinaryFile) {
    write_bin(path("ContinuityEquation_stationary.bin"), continuity_st.data(), sizeof(double) * Na);
    write_bin(path("ContinuityEquation.bin"), continuity.data(), sizeof(double) * Na);
    if (ToWriteSolvedDataToNewFiles) {
      write_bin(path("ContinuityEquation_stationary." + its.str() + ".bin"), continuity_st.data(), sizeof(double) * Na);
      write_bin(path("ContinuityEquation." + its.str() + ".bin"), continuity.data(), sizeof(double) * Na);
    }
  } else {
    write_txt(path("ContinuityEquation_stationary.txt"), continuity_st.data(), Na);
    write_txt(path("ContinuityEquation.txt"), continuity.data(), Na);
    if (ToWriteSolvedDataToNewFiles) {
      write_txt(path("ContinuityEquation_stationary." + its.str() + ".txt"), continuity_st.data(), Na);
      write_txt(path("ContinuityEquation." + its.str() + ".txt"), continuity.data(), Na);
    }
  }
}

// WriteTempDataToFile, SIMPLE_TS_MPI.cpp:5838-5942
void Oracle::write_temp() {
  if (!write_files) return;
  std::ofstream o;
  if (ToCheckForFileIsNow_Tmp && !ToReadSolvedDataFromFile) o.open(path("Tmp.txt").c_str());
  else o.open(path("Tmp.txt").c_str(), std::ios::out | std::ios::app);
  o << "it = " << it << "\tit_counter = " << it_counter << "\tIter = " << Iter << "\tIter_p_c = " << Iter_p_c
    << "\tIter_T = " << Iter_T << std::endl;
  uint sum = 0;
  for (uint c = 0; c < Iter; c++) {
    o << "\t" << c << "\t" << max_Iter_p_c[c] << std::setiosflags(std::ios::scientific) << std::setprecision(15)
      << "\t" << max_res_p0[c] << "\t" << max_res_p[c] << "\t" << max_res_T0[c] << "\t" << max_res_T[c] << std::endl;
    sum += max_Iter_p_c[c];
  }
  o << "\t\t" << sum << std::endl;
  o << std::setiosflags(std::ios::scientific) << std::setprecision(15) << "\t" << max_residual_in_u_Iter_0 << "\t"
    << max_residual_in_u << std::endl
    << "\t" << max_residual_in_v_Iter_0 << "\t" << max_residual_in_v << std::endl;
  ToCheckForFileIsNow_Tmp = false;
}

// WriteIterationsInLoopsToFile, SIMPLE_TS_MPI.cpp:5945-6006
void Oracle::write_iterations() {
  if (!write_files) return;
  std::ofstream o;
  if (ToCheckForFileIsNow_Iterations_in_loops) {
    if (ToReadSolvedDataFromFile) o.open(path("Iterations_in_loops.txt").c_str(), std::ios::out | std::ios::app);
    else {
      o.open(path("Iterations_in_loops.txt").c_str());
      o << "it" << "\tit_counter" << "\tIter" << "\tsum_max_Iter_p_c" << std::endl;
    }
  } else {
    o.open(path("Iterations_in_loops.txt").c_str(), std::ios::out | std::ios::app);
  }
  uint sum = 0;
  for (uint c = 0; c < Iter; c++) sum += max_Iter_p_c[c];
  o << it << "\t" << it_counter << "\t\t" << Iter << "\t" << sum << std::endl;
  ToCheckForFileIsNow_Iterations_in_loops = false;
}

// main() up to the time loop, SIMPLE_TS_MPI.cpp:1796-3227 (serial path)
bool Oracle::setup() {
  time_solve_start = (long)time(NULL);
  if (!read_entered_data()) return false;
  time_solve_stop = time_solve_start + max_time_for_solve * 3600.0;
  solve_is_finished = false;
  rho_gas_nd = p_gas_nd / T_gas_nd;
  V_gas_nd = std::sqrt(u_gas_nd * u_gas_nd + v_gas_nd * v_gas_nd);
  if (TypeND == 1 || TypeND == 2) {
    if (GivenReKn) u_given_xb = Re * Kn * std::sqrt(15.0 * M_PI / 128.0);
    u_given_xb_in_it = u_given_xb;
    cT = (1.0 / Re) * (u_given_xb_in_it * p_BC_xb / T_BC_xb);
    cPch = (TypeND == 1) ? 0.5 : u_given_xb_in_it * u_given_xb_in_it / (gamma1 * Ma * Ma);
  } else if (TypeND == 3) {
    Ma = std::sqrt(6.0 / 5.0);
    Pr = 2.0 / 3.0;
    gamma1 = 5.0 / 3.0;
    c_mu = (5.0 / 16.0) * std::sqrt(2.0 * M_PI / gamma1);
    cT = Kn * 5.0 * std::sqrt(M_PI) / 16.0;
    cPch = 0.5;
  }
  c_Fr_v = SolveGravityField ? 2.0 / (gamma1 * Fr * Ma * Ma) : 0;
  cT1 = gamma1 * c_mu * Kn / (Ma * Pr);
  cT2 = gamma1 * (gamma1 - 1.0) * c_mu * Kn * Ma;
  build_mesh();
  if (write_files) {
    write_txt(path("x_f.txt"), x_f.data(), Nx + 1);
    write_txt(path("hx.txt"), hx.data(), Nx);
    write_txt(path("x_v.txt"), x_v.data(), Nx);
    write_txt(path("y_f.txt"), y_f.data(), Ny + 1);
    write_txt(path("hy.txt"), hy.data(), Ny);
    write_txt(path("y_v.txt"), y_v.data(), Ny);
  }
  // bodies (gb only; the p and V objects are read but never applied, :2511-2512)
  if (imp_circ_b && !read_bodies("solve_circles_b.txt", true)) return false;
  if (imp_poly_b && !read_bodies("solve_polyhedrons_b.txt", false)) return false;
  define_vol_inf();
  auto alloc = [&](std::vector<double>& a) { a.assign(Na, 0.0); };
  for (auto* a : {&Gamma_yf, &Gamma_xf, &Fx, &Fy, &st_u0, &st_u1, &u_pseudo, &D_ux, &D_uy, &st_v0, &st_v1, &v_pseudo,
                  &D_vx, &D_vy, &st_p0, &st_p1, &st_p2, &d_p_c_12, &d_p_c_34, &apx, &apy, &bpx, &bpy, &st_r0, &st_r1,
                  &rho_u, &rho_v, &st_T0, &st_T1, &st_T2, &Tw_u, &Tw_v, &sqrt_T, &DTx, &DTy, &ScT1})
    alloc(*a);
  u = st_u0.data(); u_pr = st_u1.data(); v = st_v0.data(); v_pr = st_v1.data();
  p = st_p0.data(); p_pr = st_p1.data(); p_old = st_p2.data();
  rho = st_r0.data(); rho_pr = st_r1.data();
  Temper = st_T0.data(); Temper_pr = st_T1.data(); Temper_old = st_T2.data();
  max_res_p.assign(N_I, 0); max_res_T.assign(N_I, 0); max_res_p0.assign(N_I, 0); max_res_T0.assign(N_I, 0);
  max_Iter_p_c.assign(N_I, 0);
  for (uint c = 0; c < Na; c++) {
    u[c] = u_gas_nd; v[c] = v_gas_nd; p[c] = p_gas_nd; rho[c] = rho_gas_nd; Temper[c] = T_gas_nd;
  }
  define_area_for_solving();
  define_rule_vectors();
  if (ToReadSolvedDataFromFile) {
    if (!read_restart()) return false;
  } else {
    apply_bodies();
    rho_BC_xb = p_BC_xb / T_BC_xb;
    rho_BC_xe = p_BC_xe / T_BC_xe;
    if (Pressure_BC) {
      for (uint j = 0; j < Ny; j++)
        for (uint i = 0; i < Nx_o[0]; i++) {
          uint n = i + j * Nx;
          if (vol[n]) { p[n] = p_BC_xb; rho[n] = rho_BC_xb; Temper[n] = T_BC_xb; }
        }
      for (uint j = 0; j < Ny; j++)
        for (uint i = Nx_o[1]; i < Nx; i++) {
          uint n = i + j * Nx;
          if (vol[n]) { p[n] = p_BC_xe; rho[n] = rho_BC_xe; Temper[n] = T_BC_xe; }
        }
      if (ToStartFromExactSolution) {  // :2566-2688
        uint jb = 0, je = 0;
        for (uint j = 1; j < Ny; j++) {
          uint n = 1 + j * Nx;
          if ((!vol[n - Nx]) && vol[n]) jb = j - 1;
          if (vol[n - Nx] && (!vol[n])) je = j;
        }
        double hch = y_v[je] - y_v[jb];
        double Lch = x_v[Nx_o[1]] - x_v[Nx_o[0] - 1];
        const Body& B0 = bodies[0];
        double sig = B0.slip * B0.F_slip;
        double Px = p_BC_xb / p_BC_xe;
        std::vector<double> xa(Nx), ya(Ny);
        for (uint i = 0; i < Nx; i++) xa[i] = (x_v[i] - x_v[0]) / Lch;
        for (uint j = 0; j < Ny; j++) {
          if (j <= jb) ya[j] = -0.5 * hch;
          else if (je <= j) ya[j] = 0.5 * hch;
          else ya[j] = y_v[j + jb] - (y_v[jb] + 0.5 * hch);
        }
        for (uint j = 0; j < Ny; j++)
          for (uint i = Nx_o[0]; i < Nx_o[1]; i++) {
            uint n = i + j * Nx;
            if (vol[n])
              p[n] = p_BC_xe * (-6.0 * sig * Kn + std::sqrt(std::pow((6.0 * sig * Kn), 2) + (1.0 + 12.0 * sig * Kn) * xa[i] +
                                                            (Px + 12.0 * sig * Kn) * Px * (1.0 - xa[i])));
          }
        double ND = 0;
        if (TypeND == 1 || TypeND == 2) ND = Re * hch * hch / (4.0 * u_given_xb);
        else if (TypeND == 3) ND = hch / (5.0 * std::sqrt(M_PI * T_BC_xb) * Kn * Lch);
        for (uint j = 0; j < Ny; j++)
          for (uint i = 0; i < Nx; i++) {
            uint n = i + j * Nx;
            if (vol[n])
              u[n] = -ND *
                     ((p_BC_xe * (1.0 - Px * Px + 12.0 * sig * Kn * (1.0 - Px))) /
                      (2.0 * std::sqrt(std::pow((6.0 * sig * Kn), 2) + (1.0 + 12.0 * sig * Kn) * xa[i] +
                                       (Px + 12.0 * sig * Kn) * Px * (1.0 - xa[i])))) *
                     (1.0 - 4.0 * ya[j] * ya[j] / (hch * hch) + 4.0 * sig * Kn / p[n]);
          }
      }
    }
    if (Given_velocity_on_xb && ToStartFromExactSolution) {  // :2694-2806
      for (uint j = 0; j < Ny; j++)
        for (uint i = 0; i < Nx_o[0] + 1; i++) {
          uint n = i + j * Nx;
          if (vol[n]) p[n] = p_BC_xb;
        }
      uint jb = 0, je = 0;
      for (uint j = 1; j < Ny; j++) {
        uint n = 1 + j * Nx;
        if ((!vol[n - Nx]) && vol[n]) jb = j - 1;
        if (vol[n - Nx] && (!vol[n])) je = j;
      }
      double hch = y_f[je + 1 * (0 < Ny)] - y_f[jb];  // j == Ny after the loop above
      double Lch = x_v[Nx_o[1]] - x_v[Nx_o[0] - 1];
      double yc = y_v[jb] + 0.5 * hch;
      double q = (yc - y_v[jb] / hch - (yc - y_v[jb] / hch) * (yc - y_v[jb] / hch));
      if (correct_p_BC_xb) p_BC_xb = p_BC_xe + 4.0 * Lch * u_given_xb * u_given_xb / (Re * hch * hch * q);
      else p_BC_xe = p_BC_xb - 4.0 * Lch * u_given_xb * u_given_xb / (Re * hch * hch * q);
      double dpdx = (p_BC_xe - p_BC_xb) / Lch;
      double ND = 0;
      if (TypeND == 1 || TypeND == 2) ND = Re * hch * hch / (4.0 * u_given_xb);
      else if (TypeND == 3) ND = 4.0 * hch * hch / (5.0 * std::sqrt(M_PI * T_BC_xb) * Kn);
      const Body& B0 = bodies[0];
      for (uint j = 0; j < Ny; j++)
        for (uint i = 0; i < Nx_u[0]; i++) {
          uint n = i + j * Nx;
          if (vol[n])
            u[n] = -ND * dpdx *
                   ((y_v[j] - y_v[jb]) / hch - ((y_v[j] - y_v[jb]) / hch) * ((y_v[j] - y_v[jb]) / hch) +
                    Kn * B0.F_slip * B0.slip / hch);
        }
    }
    if (Given_velocity_on_xe && ToStartFromExactSolution) {
      for (uint j = 0; j < Ny; j++)
        for (uint i = Nx_o[1]; i < Nx; i++) {
          uint n = i + j * Nx;
          if (vol[n]) p[n] = p_BC_xe;
        }
    }
    for (uint c = 0; c < Na; c++) {
      p_pr[c] = p[c]; u_pr[c] = u[c]; v_pr[c] = v[c]; Temper_pr[c] = Temper[c]; rho_pr[c] = rho[c];
    }
    solve_rho_mid();
    apply_bodies();
    bc_velocities();
    for (uint c = 0; c < Na; c++) {
      p_pr[c] = p[c]; u_pr[c] = u[c]; v_pr[c] = v[c]; Temper_pr[c] = Temper[c]; rho_pr[c] = rho[c];
    }
    solve_rho_mid();
    it_begin = 0;
    it = it_begin;
    write_solved();
  }
  for (uint c = 0; c < Na; c++) {
    d_p_c_12[c] = 0; d_p_c_34[c] = 0; apx[c] = 0; apy[c] = 0; bpx[c] = 0; bpy[c] = 0;
    Gamma_yf[c] = 0; Gamma_xf[c] = 0; Fx[c] = 0; Fy[c] = 0; u_pseudo[c] = 0; v_pseudo[c] = 0;
  }
  for (uint c = 0; c < Na; c++) {
    D_ux[c] = 0; D_uy[c] = 0; D_vx[c] = 0; D_vy[c] = 0; DTx[c] = 0; DTy[c] = 0; ScT1[c] = 0;
    rho_u[c] = 0; rho_v[c] = 0;
  }
  Iter = 0; Iter_pr1 = Iter; Iter_pr2 = Iter_pr1;
  max_residual_in_u = 0; max_residual_in_v = 0; max_residual_in_u_Iter_0 = 0; max_residual_in_v_Iter_0 = 0;
  if (Pressure_BC && !ToReadSolvedDataFromFile) {
    for (uint j = 0; j < Ny; j++) {
      for (uint i = 0; i < Nx_o[0]; i++) {
        uint n = i + j * Nx;
        if (vol[n]) { p[n] = p_BC_xb; Temper[n] = T_BC_xb; }
      }
      for (uint i = Nx_o[1]; i < Nx; i++) {
        uint n = i + j * Nx;
        if (vol[n]) { p[n] = p_BC_xe; Temper[n] = T_BC_xe; }
      }
    }
  }
  if (ToContinueFromInterpolation) {
    apply_bodies();
    bc_slip_u();
    bc_slip_v();
    bc_tjump();
    bc_tjump_write();
  }
  for (uint c = 0; c < Na; c++) {
    sqrt_T[c] = std::sqrt(Temper[c]);
    if (vol[c]) rho[c] = p[c] / Temper[c];
    else rho[c] = 0;
  }
  solve_rho_mid();
  std::memcpy(p_old, p, Na * sizeof(double));
  std::memcpy(Temper_old, Temper, Na * sizeof(double));
  it = it_begin;
  it_counter = 0;
  countinue_time_step = true;
  for (uint c = 0; c < Na; c++) {
    p_pr[c] = p[c]; u_pr[c] = u[c]; v_pr[c] = v[c]; Temper_pr[c] = Temper[c]; sqrt_T[c] = std::sqrt(Temper[c]);
    rho_pr[c] = rho[c];
  }
  nondim_refresh();
  solve_rho_mid();
  bc_slip_u();
  bc_slip_v();
  bc_velocities();
  bc_pressure_begin_it();
  bc_tjump();
  bc_temperature();
  bc_pressure();
  solve_fluxes();
  solve_diffusion();
  std::memcpy(p_old, p, Na * sizeof(double));
  std::memcpy(Temper_old, Temper, Na * sizeof(double));
  for (uint c = 0; c < N_I; c++) {
    max_res_p[c] = 0; max_res_T[c] = 0; max_res_p0[c] = 0; max_res_T0[c] = 0; max_Iter_p_c[c] = 0;
  }
  time_solve_start = (long)time(NULL);
  return true;
}

// coupled p-T Jacobi sweeps with the EOS substitution, SIMPLE_TS_MPI.cpp:3786-4131
void Oracle::pt_sweeps() {
  const std::vector<char>& b = vol;
  // ---- coupled p-T Jacobi sweeps (:3786-4131) ----
  continue_iter_p_c = false;
  Iter_p_c = 0;
  do {
    std::swap(p, p_old);
    std::swap(Temper, Temper_old);
    const double* P = p_old;
    const double* TT = Temper_old;
    max_res_p[Iter] = 0;
    max_res_T[Iter] = 0;
    for (size_t c = 0; c < bc_o.size(); c++) {
      Idx d = bc_idx(bc_o[c]);
      uint i = d.i, j = d.j;
      double aT1 = dmax(0, Fx[d.ij]) + DTx[d.ij];
      double aT2 = dmax(0, -Fx[d.i1j]) + DTx[d.i1j];
      double aT3 = dmax(0, Fy[d.ij]) + DTy[d.ij];
      double aT4 = dmax(0, -Fy[d.ij1]) + DTy[d.ij1];
      Temper[d.ij] =
          (ht * (aT1 * (b[d.i_1j] * TT[d.i_1j] + (!b[d.i_1j]) * Tw_u[d.ij]) +
                 aT2 * (b[d.i1j] * TT[d.i1j] + (!b[d.i1j]) * Tw_u[d.i1j]) +
                 aT3 * (b[d.ij_1] * TT[d.ij_1] + (!b[d.ij_1]) * Tw_v[d.ij]) +
                 aT4 * (b[d.ij1] * TT[d.ij1] + (!b[d.ij1]) * Tw_v[d.ij1]) +
                 (1.0 - gamma1) * P[d.ij] * ((u[d.i1j] - u[d.ij]) * hy[j] + (v[d.ij1] - v[d.ij]) * hx[i])) +
           ScT1[d.ij]) /
          (ht * (aT1 + aT2 + aT3 + aT4 + Fx[d.i1j] - Fx[d.ij] + Fy[d.ij1] - Fy[d.ij]) + hx[i] * hy[j] * rho[d.ij]);
      double rT = Temper[d.ij] - Temper_old[d.ij];
      bool gxb = Given_velocity_on_xb * (i == Nx_o[0]);
      bool gxe = Given_velocity_on_xe * (i == Nx_o[1] - 1);
      p[d.ij] = (ht * (apx[d.ij] * P[d.i_1j] + apx[d.i1j] * P[d.i1j] + apy[d.ij] * P[d.ij_1] + apy[d.ij1] * P[d.ij1] +
                       bpx[d.ij] - bpx[d.i1j] + bpy[d.ij] - bpy[d.ij1] + gxb * Fx[d.ij] - gxe * Fx[d.i1j]) +
                 p_pr[d.ij] * hx[i] * hy[j] / (Temper_pr[d.ij])) /
                (ht * (apx[d.ij] + apx[d.i1j] + apy[d.ij] + apy[d.ij1]) + hx[i] * hy[j] / (Temper[d.ij]));
      double rp = p[d.ij] - p_old[d.ij];
      if (max_res_T[Iter] < std::fabs(rT)) max_res_T[Iter] = std::fabs(rT);
      if (max_res_p[Iter] < std::fabs(rp)) max_res_p[Iter] = std::fabs(rp);
    }
    for (size_t c = 0; c < nch_o.size(); c++) {
      uint n = nch_o[c];
      Idx d = clamped(n % Nx, n / Nx);
      uint i = d.i, j = d.j;
      double aT1 = dmax(0, Fx[d.ij]) + DTx[d.ij];
      double aT2 = dmax(0, -Fx[d.i1j]) + DTx[d.i1j];
      double aT3 = dmax(0, Fy[d.ij]) + DTy[d.ij];
      double aT4 = dmax(0, -Fy[d.ij1]) + DTy[d.ij1];
      Temper[d.ij] = (ht * (aT1 * TT[d.i_1j] + aT2 * TT[d.i1j] + aT3 * TT[d.ij_1] + aT4 * TT[d.ij1] +
                            (1.0 - gamma1) * P[d.ij] * ((u[d.i1j] - u[d.ij]) * hy[j] + (v[d.ij1] - v[d.ij]) * hx[i])) +
                      ScT1[d.ij]) /
                     (ht * (aT1 + aT2 + aT3 + aT4 + Fx[d.i1j] - Fx[d.ij] + Fy[d.ij1] - Fy[d.ij]) + hx[i] * hy[j] * rho[d.ij]);
      double rT = Temper[d.ij] - Temper_old[d.ij];
      p[d.ij] = (ht * (apx[d.ij] * P[d.i_1j] + apx[d.i1j] * P[d.i1j] + apy[d.ij] * P[d.ij_1] + apy[d.ij1] * P[d.ij1] +
                       bpx[d.ij] - bpx[d.i1j] + bpy[d.ij] - bpy[d.ij1]) +
                 p_pr[d.ij] * hx[i] * hy[j] / (Temper_pr[d.ij])) /
                (ht * (apx[d.ij] + apx[d.i1j] + apy[d.ij] + apy[d.ij1]) + hx[i] * hy[j] / (Temper[d.ij]));
      double rp = p[d.ij] - p_old[d.ij];
      if (max_res_p[Iter] < std::fabs(rp)) max_res_p[Iter] = std::fabs(rp);
      if (max_res_T[Iter] < std::fabs(rT)) max_res_T[Iter] = std::fabs(rT);
    }
    if (Iter_p_c == 0) {
      max_res_p0[Iter] = max_res_p[Iter];
      max_res_T0[Iter] = max_res_T[Iter];
    }
    Iter_p_c++;
    if (fixed_sweeps)
      continue_iter_p_c = (Iter_p_c < N_I_p_c);
    else
      continue_iter_p_c = (Iter_p_c < 2) ||
                          ((Iter_p_c < N_I_p_c) && ((MaxError_p_c < max_res_p[Iter]) || (MaxError_T < max_res_T[Iter])));
  } while (continue_iter_p_c);
}

// Least-squares fit and application of the mode-3 warm start.  With D_t = x_t - x_{t-1} on the
// solved cells and the regressors in the difference basis d(t) = (D_t, D_t - D_{t-1},
// D_t - 2 D_{t-1} + D_{t-2}) (the same span as D_t, D_{t-1}, D_{t-2}, but well conditioned when the
// trajectory is smooth), c minimises sum over the last kWin steps s of |D_s - c . d(s-1)|^2;
// the step's initial iterate is x_n + c . d(n), i.e. x_n + w_0 D_n + w_1 D_{n-1} + w_2 D_{n-2}
// with w = (c0 + c1 + c2, -c1 - 2 c2, c2).  Until kWin + 3 differences exist, and whenever the
// normal equations are (nearly) singular, w = (2, -1, 0) (quadratic extrapolation; (1, 0, 0)
// on the second step).
void Oracle::warm_ar() {
  std::vector<uint> cells(nch_o);
  cells.insert(cells.end(), bc_o.begin(), bc_o.end());
  const size_t m = cells.size();
  if (!warm_ready) {
    p_m1.assign(p, p + Na);
    T_m1.assign(Temper, Temper + Na);
    Dp.assign(kRing, std::vector<double>(m, 0.0));
    DT.assign(kRing, std::vector<double>(m, 0.0));
    warm_ready = 1;
    return;
  }
  const int h = warm_ready - 1;  // index of the newest difference
  for (size_t q = 0; q < m; q++) {
    const uint n = cells[q];
    Dp[h % kRing][q] = p[n] - p_m1[n];
    DT[h % kRing][q] = Temper[n] - T_m1[n];
    p_m1[n] = p[n];
    T_m1[n] = Temper[n];
  }
  const int have = h + 1;
  for (int f = 0; f < 2; f++) {
    const std::vector<std::vector<double>>& R = f ? DT : Dp;
    auto D = [&](int t, size_t q) { return R[t % kRing][q]; };
    double* x = f ? Temper : p;
    double w[3] = {2.0, -1.0, 0.0};
    if (have < 2) {
      w[0] = 1.0;
      w[1] = 0.0;
    }
    if (have >= 3 + kWin) {
      double G[3][3] = {{0}}, r[3] = {0};
      for (int s = h - kWin + 1; s <= h; s++)
        for (size_t q = 0; q < m; q++) {
          const double a0 = D(s - 1, q), a1 = D(s - 1, q) - D(s - 2, q);
          const double a2 = D(s - 1, q) - 2.0 * D(s - 2, q) + D(s - 3, q);
          const double a[3] = {a0, a1, a2}, y = D(s, q);
          for (int i = 0; i < 3; i++) {
            r[i] += a[i] * y;
            for (int j = 0; j < 3; j++) G[i][j] += a[i] * a[j];
          }
        }
      const double det = G[0][0] * (G[1][1] * G[2][2] - G[1][2] * G[2][1]) -
                         G[0][1] * (G[1][0] * G[2][2] - G[1][2] * G[2][0]) +
                         G[0][2] * (G[1][0] * G[2][1] - G[1][1] * G[2][0]);
      const double scale = G[0][0] * G[1][1] * G[2][2];
      if (scale > 0 && std::fabs(det) > 1e-6 * scale) {
        double c[3];
        for (int i = 0; i < 3; i++) {
          double Gi[3][3];
          for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) Gi[a][b] = (b == i) ? r[a] : G[a][b];
          c[i] = (Gi[0][0] * (Gi[1][1] * Gi[2][2] - Gi[1][2] * Gi[2][1]) -
                  Gi[0][1] * (Gi[1][0] * Gi[2][2] - Gi[1][2] * Gi[2][0]) +
                  Gi[0][2] * (Gi[1][0] * Gi[2][1] - Gi[1][1] * Gi[2][0])) / det;
        }
        w[0] = c[0] + c[1] + c[2];
        w[1] = -c[1] - 2.0 * c[2];
        w[2] = c[2];
      }
    }
    for (size_t q = 0; q < m; q++) {
      double e = w[0] * D(h, q);
      if (have >= 2) e += w[1] * D(h - 1, q);
      if (have >= 3) e += w[2] * D(h - 2, q);
      x[cells[q]] += e;
    }
  }
  warm_ready++;
}

// Mode 4 (no counterpart in the reference): the 36 features of cell (i, j) for the step whose
// newest difference has index t: for each of the time-basis fields D_t, D_t - D_{t-1} and the
// second and third differences (FP32, from the stored FP32 differences), the 3x3 neighbourhood
// (clamped at the mesh edge) resolved into value, gradient and curvature along x, each of those
// into value, gradient and curvature along y.
void Oracle::conv_features(int f, unsigned t, int i, int j, float* out) const {
  float S[4][3][3];
  for (int dj = -1; dj <= 1; dj++) {
    const int jj = std::min(std::max(j + dj, 0), (int)Ny - 1);
    for (int di = -1; di <= 1; di++) {
      const int ii = std::min(std::max(i + di, 0), (int)Nx - 1);
      const size_t n = (size_t)ii + (size_t)jj * Nx;
      const float d0 = cD[f][t % kCRing][n], d1 = cD[f][(t - 1) % kCRing][n];
      const float d2 = cD[f][(t - 2) % kCRing][n], d3 = cD[f][(t - 3) % kCRing][n];
      const float e1 = d0 - d1, e1b = d1 - d2, e1c = d2 - d3;
      const float e2 = e1 - e1b, e2b = e1b - e1c;
      S[0][dj + 1][di + 1] = d0;
      S[1][dj + 1][di + 1] = e1;
      S[2][dj + 1][di + 1] = e2;
      S[3][dj + 1][di + 1] = e2 - e2b;
    }
  }
  for (int k = 0; k < 4; k++) {
    float row[3][3];
    for (int r = 0; r < 3; r++) {
      const float w = S[k][r][0], c = S[k][r][1], e = S[k][r][2];
      row[r][0] = c;
      row[r][1] = 0.5f * (e - w);
      row[r][2] = (e + w) - 2.0f * c;
    }
    for (int q = 0; q < 3; q++) {
      const float lo = row[0][q], c = row[1][q], hi = row[2][q];
      out[k * 9 + q * 3 + 0] = c;
      out[k * 9 + q * 3 + 1] = 0.5f * (hi - lo);
      out[k * 9 + q * 3 + 2] = (hi + lo) - 2.0f * c;
    }
  }
}

static inline unsigned f32_bits(float x) {
  unsigned u;
  std::memcpy(&u, &x, 4);
  return u;
}
static inline float bits_f32(unsigned u) {
  float x;
  std::memcpy(&x, &u, 4);
  return x;
}

// Mode 4: the GB300 library's convolutional warm start, restated sequentially.  Per field, the
// step differences D_t = x_t - x_{t-1} are kept in FP32; the step starts from quadratic
// extrapolation (mode 2) except on the active cells -- within a diamond of radius 3 of a cell with
// |D_h| > 0.1 max |D_h| (x wrapped on periodic meshes) -- where it starts from x_h + w . features.
// The weights solve least squares over the last 6 training pairs (features of step t-1 on the
// cells active at t-1, target D_t): normal-equation terms summed in FP32 per strip of 32x2 cells
// (rows in cell order), with compensated FP32 sums over the strips with rows of each 32x8 tile,
// over the tiles with rows (tile order) and over the 6 window slots (slot order); ridge 1e-11 of
// the mean diagonal (FP64 trace); FP32 Gauss-Jordan elimination without pivoting.  Every operation has the
// library's order, so the initial iterates agree bit for bit.
void Oracle::warm_conv() {
  const unsigned r = (unsigned)warm_ready;
  if (csolved.empty()) {
    csolved.assign(Na, 0);
    for (const std::vector<uint>* list : {&nch_o, &bc_o})
      for (uint n : *list) csolved[n] = 1;
    for (int f = 0; f < 2; f++)
      for (int k = 0; k < kCRing; k++) cD[f][k].assign(Na, 0.f);
    cact[0].assign(Na, 0);
    cact[1].assign(Na, 0);
    cgram.assign((size_t)kCWin * 2 * kCTerms, 0.f);
    p_m1.assign(Na, 0.0); p_m2.assign(Na, 0.0);
    T_m1.assign(Na, 0.0); T_m2.assign(Na, 0.0);
  }
  unsigned mx[2] = {0u, 0u};
  for (uint n = 0; n < Na; n++) {
    if (csolved[n]) {
      const double x = p[n], y = Temper[n];
      if (r == 0) {
        p_m1[n] = x; p_m2[n] = x;
        T_m1[n] = y; T_m2[n] = y;
      } else {
        const double dx = x - p_m1[n], dy = y - T_m1[n];
        const float fx = (float)dx, fy = (float)dy;
        cD[0][(r - 1) % kCRing][n] = fx;
        cD[1][(r - 1) % kCRing][n] = fy;
        mx[0] = std::max(mx[0], f32_bits(std::fabs(fx)));
        mx[1] = std::max(mx[1], f32_bits(std::fabs(fy)));
        if (r >= 2) {
          p[n] = 3.0 * dx + p_m2[n];
          Temper[n] = 3.0 * dy + T_m2[n];
        } else {
          p[n] = x + dx;
          Temper[n] = y + dy;
        }
        p_m2[n] = p_m1[n]; p_m1[n] = x;
        T_m2[n] = T_m1[n]; T_m1[n] = y;
      }
    } else if (r >= 1) {
      cD[0][(r - 1) % kCRing][n] = 0.f;
      cD[1][(r - 1) % kCRing][n] = 0.f;
    }
  }
  warm_ready = (int)r + 1;
  if (r == 0) return;
  const unsigned h = r - 1;
  // active cells of the newest difference
  const float thr[2] = {0.1f * bits_f32(mx[0]), 0.1f * bits_f32(mx[1])};
  for (int j = 0; j < (int)Ny; j++)
    for (int i = 0; i < (int)Nx; i++) {
      const size_t n = (size_t)i + (size_t)j * Nx;
      unsigned char bits = 0;
      if (csolved[n])
        for (int dj = -3; dj <= 3; dj++) {
          const int jj = j + dj;
          if (jj < 0 || jj >= (int)Ny) continue;
          const int rx = 3 - std::abs(dj);
          for (int di = -rx; di <= rx; di++) {
            int ii = i + di;
            if (Periodic) ii = (ii + (int)Nx) % (int)Nx;
            else if (ii < 0 || ii >= (int)Nx) continue;
            const size_t q = (size_t)ii + (size_t)jj * Nx;
            if (std::fabs(cD[0][h % kCRing][q]) > thr[0]) bits |= 1;
            if (std::fabs(cD[1][h % kCRing][q]) > thr[1]) bits |= 2;
          }
        }
      cact[h & 1][n] = bits;
    }
  // the newest training pair
  auto neumaier = [](float& sm, float& cm, float x) {
    const float t = sm + x;
    if (std::fabs(sm) >= std::fabs(x)) cm = cm + ((sm - t) + x);
    else cm = cm + ((x - t) + sm);
    sm = t;
  };
  if (h >= 4) {
    // the newest training pair: per 32x8 tile, per strip of 32x2 cells (rows in cell order) the
    // FP32 terms; compensated sums over the tile's strips with rows, then over the tiles with rows
    const int ntx = ((int)Nx + 31) / 32, nty = ((int)Ny + 7) / 8;
    std::vector<float> F(64 * (kCFeat + 1));
    std::vector<float> total(2 * kCTerms), tot_c(2 * kCTerms, 0.f);
    std::fill(total.begin(), total.end(), 0.f);
    for (int ty = 0; ty < nty; ty++)
      for (int tx = 0; tx < ntx; tx++)
        for (int f = 0; f < 2; f++) {
          float strip_terms[4][kCTerms];
          int rows_of[4] = {0, 0, 0, 0};
          for (int sidx = 0; sidx < 4; sidx++) {
            int rows = 0;
            for (int j = 8 * ty + 2 * sidx; j < 8 * ty + 2 * sidx + 2 && j < (int)Ny; j++)
              for (int i = 32 * tx; i < 32 * tx + 32 && i < (int)Nx; i++) {
                const size_t n = (size_t)i + (size_t)j * Nx;
                if (!((cact[(h - 1) & 1][n] >> f) & 1)) continue;
                conv_features(f, h - 1, i, j, &F[rows * (kCFeat + 1)]);
                F[rows * (kCFeat + 1) + kCFeat] = cD[f][h % kCRing][n];
                rows++;
              }
            rows_of[sidx] = rows;
            int e = 0;
            for (int a = 0; a < kCFeat; a++)
              for (int b = a; b < kCFeat; b++, e++) {
                float t = 0.f;
                for (int q = 0; q < rows; q++) t = t + F[q * (kCFeat + 1) + a] * F[q * (kCFeat + 1) + b];
                strip_terms[sidx][e] = t;
              }
            for (int a = 0; a < kCFeat; a++, e++) {
              float t = 0.f;
              for (int q = 0; q < rows; q++) t = t + F[q * (kCFeat + 1) + a] * F[q * (kCFeat + 1) + kCFeat];
              strip_terms[sidx][e] = t;
            }
          }
          if (rows_of[0] + rows_of[1] + rows_of[2] + rows_of[3] == 0) continue;
          for (int e = 0; e < kCTerms; e++) {
            float sm = 0.f, cm = 0.f;
            for (int sidx = 0; sidx < 4; sidx++)
              if (rows_of[sidx] > 0) neumaier(sm, cm, strip_terms[sidx][e]);
            neumaier(total[f * kCTerms + e], tot_c[f * kCTerms + e], sm + cm);
          }
        }
    const unsigned pair = h - 4;
    for (int f = 0; f < 2; f++)
      for (int e = 0; e < kCTerms; e++)
        cgram[((size_t)(pair % kCWin) * 2 + f) * kCTerms + e] = total[f * kCTerms + e] + tot_c[f * kCTerms + e];
    for (int f = 0; f < 2; f++) {
      conv_ok[f] = false;
      if (pair + 1 < (unsigned)kCWin) continue;
      std::vector<float> G(kCTerms);
      for (int q = 0; q < kCTerms; q++) {
        float sm = 0.f, cm = 0.f;
        for (int w = 0; w < kCWin; w++) neumaier(sm, cm, cgram[((size_t)w * 2 + f) * kCTerms + q]);
        G[q] = sm + cm;
      }
      double tr = 0.0;
      for (int a = 0, e = 0; a < kCFeat; a++) {
        tr = tr + (double)G[e];
        e += kCFeat - a;
      }
      const double lam = 1e-11 * tr / (double)kCFeat;
      // Gauss-Jordan elimination without pivoting on [matrix | right-hand side]
      float M[kCFeat][kCFeat + 1], y[kCFeat];
      int e = 0;
      for (int a = 0; a < kCFeat; a++)
        for (int b = a; b < kCFeat; b++, e++) {
          if (a == b) M[a][a] = (float)((double)G[e] + lam);
          else M[a][b] = M[b][a] = G[e];
        }
      for (int a = 0; a < kCFeat; a++, e++) M[a][kCFeat] = G[e];
      bool ok = true;
      for (int k = 0; k < kCFeat && ok; k++) {
        const float piv = M[k][k];
        if (!(piv > 0.f && piv < 3.0e38f)) {
          ok = false;
          break;
        }
        const float rp = 1.0f / piv;
        float u[kCFeat + 1];
        for (int j = k + 1; j <= kCFeat; j++) u[j] = M[k][j] * rp;
        for (int i = 0; i < kCFeat; i++) {
          if (i == k) continue;
          for (int j = k + 1; j <= kCFeat; j++) M[i][j] = M[i][j] - M[i][k] * u[j];
        }
        for (int j = k + 1; j <= kCFeat; j++) M[k][j] = u[j];
      }
      if (!ok) continue;
      for (int k = 0; k < kCFeat; k++) y[k] = M[k][kCFeat];
      bool finite = true;
      for (int k = 0; k < kCFeat; k++) finite = finite && std::isfinite(y[k]);
      for (int k = 0; k < kCFeat; k++) conv_w[f][k] = y[k];
      conv_ok[f] = finite;
    }
  } else {
    conv_ok[0] = conv_ok[1] = false;
  }
  // the stencil's start on the active cells
  for (int j = 0; j < (int)Ny; j++)
    for (int i = 0; i < (int)Nx; i++) {
      const size_t n = (size_t)i + (size_t)j * Nx;
      const unsigned char bits = cact[h & 1][n];
      for (int f = 0; f < 2; f++) {
        if (!((bits >> f) & 1) || !conv_ok[f]) continue;
        float feat[kCFeat];
        conv_features(f, h, i, j, feat);
        float corr = 0.f;
        for (int k = 0; k < kCFeat; k++) corr = corr + conv_w[f][k] * feat[k];
        if (f == 0) p[n] = p_m1[n] + (double)corr;
        else Temper[n] = T_m1[n] + (double)corr;
      }
    }
}

// one pass of the time loop body, SIMPLE_TS_MPI.cpp:3230-4691
void Oracle::step() {
  std::memcpy(p_pr, p, Na * sizeof(double));
  std::memcpy(u_pr, u, Na * sizeof(double));
  std::memcpy(v_pr, v, Na * sizeof(double));
  std::memcpy(Temper_pr, Temper, Na * sizeof(double));
  std::memcpy(rho_pr, rho, Na * sizeof(double));
  for (uint c = 0; c < Iter; c++) {
    max_res_p[c] = 0; max_res_T[c] = 0; max_res_p0[c] = 0; max_res_T0[c] = 0; max_Iter_p_c[c] = 0;
  }
  if (!guess_p.empty()) {
    for (const std::vector<uint>* list : {&nch_o, &bc_o})
      for (uint n : *list) {
        p[n] = guess_p[n];
        Temper[n] = guess_T[n];
      }
    guess_p.clear();
    guess_T.clear();
  } else if (warm_start == 3) {
    warm_ar();
  } else if (warm_start == 4) {
    warm_conv();
  } else if (warm_start) {
    if (!warm_ready) {
      p_m1.assign(p, p + Na);
      T_m1.assign(Temper, Temper + Na);
      p_m2 = p_m1;
      T_m2 = T_m1;
    } else {
      const bool quad = warm_start == 2 && warm_ready >= 2;
      for (const std::vector<uint>* list : {&nch_o, &bc_o})
        for (uint n : *list) {
          const double x = p[n], y = Temper[n];
          if (quad) {
            p[n] = 3.0 * (x - p_m1[n]) + p_m2[n];
            Temper[n] = 3.0 * (y - T_m1[n]) + T_m2[n];
          } else {
            p[n] = x + (x - p_m1[n]);
            Temper[n] = y + (y - T_m1[n]);
          }
          p_m2[n] = p_m1[n];
          T_m2[n] = T_m1[n];
          p_m1[n] = x;
          T_m1[n] = y;
        }
    }
    warm_ready++;
  }
  it += ht;
  it_counter++;
  Iter_pr2 = Iter_pr1;
  Iter_pr1 = Iter;
  Iter = 0;
  continue_iter = true;
  uint step_sweeps = 0;
  const std::vector<char>& b = vol;
  do {
    // ---- u momentum, boundary list (:3269-3344) ----
    for (size_t c = 0; c < bc_u.size(); c++) {
      Idx d = bc_idx(bc_u[c]);
      uint i = d.i, j = d.j;
      double F_xu1 = 0.5 * (Fx[d.i_1j] + Fx[d.ij]);
      double F_xu2 = 0.5 * (Fx[d.ij] + Fx[d.i1j]);
      double Scu = cT * (b[d.i1j] * u[d.i1j] * sqrt_T[d.ij] * hy[j] / (hx[i] * 3.0) +
                         b[d.i_2j] * u[d.i_1j] * sqrt_T[d.i_1j] * hy[j] / (hx[d.i_1] * 3.0) +
                         Gamma_yf[d.ij1] * (v[d.ij1] * b[d.ij1] - v[d.i_1j1] * b[d.i_1j1]) -
                         Gamma_yf[d.ij] * (v[d.ij] * b[d.ij_1] - v[d.i_1j] * b[d.i_1j_1]) -
                         sqrt_T[d.ij] * (v[d.ij1] * b[d.ij1] - v[d.ij] * b[d.ij_1]) * 2.0 / 3.0 +
                         sqrt_T[d.i_1j] * (v[d.i_1j1] * b[d.i_1j1] - v[d.i_1j] * b[d.i_1j_1]) * 2.0 / 3.0);
      double Spu = -(D_ux[d.ij] + D_ux[d.i1j]) / 3.0;
      double au1 = dmax(0, F_xu1) + D_ux[d.ij];
      double au2 = dmax(0, -F_xu2) + D_ux[d.i1j];
      double au3 = 0.5 * (dmax(0, Fy[d.i_1j]) + dmax(0, Fy[d.ij])) + D_uy[d.ij];
      double au4 = 0.5 * (dmax(0, -Fy[d.i_1j1]) + dmax(0, -Fy[d.ij1])) + D_uy[d.ij1];
      double bu3 = (rho_pr[d.i_1j] * hx[d.i_1] + rho_pr[d.ij] * hx[i]) * u_pr[d.ij] * hy[j] * 0.5 / ht + Scu;
      double au0 = au1 + au2 + au3 + au4 + 0.5 * (-Fy[d.i_1j] - Fy[d.ij] + Fy[d.i_1j1] + Fy[d.ij1]) + F_xu2 - F_xu1 -
                   Spu + (rho[d.i_1j] * hx[d.i_1] + rho[d.ij] * hx[i]) * hy[j] * 0.5 / ht;
      u_pseudo[d.ij] = (au1 * b[d.i1j] * u[d.i_1j] + au2 * b[d.i_2j] * u[d.i1j] + au3 * u[d.ij_1] + au4 * u[d.ij1] + bu3) / au0;
      d_p_c_12[d.ij] = cPch * hy[j] / au0;
      double hr = hy[j] * rho_u[d.ij];
      apx[d.ij] = d_p_c_12[d.ij] * hr;
      bpx[d.ij] = b[d.i_1j] * b[d.ij] * hr * u_pseudo[d.ij];
    }
    // ---- v momentum, boundary list (:3373-3450) ----
    for (size_t c = 0; c < bc_v.size(); c++) {
      Idx d = bc_idx(bc_v[c]);
      uint i = d.i, j = d.j;
      uint jm = j - 1 * (0 <= (int)(j - 1));
      uint far = d.ij_1 - Nx * (0 <= (int)(j - 2));
      double F_yv3 = 0.5 * (Fy[d.ij_1] + Fy[d.ij]);
      double F_yv4 = 0.5 * (Fy[d.ij] + Fy[d.ij1]);
      double Scv = cT * (b[d.ij1] * v[d.ij1] * sqrt_T[d.ij] * hx[i] / (hy[j] * 3.0) +
                         b[far] * v[d.ij_1] * sqrt_T[d.ij_1] * hx[i] / (hy[jm] * 3.0) +
                         Gamma_xf[d.i1j] * (u[d.i1j] * b[d.i1j] - u[d.i1j_1] * b[d.i1j_1]) -
                         Gamma_xf[d.ij] * (u[d.ij] * b[d.i_1j] - u[d.ij_1] * b[d.i_1j_1]) -
                         sqrt_T[d.ij] * (u[d.i1j] * b[d.i1j] - u[d.ij] * b[d.i_1j]) * 2.0 / 3.0 +
                         sqrt_T[d.ij_1] * (u[d.i1j_1] * b[d.i1j_1] - u[d.ij_1] * b[d.i_1j_1]) * 2.0 / 3.0) -
                   c_Fr_v * (rho[d.ij_1] * hx[i] * 0.5 * hy[jm] + rho[d.ij] * hx[i] * 0.5 * hy[j]);
      double Spv = -(D_vy[d.ij] + D_vy[d.ij1]) / 3.0;
      double av1 = 0.5 * (dmax(0, Fx[d.ij]) + dmax(0, Fx[d.ij_1])) + D_vx[d.ij];
      double av2 = 0.5 * (dmax(0, -Fx[d.i1j]) + dmax(0, -Fx[d.i1j_1])) + D_vx[d.i1j];
      double av3 = dmax(0, F_yv3) + D_vy[d.ij];
      double av4 = dmax(0, -F_yv4) + D_vy[d.ij1];
      double bv3 = (rho_pr[d.ij_1] * hy[j - 1] + rho_pr[d.ij] * hy[j]) * v_pr[d.ij] * hx[i] * 0.5 / ht + Scv;
      double av0 = av1 + av2 + av3 + av4 + 0.5 * (Fx[d.i1j] - Fx[d.ij] + Fx[d.i1j_1] - Fx[d.ij_1]) + F_yv4 - F_yv3 -
                   Spv + (rho[d.ij_1] * hy[j - 1] + rho[d.ij] * hy[j]) * hx[i] * 0.5 / ht;
      v_pseudo[d.ij] = (av1 * v[d.i_1j] + av2 * v[d.i1j] + av3 * b[far] * v[d.ij_1] + av4 * b[d.ij1] * v[d.ij1] + bv3) / av0;
      d_p_c_34[d.ij] = cPch * hx[i] / av0;
      double hr = hx[i] * rho_v[d.ij];
      apy[d.ij] = d_p_c_34[d.ij] * hr;
      bpy[d.ij] = b[d.ij - Nx] * b[d.ij] * hr * v_pseudo[d.ij];
    }
    // ---- u momentum, interior list (:3478-3545) ----
    for (size_t c = 0; c < nch_u.size(); c++) {
      uint n = nch_u[c];
      Idx d = clamped(n % Nx, n / Nx);
      uint i = d.i, j = d.j;
      double F_xu1 = 0.5 * (Fx[d.i_1j] + Fx[d.ij]);
      double F_xu2 = 0.5 * (Fx[d.ij] + Fx[d.i1j]);
      double Scu = cT * (u[d.i1j] * sqrt_T[d.ij] * hy[j] / (hx[i] * 3.0) +
                         u[d.i_1j] * sqrt_T[d.i_1j] * hy[j] / (hx[d.i_1] * 3.0) + Gamma_yf[d.ij1] * (v[d.ij1] - v[d.i_1j1]) -
                         Gamma_yf[d.ij] * (v[d.ij] - v[d.i_1j]) - sqrt_T[d.ij] * (v[d.ij1] - v[d.ij]) * 2.0 / 3.0 +
                         sqrt_T[d.i_1j] * (v[d.i_1j1] - v[d.i_1j]) * 2.0 / 3.0);
      double Spu = -(D_ux[d.ij] + D_ux[d.i1j]) / 3.0;
      double au1 = dmax(0, F_xu1) + D_ux[d.ij];
      double au2 = dmax(0, -F_xu2) + D_ux[d.i1j];
      double au3 = 0.5 * (dmax(0, Fy[d.i_1j]) + dmax(0, Fy[d.ij])) + D_uy[d.ij];
      double au4 = 0.5 * (dmax(0, -Fy[d.i_1j1]) + dmax(0, -Fy[d.ij1])) + D_uy[d.ij1];
      double bu3 = (rho_pr[d.i_1j] * hx[d.i_1] + rho_pr[d.ij] * hx[i]) * u_pr[d.ij] * hy[j] * 0.5 / ht + Scu;
      double au0 = au1 + au2 + au3 + au4 + 0.5 * (-Fy[d.i_1j] - Fy[d.ij] + Fy[d.i_1j1] + Fy[d.ij1]) + F_xu2 - F_xu1 -
                   Spu + (rho[d.i_1j] * hx[d.i_1] + rho[d.ij] * hx[i]) * hy[j] * 0.5 / ht;
      u_pseudo[d.ij] = (au1 * u[d.i_1j] + au2 * u[d.i1j] + au3 * u[d.ij_1] + au4 * u[d.ij1] + bu3) / au0;
      d_p_c_12[d.ij] = cPch * hy[j] / au0;
      double hr = hy[j] * rho_u[n];
      apx[n] = d_p_c_12[n] * hr;
      bpx[n] = hr * u_pseudo[n];
    }
    // ---- v momentum, interior list (:3561-3630) ----
    for (size_t c = 0; c < nch_v.size(); c++) {
      uint n = nch_v[c];
      Idx d = clamped(n % Nx, n / Nx);
      uint i = d.i, j = d.j;
      double F_yv3 = 0.5 * (Fy[d.ij_1] + Fy[d.ij]);
      double F_yv4 = 0.5 * (Fy[d.ij] + Fy[d.ij1]);
      double Scv = cT * (v[d.ij1] * sqrt_T[d.ij] * hx[i] / (hy[j] * 3.0) + v[d.ij_1] * sqrt_T[d.ij_1] * hx[i] / (hy[j - 1] * 3.0) +
                         Gamma_xf[d.i1j] * (u[d.i1j] - u[d.i1j_1]) - Gamma_xf[d.ij] * (u[d.ij] - u[d.ij_1]) -
                         sqrt_T[d.ij] * (u[d.i1j] - u[d.ij]) * 2.0 / 3.0 +
                         sqrt_T[d.ij_1] * (u[d.i1j_1] - u[d.ij_1]) * 2.0 / 3.0) -
                   c_Fr_v * (rho[d.ij_1] * hx[i] * 0.5 * hy[j - 1] + rho[d.ij] * hx[i] * 0.5 * hy[j]);
      double Spv = -(D_vy[d.ij] + D_vy[d.ij1]) / 3.0;
      double av1 = 0.5 * (dmax(0, Fx[d.ij]) + dmax(0, Fx[d.ij_1])) + D_vx[d.ij];
      double av2 = 0.5 * (dmax(0, -Fx[d.i1j]) + dmax(0, -Fx[d.i1j_1])) + D_vx[d.i1j];
      double av3 = dmax(0, F_yv3) + D_vy[d.ij];
      double av4 = dmax(0, -F_yv4) + D_vy[d.ij1];
      double bv3 = (rho_pr[d.ij_1] * hy[j - 1] + rho_pr[d.ij] * hy[j]) * v_pr[d.ij] * hx[i] * 0.5 / ht + Scv;
      double av0 = av1 + av2 + av3 + av4 + 0.5 * (Fx[d.i1j] - Fx[d.ij] + Fx[d.i1j_1] - Fx[d.ij_1]) + F_yv4 - F_yv3 -
                   Spv + (rho[d.ij_1] * hy[j - 1] + rho[d.ij] * hy[j]) * hx[i] * 0.5 / ht;
      v_pseudo[d.ij] = (av1 * v[d.i_1j] + av2 * v[d.i1j] + av3 * v[d.ij_1] + av4 * v[d.ij1] + bv3) / av0;
      d_p_c_34[d.ij] = cPch * hx[i] / av0;
      double hr = hx[i] * rho_v[n];
      apy[n] = d_p_c_34[n] * hr;
      bpy[n] = hr * v_pseudo[n];
    }
    // ---- energy source ScT1 (:3655-3756) ----
    for (size_t c = 0; c < nch_o.size(); c++) {
      uint n = nch_o[c];
      Idx d = clamped(n % Nx, n / Nx);
      uint i = d.i, j = d.j;
      uint jm = j - 1 * (0 < j), jp = j + 1 * (j < (Nx - 1));  // the reference compares j against Nx here
      double dudx = (u[d.i1j] - u[d.ij]) / hx[i];
      double dvdy = (v[d.ij1] - v[d.ij]) / hy[j];
      double s0 = ((u[d.ij] - u[d.ij_1]) / (hy[jm] + hy[j])) + ((v[d.ij] - v[d.i_1j]) / (hx[d.i_1] + hx[i]));
      double s1 = ((u[d.i1j] - u[d.i1j_1]) / (hy[jm] + hy[j])) + ((v[d.i1j] - v[d.ij]) / (hx[i] + hx[d.i1]));
      double s2 = ((u[d.ij1] - u[d.ij]) / (hy[j] + hy[jp])) + ((v[d.ij1] - v[d.i_1j1]) / (hx[d.i_1] + hx[i]));
      double s3 = ((u[d.i1j1] - u[d.i1j]) / (hy[j] + hy[jp])) + ((v[d.i1j1] - v[d.ij1]) / (hx[i] + hx[d.i1]));
      ScT1[d.ij] = ht * sqrt_T[d.ij] * cT2 * hx[i] * hy[j] *
                       (2.0 * (dudx * dudx + dvdy * dvdy) + s0 * s0 + s1 * s1 + s2 * s2 + s3 * s3 -
                        (dudx + dvdy) * (dudx + dvdy) * 2.0 / 3.0) +
                   p_pr[d.ij] * hx[i] * hy[j];
    }
    for (size_t c = 0; c < bc_o.size(); c++) {
      Idx d = bc_idx(bc_o[c]);
      uint i = d.i, j = d.j;
      uint jm = j - 1 * (0 < j), jp = j + 1 * (j < (Nx - 1));
      double dudx = (b[d.i1j] * u[d.i1j] - b[d.i_1j] * u[d.ij]) / hx[i];
      double dvdy = (b[d.ij1] * v[d.ij1] - b[d.ij_1] * v[d.ij]) / hy[j];
      double s0 = ((u[d.ij] - u[d.ij_1]) / ((b[d.i_1j_1] && b[d.ij_1]) * hy[jm] + hy[j])) +
                  ((v[d.ij] - v[d.i_1j]) / ((b[d.i_1j_1] && b[d.i_1j]) * hx[d.i_1] + hx[i]));
      double s1 = ((u[d.i1j] - u[d.i1j_1]) / ((b[d.ij_1] && b[d.i1j_1]) * hy[jm] + hy[j])) +
                  ((v[d.i1j] - v[d.ij]) / (hx[i] + (b[d.i1j_1] && b[d.i1j]) * hx[d.i1]));
      double s2 = ((u[d.ij1] - u[d.ij]) / (hy[j] + (b[d.i_1j1] && b[d.ij1]) * hy[jp])) +
                  ((v[d.ij1] - v[d.i_1j1]) / ((b[d.i_1j] && b[d.i_1j1]) * hx[d.i_1] + hx[i]));
      double s3 = ((u[d.i1j1] - u[d.i1j]) / (hy[j] + (b[d.ij1] && b[d.i1j1]) * hy[jp])) +
                  ((v[d.i1j1] - v[d.ij1]) / (hx[i] + (b[d.i1j] && b[d.i1j1]) * hx[d.i1]));
      ScT1[d.ij] = ht * sqrt_T[d.ij] * cT2 * hx[i] * hy[j] *
                       (2.0 * (dudx * dudx + dvdy * dvdy) + s0 * s0 + s1 * s1 + s2 * s2 + s3 * s3 -
                        (dudx + dvdy) * (dudx + dvdy) * 2.0 / 3.0) +
                   p_pr[d.ij] * hx[i] * hy[j];
    }
    std::memcpy(p_old, p, Na * sizeof(double));
    std::memcpy(Temper_old, Temper, Na * sizeof(double));
    // ---- coupled p-T Jacobi sweeps (:3786-4131) ----
    pt_sweeps();
    max_Iter_p_c[Iter] = Iter_p_c;
    step_sweeps += Iter_p_c;
    // ---- velocity correction (:4171-4305) ----
    max_residual_in_u = 0;
    for (size_t c = 0; c < bc_u.size(); c++) {
      Idx d = bc_idx(bc_u[c]);
      double t = u[d.ij];
      u[d.ij] = u_pseudo[d.ij] - (p[d.ij] - p[d.i_1j]) * d_p_c_12[d.ij];
      double r = u[d.ij] - t;
      if (max_residual_in_u < std::fabs(r)) max_residual_in_u = std::fabs(r);
    }
    max_residual_in_v = 0;
    for (size_t c = 0; c < bc_v.size(); c++) {
      uint n = bc_v[c];
      double t = v[n];
      v[n] = v_pseudo[n] - (p[n] - p[n - Nx]) * d_p_c_34[n];
      double r = v[n] - t;
      if (max_residual_in_v < std::fabs(r)) max_residual_in_v = std::fabs(r);
    }
    for (size_t c = 0; c < nch_u.size(); c++) {
      uint n = nch_u[c];
      double t = u[n];
      u[n] = u_pseudo[n] - (p[n] - p[n - 1]) * d_p_c_12[n];
      double r = u[n] - t;
      if (max_residual_in_u < std::fabs(r)) max_residual_in_u = std::fabs(r);
    }
    for (size_t c = 0; c < nch_v.size(); c++) {
      uint n = nch_v[c];
      double t = v[n];
      v[n] = v_pseudo[n] - (p[n] - p[n - Nx]) * d_p_c_34[n];
      double r = v[n] - t;
      if (max_residual_in_v < std::fabs(r)) max_residual_in_v = std::fabs(r);
    }
    // ---- sqrt(T), density (:4323-4330) ----
    for (uint c = 0; c < Na; c++) {
      sqrt_T[c] = std::sqrt(Temper[c]);
      if (vol[c]) rho[c] = p[c] / Temper[c];
      else rho[c] = 0;
    }
    nondim_refresh();
    solve_rho_mid();
    Iter++;
    if (Iter == 1) {
      max_residual_in_u_Iter_0 = max_residual_in_u;
      max_residual_in_v_Iter_0 = max_residual_in_v;
    }
    continue_iter = (Iter < N_I && (MaxError_Velocities < max_residual_in_u || MaxError_Velocities < max_residual_in_v ||
                                    MaxError_p_c < max_res_p[Iter - 1] || MaxError_T < max_res_T[Iter - 1]));
    countinue_time_step =
        (it_counter < Nt && (!check_wallclock || time(NULL) < time_solve_stop) &&
         ((!(Iter <= 1 && Iter_p_c <= 2)) || MaxError_to_stop_program < max_residual_in_u ||
          MaxError_to_stop_program < max_residual_in_v || MaxError_to_stop_program < max_res_p0[Iter - 1] ||
          MaxError_to_stop_program < max_res_T0[Iter - 1]));
    // ---- boundary conditions, fluxes, diffusion (:4460-4532) ----
    bc_slip_u();
    bc_slip_v();
    bc_velocities();
    bc_pressure_begin_it();
    bc_tjump();
    bc_temperature();
    bc_pressure();
    solve_fluxes();
    solve_diffusion();
    if (ToSolveContinuityEquation) solve_continuity();  // :4588-4591
  } while (continue_iter);
  sweeps_per_step.push_back(step_sweeps);
  bc_function_of_time();
  Nt_save_solved_data_counter++;
  if (Nt_save_solved_data_counter >= Nt_save_solved_data) {
    if (apply_saves) {
      write_solved();
      if (ToSolveContinuityEquation) solve_continuity();  // :4635-4643
    }
    Nt_save_solved_data_counter = 0;
  }
  Nt_save_DragCoefficient_counter++;
  if (Nt_save_DragCoefficient_counter >= Nt_save_DragCoefficient) {
    if (apply_saves) write_drag();
    Nt_save_DragCoefficient_counter = 0;
  }
  Nt_save_temp_data_counter++;
  if (Nt_save_temp_data_counter >= Nt_save_temp_data) {
    write_temp();
    write_iterations();
    Nt_save_temp_data_counter = 0;
  }
}

// after the time loop, SIMPLE_TS_MPI.cpp:4695-4714
void Oracle::finish() {
  solve_is_finished = Iter <= 1 && Iter_p_c <= 1 && max_residual_in_u < MaxError_to_stop_program &&
                      max_residual_in_v < MaxError_to_stop_program && max_res_p[Iter - 1] < MaxError_to_stop_program &&
                      max_res_T[Iter - 1] < MaxError_to_stop_program;
  write_solved();
  if (ToSolveContinuityEquation) solve_continuity();
  write_drag();
  write_temp();
}

}  // namespace

// ---------------------------------------------------------------------------
// C interface used by the tests (ctypes) and the CLI below.
// ---------------------------------------------------------------------------
struct ora_handle {
  Oracle o;
};

extern "C" {

// fixed_sweeps: 1 = FIXED_NUMBER_OF_ITERATIONS_LOOP_3 defined (the shipped build), 0 = residual-terminated.
ora_handle* ora_open(const char* dir, int fixed_sweeps, int write_files) {
  ora_handle* h = new ora_handle;
  h->o.dir = dir;
  h->o.fixed_sweeps = fixed_sweeps != 0;
  h->o.write_files = write_files != 0;
  if (!h->o.setup()) {
    std::fprintf(stderr, "oracle setup failed: %s\n", h->o.err.c_str());
    delete h;
    return nullptr;
  }
  return h;
}

// Runs up to n time steps; stops early when the reference's continue rule says so.
// Returns the number of steps taken.
void ora_set_warm_start(ora_handle* h, int mode) { h->o.warm_start = mode; }

// The next step's sweeps start from p_guess, T_guess (Nx*Ny each) on the solved cells.
void ora_set_guess(ora_handle* h, const double* p_guess, const double* T_guess) {
  h->o.guess_p.assign(p_guess, p_guess + h->o.Na);
  h->o.guess_T.assign(T_guess, T_guess + h->o.Na);
}

int ora_step(ora_handle* h, int n) {
  int k = 0;
  for (; k < n; k++) {
    if (h->o.finished) break;
    h->o.step();
    if (!h->o.countinue_time_step) h->o.finished = true;
  }
  return k;
}

void ora_finish(ora_handle* h) { h->o.finish(); }
void ora_close(ora_handle* h) { delete h; }

int ora_dims(ora_handle* h, int* nx, int* ny) {
  *nx = (int)h->o.Nx;
  *ny = (int)h->o.Ny;
  return 0;
}

// Copies a named field (Nx*Ny doubles) into out; returns 0 or -1 for an unknown name.
int ora_get(ora_handle* h, const char* name, double* out) {
  Oracle& o = h->o;
  std::string s(name);
  const double* src = nullptr;
  if (s == "u") src = o.u;
  else if (s == "v") src = o.v;
  else if (s == "p") src = o.p;
  else if (s == "T") src = o.Temper;
  else if (s == "rho") src = o.rho;
  else if (s == "sqrt_T") src = o.sqrt_T.data();
  else if (s == "rho_u") src = o.rho_u.data();
  else if (s == "rho_v") src = o.rho_v.data();
  else if (s == "Fx") src = o.Fx.data();
  else if (s == "Fy") src = o.Fy.data();
  else if (s == "D_ux") src = o.D_ux.data();
  else if (s == "D_uy") src = o.D_uy.data();
  else if (s == "D_vx") src = o.D_vx.data();
  else if (s == "D_vy") src = o.D_vy.data();
  else if (s == "DTx") src = o.DTx.data();
  else if (s == "DTy") src = o.DTy.data();
  else if (s == "Gamma_xf") src = o.Gamma_xf.data();
  else if (s == "Gamma_yf") src = o.Gamma_yf.data();
  else if (s == "ScT1") src = o.ScT1.data();
  else if (s == "apx") src = o.apx.data();
  else if (s == "apy") src = o.apy.data();
  else if (s == "bpx") src = o.bpx.data();
  else if (s == "bpy") src = o.bpy.data();
  else if (s == "u_pseudo") src = o.u_pseudo.data();
  else if (s == "v_pseudo") src = o.v_pseudo.data();
  else if (s == "d_p_c_12") src = o.d_p_c_12.data();
  else if (s == "d_p_c_34") src = o.d_p_c_34.data();
  else if (s == "Tw_u") src = o.Tw_u.data();
  else if (s == "Tw_v") src = o.Tw_v.data();
  else if (s == "hx") { std::memcpy(out, o.hx.data(), sizeof(double) * o.Nx); return 0; }
  else if (s == "hy") { std::memcpy(out, o.hy.data(), sizeof(double) * o.Ny); return 0; }
  else if (s == "x_v") { std::memcpy(out, o.x_v.data(), sizeof(double) * o.Nx); return 0; }
  else if (s == "y_v") { std::memcpy(out, o.y_v.data(), sizeof(double) * o.Ny); return 0; }
  if (!src) return -1;
  std::memcpy(out, src, sizeof(double) * o.Na);
  return 0;
}

// The interior/boundary lists encoded one byte per cell: bits 0-1 u, 2-3 v, 4-5 p/T
// (1 = interior list, 2 = boundary list), bit 6 fluid.
int ora_get_class(ora_handle* h, unsigned char* out) {
  Oracle& o = h->o;
  for (uint c = 0; c < o.Na; c++) out[c] = o.vol[c] ? 0x40 : 0;
  for (uint n : o.nch_u) out[n] |= 1;
  for (uint n : o.bc_u) out[n] |= 2;
  for (uint n : o.nch_v) out[n] |= 1 << 2;
  for (uint n : o.bc_v) out[n] |= 2 << 2;
  for (uint n : o.nch_o) out[n] |= 1 << 4;
  for (uint n : o.bc_o) out[n] |= 2 << 4;
  return 0;
}

int ora_get_mask(ora_handle* h, unsigned int* out) {
  std::memcpy(out, h->o.vol_inf_fb.data(), sizeof(unsigned int) * h->o.Na);
  return 0;
}

// The p-T sweep loop alone (Oracle::pt_sweeps, the same code the time step runs) on host
// arrays: cls uses the class-byte layout of ora_get_class (bits 4-5 p/T class, bit 6 fluid);
// p and T hold the initial iterate and receive the result.
int ora_pt_sweeps(int Nx, int Ny, int periodic, int given_xb, int given_xe, int Nx_o0, int Nx_o1, double ht,
                  double gamma1, const unsigned char* cls, const double* hx, const double* hy, const double* Fx,
                  const double* Fy, const double* DTx, const double* DTy, const double* u, const double* v,
                  const double* rho, const double* ScT1, const double* apx, const double* apy, const double* bpx,
                  const double* bpy, const double* p_pr, const double* T_pr, const double* Tw_u, const double* Tw_v,
                  double* p, double* T, int max_sweeps, int fixed, double tol_p, double tol_T, int* sweeps_done,
                  double* res_p, double* res_T) {
  Oracle o;
  const uint Na = (uint)(Nx * Ny);
  o.Nx = (uint)Nx; o.Ny = (uint)Ny; o.Na = Na;
  o.Periodic = periodic != 0;
  o.Given_velocity_on_xb = given_xb != 0;
  o.Given_velocity_on_xe = given_xe != 0;
  o.Nx_o[0] = (uint)Nx_o0; o.Nx_o[1] = (uint)Nx_o1;
  o.ht = ht; o.gamma1 = gamma1;
  o.N_I_p_c = (uint)max_sweeps; o.fixed_sweeps = fixed != 0;
  o.MaxError_p_c = tol_p; o.MaxError_T = tol_T;
  auto cp = [&](std::vector<double>& dst, const double* src, uint n) { dst.assign(src, src + n); };
  cp(o.hx, hx, (uint)Nx); cp(o.hy, hy, (uint)Ny);
  cp(o.Fx, Fx, Na); cp(o.Fy, Fy, Na); cp(o.DTx, DTx, Na); cp(o.DTy, DTy, Na); cp(o.st_u0, u, Na); cp(o.st_v0, v, Na);
  cp(o.st_r0, rho, Na); cp(o.ScT1, ScT1, Na); cp(o.apx, apx, Na); cp(o.apy, apy, Na); cp(o.bpx, bpx, Na);
  cp(o.bpy, bpy, Na); cp(o.st_p1, p_pr, Na); cp(o.st_T1, T_pr, Na); cp(o.Tw_u, Tw_u, Na); cp(o.Tw_v, Tw_v, Na);
  cp(o.st_p0, p, Na); cp(o.st_p2, p, Na); cp(o.st_T0, T, Na); cp(o.st_T2, T, Na);
  o.u = o.st_u0.data(); o.v = o.st_v0.data(); o.rho = o.st_r0.data();
  o.p = o.st_p0.data(); o.p_pr = o.st_p1.data(); o.p_old = o.st_p2.data();
  o.Temper = o.st_T0.data(); o.Temper_pr = o.st_T1.data(); o.Temper_old = o.st_T2.data();
  o.vol.assign(Na, 0);
  for (uint c = 0; c < Na; c++) {
    o.vol[c] = (cls[c] >> 6) & 1;
    const int k = (cls[c] >> 4) & 3;
    if (k == 1) o.nch_o.push_back(c);
    else if (k == 2) o.bc_o.push_back(c);
  }
  o.max_res_p.assign(1, 0); o.max_res_T.assign(1, 0); o.max_res_p0.assign(1, 0); o.max_res_T0.assign(1, 0);
  o.Iter = 0;
  o.pt_sweeps();
  std::memcpy(p, o.p, sizeof(double) * Na);
  std::memcpy(T, o.Temper, sizeof(double) * Na);
  if (sweeps_done) *sweeps_done = (int)o.Iter_p_c;
  if (res_p) *res_p = o.max_res_p[0];
  if (res_T) *res_T = o.max_res_T[0];
  return 0;
}

// Global conservation sums of the current state (the GB300 library's sts_conservation, which has
// no counterpart in the reference): per fluid cell, A = hx hy, u_c = (u_ij + u_i+1,j) / 2,
// v_c = (v_ij + v_i,j+1) / 2 (neighbour clamped at the last column or row); mass rho A, momentum
// rho A u_c and rho A v_c, internal energy rho A T / (gamma - 1), kinetic energy
// rho A (u_c^2 + v_c^2).  Summed in the library's fixed order: chunks of 64 cells of a row in x
// order, the chunks of a row in order, the rows in y order.
int ora_conservation(ora_handle* h, double* out) {
  Oracle& o = h->o;
  const int Nx = (int)o.Nx, Ny = (int)o.Ny, CH = 64, nch = (Nx + CH - 1) / CH;
  double tot[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int j = 0; j < Ny; j++) {
    double row[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = 0; k < nch; k++) {
      double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
      for (int i = k * CH; i < std::min(Nx, (k + 1) * CH); i++) {
        const int n = i + j * Nx;
        if (!o.vol[n]) continue;
        const int ne = (i + 1 < Nx) ? n + 1 : n, nn = (j + 1 < Ny) ? n + Nx : n;
        const double A = o.hx[i] * o.hy[j];
        const double uc = 0.5 * (o.u[n] + o.u[ne]), vc = 0.5 * (o.v[n] + o.v[nn]);
        const double m = o.rho[n] * A;
        s[0] = s[0] + m;
        s[1] = s[1] + m * uc;
        s[2] = s[2] + m * vc;
        s[3] = s[3] + (m * o.Temper[n]) / (o.gamma1 - 1.0);
        s[4] = s[4] + m * (uc * uc + vc * vc);
      }
      for (int q = 0; q < 5; q++) row[q] = row[q] + s[q];
    }
    for (int q = 0; q < 5; q++) tot[q] = tot[q] + row[q];
  }
  for (int q = 0; q < 5; q++) out[q] = tot[q];
  return 0;
}

// Per-step sweep counts (sum over outer iterations), oldest first; returns how many were copied.
int ora_sweeps(ora_handle* h, unsigned int* out, int cap) {
  int n = (int)h->o.sweeps_per_step.size();
  if (n > cap) n = cap;
  for (int k = 0; k < n; k++) out[k] = h->o.sweeps_per_step[k];
  return n;
}

// Last step: [Iter, Iter_p_c, res_p0, res_p, res_T0, res_T, res_u, res_v, it]
int ora_stats(ora_handle* h, double* out) {
  Oracle& o = h->o;
  uint I = o.Iter ? o.Iter - 1 : 0;
  out[0] = o.Iter; out[1] = o.Iter_p_c;
  out[2] = o.max_res_p0[I]; out[3] = o.max_res_p[I]; out[4] = o.max_res_T0[I]; out[5] = o.max_res_T[I];
  out[6] = o.max_residual_in_u; out[7] = o.max_residual_in_v; out[8] = o.it;
  return 0;
}

}  // extern "C"

#ifdef STS_ORACLE_MAIN
// Drop-in CLI: runs a case directory like the serial reference binary.
int main(int argc, char** argv) {
  const char* dir = argc > 1 ? argv[1] : ".";
  int fixed = 1;
  for (int k = 2; k < argc; k++)
    if (std::strcmp(argv[k], "--residual") == 0) fixed = 0;
  ora_handle* h = ora_open(dir, fixed, 1);
  if (!h) return 2;
  h->o.check_wallclock = true;
  h->o.apply_saves = true;
  while (!h->o.finished) ora_step(h, 1 << 20);
  ora_finish(h);
  ora_close(h);
  return 0;
}
#endif
