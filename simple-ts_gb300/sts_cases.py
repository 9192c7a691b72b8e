"""Case files for the SIMPLE-TS time step: EnteredData.txt, body files, restart dumps.

The reference solver is driven entirely by files in its working directory
(SIMPLE_TS_MPI.cpp:5241-5561 reads ``EnteredData.txt``; Objects_for_Solving.h:306-412
reads ``solve_polyhedrons_b.txt``; SIMPLE_TS_MPI.cpp:5734-5835 reads the restart
dumps ``u.bin v.bin p.bin Temper.bin vol_inf_fb.bin`` and ``it_begin.txt``).
This module writes those files so that the same directory can be handed to the
reference binary, to the CPU oracle and to the GB300 driver.

The field order of ``EnteredData.txt`` is positional: one value per line, the
rest of the line is ignored (SIMPLE_TS_MPI.cpp:5253-5544).  ``ENTERED_DATA``
lists the 126 fields in that order with the values of the example input that
ships with the reference.

The workloads (channel with a confined square, Rayleigh-Benard box, batches of
channels) are described by seeded builders below; they are synthetic inputs
generated from their published shapes, sizes and parameter ranges.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# (name, kind, default) in the reader's order; kind: 'd' double, 'u' unsigned, 'b' bool.
ENTERED_DATA: List[Tuple[str, str, object]] = [
    ("u_gas_nd", "d", 0.0), ("v_gas_nd", "d", 0.0), ("T_gas_nd", "d", 1.0), ("p_gas_nd", "d", 1.0),
    ("Ma", "d", 1.09544511501033), ("Pr", "d", 0.666666666666667), ("gamma1", "d", 1.66666666666667),
    ("c_mu", "d", 0.606758097673656), ("Kn", "d", 0.050029296), ("Fr", "d", 50.0),
    ("SolveGravityField", "b", 0), ("Re", "d", 250.0), ("TypeOfNonDimensiolization", "u", 3),
    ("Nt", "d", 11000000), ("Nx", "u", 282), ("Ny", "u", 63), ("N_I", "u", 1), ("N_I_p_c", "u", 2),
    ("N_I_T", "u", 3000), ("ht", "d", 0.01),
    ("x_b", "d", -2.0), ("x_e", "d", 12.05), ("y_b", "d", -1.0), ("y_e", "d", 2.05),
    ("kind_of_mesh", "u", 5),
    ("hxmin", "d", 0.05), ("hxmax", "d", 0.05), ("xfmin", "d", -0.7), ("xfmax", "d", -2.7),
    ("xbmin", "d", 0.7), ("xbmax", "d", 2.7), ("xmid", "d", 0.0),
    ("hymin", "d", 0.05), ("hymax", "d", 0.05), ("ytmin", "d", 0.7), ("ytmax", "d", 2.7),
    ("ybmin", "d", -0.7), ("ybmax", "d", -2.7), ("ymid", "d", 0.0),
    ("MaxError_Velocities", "d", 1e-08), ("MaxError_p_c", "d", 1e-09), ("MaxError_T", "d", 1e-09),
    ("MaxError_to_stop_program", "d", 1e-12), ("max_time_for_solve", "d", 1000.0),
    ("solve_is_finished", "b", 0),
    ("Nt_save_solved_data", "u", 1), ("Nt_save_DragCoefficient", "u", 10000000),
    ("Nt_save_temp_data", "u", 1), ("N_I_check", "u", 1), ("WriteDataInShortFormat_kind", "u", 0),
    ("ToReadSolvedDataFromFile", "b", 0), ("ToReadSolvedDataFromBinaryFile", "b", 1),
    ("ToWriteSolvedDataToBinaryFile", "b", 1), ("ToWriteSolvedDataToNewFiles", "b", 0),
    ("ToContinueFromInterpolation", "b", 0),
    ("ToImport_data_for_circles_from_file_b", "b", 0), ("ToImport_data_for_polyhedrons_from_file_b", "b", 1),
    ("ToImport_data_for_circles_from_file_p", "b", 0), ("ToImport_data_for_polyhedrons_from_file_p", "b", 0),
    ("ToImport_data_for_circles_from_file_V", "b", 0), ("ToImport_data_for_polyhedrons_from_file_V", "b", 0),
    ("Given_velocity_on_xb", "b", 0), ("Given_velocity_on_xe", "b", 0),
    ("Periodic_boundary_conditions_about_OX", "b", 0), ("Pressure_BC", "b", 1),
    ("ToStartFromExactSolutionForChannelFlowWithPressureBC", "b", 0),
    ("p_BC_xb_correction_method", "u", 0), ("Pressure_ratio_correct", "b", 0), ("GivenReKn", "b", 0),
    ("correct_p_BC_xb", "b", 1), ("u_given_xb", "d", 2.2147), ("u_given_xb_error", "d", 0.0001),
    ("p_correction_auto", "b", 0), ("p_correction_min", "d", 0.001), ("p_correction_max", "d", 2.0),
    ("p_correction", "d", 0.05),
    ("p_BC_xb", "d", 3.0), ("T_BC_xb", "d", 1.0), ("p_BC_xe", "d", 1.0), ("T_BC_xe", "d", 1.0),
    ("dudx_0_BC_xb", "b", 0), ("durhodx_0_BC_xb", "b", 0), ("drhodt_durhodx_dvrhody_0_BC_xb", "b", 1),
    ("ToCalculate_ui_1j_from_equation_for_uij_at_x_b", "b", 0),
    ("dudx_0_BC_xe", "b", 0), ("durhodx_0_BC_xe", "b", 0), ("drhodt_durhodx_dvrhody_0_BC_xe", "b", 1),
    ("ToCalculate_ui1j_from_equation_for_uij_at_x_e", "b", 0), ("u_uMin_Mout_0_BC_xe", "b", 0),
    ("dudy_0_BC_yb", "b", 0), ("dudy_0_BC_ye", "b", 0),
    ("dvdx_0_BC_xb", "b", 1), ("ToCalculate_vi_1j_from_equation_for_vij_at_x_b", "b", 0),
    ("dvdx_0_BC_xe", "b", 1), ("ToCalculate_vi1j_from_equation_for_vij_at_x_e", "b", 0),
    ("dvdy_0_BC_yb", "b", 0), ("dvdy_0_BC_ye", "b", 0),
    ("dpdx_0_BC_xb", "b", 0), ("ToCalculate_pi_1j_from_equation_for_pij_at_x_b", "b", 0),
    ("dpdx_0_BC_xe", "b", 0), ("ToCalculate_pi1j_from_equation_for_pij_at_x_e", "b", 0),
    ("dpdy_0_BC_yb", "b", 0), ("dpdy_0_BC_ye", "b", 0),
    ("dTdx_0_BC_xb", "b", 0), ("ToCalculate_Temperi_1j_from_equation_for_Temperij_at_x_b", "b", 0),
    ("dTdx_0_BC_xe", "b", 1), ("ToCalculate_Temperi1j_from_equation_for_Temperij_at_x_e", "b", 0),
    ("dTdy_0_BC_yb", "b", 0), ("dTdy_0_BC_ye", "b", 0),
    ("To_Use_Kn_local_in_wall_BC", "b", 1), ("ToSolveContinuityEquation", "b", 0),
    ("use_interpolation_for_u_BC_by_time", "b", 0), ("t_BC_b", "d", 0.0), ("t_BC_e", "d", 2.0),
    ("u_BC_xb_t_BC_b", "d", 0.4), ("u_BC_xb_t_BC_e", "d", 0.5),
    ("w_u", "d", 1.0), ("w_v", "d", 1.0), ("w_p", "d", 1.0), ("w_Temper", "d", 1.0),
    ("N_SubDomains_x", "u", 2), ("N_SubDomains_y", "u", 1),
    ("ToReadSolvedDataFromSeparateFileForEachSubDomain", "b", 0),
    ("ToWriteSolvedDataToFileForEntireComputationalDomain", "b", 1),
    ("ToWriteSolvedDataToSeparateFileForEachSubDomain", "b", 0),
    ("ToOnlyWriteDataFor_Nx_Ny_ForAllSubDomains_AndExit", "b", 0),
]
assert len(ENTERED_DATA) == 126
FIELD_INDEX = {name: k for k, (name, _, _) in enumerate(ENTERED_DATA)}

# Body defaults of the reference constructors (Polyhedrons_Objects.cpp:39-67, Circles_Objects.cpp:29-50)
SLIP_F = 1.1466
JUMP_F = 2.1904


def _fmt(kind: str, value) -> str:
    if kind in "ub":
        return str(int(value))
    return repr(float(value))


def format_entered_data(values: Dict[str, object]) -> str:
    lines = []
    for name, kind, default in ENTERED_DATA:
        v = values.get(name, default)
        lines.append(f"{_fmt(kind, v)}\t//{name}")
    unknown = set(values) - set(FIELD_INDEX)
    if unknown:
        raise KeyError(f"unknown EnteredData fields: {sorted(unknown)}")
    return "\n".join(lines) + "\n"


def read_entered_data(path: str) -> Dict[str, float]:
    """Positional reader with the reference's rule: first token of each line."""
    out: Dict[str, float] = {}
    with open(path) as f:
        lines = f.read().splitlines()
    for k, (name, kind, _) in enumerate(ENTERED_DATA):
        tok = lines[k].split()[0]
        out[name] = int(tok) if kind in "ub" else float(tok)
    return out


@dataclass
class Polygon:
    vertices: Sequence[Tuple[float, float]]
    inside1: Tuple[float, float]
    inside2: Tuple[float, float]
    u_body: float = 0.0
    v_body: float = 0.0
    p_body: float = 0.0
    T_body: float = 1.0
    slip: int = 1
    F_slip: float = SLIP_F
    w_slip: float = 0.0
    jump: int = 1
    F_jump: float = JUMP_F
    dTdn0: float = 0.0
    drag: int = 0


@dataclass
class Circle:
    xc: float
    yc: float
    rc: float
    u_body: float = 0.0
    v_body: float = 0.0
    p_body: float = 0.0
    T_body: float = 1.0
    slip: int = 1
    F_slip: float = SLIP_F
    w_slip: float = 0.0
    jump: int = 1
    F_jump: float = JUMP_F
    dTdn0: float = 0.0
    drag: int = 0


def format_polygons(polys: Sequence[Polygon]) -> str:
    """Layout read by Objects_for_Solving::Import_data_for_polyhedrons_from_file."""
    out = [f"{len(polys)}\t//N_polyhedrons"]
    for P in polys:
        out += [
            f"{len(P.vertices)}\t//N_vertex_body",
            f"{P.inside1[0]!r}\t{P.inside1[1]!r}\t//point1_inside_x point1_inside_y",
            f"{P.inside2[0]!r}\t{P.inside2[1]!r}\t//point2_inside_x point2_inside_y",
            f"{P.u_body!r}\t{P.v_body!r}\t//u_body v_body",
            f"{P.p_body!r}\t//pressure in polyhedron",
            f"{P.T_body!r}\t//Temperature in polyhedron",
            f"{int(P.slip)}\t//is_VelocitySlipBC_body",
            f"{P.F_slip!r}\t//F_VelocitySlip",
            f"{P.w_slip!r}\t//w_VelocitySlipBC",
            f"{int(P.jump)}\t//is_TemperatureJumpBC_body",
            f"{P.F_jump!r}\t//F_TemperatureJump",
            f"{P.dTdn0!r}\t//dTdn_on_wall_0",
            f"{int(P.drag)}\t//ToSolveDragCoefficientForThisBody",
        ]
        out += [f"{x!r}\t{y!r}" for (x, y) in P.vertices]
    return "\n".join(out) + "\n"


def format_circles(circles: Sequence[Circle]) -> str:
    """Layout read by Objects_for_Solving::Import_data_for_circles_from_file."""
    out = [f"{len(circles)}\t//N_circles"]
    for C in circles:
        out += [
            f"{C.xc!r}\t{C.yc!r}\t{C.rc!r}\t//x_c y_c r_c",
            f"{C.u_body!r}\t{C.v_body!r}\t//u_body v_body",
            f"{C.p_body!r}\t//p_body",
            f"{C.T_body!r}\t//T_body",
            f"{int(C.slip)}\t//is_VelocitySlipBC_body",
            f"{C.F_slip!r}\t//F_VelocitySlip",
            f"{C.w_slip!r}\t//w_VelocitySlipBC",
            f"{int(C.jump)}\t//is_TemperatureJumpBC_body",
            f"{C.F_jump!r}\t//F_TemperatureJump",
            f"{C.dTdn0!r}\t//dTdn_on_wall_0",
            f"{int(C.drag)}\t//ToSolveDragCoefficientForThisBody",
        ]
    return "\n".join(out) + "\n"


@dataclass
class Case:
    """Everything one run directory holds."""
    name: str
    entered: Dict[str, object]
    polygons: List[Polygon] = field(default_factory=list)
    circles: List[Circle] = field(default_factory=list)
    # restart fields (u, v, p, Temper: float64[Ny, Nx]; vol: uint32[Ny, Nx]); None -> setup path
    restart: Optional[Dict[str, np.ndarray]] = None
    it_begin: float = 0.0
    description: str = ""

    @property
    def Nx(self) -> int:
        return int(self.entered["Nx"])

    @property
    def Ny(self) -> int:
        return int(self.entered["Ny"])

    def write(self, directory: str) -> str:
        os.makedirs(directory, exist_ok=True)
        e = dict(self.entered)
        e.setdefault("ToImport_data_for_polyhedrons_from_file_b", 1 if self.polygons else 0)
        e.setdefault("ToImport_data_for_circles_from_file_b", 1 if self.circles else 0)
        with open(os.path.join(directory, "EnteredData.txt"), "w") as f:
            f.write(format_entered_data(e))
        if self.polygons:
            with open(os.path.join(directory, "solve_polyhedrons_b.txt"), "w") as f:
                f.write(format_polygons(self.polygons))
        if self.circles:
            with open(os.path.join(directory, "solve_circles_b.txt"), "w") as f:
                f.write(format_circles(self.circles))
        if self.restart is not None:
            for name in ("u", "v", "p", "Temper"):
                np.ascontiguousarray(self.restart[name], dtype="<f8").tofile(
                    os.path.join(directory, f"{name}.bin"))
            np.ascontiguousarray(self.restart["vol_inf_fb"], dtype="<u4").tofile(
                os.path.join(directory, "vol_inf_fb.bin"))
            with open(os.path.join(directory, "it_begin.txt"), "w") as f:
                f.write(f"{self.it_begin!r}\n")
        return directory


def read_field(directory: str, name: str, Nx: int, Ny: int) -> np.ndarray:
    """Read one reference dump: raw native-endian array (WriteReadData.h:107-134), or the text
    form with one value per line (WriteReadData.h:139-173) when no .bin exists."""
    dt = "<u4" if name == "vol_inf_fb" else "<f8"
    path = os.path.join(directory, f"{name}.bin")
    if os.path.exists(path):
        a = np.fromfile(path, dtype=dt)
    else:
        a = np.loadtxt(os.path.join(directory, f"{name}.txt"), dtype=np.float64).astype(dt)
    if a.size != Nx * Ny:
        raise ValueError(f"{name}.bin holds {a.size} values, expected {Nx * Ny}")
    return a.reshape(Ny, Nx)


# ---------------------------------------------------------------------------
# geometry helpers
# ---------------------------------------------------------------------------
EPS = 1e-5          # vertex offset from cell faces so no cell centre lies on an edge
FAR = 100000.001    # "infinite" extent of wall polygons


def wall_polygons(y_bottom: float, y_top: float, T_bottom: float = 1.0, T_top: float = 1.0,
                  slip: int = 1, jump: int = 1) -> List[Polygon]:
    """Two slab bodies: everything below y_bottom and above y_top (faces at those y)."""
    bot = Polygon(
        vertices=[(-FAR, -FAR), (FAR, -FAR), (FAR, y_bottom + EPS), (-FAR, y_bottom + EPS)],
        inside1=(100.01, -2000.1), inside2=(150.01, -2000.111), T_body=T_bottom, slip=slip, jump=jump)
    top = Polygon(
        vertices=[(-FAR, y_top - EPS), (FAR, y_top - EPS), (FAR, FAR), (-FAR, FAR)],
        inside1=(100.01, 2000.1), inside2=(150.01, 2000.111), T_body=T_top, slip=slip, jump=jump)
    return [bot, top]


def square_polygon(xc: float, yc: float, side: float, T_body: float = 1.0) -> Polygon:
    a = 0.5 * side - EPS
    verts = [(xc - a, yc - a), (xc + a, yc - a), (xc + a, yc + a), (xc - a, yc + a)]
    return Polygon(vertices=verts, inside1=(xc - 0.3 * a, yc - 0.11 * a),
                   inside2=(xc + 0.21 * a, yc + 0.27 * a), T_body=T_body)


def uniform_mesh_entries(Nx: int, Ny: int, h: float, x0: float, y0: float) -> Dict[str, object]:
    """Uniform mesh (hmin == hmax == h); cell centre i sits at x0 + i*h (SIMPLE_TS_MPI.cpp:2181-2213)."""
    return dict(Nx=Nx, Ny=Ny, x_b=x0, x_e=x0 + (Nx - 1) * h, y_b=y0, y_e=y0 + (Ny - 1) * h,
                kind_of_mesh=3, hxmin=h, hxmax=h, hymin=h, hymax=h,
                xfmin=x0 - 10.0, xfmax=x0 - 20.0, xbmin=x0 + Nx * h + 10.0, xbmax=x0 + Nx * h + 20.0,
                ytmin=y0 + Ny * h + 10.0, ytmax=y0 + Ny * h + 20.0, ybmin=y0 - 10.0, ybmax=y0 - 20.0,
                xmid=0.0, ymid=0.0, N_I_T=0)


def inflow_velocity(mach: float) -> float:
    """Inflow speed in code units for a given Mach number.

    With the Kn-based scaling (TypeOfNonDimensiolization = 3) velocities are
    measured in units of sqrt(2 R T0) and gamma = 5/3 (SIMPLE_TS_MPI.cpp:2054-2064),
    so Ma = u * sqrt(2 / gamma) = u * sqrt(6/5)."""
    return mach / math.sqrt(6.0 / 5.0)


def _common(Nt: int, ht: float, Kn: float, tol: Optional[float], fixed_sweeps: int) -> Dict[str, object]:
    e: Dict[str, object] = dict(
        TypeOfNonDimensiolization=3, Kn=Kn, Nt=Nt, ht=ht, N_I=1,
        MaxError_to_stop_program=0.0, max_time_for_solve=1e6,
        Nt_save_solved_data=Nt, Nt_save_temp_data=Nt, Nt_save_DragCoefficient=10 ** 9,
        ToReadSolvedDataFromFile=1, ToReadSolvedDataFromBinaryFile=1, ToWriteSolvedDataToBinaryFile=1,
        N_SubDomains_x=1, N_SubDomains_y=1, To_Use_Kn_local_in_wall_BC=1,
        Pressure_BC=0, drhodt_durhodx_dvrhody_0_BC_xb=0, drhodt_durhodx_dvrhody_0_BC_xe=0,
        dvdx_0_BC_xb=0, dvdx_0_BC_xe=0, dTdx_0_BC_xe=0, correct_p_BC_xb=0,
    )
    if tol is None:
        e["N_I_p_c"] = fixed_sweeps
        e.update(MaxError_Velocities=1e-8, MaxError_p_c=1e-9, MaxError_T=1e-9)
    else:
        e["N_I_p_c"] = 100000
        e.update(MaxError_Velocities=tol, MaxError_p_c=tol, MaxError_T=tol)
    return e


def channel_case(name: str, nx: int, ny: int, mach: float, Kn: float, ht: float, Nt: int,
                 square_x: float = 2.5, tol: Optional[float] = 1e-8, fixed_sweeps: int = 2,
                 length: float = 10.0) -> Case:
    """Gas flow past a confined square in a 2D microchannel of height 1.

    Columns: cell 0 is the inflow ghost (unsolved, inflow faces u[0], u[1] hold
    the inflow speed: Given_velocity_on_xb, SIMPLE_TS_MPI.cpp:6069-6074), cells
    1..nx are fluid, the last two columns hold the fixed outlet pressure p = 1
    (never solved: Nx_others[1] = Nx-2, SIMPLE_TS_MPI.cpp:6122).  Row 0 and rows
    ny+1, ny+2 are isothermal slip / temperature-jump walls (polygon bodies); the
    reference leaves one row unsolved at the low side and two at the high side
    (Ny_others = [1, Ny-2], SIMPLE_TS_MPI.cpp:6140-6190).  The
    square has side H/4 and centre (square_x, H/2).  Initial state p = T = 1,
    u = v = 0 except the inflow faces, supplied through the restart path.
    """
    h = 1.0 / ny
    Nx, Ny = nx + 3, ny + 3
    x0, y0 = -0.5 * h, -0.5 * h
    e = _common(Nt, ht, Kn, tol, fixed_sweeps)
    e.update(uniform_mesh_entries(Nx, Ny, h, x0, y0))
    u_in = inflow_velocity(mach)
    e.update(Given_velocity_on_xb=1, dudx_0_BC_xe=1, dvdx_0_BC_xe=1, dTdx_0_BC_xe=1,
             u_given_xb=u_in, T_gas_nd=1.0, p_gas_nd=1.0, u_gas_nd=0.0, p_BC_xe=1.0, T_BC_xe=1.0,
             p_BC_xb=1.0, T_BC_xb=1.0)
    polys = wall_polygons(0.0, 1.0) + [square_polygon(square_x, 0.5, 0.25)]
    case = Case(name=name, entered=e, polygons=polys,
                description=f"channel {nx}x{ny}, Ma {mach}, Kn {Kn}, dt {ht}, {Nt} steps")
    case.restart = channel_initial_state(case, u_in)
    return case


def mask_for(case: Case) -> np.ndarray:
    """Body id per cell for the cell-centre tests; only for the simple geometries built here
    (axis-aligned wall slabs and squares, all edges offset from cell centres)."""
    e = case.entered
    Nx, Ny = case.Nx, case.Ny
    h = float(e["hxmax"])
    xv = float(e["x_b"]) + h * np.arange(Nx)
    yv = float(e["y_b"]) + float(e["hymax"]) * np.arange(Ny)
    X, Y = np.meshgrid(xv, yv)
    vol = np.zeros((Ny, Nx), dtype=np.uint32)
    # circles first, then polygons: later bodies overwrite earlier ones (SIMPLE_TS_MPI.cpp:6331-6355)
    for k, C in enumerate(case.circles):
        inside = (X - C.xc) ** 2 + (Y - C.yc) ** 2 <= C.rc ** 2
        vol[inside] = 1 + k
    for k, P in enumerate(case.polygons):
        xs = [v[0] for v in P.vertices]
        ys = [v[1] for v in P.vertices]
        inside = (X >= min(xs)) & (X <= max(xs)) & (Y >= min(ys)) & (Y <= max(ys))
        vol[inside] = 1 + len(case.circles) + k
    return vol


def channel_initial_state(case: Case, u_in: float) -> Dict[str, np.ndarray]:
    Nx, Ny = case.Nx, case.Ny
    vol = mask_for(case)
    fluid = vol == 0
    u = np.zeros((Ny, Nx))
    v = np.zeros((Ny, Nx))
    p = np.ones((Ny, Nx))
    T = np.ones((Ny, Nx))
    # inflow faces 0 and 1 (never solved)
    u[:, 0][fluid[:, 0]] = u_in
    u[:, 1][fluid[:, 0] & fluid[:, 1]] = u_in
    body = ~fluid
    p[body] = 0.0
    for k, P in enumerate(case.polygons):
        T[vol == 1 + len(case.circles) + k] = P.T_body
    return dict(u=u, v=v, p=p, Temper=T, vol_inf_fb=vol)


def rayleigh_benard_case(name: str, nx: int = 512, ny: int = 256, Kn: float = 0.01, ht: float = 1e-3,
                         Nt: int = 20000, seed: int = 20261203, noise: float = 1e-3,
                         tol: Optional[float] = 1e-8, fixed_sweeps: int = 2) -> Case:
    """2:1 periodic box, bottom wall T = 1.5, top T = 0.5, gravity g = 1 (Fr = 1 with the
    Kn scaling gives c_Fr_v = 2/(gamma Fr Ma^2) = 1, SIMPLE_TS_MPI.cpp:2066).  Row 0 and
    rows ny+1, ny+2 are the walls.  Initial T linear in y plus seeded uniform noise."""
    H = 1.0
    h = H / ny
    Nx, Ny = nx, ny + 3
    x0, y0 = 0.5 * h, -0.5 * h
    e = _common(Nt, ht, Kn, tol, fixed_sweeps)
    e.update(uniform_mesh_entries(Nx, Ny, h, x0, y0))
    e.update(Periodic_boundary_conditions_about_OX=1, SolveGravityField=1, Fr=1.0,
             dTdx_0_BC_xe=0, dvdx_0_BC_xe=0, dudx_0_BC_xe=0)
    polys = wall_polygons(0.0, H, T_bottom=1.5, T_top=0.5)
    case = Case(name=name, entered=e, polygons=polys,
                description=f"Rayleigh-Benard {nx}x{ny}, Kn {Kn}, dt {ht}, {Nt} steps, seed {seed}")
    vol = mask_for(case)
    fluid = vol == 0
    rng = np.random.Generator(np.random.PCG64(seed))
    yv = y0 + h * np.arange(Ny)
    T = np.broadcast_to((1.5 - yv / H)[:, None], (Ny, Nx)).copy()
    T += rng.uniform(-noise, noise, size=(Ny, Nx))
    T[~fluid & (yv[:, None] < 0.5)] = 1.5
    T[~fluid & (yv[:, None] > 0.5)] = 0.5
    p = np.ones((Ny, Nx))
    p[~fluid] = 0.0
    case.restart = dict(u=np.zeros((Ny, Nx)), v=np.zeros((Ny, Nx)), p=p, Temper=T, vol_inf_fb=vol)
    return case


def reynolds_from(mach: float, Kn: float, gamma: float = 5.0 / 3.0) -> float:
    """Hard-sphere relation Kn = (16/5) (Ma/Re) sqrt(gamma / (2 pi))."""
    return 16.0 / 5.0 * mach / Kn * math.sqrt(gamma / (2.0 * math.pi))


def batch_cases(n: int = 64, seed: int = 20261204, Nt: int = 2000, nx_range=(200, 800),
                tol: Optional[float] = 1e-8) -> List[Case]:
    """Independent channel cases of uneven size: nx ~ U{200..800}, ny = nx/10,
    Ma ~ U[0.1, 0.5], Kn log-uniform in [1e-3, 1e-2], square centre x ~ U[2H, 4H]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n):
        nx = int(rng.integers(nx_range[0], nx_range[1] + 1))
        ny = max(nx // 10, 4)
        mach = float(rng.uniform(0.1, 0.5))
        Kn = float(10 ** rng.uniform(-3, -2))
        sx = float(rng.uniform(2.0, 4.0))
        ht = 0.04 / ny
        c = channel_case(f"batch{k:02d}", nx, ny, mach, Kn, ht, Nt, square_x=sx, tol=tol,
                         length=nx / ny)
        c.description += f", Re {reynolds_from(mach, Kn):.1f}"
        out.append(c)
    return out


def config_case(which: str, scale: float = 1.0, Nt: Optional[int] = None,
                tol: Optional[float] = 1e-8) -> Case:
    """Named workloads.  ``scale`` < 1 shrinks the mesh (for oracle-sized parity cases)."""
    def s(n):
        return max(int(round(n * scale)), 4)
    if which == "channel_ma0.1":
        return channel_case("channel_ma0.1", s(400), s(40), 0.1, 0.00194, 1e-3,
                            Nt if Nt is not None else 1000, tol=tol)
    if which == "channel_ma2.43":
        return channel_case("channel_ma2.43", s(1200), s(120), 2.43, 0.00283, 2.5e-4,
                            Nt if Nt is not None else 4000, tol=tol)
    if which == "rayleigh_benard":
        # dt 5e-5, so that the 20000 steps cover t = 0 .. 1: the reference solver itself does not
        # get through this box much beyond t = 1 (its sweep count per step grows without bound
        # from about t = 1.1 at dt 2.5e-4, and at dt 1e-3 it ends in NaN at t = 2.2)
        return rayleigh_benard_case("rayleigh_benard", s(512), s(256), ht=5e-5,
                                    Nt=Nt if Nt is not None else 20000, tol=tol)
    if which == "channel_2048":
        return channel_case("channel_2048", s(2048), s(256), 0.5, 0.003, 1.25e-4,
                            Nt if Nt is not None else 1000, tol=tol)
    if which.startswith("channel_2048_ma"):  # the 2048x256 channel at another Mach number
        mach = float(which[len("channel_2048_ma"):])
        return channel_case(which, s(2048), s(256), mach, 0.003, 1.25e-4, Nt if Nt is not None else 1000, tol=tol)
    raise KeyError(which)


def shipped_example(steps: int = 5) -> Case:
    """The example input distributed with the reference: a pressure-driven channel
    (p 3 -> 1, Kn 0.05) between two reservoirs on a 282x63 polynomial mesh.  The
    EnteredData defaults above are its values; the two wall polygons are restated here."""
    e: Dict[str, object] = {name: default for name, _, default in ENTERED_DATA}
    e.update(Nt=steps, Nt_save_solved_data=steps, Nt_save_temp_data=1)
    common = dict(p_body=0.0, T_body=1.0, slip=1, F_slip=1.1466, w_slip=0.0, jump=0, F_jump=2.1904, dTdn0=0.0)
    low = Polygon(vertices=[(-100000.001, -0.99991), (0.000001, -0.99991), (0.000001, 0.00001), (10.00001, 0.00001),
                            (10.00001, -0.99991), (100000.001, -0.99991), (100000.001, -100000.001),
                            (-100000.001, -100000.001)],
                  inside1=(100.01, -2000.1), inside2=(150.01, -2000.111), **common)
    high = Polygon(vertices=[(-100000.001, 100000.001), (1000000.001, 100000.001), (1000000.001, 2.00001),
                             (10.00001, 2.00001), (10.00001, 1.00001), (0.000001, 1.00001), (0.000001, 2.00001),
                             (-100000.001, 2.000001)],
                   inside1=(100.01, 2000.1), inside2=(150.01, 2000.111), **common)
    return Case(name="shipped_example", entered=e, polygons=[low, high],
                description="example input of the reference (282x63, Pressure_BC, Kn 0.05)")
