"""Host-side logic of the GB300 library without a GPU: exports, case set-up, input errors."""
import ctypes
import os
import re
import tempfile

import numpy as np
import pytest

import sts_cases as sc
from conftest import ROOT, golden_case


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^\s*(?:int|void|const char\*)\s+(sts_\w+)\s*\(", txt, re.M))
    return names


def test_library_exports_every_declared_symbol(lib_built):
    import sts
    lib = ctypes.CDLL(sts.LIB_PATH)
    names = declared_symbols()
    assert names, "no declarations found"
    assert names <= set(sts.EXPORTS) | names
    for n in sorted(names):
        assert hasattr(lib, n), n


@pytest.mark.parametrize("name", ["channel_ma0.1_80x8_resid", "rayleigh_benard_32x16_resid",
                                  "channel_circle_120x12_resid", "shipped_example_5steps"])
def test_setup_matches_oracle(name, lib_built, oracle_built):
    """Mesh, obstacle ids and interior/boundary classes equal the oracle's (reference) lists."""
    import ora
    import sts
    case, fixed = golden_case(name)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        a = sts.inspect_case(d)
        o = ora.Oracle(d, fixed_sweeps=fixed)
        assert (a["Nx"], a["Ny"]) == (o.Nx, o.Ny)
        np.testing.assert_array_equal(a["vol"], o.mask())
        np.testing.assert_array_equal(a["cls"], o.classes())
        for k in ("hx", "hy", "x_v", "y_v"):
            np.testing.assert_array_equal(a[k], o.field(k))


def test_periodic_classes_near_the_seam(lib_built, oracle_built):
    import ora
    import sts
    case = sc.rayleigh_benard_case("rb", 16, 8, Nt=2)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        a = sts.inspect_case(d)
        cls = a["cls"]
        # every column of the interior rows is solved for p/T, the seam columns in the boundary class
        assert ((cls[2:-3, :] >> 4) & 3).all()
        assert ((cls[3, 0] >> 4) & 3) == 2 and ((cls[3, 5] >> 4) & 3) == 1
        np.testing.assert_array_equal(cls, ora.Oracle(d).classes())


def _err(fn, *args):
    import sts
    with pytest.raises(sts.StsError) as e:
        fn(*args)
    return e.value


def test_missing_entered_data(lib_built):
    import sts
    with tempfile.TemporaryDirectory() as d:
        e = _err(sts.inspect_case, d)
        assert e.code == sts.STS_ERR_INPUT and "EnteredData" in str(e)


def test_truncated_entered_data(lib_built):
    import sts
    case = sc.channel_case("c", 20, 4, 0.1, 0.002, 1e-3, 2)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        p = os.path.join(d, "EnteredData.txt")
        lines = open(p).read().split("\n")
        open(p, "w").write("\n".join(lines[:60]))
        e = _err(sts.inspect_case, d)
        assert e.code == sts.STS_ERR_INPUT


def test_missing_body_file_and_bad_polygon(lib_built):
    import sts
    case = sc.channel_case("c", 20, 4, 0.1, 0.002, 1e-3, 2)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        os.remove(os.path.join(d, "solve_polyhedrons_b.txt"))
        assert _err(sts.inspect_case, d).code == sts.STS_ERR_INPUT
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        p = os.path.join(d, "solve_polyhedrons_b.txt")
        txt = open(p).read().split("\n")
        open(p, "w").write("\n".join(txt[:20]))  # polygon cut in the middle
        assert _err(sts.inspect_case, d).code == sts.STS_ERR_INPUT


def test_zero_width_mesh(lib_built):
    import sts
    case = sc.channel_case("c", 20, 4, 0.1, 0.002, 1e-3, 2)
    case.entered.update(hxmin=0.0, hxmax=0.0)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        assert _err(sts.inspect_case, d).code == sts.STS_ERR_INPUT


def test_restart_mask_must_match_bodies(lib_built):
    import sts
    case = sc.channel_case("c", 20, 4, 0.1, 0.002, 1e-3, 2)
    case.restart["vol_inf_fb"][3, 5] = 1  # a fluid cell marked as wall in the restart file
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        assert _err(sts.inspect_case, d).code == sts.STS_ERR_INPUT


def test_entered_data_roundtrip():
    e = dict(sc.config_case("channel_ma0.1").entered)
    txt = sc.format_entered_data(e)
    assert len(txt.strip().split("\n")) == 126
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "EnteredData.txt")
        open(p, "w").write(txt)
        back = sc.read_entered_data(p)
        for k, v in e.items():
            assert back[k] == pytest.approx(float(v)), k


def test_missing_library_fails_loudly(lib_built):
    """The Python binding has no fallback: without the compiled library it raises at load."""
    import sts
    saved = sts._lib
    try:
        sts._lib = None
        with pytest.raises(FileNotFoundError, match="no fallback"):
            sts.load(os.path.join(tempfile.gettempdir(), "no_such_dir", "libsts_gb300.so"))
    finally:
        sts._lib = saved
