"""sts_pt_sweeps (the p-T sweep loop on caller-owned device arrays) against the oracle's loop."""
import tempfile

import numpy as np
import pytest

import sts_cases as sc

pytestmark = pytest.mark.gpu


def sweep_inputs(case, steps=3):
    """Consistent sweep inputs taken from a solver after a few steps, as host arrays."""
    import sts
    d = tempfile.mkdtemp()
    case.write(d)
    s = sts.Solver(d, fixed_sweeps=False)
    s.step(steps)
    f = {n: s.field(n) for n in sts.SWEEP_INPUTS}
    p, T = s.field("p"), s.field("T")
    insp = sts.inspect_case(d)
    s.close()
    e = case.entered
    Nx, Ny = insp["Nx"], insp["Ny"]
    periodic = bool(e.get("Periodic_boundary_conditions_about_OX", 0))
    pbc = bool(e.get("Pressure_BC", 0))
    gxb, gxe = bool(e.get("Given_velocity_on_xb", 0)), bool(e.get("Given_velocity_on_xe", 0))
    if periodic:
        o0, o1 = 0, Nx
    elif pbc:
        o0, o1 = 1, Nx - 2
    else:
        o0, o1 = 1, (Nx - 1 if gxe else Nx - 2)
    meta = dict(Nx=Nx, Ny=Ny, periodic=periodic, given_xb=gxb, given_xe=gxe, Nx_o0=o0, Nx_o1=o1,
                ht=float(e["ht"]), gamma1=5.0 / 3.0, cls=insp["cls"], hx=insp["hx"], hy=insp["hy"])
    return meta, f, p, T


def device_fields(meta, f, p, T):
    import torch
    import sts
    keep = {}

    def dev(a, dtype=torch.float64):
        t = torch.as_tensor(np.ascontiguousarray(a)).to(dtype).cuda().contiguous()
        keep[id(t)] = t
        return t

    F = sts.SweepFields()
    F.Nx, F.Ny = meta["Nx"], meta["Ny"]
    F.periodic, F.given_u_xb, F.given_u_xe = int(meta["periodic"]), int(meta["given_xb"]), int(meta["given_xe"])
    F.Nx_o0, F.Nx_o1, F.ht, F.gamma1 = meta["Nx_o0"], meta["Nx_o1"], meta["ht"], meta["gamma1"]
    F.cls = dev(meta["cls"], torch.uint8).data_ptr()
    F.hx, F.hy = dev(meta["hx"]).data_ptr(), dev(meta["hy"]).data_ptr()
    for n in sts.SWEEP_INPUTS:
        setattr(F, n, dev(f[n]).data_ptr())
    pt, Tt = dev(p), dev(T)
    F.p, F.T = pt.data_ptr(), Tt.data_ptr()
    return F, pt, Tt, keep


CASES = {
    "channel": lambda: sc.channel_case("c", 70, 10, 2.43, 0.00283, 2.5e-4, 100),
    "rayleigh_benard": lambda: sc.rayleigh_benard_case("rb", 24, 12, Nt=100),
    "circle": lambda: (lambda c: (setattr(c, "circles", [sc.Circle(xc=4.0, yc=0.5, rc=0.2)]),
                                  setattr(c, "restart", sc.channel_initial_state(c, 0.3)), c)[-1])(
        sc.channel_case("c", 80, 10, 0.4, 0.003, 1e-3, 100, square_x=2.2)),
}


@pytest.mark.parametrize("fixed,max_sweeps", [(True, 3), (True, 4), (False, 50)])
@pytest.mark.parametrize("which", list(CASES))
def test_pt_sweeps_match_oracle(which, fixed, max_sweeps, lib_built, oracle_built):
    import ora
    import sts
    import torch
    meta, f, p, T = sweep_inputs(CASES[which]())
    # start from a perturbed iterate so that several sweeps are needed
    rng = np.random.default_rng(7)
    p0 = p * (1 + 1e-4 * rng.standard_normal(p.shape))
    T0 = T * (1 + 1e-4 * rng.standard_normal(T.shape))
    F, pt, Tt, keep = device_fields(meta, f, p0, T0)
    n, rp, rT = sts.pt_sweeps(F, max_sweeps, fixed, 1e-10, 1e-10)
    torch.cuda.synchronize()
    po, To, no, rpo, rTo = ora.pt_sweeps(meta["Nx"], meta["Ny"], meta["periodic"], meta["given_xb"],
                                         meta["given_xe"], meta["Nx_o0"], meta["Nx_o1"], meta["ht"], meta["gamma1"],
                                         meta["cls"], meta["hx"], meta["hy"], f, p0, T0, max_sweeps, fixed,
                                         1e-10, 1e-10)
    assert n == no and (fixed is False or n == max_sweeps)
    assert (rp, rT) == (rpo, rTo)
    np.testing.assert_array_equal(pt.cpu().numpy().reshape(po.shape), po)
    np.testing.assert_array_equal(Tt.cpu().numpy().reshape(To.shape), To)
