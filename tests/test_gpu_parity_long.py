"""GPU parity at the configurations' full length, through the C ABI.

* The small cube (10^3 x 6 tet4, 10 m/s, aluminium J2) for all its 2000 steps and the
  quadratic cube (18^3 x 6 = 34,992 tet10, 20 m/s) for all its 5000 steps, each against
  the FP64 run of the same formulation (the oracle, all host threads).  The quadratic
  cube yields on about 63 % of its Gauss points; the small cube stays elastic, as its
  impact speed implies (uniaxial-strain stress rho c v = 166 MPa, von Mises (1 - 2 nu) /
  (1 - nu) of it = 85 MPa, against a 276 MPa yield stress), and the test checks that
  both runs agree on that.
* A segment of the thin shell (the same 720-cell ring, 4 mm wall and element shape; 20
  of the 140 axial cells) at 40 m/s, where the J2 return branch is taken from the
  first hundreds of steps (at the shell's own 5 m/s it is not: the peak von Mises
  stress stays near 0.4 of yield), for 2000 steps.
* The compiled reference's own tet10 trajectory (40 steps of the reference's force
  law, include/dynamics.h:471-511, through contact; tests/golden/ref_traj_tet10_c2.npz)
  on the CUDA RefCompat path.

Tolerances as in test_gpu_parity.py: end-state displacement, velocity change and
equivalent plastic strain within 1e-3 relative L2 of the FP64 run; identical
contact-node sets (nodes that ever touched the wall)."""
import json

import numpy as np
import pytest

from conftest import golden
from cppimpact_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

E, NU, RHO = 68.9e9, 0.33, 2700.0
SY0, H = 276e6, 0.689e9
TOL = 1e-3


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def von_mises(sig):
    s = np.asarray(sig, dtype=np.float64)
    p = s[..., :3].mean(-1, keepdims=True)
    d = s[..., :3] - p
    return np.sqrt(1.5 * ((d ** 2).sum(-1) + 2.0 * (s[..., 3:] ** 2).sum(-1)))


def run_pair(cilib, oracle, m, setup, nsteps):
    """The GPU solver and the FP64 oracle from the same start for nsteps steps (J2,
    HRZ lumping); returns the GPU state and energies and the oracle's state."""
    s = cilib.Solver(m.xloc, m.conn, E=E, nu=NU, rho=RHO, sigma_y0=SY0, H=H,
                     mode=cilib.MODE_J2, lumping=cilib.LUMP_HRZ,
                     wall_normal=setup["wall_normal"], wall_offset=setup["wall_offset"],
                     wall_stiffness=setup["wall_stiffness"])
    s.initialize(setup["vel"])
    s.start(setup["dt"])
    s.step(nsteps)
    st = s.state()
    en = s.energy()
    s.close()
    par = oracle.params(E, NU, RHO, SY0, H, mode=oracle.J2, lumping=oracle.LUMP_HRZ,
                        wall_normal=setup["wall_normal"], wall_offset=setup["wall_offset"],
                        wall_stiffness=setup["wall_stiffness"])
    o = oracle.Solver(m.xloc, m.conn, par, nthreads=0)
    o.initialize(setup["vel"], setup["dt"])
    o.step(nsteps)
    return st, en, o.get()


def check_pair(m, setup, st, ref):
    v0 = np.asarray(setup["vel"], dtype=np.float64)
    assert rel(st["x"] - m.xloc, ref["x"] - m.xloc) < TOL
    assert rel(st["v"] - v0, ref["v"] - v0) < TOL
    ever, ever_ref = (st["contact"] & 2) > 0, (ref["contact"] & 2) > 0
    assert ever_ref.sum() > 0
    assert np.array_equal(ever, ever_ref)


def test_small_cube_full_length_vs_fp64(cilib, oracle):
    """Small cube: 6000 tet4, 10 m/s, 1 mm gap, 2000 steps (its whole run)."""
    m = mg.cube(10, 1)
    setup = mg.impact_setup(m, 10.0, 1e-3)
    st, en, ref = run_pair(cilib, oracle, m, setup, 2000)
    check_pair(m, setup, st, ref)
    # elastic throughout in both runs; the end-state stresses agree
    assert ref["epbar"].max() == 0.0 and st["epbar"].max() == 0.0
    assert von_mises(ref["sigma"]).max() < SY0
    assert rel(st["sigma"], ref["sigma"]) < TOL
    assert abs(en["balance"]) < 0.02 * en["kinetic0"]


def test_quad_cube_full_length_vs_fp64(cilib, oracle):
    """Quadratic cube: 34,992 tet10, 20 m/s, 1 mm gap, 5000 steps (its whole run),
    through contact, rebound and plastic flow."""
    m = mg.cube(18, 2)
    setup = mg.impact_setup(m, 20.0, 1e-3)
    st, en, ref = run_pair(cilib, oracle, m, setup, 5000)
    check_pair(m, setup, st, ref)
    yielded = ref["epbar"] > 0
    assert ref["epbar"].max() > 1e-3 and yielded.mean() > 0.3, "the case must yield widely"
    assert rel(st["epbar"], ref["epbar"]) < TOL
    assert rel(st["sigma"], ref["sigma"]) < TOL
    assert en["plastic"] == pytest.approx(ref["energy"][oracle.E_PLASTIC], rel=TOL)
    assert en["internal"] == pytest.approx(ref["energy"][oracle.E_INTERNAL], rel=TOL)
    assert abs(en["balance"]) < 0.02 * en["kinetic0"]


def test_shell_segment_plastic_vs_fp64(cilib, oracle):
    """Thin-shell segment (720 x 20 x 1 cells x 6 = 86,400 tet10, the full shell's
    element shape), 40 m/s onto the tangent plane, 2000 steps."""
    m = mg.shell(n_axial=20, L=4.0 * 20 / 140)
    setup = mg.impact_setup(m, 40.0, 0.0)
    st, en, ref = run_pair(cilib, oracle, m, setup, 2000)
    check_pair(m, setup, st, ref)
    assert (ref["epbar"] > 0).mean() > 0.01, "the J2 return branch must be exercised"
    assert rel(st["epbar"], ref["epbar"]) < TOL
    assert abs(en["balance"]) < 0.02 * en["kinetic0"]


def test_refcompat_trajectory_vs_reference_tet10(cilib):
    """The compiled reference's tet10 trajectory: 40 steps of its force law (5-point
    K_e at the current positions, row-sum masses -- negative at the corners -- the
    z wall and gravity), reproduced by the CUDA RefCompat path (4-point Gauss rule,
    FP32 element math, FP64 state)."""
    g = golden("ref_traj_tet10_c2.npz")
    p = json.loads(str(g["params"]))
    s = cilib.Solver(g["xloc"], g["conn"], E=E, nu=NU, rho=RHO, mode=cilib.MODE_REFCOMPAT,
                     lumping=cilib.LUMP_ROWSUM, wall_normal=(0, 0, 1),
                     wall_offset=p["wall_location"], wall_stiffness=p["wall_stiffness"])
    s.initialize(p["vel"])
    s.solve(p["dt"], p["t_end"])
    assert s.steps_done() == p["nsteps"]
    st = s.state(("x", "v", "mass"))
    s.close()
    assert rel(st["mass"], g["mass"]) < 1e-6
    assert rel(st["x"] - g["xloc"], g["x"] - g["xloc"]) < TOL
    v0 = np.asarray(p["vel"], dtype=np.float64)
    assert rel(st["v"] - v0, g["v"] - v0) < TOL


def test_shell_segment_tilted_wall_vs_fp64(cilib, oracle):
    """The shell segment against a plane tilted by 5 degrees about the transverse axis
    (normal (sin 5, 0, cos 5)), so one end lands first: 40 m/s, 1,500 steps."""
    m = mg.shell(n_axial=20, L=4.0 * 20 / 140)
    base = mg.impact_setup(m, 40.0, 0.0)
    th = np.radians(5.0)
    n = np.array([np.sin(th), 0.0, np.cos(th)])
    setup = dict(base, wall_normal=tuple(n), wall_offset=float((m.xloc @ n).min() - 1e-4))
    st, en, ref = run_pair(cilib, oracle, m, setup, 1500)
    check_pair(m, setup, st, ref)
    assert ref["epbar"].max() > 0
    assert rel(st["epbar"], ref["epbar"]) < TOL
    assert abs(en["balance"]) < 0.02 * en["kinetic0"]
