"""Batched solves: every instance of a batch is bitwise its unbatched solve."""
import numpy as np
import pytest

from cppimpact_gb300 import sweep

pytestmark = pytest.mark.gpu


def _single(cilib, d):
    s = cilib.Solver(d["xloc"], d["conn"], E=d["E"], nu=d["nu"], rho=d["rho"],
                     sigma_y0=d["sigma_y0"], H=d["H"], wall_normal=d["wall_normal"],
                     wall_offset=d["wall_offset"], wall_stiffness=d["wall_stiffness"],
                     mode=cilib.MODE_J2, lumping=cilib.LUMP_HRZ)
    s.initialize(d["vel"])
    s.start(d["dt"])
    n = 0
    t = 0.0
    while t <= d["t_end"]:
        n += 1
        t += d["dt"]
    s.step(n)
    st = s.state()
    s.close()
    return st, n


def test_batch_equals_unbatched(cilib):
    inst = sweep.make_instances(6, t_end=2e-4, n_range=(3, 6))
    assert {d["order"] for d in inst} == {1, 2}
    b = cilib.Batch(inst)
    ms = b.run()
    assert ms > 0
    for i, d in enumerate(inst):
        bs = b.state(i)
        ss, n = _single(cilib, d)
        assert bs["nsteps"] == n
        for k in ("x", "v", "epbar", "contact"):
            assert np.array_equal(bs[k], ss[k]), (i, k)
    # a second run of the same batch repeats itself bit for bit
    x0 = b.state(0)["x"].copy()
    b.run()
    assert np.array_equal(b.state(0)["x"], x0)
    b.close()


def test_batch_against_fp64_oracle(cilib, oracle):
    d = sweep.make_instances(1, t_end=2e-4, n_range=(4, 4), seed=11)[0]
    b = cilib.Batch([d])
    b.run()
    st = b.state(0)
    par = oracle.params(d["E"], d["nu"], d["rho"], d["sigma_y0"], d["H"], mode=oracle.J2,
                        lumping=oracle.LUMP_HRZ, wall_normal=d["wall_normal"],
                        wall_offset=d["wall_offset"], wall_stiffness=d["wall_stiffness"])
    o = oracle.Solver(d["xloc"], d["conn"], par)
    o.initialize(d["vel"], d["dt"])
    o.step(st["nsteps"])
    ref = o.get()
    u, ur = st["x"] - d["xloc"], ref["x"] - d["xloc"]
    assert np.linalg.norm(u - ur) < 1e-3 * np.linalg.norm(ur)
