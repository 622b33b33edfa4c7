"""Batched solves: every instance of a batch is bitwise its unbatched solve."""
import numpy as np
import pytest

from cppimpact_gb300 import sweep

pytestmark = pytest.mark.gpu


def _single(cilib, d, **shape):
    s = cilib.Solver(d["xloc"], d["conn"], E=d["E"], nu=d["nu"], rho=d["rho"],
                     sigma_y0=d["sigma_y0"], H=d["H"], wall_normal=d["wall_normal"],
                     wall_offset=d["wall_offset"], wall_stiffness=d["wall_stiffness"],
                     mode=cilib.MODE_J2, lumping=cilib.LUMP_HRZ, **shape)
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


def test_autotuned_batch(cilib):
    """The autotuner picks a shape from the candidate set for each element type; with
    that shape passed explicitly, the unbatched run reproduces each instance bit for bit."""
    inst = sweep.make_instances(6, t_end=2e-4, n_range=(3, 7), seed=5)
    b = cilib.Batch(inst, autotune_steps=64)
    b.run()
    for npe in (4, 10):
        t = b.tuning(npe)
        assert t["chunk_elements"] in (0, 4096)
        assert t["chunk_nodes"] in (512, 768, 896, 1024)
        assert t["block_threads"] in (64, 128, 256)
        assert t["elem_lanes"] in ((1,) if npe == 4 else (1, 4))
        assert t["trial_ms_per_step"] > 0
    for i, d in enumerate(inst):
        npe = d["conn"].shape[1]
        t = b.tuning(npe)
        ss, n = _single(cilib, d, chunk_elements=t["chunk_elements"], chunk_nodes=t["chunk_nodes"],
                        block_threads=t["block_threads"],
                        elem_lanes=t["elem_lanes"] if npe == 10 else 0)
        bs = b.state(i)
        assert bs["nsteps"] == n
        for k in ("x", "v", "epbar", "contact"):
            assert np.array_equal(bs[k], ss[k]), (i, k)
    b.close()
    # fixed options are not varied
    b = cilib.Batch(inst, autotune_steps=32, block_threads=128)
    assert b.tuning(4)["block_threads"] == 128 and b.tuning(10)["block_threads"] == 128
    b.close()
