"""CPU-side checks of the product library: it loads, exports every symbol the public
header declares, and its host preprocessing (curve order, chunks, ownership, colours,
slots) and .inp reader behave.  No kernel is launched here."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from cppimpact_gb300 import meshgen as mg

HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b(ci_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(cilib):
    L = cilib.lib()
    names = declared_symbols()
    assert "ci_create" in names and "ci_step" in names
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    assert set(cilib.EXPORTS) <= names | {"ci_last_error"}
    assert L.ci_abi_version() == 1


def test_default_options(cilib):
    import ctypes as C
    o = cilib.CiOptions()
    cilib.lib().ci_default_options(C.byref(o))
    assert o.mode == cilib.MODE_J2 and o.lumping == cilib.LUMP_HRZ
    assert tuple(o.gravity) == (0.0, 0.0, -9.81)


@pytest.mark.parametrize("mesh", [mg.cube(4, 1), mg.cube(10, 1), mg.cube(3, 2), mg.cube(8, 2),
                                  mg.shell(48, 6, order=2), mg.shell(40, 5, order=1)],
                         ids=lambda m: m.name)
@pytest.mark.parametrize("chunks", [(0, 0), (17, 120), (1000, 64)])
def test_plan_invariants(cilib, mesh, chunks):
    cilib.plan_verify(mesh.xloc, mesh.conn, *chunks)


def test_plan_is_deterministic_and_bijective(cilib):
    m = mg.cube(8, 2)
    a = cilib.plan_stats(m.xloc, m.conn, perms=True)
    b = cilib.plan_stats(m.xloc, m.conn, perms=True)
    assert np.array_equal(a["perm_elems"], b["perm_elems"])
    assert np.array_equal(a["perm_nodes"], b["perm_nodes"])
    assert np.array_equal(np.sort(a["perm_elems"]), np.arange(m.num_elements))
    assert np.array_equal(np.sort(a["perm_nodes"]), np.arange(m.num_nodes))
    assert a["max_colors"] <= 64


@pytest.mark.parametrize("chunk_nodes", [896, 768])
def test_plan_invariants_on_the_shell(cilib, chunk_nodes):
    """The full shell's plans under both automatic chunk budgets (the fused kernel's 896
    local nodes, the task kernel's 768), including the task kernel's dependency lists."""
    s = mg.shell()
    cilib.plan_verify(s.xloc, s.conn, 0, chunk_nodes)


def test_plan_shell_workload_shape(cilib):
    s = mg.shell()
    assert (s.num_elements, s.num_nodes) == (604800, 1213920)
    st = cilib.plan_stats(s.xloc, s.conn)
    assert st["max_local"] <= 896             # default local-node budget per chunk
    assert st["ghosts"] < 0.30 * s.num_nodes
    # each task of the task kernel waits for a handful of neighbouring chunks (its
    # descriptor holds the list: 4 bytes per entry of shared memory, twice)
    assert 2 <= st["max_task_deps"] <= 32


def test_plan_rejects_bad_meshes(cilib):
    m = mg.cube(2, 1)
    bad = m.conn.copy()
    bad[0, 0] = m.num_nodes + 5
    with pytest.raises(cilib.CiError) as e:
        cilib.plan_verify(m.xloc, bad)
    assert e.value.code == -1
    # a node no element references
    x = np.concatenate([m.xloc, [[9.0, 9.0, 9.0]]])
    with pytest.raises(cilib.CiError):
        cilib.plan_verify(x, m.conn)


def test_hilbert_curve_locality(cilib):
    """Consecutive plan elements are spatial neighbours: mean centroid step is a small
    multiple of the cell size."""
    m = mg.cube(12, 1)
    st = cilib.plan_stats(m.xloc, m.conn, perms=True)
    cen = m.xloc[m.conn].mean(axis=1)[st["perm_elems"]]
    step = np.linalg.norm(np.diff(cen, axis=0), axis=1)
    assert step.mean() < 1.5 * (0.25 / 12)


@pytest.mark.parametrize("order", [1, 2])
def test_inp_reader_roundtrip(cilib, tmp_path, order):
    m = mg.cube(3, order)
    p = str(tmp_path / "m.inp")
    mg.write_inp(m, p, sets={"slave": m.slave, "fixed_bottom": np.array([0, 1], np.int32),
                             "other": np.array([2], np.int32)})
    mesh = cilib.Mesh(m.npe)
    assert mesh.load_mesh(p) == 0
    assert mesh.num_nodes == m.num_nodes and mesh.num_elements == m.num_elements
    assert np.array_equal(mesh.xloc.reshape(-1, 3), m.xloc)
    assert np.array_equal(mesh.element_nodes, m.conn)
    assert np.array_equal(mesh.slave_nodes, m.slave)
    assert np.array_equal(mesh.fixed_nodes, [0, 1])
    py = mg.read_inp(p)
    assert np.array_equal(py.xloc, m.xloc) and np.array_equal(py.conn, m.conn)


def test_inp_reader_errors(cilib, tmp_path):
    mesh = cilib.Mesh(4)
    assert mesh.load_mesh(str(tmp_path / "missing.inp")) == 1
    p = tmp_path / "bad.inp"
    p.write_text("*Node\n1, 0, 0, x\n*Element, Type=C3D4\n1, 1, 2, 3, 4\n")
    assert mesh.load_mesh(str(p)) == 1
    p.write_text("*Node\n1, 0, 0, 0\n2, 1, 0, 0\n3, 0, 1, 0\n4, 0, 0, 1\n*Element, Type=C3D4\n1, 1, 2, 3, 9\n")
    assert mesh.load_mesh(str(p)) == 1


REF_INPUT = os.path.join(os.environ.get("CPPIMPACT_REF_ROOT") or os.path.join(os.path.dirname(ROOT), "reference"), "input")


@pytest.mark.skipif(not os.path.isdir(REF_INPUT), reason="reference checkout not present")
@pytest.mark.parametrize("name,npe", [("0.25 cube calculix linear 5758 elem.inp", 4),
                                      ("0.25 cube calculix quad 5758 elem.inp", 10),
                                      ("fuselage 5086 elements.inp", 4),
                                      ("quad tet.inp", 10)])
def test_inp_reader_on_reference_inputs(cilib, name, npe):
    path = os.path.join(REF_INPUT, name)
    mesh = cilib.Mesh(npe)
    assert mesh.load_mesh(path) == 0
    py = mg.read_inp(path, npe)
    assert np.array_equal(mesh.xloc.reshape(-1, 3), py.xloc)
    assert np.array_equal(mesh.element_nodes, py.conn)
    assert np.array_equal(mesh.slave_nodes, py.slave)
    cilib.plan_verify(py.xloc, py.conn)


def test_surrogate_instances_share_mesh_properties():
    """Instances of one mesh get the wall stiffness and dt computed once; the values are
    those of the per-instance setup."""
    from cppimpact_gb300 import meshgen as mg
    from cppimpact_gb300 import surrogate as sg
    from cppimpact_gb300.sweep import tilted_setup
    cfg = sg.Config(n_cube=3, steps=200, every=50)
    m = mg.cube(3, 1)
    params = sg.sample_params(4, np.random.default_rng(5))
    inst = sg._instances(params, cfg, m)
    for d, (v, sy, h, tilt) in zip(inst, params):
        ref = tilted_setup(m, v, tilt)
        for k in ("wall_normal", "wall_offset", "wall_stiffness", "vel", "dt"):
            assert d[k] == ref[k], k
        assert d["t_end"] == (cfg.steps - 0.5) * ref["dt"]
