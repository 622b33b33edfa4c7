"""GPU parity: the sm_103a kernels through the C ABI against the FP64 oracle and the
reference fixtures.  Tolerances (FP32 element math, FP64 nodal state):
  * one-shot f_int, masses, strain energies: relative L2 <= 1e-5
  * trajectories: end-state displacement and equivalent plastic strain within 1e-3
    relative L2 of the FP64 run; identical contact-node sets (ever touched)."""
import json

import time

import numpy as np
import pytest

from conftest import golden
from cppimpact_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

E, NU, RHO = 68.9e9, 0.33, 2700.0
SY0, H = 276e6, 0.689e9


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def solver(cilib, m, mode, lumping=None, **kw):
    if lumping is None:
        lumping = cilib.LUMP_ROWSUM if mode == cilib.MODE_REFCOMPAT else cilib.LUMP_HRZ
    return cilib.Solver(m.xloc, m.conn, E=E, nu=NU, rho=RHO, sigma_y0=SY0, H=H, mode=mode,
                        lumping=lumping, **kw)


@pytest.mark.parametrize("order,n", [(1, 4), (2, 3), (1, 10), (2, 8)])
@pytest.mark.parametrize("lump", ["rowsum", "hrz"])
@pytest.mark.parametrize("chunks", [(0, 0), (4096, 896)], ids=["auto", "big"])
def test_lumped_mass(cilib, oracle, order, n, lump, chunks):
    """Big chunks give the mass kernel several elements per thread (a per-thread volume
    sum must not leak into the next element's HRZ masses)."""
    m = mg.cube(n, order)
    lp = cilib.LUMP_HRZ if lump == "hrz" else cilib.LUMP_ROWSUM
    s = solver(cilib, m, cilib.MODE_J2, lumping=lp, chunk_elements=chunks[0], chunk_nodes=chunks[1])
    got = s.lumped_mass()
    ref = oracle.lumped_mass(m.xloc, m.conn, oracle.params(E, NU, RHO, lumping=lp))
    assert rel(got, ref) < 1e-6


def test_mass_matches_reference_fixture(cilib):
    g = golden("ref_update_tet10_c2.npz")
    s = cilib.Solver(g["xloc"], g["conn"], E=E, nu=NU, rho=RHO, mode=cilib.MODE_REFCOMPAT,
                     lumping=cilib.LUMP_ROWSUM)
    got = s.lumped_mass()
    assert rel(got, g["mass"]) < 1e-6
    assert got.min() < 0  # the reference's row-sum corner masses of tet10


@pytest.mark.parametrize("order,n", [(1, 4), (2, 3)])
def test_internal_force_refcompat(cilib, oracle, order, n):
    m = mg.cube(n, order)
    rng = np.random.default_rng(11)
    x = m.xloc + rng.normal(scale=1e-4, size=m.xloc.shape)
    du = rng.normal(scale=1e-6, size=m.xloc.shape)
    s = solver(cilib, m, cilib.MODE_REFCOMPAT)
    f, _, _ = s.internal_force(x, du)
    fr, _, _, _ = oracle.internal_force(m.xloc, m.conn, oracle.params(E, NU, RHO, mode=oracle.REFCOMPAT),
                                        x, du)
    assert rel(f, fr.reshape(-1, 3)) < 1e-5


def test_internal_force_matches_reference_update(cilib):
    """Kernel-level parity with the reference's update() on tet10 (f_int from acc)."""
    g = golden("ref_update_tet10_c2.npz")
    p = json.loads(str(g["params"]))
    s = cilib.Solver(g["xloc"], g["conn"], E=E, nu=NU, rho=RHO, mode=cilib.MODE_REFCOMPAT,
                     lumping=cilib.LUMP_ROWSUM)
    f, _, _ = s.internal_force(g["xloc"], g["dof"])
    x_end = g["xloc"] + g["dof"]
    acc = g["acc"].copy()
    acc[:, 2] += 9.81
    d = x_end[:, 2] - p["wall_location"]
    hit = d < 0
    acc[hit, 2] -= -(1.0 / g["mass"][hit]) * d[hit] * p["wall_stiffness"]
    f_ref = -acc * g["mass"][:, None]
    assert rel(f, f_ref) < 1e-5


@pytest.mark.parametrize("order,n", [(1, 4), (2, 3)])
def test_internal_force_j2_with_stored_stress(cilib, oracle, order, n):
    m = mg.cube(n, order)
    nq = 1 if order == 1 else 4
    rng = np.random.default_rng(5)
    du = rng.normal(scale=4e-5, size=m.xloc.shape)
    sig = rng.normal(scale=1.2e8, size=(m.num_elements, nq, 6)).astype(np.float32)
    ep = rng.uniform(0, 0.01, size=(m.num_elements, nq)).astype(np.float32)
    s = solver(cilib, m, cilib.MODE_J2)
    f, so, eo = s.internal_force(m.xloc, du, sig, ep)
    fr, sr, er, _ = oracle.internal_force(m.xloc, m.conn, oracle.params(E, NU, RHO, SY0, H, mode=oracle.J2),
                                          m.xloc, du, sig.astype(np.float64), ep.astype(np.float64))
    assert rel(f, fr.reshape(-1, 3)) < 1e-5
    assert rel(so, sr) < 1e-5
    assert rel(eo, er) < 1e-5
    assert (er > ep).any()  # some points yielded


def test_strain_energy_known_answers(cilib):
    g = golden("ref_strain_kat.npz")
    rows = json.loads(str(g["rows"]))
    from golden.make_golden import single_tet
    meshes = {"single_tet1": single_tet(1), "single_tet2": single_tet(2),
              "cube4_tet4": mg.cube(4, 1), "cube4_tet10": mg.cube(4, 2)}
    for name, npe, case, W_ref, V_ref in rows:
        m = meshes[name]
        x = m.xloc
        gx = x[:, 0] if case == 0 else 0.5 * x[:, 0] ** 2
        u = np.stack([0.01 * gx, -0.01 * NU * gx, -0.01 * NU * gx], axis=1)
        s = cilib.Solver(m.xloc, m.conn, E=E, nu=NU, rho=RHO, mode=cilib.MODE_REFCOMPAT)
        W, V = s.strain_energy(u)
        assert W == pytest.approx(W_ref, rel=1e-5), (name, case)
        assert V == pytest.approx(V_ref, rel=1e-5), (name, case)


def _run_gpu(cilib, m, setup, mode, nsteps, lumping=None, **kw):
    s = solver(cilib, m, mode, lumping=lumping, wall_normal=setup["wall_normal"],
               wall_offset=setup["wall_offset"], wall_stiffness=setup["wall_stiffness"], **kw)
    s.initialize(setup["vel"])
    s.start(setup["dt"])
    s.step(nsteps)
    return s


def _run_oracle(oracle, m, setup, mode, nsteps, lumping):
    par = oracle.params(E, NU, RHO, SY0, H, mode=mode, lumping=lumping,
                        wall_normal=setup["wall_normal"], wall_offset=setup["wall_offset"],
                        wall_stiffness=setup["wall_stiffness"])
    o = oracle.Solver(m.xloc, m.conn, par)
    o.initialize(setup["vel"], setup["dt"])
    o.step(nsteps)
    return o.get()


def test_refcompat_trajectory_vs_reference_small(cilib):
    """The small workload (6000 tet4, 2000 steps through contact) against the compiled
    reference's own trajectory."""
    g = golden("ref_small_tet4.npz")
    p = json.loads(str(g["params"]))
    m = mg.TetMesh(g["xloc"], g["conn"], np.zeros(0, np.int32))
    setup = dict(vel=p["vel"], dt=p["dt"], wall_normal=(0, 0, 1), wall_offset=p["wall_location"],
                 wall_stiffness=p["wall_stiffness"])
    s = _run_gpu(cilib, m, setup, cilib.MODE_REFCOMPAT, p["nsteps"])
    st = s.state()
    u_ref = g["x"] - g["xloc"]
    assert rel(st["x"] - g["xloc"], u_ref) < 1e-3
    assert rel(st["v"], g["v"]) < 1e-3


def test_refcompat_trajectory_vs_reference_tet4(cilib):
    g = golden("ref_traj_tet4_c4.npz")
    p = json.loads(str(g["params"]))
    m = mg.TetMesh(g["xloc"], g["conn"], np.zeros(0, np.int32))
    setup = dict(vel=p["vel"], dt=p["dt"], wall_normal=(0, 0, 1), wall_offset=p["wall_location"],
                 wall_stiffness=p["wall_stiffness"])
    s = _run_gpu(cilib, m, setup, cilib.MODE_REFCOMPAT, p["nsteps"])
    st = s.state()
    assert rel(st["x"] - g["xloc"], g["x"] - g["xloc"]) < 1e-3


@pytest.mark.parametrize("order,n,steps,speed,chunks,lanes", [(1, 6, 800, 30.0, (0, 0), 0),
                                                            (2, 3, 600, 20.0, (0, 0), 4),
                                                            (2, 3, 600, 20.0, (0, 0), 1),
                                                            (2, 4, 600, 20.0, (4096, 896), 4),
                                                            (2, 4, 600, 20.0, (4096, 896), 1),
                                                            (1, 8, 600, 30.0, (4096, 896), 0)])
def test_j2_trajectory_vs_fp64(cilib, oracle, order, n, steps, speed, chunks, lanes):
    """tet10 with 4 lanes per element (k_step_qp10) and one thread per element
    (k_step_t10, barycentric form)."""
    m = mg.cube(n, order)
    setup = mg.impact_setup(m, speed, 1e-4)
    s = _run_gpu(cilib, m, setup, cilib.MODE_J2, steps, chunk_elements=chunks[0],
                 chunk_nodes=chunks[1], elem_lanes=lanes)
    st = s.state()
    ref = _run_oracle(oracle, m, setup, oracle.J2, steps, oracle.LUMP_HRZ)
    assert ref["epbar"].max() > 0, "the case must yield"
    assert rel(st["x"] - m.xloc, ref["x"] - m.xloc) < 1e-3
    assert rel(st["epbar"], ref["epbar"]) < 1e-3
    ever = (st["contact"] & 2) > 0
    ever_ref = (ref["contact"] & 2) > 0
    assert ever_ref.sum() > 0
    assert np.array_equal(ever, ever_ref)
    en = s.energy()
    assert en["kinetic"] == pytest.approx(ref["energy"][oracle.E_KINETIC], rel=1e-3)
    assert en["internal"] == pytest.approx(ref["energy"][oracle.E_INTERNAL], rel=1e-3)
    assert abs(en["balance"]) < 0.02 * en["kinetic0"]


def test_deterministic_bitwise(cilib):
    m = mg.cube(6, 2)
    setup = mg.impact_setup(m, 20.0, 1e-4)
    a = _run_gpu(cilib, m, setup, cilib.MODE_J2, 300).state()
    b = _run_gpu(cilib, m, setup, cilib.MODE_J2, 300).state()
    for k in ("x", "v", "sigma", "epbar", "contact"):
        assert np.array_equal(a[k], b[k]), k


def test_chunking_does_not_change_physics(cilib):
    """Different chunk sizes change the summation grouping only (FP32 round-off)."""
    m = mg.cube(5, 2)
    setup = mg.impact_setup(m, 20.0, 1e-4)
    a = _run_gpu(cilib, m, setup, cilib.MODE_J2, 200).state()
    b = _run_gpu(cilib, m, setup, cilib.MODE_J2, 200, chunk_elements=37, chunk_nodes=200).state()
    assert rel(a["x"] - m.xloc, b["x"] - m.xloc) < 1e-5
    c = _run_gpu(cilib, m, setup, cilib.MODE_J2, 200, chunk_elements=4096, chunk_nodes=896).state()
    assert rel(a["x"] - m.xloc, c["x"] - m.xloc) < 1e-5


def test_solve_loop_count_matches_reference(cilib):
    g = golden("ref_traj_tet4_c4.npz")
    p = json.loads(str(g["params"]))
    s = cilib.Solver(g["xloc"], g["conn"], E=E, nu=NU, rho=RHO, mode=cilib.MODE_REFCOMPAT,
                     lumping=cilib.LUMP_ROWSUM, wall_normal=(0, 0, 1),
                     wall_offset=p["wall_location"], wall_stiffness=p["wall_stiffness"])
    s.initialize(p["vel"])
    s.solve(p["dt"], p["t_end"])
    assert s.steps_done() == p["nsteps"]
    assert rel(s.state()["x"] - g["xloc"], g["x"] - g["xloc"]) < 1e-3


def test_degenerate_element_reported(cilib):
    m = mg.cube(2, 1)
    conn = m.conn.copy()
    conn[0, [1, 2]] = conn[0, [2, 1]]  # inverted element: det J < 0
    s = cilib.Solver(m.xloc, conn, E=E, nu=NU, rho=RHO)
    with pytest.raises(cilib.CiError) as ei:
        s.lumped_mass()
    assert ei.value.code == -3


def test_nonfinite_state_reported(cilib):
    m = mg.cube(2, 1)
    s = cilib.Solver(m.xloc, m.conn, E=E, nu=NU, rho=RHO)
    s.initialize((0.0, 0.0, float("nan")))
    with pytest.raises(cilib.CiError) as ei:
        s.start(1e-7)
    assert ei.value.code == -4


@pytest.mark.parametrize("order,lanes", [(1, 0), (2, 4), (2, 1)])
def test_fused_step_split_invariance(cilib, order, lanes):
    """The fused path finalises boundary nodes either at the start of the next step or
    in the end-of-call kernel; both use the same rounding, so splitting a run into
    calls of any length (graph-captured or not, odd or even) changes no bit."""
    m = mg.cube(5, order)
    setup = mg.impact_setup(m, 20.0, 1e-4)
    a = _run_gpu(cilib, m, setup, cilib.MODE_J2, 0, graph_steps=8, elem_lanes=lanes)
    a.step(77)
    b = _run_gpu(cilib, m, setup, cilib.MODE_J2, 0, graph_steps=8, elem_lanes=lanes)
    for n in (1, 2, 9, 16, 17, 32):
        b.step(n)
    sa, sb = a.state(), b.state()
    for k in ("x", "v", "sigma", "epbar", "contact"):
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.parametrize("order,lanes", [(1, 0), (2, 4), (2, 1)])
def test_fused_matches_two_kernel_path(cilib, order, lanes):
    m = mg.cube(5, order)
    setup = mg.impact_setup(m, 20.0, 1e-4)
    a = _run_gpu(cilib, m, setup, cilib.MODE_J2, 300, elem_lanes=lanes).state()
    b = _run_gpu(cilib, m, setup, cilib.MODE_J2, 300, step_kernel=1).state()
    assert rel(a["x"] - m.xloc, b["x"] - m.xloc) < 1e-5
    assert rel(a["epbar"], b["epbar"]) < 1e-4
    assert np.array_equal(a["contact"] & 2, b["contact"] & 2)


@pytest.mark.parametrize("order", [1, 2])
def test_state_file_restart_is_bitwise(cilib, tmp_path, order):
    """Save after 90 steps, run 60 more; a fresh solver loading the file and running the
    same 60 steps ends in the same bits (state, stress, plastic strain, contact,
    energies).  A file for another mesh is refused."""
    m = mg.cube(5, order)
    setup = mg.impact_setup(m, 20.0, 1e-4)
    a = _run_gpu(cilib, m, setup, cilib.MODE_J2, 90)
    path = str(tmp_path / "s.bin")
    a.save_state(path)
    a.step(60)
    b = solver(cilib, m, cilib.MODE_J2, wall_normal=setup["wall_normal"],
               wall_offset=setup["wall_offset"], wall_stiffness=setup["wall_stiffness"])
    b.load_state(path)
    b.step(60)
    sa, sb = a.state(), b.state()
    for k in ("x", "v", "mass", "sigma", "epbar", "contact"):
        assert np.array_equal(sa[k], sb[k]), k
    ea, eb = a.energy(), b.energy()
    for k in ("kinetic", "internal", "plastic", "contact", "gravity"):
        assert ea[k] == eb[k], k
    other = mg.cube(4, order)
    c = solver(cilib, other, cilib.MODE_J2)
    with pytest.raises(cilib.CiError) as e:
        c.load_state(path)
    assert e.value.code == -1


def _ref_grads(order):
    """Shape-function gradients in reference coordinates at the Gauss points (tet4: one
    point; tet10: the 4-point rule), the element geometry of include/tetrahedral.h."""
    dL = np.array([[1.0, 0, 0], [0, 1.0, 0], [-1.0, -1.0, -1.0], [0, 0, 1.0]])
    if order == 1:
        return [dL[[2, 0, 1, 3]]]
    a, b = (5 + 3 * np.sqrt(5)) / 20, (5 - np.sqrt(5)) / 20
    edges = [(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)]
    out = []
    for q in range(4):
        L = [a if q == 1 else b, a if q == 2 else b, a if q == 0 else b, a if q == 3 else b]
        G = [(4 * L[c] - 1) * dL[c] for c in range(4)]
        G += [4 * (L[i] * dL[j] + L[j] * dL[i]) for i, j in edges]
        out.append(np.array(G))
    return out


@pytest.mark.parametrize("order,n", [(1, 5), (2, 3)])
def test_deformation_gradient(cilib, order, n):
    """F = I + du/dX at the Gauss points against an FP64 evaluation from the returned
    positions (within 1e-5 relative L2 of F - I); rigid start gives F = I."""
    m = mg.cube(n, order)
    setup = mg.impact_setup(m, 20.0, 1e-4)
    s = solver(cilib, m, cilib.MODE_J2, wall_normal=setup["wall_normal"],
               wall_offset=setup["wall_offset"], wall_stiffness=setup["wall_stiffness"])
    s.initialize(setup["vel"])
    F0 = s.deformation_gradient()
    assert np.abs(F0 - np.eye(3)).max() < 1e-12
    s.start(setup["dt"])
    s.step(400)
    x = s.state(("x",))["x"]
    F = s.deformation_gradient()
    X = m.xloc
    u = x - X
    Fr = np.zeros_like(F)
    for q, G in enumerate(_ref_grads(order)):
        J0 = np.einsum("eia,ij->eaj", X[m.conn], G)
        Gu = np.einsum("eia,ij->eaj", u[m.conn], G)
        Fr[:, q] = np.eye(3) + Gu @ np.linalg.inv(J0)
    assert np.abs(Fr - np.eye(3)).max() > 1e-3, "the case must deform"
    assert rel(F - np.eye(3), Fr - np.eye(3)) < 1e-5


@pytest.mark.parametrize("order,n", [(1, 4), (2, 3)])
def test_nodal_fields_match_reference_output(cilib, oracle, order, n):
    """ci_get_nodal_fields: the reference's global_strains / global_stress for the current
    state (strain B u at xi = 0 from the current positions, elastic D, last element in
    caller order wins per node; include/dynamics_kernels.h:117-147) against the restated
    reference fed the same positions, and the stored acceleration against the change of
    the half-step velocity over one step (v_{n+1/2} - v_{n-1/2} = dt a_n)."""
    m = mg.cube(n, order)
    setup = mg.impact_setup(m, 20.0, 1e-4)
    s = _run_gpu(cilib, m, setup, cilib.MODE_J2, 150)
    v_prev = s.state(("v",))["v"]
    s.step(1)
    st = s.state(("x", "v"))
    fld = s.nodal_fields()
    rp = oracle.ref_params(E, NU, RHO, setup["wall_offset"], setup["wall_stiffness"], 1)
    eps_ref, sig_ref = oracle.ref_nodal_fields(m.xloc, st["x"], m.conn, rp)
    assert np.abs(eps_ref).max() > 1e-5  # the impact strains the cube
    assert rel(fld["strain"], eps_ref) < 1e-5
    assert rel(fld["stress"], sig_ref) < 1e-5
    acc_fd = (st["v"] - v_prev) / setup["dt"]
    assert rel(fld["acc"], acc_fd) < 1e-5


@pytest.mark.parametrize("mesh,mode,speed,calls", [
    ("cube3", "j2", 20.0, (37, 20)), ("cube6", "j2", 30.0, (1, 64, 15)),
    ("cube4", "refcompat", 20.0, (40,)), ("shellseg", "j2", 40.0, (25, 24))])
def test_task_kernel_bitwise_equal_to_fused(cilib, mesh, mode, speed, calls):
    """step_kernel = 2 (the persistent task kernel: node tasks and element tasks claimed
    from a counter, each waiting only for its neighbours' progress) computes the fused
    kernel's arithmetic, so every state array ends with the same bits, over calls of odd
    and even length."""
    m = (mg.shell(n_axial=6, L=4.0 * 6 / 140) if mesh == "shellseg"
         else mg.cube(int(mesh[4:]), 2))
    setup = mg.impact_setup(m, speed, 0.0 if mesh == "shellseg" else 1e-4)
    md = cilib.MODE_J2 if mode == "j2" else cilib.MODE_REFCOMPAT
    out = []
    for sk in (3, 2):
        # HRZ masses in both laws (tet10 row-sum corner masses are negative)
        s = solver(cilib, m, md, lumping=cilib.LUMP_HRZ, wall_normal=setup["wall_normal"],
                   wall_offset=setup["wall_offset"], wall_stiffness=setup["wall_stiffness"],
                   step_kernel=sk)
        s.initialize(setup["vel"])
        s.start(setup["dt"])
        for n in calls:
            s.step(n)
        out.append((s.state(), s.energy()))
        s.close()
    (a, ea), (b, eb) = out
    for k in ("x", "v", "sigma", "epbar", "contact"):
        assert np.array_equal(a[k], b[k]), k
    assert ea["internal"] == eb["internal"] and ea["kinetic"] == eb["kinetic"]


def test_task_kernel_long_launch_on_the_shell(cilib):
    """The full shell (2,067 chunks of at most 768 local nodes, 912 resident CTAs) for
    2,000 steps in one launch of the task kernel -- 8.3 million tasks, each CTA moving
    through thousands of task descriptors -- ends bit for bit where the fused kernel does
    on the same plan (the task kernel's automatic 768-node chunk budget, given to both).
    A task that waited past its time limit would raise here."""
    m = mg.shell()
    setup = mg.impact_setup(m, 5.0, 0.0)
    out = []
    for sk in (3, 2):
        s = solver(cilib, m, cilib.MODE_J2, wall_normal=setup["wall_normal"],
                   wall_offset=setup["wall_offset"], wall_stiffness=setup["wall_stiffness"],
                   step_kernel=sk, chunk_nodes=768)
        assert s.step_kernel() == sk
        s.initialize(setup["vel"])
        s.start(setup["dt"])
        s.step(2000)
        out.append(s.state(("x", "v", "contact")))
        s.close()
    a, b = out
    assert ((a["contact"] & 2) > 0).sum() > 0, "the run must reach the plane"
    for k in ("x", "v", "contact"):
        assert np.array_equal(a[k], b[k]), k


def test_task_kernel_wait_times_out_and_reports(cilib):
    """The task kernel's waits are bounded: with one chunk's progress never published
    (the test hook), the tasks waiting for it give up after 0.2 s, every CTA returns, the
    call reports CI_ERR_CUDA with the time-limit message, and the context stays usable --
    a new solver on the same device then steps to the fused kernel's bits."""
    m = mg.cube(6, 2)
    setup = mg.impact_setup(m, 20.0, 1e-4)

    def make(sk):
        s = solver(cilib, m, cilib.MODE_J2, wall_normal=setup["wall_normal"],
                   wall_offset=setup["wall_offset"], wall_stiffness=setup["wall_stiffness"],
                   step_kernel=sk)
        s.initialize(setup["vel"])
        s.start(setup["dt"])
        return s

    s = make(2)
    s.debug_flow_stall(3, 0.2)
    t0 = time.perf_counter()
    with pytest.raises(cilib.CiError) as e:
        s.step(50)
    assert e.value.code == -2 and "time limit" in str(e.value)
    assert time.perf_counter() - t0 < 30.0
    s.close()
    out = []
    for sk in (2, 3):
        s = make(sk)
        s.step(50)
        out.append(s.state(("x", "v")))
        s.close()
    for k in ("x", "v"):
        assert np.array_equal(out[0][k], out[1][k]), k


def test_task_kernel_rejects_other_element_types(cilib):
    m = mg.cube(3, 1)
    with pytest.raises(cilib.CiError) as e:
        solver(cilib, m, cilib.MODE_J2, step_kernel=2)
    assert e.value.code == -5


def test_step_kernel_automatic_choice(cilib):
    """step_kernel = 0 picks the fused kernel for a mesh of small chunks (the quad cube:
    604 chunks, 0.66 of a round of CTAs) and the task kernel for tet10 meshes whose
    chunks the local-node budget cuts (half the shell: 868 chunks, 0.95 of a round; the
    full shell: 1,736 chunks of the default 896-node budget, planned again with the
    task kernel's 768)."""
    for m, sk in ((mg.cube(4, 2), 3), (mg.cube(18, 2), 3), (mg.shell(n_theta=360), 2),
                  (mg.shell(), 2)):
        s = solver(cilib, m, cilib.MODE_J2)
        assert s.step_kernel() == sk
        s.close()
