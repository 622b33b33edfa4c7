"""The C++ drop-in headers (include/cppimpact/) keep the reference's class names and
signatures: the reference's own drivers compile unchanged against them and link to
libcppimpact_gb300.so.  A driver written in the reference's style runs on the GPU
(marked gpu)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from cppimpact_gb300 import meshgen as mg

# the reference checkout: $CPPIMPACT_REF_ROOT, else a "reference" directory beside the repo
REF = os.environ.get("CPPIMPACT_REF_ROOT") or os.path.join(os.path.dirname(ROOT), "reference")
INC = os.path.join(ROOT, "include", "cppimpact")
LIBDIR = os.path.join(ROOT, "cppimpact_gb300")
STUB = os.path.join(ROOT, "oracle", "stub")


def _compile(src_text, tmp, name, defines=()):
    """Compile a driver that includes "include/<header>.h" with include/ -> drop-in headers."""
    work = tmp / name
    work.mkdir()
    os.symlink(INC, work / "include")
    (work / "driver.cpp").write_text(src_text)
    exe = work / "driver"
    cmd = ["g++", "-std=c++17", "-O1", *[f"-D{d}" for d in defines], f"-I{STUB}", f"-I{work}",
           str(work / "driver.cpp"), f"-L{LIBDIR}", "-lcppimpact_gb300",
           f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout not present")
@pytest.mark.parametrize("driver,defines", [("test.cu", ()), ("FEA_debug.cu", ("USE_LINEAR_BASIS",)),
                                            ("FEA_debug.cu", ("USE_QUADRATIC_BASIS",))])
def test_reference_drivers_compile_unchanged(cilib, tmp_path, driver, defines):
    src = open(os.path.join(REF, driver)).read()
    _compile(src, tmp_path, driver.replace(".", "_") + "_".join(defines), defines)


DRIVER = r'''
#include <cstdio>
#include "include/analysis.h"
#include "include/elastoplastic.h"
#include "include/wall.h"
#include "include/dynamics.h"
int main(int argc, char** argv) {
  Mesh<T, Basis::nodes_per_element> mesh;
  if (mesh.load_mesh(argv[1]) != 0) return 1;
  Elastoplastic<T, 3> material(68.9e9, 2700, 0.33, 0.0, 0.689e9, 276e6, "AL6061");
  Wall<T, 2, Basis> w("Wall", atof(argv[2]), atof(argv[3]), mesh.slave_nodes, mesh.num_slave_nodes, 1);
  Dynamics<T, Basis, Analysis, Quadrature> dyna(&mesh, &material, &w);
  dyna.output_dir = argv[5];
  T pos[] = {0, 0, 0}, vel[] = {0, 0, -10};
  dyna.initialize(pos, vel);
  const double dt = atof(argv[4]);
  dyna.solve(dt, 199 * dt + 0.5 * dt, 100);
  FILE* f = fopen(argv[6], "wb");
  fwrite(dyna.global_xloc, sizeof(double), dyna.ndof, f);
  fwrite(dyna.vel, sizeof(double), dyna.ndof, f);
  fclose(f);
  dyna.debug_strain(0.01, 0);
  printf("W %.17g V %.17g\n", dyna.last_strain_energy, dyna.last_volume);
  return 0;
}
'''


@pytest.mark.gpu
def test_reference_style_driver_runs_on_gpu(cilib, oracle, tmp_path):
    """A test.cu-style driver through the drop-in headers: 200 steps of the reference's
    force law, VTK exports every 100 steps, matched against the restated reference."""
    m = mg.cube(4, 1)
    inp = tmp_path / "m.inp"
    mg.write_inp(m, str(inp))
    exe = _compile(DRIVER, tmp_path, "drv")
    loc = float(m.xloc[:, 2].min()) - 1e-5
    k, dt = 6.89e11, 1e-7
    out = tmp_path / "out"
    out.mkdir()
    state = tmp_path / "state.f64"
    r = subprocess.run([str(exe), str(inp), repr(loc), repr(k), repr(dt), str(out), str(state)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    xv = np.fromfile(state).reshape(2, -1, 3)
    ref = oracle.ref_solve(m.xloc, m.conn, oracle.ref_params(68.9e9, 0.33, 2700.0, loc, k, 1),
                           (0, 0, -10), dt, 199 * dt + 0.5 * dt)
    u_ref = ref["x"].reshape(-1, 3) - m.xloc
    assert np.linalg.norm(xv[0] - m.xloc - u_ref) < 1e-3 * np.linalg.norm(u_ref)
    assert sorted(os.listdir(out)) == ["simulation_0.vtk", "simulation_100.vtk"]
    W = float(r.stdout.split("W ")[1].split()[0])
    assert W == pytest.approx(84161.61854712779, rel=1e-5)


GEMV = r"""
#include <cstdio>
#include "include/cppimpact_blas.h"
int main() {
  const double a[6] = {1, 2, 3, 4, 5, 6}, x3[3] = {1, -1, 2}, x2[2] = {0.5, 3};
  double y[3] = {1, 2, 0};
  cppimpact_gemv<double, MatOp::NoTrans>(2, 3, 2.0, a, x3, 0.5, y);
  double z[3] = {1, 2, 3};
  cppimpact_gemv<double, MatOp::Trans>(2, 3, -1.0, a, x2, 0.25, z);
  printf("%.17g %.17g %.17g %.17g %.17g\n", y[0], y[1], z[0], z[1], z[2]);
  return 0;
}
"""


def _run_gemv(tmp, name, include_dir):
    work = tmp / name
    work.mkdir()
    os.symlink(include_dir, work / "include")
    (work / "g.cpp").write_text(GEMV)
    exe = work / "g"
    r = subprocess.run(["g++", "-std=c++17", "-O0", f"-I{work}",
                        str(work / "g.cpp"), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return [float(t) for t in subprocess.run([str(exe)], capture_output=True, text=True,
                                              check=True).stdout.split()]


def test_gemv_keeps_reference_semantics(tmp_path):
    """cppimpact_gemv adds beta to y and accumulates alpha op(A) x into y
    (include/cppimpact_blas.h:9-29), which differs from BLAS's beta*y unless beta = 0."""
    got = _run_gemv(tmp_path, "dropin", INC)
    # y_i + beta + alpha (A x)_i ; z_i + beta + alpha (A^T x)_i
    assert got == [1 + 0.5 + 2 * (1 - 2 + 6), 2 + 0.5 + 2 * (4 - 5 + 12),
                   1 + 0.25 - (0.5 + 12), 2 + 0.25 - (1 + 15), 3 + 0.25 - (1.5 + 18)]
    if os.path.isfile(os.path.join(REF, "include", "cppimpact_blas.h")):
        assert got == _run_gemv(tmp_path, "ref", os.path.join(REF, "include"))


DRIVER_J2 = r'''
#include <cstdio>
#include "include/analysis.h"
#include "include/elastoplastic.h"
#include "include/wall.h"
#include "include/dynamics.h"
int main(int argc, char** argv) {
  Mesh<T, Basis::nodes_per_element> mesh;
  if (mesh.load_mesh(argv[1]) != 0) return 1;
  // a low yield stress so the impact yields: the drop-in's J2 law reads Y0 and H
  Elastoplastic<T, 3> material(68.9e9, 2700, 0.33, 0.0, 0.689e9, 60e6, "AL-soft");
  Wall<T, 2, Basis> w("Wall", atof(argv[2]), atof(argv[3]), mesh.slave_nodes, mesh.num_slave_nodes, 1);
  Dynamics<T, Basis, Analysis, Quadrature> dyna(&mesh, &material, &w);
  dyna.force_law = CI_MODE_J2;
  dyna.output_dir = argv[5];
  T pos[] = {0, 0, 0}, vel[] = {0, 0, -20};
  dyna.initialize(pos, vel);
  const double dt = atof(argv[4]);
  dyna.solve(dt, 299 * dt + 0.5 * dt, 150);
  FILE* f = fopen(argv[6], "wb");
  fwrite(dyna.global_xloc, sizeof(double), dyna.ndof, f);
  fwrite(dyna.vel, sizeof(double), dyna.ndof, f);
  fwrite(dyna.global_strains, sizeof(double), 2 * dyna.ndof, f);
  fwrite(dyna.global_stress, sizeof(double), 2 * dyna.ndof, f);
  fclose(f);
  return 0;
}
'''


@pytest.mark.gpu
def test_reference_style_driver_j2_on_gpu(cilib, oracle, tmp_path):
    """The drop-in Dynamics with force_law = CI_MODE_J2: 300 steps of a 20 m/s impact
    that yields, against the FP64 run of the same formulation; its global_strains /
    global_stress hold the reference's nodal fields (include/dynamics_kernels.h:117-147)
    of the end state; VTK files at the reference's export steps carry them."""
    m = mg.cube(4, 1)
    inp = tmp_path / "m.inp"
    mg.write_inp(m, str(inp))
    exe = _compile(DRIVER_J2, tmp_path, "drvj2")
    loc = float(m.xloc[:, 2].min()) - 1e-5
    setup = mg.impact_setup(m, 20.0, 1e-5)
    k, dt = setup["wall_stiffness"], setup["dt"]
    out = tmp_path / "out"
    out.mkdir()
    state = tmp_path / "state.f64"
    r = subprocess.run([str(exe), str(inp), repr(loc), repr(k), repr(dt), str(out), str(state)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(state)
    n3 = m.xloc.size
    x, v = raw[:n3].reshape(-1, 3), raw[n3:2 * n3].reshape(-1, 3)
    eps, sig = raw[2 * n3:4 * n3].reshape(-1, 6), raw[4 * n3:].reshape(-1, 6)
    par = oracle.params(68.9e9, 0.33, 2700.0, 60e6, 0.689e9, mode=oracle.J2,
                        lumping=oracle.LUMP_HRZ, wall_normal=(0, 0, 1), wall_offset=loc,
                        wall_stiffness=k)
    o = oracle.Solver(m.xloc, m.conn, par)
    o.initialize((0, 0, -20), dt)
    o.step(300)
    ref = o.get()
    assert ref["epbar"].max() > 0
    u_ref = ref["x"] - m.xloc
    assert np.linalg.norm(x - m.xloc - u_ref) < 1e-3 * np.linalg.norm(u_ref)
    assert np.linalg.norm(v - ref["v"]) < 1e-3 * np.linalg.norm(ref["v"])
    rp = oracle.ref_params(68.9e9, 0.33, 2700.0, loc, k, 1)
    eps_ref, sig_ref = oracle.ref_nodal_fields(m.xloc, x, m.conn, rp)
    assert np.linalg.norm(eps - eps_ref) < 1e-5 * np.linalg.norm(eps_ref)
    assert np.linalg.norm(sig - sig_ref) < 1e-5 * np.linalg.norm(sig_ref)
    assert sorted(os.listdir(out)) == ["simulation_0.vtk", "simulation_150.vtk"]
    text = (out / "simulation_150.vtk").read_text()
    names = [ln.split()[1] for ln in text.splitlines() if ln.startswith("VECTORS")]
    assert names == ["velocity", "strain1", "strain2", "stress1", "stress2", "acceleration", "mass"]
