"""Generate the golden fixtures in this folder from the COMPILED REFERENCE.

Run here, where the reference checkout exists:

    make -C oracle ref            # builds oracle/_ref/ref_driver_tet{4,10}
    python tests/golden/make_golden.py

Every fixture is produced by ``oracle/_ref/ref_driver_*``, a harness compiled against the
unmodified reference headers, on seeded synthetic meshes written in ``.inp`` form and
read back by the reference's own ``Mesh::load_mesh``:

* ``ref_traj_tet4_c4.npz``: Dynamics::solve on a 4^3 x 6 tet4 cube, 10 m/s onto a
  z-wall 10 um below it, 200 steps (contact from step ~10).
* ``ref_small_tet4.npz``: the 10^3 x 6 = 6000-element tet4 cube of the small
  workload, 10 m/s, wall 1 mm below, dt = 0.5 x CFL, 2000 steps, wall stiffness
  E x (min element height) (the reference drivers' 10 E is unstable at this dt).
* ``ref_update_tet10_c2.npz`` / ``ref_update_tet4_c3.npz``: one ``update()`` call with a
  seeded random increment (kernel-level f_int / mass parity).
* ``ref_traj_tet10_c2.npz``: 40 steps of the tet10 solve (before the reference's
  negative corner masses make it diverge).
* ``ref_strain_kat.npz``: total strain energy and volume of Dynamics::debug_strain
  for both deformation cases on a single tet (legs 10), the quadratic single tet and
  a 4^3 cube, tet4 and tet10.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from cppimpact_gb300 import meshgen as mg  # noqa: E402
import oracle_py as op  # noqa: E402

E, NU, RHO = 68.9e9, 0.33, 2700.0


def single_tet(order: int) -> mg.TetMesh:
    """One tetrahedron with legs 10 along the axes."""
    if order == 1:
        x = np.array([[0, 0, 0], [10, 0, 0], [0, 10, 0], [0, 0, 10]], dtype=float)
        c = np.array([[0, 1, 2, 3]], dtype=np.int32)
    else:
        corners = np.array([[10, 0, 0], [0, 10, 0], [0, 0, 0], [0, 0, 10]], dtype=float)
        mids = np.array([0.5 * (corners[a] + corners[b]) for a, b in mg.TET10_EDGES])
        x = np.concatenate([corners, mids])
        c = np.arange(10, dtype=np.int32)[None]
    return mg.TetMesh(x, c, np.array([0], dtype=np.int32), f"single_tet{order}")


def run(args, cwd):
    r = subprocess.run(args, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return r


def solve(mesh, tmp, loc, k, vz, dt, nsteps):
    mg.write_inp(mesh, os.path.join(tmp, "m.inp"))
    t_end = (nsteps - 1) * dt + 0.5 * dt
    r = run([op.ref_driver_path(mesh.npe), "solve", "m.inp", "out", repr(E), repr(RHO), repr(NU),
             repr(float(loc)), repr(float(k)), "1", "0", "0", repr(float(vz)), repr(float(dt)),
             repr(float(t_end))], tmp)
    ns = int(r.stderr.strip().split()[-1])
    out = {s: np.fromfile(os.path.join(tmp, "out." + s)) for s in ("x", "v", "mass", "acc")}
    return out, ns, t_end


def main():
    for npe in (4, 10):
        if not op.have_ref_driver(npe):
            raise SystemExit("build the reference harness first: make -C oracle ref")
    with tempfile.TemporaryDirectory() as tmp:
        # trajectories ---------------------------------------------------
        cases = [("ref_traj_tet4_c4", mg.cube(4, 1), 1e-5, 1e-7, 200, -10.0, 10 * E),
                 ("ref_traj_tet10_c2", mg.cube(2, 2), 1e-5, 1e-7, 40, -10.0, 10 * E)]
        small = mg.cube(10, 1)
        dt_small = mg.cfl_dt(small, E, NU, RHO)
        cases.append(("ref_small_tet4", small, 1e-3, dt_small, 2000, -10.0,
                      mg.wall_stiffness(small, E)))
        for name, mesh, gap, dt, nsteps, vz, k in cases:
            loc = mesh.xloc[:, 2].min() - gap
            out, ns, t_end = solve(mesh, tmp, loc, k, vz, dt, nsteps)
            assert ns == nsteps, (name, ns)
            np.savez_compressed(
                os.path.join(HERE, name + ".npz"), xloc=mesh.xloc, conn=mesh.conn,
                x=out["x"].reshape(-1, 3), v=out["v"].reshape(-1, 3),
                mass=out["mass"].reshape(-1, 3)[:, 0], acc=out["acc"].reshape(-1, 3),
                params=json.dumps(dict(E=E, nu=NU, rho=RHO, wall_location=float(loc),
                                       wall_stiffness=float(k), wall_normal=1,
                                       vel=[0.0, 0.0, vz], dt=float(dt), t_end=float(t_end),
                                       nsteps=ns)))
            print(name, mesh.num_elements, "elements", ns, "steps")
        # single update --------------------------------------------------
        for name, mesh in (("ref_update_tet10_c2", mg.cube(2, 2)), ("ref_update_tet4_c3", mg.cube(3, 1))):
            mg.write_inp(mesh, os.path.join(tmp, "m.inp"))
            rng = np.random.default_rng(7)
            dof = rng.normal(scale=1e-6, size=mesh.xloc.size)
            dof.tofile(os.path.join(tmp, "dof.f64"))
            loc = mesh.xloc[:, 2].min() + 0.01  # a few bottom layers in contact
            run([op.ref_driver_path(mesh.npe), "update", "m.inp", "dof.f64", "uo", repr(E),
                 repr(RHO), repr(NU), repr(float(loc)), repr(10 * E), "1"], tmp)
            acc = np.fromfile(os.path.join(tmp, "uo.acc")).reshape(-1, 3)
            mass = np.fromfile(os.path.join(tmp, "uo.mass")).reshape(-1, 3)[:, 0]
            np.savez_compressed(os.path.join(HERE, name + ".npz"), xloc=mesh.xloc, conn=mesh.conn,
                                dof=dof.reshape(-1, 3), acc=acc, mass=mass,
                                params=json.dumps(dict(E=E, nu=NU, rho=RHO, wall_location=float(loc),
                                                       wall_stiffness=10 * E, wall_normal=1)))
            print(name)
        # strain-energy known answers -----------------------------------
        rows = []
        for mesh in (single_tet(1), single_tet(2), mg.cube(4, 1), mg.cube(4, 2)):
            mg.write_inp(mesh, os.path.join(tmp, "m.inp"))
            for case in (0, 1):
                r = run([op.ref_driver_path(mesh.npe), "strain", "m.inp", str(case), repr(E),
                         repr(NU), "0.01"], tmp)
                vals = dict(line.split() for line in r.stdout.strip().splitlines())
                rows.append((mesh.name, mesh.npe, case, float(vals["energy"]), float(vals["volume"])))
                print(rows[-1])
        np.savez_compressed(os.path.join(HERE, "ref_strain_kat.npz"),
                            rows=json.dumps(rows), E=E, nu=NU, alpha=0.01)


if __name__ == "__main__":
    main()
