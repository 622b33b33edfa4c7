"""The batched parameter sweep: seeded impact instances of uneven size.

Each instance is a cube (edge 0.25 m) of n^3 x 6 Kuhn tets, n ~ U{6..16}, tet4 or tet10
with equal probability, aluminium with yield ~ U[200, 350] MPa and hardening
~ U[0.5, 2] % of E, impacting at ~ U[2, 20] m/s a rigid plane tilted by ~ U[0, 15] deg
(normal rotated about x), 1 mm below the cube, run to 2 ms with its own dt = 0.5 CFL.
"""
from __future__ import annotations

import math

import numpy as np

from . import meshgen as mg

E, NU, RHO = 68.9e9, 0.33, 2700.0


def tilted_setup(mesh: mg.TetMesh, speed: float, tilt_deg: float, gap: float = 1e-3,
                 stiffness: float | None = None, dt: float | None = None) -> dict:
    """Wall tilted by tilt_deg about x, `gap` below the mesh, impact speed along -z;
    stiffness and dt (mesh properties) may be passed in when many instances share a mesh."""
    th = math.radians(tilt_deg)
    n = np.array([0.0, math.sin(th), math.cos(th)])
    d = mesh.xloc @ n
    return dict(wall_normal=tuple(n), wall_offset=float(d.min() - gap),
                wall_stiffness=mg.wall_stiffness(mesh, E) if stiffness is None else stiffness,
                vel=(0.0, 0.0, -float(speed)),
                dt=mg.cfl_dt(mesh, E, NU, RHO) if dt is None else dt)


def make_instances(count: int = 256, seed: int = mg.DEFAULT_SEED, t_end: float = 2e-3,
                   n_range=(6, 16)) -> list[dict]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        order = 2 if rng.random() < 0.5 else 1
        speed = float(rng.uniform(2.0, 20.0))
        sy = float(rng.uniform(200e6, 350e6))
        H = float(rng.uniform(0.005, 0.02)) * E
        tilt = float(rng.uniform(0.0, 15.0))
        m = mg.cube(n, order, seed=seed + i)
        st = tilted_setup(m, speed, tilt)
        out.append(dict(xloc=m.xloc, conn=m.conn, E=E, nu=NU, rho=RHO, sigma_y0=sy, H=H,
                        t_end=t_end, n=n, order=order, speed=speed, tilt=tilt, **st))
    return out
