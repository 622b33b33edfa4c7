"""Seeded synthetic tetrahedral meshes and the Abaqus/CalculiX ``.inp`` format.

The meshes are the structured workloads of the impact solver:

* ``cube(n, ...)``: an ``L``-sided cube cut into ``n**3`` sub-cubes, each split into
  six Kuhn tetrahedra (all sub-cubes share the same main diagonal, so the split is
  conforming).  Interior vertices are jittered uniformly by ``+-jitter*h``.
  Linear (tet4) or quadratic (tet10, midside nodes at the straight edge midpoints).
  The tet10 node count is ``(2n+1)**3``.
* ``shell(...)``: a cylinder along ``x`` (mid-surface radius ``R``, length ``L``,
  thickness ``t``) built from ``n_theta x n_axial x 1`` hexahedral cells split the
  same way, periodic in the circumferential direction.  Vertex radii are jittered by
  ``+-radial_jitter*t``.

Node ordering follows the reference's element conventions:

* tet4 corners ``(0,1,2,3)`` with a positive signed volume (``include/tetrahedral.h:521-531``);
* tet10 corners ``0..3`` then the edge nodes ``4:(0,1) 5:(1,2) 6:(2,0) 7:(0,3) 8:(1,3)
  9:(2,3)``, the CalculiX C3D10 order that ``TetrahedralBasisQuadratic::eval_basis``
  (``include/tetrahedral.h:182-197``) is written for.

The ``.inp`` writer emits the subset that ``Mesh::load_mesh`` (``include/mesh.h:57-267``)
parses: ``*Node`` lines ``id, x, y, z``; one element per ``*Element`` line; comma lists
under ``*Nset, Nset=<name>``; 1-based ids.
"""
from __future__ import annotations

import dataclasses
import itertools
import os

import numpy as np

DEFAULT_SEED = 20261203

# tet10 edge table: local edge node k (4..9) sits between these corners
TET10_EDGES = np.array([[0, 1], [1, 2], [2, 0], [0, 3], [1, 3], [2, 3]], dtype=np.int64)


@dataclasses.dataclass
class TetMesh:
    xloc: np.ndarray            # (num_nodes, 3) float64
    conn: np.ndarray            # (num_elements, npe) int32, 0-based
    slave: np.ndarray           # int32 node ids of the impacting face (0-based)
    name: str = "mesh"

    @property
    def num_nodes(self) -> int:
        return int(self.xloc.shape[0])

    @property
    def num_elements(self) -> int:
        return int(self.conn.shape[0])

    @property
    def npe(self) -> int:
        return int(self.conn.shape[1])

    def signed_volumes(self) -> np.ndarray:
        c = self.conn[:, :4]
        a, b, cc, d = (self.xloc[c[:, i]] for i in range(4))
        return np.einsum("ij,ij->i", b - a, np.cross(cc - a, d - a)) / 6.0


def _kuhn_corner_tets() -> np.ndarray:
    """The six Kuhn tetrahedra of a unit cell as (6, 4, 3) integer corner offsets."""
    tets = []
    for perm in itertools.permutations(range(3)):
        p = np.zeros(3, dtype=np.int64)
        path = [p.copy()]
        for axis in perm:
            p[axis] += 1
            path.append(p.copy())
        tets.append(path)
    return np.array(tets, dtype=np.int64)


def _orient(xyz: np.ndarray, conn4: np.ndarray) -> np.ndarray:
    """Swap corners 1 and 2 of elements with a negative signed volume."""
    a, b, c, d = (xyz[conn4[:, i]] for i in range(4))
    vol = np.einsum("ij,ij->i", b - a, np.cross(c - a, d - a))
    neg = vol < 0
    conn4 = conn4.copy()
    conn4[neg, 1], conn4[neg, 2] = conn4[neg, 2].copy(), conn4[neg, 1].copy()
    return conn4


def _add_midside_nodes(xyz: np.ndarray, conn4: np.ndarray):
    """Append one node at the midpoint of every unique edge; return (xyz10, conn10)."""
    nv = xyz.shape[0]
    ends = conn4[:, TET10_EDGES]                       # (E, 6, 2)
    lo = np.minimum(ends[..., 0], ends[..., 1])
    hi = np.maximum(ends[..., 0], ends[..., 1])
    key = lo.astype(np.int64) * nv + hi
    uniq, inv = np.unique(key.ravel(), return_inverse=True)
    ea, eb = uniq // nv, uniq % nv
    mid = 0.5 * (xyz[ea] + xyz[eb])
    conn10 = np.concatenate([conn4, nv + inv.reshape(-1, 6)], axis=1)
    return np.concatenate([xyz, mid], axis=0), conn10


def cube(n: int = 10, order: int = 1, L: float = 0.25, jitter: float = 0.10,
         seed: int = DEFAULT_SEED, origin=(0.0, 0.0, 0.0)) -> TetMesh:
    """``n**3`` sub-cubes x 6 Kuhn tets of an ``L`` cube; ``order`` 1 = tet4, 2 = tet10."""
    rng = np.random.default_rng(seed)
    h = L / n
    g = np.arange(n + 1)
    I, J, K = np.meshgrid(g, g, g, indexing="ij")
    ijk = np.stack([I.ravel(), J.ravel(), K.ravel()], axis=1)
    xyz = ijk.astype(np.float64) * h
    interior = np.all((ijk > 0) & (ijk < n), axis=1)
    xyz[interior] += rng.uniform(-jitter * h, jitter * h, size=(int(interior.sum()), 3))
    xyz += np.asarray(origin, dtype=np.float64)

    def vid(i, j, k):
        return (i * (n + 1) + j) * (n + 1) + k

    cells = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"),
                     axis=-1).reshape(-1, 3)
    kt = _kuhn_corner_tets()                            # (6, 4, 3)
    corners = cells[:, None, None, :] + kt[None]        # (C, 6, 4, 3)
    conn4 = vid(corners[..., 0], corners[..., 1], corners[..., 2]).reshape(-1, 4)
    conn4 = _orient(xyz, conn4)
    if order == 2:
        xyz, conn = _add_midside_nodes(xyz, conn4)
    else:
        conn = conn4
    zmin = xyz[:, 2].min()
    slave = np.nonzero(np.abs(xyz[:, 2] - zmin) < 1e-12 + 0.2 * h)[0].astype(np.int32)
    name = f"cube{n}_{'tet10' if order == 2 else 'tet4'}"
    return TetMesh(xyz, conn.astype(np.int32), slave, name)


def shell(n_theta: int = 720, n_axial: int = 140, R: float = 1.0, L: float = 4.0,
          t: float = 0.004, radial_jitter: float = 0.05, order: int = 2,
          seed: int = DEFAULT_SEED) -> TetMesh:
    """Thin cylinder along x, ``n_theta x n_axial x 1`` cells x 6 Kuhn tets, periodic in theta."""
    rng = np.random.default_rng(seed)
    it = np.arange(n_theta)
    ja = np.arange(n_axial + 1)
    kr = np.arange(2)
    I, J, K = np.meshgrid(it, ja, kr, indexing="ij")
    theta = 2.0 * np.pi * I.ravel() / n_theta
    x = L * J.ravel() / n_axial
    r = R + (K.ravel() - 0.5) * t
    r = r + rng.uniform(-radial_jitter * t, radial_jitter * t, size=r.shape)
    xyz = np.stack([x, r * np.cos(theta), r * np.sin(theta)], axis=1)

    def vid(i, j, k):
        return ((i % n_theta) * (n_axial + 1) + j) * 2 + k

    cells = np.stack(np.meshgrid(np.arange(n_theta), np.arange(n_axial), np.arange(1),
                                 indexing="ij"), axis=-1).reshape(-1, 3)
    kt = _kuhn_corner_tets()
    corners = cells[:, None, None, :] + kt[None]
    conn4 = vid(corners[..., 0], corners[..., 1], corners[..., 2]).reshape(-1, 4)
    conn4 = _orient(xyz, conn4)
    if order == 2:
        xyz, conn = _add_midside_nodes(xyz, conn4)
    else:
        conn = conn4
    zmin = xyz[:, 2].min()
    slave = np.nonzero(xyz[:, 2] < zmin + 0.05 * R)[0].astype(np.int32)
    return TetMesh(xyz, conn.astype(np.int32), slave,
                   f"shell{n_theta}x{n_axial}_{'tet10' if order == 2 else 'tet4'}")


# ---------------------------------------------------------------------------
# Impact set-up shared by tests, benchmarks and the oracle harness
# ---------------------------------------------------------------------------

AL_J2 = dict(E=68.9e9, nu=0.33, rho=2700.0, sigma_y0=276e6, H=0.689e9)


def dilatational_speed(E: float, nu: float, rho: float) -> float:
    return float(np.sqrt(E * (1 - nu) / (rho * (1 + nu) * (1 - 2 * nu))))


def min_element_height(mesh: TetMesh) -> float:
    """Smallest corner-to-opposite-face distance over the vertex tetrahedra."""
    c = mesh.conn[:, :4]
    p = [mesh.xloc[c[:, i]] for i in range(4)]
    vol6 = np.abs(np.einsum("ij,ij->i", p[1] - p[0], np.cross(p[2] - p[0], p[3] - p[0])))
    hmin = np.inf
    for f in ((1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)):
        a, b, cc = (p[i] for i in f)
        area2 = np.linalg.norm(np.cross(b - a, cc - a), axis=1)
        hmin = min(hmin, float(np.min(vol6 / area2)))
    return hmin


def cfl_dt(mesh: TetMesh, E: float, nu: float, rho: float, fraction: float = 0.5) -> float:
    """``fraction x`` (min element height / dilatational wave speed); tet10 halves the height."""
    h = min_element_height(mesh)
    if mesh.npe == 10:
        h *= 0.5
    return fraction * h / dilatational_speed(E, nu, rho)


def wall_stiffness(mesh: TetMesh, E: float) -> float:
    """Penalty stiffness ``E x (min element height)`` (N/m).

    The reference drivers use ``10 E`` (test.cu:91), which on these meshes at
    ``dt = 0.5 CFL`` puts the wall's penalty frequency above the explicit stability
    limit (omega dt > 2), so trajectories through contact amplify round-off.  Scaling
    the penalty with the element stiffness keeps omega dt below 1.
    """
    return float(E * min_element_height(mesh))


def impact_setup(mesh: TetMesh, speed: float, gap: float, E: float = AL_J2["E"],
                 nu: float = AL_J2["nu"], rho: float = AL_J2["rho"]) -> dict:
    """Impact along -z onto the plane z = min z - gap (normal +z), dt = 0.5 CFL."""
    zmin = float(mesh.xloc[:, 2].min())
    return dict(vel=(0.0, 0.0, -float(speed)), wall_normal=(0.0, 0.0, 1.0),
                wall_offset=zmin - gap, wall_stiffness=wall_stiffness(mesh, E),
                dt=cfl_dt(mesh, E, nu, rho))


# ---------------------------------------------------------------------------
# .inp I/O
# ---------------------------------------------------------------------------

def write_inp(mesh: TetMesh, path: str, sets: dict | None = None) -> None:
    etype = "C3D10" if mesh.npe == 10 else "C3D4"
    sets = {"slave": mesh.slave} if sets is None else sets
    with open(path, "w") as f:
        f.write("**\n*Heading\nsynthetic mesh %s\n**\n*Node\n" % mesh.name)
        ids = np.arange(1, mesh.num_nodes + 1)
        body = np.column_stack([ids, mesh.xloc])
        f.write("\n".join("%d, %.17g, %.17g, %.17g" % tuple(r) for r in body))
        f.write("\n**\n*Element, Type=%s, Elset=Solid\n" % etype)
        eids = np.arange(1, mesh.num_elements + 1)[:, None]
        rows = np.concatenate([eids, mesh.conn.astype(np.int64) + 1], axis=1)
        f.write("\n".join(", ".join(str(v) for v in r) for r in rows))
        f.write("\n")
        for name, nodes in sets.items():
            f.write("**\n*Nset, Nset=%s\n" % name)
            nodes = np.asarray(nodes, dtype=np.int64) + 1
            for k in range(0, len(nodes), 16):
                f.write(", ".join(str(v) for v in nodes[k:k + 16]) + "\n")
        f.write("**\n")


def read_inp(path: str, npe: int | None = None) -> TetMesh:
    """Python mirror of the ``.inp`` subset read by ``Mesh::load_mesh`` (include/mesh.h:57-267).

    Ids are mapped ``id -> id-1`` exactly like the reference (which assumes dense ids).
    Node sets whose name contains ``slave`` (any case) are concatenated in name order,
    like ``collect_slave_nodes`` (include/mesh.h:301-329) iterating a ``std::map``.
    """
    nodes, elems, sets = {}, {}, {}
    section, cur = None, None
    with open(path) as f:
        for raw in f:
            line = raw.strip()
            if not line or line[0] == "*":
                section = None
                if "*Node" in line:
                    section = "node"
                if "*Element" in line:
                    section = "elem"
                if "*Nset" in line:
                    section = "nset"
                    pos = line.find("Nset=")
                    if pos >= 0:
                        cur = line[pos + 5:]
                        sets[cur] = []
                continue
            if section == "node":
                parts = line.split(",")
                nodes[int(parts[0])] = (float(parts[1]), float(parts[2]), float(parts[3]))
            elif section == "elem":
                parts = [p.strip() for p in line.split(",") if p.strip()]
                vals = [int(p) for p in parts]
                elems[vals[0]] = vals[1:]
            elif section == "nset":
                for tok in line.split(","):
                    tok = tok.strip()
                    if tok:
                        sets[cur].append(int(tok))
    nn = len(nodes)
    xyz = np.zeros((nn, 3))
    for k, v in nodes.items():
        xyz[k - 1] = v
    ne = len(elems)
    npe = npe or len(next(iter(elems.values())))
    conn = np.zeros((ne, npe), dtype=np.int32)
    for k, v in elems.items():
        conn[k - 1] = np.asarray(v[:npe]) - 1
    slave = []
    for name in sorted(sets):
        if "slave" in name.lower():
            slave.extend(sets[name])
    return TetMesh(xyz, conn, np.asarray(slave, dtype=np.int32) - 1,
                   os.path.basename(path))
