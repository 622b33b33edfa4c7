"""ctypes binding of liboracle.so -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference legs
import this module, and only as the checker or the timed CPU baseline.  See
``oracle/oracle.h`` for what each function restates.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class OrcMesh(C.Structure):
    _fields_ = [("num_nodes", C.c_int), ("num_elements", C.c_int),
                ("nodes_per_element", C.c_int), ("xloc", _dp), ("conn", _ip)]


class OrcRefParams(C.Structure):
    _fields_ = [("E", C.c_double), ("nu", C.c_double), ("rho", C.c_double),
                ("wall_dim", C.c_int), ("wall_location", C.c_double),
                ("wall_stiffness", C.c_double), ("wall_normal", C.c_int),
                ("gravity_dim", C.c_int), ("gravity", C.c_double)]


class OrcParams(C.Structure):
    _fields_ = [("E", C.c_double), ("nu", C.c_double), ("rho", C.c_double),
                ("sigma_y0", C.c_double), ("H", C.c_double), ("mode", C.c_int),
                ("lumping", C.c_int), ("wall_normal", C.c_double * 3),
                ("wall_offset", C.c_double), ("wall_stiffness", C.c_double),
                ("gravity", C.c_double * 3)]


J2, REFCOMPAT = 0, 1
LUMP_ROWSUM, LUMP_HRZ = 0, 1
E_KINETIC, E_INTERNAL, E_PLASTIC, E_CONTACT, E_GRAVITY, E_KINETIC0, E_BALANCE = range(7)


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcMesh), C.POINTER(OrcParams)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_initialize.argtypes = [C.c_void_p, _dp, _dp, C.c_double]
        L.orc_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_get.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, C.POINTER(C.c_ubyte)]
        L.orc_j2_update.argtypes = [C.c_double] * 4 + [_dp, _dp, _dp]
        L.orc_ref_solve.argtypes = [C.POINTER(OrcMesh), C.POINTER(OrcRefParams), _dp, _dp,
                                    C.c_double, C.c_double, C.c_int, _dp, _dp, _dp, _dp, _ip]
        L.orc_ref_update.argtypes = [C.POINTER(OrcMesh), C.POINTER(OrcRefParams), _dp, _dp, _dp,
                                     _dp, _dp, _dp, _dp, C.c_int]
        L.orc_ref_lumped_mass.argtypes = [C.POINTER(OrcMesh), C.c_double, _dp, _dp]
        L.orc_ref_debug_strain.argtypes = [C.POINTER(OrcMesh), C.c_double, C.c_double,
                                           C.c_double, C.c_int, _dp, _dp]
        L.orc_lumped_mass.argtypes = [C.POINTER(OrcMesh), C.POINTER(OrcParams), _dp, _dp]
        L.orc_internal_force.argtypes = [C.POINTER(OrcMesh), C.POINTER(OrcParams), _dp, _dp,
                                         _dp, _dp, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


class _MeshHold:
    """Keeps the numpy arrays behind an OrcMesh alive."""

    def __init__(self, xloc, conn):
        self.x = np.ascontiguousarray(xloc, dtype=np.float64).reshape(-1)
        self.c = np.ascontiguousarray(conn, dtype=np.int32)
        self.s = OrcMesh(self.x.size // 3, self.c.shape[0], self.c.shape[1],
                         self.x.ctypes.data_as(_dp), self.c.ctypes.data_as(_ip))


def params(E, nu, rho, sigma_y0=276e6, H=0.689e9, mode=J2, lumping=LUMP_HRZ,
           wall_normal=(0.0, 0.0, 1.0), wall_offset=-1e30, wall_stiffness=0.0,
           gravity=(0.0, 0.0, -9.81)) -> OrcParams:
    return OrcParams(E, nu, rho, sigma_y0, H, mode, lumping, (C.c_double * 3)(*wall_normal),
                     wall_offset, wall_stiffness, (C.c_double * 3)(*gravity))


def ref_params(E, nu, rho, wall_location, wall_stiffness, wall_normal=1, wall_dim=2,
               gravity=-9.81) -> OrcRefParams:
    return OrcRefParams(E, nu, rho, wall_dim, wall_location, wall_stiffness, wall_normal, 2,
                        gravity)


def ref_solve(xloc, conn, rp: OrcRefParams, vel, dt, time_end, nthreads=1):
    """Restated reference Dynamics::solve; returns dict of x, v, mass, acc, nsteps."""
    h = _MeshHold(xloc, conn)
    n3 = h.x.size
    out = {k: np.zeros(n3) for k in ("x", "v", "mass", "acc")}
    ns = C.c_int(0)
    pos = np.zeros(3)
    vel = np.asarray(vel, dtype=np.float64)
    rc = lib().orc_ref_solve(C.byref(h.s), C.byref(rp), _d(pos), _d(vel), dt, time_end, nthreads,
                             _d(out["x"]), _d(out["v"]), _d(out["mass"]), _d(out["acc"]),
                             C.byref(ns))
    assert rc == 0
    out["nsteps"] = ns.value
    return out


def ref_update(xloc, conn, rp: OrcRefParams, dof, nthreads=1):
    h = _MeshHold(xloc, conn)
    n3 = h.x.size
    acc, mass = np.zeros(n3), np.zeros(n3)
    x = h.x.copy()
    dof = np.ascontiguousarray(dof, dtype=np.float64).reshape(-1)
    rc = lib().orc_ref_update(C.byref(h.s), C.byref(rp), _d(h.x), _d(x), _d(dof), _d(acc),
                              _d(mass), None, None, nthreads)
    assert rc == 0
    return acc, mass


def ref_nodal_fields(xloc0, x, conn, rp: OrcRefParams):
    """The reference's global_strains / global_stress ([N, 6] each, last element wins)
    for the state at positions x of a mesh with reference positions xloc0: one update
    call with a zero increment, so the strain is B(x) (x - xloc0) at xi = 0
    (include/dynamics_kernels.h:117-147)."""
    h = _MeshHold(xloc0, conn)
    n3 = h.x.size
    acc, mass = np.zeros(n3), np.zeros(n3)
    xs = np.ascontiguousarray(x, dtype=np.float64).reshape(-1).copy()
    strains, stress = np.zeros(2 * n3), np.zeros(2 * n3)
    rc = lib().orc_ref_update(C.byref(h.s), C.byref(rp), _d(h.x), _d(xs), _d(np.zeros(n3)),
                              _d(acc), _d(mass), _d(strains), _d(stress), 1)
    assert rc == 0
    return strains.reshape(-1, 6), stress.reshape(-1, 6)


def ref_time_steps(xloc, conn, rp: OrcRefParams, dof, steps, nthreads=1, warmup=0):
    """Wall time (s) of `steps` calls of the reference's per-step update on the whole
    mesh -- element loop with the 5-point K_e, gemv, scatter, the stress/strain output
    the reference computes every step, wall and gravity -- after the lumped mass was
    assembled once (as Dynamics::solve does: the reference's update skips the mass when
    global_mass[0] != 0, include/dynamics_kernels.h:36).  `warmup` untimed calls first."""
    import time
    h = _MeshHold(xloc, conn)
    n3 = h.x.size
    acc, mass = np.zeros(n3), np.zeros(n3)
    strains, stress = np.zeros(2 * n3), np.zeros(2 * n3)
    x = h.x.copy()
    dof = np.ascontiguousarray(dof, dtype=np.float64).reshape(-1)
    assert lib().orc_ref_lumped_mass(C.byref(h.s), rp.rho, _d(h.x), _d(mass)) == 0

    def one():
        assert lib().orc_ref_update(C.byref(h.s), C.byref(rp), _d(h.x), _d(x), _d(dof),
                                    _d(acc), _d(mass), _d(strains), _d(stress), nthreads) == 0
    for _ in range(warmup):
        one()
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    return time.perf_counter() - t0


def ref_debug_strain(xloc, conn, E, nu, alpha, case):
    h = _MeshHold(xloc, conn)
    W, V = C.c_double(0), C.c_double(0)
    assert lib().orc_ref_debug_strain(C.byref(h.s), E, nu, alpha, case, C.byref(W), C.byref(V)) == 0
    return W.value, V.value


def lumped_mass(xloc, conn, p: OrcParams):
    h = _MeshHold(xloc, conn)
    m = np.zeros(h.x.size // 3)
    assert lib().orc_lumped_mass(C.byref(h.s), C.byref(p), _d(h.x), _d(m)) == 0
    return m


def internal_force(xloc, conn, p: OrcParams, x, du, sigma=None, epbar=None):
    """Assembled f_int, updated (sigma, epbar) and [W_int, W_plastic] increments."""
    h = _MeshHold(xloc, conn)
    E, npe = h.c.shape
    nq = 1 if npe == 4 else 4
    f = np.zeros(h.x.size)
    so, eo, w = np.zeros(E * nq * 6), np.zeros(E * nq), np.zeros(2)
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
    du = np.ascontiguousarray(du, dtype=np.float64).reshape(-1)
    si = None if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64).reshape(-1)
    ei = None if epbar is None else np.ascontiguousarray(epbar, dtype=np.float64).reshape(-1)
    assert lib().orc_internal_force(C.byref(h.s), C.byref(p), _d(x), _d(du), _d(si), _d(ei),
                                    _d(f), _d(so), _d(eo), _d(w)) == 0
    return f, so.reshape(E, nq, 6), eo.reshape(E, nq), w


def j2_update(E, nu, sy0, H, deps, sigma, epbar):
    s = np.ascontiguousarray(sigma, dtype=np.float64).copy()
    d = np.ascontiguousarray(deps, dtype=np.float64)
    e = C.c_double(epbar)
    lib().orc_j2_update(E, nu, sy0, H, _d(d), _d(s), C.byref(e))
    return s, e.value


class Solver:
    """The FP64 run of the GB300 solver's formulation."""

    def __init__(self, xloc, conn, p: OrcParams, nthreads: int = 1):
        """nthreads > 1 (0 = all host cores) runs the step's loops in parallel; the
        results are the same bits for any thread count."""
        self._h = _MeshHold(xloc, conn)
        self.p = p
        self.N = self._h.x.size // 3
        self.E, self.npe = self._h.c.shape
        self.nq = 1 if self.npe == 4 else 4
        self._s = lib().orc_create(C.byref(self._h.s), C.byref(p))
        assert self._s
        nthreads = nthreads or os.cpu_count() or 1
        if nthreads > 1:
            assert lib().orc_set_threads(self._s, int(nthreads)) == 0

    def __del__(self):
        if getattr(self, "_s", None):
            lib().orc_destroy(self._s)
            self._s = None

    def initialize(self, vel, dt, pos=(0.0, 0.0, 0.0)):
        pos = np.asarray(pos, dtype=np.float64)
        vel = np.asarray(vel, dtype=np.float64)
        assert lib().orc_initialize(self._s, _d(pos), _d(vel), dt) == 0

    def step(self, n):
        assert lib().orc_step(self._s, int(n)) == 0

    def get(self):
        x, v, m = np.zeros(3 * self.N), np.zeros(3 * self.N), np.zeros(self.N)
        sg, ep = np.zeros(self.E * self.nq * 6), np.zeros(self.E * self.nq)
        en = np.zeros(8)
        ct = np.zeros(self.N, dtype=np.uint8)
        assert lib().orc_get(self._s, _d(x), _d(v), _d(m), _d(sg), _d(ep), _d(en),
                             ct.ctypes.data_as(C.POINTER(C.c_ubyte))) == 0
        return dict(x=x.reshape(-1, 3), v=v.reshape(-1, 3), mass=m,
                    sigma=sg.reshape(self.E, self.nq, 6), epbar=ep.reshape(self.E, self.nq),
                    energy=en, contact=ct)


# ---------------------------------------------------------------------------
# Compiled reference harness (oracle/_ref): present only where the reference
# checkout was available at build time.
# ---------------------------------------------------------------------------

def ref_driver_path(npe: int) -> str:
    return os.path.join(REF_DIR, "ref_driver_tet4" if npe == 4 else "ref_driver_tet10")


def have_ref_driver(npe: int) -> bool:
    return os.access(ref_driver_path(npe), os.X_OK)
