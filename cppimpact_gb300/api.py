"""Python host mirror of the reference interface, over the C ABI (ctypes).

Class names and methods follow smdogroup/cppimpact:

* ``Mesh.load_mesh(filename)``                 -- include/mesh.h:57-267
* ``BaseMaterial(type, E, rho, nu)`` /
  ``Elastoplastic(E, rho, nu, beta, H, Y0)``    -- include/basematerial.h, elastoplastic.h
* ``Wall(name, location, stiffness, slave, n, normal, dim=2)`` -- include/wall.h:23-43
* ``Dynamics(mesh, material, wall)`` with ``initialize(pos, vel)``, ``solve(dt,
  time_end, export_interval)``, ``debug_strain(alpha, case)`` and the public arrays
  ``global_xloc``, ``vel``, ``global_mass``          -- include/dynamics.h:43-512

Everything runs in ``libcppimpact_gb300.so`` on the GPU; there is no CPU fallback.
Importing this module raises if the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
# CPPIMPACT_GB300_LIB selects another build of the library (e.g. one configured with
# different compile-time options by ``python -m cppimpact_gb300.build --out``)
LIB_PATH = os.environ.get("CPPIMPACT_GB300_LIB") or os.path.join(_PKG, "libcppimpact_gb300.so")

CI_OK = 0
ERRORS = {-1: "CI_ERR_INVALID", -2: "CI_ERR_CUDA", -3: "CI_ERR_DEGENERATE",
          -4: "CI_ERR_NONFINITE", -5: "CI_ERR_UNSUPPORTED", -6: "CI_ERR_IO",
          -7: "CI_ERR_NOMEM", -8: "CI_ERR_TOO_LARGE"}
MODE_J2, MODE_REFCOMPAT = 0, 1
LUMP_ROWSUM, LUMP_HRZ = 0, 1

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_ubp = C.POINTER(C.c_ubyte)


class CiMesh(C.Structure):
    _fields_ = [("num_nodes", C.c_int), ("num_elements", C.c_int),
                ("nodes_per_element", C.c_int), ("xloc", _dp), ("element_nodes", _ip),
                ("num_slave_nodes", C.c_int), ("slave_nodes", _ip),
                ("num_fixed_nodes", C.c_int), ("fixed_nodes", _ip)]


class CiMaterial(C.Structure):
    _fields_ = [("E", C.c_double), ("nu", C.c_double), ("rho", C.c_double),
                ("sigma_y0", C.c_double), ("H", C.c_double), ("beta", C.c_double)]


class CiWall(C.Structure):
    _fields_ = [("normal", C.c_double * 3), ("offset", C.c_double), ("stiffness", C.c_double)]


class CiOptions(C.Structure):
    _fields_ = [("mode", C.c_int), ("lumping", C.c_int), ("gravity", C.c_double * 3),
                ("device", C.c_int), ("chunk_elements", C.c_int), ("chunk_nodes", C.c_int),
                ("graph_steps", C.c_int), ("step_kernel", C.c_int), ("block_threads", C.c_int),
                ("elem_lanes", C.c_int), ("autotune_steps", C.c_int)]


class CiInstance(C.Structure):
    _fields_ = [("mesh", CiMesh), ("mat", CiMaterial), ("wall", CiWall),
                ("pos", C.c_double * 3), ("vel", C.c_double * 3), ("dt", C.c_double),
                ("t_end", C.c_double)]


class CiEnergy(C.Structure):
    _fields_ = [("kinetic", C.c_double), ("internal", C.c_double), ("plastic", C.c_double),
                ("contact", C.c_double), ("gravity", C.c_double), ("kinetic0", C.c_double),
                ("balance", C.c_double)]


EXPORTS = {
    # name: (restype, argtypes)
    "ci_abi_version": (C.c_int, []),
    "ci_last_error": (C.c_char_p, []),
    "ci_default_options": (None, [C.POINTER(CiOptions)]),
    "ci_create": (C.c_int, [C.POINTER(CiMesh), C.POINTER(CiMaterial), C.POINTER(CiWall),
                            C.POINTER(CiOptions), C.POINTER(C.c_void_p)]),
    "ci_destroy": (C.c_int, [C.c_void_p]),
    "ci_initialize": (C.c_int, [C.c_void_p, _dp, _dp]),
    "ci_solve": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int]),
    "ci_start": (C.c_int, [C.c_void_p, C.c_double]),
    "ci_step": (C.c_int, [C.c_void_p, C.c_int]),
    "ci_steps_done": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "ci_get_state": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _fp, _fp, _ubp]),
    "ci_set_state": (C.c_int, [C.c_void_p, _dp, _dp]),
    "ci_deformation_gradient": (C.c_int, [C.c_void_p, _dp]),
    "ci_get_nodal_fields": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "ci_save_state": (C.c_int, [C.c_void_p, C.c_char_p]),
    "ci_load_state": (C.c_int, [C.c_void_p, C.c_char_p]),
    "ci_get_energy": (C.c_int, [C.c_void_p, C.POINTER(CiEnergy)]),
    "ci_get_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint)]),
    "ci_internal_force": (C.c_int, [C.c_void_p, _dp, _dp, _fp, _fp, _dp, _fp, _fp]),
    "ci_lumped_mass": (C.c_int, [C.c_void_p, _dp, _dp]),
    "ci_strain_energy": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "ci_time_steps": (C.c_int, [C.c_void_p, C.c_int, _fp]),
    "ci_time_kernels": (C.c_int, [C.c_void_p, C.c_int, _fp]),
    "ci_launches_per_step": (C.c_int, [C.c_void_p]),
    "ci_step_kernel": (C.c_int, [C.c_void_p]),
    "ci_debug_flow_stall": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "ci_mesh_load_inp": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(CiMesh)]),
    "ci_mesh_free": (None, [C.POINTER(CiMesh)]),
    "ci_plan_stats": (C.c_int, [C.POINTER(CiMesh), C.c_int, C.c_int, C.POINTER(C.c_longlong),
                                _ip, _ip]),
    "ci_plan_verify": (C.c_int, [C.POINTER(CiMesh), C.c_int, C.c_int]),
    "ci_batch_create": (C.c_int, [C.POINTER(CiInstance), C.c_int, C.POINTER(CiOptions),
                                  C.POINTER(C.c_void_p)]),
    "ci_batch_run": (C.c_int, [C.c_void_p, _fp]),
    "ci_batch_get_state": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _fp, _ubp,
                                     C.POINTER(C.c_longlong)]),
    "ci_batch_destroy": (C.c_int, [C.c_void_p]),
    "ci_batch_tuning": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, _ip, _ip, _fp]),
    "ci_batch_run_snapshots": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, _fp]),
    "ci_batch_run_peaks": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _fp, _fp, _fp]),
    "ci_batch_node_order": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip]),
    "ci_mlp_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(C.c_void_p)]),
    "ci_mlp_destroy": (C.c_int, [C.c_void_p]),
    "ci_mlp_num_params": (C.c_longlong, [C.c_void_p]),
    "ci_mlp_set_params": (C.c_int, [C.c_void_p, _fp]),
    "ci_mlp_get_params": (C.c_int, [C.c_void_p, _fp]),
    "ci_mlp_predict": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "ci_mlp_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, _fp,
                                   C.POINTER(C.c_double)]),
    "ci_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                               C.c_float, C.c_ulonglong, _dp, C.c_void_p]),
    "ci_gemm_bf16": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int,
                               C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                               C.c_float, C.c_float, C.c_void_p, C.c_int, C.c_void_p,
                               C.c_void_p]),
    "ci_strain_energy_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                           C.c_void_p, C.c_double, C.c_double, C.c_void_p,
                                           C.c_void_p]),
}


class CiError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    """Load libcppimpact_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m cppimpact_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in EXPORTS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != CI_OK:
        raise CiError(rc, lib().ci_last_error().decode())


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _f(a):
    return None if a is None else a.ctypes.data_as(_fp)


class MeshArrays:
    """Owns contiguous copies of a mesh and the CiMesh view of them."""

    def __init__(self, xloc, conn, slave=None, fixed=None):
        self.xloc = np.ascontiguousarray(xloc, dtype=np.float64).reshape(-1, 3)
        self.conn = np.ascontiguousarray(conn, dtype=np.int32)
        self.slave = np.ascontiguousarray([] if slave is None else slave, dtype=np.int32)
        self.fixed = np.ascontiguousarray([] if fixed is None else fixed, dtype=np.int32)
        self.c = CiMesh(self.xloc.shape[0], self.conn.shape[0], self.conn.shape[1],
                        self.xloc.ctypes.data_as(_dp), self.conn.ctypes.data_as(_ip),
                        self.slave.size, self.slave.ctypes.data_as(_ip),
                        self.fixed.size, self.fixed.ctypes.data_as(_ip))


def plan_stats(xloc, conn, chunk_elements=0, chunk_nodes=0, perms=False):
    m = MeshArrays(xloc, conn)
    st = (C.c_longlong * 8)()
    pe = np.zeros(m.conn.shape[0], dtype=np.int32) if perms else None
    pn = np.zeros(m.xloc.shape[0], dtype=np.int32) if perms else None
    check(lib().ci_plan_stats(C.byref(m.c), chunk_elements, chunk_nodes, st,
                              None if pe is None else pe.ctypes.data_as(_ip),
                              None if pn is None else pn.ctypes.data_as(_ip)))
    keys = ["chunks", "max_colors", "max_local", "slots", "max_chunk_elems", "ghosts",
            "boundary_nodes", "max_task_deps"]
    out = {k: int(st[i]) for i, k in enumerate(keys)}
    if perms:
        out["perm_elems"], out["perm_nodes"] = pe, pn
    return out


def plan_verify(xloc, conn, chunk_elements=0, chunk_nodes=0) -> None:
    m = MeshArrays(xloc, conn)
    check(lib().ci_plan_verify(C.byref(m.c), chunk_elements, chunk_nodes))


class Solver:
    """Direct handle on a ``ci_solver``: the per-step hot path on one GPU."""

    def __init__(self, xloc, conn, *, E, nu, rho, sigma_y0=0.0, H=0.0, beta=0.0,
                 wall_normal=(0.0, 0.0, 1.0), wall_offset=-1e30, wall_stiffness=0.0,
                 mode=MODE_J2, lumping=LUMP_HRZ, gravity=(0.0, 0.0, -9.81), device=0,
                 chunk_elements=0, chunk_nodes=0, graph_steps=0, step_kernel=0, block_threads=0,
                 elem_lanes=0, slave=None, fixed=None):
        self.mesh = MeshArrays(xloc, conn, slave, fixed)
        self.N, self.E = self.mesh.xloc.shape[0], self.mesh.conn.shape[0]
        self.npe = self.mesh.conn.shape[1]
        self.nq = 1 if self.npe == 4 else 4
        mat = CiMaterial(E, nu, rho, sigma_y0, H, beta)
        wall = CiWall((C.c_double * 3)(*wall_normal), wall_offset, wall_stiffness)
        opt = CiOptions(mode, lumping, (C.c_double * 3)(*gravity), device, chunk_elements,
                        chunk_nodes, graph_steps, step_kernel, block_threads, elem_lanes)
        self._h = C.c_void_p()
        check(lib().ci_create(C.byref(self.mesh.c), C.byref(mat), C.byref(wall), C.byref(opt),
                              C.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().ci_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize(self, vel, pos=(0.0, 0.0, 0.0)):
        p = np.asarray(pos, dtype=np.float64)
        v = np.asarray(vel, dtype=np.float64)
        check(lib().ci_initialize(self._h, _d(p), _d(v)))

    def start(self, dt):
        check(lib().ci_start(self._h, dt))

    def step(self, n):
        check(lib().ci_step(self._h, int(n)))

    def solve(self, dt, time_end, export_interval=1 << 30):
        check(lib().ci_solve(self._h, dt, time_end, export_interval))

    def steps_done(self) -> int:
        n = C.c_longlong(0)
        check(lib().ci_steps_done(self._h, C.byref(n)))
        return n.value

    def state(self, fields=("x", "v", "mass", "sigma", "epbar", "contact")):
        """Nodal state in the caller's order; only the requested fields are copied."""
        want = set(fields)
        x = np.zeros((self.N, 3)) if "x" in want else None
        v = np.zeros((self.N, 3)) if "v" in want else None
        m = np.zeros(self.N) if "mass" in want else None
        sg = np.zeros((self.E, self.nq, 6), dtype=np.float32) if "sigma" in want else None
        ep = np.zeros((self.E, self.nq), dtype=np.float32) if "epbar" in want else None
        ct = np.zeros(self.N, dtype=np.uint8) if "contact" in want else None
        check(lib().ci_get_state(self._h, _d(x), _d(v), _d(m), _f(sg), _f(ep),
                                 None if ct is None else ct.ctypes.data_as(_ubp)))
        out = dict(x=x, v=v, mass=m, sigma=sg, epbar=ep, contact=ct)
        return {k: val for k, val in out.items() if k in want}

    def get_xv(self, x_out, v_out):
        """Positions and velocities into caller-owned float64 [N, 3] arrays (no
        allocation; pinned host arrays make the copies direct DMA)."""
        for a in (x_out, v_out):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != 3 * self.N:
                raise ValueError("x_out / v_out must be C-contiguous float64 with 3N entries")
        check(lib().ci_get_state(self._h, _d(x_out), _d(v_out), None, None, None, None))

    def deformation_gradient(self):
        """F = I + du/dX at every Gauss point of the current state, float64 [E, nq, 3, 3]
        in the caller's element order (ci_deformation_gradient)."""
        F = np.zeros((self.E, self.nq, 3, 3))
        check(lib().ci_deformation_gradient(self._h, _d(F)))
        return F

    def nodal_fields(self):
        """The reference's nodal export fields: acceleration [N, 3] of the last step,
        strain and stress [N, 6] (Voigt xx yy zz gamma_xy gamma_yz gamma_xz; each node
        takes the value of the last element containing it)."""
        acc, eps, sig = np.zeros((self.N, 3)), np.zeros((self.N, 6)), np.zeros((self.N, 6))
        check(lib().ci_get_nodal_fields(self._h, _d(acc), _d(eps), _d(sig)))
        return {"acc": acc, "strain": eps, "stress": sig}

    def set_state(self, x, v):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        check(lib().ci_set_state(self._h, _d(x), _d(v)))

    def save_state(self, path):
        """Binary state file for a restart (ci_save_state)."""
        check(lib().ci_save_state(self._h, os.fsencode(path)))

    def load_state(self, path):
        """Restore a state file written for the same mesh and options (ci_load_state)."""
        check(lib().ci_load_state(self._h, os.fsencode(path)))

    def energy(self) -> dict:
        e = CiEnergy()
        check(lib().ci_get_energy(self._h, C.byref(e)))
        return {k: getattr(e, k) for k, _ in CiEnergy._fields_}

    def status(self) -> int:
        s = C.c_uint(0)
        check(lib().ci_get_status(self._h, C.byref(s)))
        return s.value

    def internal_force(self, x, du, sigma=None, epbar=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        du = np.ascontiguousarray(du, dtype=np.float64)
        si = None if sigma is None else np.ascontiguousarray(sigma, dtype=np.float32)
        ei = None if epbar is None else np.ascontiguousarray(epbar, dtype=np.float32)
        f = np.zeros((self.N, 3))
        so = np.zeros((self.E, self.nq, 6), dtype=np.float32)
        eo = np.zeros((self.E, self.nq), dtype=np.float32)
        check(lib().ci_internal_force(self._h, _d(x), _d(du), _f(si), _f(ei), _d(f), _f(so),
                                      _f(eo)))
        return f, so, eo

    def lumped_mass(self, x=None):
        x = self.mesh.xloc if x is None else np.ascontiguousarray(x, dtype=np.float64)
        m = np.zeros(self.N)
        check(lib().ci_lumped_mass(self._h, _d(x), _d(m)))
        return m

    def strain_energy(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        W, V = C.c_double(0), C.c_double(0)
        check(lib().ci_strain_energy(self._h, _d(u), C.byref(W), C.byref(V)))
        return W.value, V.value

    def time_steps(self, n) -> float:
        ms = C.c_float(0)
        check(lib().ci_time_steps(self._h, int(n), C.byref(ms)))
        return ms.value

    def time_kernels(self, n):
        out = (C.c_float * 2)()
        check(lib().ci_time_kernels(self._h, int(n), out))
        return out[0], out[1]

    def launches_per_step(self) -> int:
        return lib().ci_launches_per_step(self._h)

    def step_kernel(self) -> int:
        """The step kernel this solver runs: 1 element + node kernels, 2 persistent task
        kernel, 3 fused (the automatic choice of step_kernel=0 resolved)."""
        return lib().ci_step_kernel(self._h)

    def debug_flow_stall(self, chunk: int, wait_seconds: float) -> None:
        """Test hook (ci_debug_flow_stall): the next task-kernel launch never publishes
        chunk `chunk`'s progress, so its waits give up after wait_seconds."""
        check(lib().ci_debug_flow_stall(self._h, int(chunk), float(wait_seconds)))


class Batch:
    """Many instances (each: mesh, J2 material, wall, velocity, dt, end time) advanced
    together, one launch per step per element type (``ci_batch_*``).

    ``instances``: dicts with keys xloc, conn, E, nu, rho, sigma_y0, H, wall_normal,
    wall_offset, wall_stiffness, vel, dt, t_end (and optionally pos)."""

    def __init__(self, instances, *, gravity=(0.0, 0.0, -9.81), device=0, chunk_nodes=0,
                 block_threads=0, elem_lanes=0, autotune_steps=0, chunk_elements=0):
        self._meshes = []
        arr = (CiInstance * len(instances))()
        shared = {}  # instances passing the same arrays share one copy (and one plan)
        for i, d in enumerate(instances):
            key = (id(d["xloc"]), id(d["conn"]))
            if key not in shared:
                shared[key] = MeshArrays(d["xloc"], d["conn"])
            m = shared[key]
            self._meshes.append(m)
            arr[i].mesh = m.c
            arr[i].mat = CiMaterial(d["E"], d["nu"], d["rho"], d.get("sigma_y0", 0.0),
                                    d.get("H", 0.0), 0.0)
            arr[i].wall = CiWall((C.c_double * 3)(*d["wall_normal"]), d["wall_offset"],
                                 d["wall_stiffness"])
            arr[i].pos = (C.c_double * 3)(*d.get("pos", (0.0, 0.0, 0.0)))
            arr[i].vel = (C.c_double * 3)(*d["vel"])
            arr[i].dt = d["dt"]
            arr[i].t_end = d["t_end"]
        opt = CiOptions()
        lib().ci_default_options(C.byref(opt))
        opt.gravity = (C.c_double * 3)(*gravity)
        opt.device, opt.chunk_nodes, opt.chunk_elements = device, chunk_nodes, chunk_elements
        opt.block_threads, opt.elem_lanes = block_threads, elem_lanes
        opt.autotune_steps = autotune_steps
        self._arr = arr
        self._h = C.c_void_p()
        check(lib().ci_batch_create(arr, len(instances), C.byref(opt), C.byref(self._h)))
        self.n = len(instances)

    def tuning(self, npe) -> dict:
        """Tile shape of the group of npe-node elements (the autotuner's choice if tuned)."""
        ce, cn, bs, ln, ms = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0), C.c_float(0)
        check(lib().ci_batch_tuning(self._h, npe, C.byref(ce), C.byref(cn), C.byref(bs),
                                    C.byref(ln), C.byref(ms)))
        return dict(chunk_elements=ce.value, chunk_nodes=cn.value, block_threads=bs.value,
                    elem_lanes=ln.value, trial_ms_per_step=ms.value)

    def run(self) -> float:
        """Runs every instance to its end time; returns the batch's device time in ms."""
        ms = C.c_float(0)
        check(lib().ci_batch_run(self._h, C.byref(ms)))
        return ms.value

    def run_snapshots(self, every, d_snap_ptr, max_snaps) -> float:
        """Run with displacement snapshots (device buffer [max_snaps][N_total][3] FP32)."""
        ms = C.c_float(0)
        check(lib().ci_batch_run_snapshots(self._h, int(every), C.c_void_p(d_snap_ptr),
                                           int(max_snaps), C.byref(ms)))
        return ms.value

    def run_peaks(self, every, max_snaps):
        """Run keeping per instance the largest displacement norm over the snapshot
        states and the final largest equivalent plastic strain (ci_batch_run_peaks):
        (peak_disp [n], peak_epbar [n], device ms)."""
        n = len(self._meshes)
        pd, pe = np.zeros(n, dtype=np.float32), np.zeros(n, dtype=np.float32)
        ms = C.c_float(0)
        check(lib().ci_batch_run_peaks(self._h, int(every), int(max_snaps), _f(pd), _f(pe),
                                       C.byref(ms)))
        return pd, pe, ms.value

    def node_order(self, i):
        m = self._meshes[i]
        perm = np.zeros(m.xloc.shape[0], dtype=np.int32)
        off = C.c_int(0)
        check(lib().ci_batch_node_order(self._h, i, perm.ctypes.data_as(_ip), C.byref(off)))
        return perm, off.value

    def state(self, i):
        m = self._meshes[i]
        N, (E, npe) = m.xloc.shape[0], m.conn.shape
        nq = 1 if npe == 4 else 4
        x, v = np.zeros((N, 3)), np.zeros((N, 3))
        ep = np.zeros((E, nq), dtype=np.float32)
        ct = np.zeros(N, dtype=np.uint8)
        ns = C.c_longlong(0)
        check(lib().ci_batch_get_state(self._h, i, _d(x), _d(v), _f(ep),
                                       ct.ctypes.data_as(_ubp), C.byref(ns)))
        return dict(x=x, v=v, epbar=ep, contact=ct, nsteps=ns.value)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().ci_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Reference-named classes (drop-in mirror)
# ---------------------------------------------------------------------------

class Mesh:
    """``Mesh<T, npe>``: fields num_nodes, num_elements, xloc, element_nodes, slave/fixed."""

    def __init__(self, nodes_per_element: int = 4):
        self.nodes_per_element = nodes_per_element
        self.num_nodes = self.num_elements = 0
        self.xloc = np.zeros(0)
        self.element_nodes = np.zeros((0, nodes_per_element), dtype=np.int32)
        self.slave_nodes = np.zeros(0, dtype=np.int32)
        self.fixed_nodes = np.zeros(0, dtype=np.int32)

    def load_mesh(self, filename: str) -> int:
        """0 on success, 1 if the file cannot be read (the reference's convention)."""
        m = CiMesh()
        rc = lib().ci_mesh_load_inp(filename.encode(), self.nodes_per_element, C.byref(m))
        if rc != CI_OK:
            return 1
        try:
            N, E, npe = m.num_nodes, m.num_elements, m.nodes_per_element
            self.num_nodes, self.num_elements = N, E
            self.xloc = np.ctypeslib.as_array(m.xloc, shape=(3 * N,)).copy()
            self.element_nodes = np.ctypeslib.as_array(m.element_nodes, shape=(E * npe,)).reshape(E, npe).copy()
            self.slave_nodes = (np.ctypeslib.as_array(m.slave_nodes, shape=(m.num_slave_nodes,)).copy()
                                if m.num_slave_nodes else np.zeros(0, dtype=np.int32))
            self.fixed_nodes = (np.ctypeslib.as_array(m.fixed_nodes, shape=(m.num_fixed_nodes,)).copy()
                                if m.num_fixed_nodes else np.zeros(0, dtype=np.int32))
        finally:
            lib().ci_mesh_free(C.byref(m))
        return 0


class BaseMaterial:
    def __init__(self, type: str, E: float, rho: float, nu: float, name: str = "Material"):
        self.type, self.E, self.rho, self.nu, self.name = type, E, rho, nu, name
        self.beta, self.H, self.Y0 = 0.0, 0.0, 0.0


class Elastoplastic(BaseMaterial):
    """``Elastoplastic(E, rho, nu, beta, H, Y0)``; beta is the kinematic fraction (0 only)."""

    def __init__(self, E, rho, nu, beta, H, Y0, name="Material"):
        super().__init__("InfinitesimalElastoplastic", E, rho, nu, name)
        self.beta, self.H, self.Y0 = beta, H, Y0


class Wall:
    """``Wall<T, dim, Basis>(name, location, stiffness, slave, n_slave, normal)``."""

    def __init__(self, name, location, stiffness, slave_node_indices=None, num_slave_nodes=0,
                 normal=1, dim=2):
        self.name, self.location, self.stiffness, self.normal, self.dim = (
            name, location, stiffness, normal, dim)
        self.slave_node_indices = slave_node_indices
        self.num_slave_nodes = num_slave_nodes

    def plane(self):
        n = [0.0, 0.0, 0.0]
        n[self.dim] = float(self.normal)
        return tuple(n), float(self.normal) * float(self.location)


class Dynamics:
    """``Dynamics<T, Basis, Analysis, Quadrature>(mesh, material, wall)`` on the GPU.

    ``mode`` defaults to the reference's own force law (RefCompat) so results match the
    reference; pass ``mode=MODE_J2`` for the elastoplastic solver.
    """

    def __init__(self, mesh: Mesh, material: BaseMaterial, wall: Wall | None = None, *,
                 mode=MODE_REFCOMPAT, lumping=None, gravity=(0.0, 0.0, -9.81), **kw):
        self.mesh, self.material, self.wall = mesh, material, wall
        npe = mesh.element_nodes.shape[1]
        if lumping is None:
            lumping = LUMP_ROWSUM if mode == MODE_REFCOMPAT else LUMP_HRZ
        n, off = wall.plane() if wall is not None else ((0.0, 0.0, 1.0), -1e300)
        k = wall.stiffness if wall is not None else 0.0
        sy = getattr(material, "Y0", 0.0) if mode == MODE_J2 else 0.0
        self._s = Solver(np.asarray(mesh.xloc).reshape(-1, 3), mesh.element_nodes,
                         E=material.E, nu=material.nu, rho=material.rho, sigma_y0=sy,
                         H=getattr(material, "H", 0.0), beta=getattr(material, "beta", 0.0),
                         wall_normal=n, wall_offset=off, wall_stiffness=k, mode=mode,
                         lumping=lumping, gravity=gravity, **kw)
        self.ndof = 3 * mesh.num_nodes
        self.timestep = 0
        self.global_xloc = np.asarray(mesh.xloc, dtype=np.float64).copy()
        self.vel = np.zeros(self.ndof)
        self.global_mass = np.zeros(self.ndof)

    def initialize(self, init_position, init_velocity):
        self._s.initialize(init_velocity, init_position)
        self.vel[:] = np.tile(np.asarray(init_velocity, dtype=np.float64), self.mesh.num_nodes)

    def solve(self, dt, time_end, export_interval=1 << 30):
        self._s.solve(dt, time_end, export_interval)
        st = self._s.state()
        self.global_xloc = st["x"].reshape(-1)
        self.vel = st["v"].reshape(-1)
        self.global_mass = np.repeat(st["mass"], 3)
        self.timestep += self._s.steps_done()
        return st

    def debug_strain(self, alpha, def_case):
        x = np.asarray(self.mesh.xloc).reshape(-1, 3)
        nu = self.material.nu
        u = np.zeros_like(x)
        g = x[:, 0] if def_case == 0 else 0.5 * x[:, 0] ** 2
        u[:, 0], u[:, 1], u[:, 2] = alpha * g, -alpha * g * nu, -alpha * g * nu
        return self._s.strain_energy(u)
