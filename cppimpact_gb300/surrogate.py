"""Learned surrogate for parameter sweeps: POD basis of displacement snapshots + MLP.

Pipeline (all dense algebra on the GPU through the library's BF16 tcgen05 GEMM and
MLP entry points; PyTorch only holds device buffers):

1. ``generate``: seeded impact parameters (velocity, yield stress, hardening, wall
   tilt) -> one batched solve of the tet4 cube per parameter set, with the
   displacement of every node recorded every ``every`` steps (``ci_batch_run_snapshots``).
2. ``pod``: rank-r POD basis of all training snapshots by a randomized range finder
   (Halko, Martinsson & Tropp 2011): Y = S Omega, Q = orth(Y), W = S^T Q, then the small
   eigenproblem of W^T W by cyclic Jacobi rotations in FP64 on the host.
3. modal trajectories A = S Phi; an MLP (4 -> H -> H -> r*snaps) maps normalised
   parameters to normalised modal trajectories, trained with ``ci_mlp_train``.
4. ``predict``: ensemble mean of several MLPs, reconstruction u = A Phi^T, peak
   displacement; queries whose ensemble spread exceeds the threshold, and an audited
   random fraction, are re-run by the plain solver (``fallback``).
The method without the network, for comparison, interpolates the training runs'
modal trajectories by inverse-distance weighting in parameter space.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import time

import numpy as np

from . import api
from . import meshgen as mg
from .sweep import tilted_setup

E, NU, RHO = 68.9e9, 0.33, 2700.0
LO = np.array([2.0, 200e6, 0.005, 0.0])   # velocity, yield, hardening / E, tilt (deg)
HI = np.array([20.0, 350e6, 0.02, 15.0])


@dataclasses.dataclass
class Config:
    n_cube: int = 12
    steps: int = 4000
    every: int = 50
    rank: int = 64
    hidden: int = 256
    n_train: int = 4096
    n_test: int = 512
    epochs: int = 1500
    batch: int = 256
    lr: float = 2e-3
    ensemble: int = 5
    spread_threshold: float = 0.0075
    audit_fraction: float = 0.05
    error_threshold: float = 0.02
    seed: int = mg.DEFAULT_SEED

    @property
    def snaps(self) -> int:
        return self.steps // self.every


def sample_params(n: int, rng) -> np.ndarray:
    return LO + (HI - LO) * rng.random((n, 4))


def normalise(p: np.ndarray) -> np.ndarray:
    return (2.0 * (p - LO) / (HI - LO) - 1.0).astype(np.float32)


def _torch():
    import torch
    return torch


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def gemm(A, B, transA=False, transB=False, out=None, out_bf16=None, beta=0.0):
    """C = op(A) op(B) with the library's BF16 tensor-core GEMM (torch CUDA tensors)."""
    torch = _torch()
    assert A.dtype == torch.bfloat16 and B.dtype == torch.bfloat16
    M = A.shape[1] if transA else A.shape[0]
    K = A.shape[0] if transA else A.shape[1]
    N = B.shape[0] if transB else B.shape[1]
    if out is None:
        out = torch.zeros((M, N), dtype=torch.float32, device=A.device)
    err = torch.zeros(1, dtype=torch.int32, device=A.device)
    api.check(api.lib().ci_gemm_bf16(A.data_ptr(), A.shape[1], int(transA), B.data_ptr(), B.shape[1],
                                     int(transB), out.data_ptr(), out.shape[1],
                                     None if out_bf16 is None else out_bf16.data_ptr(), M, N, K,
                                     1.0, beta, None, 0, err.data_ptr(), _stream(torch)))
    if int(err.item()) != 0:
        raise RuntimeError("tensor-core GEMM timed out")
    return out


def jacobi_eigh(A: np.ndarray, sweeps: int = 60, tol: float = 1e-14):
    """Eigen-decomposition of a small symmetric matrix by cyclic Jacobi rotations
    (Golub & Van Loan, Matrix Computations, 4th ed., section 8.5); descending order."""
    A = np.array(A, dtype=np.float64, copy=True)
    n = A.shape[0]
    V = np.eye(n)
    for _ in range(sweeps):
        off = np.sqrt(np.sum(np.tril(A, -1) ** 2))
        if off <= tol * np.sqrt(np.sum(A * A)):
            break
        for p in range(n - 1):
            for q in range(p + 1, n):
                if abs(A[p, q]) < 1e-300:
                    continue
                tau = (A[q, q] - A[p, p]) / (2.0 * A[p, q])
                t = math.copysign(1.0, tau) / (abs(tau) + math.sqrt(1.0 + tau * tau))
                c = 1.0 / math.sqrt(1.0 + t * t)
                s = t * c
                Ap, Aq = A[:, p].copy(), A[:, q].copy()
                A[:, p], A[:, q] = c * Ap - s * Aq, s * Ap + c * Aq
                Ap, Aq = A[p, :].copy(), A[q, :].copy()
                A[p, :], A[q, :] = c * Ap - s * Aq, s * Ap + c * Aq
                Vp, Vq = V[:, p].copy(), V[:, q].copy()
                V[:, p], V[:, q] = c * Vp - s * Vq, s * Vp + c * Vq
    w = np.diag(A).copy()
    order = np.argsort(-w)
    return w[order], V[:, order]


def _instances(params, cfg, mesh):
    # the wall stiffness and the stable dt depend on the mesh only
    k, dt = mg.wall_stiffness(mesh, E), mg.cfl_dt(mesh, E, NU, RHO)
    inst = []
    for v, sy, h, tilt in params:
        st = tilted_setup(mesh, v, tilt, stiffness=k, dt=dt)
        st["t_end"] = (cfg.steps - 0.5) * st["dt"]
        inst.append(dict(xloc=mesh.xloc, conn=mesh.conn, E=E, nu=NU, rho=RHO, sigma_y0=sy,
                         H=h * E, **st))
    return inst


def tune_shape(params: np.ndarray, cfg: Config, mesh: mg.TetMesh | None = None,
               steps: int = 64) -> dict:
    """Tile shape the batch autotuner picks for a batch like `params` (timed on it)."""
    mesh = mesh or mg.cube(cfg.n_cube, 1)
    b = api.Batch(_instances(params, cfg, mesh), autotune_steps=steps)
    t = b.tuning(mesh.npe)
    b.close()
    return {k: t[k] for k in ("chunk_elements", "chunk_nodes", "block_threads")}


def generate(params: np.ndarray, cfg: Config, mesh: mg.TetMesh | None = None,
             shape: dict | None = None):
    """Batched solves (tile shape `shape`, e.g. from tune_shape; default plan otherwise);
    returns (snapshots [n, snaps, 3N] FP32 torch in caller node order, peak equivalent
    plastic strain [n], device ms)."""
    torch = _torch()
    mesh = mesh or mg.cube(cfg.n_cube, 1)
    inst = _instances(params, cfg, mesh)
    b = api.Batch(inst, **(shape or {}))
    n, N = len(inst), mesh.num_nodes
    snap = torch.zeros((cfg.snaps, n * N, 3), dtype=torch.float32, device="cuda")
    ms = b.run_snapshots(cfg.every, snap.data_ptr(), cfg.snaps)
    perm, _ = b.node_order(0)
    inv = np.argsort(perm)          # caller node -> plan position
    s = snap.view(cfg.snaps, n, N, 3)[:, :, torch.as_tensor(inv, device="cuda"), :]
    s = s.permute(1, 0, 2, 3).reshape(n, cfg.snaps, 3 * N).contiguous()
    peak_ep = np.array([float(b.state(i)["epbar"].max()) for i in range(n)])
    b.close()
    return s, peak_ep, ms


def peak_disp(snaps) -> "torch.Tensor":
    """max over snapshots and nodes of the nodal displacement norm, per run."""
    n, k, d = snaps.shape
    return snaps.view(n, k, d // 3, 3).norm(dim=3).amax(dim=(1, 2))


def pod(S, rank: int, oversample: int = 32, seed: int = 0):
    """Rank-r right singular vectors of the snapshot matrix S [rows x dofs] (BF16)."""
    torch = _torch()
    g = torch.Generator(device="cuda").manual_seed(seed)
    k = rank + oversample
    dofs = S.shape[1]
    # the two products with the long dimensions run as A B^T with K-major operands
    # (the pipelined tensor-core path): Omega is drawn transposed, S^T formed once
    OmT = torch.randn((k, dofs), generator=g, device="cuda").to(torch.bfloat16)
    Yb = torch.empty((S.shape[0], k), dtype=torch.bfloat16, device="cuda")
    gemm(S, OmT, transB=True, out_bf16=Yb)                 # Y = S Omega
    G = gemm(Yb, Yb, transA=True).double().cpu().numpy()   # Y^T Y
    w, U = jacobi_eigh(G)
    keep = w > w[0] * 1e-10
    Rinv = U[:, keep] / np.sqrt(w[keep])[None, :]          # Q = Y U diag(w)^-1/2
    Rb = torch.tensor(Rinv, dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
    Qb = torch.empty((S.shape[0], Rb.shape[1]), dtype=torch.bfloat16, device="cuda")
    gemm(Yb, Rb, out_bf16=Qb)
    St = S.t().contiguous()
    W = gemm(St, Qb.t().contiguous(), transB=True).double().cpu().numpy()  # W = S^T Q [dofs x k]
    del St
    w2, U2 = jacobi_eigh(W.T @ W)
    V = W @ U2[:, :rank] / np.sqrt(np.maximum(w2[:rank], 1e-300))[None, :]
    # orthonormalise (modified Gram-Schmidt, FP64)
    for j in range(rank):
        for i in range(j):
            V[:, j] -= (V[:, i] @ V[:, j]) * V[:, i]
        V[:, j] /= np.linalg.norm(V[:, j])
    return V, np.sqrt(np.maximum(w2[:rank], 0.0))


class MLP:
    """Handle on a library MLP (ci_mlp_*)."""

    def __init__(self, n_in, hidden, n_out, seed):
        self._h = C.c_void_p()
        api.check(api.lib().ci_mlp_create(n_in, hidden, n_out, seed, C.byref(self._h)))
        self.n_in, self.n_out = n_in, n_out

    def train(self, X, T, epochs, batch, lr, seed):
        torch = _torch()
        loss = np.zeros(epochs)
        api.check(api.lib().ci_mlp_train(self._h, X.data_ptr(), T.data_ptr(), X.shape[0], batch,
                                         epochs, lr, seed, loss.ctypes.data_as(C.POINTER(C.c_double)),
                                         _stream(torch)))
        torch.cuda.current_stream().synchronize()
        return loss

    def predict(self, X):
        torch = _torch()
        Y = torch.empty((X.shape[0], self.n_out), dtype=torch.float32, device="cuda")
        api.check(api.lib().ci_mlp_predict(self._h, X.data_ptr(), X.shape[0], Y.data_ptr(),
                                           _stream(torch)))
        return Y

    def gradients(self, X, T):
        n = api.lib().ci_mlp_num_params(self._h)
        g = np.zeros(n, dtype=np.float32)
        loss = C.c_double(0)
        api.check(api.lib().ci_mlp_gradients(self._h, X.data_ptr(), T.data_ptr(), X.shape[0],
                                             g.ctypes.data_as(C.POINTER(C.c_float)),
                                             C.byref(loss)))
        return g, loss.value

    def params(self):
        n = api.lib().ci_mlp_num_params(self._h)
        p = np.zeros(n, dtype=np.float32)
        api.check(api.lib().ci_mlp_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        api.check(api.lib().ci_mlp_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def close(self):
        if self._h.value:
            api.lib().ci_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Surrogate:
    def __init__(self, cfg: Config):
        self.cfg = cfg
        self.mesh = mg.cube(cfg.n_cube, 1)
        self.timings = {}

    def fit(self, params: np.ndarray, snaps, peak_ep=None):
        """params [n x 4], snaps [n, snaps, 3N] (torch FP32), peak_ep [n] (peak equivalent
        plastic strain; optional: the networks then predict it as one more output)."""
        torch = _torch()
        cfg = self.cfg
        n, k, d = snaps.shape
        t0 = time.perf_counter()
        S = snaps.reshape(n * k, d).to(torch.bfloat16).contiguous()
        Phi, sv = pod(S, cfg.rank, seed=cfg.seed)
        self.Phi = Phi
        self.Phib = torch.tensor(Phi, dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
        A = gemm(S, self.Phib.t().contiguous(), transB=True)  # modal trajectories [n*k x r]
        torch.cuda.synchronize()
        self.timings["pod_s"] = time.perf_counter() - t0
        rel = float((S.float() - gemm(A.to(torch.bfloat16).contiguous(), self.Phib, transB=True)).norm()
                    / S.float().norm())
        self.pod_error = rel
        # modal trajectories per unit impact speed (displacements scale with it), then
        # one scale for all outputs: the squared error of a normalised output is then
        # proportional to the error of the reconstructed displacement relative to v t
        Y = A.view(n, k * cfg.rank) / self._speed(params)[:, None]
        self.y_mean = Y.mean(dim=0, keepdim=True)
        self.y_std = (Y - self.y_mean).std() + 1e-30
        Yn = ((Y - self.y_mean) / self.y_std).contiguous()
        X = torch.tensor(normalise(params), device="cuda")
        self.train_X, self.train_Y = X, Y
        t0 = time.perf_counter()
        self.nets = [MLP(4, cfg.hidden, Yn.shape[1], cfg.seed + 101 * j) for j in range(cfg.ensemble)]
        jobs = [(net, X, Yn, cfg.seed + 7 * j) for j, net in enumerate(self.nets)]
        # peak equivalent plastic strain: a smaller network per ensemble member
        self.with_ep = peak_ep is not None
        self.ep_nets = []
        if self.with_ep:
            ep = torch.tensor(np.asarray(peak_ep, dtype=np.float32), device="cuda")[:, None]
            self.ep_mean, self.ep_std = ep.mean(), ep.std() + 1e-30
            self.train_ep = ep[:, 0]
            Tn = ((ep - self.ep_mean) / self.ep_std).contiguous()
            self.ep_nets = [MLP(4, 64, 1, cfg.seed + 303 * j) for j in range(cfg.ensemble)]
            jobs += [(net, X, Tn, cfg.seed + 11 * j) for j, net in enumerate(self.ep_nets)]
        losses = self._train_concurrently(jobs)
        self.losses = losses[:cfg.ensemble]
        torch.cuda.synchronize()
        self.timings["train_s"] = time.perf_counter() - t0

    @staticmethod
    def _speed(params):
        torch = _torch()
        return torch.tensor(np.asarray(params, dtype=np.float32)[:, 0], device="cuda")

    def _train_concurrently(self, jobs):
        """Trains independent networks at the same time, each on its own CUDA stream
        driven by its own host thread (the training kernels of one member are small and
        latency bound, so members overlap on the GPU); returns their loss histories.
        Every member's result is the same as when trained alone."""
        torch = _torch()
        from concurrent.futures import ThreadPoolExecutor
        main = torch.cuda.current_stream()
        streams = [torch.cuda.Stream() for _ in jobs]

        def run(j):
            net, X, T, seed = jobs[j]
            streams[j].wait_stream(main)
            with torch.cuda.stream(streams[j]):
                return self._train(net, X, T, seed)

        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            out = list(ex.map(run, range(len(jobs))))
        for st in streams:
            main.wait_stream(st)
        return out

    def _train(self, net, X, T, seed):
        """Adam in three phases of decreasing step size (lr, lr/5, lr/25)."""
        cfg = self.cfg
        parts = [cfg.epochs // 2, cfg.epochs // 4, cfg.epochs - cfg.epochs // 2 - cfg.epochs // 4]
        losses = []
        for i, (ep, lr) in enumerate(zip(parts, (cfg.lr, cfg.lr / 5, cfg.lr / 25))):
            if ep > 0:
                losses.append(net.train(X, T, ep, cfg.batch, lr, seed + 1000 * i))
        return np.concatenate(losses)

    def _reconstruct_peak(self, A):
        """A [n, snaps * r] modal trajectories -> peak displacement per run."""
        torch = _torch()
        n = A.shape[0]
        k, r = self.cfg.snaps, self.cfg.rank
        U = gemm(A.view(n * k, r).to(torch.bfloat16).contiguous(), self.Phib, transB=True)
        return peak_disp(U.view(n, k, -1))

    def predict(self, params: np.ndarray, with_ep: bool = False):
        """Ensemble prediction: (peak displacement mean, relative spread) per query, and
        the ensemble-mean peak equivalent plastic strain when ``with_ep``."""
        torch = _torch()
        X = torch.tensor(normalise(params), device="cuda")
        v = self._speed(params)[:, None]
        peaks = []
        for net in self.nets:
            A = (net.predict(X) * self.y_std + self.y_mean) * v
            peaks.append(self._reconstruct_peak(A))
        P = torch.stack(peaks)
        mean = P.mean(dim=0)
        spread = P.std(dim=0) / mean.clamp_min(1e-30) if len(peaks) > 1 else torch.zeros_like(mean)
        if not with_ep:
            return mean, spread
        ep = None
        if self.ep_nets:
            ep = torch.stack([net.predict(X)[:, 0] for net in self.ep_nets]).mean(dim=0)
            ep = ep * self.ep_std + self.ep_mean
        return mean, spread, ep

    def predict_idw(self, params: np.ndarray, k_nn: int = 8):
        """The method without the network: inverse-distance-weighted interpolation of the
        training runs' modal trajectories in normalised parameter space."""
        torch = _torch()
        X = torch.tensor(normalise(params), device="cuda")
        d = torch.cdist(X, self.train_X)
        dist, idx = d.topk(k_nn, largest=False)
        w = 1.0 / dist.clamp_min(1e-6) ** 2
        w = w / w.sum(dim=1, keepdim=True)
        A = (self.train_Y[idx] * w[..., None]).sum(dim=1) * self._speed(params)[:, None]
        if getattr(self, "with_ep", False):
            return self._reconstruct_peak(A), (self.train_ep[idx] * w).sum(dim=1)
        return self._reconstruct_peak(A)


def fallback_runs(params: np.ndarray, cfg: Config, mesh=None, shape=None):
    """The solver for the given queries (one batch): peak displacement, peak equivalent
    plastic strain, device ms."""
    if len(params) == 0:
        return np.zeros(0), np.zeros(0), 0.0
    mesh = mesh or mg.cube(cfg.n_cube, 1)
    b = api.Batch(_instances(params, cfg, mesh), **(shape or {}))
    pd, pe, ms = b.run_peaks(cfg.every, cfg.snaps)
    b.close()
    return pd.astype(np.float64), pe.astype(np.float64), ms


def plain_run_ms(params: np.ndarray, cfg: Config, mesh=None) -> list[float]:
    """Device time of whole runs of the plain (unbatched) GPU solver, one at a time."""
    mesh = mesh or mg.cube(cfg.n_cube, 1)
    out = []
    for v, sy, h, tilt in params:
        st = tilted_setup(mesh, v, tilt)
        s = api.Solver(mesh.xloc, mesh.conn, E=E, nu=NU, rho=RHO, sigma_y0=sy, H=h * E,
                       wall_normal=st["wall_normal"], wall_offset=st["wall_offset"],
                       wall_stiffness=st["wall_stiffness"])
        s.initialize(st["vel"])
        s.start(st["dt"])
        out.append(s.time_steps(cfg.steps))
        s.close()
    return out


def _errstats(e: np.ndarray) -> dict:
    e = np.asarray(e, dtype=np.float64)
    if e.size == 0:
        return {}
    return dict(mean=float(e.mean()), p50=float(np.median(e)), p95=float(np.quantile(e, 0.95)),
                max=float(e.max()), frac_over_2pct=float((e > 0.02).mean()))


def _time_gemm(A, B, out, reps):
    torch = _torch()
    gemm(A, B, transB=True, out=out)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        gemm(A, B, transB=True, out=out)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def gemm_tflops(rows: int, dofs: int, k: int, reps: int = 5, square: int = 8192) -> dict:
    """Throughput of the POD's largest product, W = S^T Q ([dofs x rows] x [rows x k]),
    run as A B^T with K-major operands (its arithmetic intensity is ~k/2 flop per byte
    of S, so HBM bounds it), and of a square A B^T of side `square` (tensor bound)."""
    torch = _torch()
    St = torch.randn((dofs, rows), device="cuda").to(torch.bfloat16)   # S^T, K-major
    Qt = torch.randn((k, rows), device="cuda").to(torch.bfloat16)      # Q^T, K-major
    out = torch.empty((dofs, k), dtype=torch.float32, device="cuda")
    ms = _time_gemm(St, Qt, out, reps)
    pod = dict(shape=[dofs, k, rows], ms=ms, tflops=2.0 * rows * dofs * k / (ms * 1e-3) / 1e12,
               hbm_gbs=(St.numel() + Qt.numel()) * 2 / (ms * 1e-3) / 1e9)
    del St, Qt, out
    A = torch.randn((square, square), device="cuda").to(torch.bfloat16)
    B = torch.randn((square, square), device="cuda").to(torch.bfloat16)
    out = torch.empty((square, square), dtype=torch.float32, device="cuda")
    ms = _time_gemm(A, B, out, reps)
    sq = dict(shape=[square] * 3, ms=ms, tflops=2.0 * square ** 3 / (ms * 1e-3) / 1e12)
    return dict(pod=pod, square=sq)


def study(cfg: Config, plain_sample: int = 4, audit_fail_fraction: float = 0.1) -> dict:
    """The surrogate sweep end to end: training runs, fit, prediction of held-out
    parameter sets with audit and fallback, errors against the solver, and runs/hour
    against the plain GPU solver and the batched solver alone."""
    torch = _torch()
    rng = np.random.default_rng(cfg.seed)
    ptr, pte = sample_params(cfg.n_train, rng), sample_params(cfg.n_test, rng)
    mesh = mg.cube(cfg.n_cube, 1)
    out = {"config": dataclasses.asdict(cfg), "mesh": {"elements": mesh.num_elements,
                                                       "nodes": mesh.num_nodes}}
    # tile shapes for big batches (training and evaluation runs) and for fallback-sized
    # ones, each picked by the autotuner on a batch of that size (one-off)
    t0 = time.perf_counter()
    n_fb = max(1, int(math.ceil((cfg.audit_fraction + 0.02) * cfg.n_test)))
    shape_big = tune_shape(ptr[:min(len(ptr), 256)], cfg, mesh)
    shape_fb = tune_shape(pte[:n_fb], cfg, mesh)
    out["tuning"] = {"big": shape_big, "fallback": shape_fb, "fallback_batch": n_fb,
                     "wall_s": time.perf_counter() - t0}
    t0 = time.perf_counter()
    s_tr, ep_tr, ms_tr = generate(ptr, cfg, mesh, shape_big)
    out["train_runs"] = {"wall_s": time.perf_counter() - t0, "device_ms": ms_tr}
    t0 = time.perf_counter()
    # the batched solver answering the whole sweep: per-run peaks reduced on the GPU
    truth_d, truth_ep, ms_te = fallback_runs(pte, cfg, mesh, shape_big)
    wall_te = time.perf_counter() - t0
    sur = Surrogate(cfg)
    t0 = time.perf_counter()
    sur.fit(ptr, s_tr, ep_tr)
    out["fit"] = {"wall_s": time.perf_counter() - t0, **sur.timings, "pod_rel_error": sur.pod_error,
                  "final_loss": [float(l[-1]) for l in sur.losses]}
    del s_tr
    torch.cuda.synchronize()
    # surrogate answers: ensemble prediction, then the solver for flagged + audited queries
    sur.predict(pte[:8], with_ep=True)   # first use loads the reduction kernels
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mean, spread, ep_pred = sur.predict(pte, with_ep=True)
    mean, spread, ep_pred = mean.cpu().numpy(), spread.cpu().numpy(), ep_pred.cpu().numpy()
    t_pred = time.perf_counter() - t0
    n = len(pte)
    # flag by ensemble spread, re-run the flagged queries and a random audited share of
    # the rest with the solver; an audit that misses too often re-runs everything.  The
    # spread does not catch every miss (a few answers on which all members agree are off
    # by more than the threshold), so the fraction of answers within it is reported
    # beside the throughput.
    flagged = spread > cfg.spread_threshold
    arng = np.random.default_rng(cfg.seed + 1)
    cand = np.flatnonzero(~flagged)
    n_audit = min(len(cand), int(math.ceil(cfg.audit_fraction * n)))
    audit = np.zeros(n, bool)
    audit[arng.choice(cand, n_audit, replace=False)] = True
    rerun = flagged | audit
    t0 = time.perf_counter()
    fb_d, fb_ep, fb_ms = fallback_runs(pte[rerun], cfg, mesh, shape_fb)
    t_fb = time.perf_counter() - t0
    final_d, final_ep = mean.copy(), ep_pred.copy()
    final_d[rerun], final_ep[rerun] = fb_d, fb_ep
    in_audit = audit[rerun]            # audited among the re-run queries, in fb_d order
    aud_err = np.abs(mean[rerun][in_audit] - fb_d[in_audit]) / fb_d[in_audit]
    full_fallback = bool(n_audit and (aud_err > cfg.error_threshold).mean() > audit_fail_fraction)
    t_full = 0.0
    if full_fallback:
        rest = ~rerun
        t0 = time.perf_counter()
        d2, e2, _ = fallback_runs(pte[rest], cfg, mesh, shape_big)
        t_full = time.perf_counter() - t0
        final_d[rest], final_ep[rest] = d2, e2
    t_sur = t_pred + t_fb + t_full
    ep_scale = max(float(truth_ep.max()), 1e-30)
    # the method without the network: inverse-distance interpolation of training runs
    idw_d, idw_ep = sur.predict_idw(pte)
    idw_d, idw_ep = idw_d.cpu().numpy(), idw_ep.cpu().numpy()
    out["errors"] = {
        "surrogate_only_peak_disp": _errstats(np.abs(mean - truth_d) / truth_d),
        "final_peak_disp": _errstats(np.abs(final_d - truth_d) / truth_d),
        "idw_peak_disp": _errstats(np.abs(idw_d - truth_d) / truth_d),
        "surrogate_only_peak_epbar_abs_over_max": _errstats(np.abs(ep_pred - truth_ep) / ep_scale),
        "final_peak_epbar_abs_over_max": _errstats(np.abs(final_ep - truth_ep) / ep_scale),
        "idw_peak_epbar_abs_over_max": _errstats(np.abs(idw_ep - truth_ep) / ep_scale),
        "peak_epbar_max": ep_scale,
        "audit_error": _errstats(aud_err),
    }
    out["audit"] = {"flagged_by_spread": int(flagged.sum()), "audited": int(n_audit),
                    "rerun": int(rerun.sum()), "full_fallback": full_fallback,
                    "spread_threshold": cfg.spread_threshold,
                    "audited_misses": int((aud_err > cfg.error_threshold).sum())}
    # how the spread threshold trades re-runs against the error left in the answers
    err_only = np.abs(mean - truth_d) / truth_d
    out["spread_threshold_scan"] = [
        {"threshold": th, "flagged": int((spread > th).sum()),
         "unflagged_frac_over_2pct": float((err_only[spread <= th] > 0.02).mean()) if (spread <= th).any() else 0.0,
         "unflagged_max": float(err_only[spread <= th].max()) if (spread <= th).any() else 0.0}
        for th in (0.0025, 0.005, 0.0075, 0.01, 0.02)]
    plain = plain_run_ms(pte[:plain_sample], cfg, mesh)
    plain_ms = float(np.mean(plain))
    out["timing"] = {"predict_s": t_pred, "fallback_wall_s": t_fb, "fallback_device_ms": fb_ms,
                     "full_fallback_s": t_full, "surrogate_sweep_s": t_sur,
                     "batched_sweep_wall_s": wall_te, "batched_sweep_device_ms": ms_te,
                     "plain_run_device_ms": plain_ms}
    rph = lambda count, sec: count / max(sec, 1e-12) * 3600.0
    one_off = out["tuning"]["wall_s"] + out["train_runs"]["wall_s"] + out["fit"]["wall_s"]
    out["runs_per_hour"] = {
        "surrogate": rph(n, t_sur),
        "batched_solver": rph(n, wall_te),
        "plain_gpu_solver": rph(1, plain_ms / 1e3),
        "surrogate_incl_training_for_this_sweep": rph(n, t_sur + one_off),
        "break_even_queries": one_off / max(plain_ms / 1e3 - t_sur / n, 1e-12),
    }
    out["speedup_vs_plain_gpu"] = out["runs_per_hour"]["surrogate"] / out["runs_per_hour"]["plain_gpu_solver"]
    # amortised over a sweep of Q queries: the one-off cost (tile tuning, training runs,
    # fit) plus Q times this sweep's cost per query (prediction, audit, re-runs)
    per_q = t_sur / n
    out["amortised"] = [
        {"queries": q, "runs_per_hour": rph(q, one_off + q * per_q),
         "vs_plain_gpu": rph(q, one_off + q * per_q) / out["runs_per_hour"]["plain_gpu_solver"],
         "vs_batched_solver": rph(q, one_off + q * per_q) / out["runs_per_hour"]["batched_solver"]}
        for q in (n, 10_000, 100_000, 1_000_000)]
    out["one_off_s"] = one_off
    out["gemm"] = gemm_tflops(cfg.n_train * cfg.snaps, 3 * mesh.num_nodes, cfg.rank + 32)
    return out


def time_training(n_in=4, hidden=256, n_out=5120, rows=4096, batch=256, epochs=20, seed=0):
    """Milliseconds per training epoch of one MLP member (ci_mlp_train) on seeded random
    data of the surrogate's shapes."""
    torch = _torch()
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    X = torch.randn(rows, n_in, device="cuda", generator=g)
    T = 0.1 * torch.randn(rows, n_out, device="cuda", generator=g)
    net = MLP(n_in, hidden, n_out, seed + 1)
    net.train(X, T, 1, batch, 2e-3, seed)  # warm-up (tensor maps, first launches)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    net.train(X, T, epochs, batch, 2e-3, seed)
    torch.cuda.synchronize()
    ms = 1e3 * (time.perf_counter() - t0) / epochs
    net.close()
    return ms


def time_square_gemm(n: int, reps: int = 10) -> dict:
    """TFLOP/s of C = A B^T for n x n BF16 operands (K-major, the persistent TMA kernel),
    best of three timings of `reps` back-to-back calls."""
    torch = _torch()
    A = torch.randn((n, n), device="cuda").to(torch.bfloat16)
    B = torch.randn((n, n), device="cuda").to(torch.bfloat16)
    out = torch.empty((n, n), dtype=torch.float32, device="cuda")
    ms = min(_time_gemm(A, B, out, reps) for _ in range(3))
    return dict(n=n, ms=ms, tflops=2.0 * n ** 3 / (ms * 1e-3) / 1e12)


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="time one surrogate MLP member's training, or "
                                             "(--gemm N) the square BF16 GEMM")
    ap.add_argument("--hidden", type=int, default=256)
    ap.add_argument("--n-out", type=int, default=5120)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--gemm", type=int, default=0, help="time an N x N x N A B^T instead")
    ap.add_argument("--reps", type=int, default=10)
    a = ap.parse_args()
    if a.gemm:
        r = time_square_gemm(a.gemm, a.reps)
        print(f"{r['n']}^3 BF16 A B^T: {r['ms']:.3f} ms, {r['tflops']:.1f} TFLOP/s")
    else:
        print(f"{a.epochs} epochs, 4 -> {a.hidden} -> {a.hidden} -> {a.n_out}: "
              f"{time_training(hidden=a.hidden, n_out=a.n_out, epochs=a.epochs):.2f} ms/epoch")
