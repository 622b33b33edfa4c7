"""Surrogate pieces on the GPU: MLP gradients against the float64 oracle, POD of a
known low-rank matrix, snapshots against the batch's own final state, and a small
end-to-end fit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_mlp_gradients_match_fp64_oracle(cilib):
    torch = pytest.importorskip("torch")
    import mlp_oracle
    from cppimpact_gb300 import surrogate as sg
    n_in, H, n_out, n = 4, 32, 40, 96
    rng = np.random.default_rng(3)
    X = rng.uniform(-1, 1, (n, n_in)).astype(np.float32)
    T = rng.standard_normal((n, n_out)).astype(np.float32)
    net = sg.MLP(n_in, H, n_out, seed=5)
    p = net.params()
    g, loss = net.gradients(torch.tensor(X, device="cuda"), torch.tensor(T, device="cuda"))
    # the GPU multiplies BF16-rounded operands: give the oracle the same weights
    pb = torch.tensor(p).to(torch.bfloat16).float().numpy()
    loss_ref, g_ref = mlp_oracle.loss_and_grad(pb, X, T, n_in, H, n_out)
    assert loss == pytest.approx(loss_ref, rel=2e-2)
    assert np.linalg.norm(g - g_ref) <= 3e-2 * np.linalg.norm(g_ref)
    # and the direction is right per layer block
    o = 0
    for size in (n_in * H, H, H * H, H, H * n_out, n_out):
        a, b = g[o:o + size], g_ref[o:o + size]
        assert a @ b > 0.98 * np.linalg.norm(a) * np.linalg.norm(b)
        o += size


def test_mlp_training_reduces_loss(cilib):
    torch = pytest.importorskip("torch")
    from cppimpact_gb300 import surrogate as sg
    rng = np.random.default_rng(1)
    X = rng.uniform(-1, 1, (512, 4)).astype(np.float32)
    W = rng.standard_normal((4, 20))
    T = np.tanh(X @ W).astype(np.float32)
    net = sg.MLP(4, 64, 20, seed=2)
    loss = net.train(torch.tensor(X, device="cuda"), torch.tensor(T, device="cuda"), epochs=60,
                     batch=64, lr=3e-3, seed=4)
    assert loss[-1] < 0.05 * loss[0]


def test_pod_recovers_low_rank_subspace(cilib):
    torch = pytest.importorskip("torch")
    from cppimpact_gb300 import surrogate as sg
    rng = np.random.default_rng(0)
    rows, dofs, r = 3000, 500, 6
    V = np.linalg.qr(rng.standard_normal((dofs, r)))[0]
    S = (rng.standard_normal((rows, r)) * np.array([10, 7, 5, 3, 2, 1.5])) @ V.T
    S += 1e-3 * rng.standard_normal(S.shape)
    Phi, sv = sg.pod(torch.tensor(S, dtype=torch.float32, device="cuda").to(torch.bfloat16), r)
    # principal angles between span(Phi) and span(V)
    s = np.linalg.svd(Phi.T @ V, compute_uv=False)
    assert s.min() > 0.999
    assert np.allclose(Phi.T @ Phi, np.eye(r), atol=1e-10)


def test_jacobi_eigh():
    from cppimpact_gb300 import surrogate as sg
    rng = np.random.default_rng(2)
    A = rng.standard_normal((12, 12))
    A = A + A.T
    w, V = sg.jacobi_eigh(A)
    wr = np.sort(np.linalg.eigvalsh(A))[::-1]
    assert np.allclose(w, wr, atol=1e-10)
    assert np.allclose(V @ np.diag(w) @ V.T, A, atol=1e-9)


def test_snapshots_match_final_state(cilib):
    torch = pytest.importorskip("torch")
    from cppimpact_gb300 import surrogate as sg
    cfg = sg.Config(n_cube=3, steps=200, every=50)
    params = sg.sample_params(3, np.random.default_rng(9))
    snaps, peak_ep, ms = sg.generate(params, cfg)
    assert snaps.shape == (3, 4, 3 * 64)
    # the last snapshot (after all 200 steps) is the unbatched solver's end state
    # rounded to FP32 (x - X recomputed in FP64 may differ by one FP32 rounding)
    from cppimpact_gb300 import meshgen as mg
    from cppimpact_gb300.sweep import tilted_setup
    m = mg.cube(3, 1)
    for i, (v, sy, h, tilt) in enumerate(params):
        st = tilted_setup(m, v, tilt)
        s = cilib.Solver(m.xloc, m.conn, E=sg.E, nu=sg.NU, rho=sg.RHO, sigma_y0=sy, H=h * sg.E,
                         wall_normal=st["wall_normal"], wall_offset=st["wall_offset"],
                         wall_stiffness=st["wall_stiffness"])
        s.initialize(st["vel"])
        s.start(st["dt"])
        s.step(200)
        u = (s.state(fields=("x",))["x"] - m.xloc).reshape(-1)
        got = snaps[i, -1].cpu().numpy().astype(np.float64)
        assert np.abs(got - u).max() <= 2e-7 * np.abs(u).max() + 1e-15


def test_run_peaks_match_snapshots(cilib):
    """ci_batch_run_peaks keeps per run the largest displacement norm over the snapshot
    states (the same FP32 values the snapshots hold) and the final largest plastic
    strain: equal to the snapshot path up to the FP32 norm's rounding, and exactly."""
    pytest.importorskip("torch")
    from cppimpact_gb300 import surrogate as sg
    cfg = sg.Config(n_cube=4, steps=400, every=50)
    params = sg.sample_params(6, np.random.default_rng(11))
    snaps, peak_ep, _ = sg.generate(params, cfg)
    ref = sg.peak_disp(snaps).cpu().numpy().astype(np.float64)
    pd, pe, ms = sg.fallback_runs(params, cfg)
    assert ms > 0 and ref.min() > 0
    assert np.abs(pd - ref).max() <= 1e-6 * ref.max()
    assert np.array_equal(pe.astype(np.float32), peak_ep.astype(np.float32))


def test_small_surrogate_end_to_end(cilib):
    pytest.importorskip("torch")
    from cppimpact_gb300 import surrogate as sg
    cfg = sg.Config(n_cube=4, steps=400, every=50, rank=8, hidden=64, n_train=128, n_test=16,
                    epochs=300, batch=32, ensemble=2)
    rng = np.random.default_rng(cfg.seed)
    ptr, pte = sg.sample_params(cfg.n_train, rng), sg.sample_params(cfg.n_test, rng)
    s_tr, _, _ = sg.generate(ptr, cfg)
    s_te, _, _ = sg.generate(pte, cfg)
    sur = sg.Surrogate(cfg)
    sur.fit(ptr, s_tr)
    assert sur.pod_error < 0.05
    truth = sg.peak_disp(s_te).cpu().numpy()
    mean, spread = sur.predict(pte)
    err = np.abs(mean.cpu().numpy() - truth) / truth
    assert np.all(np.isfinite(err)) and np.median(err) < 0.2


def test_small_study_audit_and_fallback(cilib):
    """The sweep driver on a small case: every flagged or audited query carries the
    solver's answer, the rest the ensemble's; timings and runs/hour are reported."""
    pytest.importorskip("torch")
    from cppimpact_gb300 import surrogate as sg
    cfg = sg.Config(n_cube=4, steps=400, every=50, rank=8, hidden=64, n_train=96, n_test=40,
                    epochs=120, batch=32, ensemble=2, audit_fraction=0.1)
    r = sg.study(cfg, plain_sample=2)
    a = r["audit"]
    assert a["audited"] == 4 or a["audited"] == 40 - a["flagged_by_spread"]
    assert a["rerun"] == a["flagged_by_spread"] + a["audited"]
    am = {row["queries"]: row for row in r["amortised"]}
    assert am[40]["runs_per_hour"] < am[1_000_000]["runs_per_hour"]
    assert r["errors"]["final_peak_disp"]["max"] <= r["errors"]["surrogate_only_peak_disp"]["max"] + 1e-12
    rph = r["runs_per_hour"]
    assert rph["surrogate"] > 0 and rph["plain_gpu_solver"] > 0 and rph["batched_solver"] > 0
    assert r["gemm"]["pod"]["tflops"] > 0 and r["gemm"]["square"]["tflops"] > 0


def test_network_beats_the_method_without_it(cilib):
    """What the trained network gains: on held-out parameter sets its peak-displacement
    error is well below that of the same pipeline without the network (inverse-distance
    interpolation of the training runs' modal trajectories, Surrogate.predict_idw)."""
    pytest.importorskip("torch")
    from cppimpact_gb300 import surrogate as sg
    cfg = sg.Config(n_cube=6, steps=800, every=50, rank=16, hidden=128, n_train=512,
                    n_test=128, epochs=400, batch=64, ensemble=2)
    rng = np.random.default_rng(cfg.seed)
    ptr, pte = sg.sample_params(cfg.n_train, rng), sg.sample_params(cfg.n_test, rng)
    s_tr, ep_tr, _ = sg.generate(ptr, cfg)
    s_te, _, _ = sg.generate(pte, cfg)
    truth = sg.peak_disp(s_te).cpu().numpy()
    sur = sg.Surrogate(cfg)
    sur.fit(ptr, s_tr, ep_tr)
    mean, _ = sur.predict(pte)
    idw, _ = sur.predict_idw(pte)
    e_net = np.abs(mean.cpu().numpy() - truth) / truth
    e_idw = np.abs(idw.cpu().numpy() - truth) / truth
    assert np.median(e_net) < 0.5 * np.median(e_idw)
    assert np.quantile(e_net, 0.95) < np.quantile(e_idw, 0.95)


def test_concurrent_member_training_is_bitwise_sequential(cilib):
    """Ensemble members trained at the same time on their own streams (as Surrogate.fit
    does) end with the same parameters as members trained one after the other; the
    split-K products of their backward pass use per-stream workspaces."""
    torch = pytest.importorskip("torch")
    from cppimpact_gb300 import surrogate as sg
    rng = np.random.default_rng(7)
    X = torch.tensor(rng.uniform(-1, 1, (1024, 4)).astype(np.float32), device="cuda")
    T = torch.tensor(0.3 * rng.standard_normal((1024, 1280)).astype(np.float32), device="cuda")
    cfg = sg.Config(epochs=12, batch=256)
    sur = sg.Surrogate.__new__(sg.Surrogate)
    sur.cfg = cfg
    seq = [sg.MLP(4, 256, 1280, 11 + j) for j in range(3)]
    for j, net in enumerate(seq):
        sur._train(net, X, T, 5 + j)
    par = [sg.MLP(4, 256, 1280, 11 + j) for j in range(3)]
    sur._train_concurrently([(net, X, T, 5 + j) for j, net in enumerate(par)])
    torch.cuda.synchronize()
    for a, b in zip(seq, par):
        assert np.array_equal(a.params(), b.params())
