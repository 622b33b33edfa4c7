"""The BF16 tcgen05 GEMM of the surrogate against a float64 product of the same
BF16-rounded operands (FP32 accumulation: relative error <= 1e-3 here)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gemm(cilib, torch, A, B, transA, transB, bias=None, act=0, beta=0.0, C0=None):
    dev = torch.device("cuda:0")
    a = torch.tensor(A, dtype=torch.float32, device=dev).to(torch.bfloat16).contiguous()
    b = torch.tensor(B, dtype=torch.float32, device=dev).to(torch.bfloat16).contiguous()
    M = A.shape[1] if transA else A.shape[0]
    K = A.shape[0] if transA else A.shape[1]
    N = B.shape[0] if transB else B.shape[1]
    c = (torch.zeros((M, N), dtype=torch.float32, device=dev) if C0 is None
         else torch.tensor(C0, dtype=torch.float32, device=dev))
    cb = torch.zeros((M, N), dtype=torch.bfloat16, device=dev)
    bb = None if bias is None else torch.tensor(bias, dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    rc = cilib.lib().ci_gemm_bf16(a.data_ptr(), A.shape[1], transA, b.data_ptr(), B.shape[1],
                                  transB, c.data_ptr(), N, cb.data_ptr(), M, N, K, 1.0, beta,
                                  None if bb is None else bb.data_ptr(), act, err.data_ptr(),
                                  C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    assert rc == 0, cilib.lib().ci_last_error()
    torch.cuda.synchronize(dev)
    assert int(err.item()) == 0
    Ar = a.float().cpu().numpy().astype(np.float64)
    Br = b.float().cpu().numpy().astype(np.float64)
    ref = (Ar.T if transA else Ar) @ (Br.T if transB else Br)
    if C0 is not None:
        ref = ref + beta * C0
    if bias is not None:
        ref = ref + bias[None, :]
    if act == 1:
        ref = np.tanh(ref)
    return c.cpu().numpy(), ref, cb.float().cpu().numpy()


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (128, 128, 128), (200, 100, 130), (64, 300, 40),
                                   (1000, 96, 700)])
@pytest.mark.parametrize("tA,tB", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_gemm_bf16(cilib, M, N, K, tA, tB):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(M * 7 + N * 3 + K + 10 * tA + 20 * tB)
    A = rng.standard_normal((K, M) if tA else (M, K))
    B = rng.standard_normal((N, K) if tB else (K, N))
    c, ref, _ = _gemm(cilib, torch, A, B, tA, tB)
    assert np.linalg.norm(c - ref) <= 1e-3 * np.linalg.norm(ref)


@pytest.mark.parametrize("M,N,K", [(256, 1, 64), (64, 1, 256), (64, 64, 256), (256, 64, 1),
                                   (33, 17, 5)])
@pytest.mark.parametrize("tA,tB", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_gemm_bf16_small_products(cilib, M, N, K, tA, tB):
    """Products of at most 2^20 multiply-adds outside the TMA shape (the plastic-strain
    network's layers) run on the CUDA cores: same operands, accumulation and epilogue
    (beta C added, bias, tanh, BF16 copy of C); two calls give identical bits."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(M + 5 * N + 11 * K + tA + 2 * tB)
    A = rng.standard_normal((K, M) if tA else (M, K))
    B = rng.standard_normal((N, K) if tB else (K, N))
    bias = rng.standard_normal(N)
    c, ref, cb = _gemm(cilib, torch, A, B, tA, tB, bias=bias, act=1)
    assert np.abs(c - ref).max() <= 1e-2 * max(1.0, np.abs(ref).max())
    c2, _, _ = _gemm(cilib, torch, A, B, tA, tB, bias=bias, act=1)
    assert np.array_equal(c, c2)
    # beta != 0 reads C before writing it; the BF16 copy is C rounded to nearest
    # (relative error at most 2^-8 for a 8-bit significand)
    C0 = rng.standard_normal((M, N))
    for act in (0, 1):
        c, ref, cb = _gemm(cilib, torch, A, B, tA, tB, bias=bias, act=act, beta=0.75, C0=C0)
        assert np.abs(c - ref).max() <= 1e-2 * max(1.0, np.abs(ref).max())
        assert np.all(np.abs(cb - c) <= 2.0 ** -8 * np.abs(c))


@pytest.mark.parametrize("M,N,K", [(64, 64, 20000), (130, 5, 9000), (8, 200, 4096)])
@pytest.mark.parametrize("tA,tB", [(1, 0), (0, 1)])
def test_gemm_bf16_split_k(cilib, M, N, K, tA, tB):
    """Few output tiles and a long K (the POD's Gram and projection products): the
    split-K path with its fixed-order reduction; two calls give identical bits."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(M + N + K + tA)
    A = rng.standard_normal((K, M) if tA else (M, K))
    B = rng.standard_normal((N, K) if tB else (K, N))
    bias = rng.standard_normal(N)
    c, ref, _ = _gemm(cilib, torch, A, B, tA, tB, bias=bias)
    assert np.linalg.norm(c - ref) <= 1e-3 * np.linalg.norm(ref)
    c2, _, _ = _gemm(cilib, torch, A, B, tA, tB, bias=bias)
    assert np.array_equal(c, c2)


def test_gemm_bias_tanh_beta(cilib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    A, B = rng.standard_normal((300, 40)) * 0.2, rng.standard_normal((40, 256)) * 0.2
    bias = rng.standard_normal(256) * 0.1
    c, ref, cb = _gemm(cilib, torch, A, B, 0, 0, bias=bias, act=1)
    assert np.abs(c - ref).max() < 2e-3
    assert np.abs(cb - c).max() < 1e-2
    C0 = rng.standard_normal((300, 256))
    c, ref, _ = _gemm(cilib, torch, A, B, 0, 0, beta=0.5, C0=C0)
    assert np.linalg.norm(c - ref) <= 1e-3 * np.linalg.norm(ref)


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 128, 512), (200, 100, 136), (1000, 300, 1000),
                                   (384, 96, 20000), (129, 16, 64), (640, 256, 4096)])
def test_gemm_bf16_nt_pipelined(cilib, M, N, K):
    """A B^T with K-major operands: the TMA + tcgen05 pipelined path (ragged tiles are
    zero-filled by TMA; long K is split with a fixed-order reduction)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(M + 3 * N + 7 * K)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((N, K))
    bias = rng.standard_normal(N)
    c, ref, cb = _gemm(cilib, torch, A, B, 0, 1, bias=bias)
    assert np.linalg.norm(c - ref) <= 1e-3 * np.linalg.norm(ref)
    c2, _, _ = _gemm(cilib, torch, A, B, 0, 1, bias=bias)
    assert np.array_equal(c, c2)
    c3, ref3, _ = _gemm(cilib, torch, A * 0.1, B * 0.1, 0, 1, act=1, beta=0.5, C0=rng.standard_normal((M, N)))
    assert np.abs(c3 - ref3).max() < 5e-3


@pytest.mark.parametrize("M,N,K,act", [(4173, 1100, 160, 0), (16389, 640, 128, 1), (300, 2000, 1000, 0)])
def test_gemm_tma_persistent_many_tiles(cilib, M, N, K, act):
    """A B^T with K-major operands on the persistent kernel: more output tiles than SMs
    (each CTA walks several tiles through the two TMEM accumulators), ragged M, N and K,
    beta C, bias and tanh in the epilogue; two calls give identical bits."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)) * 0.3
    B = rng.standard_normal((N, K)) * 0.3
    bias = rng.standard_normal(N) * 0.1
    C0 = rng.standard_normal((M, N))
    c, ref, cb = _gemm(cilib, torch, A, B, 0, 1, bias=bias, act=act, beta=0.5, C0=C0)
    assert np.linalg.norm(c - ref) <= 1e-3 * np.linalg.norm(ref)
    assert np.all(np.abs(cb - c) <= 2.0 ** -8 * np.abs(c))
    c2, _, _ = _gemm(cilib, torch, A, B, 0, 1, bias=bias, act=act, beta=0.5, C0=C0)
    assert np.array_equal(c, c2)


def test_gemm_split_k_on_many_streams(cilib):
    """Split-K products on 40 streams in turn (more than the 32 workspaces kept per
    device, so older streams' workspaces are freed and rebuilt) all give the result of
    a single-stream call, bit for bit."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(17)
    A = rng.standard_normal((64, 20000))
    B = rng.standard_normal((20000, 64))
    ref, _, _ = _gemm(cilib, torch, A, B, 0, 0)
    # torch hands out streams from pools of 32 per priority: 20 of each of two
    # priorities are 40 distinct streams
    streams = [torch.cuda.Stream(priority=p) for p in (0, -1) for _ in range(20)]
    assert len({st.cuda_stream for st in streams}) == 40
    for _ in range(2):
        for st in streams:
            with torch.cuda.stream(st):
                c, _, _ = _gemm(cilib, torch, A, B, 0, 0)
            assert np.array_equal(c, ref)
