"""ci_strain_energy_noalloc, the allocation-free variant of ci_strain_energy.

Callers that cannot allocate device memory (a host program that owns all GPU memory
through its own pool, a plug-in inside such a program, a time-critical loop that
must not pay for cudaMalloc) pass their own device buffers; the library uses only a
scratch array compiled into it.  This test checks, through the C ABI, that two calls
in a row give the strain energy and volume of the existing entry point within the
tolerance of the other strain-energy tests, and that oversize meshes are refused.
It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

from cppimpact_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

E, NU = 68.9e9, 0.33


@pytest.mark.parametrize("order,n,case", [(1, 4, 0), (2, 3, 1)])
def test_noalloc_matches_strain_energy(cilib, order, n, case):
    torch = pytest.importorskip("torch")
    m = mg.cube(n, order)
    g = m.xloc[:, 0] if case == 0 else 0.5 * m.xloc[:, 0] ** 2
    u = np.stack([0.01 * g, -0.01 * NU * g, -0.01 * NU * g], axis=1)
    s = cilib.Solver(m.xloc, m.conn, E=E, nu=NU, rho=2700.0, mode=cilib.MODE_REFCOMPAT)
    W_ref, V_ref = s.strain_energy(u)
    s.close()

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    dx = torch.tensor(m.xloc.reshape(-1), dtype=torch.float64, device=dev)
    dc = torch.tensor(m.conn.reshape(-1), dtype=torch.int32, device=dev)
    du = torch.tensor(u.reshape(-1), dtype=torch.float64, device=dev)
    out = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    L = cilib.lib()
    for _ in range(2):
        out.fill_(-1.0)
        rc = L.ci_strain_energy_noalloc(dx.data_ptr(), dc.data_ptr(), m.num_nodes,
                                        m.num_elements, m.npe, du.data_ptr(), E, NU,
                                        out.data_ptr(), C.c_void_p(stream))
        assert rc == 0, L.ci_last_error()
        torch.cuda.synchronize(dev)
        W, V = out.cpu().tolist()
        assert W == pytest.approx(W_ref, rel=1e-5)
        assert V == pytest.approx(V_ref, rel=1e-5)


def test_noalloc_rejects_oversize(cilib):
    L = cilib.lib()
    limit = 1 << 22
    rc = L.ci_strain_energy_noalloc(C.c_void_p(16), C.c_void_p(16), 4, limit + 1, 4,
                                    C.c_void_p(16), E, NU, C.c_void_p(16), None)
    assert rc == -8
    assert b"CI_NOALLOC_MAX_ELEMENTS" in L.ci_last_error()


def _call(cilib, torch, xloc, conn, u):
    """One call through the C ABI on device buffers made from host arrays; returns
    (energy, volume)."""
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    dx = torch.tensor(np.ascontiguousarray(xloc).reshape(-1), dtype=torch.float64, device=dev)
    dc = torch.tensor(np.ascontiguousarray(conn).reshape(-1), dtype=torch.int32, device=dev)
    du = torch.tensor(np.ascontiguousarray(u).reshape(-1), dtype=torch.float64, device=dev)
    out = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
    L = cilib.lib()
    rc = L.ci_strain_energy_noalloc(dx.data_ptr(), dc.data_ptr(), xloc.shape[0], conn.shape[0],
                                    conn.shape[1], du.data_ptr(), E, NU, out.data_ptr(),
                                    C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    assert rc == 0, L.ci_last_error()
    torch.cuda.synchronize(dev)
    return out.cpu().tolist()


def test_noalloc_status_word_is_cleared_between_calls(cilib):
    """The status word is the one piece of state the shared scratch carries from call to
    call.  An inverted element makes that call's energy NaN; an out-of-range node index
    (caught in the kernel: the element's loads are skipped) makes both outputs NaN; the
    next call on a valid mesh must again match ci_strain_energy."""
    torch = pytest.importorskip("torch")
    m = mg.cube(3, 1)
    g = m.xloc[:, 0]
    u = np.stack([0.01 * g, -0.01 * NU * g, -0.01 * NU * g], axis=1)
    s = cilib.Solver(m.xloc, m.conn, E=E, nu=NU, rho=2700.0, mode=cilib.MODE_REFCOMPAT)
    W_ref, V_ref = s.strain_energy(u)
    s.close()

    inverted = m.conn.copy()
    inverted[5, [1, 2]] = inverted[5, [2, 1]]  # swapping two corners makes det J < 0
    W, V = _call(cilib, torch, m.xloc, inverted, u)
    assert np.isnan(W) and np.isfinite(V)
    W, V = _call(cilib, torch, m.xloc, m.conn, u)
    assert W == pytest.approx(W_ref, rel=1e-5) and V == pytest.approx(V_ref, rel=1e-5)

    for bad in (m.num_nodes, -1):
        wrong = m.conn.copy()
        wrong[7, 3] = bad
        W, V = _call(cilib, torch, m.xloc, wrong, u)
        assert np.isnan(W) and np.isnan(V)
        W, V = _call(cilib, torch, m.xloc, m.conn, u)
        assert W == pytest.approx(W_ref, rel=1e-5) and V == pytest.approx(V_ref, rel=1e-5)
