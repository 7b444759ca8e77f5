"""Failure detection on a healthy device, with no kernel made to fault.

Every device and pinned-host allocation of the library can be made to fail in turn
(dpf_debug_fail_alloc): each must surface as DPF_OOM, leave no allocation behind and
leave the library, and a handle that already exists, usable. The bounded wait of the
staging kernels is made to expire on a barrier that nothing arrives on
(dpf_debug_expired_wait): it must end by its bound with DPF_TIMEOUT and a usable device.
"""
import ctypes

import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu

DPF_OOM, DPF_TIMEOUT = 4, 9


def _stats(lib):
    made, live = ctypes.c_int64(), ctypes.c_int64()
    lib.dpf_debug_alloc_stats(ctypes.byref(made), ctypes.byref(live))
    return made.value, live.value


def _case(pkg):
    shapes = [(24, 20, 6), (9, 9, 9)]
    mins = [(0.0, 0.0, 0.0)] * 2
    maxs = [tuple(float(n - 1) for n in ns) for ns in shapes]
    dn = [np.array([int(np.prod(ns)) - 1]) for ns in shapes]
    N = sum(int(np.prod(ns)) for ns in shapes)
    rng = np.random.default_rng(3)
    logK = -9.0 + 0.5 * rng.standard_normal(N)
    Qs = np.zeros(N)
    Qs[0] = 1e-4
    Qs[int(np.prod(shapes[0]))] = 1e-4
    obs = [np.array([5, 40, 100]), np.array([3, 77])]
    return shapes, mins, maxs, dn, logK, np.zeros(N), Qs, obs


@pytest.fixture
def lib(gpu_lib):
    L = gpu_lib.load()
    L.dpf_debug_fail_alloc(-1)
    yield L
    L.dpf_debug_fail_alloc(-1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_each_create_allocation_failure(gpu_lib, lib, precision):
    pkg = gpu_lib
    shapes, mins, maxs, dn, *_ = _case(pkg)
    make = lambda: pkg.GroundwaterBatch(shapes, mins, maxs, dn, precision=precision)
    m0, live0 = _stats(lib)
    make().close()
    m1, live1 = _stats(lib)
    assert live1 == live0
    count = m1 - m0
    assert count > 10
    for k in range(count):
        lib.dpf_debug_fail_alloc(k)
        with pytest.raises(pkg.DPFError) as ei:
            make()
        assert ei.value.code == DPF_OOM, (k, str(ei.value))
        assert _stats(lib)[1] == live0, k
    lib.dpf_debug_fail_alloc(-1)
    B = make()
    B.close()
    assert _stats(lib)[1] == live0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_each_solve_allocation_failure(gpu_lib, lib, precision):
    """A solve whose k-th allocation fails reports DPF_OOM; the next solve on the same
    handle gives the answer of an undisturbed one."""
    pkg = gpu_lib
    shapes, mins, maxs, dn, logK, dh, Qs, obs = _case(pkg)
    make = lambda: pkg.GroundwaterBatch(shapes, mins, maxs, dn, precision=precision, reltol=1e-11)
    live0 = _stats(lib)[1]
    B = make()
    m0 = _stats(lib)[0]
    h_ref, g_ref = B.solve_grad_logk(logK, dh, Qs, obs)
    count = _stats(lib)[0] - m0
    B.close()
    assert _stats(lib)[1] == live0
    assert count >= 1
    for k in range(count):
        B = make()
        lib.dpf_debug_fail_alloc(k)
        with pytest.raises(pkg.DPFError) as ei:
            B.solve_grad_logk(logK, dh, Qs, obs)
        assert ei.value.code == DPF_OOM, (k, str(ei.value))
        lib.dpf_debug_fail_alloc(-1)
        h, g = B.solve_grad_logk(logK, dh, Qs, obs)
        assert rel(h, h_ref) < 1e-9, k
        assert rel(g, g_ref) < 1e-7, k
        B.close()
        assert _stats(lib)[1] == live0, k


def test_general_path_allocation_failure(gpu_lib, lib):
    """The CSR path (a graph that is not a regular grid): every allocation of create and
    of the first forward solve."""
    pkg = gpu_lib
    _, nb, aol, _ = pkg.regulargrid3d((0.0, 0.0, 0.0), (9.0, 7.0, 3.0), (10, 8, 4))
    nb = np.concatenate([nb, nb[::5]])           # duplicated faces: no longer a regular grid
    aol = np.concatenate([aol, 0.5 * aol[::5]])
    N = 320
    dn = [N - 1]
    Ks = np.exp(np.random.default_rng(5).normal(-9, 0.5, len(nb)))
    Qs = np.zeros(N)
    Qs[0] = 1e-4
    live0 = _stats(lib)[1]
    m0 = _stats(lib)[0]
    P = pkg.GroundwaterProblem(nb, aol, dn, N, reltol=1e-11)
    assert not P.structured
    m1 = _stats(lib)[0]
    h_ref = P.forward(Ks, np.zeros(N), Qs)
    m2 = _stats(lib)[0]
    P.close()
    assert _stats(lib)[1] == live0
    for k in range(m1 - m0):
        lib.dpf_debug_fail_alloc(k)
        with pytest.raises(pkg.DPFError) as ei:
            pkg.GroundwaterProblem(nb, aol, dn, N, reltol=1e-11)
        assert ei.value.code == DPF_OOM, (k, str(ei.value))
        assert _stats(lib)[1] == live0, k
    for k in range(m2 - m1):
        P = pkg.GroundwaterProblem(nb, aol, dn, N, reltol=1e-11)
        lib.dpf_debug_fail_alloc(k)
        with pytest.raises(pkg.DPFError) as ei:
            P.forward(Ks, np.zeros(N), Qs)
        assert ei.value.code == DPF_OOM, (k, str(ei.value))
        lib.dpf_debug_fail_alloc(-1)
        assert rel(P.forward(Ks, np.zeros(N), Qs), h_ref) < 1e-9, k
        P.close()
        assert _stats(lib)[1] == live0, k


def test_expired_wait_reports_timeout(gpu_lib, lib):
    pkg = gpu_lib
    ms = ctypes.c_double(-1.0)
    rc = lib.dpf_debug_expired_wait(ctypes.byref(ms))
    assert rc == DPF_TIMEOUT, pkg._lib.STATUS_NAMES.get(rc, rc)
    assert 900.0 <= ms.value <= 1100.0           # the wait is bounded by one second of device time
    # the device and the library stay usable
    shapes, mins, maxs, dn, logK, dh, Qs, obs = _case(pkg)
    B = pkg.GroundwaterBatch(shapes, mins, maxs, dn, precision="mixed", reltol=1e-11)
    h, g = B.solve_grad_logk(logK, dh, Qs, obs)
    assert np.all(np.isfinite(h)) and np.all(np.isfinite(g))
    B.close()
