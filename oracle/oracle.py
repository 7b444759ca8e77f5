"""ctypes binding of the CPU oracle (gw_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline leg of bench.py, never by the shipped library. See gw_oracle.c for
what it restates and for its parity status.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gw_oracle.c")
LIB = os.path.join(HERE, "_build", "libgw_oracle.so")

_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force=False):
    """Compile gw_oracle.c into oracle/_build/libgw_oracle.so (gcc, OpenMP)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", tmp, SRC, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int64, ctypes.c_int64, _i64p, _i64p, _f64p, ctypes.c_int64, _i64p]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_nfree.restype = ctypes.c_int64
        L.orc_nfree.argtypes = [ctypes.c_void_p]
        L.orc_nnz.restype = ctypes.c_int64
        L.orc_nnz.argtypes = [ctypes.c_void_p]
        L.orc_levels.argtypes = [ctypes.c_void_p]
        L.orc_set_amg.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int64, ctypes.c_int]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_assemble.argtypes = [ctypes.c_void_p, _f64p, _f64p, _f64p, _i64p, _i32p, _f64p, _f64p]
        L.orc_steady_solve.argtypes = [ctypes.c_void_p, _f64p, _f64p, _f64p, ctypes.c_double, ctypes.c_int,
                                       _f64p, _ip, _f64p]
        L.orc_steady_adjoint.argtypes = [ctypes.c_void_p, _f64p, _f64p, ctypes.c_double, ctypes.c_int,
                                         _f64p, _f64p, _f64p, _ip, _f64p]
        L.orc_logk_to_faces.argtypes = [ctypes.c_int64, _i64p, _i64p, _f64p, ctypes.c_int, _f64p]
        L.orc_logk_to_faces_vjp.argtypes = [ctypes.c_int64, ctypes.c_int64, _i64p, _i64p, _f64p, ctypes.c_int,
                                            _f64p, _f64p]
        L.orc_transient_forward.argtypes = [ctypes.c_void_p, _f64p, _f64p, _f64p, _f64p, _f64p, ctypes.c_double,
                                            ctypes.c_int, _f64p, ctypes.c_double, ctypes.c_int, _f64p, _f64p, _ip]
        L.orc_transient_adjoint.argtypes = [ctypes.c_void_p, _f64p, ctypes.c_int, _f64p, ctypes.c_int64, _i64p,
                                            _f64p, _f64p, ctypes.c_double, ctypes.c_int, _f64p, _f64p, _f64p,
                                            _f64p, _ip]
        _lib = L
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def _p(a, t=_f64p):
    return None if a is None else a.ctypes.data_as(t)


def set_threads(n):
    lib().orc_set_threads(int(n))


MEAN_GEOMETRIC = 0
MEAN_HARMONIC = 1


def logk_to_faces(neighbors, logK, kind=MEAN_GEOMETRIC):
    nb = _i(neighbors)
    a, b = _i(nb[:, 0]), _i(nb[:, 1])
    logK = _f(logK)
    out = np.empty(len(a))
    lib().orc_logk_to_faces(len(a), _p(a, _i64p), _p(b, _i64p), _p(logK), int(kind), _p(out))
    return out


def logk_to_faces_vjp(neighbors, logK, dKs, kind=MEAN_GEOMETRIC):
    nb = _i(neighbors)
    a, b = _i(nb[:, 0]), _i(nb[:, 1])
    logK = _f(logK)
    dKs = _f(dKs)
    out = np.empty(len(logK))
    lib().orc_logk_to_faces_vjp(len(logK), len(a), _p(a, _i64p), _p(b, _i64p), _p(logK), int(kind), _p(dKs), _p(out))
    return out


class OracleError(RuntimeError):
    pass


class Problem:
    """Topology (faces, areas over lengths, Dirichlet set) of one groundwater problem."""

    def __init__(self, N, neighbors, areasoverlengths, dirichletnodes):
        L = lib()
        nb = _i(neighbors).reshape(-1, 2)
        self.N = int(N)
        self.F = nb.shape[0]
        self.a, self.b = _i(nb[:, 0]), _i(nb[:, 1])
        self.aol = _f(areasoverlengths)[: self.F].copy()
        self.dn = _i(dirichletnodes)
        self._h = L.orc_create(self.N, self.F, _p(self.a, _i64p), _p(self.b, _i64p), _p(self.aol),
                               len(self.dn), _p(self.dn, _i64p))
        if not self._h:
            raise OracleError("invalid topology")
        self.nfree = L.orc_nfree(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def set_amg(self, theta=0.25, max_coarse=500, max_levels=30):
        lib().orc_set_amg(self._h, theta, max_coarse, max_levels)

    def assemble(self, Ks, dirichleths, Qs):
        """Free-node operator (scipy CSR) and right-hand side, S = V = 1."""
        import scipy.sparse as sp
        L = lib()
        L.orc_assemble(self._h, _p(_f(Ks)), _p(_f(dirichleths)), _p(_f(Qs)), None, None, None, None)
        nnz = L.orc_nnz(self._h)
        rp = np.empty(self.nfree + 1, np.int64)
        ci = np.empty(nnz, np.int32)
        v = np.empty(nnz)
        b = np.empty(self.nfree)
        L.orc_assemble(self._h, _p(_f(Ks)), _p(_f(dirichleths)), _p(_f(Qs)), _p(rp, _i64p), _p(ci, _i32p),
                       _p(v), _p(b))
        return sp.csr_matrix((v, ci, rp), shape=(self.nfree, self.nfree)), b

    def steady(self, Ks, dirichleths, Qs, reltol=1e-14, maxiter=2000):
        h = np.empty(self.N)
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0)
        rc = lib().orc_steady_solve(self._h, _p(_f(Ks)), _p(_f(dirichleths)), _p(_f(Qs)), reltol, maxiter, _p(h),
                                    ctypes.byref(it), ctypes.byref(rr))
        self.last = {"status": rc, "iters": it.value, "relres": rr.value, "levels": lib().orc_levels(self._h)}
        if rc not in (0, 2):
            raise OracleError("oracle steady solve failed, status %d" % rc)
        return h

    def adjoint(self, dirichleths, delta, reltol=1e-14, maxiter=2000):
        dKs = np.empty(self.F)
        ddh = np.empty(self.N)
        dQs = np.empty(self.N)
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0)
        rc = lib().orc_steady_adjoint(self._h, _p(_f(dirichleths)), _p(_f(delta)), reltol, maxiter, _p(dKs),
                                      _p(ddh), _p(dQs), ctypes.byref(it), ctypes.byref(rr))
        self.last_adj = {"status": rc, "iters": it.value, "relres": rr.value}
        if rc not in (0, 2):
            raise OracleError("oracle adjoint failed, status %d" % rc)
        return dKs, ddh, dQs

    def transient(self, Ks, dirichleths, Qs, Ss, V, dt, nsteps, h0free, reltol=1e-14, maxiter=2000):
        states = np.empty((nsteps, self.nfree))
        hT = np.empty(self.nfree)
        it = ctypes.c_int(0)
        rc = lib().orc_transient_forward(self._h, _p(_f(Ks)), _p(_f(dirichleths)), _p(_f(Qs)), _p(_f(Ss)),
                                         _p(_f(V)), float(dt), int(nsteps), _p(_f(h0free)), reltol, maxiter,
                                         _p(states), _p(hT), ctypes.byref(it))
        self.last_tr = {"status": rc, "iters": it.value}
        if rc not in (0, 2):
            raise OracleError("oracle transient failed, status %d" % rc)
        self._states = states
        return states

    def transient_adjoint(self, dirichleths, obs, w=None, gT=None, reltol=1e-14, maxiter=2000):
        nsteps = self._states.shape[0]
        obs = _i(obs)
        w = np.ones(len(obs)) if w is None else _f(w)
        dKs = np.empty(self.F)
        ddh = np.empty(self.N)
        dQs = np.empty(self.N)
        dh0 = np.empty(self.nfree)
        it = ctypes.c_int(0)
        rc = lib().orc_transient_adjoint(self._h, _p(_f(dirichleths)), nsteps, _p(self._states), len(obs),
                                         _p(obs, _i64p), _p(w), _p(None if gT is None else _f(gT)), reltol,
                                         maxiter, _p(dKs), _p(ddh), _p(dQs), _p(dh0), ctypes.byref(it))
        if rc not in (0, 2):
            raise OracleError("oracle transient adjoint failed, status %d" % rc)
        return dKs, ddh, dQs, dh0
