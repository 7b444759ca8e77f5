"""GB300-native groundwater solve with DPFEHM.jl's interface.

Host-side mirror of the reference's groundwater API (DPFEHM.jl
src/groundwater.jl:75-109, src/utilities.jl:10-40, src/grid.jl) on top of the
C ABI of libdpfehm_gpu.so. Every solve, assembly and gradient runs in the
library's sm_103a kernels; this module only marshals arrays. Indices are 0-based
(the reference is 1-based Julia).

    h = groundwater_steadystate(Ks, neighbors, areasoverlengths, dirichletnodes, dirichleths, Qs)
    h, pullback = rrule_groundwater_steadystate(Ks, neighbors, areasoverlengths, dirichletnodes, dirichleths, Qs)
    _, dKs, _, _, _, ddirichleths, dQs = pullback(delta)

Arrays may be numpy arrays (host) or torch CUDA tensors (used in place on the
device); outputs follow the type of ``Ks`` / ``logK``.
"""
import ctypes
import hashlib
import warnings
from collections import OrderedDict

import numpy as np

from . import _lib
from . import fields, grid
from ._lib import (MEAN_GEOMETRIC, MEAN_HARMONIC, PREC_FP64, PREC_MIXED, SOLVER_CG, SOLVER_CHOLESKY,
                   default_options, load)
from .grid import addboundaryconditions, getfreenodes, load_uge, regulargrid1d, regulargrid2d, regulargrid3d

__all__ = [
    "groundwater_steadystate", "rrule_groundwater_steadystate", "logKs2Ks_neighbors", "GroundwaterProblem",
    "GroundwaterBatch", "DPFError", "NoTangent", "getfreenodes", "addboundaryconditions", "regulargrid1d",
    "regulargrid2d", "regulargrid3d", "load_uge", "fields", "grid", "load", "default_options", "MEAN_GEOMETRIC",
    "MEAN_HARMONIC", "PREC_FP64", "PREC_MIXED", "SOLVER_CG", "SOLVER_CHOLESKY", "solvepressure", "rrule_solvepressure", "amg_solver",
    "cholesky_solver", "autotune_batch", "richards_steadystate", "rrule_richards_steadystate",
]


class DPFError(RuntimeError):
    """A non-OK dpf_status; ``code`` holds the status, the message dpf_last_error()."""

    def __init__(self, code, msg):
        super().__init__("%s: %s" % (_lib.STATUS_NAMES.get(code, str(code)), msg))
        self.code = code


class _NoTangent:
    def __repr__(self):
        return "NoTangent()"


NoTangent = _NoTangent()

_MEANS = {"geometric": MEAN_GEOMETRIC, "harmonic": MEAN_HARMONIC, MEAN_GEOMETRIC: MEAN_GEOMETRIC,
          MEAN_HARMONIC: MEAN_HARMONIC}
_PRECS = {"fp64": PREC_FP64, "mixed": PREC_MIXED, PREC_FP64: PREC_FP64, PREC_MIXED: PREC_MIXED}
_SOLVERS = {"cg": SOLVER_CG, "cholesky": SOLVER_CHOLESKY}


def _is_torch(x):
    return type(x).__module__.startswith("torch")


class _Buf:
    """A contiguous float64/int64 buffer (numpy host array or torch CUDA tensor) and its address."""

    def __init__(self, x, dtype=np.float64, n=None):
        if _is_torch(x):
            import torch
            tdt = torch.float64 if dtype == np.float64 else torch.int64
            t = x.detach()
            if t.dtype != tdt:
                t = t.to(tdt)
            t = t.contiguous()
            self.obj, self.ptr, self.device = t, t.data_ptr(), t.is_cuda
        else:
            a = np.ascontiguousarray(x, dtype=dtype)
            self.obj, self.ptr, self.device = a, a.ctypes.data, False
        self.size = self.obj.numel() if _is_torch(self.obj) else self.obj.size
        if n is not None and self.size != n:
            raise ValueError("expected %d entries, got %d" % (n, self.size))


def _out(like, n, dtype=np.float64):
    """Output buffer on the same side (host/device) as `like`."""
    if like is not None and _is_torch(like.obj) and like.device:
        import torch
        t = torch.empty(n, dtype=torch.float64, device=like.obj.device)
        return t, t.data_ptr()
    a = np.empty(n, dtype=dtype)
    return a, a.ctypes.data


def _out_into(given, like, n):
    """`given` (a caller's float64 buffer of n entries: numpy array or torch tensor, e.g. in
    page-locked host memory) as an output buffer, or a new one on the side of `like`."""
    if given is None:
        return _out(like, n)
    b = _Buf(given, n=n)
    if b.obj is not given and not (_is_torch(given) and b.obj.data_ptr() == given.data_ptr()):
        raise ValueError("output buffers must be contiguous float64")
    return given, b.ptr


def _check(lib, h, rc, allow_not_converged=True, what="groundwater solve"):
    if rc == _lib.DPF_OK:
        return
    msg = lib.dpf_last_error(h)
    msg = msg.decode() if msg else ""
    if rc == _lib.DPF_NOT_CONVERGED and allow_not_converged:
        warnings.warn("%s did not reach its tolerance: %s" % (what, msg), RuntimeWarning, stacklevel=3)
        return
    raise DPFError(rc, msg)


def _options(reltol=None, maxiter=None, precision=None, **kw):
    o = default_options()
    if reltol is not None:
        o.reltol = float(reltol)
    if maxiter is not None:
        o.maxiter = int(maxiter)
    if precision is not None:
        o.precision = _PRECS[precision]
    if isinstance(kw.get("solver"), str):
        kw = dict(kw, solver=_SOLVERS[kw["solver"]])
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError("unknown solver option %r" % k)
        setattr(o, k, v)
    return o


class GroundwaterProblem:
    """One groundwater topology on the GPU (faces, areas over lengths, Dirichlet set).

    Construct from the reference's arrays (``neighbors`` as an (F, 2) 0-based
    array) or with :meth:`regular3d`. Face lists produced by ``regulargrid3d``
    are recognised and solved matrix-free on the structured path.
    """

    def __init__(self, neighbors=None, areasoverlengths=None, dirichletnodes=(), N=None, volumes=None, _handle=None,
                 general=False, **options):
        self._lib = load()
        if _handle is not None:
            self._h = _handle
        else:
            nb = np.ascontiguousarray(np.asarray(neighbors, dtype=np.int64).reshape(-1, 2))
            F = nb.shape[0]
            if N is None:
                raise ValueError("N (number of cells) is required")
            a = np.ascontiguousarray(nb[:, 0])
            b = np.ascontiguousarray(nb[:, 1])
            aol = np.ascontiguousarray(np.asarray(areasoverlengths, dtype=np.float64)[:F])
            dn = np.ascontiguousarray(np.asarray(dirichletnodes, dtype=np.int64))
            vol = None if volumes is None else np.ascontiguousarray(volumes, dtype=np.float64)
            h = ctypes.c_void_p()
            o = _options(**options)
            create = self._lib.dpf_create_general if general else self._lib.dpf_create
            rc = create(int(N), F, a.ctypes.data, b.ctypes.data, aol.ctypes.data,
                        None if vol is None else vol.ctypes.data, dn.size, dn.ctypes.data, ctypes.byref(o),
                        ctypes.byref(h))
            if rc != _lib.DPF_OK:
                raise DPFError(rc, self._lib.dpf_last_error(None).decode())
            self._h = h
        self._info()

    @classmethod
    def regular3d(cls, mins, maxs, ns, dirichletnodes=(), **options):
        lib = load()
        mn = np.ascontiguousarray(mins, dtype=np.float64)
        mx = np.ascontiguousarray(maxs, dtype=np.float64)
        dn = np.ascontiguousarray(np.asarray(dirichletnodes, dtype=np.int64))
        h = ctypes.c_void_p()
        o = _options(**options)
        rc = lib.dpf_create_regular3d(int(ns[0]), int(ns[1]), int(ns[2]), mn.ctypes.data, mx.ctypes.data, dn.size,
                                      dn.ctypes.data, ctypes.byref(o), ctypes.byref(h))
        if rc != _lib.DPF_OK:
            raise DPFError(rc, lib.dpf_last_error(None).decode())
        return cls(_handle=h)

    def _info(self):
        N, F, nf = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        st, lv = ctypes.c_int(), ctypes.c_int()
        self._lib.dpf_info(self._h, ctypes.byref(N), ctypes.byref(F), ctypes.byref(nf), ctypes.byref(st),
                           ctypes.byref(lv))
        self.N, self.F, self.nfree = N.value, F.value, nf.value
        self.structured, self.levels = bool(st.value), lv.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.dpf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stats(self):
        it, ou, rr = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        self._lib.dpf_last_stats(self._h, ctypes.byref(it), ctypes.byref(ou), ctypes.byref(rr))
        return {"iterations": it.value, "outer": ou.value, "relres": rr.value}

    # ---- diagnostics
    def profile(self, enable=True):
        """Start/stop per-kernel CUDA-event timing on the handle's stream."""
        self._lib.dpf_profile(self._h, 1 if enable else 0)

    def profile_report(self):
        """{kernel name: (launches, total ms, total scheduled cells)} since profile(True)."""
        cap = 256
        names = (ctypes.c_char_p * cap)()
        cnt = (ctypes.c_longlong * cap)()
        ms = (ctypes.c_double * cap)()
        cells = (ctypes.c_longlong * cap)()
        n = self._lib.dpf_profile_report(self._h, cap, names, cnt, ms, cells)
        if n < 0:
            raise DPFError(-n, self._lib.dpf_last_error(self._h).decode())
        return {names[k].decode(): (cnt[k], ms[k], cells[k]) for k in range(min(n, cap))}

    @property
    def launch_count(self):
        return int(self._lib.dpf_launch_count(self._h))

    # ---- Richards (face-list handles: GroundwaterProblem(..., general=True))
    def richards_steady(self, psi0, Ks, dirichletpsis, z, alphas, Ns, Qs, tol=1e-10, maxiter=200):
        """The steady Richards solution psi (N) for the handle's faces (src/richards.jl:148-167);
        z are the cell elevations (the reference's coords[3, :])."""
        p0, K, dp, zz = _Buf(psi0, n=self.N), _Buf(Ks, n=self.F), _Buf(dirichletpsis, n=self.N), _Buf(z, n=self.N)
        al, n_, q = _Buf(alphas, n=self.F), _Buf(Ns, n=self.F), _Buf(Qs, n=self.N)
        psi, pp = _out(p0, self.N)
        _check(self._lib, self._h, self._lib.dpf_richards_steady(self._h, p0.ptr, K.ptr, dp.ptr, zz.ptr, al.ptr, n_.ptr,
                                                                 q.ptr, float(tol), int(maxiter), pp),
               what="Richards solve")
        return psi

    def richards_adjoint(self, delta, tol=1e-10, maxiter=200):
        """(dKs, ddirichletpsis, dalphas, dNs, dQs) of the rrule at the last Richards solve."""
        dl = _Buf(delta, n=self.N)
        dK, dKp = _out(dl, self.F)
        ddp, ddpp = _out(dl, self.N)
        dal, dalp = _out(dl, self.F)
        dN, dNp = _out(dl, self.F)
        dQ, dQp = _out(dl, self.N)
        _check(self._lib, self._h, self._lib.dpf_richards_adjoint(self._h, dl.ptr, float(tol), int(maxiter), dKp,
                                                                  ddpp, dalp, dNp, dQp),
               what="Richards adjoint solve")
        return dK, ddp, dal, dN, dQ

    def richards_transient_forward(self, psi0, Ks, dirichletpsis, z, alphas, Ns, Qs, specificstorage, dt, nsteps,
                                   tol=1e-10, maxiter=200, return_states=False):
        """Fixed-step backward Euler of S V dpsi/dt = R(psi): psi at the final step (and all steps,
        (nsteps, N), with return_states)."""
        p0, K, dp, zz = _Buf(psi0, n=self.N), _Buf(Ks, n=self.F), _Buf(dirichletpsis, n=self.N), _Buf(z, n=self.N)
        al, n_, q, ss = _Buf(alphas, n=self.F), _Buf(Ns, n=self.F), _Buf(Qs, n=self.N), _Buf(specificstorage, n=self.N)
        psiT, pp = _out(p0, self.N)
        states, sp = _out(p0, int(nsteps) * self.N) if return_states else (None, None)
        _check(self._lib, self._h, self._lib.dpf_richards_transient_forward(
            self._h, p0.ptr, K.ptr, dp.ptr, zz.ptr, al.ptr, n_.ptr, q.ptr, ss.ptr, float(dt), int(nsteps), float(tol),
            int(maxiter), sp, pp), what="transient Richards solve")
        if return_states:
            return psiT, states.reshape(int(nsteps), self.N)
        return psiT

    def richards_transient_adjoint(self, obs, weights=None, gT=None, tol=1e-10, maxiter=200):
        """(dKs, ddirichletpsis, dalphas, dNs, dQs, dpsi0) of J = sum_n sum_k w_k psi^n[obs_k]^2 + gT . psi^T."""
        ob = np.ascontiguousarray(np.asarray(obs, dtype=np.int64).ravel())
        w = None if weights is None else np.ascontiguousarray(np.asarray(weights, dtype=np.float64).ravel())
        if w is not None and w.size != ob.size:
            raise ValueError("weights must have one entry per observation (%d), got %d" % (ob.size, w.size))
        g = None if gT is None else _Buf(gT, n=self.N)
        like = g
        dK, dKp = _out(like, self.F)
        ddp, ddpp = _out(like, self.N)
        dal, dalp = _out(like, self.F)
        dN, dNp = _out(like, self.F)
        dQ, dQp = _out(like, self.N)
        d0, d0p = _out(like, self.N)
        _check(self._lib, self._h, self._lib.dpf_richards_transient_adjoint(
            self._h, ob.size, ob.ctypes.data, None if w is None else w.ctypes.data, None if g is None else g.ptr,
            float(tol), int(maxiter), dKp, ddpp, dalp, dNp, dQp, d0p), what="transient Richards adjoint solve")
        return dK, ddp, dal, dN, dQ, d0

    @property
    def richards_stats(self):
        it, ai, rr = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        self._lib.dpf_richards_stats(self._h, ctypes.byref(it), ctypes.byref(ai), ctypes.byref(rr))
        return {"iterations": it.value, "adjoint_iterations": ai.value, "relres": rr.value}

    def set_stream(self, stream):
        """Issue this handle's work on `stream` (a torch.cuda.Stream, a raw cudaStream_t as an
        int, or None for the legacy default stream)."""
        raw = getattr(stream, "cuda_stream", stream)
        _check(self._lib, self._h, self._lib.dpf_set_stream(self._h, ctypes.c_void_p(raw or None)))

    # ---- steady state
    def forward(self, Ks, dirichleths, Qs):
        K = _Buf(Ks, n=self.F)
        d = _Buf(dirichleths, n=self.N)
        q = _Buf(Qs, n=self.N)
        h, hp = _out(K, self.N)
        _check(self._lib, self._h, self._lib.dpf_steady_forward(self._h, K.ptr, d.ptr, q.ptr, hp))
        return h

    def adjoint(self, delta):
        dl = _Buf(delta, n=self.N)
        dK, dKp = _out(dl, self.F)
        ddh, ddhp = _out(dl, self.N)
        dQ, dQp = _out(dl, self.N)
        _check(self._lib, self._h, self._lib.dpf_steady_adjoint(self._h, dl.ptr, dKp, ddhp, dQp))
        return dK, ddh, dQ

    def forward_logk(self, logK, dirichleths, Qs, mean="geometric"):
        lk = _Buf(logK, n=self.N)
        d = _Buf(dirichleths, n=self.N)
        q = _Buf(Qs, n=self.N)
        h, hp = _out(lk, self.N)
        _check(self._lib, self._h, self._lib.dpf_steady_forward_logk(self._h, lk.ptr, _MEANS[mean], d.ptr, q.ptr, hp))
        return h

    def adjoint_logk(self, delta):
        dl = _Buf(delta, n=self.N)
        g, gp = _out(dl, self.N)
        ddh, ddhp = _out(dl, self.N)
        dQ, dQp = _out(dl, self.N)
        _check(self._lib, self._h, self._lib.dpf_steady_adjoint_logk(self._h, dl.ptr, gp, ddhp, dQp))
        return g, ddh, dQ

    def solve_grad_logk(self, logK, dirichleths, Qs, obs, mean="geometric", out=None):
        """Forward solve, J = sum(h[obs]^2), adjoint; returns (h, dJ/dlogK). `out` = (h, g)
        writes into the caller's buffers (e.g. page-locked host arrays)."""
        lk = _Buf(logK, n=self.N)
        d = _Buf(dirichleths, n=self.N)
        q = _Buf(Qs, n=self.N)
        ob = np.ascontiguousarray(obs, dtype=np.int64)
        h, hp = _out_into(out[0] if out else None, lk, self.N)
        g, gp = _out_into(out[1] if out else None, lk, self.N)
        _check(self._lib, self._h, self._lib.dpf_solve_grad_logk(self._h, lk.ptr, _MEANS[mean], d.ptr, q.ptr, ob.size,
                                                                 ob.ctypes.data, hp, gp))
        return h, g

    def logk_to_faces(self, logK, mean="geometric"):
        lk = _Buf(logK, n=self.N)
        K, Kp = _out(lk, self.F)
        _check(self._lib, self._h, self._lib.dpf_logk_to_faces(self._h, lk.ptr, _MEANS[mean], Kp))
        return K

    def logk_to_faces_vjp(self, logK, dKs, mean="geometric"):
        lk = _Buf(logK, n=self.N)
        dk = _Buf(dKs, n=self.F)
        g, gp = _out(lk, self.N)
        _check(self._lib, self._h, self._lib.dpf_logk_to_faces_vjp(self._h, lk.ptr, _MEANS[mean], dk.ptr, gp))
        return g

    def apply(self, x):
        xb = _Buf(x, n=self.N)
        y, yp = _out(xb, self.N)
        _check(self._lib, self._h, self._lib.dpf_apply_operator(self._h, xb.ptr, yp))
        return y

    # ---- transient
    def transient_forward(self, Ks, dirichleths, Qs, specificstorage, dt, nsteps, h0, checkpoint_every=1,
                          return_states=False):
        K = _Buf(Ks, n=self.F)
        d = _Buf(dirichleths, n=self.N)
        q = _Buf(Qs, n=self.N)
        s = _Buf(specificstorage, n=self.N)
        h0b = _Buf(h0, n=self.N)
        hT, hTp = _out(K, self.N)
        states, sp = (None, None)
        if return_states:
            states, sp = _out(K, int(nsteps) * self.N)
        _check(self._lib, self._h, self._lib.dpf_transient_forward(self._h, K.ptr, d.ptr, q.ptr, s.ptr, float(dt),
                                                                   int(nsteps), h0b.ptr, int(checkpoint_every), sp,
                                                                   hTp))
        if return_states:
            return hT, states.reshape(int(nsteps), self.N)
        return hT

    def transient_adjoint(self, obs, weights=None, gT=None):
        ob = np.ascontiguousarray(obs, dtype=np.int64)
        w = None if weights is None else _Buf(weights, n=ob.size)
        g = None if gT is None else _Buf(gT, n=self.N)
        like = w or g
        dK, dKp = _out(like, self.F)
        ddh, ddhp = _out(like, self.N)
        dQ, dQp = _out(like, self.N)
        dh0, dh0p = _out(like, self.N)
        _check(self._lib, self._h, self._lib.dpf_transient_adjoint(self._h, ob.size, ob.ctypes.data,
                                                                   None if w is None else w.ptr,
                                                                   None if g is None else g.ptr, dKp, ddhp, dQp,
                                                                   dh0p))
        return dK, ddh, dQ, dh0


class GroundwaterBatch(GroundwaterProblem):
    """Many independent regular grids (uneven sizes allowed) solved in one set of launches."""

    def __init__(self, dims, mins, maxs, dirichletnodes, **options):
        lib = load()
        dims = np.ascontiguousarray(np.asarray(dims, dtype=np.int32).reshape(-1, 3))
        nprob = dims.shape[0]
        mn = np.ascontiguousarray(np.asarray(mins, dtype=np.float64).reshape(nprob, 3))
        mx = np.ascontiguousarray(np.asarray(maxs, dtype=np.float64).reshape(nprob, 3))
        nd = np.ascontiguousarray([len(d) for d in dirichletnodes], dtype=np.int64)
        dn = np.ascontiguousarray(np.concatenate([np.asarray(d, dtype=np.int64) for d in dirichletnodes])
                                  if nd.sum() else np.zeros(0, np.int64))
        h = ctypes.c_void_p()
        o = _options(**options)
        rc = lib.dpf_batch_create(nprob, dims.ctypes.data, mn.ctypes.data, mx.ctypes.data, nd.ctypes.data,
                                  dn.ctypes.data, ctypes.byref(o), ctypes.byref(h))
        if rc != _lib.DPF_OK:
            raise DPFError(rc, lib.dpf_last_error(None).decode())
        super().__init__(_handle=h)
        self.nprob = nprob
        co, fo = ctypes.c_int64(), ctypes.c_int64()
        self.cell_offsets = np.zeros(nprob + 1, np.int64)
        self.face_offsets = np.zeros(nprob + 1, np.int64)
        for p in range(nprob + 1):
            lib.dpf_batch_offsets(self._h, p, ctypes.byref(co), ctypes.byref(fo))
            self.cell_offsets[p], self.face_offsets[p] = co.value, fo.value

    def sample_logk(self, seeds, ell, sigma, mean=-9.0, nmodes=512, out=None):
        """Seeded Matern(nu = 1) log-conductivity fields for every problem, drawn on the GPU
        (dpf_batch_sample_logk): one seed, correlation length, sigma and mean per problem (scalars
        are broadcast). With out=None the fields stay in the handle for solve_grad_logk(None, ...);
        out may be "cuda" (a new torch CUDA tensor), "host" (a new numpy array) or a float64 buffer."""
        lib = self._lib
        sd = np.ascontiguousarray(np.broadcast_to(np.asarray(seeds, dtype=np.uint64), (self.nprob,)))
        el, sg, mu = (np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (self.nprob,)))
                      for v in (ell, sigma, mean))
        res, ptr = None, None
        if isinstance(out, str):
            if out == "cuda":
                import torch
                res = torch.empty(self.N, dtype=torch.float64, device="cuda")
                ptr = res.data_ptr()
            elif out == "host":
                res = np.empty(self.N)
                ptr = res.ctypes.data
            else:
                raise ValueError("out must be None, 'cuda', 'host' or a float64 buffer")
        elif out is not None:
            res, ptr = _out_into(out, None, self.N)
        _check(lib, self._h, lib.dpf_batch_sample_logk(self._h, int(nmodes), sd.ctypes.data, el.ctypes.data,
                                                       sg.ctypes.data, mu.ctypes.data, ptr))
        return res

    def solve_grad_logk(self, logK, dirichleths, Qs, obs_per_problem, mean="geometric", out=None):
        """Forward solves, J_p = sum(h_p[obs_p]^2), adjoints for every problem; returns the
        concatenated (h, dJ/dlogK). `out` = (h, g) writes into the caller's buffers. logK=None
        solves on the fields last drawn into the handle by sample_logk (outputs on the device)."""
        if logK is None:
            import torch
            lk = _Buf(torch.empty(0, dtype=torch.float64, device="cuda"))
            lk.ptr, lk.size = None, self.N
        else:
            lk = _Buf(logK, n=self.N)
        d = _Buf(dirichleths, n=self.N)
        q = _Buf(Qs, n=self.N)
        if len(obs_per_problem) != self.nprob:
            raise ValueError("obs_per_problem needs one index list per problem (%d), got %d"
                             % (self.nprob, len(obs_per_problem)))
        offs = np.zeros(self.nprob + 1, np.int64)
        offs[1:] = np.cumsum([len(o) for o in obs_per_problem])
        ob = np.ascontiguousarray(np.concatenate([np.asarray(o, np.int64) for o in obs_per_problem])
                                  if offs[-1] else np.zeros(0, np.int64))
        h, hp = _out_into(out[0] if out else None, lk, self.N)
        g, gp = _out_into(out[1] if out else None, lk, self.N)
        _check(self._lib, self._h, self._lib.dpf_batch_solve_grad_logk(self._h, lk.ptr, _MEANS[mean], d.ptr, q.ptr,
                                                                       offs.ctypes.data, ob.ctypes.data, hp, gp))
        return h, g


_TUNED = ("cheb_degree", "plane_cells", "plane_blocks_per_sm", "tail_cells", "blocks_per_sm", "df_plane_cells",
          "tail_cluster", "plane_levels", "streams", "fuse")


def autotune_batch(dims, mins, maxs, dirichletnodes, logK, dirichleths, Qs, obs_per_problem, mean="geometric",
                   repeats=2, **options):
    """Choose the smoother degree and launch shapes for a batch by timing forward + adjoint
    solves of these inputs (the library's dpf_batch_autotune). Returns ({option: value}
    for the tuned options, ms per solve call); pass the dict to GroundwaterBatch."""
    lib = load()
    dims = np.ascontiguousarray(np.asarray(dims, dtype=np.int32).reshape(-1, 3))
    nprob = dims.shape[0]
    mn = np.ascontiguousarray(np.asarray(mins, dtype=np.float64).reshape(nprob, 3))
    mx = np.ascontiguousarray(np.asarray(maxs, dtype=np.float64).reshape(nprob, 3))
    nd = np.ascontiguousarray([len(d) for d in dirichletnodes], dtype=np.int64)
    dn = np.ascontiguousarray(np.concatenate([np.asarray(d, dtype=np.int64) for d in dirichletnodes])
                              if nd.sum() else np.zeros(0, np.int64))
    N = int(np.prod(dims, axis=1).sum())
    lk, d, q = _Buf(logK, n=N), _Buf(dirichleths, n=N), _Buf(Qs, n=N)
    if len(obs_per_problem) != nprob or len(dirichletnodes) != nprob:
        raise ValueError("obs_per_problem and dirichletnodes need one list per problem (%d)" % nprob)
    offs = np.zeros(nprob + 1, np.int64)
    offs[1:] = np.cumsum([len(o) for o in obs_per_problem])
    ob = np.ascontiguousarray(np.concatenate([np.asarray(o, np.int64) for o in obs_per_problem])
                              if offs[-1] else np.zeros(0, np.int64))
    base = _options(**options)
    best = _lib.Options()
    ms = ctypes.c_double()
    rc = lib.dpf_batch_autotune(nprob, dims.ctypes.data, mn.ctypes.data, mx.ctypes.data, nd.ctypes.data,
                                dn.ctypes.data, ctypes.byref(base), lk.ptr, _MEANS[mean], d.ptr, q.ptr,
                                offs.ctypes.data, ob.ctypes.data, int(repeats), ctypes.byref(best), ctypes.byref(ms))
    if rc != _lib.DPF_OK:
        msg = lib.dpf_last_error(None).decode() if rc == _lib.DPF_CUDA else ""
        raise DPFError(rc, msg or "autotuning failed (the starting options do not give a converged solve)")
    return {k: getattr(best, k) for k in _TUNED}, ms.value


# ------------------------------------------------------ reference-shaped API
_cache = OrderedDict()
_CACHE_MAX = 8


def _problem_for(neighbors, areasoverlengths, dirichletnodes, N, options):
    nb = np.ascontiguousarray(np.asarray(neighbors, dtype=np.int64).reshape(-1, 2))
    aol = np.ascontiguousarray(np.asarray(areasoverlengths, dtype=np.float64)[: nb.shape[0]])
    dn = np.ascontiguousarray(np.asarray(dirichletnodes, dtype=np.int64))
    hsh = hashlib.blake2b(digest_size=16)
    for arr in (nb, aol, dn):
        hsh.update(arr.tobytes())
    key = (int(N), hsh.hexdigest(), tuple(sorted(options.items())))
    P = _cache.get(key)
    if P is None:
        P = GroundwaterProblem(nb, aol, dn, N=N, **options)
        _cache[key] = P
        while len(_cache) > _CACHE_MAX:
            _cache.popitem(last=False)
    else:
        _cache.move_to_end(key)
    return P


def amg_solver(*_a, **_k):
    """Selector for ``linear_solver=`` (src/groundwater.jl:45-49): the GPU's AMG-preconditioned
    CG to ``reltol`` (the default)."""
    raise TypeError("amg_solver selects the solver; pass it as linear_solver=amg_solver")


def cholesky_solver(*_a, **_k):
    """Selector for ``linear_solver=`` (src/groundwater.jl:56-60): a direct solve. The GPU
    factors the operator as L L^T in a narrow band (rows renumbered: regular grids with their two
    shortest axes fastest, other meshes in reverse Cuthill-McKee order) once per assembly and
    answers each solve with two triangular solves (options ``solver="cholesky"``). A band too wide
    for the device falls back to the AMG-preconditioned CG run to the FP64 rounding floor of the
    system (the mixed-precision solver with a tolerance below any floor, whose FP64 check accepts
    with status OK once the true residual is at the floor)."""
    raise TypeError("cholesky_solver selects the solver; pass it as linear_solver=cholesky_solver")


def _solver_options(linear_solver, kwargs):
    if linear_solver is None or linear_solver is amg_solver or linear_solver == "amg":
        return kwargs
    if linear_solver is cholesky_solver or linear_solver == "cholesky":
        o = dict(kwargs)
        o["solver"] = SOLVER_CHOLESKY
        # the fallback for bands too wide for the device: the solver with the FP64 floor check,
        # at a tolerance below any FP64 floor (the solve ends at the floor, status OK)
        o["precision"] = "mixed"
        o["reltol"] = 1e-30
        o.setdefault("max_outer", 12)
        return o
    raise ValueError("linear_solver must be amg_solver or cholesky_solver")


def groundwater_steadystate(Ks, neighbors, areasoverlengths, dirichletnodes, dirichleths, Qs, *, linear_solver=None,
                            **kwargs):
    """Steady-state heads over all cells (src/groundwater.jl:75-83).

    ``linear_solver``: ``amg_solver`` (default; CG + AMG to ``reltol``) or ``cholesky_solver``
    (a banded Cholesky factorisation on the GPU). ``kwargs`` are solver options (reltol, maxiter,
    precision='fp64'|'mixed', solver='cg'|'cholesky', ...).
    """
    N = len(Qs) if not _is_torch(Qs) else Qs.numel()
    P = _problem_for(neighbors, areasoverlengths, dirichletnodes, N, _solver_options(linear_solver, kwargs))
    return P.forward(Ks, dirichleths, Qs)


def rrule_groundwater_steadystate(Ks, neighbors, areasoverlengths, dirichletnodes, dirichleths, Qs, *,
                                  linear_solver=None, **kwargs):
    """(h, pullback) like ChainRulesCore.rrule (src/groundwater.jl:85-109).

    pullback(delta) returns (NoTangent, dKs, NoTangent, NoTangent, NoTangent,
    ddirichleths, dQs). The handle (and so the solved state and hierarchy)
    lives as long as the pullback closure.
    """
    N = len(Qs) if not _is_torch(Qs) else Qs.numel()
    P = GroundwaterProblem(neighbors, areasoverlengths, dirichletnodes, N=N,
                           **_solver_options(linear_solver, kwargs))
    h = P.forward(Ks, dirichleths, Qs)

    def pullback(delta):
        dKs, ddh, dQs = P.adjoint(delta)
        return (NoTangent, dKs, NoTangent, NoTangent, NoTangent, ddh, dQs)

    pullback.problem = P
    return h, pullback


def _scaled(x, c):
    return x * c


def solvepressure(Ks_neighbors, neighbors, areasoverlengths, dirichletnodes, dirichleths, Qs, **kwargs):
    """Two-phase pressure solve (src/twophase.jl:48-56): the steady system of
    groundwater_steadystate with transmissibility 2 aol K (src/twophase.jl:25), i.e. the
    steady solve with conductances 2 K. Solved to reltol 1e-14 unless given, like the
    reference's cg_solver (src/twophase.jl:9-13); at the FP64 floor the solve is accepted."""
    kwargs.setdefault("reltol", 1e-14)
    kwargs.setdefault("precision", "mixed")
    return groundwater_steadystate(_scaled(Ks_neighbors, 2.0), neighbors, areasoverlengths, dirichletnodes,
                                   dirichleths, Qs, **kwargs)


def rrule_solvepressure(Ks_neighbors, neighbors, areasoverlengths, dirichletnodes, dirichleths, Qs, **kwargs):
    """(h, pullback) of solvepressure (src/twophase.jl:59-82): the tangents of the steady
    rrule at conductances 2 K, with dKs scaled by 2 (d(2K)/dK)."""
    kwargs.setdefault("reltol", 1e-14)
    kwargs.setdefault("precision", "mixed")
    h, pb = rrule_groundwater_steadystate(_scaled(Ks_neighbors, 2.0), neighbors, areasoverlengths, dirichletnodes,
                                          dirichleths, Qs, **kwargs)

    def pullback(delta):
        t = pb(delta)
        return (t[0], _scaled(t[1], 2.0)) + tuple(t[2:])

    pullback.problem = pb.problem
    return h, pullback


def _z_of(coords):
    """The cell elevations: row 3 of a (3, N) coords array (src/richards.jl:105-111 use coords[3, node])."""
    if _is_torch(coords):
        return coords[2].contiguous()
    c = np.asarray(coords, dtype=np.float64)
    return np.ascontiguousarray(c[2] if c.ndim == 2 else c)


def richards_steadystate(psi0, Ks, neighbors, areasoverlengths, dirichletnodes, dirichletpsis, coords, alphas, Ns,
                         Qs, *, tol=1e-10, maxiter=200, **options):
    """Drop-in for DPFEHM.richards_steadystate (src/richards.jl:148-167): the steady unsaturated
    head psi (N) with van Genuchten kr per face (alphas, Ns), harmonic face means and gravity."""
    N = _len(Qs)
    P = GroundwaterProblem(neighbors, areasoverlengths, dirichletnodes, N=N, general=True, **options)
    return P.richards_steady(psi0, Ks, dirichletpsis, _z_of(coords), alphas, Ns, Qs, tol, maxiter)


def rrule_richards_steadystate(psi0, Ks, neighbors, areasoverlengths, dirichletnodes, dirichletpsis, coords, alphas,
                               Ns, Qs, *, tol=1e-10, maxiter=200, **options):
    """(psi, pullback) as ChainRulesCore.rrule(richards_steadystate, ...) (src/richards.jl:168-190):
    pullback(delta) returns (NoTangent, dpsi0 = 0, dKs, NoTangent x3, ddirichletpsis, NoTangent,
    dalphas, dNs, dQs)."""
    N = _len(Qs)
    P = GroundwaterProblem(neighbors, areasoverlengths, dirichletnodes, N=N, general=True, **options)
    psi = P.richards_steady(psi0, Ks, dirichletpsis, _z_of(coords), alphas, Ns, Qs, tol, maxiter)

    def pullback(delta):
        dK, ddp, dal, dN, dQ = P.richards_adjoint(delta, tol, maxiter)
        zero = dQ * 0
        return (NoTangent, zero, dK, NoTangent, NoTangent, NoTangent, ddp, NoTangent, dal, dN, dQ)

    pullback.problem = P
    return psi, pullback


def _len(x):
    return x.numel() if _is_torch(x) else len(x)


def logKs2Ks_neighbors(logKs, neighbors, mean="geometric", N=None):
    """Face conductances from cell log-conductivities on the GPU
    (geometric: examples/gw_steadystate_3d/inputdeck.jl:51; harmonic: src/richards.jl:50-52)."""
    N = N if N is not None else (logKs.numel() if _is_torch(logKs) else len(logKs))
    nb = np.asarray(neighbors, dtype=np.int64).reshape(-1, 2)
    P = _problem_for(nb, np.ones(nb.shape[0]), [], N, {})
    return P.logk_to_faces(logKs, mean)
