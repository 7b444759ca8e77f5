"""Cases run against the checked build of the library (DPF_CHECK: device-side bounds and
alignment checks). Run as a child process with DPFEHM_GPU_LIB pointing at that build;
prints one JSON line: the violations the checks recorded, the first one, and the largest
relative errors against the oracle, per case family.

Small grids (2x2x2 up to 8x8x8 and a few ragged shapes) reach every edge of the index
arithmetic: one-cell-thick axes, odd extents whose last aggregate is partial, slabs that
hold a whole plane, batches of uneven grids, the plane-marching and grid-stride kernels,
the fused tail and the CSR path.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
sys.path.insert(0, HERE)

import __graft_entry__ as g  # noqa: E402
import oracle as orc  # noqa: E402
import richards_oracle as ro  # noqa: E402
from helpers import rel, steady_case  # noqa: E402
from richards_cases import oracle_args, richards_case, transient_case  # noqa: E402

SHAPES = [(2, 2, 2), (3, 3, 3), (1, 5, 4), (4, 1, 3), (5, 4, 1), (7, 5, 3), (8, 8, 8), (17, 9, 6), (33, 20, 11)]


def oracle_pair(c, delta):
    O = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
    h = O.steady(c["Ks"], c["dh"], c["Qs"], reltol=1e-14)
    dKs, ddh, dQs = O.adjoint(c["dh"], delta, reltol=1e-14)
    return h, dKs


def main():
    pkg = g.load_package()
    lib = pkg.load()
    orc.build()
    err = {"steady": 0.0, "adjoint": 0.0, "batch": 0.0, "csr": 0.0, "transient": 0.0, "richards": 0.0,
           "richards_adjoint": 0.0}
    for k, ns in enumerate(SHAPES):
        c = steady_case(pkg, ns, sigma=1.0, seed=40 + k, ndir=1 if k % 2 == 0 else 3, nq=1)
        delta = np.random.default_rng(k).standard_normal(c["N"])
        h_or, dK_or = oracle_pair(c, delta)
        for opts in ({"precision": "fp64"}, {"precision": "mixed"}, {"precision": "mixed", "tail_cells": -1},
                     {"precision": "mixed", "plane": 2}, {"precision": "mixed", "plane": 2, "plane_cells": 256},
                     {"precision": "mixed", "tail_cluster": 8}):
            P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], reltol=1e-12, **opts)
            h = P.forward(c["Ks"], c["dh"], c["Qs"])
            dKs, _, _ = P.adjoint(delta)
            err["steady"] = max(err["steady"], rel(h, h_or))
            err["adjoint"] = max(err["adjoint"], rel(dKs, dK_or))
            P.close()
    # an uneven batch through the batched entry point
    shapes = [(9, 7, 5), (2, 2, 2), (16, 16, 4), (5, 1, 6)]
    cases = [steady_case(pkg, ns, seed=70 + k) for k, ns in enumerate(shapes)]
    for prec in ("fp64", "mixed"):
        B = pkg.GroundwaterBatch([c["ns"] for c in cases], [c["mins"] for c in cases], [c["maxs"] for c in cases],
                                 [c["dn"] for c in cases], reltol=1e-12, precision=prec)
        cat = lambda key: np.concatenate([c[key] for c in cases])
        obs = [np.array([0, c["N"] // 2]) for c in cases]
        h, _ = B.solve_grad_logk(cat("logK"), cat("dh"), cat("Qs"), obs)
        for k, c in enumerate(cases):
            O = orc.Problem(c["N"], c["nb"], c["aol"], c["dn"])
            h_or = O.steady(c["Ks"], c["dh"], c["Qs"], reltol=1e-14)
            a, b = B.cell_offsets[k], B.cell_offsets[k + 1]
            err["batch"] = max(err["batch"], rel(h[a:b], h_or))
        B.close()
    # the CSR path: a regular grid with duplicated faces is not a regulargrid3d
    c = steady_case(pkg, (9, 6, 5), seed=90)
    nb = np.concatenate([c["nb"], c["nb"][::4]])
    aol = np.concatenate([c["aol"], 0.5 * c["aol"][::4]])
    Ks = np.concatenate([c["Ks"], c["Ks"][::4]])
    O = orc.Problem(c["N"], nb, aol, c["dn"])
    h_or = O.steady(Ks, c["dh"], c["Qs"], reltol=1e-14)
    for prec in ("fp64", "mixed"):
        P = pkg.GroundwaterProblem(nb, aol, c["dn"], N=c["N"], reltol=1e-12, precision=prec)
        assert not P.structured
        err["csr"] = max(err["csr"], rel(P.forward(Ks, c["dh"], c["Qs"]), h_or))
        P.close()
    # a short transient run on a regular grid
    c = steady_case(pkg, (10, 8, 4), seed=95)
    N = c["N"]
    Ss = np.full(N, 1e-5)
    O = orc.Problem(N, c["nb"], c["aol"], c["dn"])
    st_or = O.transient(c["Ks"], c["dh"], c["Qs"], Ss, c["vol"], 3600.0, 4, np.zeros(O.nfree), reltol=1e-14)
    isf, _, _ = pkg.getfreenodes(N, c["dn"])
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=N, volumes=c["vol"], reltol=1e-12)
    _, states = P.transient_forward(c["Ks"], c["dh"], c["Qs"], Ss, 3600.0, 4, np.zeros(N), return_states=True)
    err["transient"] = rel(states[:, isf], st_or)
    P.close()

    # Richards: a steady solve with its pullback and a short transient run, on the CSR handle
    c = richards_case(pkg, ns=(7, 5, 4), seed=12)
    psi_or = ro.steady(c["psi0"], c["Ks"], c["nb"], c["aol"], c["dn"], c["dpsi"], c["z"], c["alphas"], c["Ns"],
                       c["Qs"], tol=1e-14)
    w = np.random.default_rng(6).standard_normal(c["N"])
    g_or = ro.pullback(psi_or, w, *oracle_args(c))
    psi, pb = pkg.rrule_richards_steadystate(c["psi0"], c["Ks"], c["nb"], c["aol"], c["dn"], c["dpsi"], c["coords"],
                                             c["alphas"], c["Ns"], c["Qs"], tol=1e-12, reltol=1e-12)
    err["richards"] = rel(psi, psi_or)
    t = pb(w)
    err["richards_adjoint"] = max(rel(t[2], g_or[0]), rel(t[10], g_or[4]))
    c = transient_case(pkg, ns=(6, 5, 4))
    st_or = ro.transient(c["psi0"], c["Ks"], c["nb"], c["aol"], c["dn"], c["dpsi"], c["z"], c["alphas"], c["Ns"],
                         c["Qs"], c["Ss"], c["vol"], c["dt"], c["nsteps"], tol=1e-14)
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"], volumes=c["vol"], general=True, reltol=1e-12)
    _, st = P.richards_transient_forward(c["psi0"], c["Ks"], c["dpsi"], c["z"], c["alphas"], c["Ns"], c["Qs"],
                                         c["Ss"], c["dt"], c["nsteps"], tol=1e-12, return_states=True)
    err["richards"] = max(err["richards"], rel(st, st_or))
    P.close()

    import ctypes
    nv = ctypes.c_int64(-1)
    first = (ctypes.c_int64 * 3)()
    rc = lib.dpf_debug_check_report(ctypes.byref(nv), first)
    print(json.dumps({"rc": rc, "violations": nv.value, "first": list(first), "errors": err}))


if __name__ == "__main__":
    main()
