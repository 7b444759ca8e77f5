"""Transient backward Euler and its checkpointed adjoint on the GPU against the golden
vectors and the oracle (relative L2: states 1e-8, gradients 1e-6)."""
import os

import numpy as np
import pytest

from helpers import rel, steady_case

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_transient_golden(gpu_lib):
    pkg = gpu_lib
    g = dict(np.load(os.path.join(GOLD, "transient_regular3d.npz")))
    N = int(np.prod(g["ns"]))
    P = pkg.GroundwaterProblem(g["nb"], g["aol"], g["dn"], N=N, volumes=g["V"], reltol=1e-13)
    assert P.structured
    isf, n2f, f2n = pkg.getfreenodes(N, g["dn"])
    nsteps = int(g["nsteps"])
    hT, states = P.transient_forward(g["Ks"], g["dh"], g["Qs"], g["Ss"], float(g["dt"]), nsteps, np.zeros(N),
                                     checkpoint_every=2, return_states=True)
    assert rel(states[:, isf], g["states"]) < 1e-8
    assert np.array_equal(states[:, ~isf], np.tile(g["dh"][~isf], (nsteps, 1)))
    dKs, ddh, dQs, dh0 = P.transient_adjoint(g["obs"])
    assert rel(dKs, g["dKs"]) < 1e-6
    assert rel(ddh, g["ddh"]) < 1e-6
    assert rel(dQs, g["dQs"]) < 1e-6
    assert rel(dh0[isf], g["dh0"]) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_transient_vs_oracle_and_checkpointing(gpu_lib, orc, precision):
    pkg = gpu_lib
    c = steady_case(pkg, (30, 24, 8), sigma=1.5, seed=19, ndir=1, nq=4)
    N = c["N"]
    # a Dirichlet face (x = max) as in the 800k-cell transient configuration
    dn = np.arange(N - 24 * 8, N)
    dh = np.zeros(N)
    Ss = np.full(N, 1e-5)
    dt, nsteps = 3600.0, 12
    obs = np.random.default_rng(4).choice(N - 24 * 8, 15, replace=False)
    O = orc.Problem(N, c["nb"], c["aol"], dn)
    st_or = O.transient(c["Ks"], dh, c["Qs"], Ss, c["vol"], dt, nsteps, np.zeros(O.nfree), reltol=1e-14)
    dK_or, ddh_or, dQ_or, dh0_or = O.transient_adjoint(dh, obs, reltol=1e-14)
    isf, n2f, f2n = pkg.getfreenodes(N, dn)
    res = []
    for ck in (1, 5):
        P = pkg.GroundwaterProblem(c["nb"], c["aol"], dn, N=N, volumes=c["vol"], reltol=1e-12, precision=precision)
        hT, states = P.transient_forward(c["Ks"], dh, c["Qs"], Ss, dt, nsteps, np.zeros(N), checkpoint_every=ck,
                                         return_states=True)
        assert rel(states[:, isf], st_or) < 1e-8
        res.append(P.transient_adjoint(obs))
    for dK, ddh, dQ, dh0 in res:
        assert rel(dK, dK_or) < 1e-6
        assert rel(ddh, ddh_or) < 1e-6
        assert rel(dQ, dQ_or) < 1e-6
        assert rel(dh0[isf], dh0_or) < 1e-6
    # checkpoint spacing changes only when states are recomputed, not the result
    for a, b in zip(res[0], res[1]):
        assert rel(a, b) < 1e-12


def test_transient_adjoint_needs_forward(gpu_lib):
    pkg = gpu_lib
    c = steady_case(pkg, (6, 5, 4), seed=1)
    P = pkg.GroundwaterProblem(c["nb"], c["aol"], c["dn"], N=c["N"])
    with pytest.raises(pkg.DPFError) as e:
        P.transient_adjoint([1, 2])
    assert e.value.code == 7
