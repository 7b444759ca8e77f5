"""The allocation-free entry point against the handle-based one.

dpf_logk_to_faces_regular_noalloc serves callers that cannot let the library
allocate device memory (applications that own all device memory through their
own pool). It must give the same face conductances as dpf_logk_to_faces on a
regulargrid3d handle, call after call, although its scratch array is shared and
keeps the previous call's contents. Collected last (file name) so that a run
stopping at the first failure has already run every other test.
"""
import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu


def _noalloc(lib, ns, d_logK, kind, d_Ks):
    return lib.dpf_logk_to_faces_regular_noalloc(int(ns[0]), int(ns[1]), int(ns[2]), d_logK.data_ptr(), kind,
                                                 d_Ks.data_ptr())


def test_noalloc_matches_handle_path_two_calls_in_a_row(gpu_lib, orc):
    """Both paths do the same arithmetic per face, so they agree bit for bit; the first call is
    also checked against the oracle's face means (relative L2 1e-14)."""
    import torch
    pkg = gpu_lib
    lib = pkg.load()
    ns, mins, maxs = (37, 29, 11), (0.0, 0.0, 0.0), (18.0, 14.0, 5.0)
    P = pkg.GroundwaterProblem.regular3d(mins, maxs, ns, [0])
    _, nb, _, _ = pkg.regulargrid3d(mins, maxs, ns)
    dev = torch.device("cuda", torch.cuda.current_device())
    d_Ks = torch.full((P.F,), np.nan, dtype=torch.float64, device=dev)
    for call in range(2):
        for mean, kind in (("geometric", 0), ("harmonic", 1)):
            logK = pkg.fields.volume_logk(ns, mins, maxs, 6.0, 1.5, -9.0, seed=100 + 10 * call + kind)
            ref = P.logk_to_faces(logK, mean)
            d_logK = torch.tensor(logK, device=dev)
            rc = _noalloc(lib, ns, d_logK, kind, d_Ks)
            assert rc == 0, lib.dpf_last_error(None)
            got = d_Ks.cpu().numpy()
            assert np.all(np.isfinite(got))
            assert np.array_equal(got, ref)
            if call == 0:
                assert rel(got, orc.logk_to_faces(nb, logK, kind)) < 1e-14


def test_noalloc_rejects_oversize_grid_and_host_pointers(gpu_lib):
    import torch
    pkg = gpu_lib
    lib = pkg.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    small = torch.zeros(8, dtype=torch.float64, device=dev)
    rc = lib.dpf_logk_to_faces_regular_noalloc(200, 200, 60, small.data_ptr(), 0, small.data_ptr())
    assert rc == 1
    assert b"at most" in lib.dpf_last_error(None)
    host = np.zeros(8)
    rc = lib.dpf_logk_to_faces_regular_noalloc(2, 2, 2, host.ctypes.data, 0, small.data_ptr())
    assert rc == 1
