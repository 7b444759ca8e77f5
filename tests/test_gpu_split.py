"""The integer-only 48-bit split of doubles (split48: mixed-precision assembly and round start)
on the GPU, bit for bit against its numpy statement."""
import numpy as np
import pytest

from test_df_arithmetic import split48_reference

pytestmark = pytest.mark.gpu


def test_split48_matches_reference(gpu_lib):
    import torch
    pkg = gpu_lib
    rng = np.random.default_rng(7)
    v = rng.normal(0.0, 1.0, 50000) * 10.0 ** rng.integers(-30, 30, 50000)
    special = np.array([0.0, -0.0, 2.0 ** -79, -(2.0 ** -79), 2.0 ** -80, 5e-324, 2.0 ** 127, 2.0 ** 128, -(2.0 ** 130),
                        np.inf, -np.inf, np.nan, 1.0, -1.0, 1.0 + 2.0 ** -52, np.nextafter(2.0 ** -79, 0.0)])
    v = np.concatenate([v, special])
    n = len(v)
    dv = torch.tensor(v, device="cuda")
    hi = torch.empty(n, dtype=torch.float32, device="cuda")
    lo = torch.empty(n, dtype=torch.float32, device="cuda")
    v48 = torch.empty(n, dtype=torch.float64, device="cuda")
    ok = torch.empty(n, dtype=torch.int32, device="cuda")
    rc = pkg.load().dpf_debug_split48(n, dv.data_ptr(), hi.data_ptr(), lo.data_ptr(), v48.data_ptr(),
                                      ok.data_ptr())
    assert rc == pkg._lib.DPF_OK
    rh, rl, r48, rok = split48_reference(v)
    got_ok = ok.cpu().numpy().astype(bool)
    assert np.array_equal(got_ok, rok)
    m = rok
    assert np.array_equal(hi.cpu().numpy()[m].view(np.uint32), rh[m].view(np.uint32))
    assert np.array_equal(lo.cpu().numpy()[m].view(np.uint32), rl[m].view(np.uint32))
    assert np.array_equal(v48.cpu().numpy()[m].view(np.uint64), r48[m].view(np.uint64))
