"""The checked build (DPF_CHECK: device-side bounds and alignment checks that record a
violation instead of trapping) runs small and ragged cases of every kernel family with no
violation and the oracle's answers; the regular build reports the checks as absent."""
import ctypes
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_checked_build_runs_clean(gpu_lib):
    import __graft_entry__ as g
    b = g._load_build_module()
    lib = b.build(out_dir=os.path.join(ROOT, "dpfehm.jl_gb300", "_build_check"), defines=["DPF_CHECK"])
    env = dict(os.environ, DPFEHM_GPU_LIB=os.path.abspath(lib))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "checked_cases.py")], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["rc"] == 0
    assert out["violations"] == 0, out["first"]
    e = out["errors"]
    assert e["steady"] < 1e-8 and e["batch"] < 1e-8 and e["csr"] < 1e-8 and e["transient"] < 1e-8, e
    assert e["adjoint"] < 1e-6, e
    assert e["richards"] < 1e-8 and e["richards_adjoint"] < 1e-6, e


def test_regular_build_has_no_checks(gpu_lib):
    lib = gpu_lib.load()
    nv = ctypes.c_int64(-1)
    assert lib.dpf_debug_check_report(ctypes.byref(nv), None) == 8   # DPF_UNSUPPORTED
