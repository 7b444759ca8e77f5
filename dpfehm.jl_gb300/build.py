"""Build recipe of libdpfehm_gpu.so: nvcc for sm_103a, one translation unit per
process (compiled in parallel), linked with the static CUDA runtime.

Output: dpfehm.jl_gb300/_build/libdpfehm_gpu.so (git-ignored; rebuilt on each machine).
"""
import concurrent.futures
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdpfehm_gpu.so")
SOURCES = ["dpf_struct.cu", "dpf_general.cu", "dpf_api.cu", "dpf_noalloc.cu", "dpf_tune.cu", "dpf_debug.cu",
           "dpf_richards.cu", "dpf_sampler.cu", "dpf_direct.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "--extended-lambda", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
              "-I" + os.path.join(HERE, "..", "include")]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "dpfehm_gpu.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False, out_dir=None, defines=()):
    """Compile (if sources changed) and return the library path. `out_dir` and
    `defines` (extra -D flags) build a variant elsewhere, e.g. for tuning runs."""
    out = out_dir or OUT
    lib = os.path.join(out, "libdpfehm_gpu.so")
    os.makedirs(out, exist_ok=True)
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= _deps():
        return lib
    nvcc = _nvcc()
    extra = ["-D" + d for d in defines]

    def compile_one(src):
        obj = os.path.join(out, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + ARCH + NVCC_FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s" % (src, r.stderr))
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib + ".tmp%d" % os.getpid()
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
