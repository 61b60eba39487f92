"""Build ``libfdtd_gb300.so`` in place with nvcc for sm_103a.

Each translation unit compiles in its own nvcc process (in parallel), then one
link step produces the shared library next to this file.  The CUDA runtime is
linked statically, so the library loads without a GPU (compute calls then
return an error).

    python -m fdtd_gb300.build
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
SOURCES = ["fdtd_f32.cu", "fdtd_f64.cu", "fdtd_adjoint.cu", "fdtd_onepass.cu", "fdtd_capi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC"] + ARCH


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        exe = "/usr/local/cuda/bin/nvcc"
    if exe is None:
        raise RuntimeError("nvcc not found")
    return exe


def build(verbose=False, out_dir=None):
    """Compile every translation unit and link the shared library; return its path."""
    from fdtd_gb300 import _native

    out_dir = out_dir or os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    cc = nvcc()
    objs = []
    cmds = []
    for src in SOURCES:
        obj = os.path.join(out_dir, src.replace(".cu", ".o"))
        objs.append(obj)
        cmds.append([cc] + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj])

    def run(cmd):
        res = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, res

    with concurrent.futures.ThreadPoolExecutor(len(cmds)) as ex:
        for cmd, res in ex.map(run, cmds):
            if verbose or res.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + res.stdout + res.stderr)
            if res.returncode != 0:
                raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    tmp = _native.LIB_PATH + ".tmp"
    link = [cc, "-shared"] + ARCH + ["-o", tmp] + objs
    res = subprocess.run(link, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(" ".join(link) + "\n" + res.stdout + res.stderr)
        raise RuntimeError("link of libfdtd_gb300.so failed")
    os.replace(tmp, _native.LIB_PATH)
    return _native.LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
