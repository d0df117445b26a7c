"""In-tree build of libjmmgpu.so (sm_103a).

    python -m jmmonedmc_gb300.build          # the CUDA library
    python -c "import __graft_entry__ as g; g.build()"   # with the oracle (tests)

The CUDA library is compiled with nvcc straight for sm_103a, one object per
translation unit, in parallel, then linked with ``nvcc -shared``; no
PyTorch extension machinery and no cmake.  Outputs go to
``jmmonedmc_gb300/_lib/`` (git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIBNAME = "libjmmgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation unit -> extra flags.  plain.cu must not contract FP64
# expressions into fused multiply-adds (bit parity with the reference).
UNITS = {
    "common.cu": [],
    "plain.cu": ["-fmad=false"],
    "batch.cu": [],
    "batch_wide.cu": [],
    "grad.cu": [],
    "noalloc.cu": ["-fmad=false"],
    "peak.cu": [],
    "large.cu": [],
}


def nvcc_path():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libjmmgpu.so")


def _compile(nvcc, src, obj, extra, verbose):
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", os.path.join(REPO, "include"), "-c", src, "-o", obj, *extra]
    if verbose:
        cmd.append("-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{res.stderr}")
    return res.stderr


def build_native(verbose=False, jobs=None):
    nvcc = nvcc_path()
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    jobs = jobs or min(len(units), os.cpu_count() or 4)
    objs = []
    logs = {}
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {}
        for u in units:
            src = os.path.join(CSRC, u)
            obj = os.path.join(objdir, u.replace(".cu", ".o"))
            objs.append(obj)
            futs[ex.submit(_compile, nvcc, src, obj, UNITS[u], verbose)] = u
        for fut in cf.as_completed(futs):
            logs[futs[fut]] = fut.result()
    out = os.path.join(LIBDIR, LIBNAME)
    tmp = out + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{res.stderr}")
    os.replace(tmp, out)
    if verbose:
        for u, log in logs.items():
            sys.stdout.write(f"== {u}\n{log}")
    return out


if __name__ == "__main__":
    print(build_native(verbose="-v" in sys.argv))
