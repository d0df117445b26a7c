"""The C-ABI library loads and exports every entry point that include/*.h
declares, and the ctypes mirrors have the header's layouts.  No compute call
is made here (this file runs without a GPU)."""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

from jmmonedmc_gb300 import _native, abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECL = re.compile(r"^\s*(?:int|const char \*|void)\s*\*?\s*(jmm_[a-z0-9_]+)\s*\(", re.M)


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        with open(h) as f:
            names.update(DECL.findall(f.read()))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "jmm_plain_create" in names and "jmm_last_error" in names


def test_library_exports_every_declared_symbol(native):
    missing = [s for s in declared_symbols() if not hasattr(native, s)]
    assert not missing, f"libjmmgpu.so lacks {missing}"


def test_library_exports_are_c_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", _native.lib_path()],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    for s in declared_symbols():
        assert s in exported, f"{s} is not an unmangled export"


def _c_sizeof(type_name):
    src = f'#include "jmm_gpu.h"\n#include <stdio.h>\nint main(void){{printf("%zu", sizeof({type_name}));return 0;}}\n'
    exe = os.path.join(REPO, "oracle", "_build", f"sizeof_{type_name}")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    subprocess.run(["gcc", "-x", "c", "-I", os.path.join(REPO, "include"), "-o", exe, "-"],
                   input=src, text=True, check=True)
    return int(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)


@pytest.mark.parametrize("cname,pytype", [
    ("jmm_params", abi.Params), ("jmm_state", abi.State), ("jmm_draw", abi.Draw),
    ("jmm_step_record", abi.StepRecord), ("jmm_chain_desc", abi.ChainDesc),
    ("jmm_batch_config", abi.BatchConfig), ("jmm_chain_result", abi.ChainResult),
    ("jmm_grad_chain", abi.GradChain), ("jmm_grad_stats", abi.GradStats),
    ("jmm_large_result", abi.LargeResult),
])
def test_struct_layouts_match_header(cname, pytype):
    assert _c_sizeof(cname) == C.sizeof(pytype)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_native, "_LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_native, "_lib", None)
    with pytest.raises(ImportError):
        _native.load()


def test_noalloc_refuses_bad_box_before_any_device_work(native):
    """The allocation-free entry point checks its scalar arguments on the
    host first: a box length that is not finite and positive is refused
    without touching the (here absent) device or the pointers."""
    fn = native.jmm_plain_full_energy_noalloc
    fn.argtypes = [C.POINTER(abi.Params), C.c_void_p, C.c_uint64, C.c_double, C.c_void_p,
                   C.c_void_p]
    fn.restype = C.c_int
    params = abi.make_params(n=16, l=32.0)
    fake = C.c_void_p(256)  # never dereferenced: the check comes first
    for l in (float("nan"), 0.0, -2.0, float("inf")):
        assert fn(C.byref(params), fake, 16, l, fake, None) == abi.JMM_ERR_INVALID
