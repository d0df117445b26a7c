"""Build recipe of the oracle (TEST INFRASTRUCTURE, never shipped).

    python oracle/build_oracle.py          # CPU restatement, and the reference where present

* build_oracle(): the CPU restatement, oracle/_build/libjmmoracle.so
  (``make -C oracle``).
* build_reference_if_present(): the reference compiled from its own sources
  where they lie, GSL replaced by gsl_shim/ (``make -C oracle ref
  REF_SRC=...``), into oracle/_ref/.  The sources are taken from JMM_REF_SRC,
  else from the reference checkout's usual place in the build container;
  where neither exists (the GPU machine) nothing is built.
"""
import os
import subprocess
import sys

ORACLE = os.path.dirname(os.path.abspath(__file__))
# where the build container keeps the reference's source tree
_DEFAULT_REF_SRC = "/root/reference/src"


def reference_sources():
    """The reference's src directory, or None where it is not present."""
    ref = os.environ.get("JMM_REF_SRC") or _DEFAULT_REF_SRC
    return ref if os.path.exists(os.path.join(ref, "jmmMCState.cpp")) else None


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE], check=True)
    return os.path.join(ORACLE, "_build", "libjmmoracle.so")


def build_reference_if_present():
    ref = reference_sources()
    if ref is None:
        return None
    subprocess.run(["make", "-s", "-C", ORACLE, "ref", f"REF_SRC={ref}"], check=True)
    return os.path.join(ORACLE, "_ref")


if __name__ == "__main__":
    print(build_oracle())
    print(build_reference_if_present() or "reference tree not present: oracle/_ref not built")
    sys.exit(0)
