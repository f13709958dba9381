"""TEST INFRASTRUCTURE (oracle): compile the CPU oracle.

* oracle/port/oracle.cpp -> oracle/_build/liboracle.so, everywhere (g++,
  OpenMP, no floating-point contraction).
* oracle/ref_driver.cpp -> oracle/_ref/libdust2_ref.so, only where the
  reference sources exist (oracle/Makefile reads them in place).

Only tests, the smoke check and the CPU-baseline leg of bench.py load
these libraries.
"""

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
CSRC = REPO / "dust2_gb300" / "csrc"
PORT_SRC = HERE / "port" / "oracle.cpp"
PORT_LIB = HERE / "_build" / "liboracle.so"
PORT_LIBM_LIB = HERE / "_build" / "liboracle_libm.so"
REF_LIB = HERE / "_ref" / "libdust2_ref.so"


def ref_include(path=None):
    """The reference's inst/include directory: the argument, else the
    DUST2_REF environment variable; None when neither is given."""
    path = path or os.environ.get("DUST2_REF")
    return Path(path) if path else None


def _inputs():
    return ([PORT_SRC] + list((CSRC / "dust2gpu").glob("*.hpp")) +
            list((CSRC / "systems").glob("*.hpp")) +
            list((CSRC / "compat").rglob("*.hpp")) +
            [CSRC / "engine" / "error_text.hpp", Path(__file__)])


def build_port(force=False, libm=False):
    """The CPU restatement.  libm=True builds the timing variant, which
    evaluates exp and log with the host's libm as dust2 does (through
    monty) instead of the project's bit-exact functions: it times the CPU
    path as the reference runs it, and is never used as a checker."""
    lib = PORT_LIBM_LIB if libm else PORT_LIB
    newest = max(p.stat().st_mtime for p in _inputs())
    if not force and lib.exists() and lib.stat().st_mtime >= newest:
        return lib
    lib.parent.mkdir(exist_ok=True)
    tmp = lib.with_suffix(".so.tmp")
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared",
           "-ffp-contract=off", "-fno-strict-aliasing", "-I", str(CSRC),
           "-I", str(CSRC / "compat")]
    if libm:
        cmd.append("-DDUST2_HOST_LIBM")
    cmd += [str(PORT_SRC), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    return lib


def build_ref(force=False, include=None):
    """Build the reference-engine oracle from the reference's
    inst/include directory (`include`, else $DUST2_REF); None when the
    sources are not there."""
    inc = ref_include(include)
    if inc is None or not (inc / "dust2" / "filter.hpp").exists():
        return None
    cmd = ["make", "-s", "-C", str(HERE), f"REF={inc}"]
    if force:
        subprocess.run(["make", "-s", "-C", str(HERE), f"REF={inc}",
                        "clean"], check=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{res.stdout}\n"
                           f"{res.stderr}")
    return REF_LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_port(force))
    print(build_ref(force))
