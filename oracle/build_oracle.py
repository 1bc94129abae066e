"""Build recipe for the ORACLE (test infrastructure only).

* ``build_oracle()`` compiles this directory's C restatement (sv_oracle.c, traj_oracle.c,
  adjoint_oracle.c) into ``oracle/_build/liboracle.so`` with gcc.  It builds on x86 and Arm.
* ``build_ref()`` compiles the reference's own sources where they lie (never copied) into
  ``oracle/_ref/``: the pybind11 modules ``quantum_sim_v3`` (src/StateVectorOptimized.cpp) and
  ``quantum_sim_v2`` (src/bindings_v2.cpp) with the reference's own build flags
  (README.md:124-133: ``-O3 -Wall -shared -std=c++17 -fopenmp -fPIC``), and ``libref.so`` from
  ref_capi.cpp over the header-only src/Backend.h, src/StateVectorBackend.h, src/Algorithms.h and
  src/Mitigation.h.
  It needs the reference tree and pybind11 headers, so it only runs where both exist.

Where the reference tree lies: the environment variable LLG_REFERENCE_ROOT, else DEFAULT_REF (the
place this recipe reads it from on the build machine).  ``reference_root()`` returns None where
neither holds the tree (the GPU machine): the reference build and the tests that need the tree skip.

Run ``python oracle/build_oracle.py [--ref]``.
"""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
DEFAULT_REF = "/root/reference"
REF_ENV = "LLG_REFERENCE_ROOT"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def oracle_lib_path() -> str:
    return os.path.join(BUILD, "liboracle.so")


def _locked(path: str):
    """An exclusive file lock: concurrent builds of the oracle wait for each other."""
    import contextlib
    import fcntl

    @contextlib.contextmanager
    def lock():
        fd = os.open(path, os.O_CREAT | os.O_RDWR, 0o644)
        try:
            fcntl.flock(fd, fcntl.LOCK_EX)
            yield
        finally:
            fcntl.flock(fd, fcntl.LOCK_UN)
            os.close(fd)

    return lock()


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with _locked(os.path.join(BUILD, ".build.lock")):
        return _build_oracle_locked(force)


def _build_oracle_locked(force: bool) -> str:
    srcs = [os.path.join(HERE, f) for f in ("sv_oracle.c", "traj_oracle.c", "adjoint_oracle.c", "noise_oracle.c", "dm_oracle.c", "tsolver_oracle.c")]
    out = oracle_lib_path()
    if force or _stale(out, srcs + [os.path.join(HERE, "sv_oracle.h")]):
        tmp = out + ".tmp"
        _run(["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
              "-o", tmp, *srcs, "-lm"])
        os.replace(tmp, out)
    return out


def _is_tree(ref: str | None) -> bool:
    return bool(ref) and os.path.isfile(os.path.join(ref, "src", "StateVectorBackend.h"))


def reference_root() -> str | None:
    """The reference tree (LLG_REFERENCE_ROOT, else DEFAULT_REF), or None where it is absent."""
    for ref in (os.environ.get(REF_ENV), DEFAULT_REF):
        if _is_tree(ref):
            return ref
    return None


def ref_available(ref: str | None = None) -> bool:
    return _is_tree(ref) if ref else reference_root() is not None


def build_ref(ref: str | None = None, force: bool = False) -> dict[str, str]:
    """Compile the reference's own sources into oracle/_ref (only where the tree exists)."""
    ref = ref or reference_root()
    if not _is_tree(ref):
        raise FileNotFoundError(f"reference sources not found under {ref}")
    import pybind11  # only needed here, where the reference is built

    os.makedirs(REF_OUT, exist_ok=True)
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    py_inc = sysconfig.get_paths()["include"]
    pb_inc = pybind11.get_include()
    src = os.path.join(ref, "src")
    jobs = {
        os.path.join(REF_OUT, "quantum_sim_v3" + ext): (
            [os.path.join(src, "StateVectorOptimized.cpp")],
            ["g++", "-O3", "-Wall", "-shared", "-std=c++17", "-fopenmp", "-fPIC",
             os.path.join(src, "StateVectorOptimized.cpp"), "-I" + py_inc, "-I" + pb_inc]),
        os.path.join(REF_OUT, "quantum_sim_v2" + ext): (
            [os.path.join(src, "bindings_v2.cpp")],
            ["g++", "-O3", "-Wall", "-shared", "-std=c++17", "-fopenmp", "-fPIC",
             os.path.join(src, "bindings_v2.cpp"), "-I" + py_inc, "-I" + pb_inc]),
        os.path.join(REF_OUT, "libref.so"): (
            [os.path.join(HERE, "ref_capi.cpp"), os.path.join(src, "StateVectorBackend.h"),
             os.path.join(src, "Algorithms.h"), os.path.join(src, "Backend.h"), os.path.join(src, "Mitigation.h")],
            ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-I" + src, "-I" + HERE,
             os.path.join(HERE, "ref_capi.cpp")]),
    }
    todo = [(out, cmd) for out, (deps, cmd) in jobs.items() if force or _stale(out, deps)]
    with ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(lambda oc: _run(oc[1] + ["-o", oc[0]]), todo))
    return {os.path.basename(k): k for k in jobs}


if __name__ == "__main__":
    print(build_oracle(force=True))
    if "--ref" in sys.argv:
        print(build_ref(force=True))
