"""Builds the engine in-tree: libllgpu.so (CUDA kernels + C ABI, sm_103a) and the pybind11 drop-in
modules quantum_sim_v3 / quantum_sim_v2 / quantum_sim_algorithms that sit on top of it.

Compiles each translation unit in parallel with nvcc (-gencode arch=compute_103a,code=sm_103a) or
g++, links with nvcc.  pybind11 headers come from the ones PyTorch ships (torch/include), so the
same recipe works wherever torch is installed; the modules themselves do not link torch.
Outputs land next to this file (git-ignored).  Run ``python build_ext.py`` or call ``build()``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
REPO = os.path.dirname(HERE)
INCLUDE = os.path.join(REPO, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", *ARCH, "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-I" + INCLUDE, "-I" + CSRC]

CU_SOURCES = ["llg_kernels.cu", "llg_engine.cu", "llg_noalloc.cu", "llg_adjoint.cu", "llg_traj.cu", "llg_batch.cu",
              "llg_tune.cu", "llg_block.cu", "llg_block_tc.cu",
              "llg_tsolver.cu", "llg_diag.cu", "llg_tile_reg.cu"]
CXX_SOURCES = ["llg_plan.cpp", "llg_diag_host.cpp"]

LIB = os.path.join(HERE, "libllgpu.so")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _newer(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "llgpu.h"))
    return hs


def cuda_lib_dir() -> str:
    for d in ("lib64", os.path.join("targets", "sbsa-linux", "lib"), os.path.join("targets", "x86_64-linux", "lib"), "lib"):
        p = os.path.join(CUDA_HOME, d)
        if os.path.exists(os.path.join(p, "libcudart.so")) or os.path.exists(os.path.join(p, "libcudart_static.a")):
            return p
    return os.path.join(CUDA_HOME, "lib64")


def torch_pybind_include() -> str:
    import importlib.util

    spec = importlib.util.find_spec("torch")
    if spec is None or not spec.origin:
        raise RuntimeError("torch is needed for its bundled pybind11 headers")
    inc = os.path.join(os.path.dirname(spec.origin), "include")
    if not os.path.isdir(os.path.join(inc, "pybind11")):
        raise RuntimeError("pybind11 headers not found under " + inc)
    return inc


class _BuildLock:
    """An exclusive lock on a file in the build folder: builds started at the same time (a test
    run and a bench, two processes importing the package) wait for each other instead of writing
    the same objects and library at once; the later one then finds everything up to date."""

    def __init__(self, path: str):
        self.path = path
        self.fd = -1

    def __enter__(self):
        import fcntl

        self.fd = os.open(self.path, os.O_CREAT | os.O_RDWR, 0o644)
        fcntl.flock(self.fd, fcntl.LOCK_EX)
        return self

    def __exit__(self, *exc):
        import fcntl

        fcntl.flock(self.fd, fcntl.LOCK_UN)
        os.close(self.fd)
        return False


def build(force: bool = False, jobs: int = 8) -> str:
    os.makedirs(OBJ, exist_ok=True)
    with _BuildLock(os.path.join(OBJ, ".build.lock")):
        return _build_locked(force, jobs)


def _build_locked(force: bool, jobs: int) -> str:
    hdrs = _headers()
    tasks = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            tasks.append([NVCC, *NVCC_FLAGS, "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            tasks.append(["g++", *CXX_FLAGS, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(_run, tasks))
    if force or _newer(LIB, objs):
        tmp = LIB + ".tmp"
        _run([NVCC, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"])
        os.replace(tmp, LIB)

    # pybind11 drop-in modules over the C ABI
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    py_inc = sysconfig.get_paths()["include"]
    pb_inc = torch_pybind_include()
    mods = []
    for mod, src, define in (("quantum_sim_v3", "py_quantum_sim.cpp", "LLG_MODULE_V3"),
                             ("quantum_sim_v2", "py_quantum_sim.cpp", "LLG_MODULE_V2"),
                             ("quantum_sim_algorithms", "py_algorithms.cpp", "LLG_MODULE_ALGORITHMS")):
        pb_src = os.path.join(CSRC, src)
        out = os.path.join(HERE, mod + ext)
        if force or _newer(out, [pb_src, LIB] + hdrs):
            mods.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fvisibility=hidden", "-D" + define,
                         "-I" + INCLUDE, "-I" + py_inc, "-I" + pb_inc, pb_src, "-o", out, "-L" + HERE, "-lllgpu",
                         "-Wl,-rpath,$ORIGIN"])
    with ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(_run, mods))
    return LIB


def clean() -> None:
    shutil.rmtree(OBJ, ignore_errors=True)


if __name__ == "__main__":
    print(build(force=True))
