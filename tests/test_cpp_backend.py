"""ll::GpuBackend (include/ll_gpu_backend.h), the C++ drop-in for ll::StateVectorBackend."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

import build_oracle
import llgpu
from conftest import PKG, REPO

_REF = build_oracle.reference_root()
REF_SRC = os.path.join(_REF, "src") if _REF else ""
CPP = os.path.join(REPO, "tests", "cpp")
BUILD = os.path.join(PKG, "_build", "cpp_tests")


def compile_driver(src: str, out: str, iface: str) -> str:
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, out)
    cmd = ["g++", "-O2", "-std=c++17", "-I" + iface, "-I" + os.path.join(REPO, "include"),
           os.path.join(CPP, src), "-o", exe, "-L" + PKG, "-lllgpu", "-Wl,-rpath," + PKG]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.skipif(not REF_SRC, reason="reference tree not present on this machine")
def test_reference_algorithms_compile_against_gpu_backend(built, golden):
    exe = compile_driver("reference_algorithms_on_gpu.cpp", "ref_alg_gpu", REF_SRC)
    v = golden("vqe_param_shift")
    theta = v["n4_l2_theta"]
    r = subprocess.run([exe] + [repr(float(t)) for t in theta], capture_output=True, text=True, timeout=120)
    if llgpu.device_count() == 0:
        assert r.returncode == 4 and "runtime_error" in r.stderr  # loud failure, no CPU fallback
        return
    assert r.returncode == 0, r.stderr
    lines = {ln.split()[0]: ln.split()[1:] for ln in r.stdout.strip().split("\n")}
    it, mi, p = lines["grover"]
    assert int(it) == 12 and int(mi) == 85 and abs(float(p) - 0.99994704) < 5e-9
    a = golden("algorithms")
    q = [float(x) for x in lines["qaoa"]]
    assert q[0] == float(a["qaoa_ring4_p1_best_cut"])
    assert np.max(np.abs(np.array(q[1:]) - a["qaoa_ring4_p1_probs"])) <= 1e-12
    probs = np.array([float(x) for x in lines["vqe"]])
    assert np.max(np.abs(probs - np.abs(v["n4_l2_state"]) ** 2)) <= 1e-12


def test_restated_interface_matches_reference_signatures():
    # the restated interface (tests/cpp/iface/Backend.h) must declare the same virtuals as the
    # reference's src/Backend.h:25-45
    import re

    ours = open(os.path.join(CPP, "iface", "Backend.h")).read()
    sigs = sorted(set(re.findall(r"virtual ([^;{]+?)\s*=\s*0;", ours)))
    assert len(sigs) == 11
    if REF_SRC:
        ref = open(os.path.join(REF_SRC, "Backend.h")).read()
        ref_block = ref[ref.index("class Backend {"):ref.index("};", ref.index("class Backend {"))]
        ref_sigs = sorted(set(re.findall(r"virtual ([^;{]+?)\s*=\s*0;", ref_block)))
        norm = lambda s: re.sub(r"\s+", " ", s.replace("control", "c").replace("target", "t"))  # noqa: E731
        assert [norm(s) for s in sigs] == [norm(s) for s in ref_sigs]


@pytest.mark.gpu
def test_grover_through_gpu_backend(built, golden):
    exe = compile_driver("grover_on_gpu_backend.cpp", "grover_gpu", os.path.join(CPP, "iface"))
    g = golden("grover")
    for key, n in (("n8_m85", 8), ("n10_i10", 10)):
        args = [exe, str(n), str(int(g[key + "_iterations"]))] + [str(m) for m in g[key + "_marked"]]
        r = subprocess.run(args, capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr
        p = np.array([float(x) for x in r.stdout.split()])
        assert np.max(np.abs(p - g[key + "_probs"])) <= 1e-12


def test_gpu_zne_header_compiles_and_validates(built):
    # CPU side: the driver builds against the restated interface; bad arguments are rejected on
    # the host before any GPU work (p out of range -> invalid_argument)
    exe = compile_driver("zne_on_gpu.cpp", "zne_gpu", os.path.join(CPP, "iface"))
    r = subprocess.run([exe, "1.5", "10"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 3 and "p must be in [0, 1]" in r.stderr


@pytest.mark.gpu
def test_gpu_zne_through_the_cpp_interface(built):
    exe = compile_driver("zne_on_gpu.cpp", "zne_gpu", os.path.join(CPP, "iface"))
    r = subprocess.run([exe, "0.03", "40000"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    value, se = (float(x) for x in lines[0].split())
    r2 = 1 - 16 * 0.03 / 15
    for line in lines[1:3]:
        s, v, e = (float(x) for x in line.split())
        assert abs(v - r2 ** s) < 5 * e
    assert abs(value - 1.0) < abs(float(lines[1].split()[1]) - 1.0)  # mitigated closer to the ideal 1
