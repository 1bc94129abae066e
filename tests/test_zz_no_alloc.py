"""llg_expect_zz_noalloc: the expectation-value reduction for callers that cannot allocate GPU
memory (their device memory is owned by another allocator, or cudaMalloc/cudaFree would
synchronise a latency-critical loop).  The test owns the device buffers (allocated with torch)
and checks, on two calls in a row per precision, that the allocation-free entry point returns
what the existing llg_expect_zz entry point returns, within the tolerances the other tests use.

Kept in a file of its own, collected last."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import llgpu

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "df64": 1e-12, "complex64": 1e-6}


def device_layout(psi: np.ndarray, precision: str) -> np.ndarray:
    """Host array with the engine's HBM element layout for `precision`."""
    if precision == "fp64":
        return np.ascontiguousarray(psi).view(np.float64)
    if precision == "complex64":
        return np.ascontiguousarray(psi.astype(np.complex64)).view(np.float32)
    hr = psi.real.astype(np.float32)
    hi = psi.imag.astype(np.float32)
    lr = (psi.real - hr.astype(np.float64)).astype(np.float32)
    li = (psi.imag - hi.astype(np.float64)).astype(np.float32)
    return np.ascontiguousarray(np.stack([hr, hi, lr, li], axis=1)).reshape(-1)


def call_noalloc(d_amps, n, precision, a, b, c, d_out, stream) -> int:
    aa = np.ascontiguousarray(a, dtype=np.int32)
    bb = np.ascontiguousarray(b, dtype=np.int32)
    cc = np.ascontiguousarray(c, dtype=np.float64)
    return llgpu.lib().llg_expect_zz_noalloc(d_amps, n, llgpu.PRECISIONS[precision], aa.size, aa.ctypes.data,
                                              bb.ctypes.data, cc.ctypes.data, d_out, stream)


def test_noalloc_expectation_matches_existing_entry_point(built):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    n = 16
    a, b, c = llgpu.ring_zz_terms(n)
    a, b, c = a + [0, 5], b + [-1, -1], c + [0.5, -0.25]
    rng = np.random.default_rng(2718)
    stream = torch.cuda.current_stream().cuda_stream
    for precision in ("fp64", "df64", "complex64"):
        for _ in range(2):  # two calls in a row share the scratch array
            psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
            psi /= np.linalg.norm(psi)
            st = llgpu.State(precision=precision, amps=psi)
            want = st.expect_zz(a, b, c)
            want_norm = st.norm2()
            st.close()
            d_amps = torch.from_numpy(device_layout(psi, precision)).cuda()
            d_out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
            rc = call_noalloc(d_amps.data_ptr(), n, precision, a, b, c, d_out.data_ptr(), stream)
            assert rc == 0, llgpu.last_error()
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            assert abs(got[0] - want) <= TOL[precision], (precision, got[0], want)
            assert abs(got[1] - want_norm) <= TOL[precision]


def test_noalloc_large_then_small_call(built):
    # a 22-qubit state fills every one of the 1024 scratch rows (the grid cap binds and the blocks
    # stride past it); a 12-qubit call right after it on the same stream reads only its own rows
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(99)
    for n in (22, 12):
        a, b, c = llgpu.ring_zz_terms(n)
        psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        psi /= np.linalg.norm(psi)
        st = llgpu.State(precision="fp64", amps=psi)
        want, want_norm = st.expect_zz(a, b, c), st.norm2()
        st.close()
        d_amps = torch.from_numpy(device_layout(psi, "fp64")).cuda()
        d_out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        assert call_noalloc(d_amps.data_ptr(), n, "fp64", a, b, c, d_out.data_ptr(), stream) == 0, llgpu.last_error()
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert abs(got[0] - want) <= TOL["fp64"] and abs(got[1] - want_norm) <= TOL["fp64"], (n, got, want)


def test_noalloc_rejects_sizes_beyond_its_limits(built):
    torch = pytest.importorskip("torch")
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    assert call_noalloc(d.data_ptr(), 35, "fp64", [0], [-1], [1.0], out.data_ptr(), None) == llgpu.LLG_EINVAL
    assert "n_qubits" in llgpu.last_error()
    assert call_noalloc(d.data_ptr(), 2, "fp64", [0] * 65, [-1] * 65, [1.0] * 65, out.data_ptr(), None) == llgpu.LLG_EINVAL
    assert "terms" in llgpu.last_error()
    host = np.zeros(8)
    assert call_noalloc(host.ctypes.data, 2, "fp64", [0], [-1], [1.0], out.data_ptr(), None) == llgpu.LLG_EINVAL
    assert "device" in llgpu.last_error()
