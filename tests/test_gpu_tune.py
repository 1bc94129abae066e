"""Autotuners and CUDA-graph replays: the state autotuner picks a configuration that still
matches the oracle; trajectory handles replay a captured graph with the same jump decisions as
the one-shot call under every tuned (cluster, threads) shape; auto-tuned mixed batches match the
oracle per circuit."""
from __future__ import annotations

import numpy as np
import pytest

import llgpu
import oracle
import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    assert llgpu.device_count() > 0


@pytest.mark.parametrize("precision", ["df64", "complex64"])
def test_state_autotune_then_parity(precision):
    llgpu.tune_cache_clear()
    n = 16
    ops = workloads.layered_rotations(n, 4)
    st = llgpu.State(n, precision)
    res = st.autotune(ops, sample_ops=120)
    assert res["candidates"] >= 3 and res["cached"] == 0
    assert res["best_ms"] > 0 and res["default_ms"] > 0
    tun = st.tuning()
    if res["fuse_mode"] == llgpu.LLG_FUSE_TILE:
        assert tun["fuse_mode"] == "tile" and tun["tile_qubits"] == res["tile_qubits"]
        assert tun["cta_threads"] == res["cta_threads"]
    elif res["fuse_mode"] == llgpu.LLG_FUSE_REG:  # complex64 only: the register-tiled pass
        assert precision == "complex64"
        assert tun["fuse_mode"] == "reg" and tun["tile_qubits"] == res["tile_qubits"]
    else:
        assert tun["fuse_mode"] == "none"
    st.apply_ops(ops)
    tol = 1e-12 if precision == "df64" else 5e-5
    assert np.max(np.abs(st.state() - oracle.run_ops(n, ops))) <= tol
    # the same circuit shape again is a cache hit (angles do not matter)
    ops2 = ops.copy()
    ops2["theta"] += 0.25
    st2 = llgpu.State(n, precision)
    res2 = st2.autotune(ops2, sample_ops=120)
    assert res2["cached"] == 1 and res2["tile_qubits"] == res["tile_qubits"]
    st.close()
    st2.close()


@pytest.mark.parametrize("tile,threads", [(8, 128), (10, 256), (12, 512), (12, 64), (12, 1024), (11, 1024)])
def test_tile_threads_parity(tile, threads):
    n = 14
    ops = workloads.layered_rotations(n, 3)
    st = llgpu.State(n, "df64")
    st.set_fusion("tile", tile)
    st.set_tile_threads(threads)
    st.apply_ops(ops)
    assert np.max(np.abs(st.state() - oracle.run_ops(n, ops))) <= 1e-12
    with pytest.raises(ValueError):
        st.set_tile_threads(2048)
    with pytest.raises(ValueError):
        st.set_tile_threads(100)
    st.close()


@pytest.mark.parametrize("n,precision", [(10, "df64"), (14, "df64"), (14, "complex64"), (9, "fp64")])
def test_traj_handle_replays_match_one_shot(n, precision):
    ops = workloads.noisy_layers(n, 3)
    seed = 77
    z_ref, j_ref, _, _ = llgpu.traj_run(n, ops, 0.02, 0.01, seed, 300, precision=precision)
    h = llgpu.Traj(n, ops, 0.02, 0.01, 300, precision)
    for _ in range(2):  # the second launch replays the same graph
        z, j, _ = h.launch(seed, 300)
        assert np.array_equal(j, j_ref) and np.array_equal(z, z_ref)
    # a sub-range with a new seed equals the one-shot call on that range
    z2, j2, _ = h.launch(seed + 1, 120, begin=50)
    zr2, jr2, _, _ = llgpu.traj_run(n, ops, 0.02, 0.01, seed + 1, 120, begin=50, precision=precision)
    assert np.array_equal(j2, jr2) and np.array_equal(z2, zr2)
    with pytest.raises(ValueError):
        h.launch(seed, 301)
    h.close()


@pytest.mark.parametrize("n,precision", [(14, "df64"), (14, "complex64"), (11, "df64")])
def test_traj_autotune_keeps_decisions(n, precision):
    llgpu.tune_cache_clear()
    ops = workloads.noisy_layers(n, 3)
    z_ref, j_ref, _, _ = llgpu.traj_run(n, ops, 0.02, 0.01, 5, 400, precision=precision)
    h = llgpu.Traj(n, ops, 0.02, 0.01, 400, precision)
    res = h.autotune()
    cfg = h.config()
    assert res["candidates"] >= 1 and cfg["cluster"] == res["cluster"] and cfg["cta_threads"] == res["cta_threads"]
    if n == 14 and precision == "df64":
        assert cfg["cluster"] == 2  # 256 KiB of amplitudes never fit one CTA
    z, j, _ = h.launch(5, 400)
    # jump choices are the same; <Z0> differs only by the reduction order of the tuned shape
    assert np.array_equal(j, j_ref)
    assert np.max(np.abs(z - z_ref)) <= (1e-12 if precision != "complex64" else 1e-5)
    h.close()
    # every explicit shape also agrees
    for cl, th in [(1, 256), (2, 512), (1, 1024)]:
        try:
            h2 = llgpu.Traj(n, ops, 0.02, 0.01, 400, precision, cluster=cl, cta_threads=th)
        except ValueError:
            continue  # the shape cannot hold this state
        _, j2, _ = h2.launch(5, 400)
        assert np.array_equal(j2, j_ref), (cl, th)
        h2.close()


def test_batch_autotune_parity():
    llgpu.tune_cache_clear()
    rng = np.random.default_rng(9)
    nq, ops, off = workloads.mixed_batch(24, 8, 14, 60, seed=int(rng.integers(1 << 30)))
    res = llgpu.batch_autotune(nq, ops, off, "df64")
    assert res["candidates"] >= 2 and 8 <= res["tile_qubits"] <= 13
    b = llgpu.Batch(nq, ops, off, "df64", llgpu.TUNE_AUTO)
    assert b.info()["tile_qubits"] == res["tile_qubits"]
    for _ in range(2):  # graph replay
        b.run()
        for i in (0, 5, 23):
            want = oracle.run_ops(int(nq[i]), ops[off[i]:off[i + 1]])
            assert np.max(np.abs(b.state(i) - want)) <= 1e-12
    b.close()
