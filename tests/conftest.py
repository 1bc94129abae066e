"""Shared test setup: import paths, the `gpu` marker, golden-fixture loading."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "lightning-lite-quantum-simulator_gb300")
ORACLE = os.path.join(REPO, "oracle")
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (PKG, ORACLE, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: long-running GPU case")


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def load(name: str):
        if name not in cache:
            cache[name] = dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))
        return cache[name]

    return load


def split(ops, offsets):
    return [ops[offsets[k]:offsets[k + 1]] for k in range(len(offsets) - 1)]


def split_states(states, offsets):
    return [states[offsets[k]:offsets[k + 1]] for k in range(len(offsets) - 1)]


@pytest.fixture(scope="session")
def built():
    """The engine library and drop-in modules, built in-tree (no fallback if this fails)."""
    import build_ext

    build_ext.build()
    return build_ext.LIB
