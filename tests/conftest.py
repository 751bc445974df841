"""Shared fixtures.  Tests marked `gpu` need a CUDA device (sm_103a); the
rest run on any host."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")
    config.addinivalue_line("markers", "slow: long-running parity case")


def golden_json(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def golden_npz(name):
    """All arrays of a fixture, loaded once (an NpzFile re-reads on every index)."""
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def words_of_hex(hexes):
    return tuple(int(h, 16) for h in hexes)


MASK64 = (1 << 64) - 1


def fingerprint(words) -> int:
    """Same 64-bit fingerprint as tests/golden/make_golden.py."""
    h = 0xCBF29CE484222325
    for w in words:
        h ^= int(w)
        h = (h * 0x100000001B3) & MASK64
        h ^= h >> 29
    return h


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    return O.Oracle(1)


@pytest.fixture(scope="session")
def pg():
    """The GPU engine, initialised once per test session."""
    import perft_gpu_gb300 as pg
    pg.load_library()
    pg.init()
    yield pg
