"""Parity on positions no fixture holds: fresh seeded random playouts,
counted on the GPU (batched, every slider policy) and by the oracle on the
host in the same run.  Playouts run up to 120 plies with a filter of at
least one legal move, so checks, pins, promotions, en passant and castling
rights all occur; the depths keep the oracle's work to a few seconds."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def orc():
    import oracle
    oracle.build()
    return oracle.Oracle(1)


@pytest.mark.parametrize("seed,n,depth", [(11, 200000, 3), (12, 20000, 4)])
def test_random_playouts_match_oracle(pg, orc, seed, n, depth):
    boards = pg.random_playouts(seed, n, 0, 120, 1)
    depths = np.full(n, depth, dtype=np.uint8)
    want, _ = orc.perft_batch(boards, depths, os.cpu_count() or 1)
    for sl in ("ks", "fancy", "byte", "hybrid"):
        got = pg.perft_batch(boards, depths, slider=sl)
        bad = np.nonzero(got != want)[0]
        assert len(bad) == 0, (sl, int(bad[0]), int(got[bad[0]]), int(want[bad[0]]))


def test_random_playouts_mixed_depths_with_tt(pg, orc):
    boards, depths = pg.random_playouts(13, 20000, 0, 120, 1, 1, 4, with_depths=True)
    want, _ = orc.perft_batch(boards, depths, os.cpu_count() or 1)
    pg.tt_clear()
    got = pg.perft_batch(boards, depths, use_tt=True, tt_bytes=256 << 20)
    pg.tt_clear()
    assert np.array_equal(got, want)


def test_random_playouts_persistent_and_dedup_match_oracle(pg, orc):
    """The persistent launch and the in-level duplicate pass on fresh
    playouts of mixed depth, against the oracle."""
    boards, depths = pg.random_playouts(14, 20000, 0, 120, 1, 0, 4, with_depths=True)
    want, _ = orc.perft_batch(boards, depths, os.cpu_count() or 1)
    got = pg.perft_batch(boards, depths, persistent=True)
    bad = np.nonzero(got != want)[0]
    assert len(bad) == 0, ("persistent", int(bad[0]), int(got[bad[0]]), int(want[bad[0]]))
    got = pg.perft_batch(boards, depths, use_tt="dedup")
    assert np.array_equal(got, want)
