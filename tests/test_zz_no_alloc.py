"""pg_perft_batch_noalloc -- the entry point for callers that cannot allocate
device memory (a process whose memory pool already owns the GPU, a framework
allocator that forbids side allocations): all of its working memory is one
fixed device array inside the library.  Its counts must equal the regular
batch entry point's, the reference's golden counts and the oracle's on the
same positions, on two calls in a row (the second call reuses the array the
first one left behind), and a call must leave the device's free memory
unchanged.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from conftest import golden_npz

pytestmark = pytest.mark.gpu

PG_ERR_CAPACITY = 8


def _entry():
    import perft_gpu_gb300 as pg
    lib = pg.load_library()
    return pg, lib.pg_perft_batch_noalloc


def _call(fn, boards, depths):
    import torch
    d_b = torch.from_numpy(np.ascontiguousarray(boards).view(np.uint8).copy()).cuda()
    d_d = torch.from_numpy(np.ascontiguousarray(depths, dtype=np.uint8).copy()).cuda()
    d_o = torch.full((len(boards),), -1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    st = fn(d_b.data_ptr(), d_d.data_ptr(), len(boards), d_o.data_ptr(), None)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    return st, d_o.cpu().numpy().view(np.uint64), free0, free1


def test_noalloc_matches_batch_entry_point_twice():
    import oracle as O
    pg, fn = _entry()
    pg.init()
    # call 1: the depth-3 positions of the batched workload, against the
    # reference's golden counts and the regular batch entry point
    g = golden_npz("config3.npz")
    sel = np.flatnonzero(g["depths"] <= 3)
    b1 = g["boards"][sel].copy().view(pg.BOARD_DTYPE).reshape(-1)
    d1 = g["depths"][sel].copy()
    exp1 = pg.perft_batch(b1, d1)
    assert np.array_equal(exp1, g["totals"][sel])
    st, got1, _, _ = _call(fn, b1, d1)
    assert st == 0, pg.load_library().pg_last_error()
    assert np.array_equal(got1, g["totals"][sel])
    # call 2: fresh playouts at depths 0..3, against the regular entry point
    # and the oracle; the device's free memory is the same after the call
    b2, d2 = pg.random_playouts(22, 3000, 0, 50, 1, 0, 3, with_depths=True)
    exp2 = pg.perft_batch(b2, d2)
    ref2, _ = O.Oracle(1).perft_batch(b2, d2, 8)
    assert np.array_equal(exp2, ref2)
    st, got2, free0, free1 = _call(fn, b2, d2)
    assert st == 0, pg.load_library().pg_last_error()
    assert np.array_equal(got2, exp2)
    assert int(got2.sum()) > 0
    assert free1 == free0, "the call changed the device's free memory by %d bytes" % (free1 - free0)


def test_noalloc_rejects_sizes_beyond_its_maximum():
    import torch
    pg, fn = _entry()
    d_b = torch.zeros((70000, 48), dtype=torch.uint8, device="cuda")
    d_d = torch.zeros(70000, dtype=torch.uint8, device="cuda")
    d_o = torch.zeros(70000, dtype=torch.int64, device="cuda")
    assert fn(d_b.data_ptr(), d_d.data_ptr(), 70000, d_o.data_ptr(), None) == PG_ERR_CAPACITY
    b = pg.board_from_fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    one = np.frombuffer(bytes(b), dtype=np.uint8).copy().view(pg.BOARD_DTYPE)
    st, _, _, _ = _call(fn, one, [4])
    assert st == PG_ERR_CAPACITY
    # children of the depth-3 positions, counted over both sides to move:
    # each side alone stays under 1,048,576, together they exceed it; the
    # call fails before counting and leaves zeros
    boards = pg.random_playouts(23, 40000, 4, 40, 25)
    side = boards["pawns"] >> np.uint64(63)
    kids = pg.count_moves_batch(boards).astype(np.int64)
    assert kids[side == 0].sum() < (1 << 20) and kids[side == 1].sum() < (1 << 20) < kids.sum()
    st, out, _, _ = _call(fn, boards, np.full(len(boards), 3, np.uint8))
    assert st == PG_ERR_CAPACITY
    assert not out.any()
