"""pg_perft_batch_noalloc -- the entry point for callers that cannot allocate
device memory (all of its working memory is one fixed device array inside the
library).  Its counts must equal the regular batch entry point's on the same
positions, on two calls in a row (the second call reuses the array the first
one left behind).  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PG_ERR_CAPACITY = 8


def _entry():
    import perft_gpu_gb300 as pg
    lib = pg.load_library()
    fn = lib.pg_perft_batch_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return pg, fn


def test_noalloc_matches_batch_entry_point_twice():
    import torch
    pg, fn = _entry()
    pg.init()
    for call, seed in enumerate((21, 22)):
        boards, depths = pg.random_playouts(seed, 3000, 0, 50, 1, 0, 3, with_depths=True)
        expected = pg.perft_batch(boards, depths)
        d_b = torch.from_numpy(boards.view(np.uint8).copy()).cuda()
        d_d = torch.from_numpy(depths.copy()).cuda()
        d_o = torch.full((len(boards),), -1, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        st = fn(d_b.data_ptr(), d_d.data_ptr(), len(boards), d_o.data_ptr(), None)
        assert st == 0, pg.load_library().pg_last_error()
        got = d_o.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, expected), "call %d" % call
        assert int(got.sum()) > 0


def test_noalloc_rejects_sizes_beyond_its_maximum():
    import torch
    pg, fn = _entry()
    d_b = torch.zeros((70000, 48), dtype=torch.uint8, device="cuda")
    d_d = torch.zeros(70000, dtype=torch.uint8, device="cuda")
    d_o = torch.zeros(70000, dtype=torch.int64, device="cuda")
    assert fn(d_b.data_ptr(), d_d.data_ptr(), 70000, d_o.data_ptr(), None) == PG_ERR_CAPACITY
    b = pg.board_from_fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    one = torch.from_numpy(np.frombuffer(bytes(b), dtype=np.uint8).copy()).cuda()
    d4 = torch.tensor([4], dtype=torch.uint8, device="cuda")
    o = torch.zeros(1, dtype=torch.int64, device="cuda")
    assert fn(one.data_ptr(), d4.data_ptr(), 1, o.data_ptr(), None) == PG_ERR_CAPACITY
