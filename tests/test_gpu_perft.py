"""GPU perft against the reference's counts (golden vectors), bit-exact, and
size-independent properties at the full workload sizes."""
import numpy as np
import pytest

from conftest import golden_json, golden_npz, words_of_hex

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("slider", ["ks", "fancy", "byte", "hybrid"])
def test_reference_fens_perft(pg, slider):
    for item in golden_json("fens.json"):
        b = pg.board_from_fen(item["fen"])
        for d, v in item["perft"].items():
            assert pg.perft(b, int(d), slider=slider) == v, (item["name"], d, slider)


@pytest.mark.parametrize("block", [128, 256, 512])
def test_block_sizes(pg, block):
    item = golden_json("fens.json")[1]
    b = pg.board_from_fen(item["fen"])
    assert pg.perft(b, 5, block_size=block) == item["perft"]["5"]


def test_divide_matches_reference(pg):
    for item in golden_json("fens.json"):
        b = pg.board_from_fen(item["fen"])
        assert [[m, c] for m, c in pg.perft_divide(b, 3)] == item["divide3"], item["name"]


def test_depth_edges(pg):
    b = pg.board_from_fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    assert pg.perft(b, 0) == 1
    assert pg.perft(b, 1) == 20
    assert pg.perft(b, 2) == 400
    mate = pg.board_from_fen("rnb1kbnr/pppp1ppp/8/4p3/6Pq/5P2/PPPPP2P/RNBQKBNR w KQkq - 1 3")
    assert pg.count_moves(mate) == 0
    assert pg.perft(mate, 1) == 0 and pg.perft(mate, 3) == 0
    stale = pg.board_from_fen("7k/5Q2/6K1/8/8/8/8/8 b - - 0 1")
    assert pg.count_moves(stale) == 0 and pg.perft(stale, 4) == 0
    out = pg.perft_batch(np.zeros(0, dtype=pg.BOARD_DTYPE), [])
    assert len(out) == 0


def test_config1_batch_and_divide(pg):
    g = golden_json("config1.json")
    boards = np.array([words_of_hex(p["board"]) for p in g["positions"]], dtype=np.uint64)
    boards = boards.view(pg.BOARD_DTYPE).reshape(-1)
    depths = [p["depth"] for p in g["positions"]]
    out = pg.perft_batch(boards, depths, slider="ks")
    assert [int(x) for x in out] == [p["total"] for p in g["positions"]]
    for p in g["positions"][:8]:
        got = pg.perft_divide(pg.HexaBitBoardPosition(*words_of_hex(p["board"])), p["depth"])
        assert [[m, c] for m, c in got] == p["divide"]


def test_config2_deep_single_position(pg):
    g = golden_json("config2.json")
    b = pg.HexaBitBoardPosition(*words_of_hex(g["board"]))
    assert pg.count_moves(b) >= 35
    assert pg.perft(b, 5) == g["perft5"]
    assert pg.perft(b, 6) == g["perft6"]
    assert [[m, c] for m, c in pg.perft_divide(b, 6)] == g["divide6"]


@pytest.mark.slow
def test_config2_depth7(pg):
    g = golden_json("config2.json")
    b = pg.HexaBitBoardPosition(*words_of_hex(g["board"]))
    assert pg.perft(b, 7) == g["perft7"]


def test_config3_batched_uneven(pg):
    g = golden_npz("config3.npz")
    boards = g["boards"].copy().view(pg.BOARD_DTYPE).reshape(-1)
    out = pg.perft_batch(boards, g["depths"])
    assert np.array_equal(out, g["totals"])


def test_config3_playouts_regenerate_on_gpu(pg):
    g = golden_npz("config3.npz")
    boards, depths = pg.random_playouts(3, 4096, 0, 60, 1, 3, 6, with_depths=True)
    assert np.array_equal(boards.view(np.uint64).reshape(-1, 6), g["boards"])
    assert np.array_equal(depths, g["depths"])


def test_chunked_levels_small_budget(pg):
    """A small HBM budget forces every expansion into many chunks."""
    item = golden_json("fens.json")[1]
    pg.shutdown()
    pg.init(hbm_budget_bytes=64 << 20)
    try:
        b = pg.board_from_fen(item["fen"])
        assert pg.perft(b, 5) == item["perft"]["5"]
        g = golden_npz("config4_d5.npz")
        boards = g["boards"][:64].copy().view(pg.BOARD_DTYPE).reshape(-1)
        assert np.array_equal(pg.perft_batch(boards, [5] * 64), g["totals"][:64])
    finally:
        pg.shutdown()
        pg.init()


def test_batch_equals_sum_of_singles(pg):
    """Each result alone equals its result inside a mixed batch."""
    g = golden_npz("config3.npz")
    idx = np.arange(0, 4096, 97)
    boards = g["boards"][idx].copy().view(pg.BOARD_DTYPE).reshape(-1)
    depths = np.minimum(g["depths"][idx], 5)
    mixed = pg.perft_batch(boards, depths)
    alone = [pg.perft(pg.board_of(boards[i]), int(depths[i])) for i in range(len(idx))]
    assert [int(x) for x in mixed] == alone


def test_switch_depth_one_ply_leaf(pg):
    """Breadth-first down to the leaf-parents, count-only leaf: same counts."""
    for item in golden_json("fens.json")[:4]:
        b = pg.board_from_fen(item["fen"])
        for d in ("3", "4", "5"):
            assert pg.perft(b, int(d), leaf_plies=1, slider="ks") == item["perft"][d]
    g = golden_npz("config3.npz")
    idx = np.arange(0, 4096, 13)
    boards = g["boards"][idx].copy().view(pg.BOARD_DTYPE).reshape(-1)
    depths = np.minimum(g["depths"][idx], 5)
    assert np.array_equal(pg.perft_batch(boards, depths, leaf_plies=1, slider="fancy"),
                          pg.perft_batch(boards, depths, slider="ks"))


def test_autotuner_choices_and_auto_counts(pg):
    t = pg.autotune()
    assert t["leaf_plies"] in (1, 2) and t["seconds"] > 0
    for d, c in t["per_depth"].items():
        assert c["slider"] in ("ks", "fancy", "byte", "hybrid") and c["block_size"] in (128, 256, 512)
        assert c["calibration_leaves_per_s"] > 0
    g = golden_npz("config3.npz")
    idx = np.arange(0, 4096, 29)
    boards = g["boards"][idx].copy().view(pg.BOARD_DTYPE).reshape(-1)
    assert np.array_equal(pg.perft_batch(boards, g["depths"][idx]), g["totals"][idx])


def test_graph_capture_and_replay(pg):
    """First call records its plan and captures a graph; repeats replay it;
    new contents at the same pointers are detected and recaptured."""
    g = golden_npz("config3.npz")
    idx = np.arange(0, 4096, 11)
    boards = g["boards"][idx].copy().view(pg.BOARD_DTYPE).reshape(-1)
    depths = g["depths"][idx].copy()
    seen = []
    for k in range(3):
        st = pg.PgStats()
        out = pg.perft_batch(boards, depths, graph=True, stats=st)
        assert np.array_equal(out, g["totals"][idx])
        seen.append((st.graph_captures, st.graph_replays))
    assert seen[0] == (1, 0) and seen[1] == (0, 1) and seen[2] == (0, 1)
    other = np.arange(1, 4096, 11)[:len(idx)]
    b2 = g["boards"][other].copy().view(pg.BOARD_DTYPE).reshape(-1)
    st = pg.PgStats()
    out2 = pg.perft_batch(b2, g["depths"][other], graph=True, stats=st)
    assert np.array_equal(out2, g["totals"][other]) and st.graph_captures == 1


def test_graph_recaptured_after_buffers_are_reallocated(pg):
    """A captured graph names the engine's level and scan buffers.  A later
    call that grows those buffers (here: a batch with a much larger first
    level) frees the ones the graph was captured with, so the next graph call
    on the same inputs must capture again, never replay into freed memory."""
    import torch
    pg.shutdown()
    pg.init()
    g = golden_npz("config3.npz")
    idx = np.arange(0, 4096, 11)
    d_b = torch.from_numpy(g["boards"][idx].copy().view(np.uint8)).cuda()
    d_d = torch.from_numpy(g["depths"][idx].copy()).cuda()
    d_o = torch.zeros(len(idx), dtype=torch.int64, device="cuda")

    def graph_call():
        st = pg.PgStats()
        pg.perft_batch_device(d_b.data_ptr(), d_d.data_ptr(), len(idx), d_o.data_ptr(), slider="ks",
                              graph=True, stats=st)
        assert np.array_equal(d_o.cpu().numpy().view(np.uint64), g["totals"][idx])
        return st.graph_captures, st.graph_replays

    assert graph_call() == (1, 0)
    assert graph_call() == (0, 1)
    big, big_d = pg.random_playouts(31, 20000, 0, 40, 1, 3, 3, with_depths=True)
    assert pg.perft_batch(big, big_d, slider="ks").sum() > 0
    assert graph_call() == (1, 0)
    assert graph_call() == (0, 1)


def test_persistent_launch_matches_golden(pg):
    """The whole batch as one persistent cooperative launch (levels, chunks
    and phases walked on the device): the reference's golden counts, one
    kernel launch per call."""
    import torch
    g = golden_npz("config3.npz")
    idx = np.arange(0, 4096, 7)
    boards = g["boards"][idx].copy().view(pg.BOARD_DTYPE).reshape(-1)
    st = pg.PgStats()
    out = pg.perft_batch(boards, g["depths"][idx], persistent=True, stats=st)
    assert np.array_equal(out, g["totals"][idx])
    assert st.launches == 1
    # every golden FEN depth in one mixed batch (depths 0..2 take only the leaf phase)
    bs, ds, want = [], [], []
    for f in golden_json("fens.json"):
        b = pg.board_from_fen(f["fen"])
        for d, v in f["perft"].items():
            if int(d) <= 5:
                bs.append(b)
                ds.append(int(d))
                want.append(v)
    assert [int(x) for x in pg.perft_batch(pg.boards_array(bs), ds, persistent=True)] == want
    # device pointers (the largest depth is read back once)
    d_b = torch.from_numpy(g["boards"][idx].copy().view(np.uint8)).cuda()
    d_d = torch.from_numpy(g["depths"][idx].copy()).cuda()
    d_o = torch.zeros(len(idx), dtype=torch.int64, device="cuda")
    pg.perft_batch_device(d_b.data_ptr(), d_d.data_ptr(), len(idx), d_o.data_ptr(), persistent=True)
    assert np.array_equal(d_o.cpu().numpy().view(np.uint64), g["totals"][idx])


def test_persistent_launch_deep_position(pg):
    g = golden_json("config2.json")
    b = pg.HexaBitBoardPosition(*words_of_hex(g["board"]))
    assert pg.perft(b, 7, persistent=True) == g["perft7"]


def test_persistent_launch_chunked_small_budget(pg):
    """A 64 MB budget gives the persistent launch small levels: the device
    splits levels into many chunks and walks them depth first."""
    item = golden_json("fens.json")[1]
    pg.shutdown()
    pg.init(hbm_budget_bytes=64 << 20)
    try:
        b = pg.board_from_fen(item["fen"])
        assert pg.perft(b, 5, persistent=True) == item["perft"]["5"]
        g = golden_npz("config4_d5.npz")
        boards = g["boards"][:64].copy().view(pg.BOARD_DTYPE).reshape(-1)
        assert np.array_equal(pg.perft_batch(boards, [5] * 64, persistent=True), g["totals"][:64])
    finally:
        pg.shutdown()
        pg.init()


def test_persistent_graph_replays_any_contents(pg):
    """The persistent launch captured in a graph plans its chunks on the
    device: new contents in the same buffers (same size and largest depth)
    replay the same graph and give their own golden counts."""
    import torch
    g = golden_npz("config3.npz")
    b = np.arange(5, 4096, 13)
    a = np.arange(0, 4096, 13)[:len(b)]
    sel = [a, b]
    assert g["depths"][a].max() == g["depths"][b].max()
    d_b = torch.from_numpy(g["boards"][a].copy().view(np.uint8)).cuda()
    d_d = torch.from_numpy(g["depths"][a].copy()).cuda()
    d_o = torch.zeros(len(a), dtype=torch.int64, device="cuda")
    seen = []
    for k in range(4):
        idx = sel[k // 2]
        d_b.copy_(torch.from_numpy(g["boards"][idx].copy().view(np.uint8)))
        d_d.copy_(torch.from_numpy(g["depths"][idx].copy()))
        st = pg.PgStats()
        pg.perft_batch_device(d_b.data_ptr(), d_d.data_ptr(), len(idx), d_o.data_ptr(), graph=True,
                              persistent=True, stats=st)
        assert np.array_equal(d_o.cpu().numpy().view(np.uint64), g["totals"][idx]), k
        seen.append((st.graph_captures, st.graph_replays))
    assert seen == [(1, 0), (0, 1), (0, 1), (0, 1)]
