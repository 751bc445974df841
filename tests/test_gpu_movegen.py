"""GPU operator surface (countMoves / generateMoves / generateBoards /
makeMove / playouts) against the reference's golden vectors, bit-exact."""
import numpy as np
import pytest

from conftest import fingerprint, golden_json, golden_npz, words_of_hex

pytestmark = pytest.mark.gpu


def _walk():
    g = golden_npz("walk.npz")
    import perft_gpu_gb300 as pg
    boards = g["boards"].copy().view(pg.BOARD_DTYPE).reshape(-1)
    return g, boards


@pytest.mark.parametrize("slider", ["ks", "fancy", "byte", "hybrid"])
def test_count_moves_batch_matches_reference(pg, slider):
    g, boards = _walk()
    pg.shutdown()
    pg.init(slider=slider)
    try:
        assert np.array_equal(pg.count_moves_batch(boards), g["counts"])
    finally:
        pg.shutdown()
        pg.init()


def test_generate_moves_order_and_flags(pg):
    g, boards = _walk()
    for i in range(0, len(boards), 3):
        b = pg.board_of(boards[i])
        n = int(g["nmoves"][i])
        assert pg.generate_moves(b) == [int(x) for x in g["moves"][i][:n]], i


def test_make_move_children_bit_exact(pg):
    g, boards = _walk()
    for i in range(0, len(boards), 7):
        b = pg.board_of(boards[i])
        n = int(g["nmoves"][i])
        for k in range(n):
            child = pg.make_move(b, int(g["moves"][i][k]))
            assert fingerprint(child.words()) == int(g["child_fp"][i][k]), (i, k)


def test_generate_boards_bit_exact(pg):
    g, boards = _walk()
    for i in range(0, len(boards), 5):
        got = pg.generate_boards(pg.board_of(boards[i]))
        assert len(got) == g["nboards"][i]
        assert [fingerprint(x.words()) for x in got] == [int(v) for v in g["boards_fp"][i][:len(got)]]


def test_reference_fens_moves(pg):
    for item in golden_json("fens.json"):
        b = pg.board_from_fen(item["fen"])
        assert b.words() == words_of_hex(item["board"])
        assert pg.count_moves(b) == item["perft"]["1"]
        assert pg.generate_moves(b) == item["moves"]


def test_gpu_playouts_match_oracle_fixture(pg):
    import perft_gpu_gb300 as P
    for name, item in golden_json("playouts.json").items():
        spec = item["spec"]
        n = len(item["fp"])
        boards, depths = pg.random_playouts(spec["seed"], n, spec["min_plies"], spec["max_plies"],
                                            spec["min_moves"], spec["depth_lo"], spec["depth_hi"],
                                            with_depths=True)
        got = ["%016x" % fingerprint(tuple(int(r[k]) for k in P.BOARD_DTYPE.names)) for r in boards]
        assert got == item["fp"], name
        assert [int(d) for d in depths] == item["depths"], name


def test_invalid_positions_rejected(pg):
    b = pg.board_from_fen("8/8/8/8/8/8/8/8 w - - 0 1")  # no kings
    with pytest.raises(pg.PerftError) as e:
        pg.count_moves(b)
    assert e.value.status == 3
    b = pg.board_from_fen("k7/8/8/8/8/8/8/KK6 w - - 0 1")  # two white kings
    with pytest.raises(pg.PerftError):
        pg.perft(b, 2)
