"""The CPU oracle against the reference's golden vectors (no GPU).

The golden vectors in tests/golden/ were produced by the reference's own host
move generator (oracle/build_ref.sh + tests/golden/make_golden.py); these
tests pin the oracle restatement before anything is compared with it."""
import numpy as np
import pytest

import oracle as O
from conftest import fingerprint, golden_json, golden_npz, words_of_hex


@pytest.fixture(scope="module", params=[1, 0], ids=["magic", "kogge_stone"])
def orc(request):
    o = O.Oracle(request.param)
    yield o
    o.set_sliders(1)


def test_fen_boards_and_perft(orc):
    for item in golden_json("fens.json"):
        b = orc.fen(item["fen"])
        assert b.as_tuple() == words_of_hex(item["board"]), item["name"]
        for d, v in item["perft"].items():
            if int(d) <= 4 or item["name"] in ("position3", "moves218"):
                assert orc.perft(b, int(d)) == v, (item["name"], d)
        assert orc.generate_moves(b) == item["moves"], item["name"]


def test_fen_divide(orc):
    for item in golden_json("fens.json"):
        b = orc.fen(item["fen"])
        got = orc.perft_divide(b, 3)
        assert [[m, c] for m, c in got.items()] == item["divide3"], item["name"]


def test_walk_vectors(orc):
    g = golden_npz("walk.npz")
    for i in range(len(g["boards"])):
        b = O.Board(*(int(x) for x in g["boards"][i]))
        assert orc.count_moves(b) == g["counts"][i]
        mv = orc.generate_moves(b)
        n = int(g["nmoves"][i])
        assert mv == [int(x) for x in g["moves"][i][:n]]
        for k, m in enumerate(mv):
            assert fingerprint(orc.make_move(b, m).as_tuple()) == int(g["child_fp"][i][k])
        gb = orc.generate_boards(b)
        assert len(gb) == g["nboards"][i]
        assert [fingerprint(w) for w in gb] == [int(x) for x in g["boards_fp"][i][:len(gb)]]


def test_perft_via_moves_equals_boards(orc):
    for item in golden_json("fens.json")[:6]:
        b = orc.fen(item["fen"])
        assert orc.perft_moves(b, 4) == item["perft"]["4"]


def test_config1_totals_and_divide():
    orc = O.Oracle(0)  # config 1 names Kogge-Stone sliders
    g = golden_json("config1.json")
    boards = np.array([words_of_hex(p["board"]) for p in g["positions"]], dtype=np.uint64)
    depths = np.array([p["depth"] for p in g["positions"]], dtype=np.uint8)
    out, secs = orc.perft_batch(boards.view(O.BOARD_DTYPE).reshape(-1), depths, 8)
    assert [int(x) for x in out] == [p["total"] for p in g["positions"]]
    assert int(out.sum()) == g["total"]
    for p in g["positions"][:4]:
        b = O.Board(*words_of_hex(p["board"]))
        div = orc.perft_divide(b, p["depth"])
        assert [[m, c] for m, c in div.items()] == p["divide"]
    orc.set_sliders(1)


def test_playouts_match_fixture(orc):
    g = golden_json("playouts.json")
    for name, item in g.items():
        spec = item["spec"]
        n = min(len(item["fp"]), 64)
        boards, depths = orc.playouts(spec["seed"], n, spec["min_plies"], spec["max_plies"],
                                      spec["min_moves"], spec["depth_lo"], spec["depth_hi"],
                                      with_depths=True)
        got = ["%016x" % fingerprint(tuple(int(r[k]) for k in O.BOARD_DTYPE.names)) for r in boards]
        assert got == item["fp"][:n], name
        assert [int(d) for d in depths] == item["depths"][:n], name


def test_config3_sample():
    g = golden_npz("config3.npz")
    orc = O.Oracle(1)
    idx = [i for i in range(len(g["depths"])) if g["depths"][i] <= 4][:200]
    boards = g["boards"][idx].copy().view(O.BOARD_DTYPE).reshape(-1)
    out, _ = orc.perft_batch(boards, g["depths"][idx], 8)
    assert np.array_equal(out, g["totals"][idx])


@pytest.mark.skipif(not O.reference_available(), reason="reference build (x86 + sources) absent")
def test_oracle_against_reference_random_walk():
    import random
    orc, ref = O.Oracle(1), O.Reference()
    rng = random.Random(11)
    for _ in range(300):
        b = orc.fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
        for _ in range(rng.randrange(0, 100)):
            mv = orc.generate_moves(b)
            assert mv == ref.generate_moves(b)
            assert orc.generate_boards(b) == ref.generate_boards(b)
            if not mv:
                break
            m = mv[rng.randrange(len(mv))]
            assert orc.make_move(b, m).as_tuple() == ref.make_move(b, m).as_tuple()
            b = orc.make_move(b, m)
