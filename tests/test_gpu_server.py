"""Continuous-batching server: requests of mixed depth submitted while others
run; each result must equal the reference's golden count and the result of
the same request computed alone."""
import time

import numpy as np
import pytest

from conftest import golden_json, golden_npz, words_of_hex

pytestmark = pytest.mark.gpu


def test_server_mixed_requests_match_alone_and_golden(pg):
    g3 = golden_npz("config3.npz")
    g2 = golden_json("config2.json")
    fens = {f["name"]: f for f in golden_json("fens.json")}
    deep = pg.HexaBitBoardPosition(*words_of_hex(g2["board"]))
    pos2 = pg.board_from_fen(fens["position2"]["fen"])
    idx = np.arange(0, 4096, 41)
    boards = g3["boards"][idx].copy().view(pg.BOARD_DTYPE).reshape(-1)
    srv = pg.Server(hbm_budget_bytes=1 << 30, max_inflight=512)
    try:
        want = {}
        want[srv.submit(deep, 7)] = g2["perft7"]            # deep request first: 8.7e10 leaves
        for k, i in enumerate(idx[:50]):
            want[srv.submit(pg.board_of(boards[k]), int(g3["depths"][i]))] = int(g3["totals"][i])
        time.sleep(0.02)                                      # more arrive while the deep one runs
        want[srv.submit(pos2, 6)] = fens["position2"]["perft"]["6"] if "6" in fens["position2"]["perft"] else None
        for k, i in enumerate(idx[50:], start=50):
            want[srv.submit(pg.board_of(boards[k]), int(g3["depths"][i]))] = int(g3["totals"][i])
        got = {rid: srv.wait(rid, timeout=300)[0] for rid in want}
    finally:
        srv.stop()
    for rid, w in want.items():
        if w is not None:
            assert got[rid] == w, rid
    # the same requests alone
    assert pg.perft(pos2, 6) == [v for r, v in got.items() if want[r] is None][0]
    for k, i in enumerate(idx[:10]):
        assert pg.perft(pg.board_of(boards[k]), int(g3["depths"][i])) == int(g3["totals"][i])


def test_server_rejects_invalid_and_reports_latency(pg):
    srv = pg.Server(hbm_budget_bytes=64 << 20, max_inflight=4)
    try:
        with pytest.raises(pg.PerftError):
            srv.submit(pg.board_from_fen("8/8/8/8/8/8/8/8 w - - 0 1"), 3)
        b = pg.board_from_fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
        ids = [srv.submit(b, d) for d in (1, 2, 3, 4, 5, 6, 0)]
        res = [srv.wait(i) for i in ids]
    finally:
        srv.stop()
    assert [r for r, _ in res] == [20, 400, 8902, 197281, 4865609, 119060324, 1]
    assert all(lat >= 0 for _, lat in res)


def test_server_with_tt_matches_golden_and_repeats(pg):
    """Served through the transposition tables: each count equals the golden
    count; the same requests submitted again (the tables now hold their
    subtrees) give the same counts."""
    g3 = golden_npz("config3.npz")
    g2 = golden_json("config2.json")
    deep = pg.HexaBitBoardPosition(*words_of_hex(g2["board"]))
    idx = np.arange(7, 4096, 53)
    boards = g3["boards"][idx].copy().view(pg.BOARD_DTYPE).reshape(-1)
    pg.tt_clear()
    srv = pg.Server(hbm_budget_bytes=1 << 30, max_inflight=256, use_tt=True, tt_bytes=1 << 30)
    try:
        for _ in range(2):
            want = {srv.submit(deep, 7): g2["perft7"]}
            for k, i in enumerate(idx):
                want[srv.submit(pg.board_of(boards[k]), int(g3["depths"][i]))] = int(g3["totals"][i])
            got = {rid: srv.wait(rid, timeout=300)[0] for rid in want}
            assert got == want
    finally:
        srv.stop()
        pg.tt_clear()


def test_short_request_overtakes_running_deep_one(pg):
    """A short request submitted while a deep one runs is admitted at the next
    wave boundary and finishes long before the deep one (waves are a few
    milliseconds of work, filled by least remaining work first)."""
    g2 = golden_json("config2.json")
    fens = {f["name"]: f for f in golden_json("fens.json")}
    deep = pg.HexaBitBoardPosition(*words_of_hex(g2["board"]))
    pos2 = pg.board_from_fen(fens["position2"]["fen"])
    assert pg.perft(deep, 5) > 0                              # autotuner and tables ready
    srv = pg.Server(hbm_budget_bytes=1 << 30, max_inflight=16)
    try:
        t_deep = time.perf_counter()
        rid_deep = srv.submit(deep, 7)                        # 8.7e10 leaves
        time.sleep(0.005)
        t_short = time.perf_counter()
        rid_short = srv.submit(pos2, 4)
        n_short, lat_short = srv.wait(rid_short, timeout=300)
        n_deep, lat_deep = srv.wait(rid_deep, timeout=300)
    finally:
        srv.stop()
    assert n_short == fens["position2"]["perft"]["4"]
    assert n_deep == g2["perft7"]
    # completion times on the host clock: the short one first, by a margin
    assert t_short + lat_short / 1e3 < t_deep + lat_deep / 1e3 - 0.02, (lat_short, lat_deep)


def test_hbm_admission_binds_and_no_request_starves(pg):
    """A frontier pool that holds only one or two deep requests' frontiers at
    once (3,200 positions; a depth-7 request keeps its positions two plies
    below the root, about 1,000-2,500 of them, on the device): several deep requests
    submitted together are admitted as space frees up, first in line first.
    Every count equals the batch engine's count of the same request, every
    request completes, and the counters show that memory, not slots, bounded
    admission."""
    g2 = golden_json("config2.json")
    deep = pg.HexaBitBoardPosition(*words_of_hex(g2["board"]))
    boards, _ = pg.random_playouts(57, 8, 10, 30, 32, with_depths=True)
    reqs = [(pg.board_of(b), 7) for b in boards] + [(deep, 7)]
    want = pg.perft_batch(pg.boards_array([b for b, _ in reqs]), [d for _, d in reqs])
    assert int(want[-1]) == g2["perft7"]
    srv = pg.Server(hbm_budget_bytes=3200 * 48, max_inflight=64)
    try:
        ids = [srv.submit(b, d) for b, d in reqs]
        got = [srv.wait(r, timeout=300)[0] for r in ids]
        st = srv.stats()
    finally:
        srv.stop()
    assert got == [int(x) for x in want]
    assert st["completed"] == st["submitted"] == len(reqs)
    assert st["admissions_deferred"] > 0
    assert st["max_active"] >= 2
    assert 0 < st["pool_peak"] <= st["pool_capacity"] == 3200


def test_server_persistent_waves_match_golden(pg):
    """Waves run as one persistent launch each: every count equals the
    reference's golden count, with requests arriving while others run."""
    g3 = golden_npz("config3.npz")
    g2 = golden_json("config2.json")
    deep = pg.HexaBitBoardPosition(*words_of_hex(g2["board"]))
    idx = np.arange(3, 4096, 37)
    boards = g3["boards"][idx].copy().view(pg.BOARD_DTYPE).reshape(-1)
    srv = pg.Server(hbm_budget_bytes=1 << 30, max_inflight=256, persistent=True)
    try:
        want = {srv.submit(deep, 7): g2["perft7"]}
        for k, i in enumerate(idx):
            want[srv.submit(pg.board_of(boards[k]), int(g3["depths"][i]))] = int(g3["totals"][i])
            if k == 40:
                time.sleep(0.01)
        got = {rid: srv.wait(rid, timeout=300)[0] for rid in want}
    finally:
        srv.stop()
    assert got == want
