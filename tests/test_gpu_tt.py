"""Transposition-table perft: every count equals the reference's golden count
and the no-TT count, also when a tiny table forces constant overwrites."""
import numpy as np
import pytest

from conftest import golden_json, golden_npz, words_of_hex

pytestmark = pytest.mark.gpu


def test_tt_reference_fens(pg):
    pg.tt_clear()
    for item in golden_json("fens.json"):
        b = pg.board_from_fen(item["fen"])
        for d, v in item["perft"].items():
            if int(d) <= 5:
                assert pg.perft(b, int(d), use_tt=True) == v, (item["name"], d)


def test_tt_config4_depth5_and_stats(pg):
    g = golden_npz("config4_d5.npz")
    boards = g["boards"].copy().view(pg.BOARD_DTYPE).reshape(-1)
    pg.tt_clear()
    st = pg.PgStats()
    out = pg.perft_batch(boards, [5] * len(boards), use_tt=True, stats=st)
    assert np.array_equal(out, g["totals"])
    # breadth-first: a level is probed before any of it is stored, so a cold
    # single pass stores but finds transpositions through the level's
    # duplicate pass instead; the second pass hits the stored entries
    assert st.tt_probes > 0 and st.tt_stores > 0
    st2 = pg.PgStats()
    out2 = pg.perft_batch(boards, [5] * len(boards), use_tt=True, stats=st2)
    assert np.array_equal(out2, g["totals"])
    assert st2.tt_hits > 0


def test_tt_equals_no_tt_on_batched_workload(pg):
    g = golden_npz("config3.npz")
    idx = np.arange(0, 4096, 5)
    boards = g["boards"][idx].copy().view(pg.BOARD_DTYPE).reshape(-1)
    depths = np.minimum(g["depths"][idx], 5)
    pg.tt_clear()
    assert np.array_equal(pg.perft_batch(boards, depths, use_tt=True), pg.perft_batch(boards, depths))


def test_tt_tiny_table_and_duplicate_roots(pg):
    fens = {f["name"]: f for f in golden_json("fens.json")}
    b = pg.board_from_fen(fens["position2"]["fen"])
    boards = pg.boards_array([b, b, pg.board_from_fen(fens["start"]["fen"]), b])
    out = pg.perft_batch(boards, [4, 4, 5, 3], use_tt=True, tt_bytes=1 << 20)
    assert [int(x) for x in out] == [fens["position2"]["perft"]["4"]] * 2 + [fens["start"]["perft"]["5"],
                                                                              fens["position2"]["perft"]["3"]]
    pg.tt_clear()


def test_tt_config2_depth7(pg):
    g = golden_json("config2.json")
    b = pg.HexaBitBoardPosition(*words_of_hex(g["board"]))
    pg.tt_clear()
    assert pg.perft(b, 7, use_tt=True) == g["perft7"]
    assert pg.perft(b, 6, use_tt=True) == g["perft6"]


def test_tt_snapshot_save_load(pg, tmp_path):
    """A snapshot written after a TT run and read back after clearing gives
    TT hits on the first pass of the same run, with the same counts; files
    that are not snapshots are refused."""
    fens = {f["name"]: f for f in golden_json("fens.json")}
    b = pg.board_from_fen(fens["position2"]["fen"])
    want = fens["position2"]["perft"]["5"]
    size = 64 << 20
    pg.tt_clear()
    assert pg.perft(b, 5, use_tt=True, tt_bytes=size) == want
    snap = str(tmp_path / "tt.snap")
    pg.tt_save(snap)
    pg.tt_clear()
    st0 = pg.PgStats()
    assert pg.perft(b, 5, use_tt=True, tt_bytes=size, stats=st0) == want
    assert st0.tt_hits == 0                     # cleared: a single pass finds nothing stored
    pg.tt_clear()
    pg.tt_load(snap)
    st1 = pg.PgStats()
    assert pg.perft(b, 5, use_tt=True, tt_bytes=size, stats=st1) == want
    assert st1.tt_hits > 0                      # the snapshot's entries are found
    bad = tmp_path / "bad.snap"
    bad.write_bytes(b"not a snapshot" * 10)
    with pytest.raises(pg.PerftError):
        pg.tt_load(str(bad))
    with pytest.raises(pg.PerftError):
        pg.tt_load(str(tmp_path / "missing.snap"))
    pg.tt_clear()


def test_tt_dedup_only_mode(pg):
    """use_tt="dedup": the TT driver with only the in-level duplicate pass;
    no table is probed or stored, counts are unchanged."""
    g = golden_npz("config4_d5.npz")
    boards = g["boards"].copy().view(pg.BOARD_DTYPE).reshape(-1)
    st = pg.PgStats()
    out = pg.perft_batch(boards, [5] * len(boards), use_tt="dedup", stats=st)
    assert np.array_equal(out, g["totals"])
    assert st.tt_probes == 0 and st.tt_hits == 0 and st.tt_stores == 0
    fens = {f["name"]: f for f in golden_json("fens.json")}
    b = pg.board_from_fen(fens["position2"]["fen"])
    assert pg.perft(b, 5, use_tt="dedup") == fens["position2"]["perft"]["5"]
    with pytest.raises(pg.PerftError):
        pg.perft(b, 3, use_tt=7)


def test_tt_full_key_separates_positions_in_one_level(pg):
    """Many distinct positions at one level with a tiny table (1 MB, constant
    overwrites) and duplicates of each: every count equals the no-TT count."""
    boards, depths = pg.random_playouts(41, 3000, 0, 60, 1, 3, 5, with_depths=True)
    boards = np.concatenate([boards, boards[::3]])
    depths = np.concatenate([depths, depths[::3]])
    pg.tt_clear()
    ref = pg.perft_batch(boards, depths)
    for _ in range(2):
        assert np.array_equal(pg.perft_batch(boards, depths, use_tt=True, tt_bytes=1 << 20), ref)
    pg.tt_clear()


def test_tt_chunked_levels_small_budget(pg):
    """A small HBM budget makes the TT driver split its levels into many
    chunks sized with the per-node TT metadata (later chunks then hit the
    tables earlier chunks stored): counts still equal the golden counts and
    the no-TT counts."""
    fens = {f["name"]: f for f in golden_json("fens.json")}
    pg.shutdown()
    pg.init(hbm_budget_bytes=256 << 20)
    try:
        b = pg.board_from_fen(fens["position2"]["fen"])
        pg.tt_clear()
        st = pg.PgStats()
        assert pg.perft(b, 5, use_tt=True, tt_bytes=16 << 20, stats=st) == fens["position2"]["perft"]["5"]
        assert st.tt_stores > 0
        g = golden_npz("config4_d5.npz")
        boards = g["boards"][:64].copy().view(pg.BOARD_DTYPE).reshape(-1)
        for mode in (True, "dedup"):
            assert np.array_equal(pg.perft_batch(boards, [5] * 64, use_tt=mode, tt_bytes=16 << 20), g["totals"][:64])
    finally:
        pg.tt_clear()
        pg.shutdown()
        pg.init()
