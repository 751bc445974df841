"""The C ABI library: builds, loads, exports every declared entry point, and
its host-only logic behaves (no GPU needed)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT, golden_json, words_of_hex

HEADER = os.path.join(ROOT, "include", "perft_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pg_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_surface():
    syms = declared_symbols()
    for s in ["pg_init", "pg_shutdown", "pg_last_error", "pg_count_moves", "pg_generate_moves",
              "pg_generate_boards", "pg_make_move", "pg_perft", "pg_perft_divide", "pg_perft_batch",
              "pg_perft_batch_device", "pg_board_from_fen", "pg_random_playouts",
              "pg_server_start", "pg_server_submit", "pg_server_poll", "pg_server_stop"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    import perft_gpu_gb300 as pg
    lib = pg.load_library()
    for s in declared_symbols():
        assert hasattr(lib, s), s
    out = os.popen("nm -D --defined-only %s" % pg.library_path()).read()
    for s in declared_symbols():
        assert re.search(r"\bT %s\b" % s, out), s


def test_fen_parser_matches_reference_boards():
    import perft_gpu_gb300 as pg
    for item in golden_json("fens.json"):
        assert pg.board_from_fen(item["fen"]).words() == words_of_hex(item["board"])


def test_board_layout_is_48_bytes():
    import perft_gpu_gb300 as pg
    assert ctypes.sizeof(pg.HexaBitBoardPosition) == 48
    assert pg.BOARD_DTYPE.itemsize == 48


def test_compact_move_string():
    import perft_gpu_gb300 as pg
    assert pg.Utils.getCompactMoveString((12) | (28 << 6)) == "e2-e4"
    assert pg.Utils.getCompactMoveString((28) | (35 << 6) | (4 << 12)) == "e4*d5"
