"""Transposition-table keys and entries, host side (no GPU needed).

The device tables use the same inline code as the C-ABI helpers called here
(pg_zobrist.cuh): 128-bit Zobrist keys in the shape of the reference's
HashKey128b (chess.h:410-452) and 32-byte entries that XOR the count into
every key bit.  The reference's 16-byte entries verify the high word and the
non-index bits of the low word (perft_bb.h:690-693); these tests pin that an
entry is accepted only for its own full 128-bit key, that torn entries (halves
of two stores) never yield a wrong count, and that the key is the documented
function of the board."""
import random

import pytest

from conftest import golden_json, golden_npz

MASK = (1 << 64) - 1


@pytest.fixture(scope="module")
def pg():
    import perft_gpu_gb300 as pg
    pg.load_library()
    return pg


def _splitmix_stream(seed, n):
    s, out = seed, []
    for _ in range(n):
        s = (s + 0x9E3779B97F4A7C15) & MASK
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        out.append(z ^ (z >> 31))
    return out


KEYS0 = _splitmix_stream(0x5EED2B1D0C0FFEE5, 781)
KEYS1 = _splitmix_stream(0xA24BAED4963EE407, 781)


def _key_of_words(w):
    """Independent restatement of the documented key: 768 piece-square
    features (kinds pawn, knight, bishop, rook, queen, king; white then
    black), castling bits 0-3 of the state, en-passant file, side to move."""
    white, pw, kn, bq, rq, kg = (int(x) for x in w)
    pawns = pw & 0x00FFFFFFFFFFFF00
    sets = [pawns, kn, bq & ~rq & MASK, rq & ~bq & MASK, bq & rq, kg]
    h0 = h1 = 0
    for t, s in enumerate(sets):
        for colour, mask in ((0, white), (1, ~white & MASK)):
            x = s & mask
            while x:
                sq = (x & -x).bit_length() - 1
                i = (6 * colour + t) * 64 + sq
                h0 ^= KEYS0[i]
                h1 ^= KEYS1[i]
                x &= x - 1
    for c in range(4):
        if (pw >> c) & 1:
            h0 ^= KEYS0[768 + c]
            h1 ^= KEYS1[768 + c]
    ep = (pw >> 4) & 15
    if ep:
        h0 ^= KEYS0[772 + ((ep - 1) & 7)]
        h1 ^= KEYS1[772 + ((ep - 1) & 7)]
    if pw >> 63:
        h0 ^= KEYS0[780]
        h1 ^= KEYS1[780]
    if h0 == 0 and h1 == 0:
        h0 = 1
    return h0, h1


def test_key_is_the_documented_function_of_the_board(pg):
    walk = golden_npz("walk.npz")["boards"]
    for w in walk[:400]:
        b = pg.HexaBitBoardPosition(*(int(x) for x in w))
        assert pg.zobrist_key(b) == _key_of_words(w)


def test_keys_distinct_over_distinct_positions_and_state(pg):
    walk = golden_npz("walk.npz")["boards"]
    seen = {}
    for w in walk:
        words = tuple(int(x) for x in w)
        canon = (words[0], words[1] & ~(0x7F << 56), *words[2:])  # half-move clock masked
        k = pg.zobrist_key(pg.HexaBitBoardPosition(*words))
        if k in seen:
            assert seen[k] == canon
        seen[k] = canon
    start = pg.board_from_fen(golden_json("fens.json")[0]["fen"])
    k = pg.zobrist_key(start)
    variants = []
    for bit in range(4):  # each castling right
        b = start.copy()
        b.pawns ^= 1 << bit
        variants.append(b)
    b = start.copy()
    b.pawns ^= 1 << 63  # side to move
    variants.append(b)
    b = start.copy()
    b.pawns |= 5 << 4  # en-passant file e
    variants.append(b)
    keys = {pg.zobrist_key(v) for v in variants}
    assert k not in keys and len(keys) == len(variants)
    b = start.copy()
    b.pawns |= 37 << 56  # half-move clock: not part of the key
    assert pg.zobrist_key(b) == k


def test_entry_round_trip(pg):
    rng = random.Random(7)
    for _ in range(500):
        key = (rng.getrandbits(64), rng.getrandbits(64))
        v = rng.getrandbits(rng.choice([8, 24, 40, 52, 64]))
        e = pg.tt_entry_pack(key, v)
        assert pg.tt_entry_match(e, key) == v


def test_entry_rejects_keys_that_share_one_64_bit_half(pg):
    """The 64-bit keys of the earlier format were accepted on one word: an
    entry is now refused for any key that differs in either word, including
    keys that agree on the whole low word (same slot) or the whole high
    word."""
    rng = random.Random(11)
    for _ in range(500):
        k0, k1 = rng.getrandbits(64), rng.getrandbits(64)
        v = rng.getrandbits(48)
        e = pg.tt_entry_pack((k0, k1), v)
        for other in [(k0, k1 ^ (1 << rng.randrange(64))), (k0 ^ (1 << rng.randrange(64)), k1),
                      (k0, rng.getrandbits(64)), (rng.getrandbits(64), k1), (k1, k0)]:
            if other != (k0, k1):
                assert pg.tt_entry_match(e, other) is None
    # the reference-format trap: count XORed into only one word would let a
    # key whose low word equals e0 ^ e2 pass; here the other checks refuse it
    k = (0x0123456789ABCDEF, 0xFEDCBA9876543210)
    e = pg.tt_entry_pack(k, 1000)
    assert pg.tt_entry_match(e, (k[0], k[1] ^ 0xFFFF)) is None


def test_torn_and_empty_entries_never_give_a_wrong_count(pg):
    rng = random.Random(13)
    for _ in range(2000):
        ka = (rng.getrandbits(64), rng.getrandbits(64))
        kb = (ka[0], rng.getrandbits(64)) if rng.random() < 0.5 else (rng.getrandbits(64), rng.getrandbits(64))
        va = rng.getrandbits(40)
        vb = va if rng.random() < 0.3 else rng.getrandbits(40)
        ea, eb = pg.tt_entry_pack(ka, va), pg.tt_entry_pack(kb, vb)
        for torn in [ea[:2] + eb[2:], eb[:2] + ea[2:]]:
            for key, true_v in [(ka, va), (kb, vb)]:
                got = pg.tt_entry_match(torn, key)
                assert got is None or got == true_v
    for key in [(1, 0), (0, 1), (rng.getrandbits(64), rng.getrandbits(64))]:
        assert pg.tt_entry_match((0, 0, 0, 0), key) is None


def test_entry_rejects_synthetic_low_word_collision_of_real_positions(pg):
    """Two real positions' keys, the second forced to share the first's low
    word (a collision of the old 64-bit key): the first's entry is refused
    for the second."""
    walk = golden_npz("walk.npz")["boards"]
    a = pg.zobrist_key(pg.HexaBitBoardPosition(*(int(x) for x in walk[3])))
    b = pg.zobrist_key(pg.HexaBitBoardPosition(*(int(x) for x in walk[700])))
    assert a != b
    e = pg.tt_entry_pack(a, 123456789)
    assert pg.tt_entry_match(e, (a[0], b[1])) is None
    assert pg.tt_entry_match(e, a) == 123456789


def test_tt_mode_values(pg):
    assert pg._tt_mode(True) == pg.TT_ON and pg._tt_mode(False) == pg.TT_OFF
    assert pg._tt_mode("dedup") == pg.TT_DEDUP_ONLY and pg._tt_mode(2) == 2


def test_incremental_key_equals_full_key_for_every_child(pg, oracle):
    """The probe kernel keys a node below the root from its parent's key
    (pg_zobrist_key_from, the reference's incremental update in makeMove):
    over every child of 300 walk positions (captures, castling, en passant,
    promotions) and their grandchildren keyed from the updated key, the
    update equals the full key."""
    walk = golden_npz("walk.npz")["boards"]
    kinds = 0
    for w in walk[::4][:300]:
        parent = pg.HexaBitBoardPosition(*(int(x) for x in w))
        kp = pg.zobrist_key(parent)
        for c in oracle.generate_boards(oracle_board(w)):
            child = pg.HexaBitBoardPosition(*c)
            kc = pg.zobrist_key_from(parent, kp, child)
            assert kc == pg.zobrist_key(child) == _key_of_words(c)
            kinds |= 1 << bin((int(w[1]) ^ c[1]) & 0x0F).count("1")  # castling rights cleared
            for g in oracle.generate_boards(oracle_board(c))[:3]:
                grand = pg.HexaBitBoardPosition(*g)
                assert pg.zobrist_key_from(child, kc, grand) == pg.zobrist_key(grand)
    assert kinds & 0b110, "no child cleared a castling right"


def test_incremental_key_holds_for_any_two_boards_and_the_remapped_zero(pg):
    """The update is exact for any pair of boards (XOR over the features that
    differ), and a source key of (1, 0) -- which may stand for the raw key 0
    -- falls back to the full key."""
    walk = golden_npz("walk.npz")["boards"]
    rng = random.Random(17)
    for _ in range(300):
        a, b = (walk[rng.randrange(len(walk))] for _ in range(2))
        pa = pg.HexaBitBoardPosition(*(int(x) for x in a))
        pb = pg.HexaBitBoardPosition(*(int(x) for x in b))
        assert pg.zobrist_key_from(pa, pg.zobrist_key(pa), pb) == pg.zobrist_key(pb)
        assert pg.zobrist_key_from(pa, (1, 0), pb) == pg.zobrist_key(pb)


def oracle_board(words):
    import oracle as O
    return O.Board(*(int(x) for x in words))


def test_key_helpers_refuse_null_arguments(pg):
    """The host-side key and entry helpers return PG_ERR_INVALID_ARGUMENT
    for a null pointer, with a message, instead of reading through it."""
    import ctypes
    PG_ERR_INVALID_ARGUMENT = 2  # include/perft_gb300.h
    lib = pg.load_library()
    b = pg.board_from_fen(golden_json("fens.json")[0]["fen"])
    k = (ctypes.c_uint64 * 2)()
    assert lib.pg_zobrist_key(None, k) == PG_ERR_INVALID_ARGUMENT
    assert lib.pg_zobrist_key_from(ctypes.byref(b), None, ctypes.byref(b), k) == PG_ERR_INVALID_ARGUMENT
    assert lib.pg_zobrist_key_from(ctypes.byref(b), k, ctypes.byref(b), None) == PG_ERR_INVALID_ARGUMENT
    assert b"null" in lib.pg_last_error()
    e = (ctypes.c_uint64 * 4)()
    assert lib.pg_tt_entry_pack(None, 5, e) == PG_ERR_INVALID_ARGUMENT
    assert lib.pg_tt_entry_match(e, k, None, None) == PG_ERR_INVALID_ARGUMENT
