"""Generates the golden vectors in tests/golden/ from the reference itself.

Run where the reference sources are present (REF_DIR, default the directory
"reference" beside this repository):

    python tests/golden/make_golden.py            # all fixtures
    python tests/golden/make_golden.py fens walk  # a subset

Every count, move list and child board here comes from the reference's own
host move generator (MoveGeneratorBitboard.h, compiled unchanged by
oracle/build_ref.sh).  The workload positions come from the seeded playout
generator of the oracle (or_playouts; its procedure is documented in
oracle/oracle.h); the playout positions are re-checked move by move against
the reference before their counts are taken.
"""
from __future__ import annotations

import json
import os
import random
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
THREADS = os.cpu_count() or 1

# test positions listed in the reference's perft.cu:62-70
REFERENCE_FENS = [
    ("start", "rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1"),
    ("position2", "r3k2r/p1ppqpb1/bn2pnp1/3PN3/1p2P3/2N2Q1p/PPPBBPPP/R3K2R w KQkq -"),
    ("position3", "8/2p5/3p4/KP5r/1R3p1k/8/4P1P1/8 w - -"),
    ("position4", "r2q1rk1/pP1p2pp/Q4n2/bbp1p3/Np6/1B3NBn/pPPP1PPP/R3K2R b KQ - 0 1"),
    ("position4_mirror", "r3k2r/Pppp1ppp/1b3nbN/nP6/BBP1P3/q4N2/Pp1P2PP/R2Q1RK1 w kq - 0 1"),
    ("position5", "rnbqkb1r/pp1p1ppp/2p5/4P3/2B5/8/PPP1NnPP/RNBQK2R w KQkq - 0 6"),
    ("moves218", "3Q4/1Q4Q1/4Q3/2Q4R/Q4Q2/3Q4/1Q4Rp/1K1BBNNk w - - 0 1"),
    ("temp_test", "r1b1kbnr/pppp1ppp/2n1p3/6q1/6Q1/2N1P3/PPPP1PPP/R1B1KBNR w KQkq - 4 4"),
]
FEN_DEPTHS = {"start": 6, "position2": 5, "position3": 6, "position4": 5, "position4_mirror": 5,
              "position5": 5, "moves218": 4, "temp_test": 5}

# workload definitions (seed, count, playout plies, minimum legal moves, depths)
WORKLOADS = {
    "config1": dict(seed=1, n=64, min_plies=8, max_plies=20, min_moves=1, depth_lo=5, depth_hi=5),
    "config2": dict(seed=2, n=1, min_plies=30, max_plies=30, min_moves=35, depth_lo=7, depth_hi=7),
    "config3": dict(seed=3, n=4096, min_plies=0, max_plies=60, min_moves=1, depth_lo=3, depth_hi=6),
    "config4": dict(seed=4, n=256, min_plies=0, max_plies=60, min_moves=1, depth_lo=7, depth_hi=7),
}

MASK64 = (1 << 64) - 1


def fingerprint(words) -> int:
    """64-bit fingerprint of the six words of a board (FNV-1a style mix)."""
    h = 0xCBF29CE484222325
    for w in words:
        h ^= int(w)
        h = (h * 0x100000001B3) & MASK64
        h ^= h >> 29
    return h


def hexb(words) -> list[str]:
    return ["%016x" % int(w) for w in words]


def board_words(row) -> tuple:
    return tuple(int(row[k]) for k in O.BOARD_DTYPE.names)


def ref_divide(ref: O.Reference, b: O.Board, depth: int) -> list[list[int]]:
    moves = ref.generate_moves(b)
    kids = np.zeros(len(moves), dtype=O.BOARD_DTYPE)
    for i, m in enumerate(moves):
        kids[i] = ref.make_move(b, m).as_tuple()
    counts, _ = ref.perft_batch(kids, np.full(len(moves), depth - 1, np.uint8), THREADS)
    return [[int(m), int(c)] for m, c in zip(moves, counts)]


def make_fens(ref):
    out = []
    for name, fen in REFERENCE_FENS:
        b = ref.fen(fen)
        d = FEN_DEPTHS[name]
        perft = {}
        for k in range(1, d + 1):
            perft[str(k)] = int(ref.perft_batch(np.array([b.as_tuple()], O.BOARD_DTYPE),
                                                np.array([k], np.uint8), 1)[0][0])
        out.append(dict(name=name, fen=fen, board=hexb(b.as_tuple()), perft=perft,
                        moves=ref.generate_moves(b), divide3=ref_divide(ref, b, 3)))
        print("fen", name, perft, flush=True)
    with open(os.path.join(HERE, "fens.json"), "w") as f:
        json.dump(out, f, indent=1)


def make_walk(ref, n_positions=1200, seed=7):
    """Random walks from the reference FENs; per position the reference's
    countMoves, generateMoves list, and fingerprints of makeMove children
    and generateBoards children."""
    rng = random.Random(seed)
    boards, counts, nmoves, moves, child_fp, nboards, boards_fp = [], [], [], [], [], [], []
    while len(boards) < n_positions:
        b = ref.fen(REFERENCE_FENS[rng.randrange(len(REFERENCE_FENS))][1])
        for _ in range(rng.randrange(0, 80)):
            mv = ref.generate_moves(b)
            if not mv:
                break
            b = ref.make_move(b, mv[rng.randrange(len(mv))])
        mv = ref.generate_moves(b)
        row_m = np.zeros(256, np.uint16)
        row_m[:len(mv)] = mv
        row_c = np.zeros(256, np.uint64)
        for i, m in enumerate(mv):
            row_c[i] = fingerprint(ref.make_move(b, m).as_tuple())
        gb = ref.generate_boards(b)
        row_b = np.zeros(256, np.uint64)
        for i, w in enumerate(gb):
            row_b[i] = fingerprint(w)
        boards.append(b.as_tuple())
        counts.append(ref.count_moves(b))
        nmoves.append(len(mv))
        moves.append(row_m)
        child_fp.append(row_c)
        nboards.append(len(gb))
        boards_fp.append(row_b)
    np.savez_compressed(os.path.join(HERE, "walk.npz"),
                        boards=np.array(boards, np.uint64), counts=np.array(counts, np.uint32),
                        nmoves=np.array(nmoves, np.uint32), moves=np.array(moves),
                        child_fp=np.array(child_fp), nboards=np.array(nboards, np.uint32),
                        boards_fp=np.array(boards_fp))
    print("walk", len(boards), flush=True)


def playout_boards(orc, ref, spec):
    boards, depths = orc.playouts(spec["seed"], spec["n"], spec["min_plies"], spec["max_plies"],
                                  spec["min_moves"], spec["depth_lo"], spec["depth_hi"],
                                  with_depths=True)
    # re-derive each count on the reference (the playout itself is ours)
    for row in boards[:64]:
        b = O.board_from_array(row)
        assert ref.count_moves(b) == orc.count_moves(b) >= spec["min_moves"]
    return boards, depths


def make_config1(orc, ref):
    spec = WORKLOADS["config1"]
    boards, depths = playout_boards(orc, ref, spec)
    t0 = time.time()
    totals, _ = ref.perft_batch(boards, depths, THREADS)
    items = []
    for row, d, tot in zip(boards, depths, totals):
        b = O.board_from_array(row)
        div = ref_divide(ref, b, int(d))
        assert sum(c for _, c in div) == int(tot)
        items.append(dict(board=hexb(board_words(row)), depth=int(d), total=int(tot), divide=div))
    with open(os.path.join(HERE, "config1.json"), "w") as f:
        json.dump(dict(spec=spec, positions=items, total=int(totals.sum())), f)
    print("config1", int(totals.sum()), "%.1fs" % (time.time() - t0), flush=True)


def make_config2(orc, ref):
    spec = WORKLOADS["config2"]
    boards, depths = playout_boards(orc, ref, spec)
    b = O.board_from_array(boards[0])
    t0 = time.time()
    out = dict(spec=spec, board=hexb(board_words(boards[0])), moves=ref.count_moves(b))
    for d in (5, 6, 7):
        div = ref_divide(ref, b, d)
        out["divide%d" % d] = div
        out["perft%d" % d] = sum(c for _, c in div)
        print("config2 depth", d, out["perft%d" % d], "%.1fs" % (time.time() - t0), flush=True)
    with open(os.path.join(HERE, "config2.json"), "w") as f:
        json.dump(out, f)


def make_config3(orc, ref):
    spec = WORKLOADS["config3"]
    boards, depths = playout_boards(orc, ref, spec)
    t0 = time.time()
    totals, secs = ref.perft_batch(boards, depths, THREADS)
    np.savez_compressed(os.path.join(HERE, "config3.npz"), boards=boards.view(np.uint64).reshape(-1, 6),
                        depths=depths, totals=totals,
                        spec=np.array(json.dumps(spec)))
    print("config3", int(totals.sum()), "%.1fs" % secs, flush=True)


def make_config4(orc, ref):
    """The 256 TT-workload positions; reference counts at depth 5 (the full
    depth-7 counts are checked TT-vs-no-TT on the GPU)."""
    spec = WORKLOADS["config4"]
    boards, depths = playout_boards(orc, ref, spec)
    totals, secs = ref.perft_batch(boards, np.full(len(boards), 5, np.uint8), THREADS)
    np.savez_compressed(os.path.join(HERE, "config4_d5.npz"), boards=boards.view(np.uint64).reshape(-1, 6),
                        totals=totals, spec=np.array(json.dumps(spec)))
    print("config4 d5", int(totals.sum()), "%.1fs" % secs, flush=True)


def make_playouts(orc):
    """Fingerprints of the oracle's playout positions, so the GPU playout
    generator can be checked without the oracle's playout code."""
    out = {}
    for name, spec in WORKLOADS.items():
        boards, depths = orc.playouts(spec["seed"], min(spec["n"], 512), spec["min_plies"],
                                      spec["max_plies"], spec["min_moves"], spec["depth_lo"],
                                      spec["depth_hi"], with_depths=True)
        out[name] = dict(spec=spec, fp=["%016x" % fingerprint(board_words(r)) for r in boards],
                         depths=[int(d) for d in depths])
    with open(os.path.join(HERE, "playouts.json"), "w") as f:
        json.dump(out, f)
    print("playouts", flush=True)


def main(argv):
    if not O.reference_available():
        if O.build_ref() is None:
            sys.exit("reference build unavailable: needs the reference sources on an x86-64 host")
    ref = O.Reference()
    orc = O.Oracle(1)
    jobs = argv or ["fens", "walk", "playouts", "config1", "config2", "config4", "config3"]
    for j in jobs:
        {"fens": lambda: make_fens(ref), "walk": lambda: make_walk(ref),
         "playouts": lambda: make_playouts(orc),
         "config1": lambda: make_config1(orc, ref), "config2": lambda: make_config2(orc, ref),
         "config3": lambda: make_config3(orc, ref), "config4": lambda: make_config4(orc, ref)}[j]()


if __name__ == "__main__":
    main(sys.argv[1:])
