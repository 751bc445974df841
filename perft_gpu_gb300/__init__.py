"""perft_gpu_gb300 -- GB300 (sm_103a) perft engine, Python host side.

Thin ctypes layer over the C ABI in include/perft_gb300.h (the library
libperft_gb300.so is built in-tree by perft_gpu_gb300/build.py).  It mirrors
the reference's operator surface for the perft path (sarona-RD/perft_gpu):

    MoveGeneratorBitboard.init / countMoves / generateMoves / generateBoards /
    makeMove                      (MoveGeneratorBitboard.h:982, 3008, 2469,
                                   1940, 3310)
    perft_bb(pos, depth)          (perft_bb.h:79)
    perftLauncher(pos, depth, launchDepth)   (launcher.h:1455, prints)
    Utils.readFENString           (util.cpp:189, returns the board)

Every call runs CUDA kernels on the GPU; there is no CPU path.  If the library
is missing or cannot be loaded the import of the engine fails loudly.
"""
from __future__ import annotations

import ctypes
import os
import time
from typing import Iterable

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libperft_gb300.so")

BOARD_DTYPE = np.dtype([("white", "<u8"), ("pawns", "<u8"), ("knights", "<u8"),
                        ("bishop_queens", "<u8"), ("rook_queens", "<u8"), ("kings", "<u8")])

PG_OK = 0
STATUS_NAMES = {0: "PG_OK", 1: "PG_ERR_NOT_INITIALIZED", 2: "PG_ERR_INVALID_ARGUMENT",
                3: "PG_ERR_INVALID_POSITION", 4: "PG_ERR_CUDA", 5: "PG_ERR_OUT_OF_MEMORY",
                6: "PG_ERR_DEVICE_TIMEOUT", 7: "PG_ERR_BUSY", 8: "PG_ERR_CAPACITY"}

SLIDER_AUTO, SLIDER_KOGGE_STONE, SLIDER_FANCY, SLIDER_BYTE_SMEM, SLIDER_HYBRID = 0, 1, 2, 3, 4
# pg_tt_mode: use_tt=True is TT_ON; "dedup" (or TT_DEDUP_ONLY) runs the TT
# driver with only the in-level duplicate pass (no HBM tables)
TT_OFF, TT_ON, TT_DEDUP_ONLY = 0, 1, 2
SLIDERS = {"auto": 0, "ks": 1, "fancy": 2, "byte": 3, "hybrid": 4}

# CMove flags (chess.h:272-293)
CM_FLAG_QUIET_MOVE, CM_FLAG_DOUBLE_PAWN_PUSH, CM_FLAG_KING_CASTLE, CM_FLAG_QUEEN_CASTLE = 0, 1, 2, 3
CM_FLAG_CAPTURE, CM_FLAG_EP_CAPTURE, CM_FLAG_PROMOTION = 4, 5, 8


class PerftError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class HexaBitBoardPosition(ctypes.Structure):
    """The reference's 48-byte board (chess.h:207-230)."""
    _fields_ = [("whitePieces", ctypes.c_uint64), ("pawns", ctypes.c_uint64),
                ("knights", ctypes.c_uint64), ("bishopQueens", ctypes.c_uint64),
                ("rookQueens", ctypes.c_uint64), ("kings", ctypes.c_uint64)]

    # packed state (chess.h:211-226)
    @property
    def chance(self) -> int:
        return self.pawns >> 63

    @property
    def whiteCastle(self) -> int:
        return self.pawns & 3

    @property
    def blackCastle(self) -> int:
        return (self.pawns >> 2) & 3

    @property
    def enPassent(self) -> int:
        return (self.pawns >> 4) & 15

    def words(self) -> tuple:
        return (self.whitePieces, self.pawns, self.knights, self.bishopQueens, self.rookQueens,
                self.kings)

    def copy(self) -> "HexaBitBoardPosition":
        return HexaBitBoardPosition(*self.words())

    def __eq__(self, other):
        return isinstance(other, HexaBitBoardPosition) and self.words() == other.words()

    def __repr__(self):
        return "HexaBitBoardPosition(%s)" % ", ".join("0x%016x" % w for w in self.words())


class PgConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_uint64),
                ("slider", ctypes.c_int), ("verbose", ctypes.c_int)]


class PgStats(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("leaves", ctypes.c_uint64),
                ("launches", ctypes.c_uint64), ("peak_level_bytes", ctypes.c_uint64),
                ("tt_probes", ctypes.c_uint64), ("tt_hits", ctypes.c_uint64),
                ("tt_stores", ctypes.c_uint64), ("leaf_kernel_launches", ctypes.c_uint64),
                ("leaf_kernel_ms", ctypes.c_double), ("leaf_parent_nodes", ctypes.c_uint64),
                ("graph_captures", ctypes.c_uint64), ("graph_replays", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class PgOpts(ctypes.Structure):
    _fields_ = [("slider", ctypes.c_int), ("block_size", ctypes.c_int),
                ("leaf_plies", ctypes.c_int), ("use_tt", ctypes.c_int),
                ("tt_bytes", ctypes.c_uint64), ("graph", ctypes.c_int),
                ("stats", ctypes.POINTER(PgStats)), ("persistent", ctypes.c_int)]


class PgTuning(ctypes.Structure):
    _fields_ = [("leaf_plies", ctypes.c_int), ("slider", ctypes.c_int * 16),
                ("block_size", ctypes.c_int * 16), ("leaves_per_s", ctypes.c_double * 16),
                ("seconds", ctypes.c_double)]

    def as_dict(self) -> dict:
        names = {v: k for k, v in SLIDERS.items()}
        return {"leaf_plies": self.leaf_plies, "seconds": self.seconds,
                "per_depth": {d: {"slider": names.get(self.slider[d], self.slider[d]),
                                  "block_size": self.block_size[d],
                                  "calibration_leaves_per_s": self.leaves_per_s[d]}
                              for d in range(3, 7)}}


class PgServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_inflight", ctypes.c_uint32),
                ("slider", ctypes.c_int), ("max_wave_nodes", ctypes.c_uint32),
                ("use_tt", ctypes.c_int), ("tt_bytes", ctypes.c_uint64), ("persistent", ctypes.c_int)]


class PgServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("waves", ctypes.c_uint64),
                ("admissions_deferred", ctypes.c_uint64), ("max_active", ctypes.c_uint32),
                ("pool_capacity", ctypes.c_uint64), ("pool_peak", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_BP = ctypes.POINTER(HexaBitBoardPosition)
_U16P = ctypes.POINTER(ctypes.c_uint16)
_U32P = ctypes.POINTER(ctypes.c_uint32)
_U64P = ctypes.POINTER(ctypes.c_uint64)
_U8P = ctypes.POINTER(ctypes.c_uint8)
_OP = ctypes.POINTER(PgOpts)

_SIGNATURES = {
    "pg_init": [ctypes.POINTER(PgConfig)],
    "pg_shutdown": [],
    "pg_last_error": [],
    "pg_board_from_fen": [ctypes.c_char_p, _BP],
    "pg_get_stream": [ctypes.POINTER(ctypes.c_void_p)],
    "pg_count_moves": [_BP, _U32P],
    "pg_count_moves_batch": [_BP, ctypes.c_uint32, _U32P],
    "pg_generate_moves": [_BP, _U16P, _U32P],
    "pg_generate_boards": [_BP, _BP, _U32P],
    "pg_make_move": [_BP, ctypes.c_uint16],
    "pg_perft": [_BP, ctypes.c_int, _U64P, _OP],
    "pg_perft_divide": [_BP, ctypes.c_int, _U16P, _U64P, _U32P, _OP],
    "pg_perft_batch": [_BP, _U8P, ctypes.c_uint32, _U64P, _OP],
    "pg_perft_batch_device": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, _OP],
    "pg_random_playouts": [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                           ctypes.c_int, ctypes.c_int, _BP, _U8P],
    "pg_server_start": [ctypes.POINTER(PgServerConfig)],
    "pg_server_submit": [_BP, ctypes.c_int, _U64P],
    "pg_server_poll": [ctypes.c_uint64, _U64P, ctypes.POINTER(ctypes.c_int),
                       ctypes.POINTER(ctypes.c_double)],
    "pg_server_stop": [],
    "pg_server_get_stats": [ctypes.POINTER(PgServerStats)],
    "pg_tt_clear": [],
    "pg_tt_save": [ctypes.c_char_p],
    "pg_tt_load": [ctypes.c_char_p],
    "pg_autotune": [ctypes.POINTER(PgTuning)],
    "pg_perft_split": [_BP, ctypes.c_int, ctypes.c_int, _U16P, _U64P, _U32P, _OP],
    "pg_selftest": [ctypes.c_int],
    "pg_zobrist_key": [_BP, _U64P],
    "pg_zobrist_key_from": [_BP, _U64P, _BP, _U64P],
    "pg_tt_entry_pack": [_U64P, ctypes.c_uint64, _U64P],
    "pg_tt_entry_match": [_U64P, _U64P, ctypes.POINTER(ctypes.c_int), _U64P],
    "pg_perft_batch_noalloc": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                               ctypes.c_void_p],
}

_lib = None


def library_path() -> str:
    return LIB_PATH


def load_library(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libperft_gb300.so, building it in-tree when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise ImportError("libperft_gb300.so is missing; run perft_gpu_gb300.build.build()")
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_char_p if name == "pg_last_error" else ctypes.c_int
    _lib = lib
    return lib


def _check(status: int):
    if status != PG_OK:
        raise PerftError(status, load_library().pg_last_error().decode(errors="replace"))


def _tt_mode(use_tt) -> int:
    if isinstance(use_tt, str):
        return {"off": TT_OFF, "on": TT_ON, "dedup": TT_DEDUP_ONLY}[use_tt]
    if isinstance(use_tt, bool) or use_tt is None:
        return TT_ON if use_tt else TT_OFF
    return int(use_tt)


def _opts(slider=None, block_size=0, use_tt=False, tt_bytes=0, graph=False, stats=None, leaf_plies=0,
          persistent=False):
    o = PgOpts()
    o.slider = SLIDERS[slider] if isinstance(slider, str) else (slider or 0)
    o.block_size = block_size
    o.leaf_plies = leaf_plies
    o.use_tt = _tt_mode(use_tt)
    o.tt_bytes = tt_bytes
    o.graph = 1 if graph else 0
    o.persistent = 1 if persistent else 0
    o.stats = ctypes.pointer(stats) if stats is not None else None
    return o


# ---------------------------------------------------------------------------
# engine
# ---------------------------------------------------------------------------

def init(device: int = 0, hbm_budget_bytes: int = 0, slider: int | str = 0, verbose: int = 0):
    cfg = PgConfig(device, hbm_budget_bytes, SLIDERS[slider] if isinstance(slider, str) else slider,
                   verbose)
    _check(load_library().pg_init(ctypes.byref(cfg)))


def shutdown():
    _check(load_library().pg_shutdown())


def get_stream() -> int:
    """The engine's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
    s = ctypes.c_void_p()
    _check(load_library().pg_get_stream(ctypes.byref(s)))
    return s.value or 0


def board_from_fen(fen: str) -> HexaBitBoardPosition:
    b = HexaBitBoardPosition()
    _check(load_library().pg_board_from_fen(fen.encode(), ctypes.byref(b)))
    return b


def count_moves(pos: HexaBitBoardPosition) -> int:
    n = ctypes.c_uint32()
    _check(load_library().pg_count_moves(ctypes.byref(pos), ctypes.byref(n)))
    return n.value


def count_moves_batch(boards: np.ndarray) -> np.ndarray:
    boards = np.ascontiguousarray(boards, dtype=BOARD_DTYPE)
    out = np.zeros(len(boards), dtype=np.uint32)
    _check(load_library().pg_count_moves_batch(boards.ctypes.data_as(_BP), len(boards),
                                                out.ctypes.data_as(_U32P)))
    return out


def generate_moves(pos: HexaBitBoardPosition) -> list[int]:
    buf = (ctypes.c_uint16 * 256)()
    n = ctypes.c_uint32()
    _check(load_library().pg_generate_moves(ctypes.byref(pos), buf, ctypes.byref(n)))
    return list(buf[:n.value])


def generate_boards(pos: HexaBitBoardPosition) -> list[HexaBitBoardPosition]:
    buf = (HexaBitBoardPosition * 256)()
    n = ctypes.c_uint32()
    _check(load_library().pg_generate_boards(ctypes.byref(pos), buf, ctypes.byref(n)))
    return [buf[i].copy() for i in range(n.value)]


def make_move(pos: HexaBitBoardPosition, move: int) -> HexaBitBoardPosition:
    """Returns the board after `move` (the argument is left unchanged)."""
    b = pos.copy()
    _check(load_library().pg_make_move(ctypes.byref(b), move))
    return b


def perft(pos: HexaBitBoardPosition, depth: int, **kw) -> int:
    out = ctypes.c_uint64()
    o = _opts(**kw)
    _check(load_library().pg_perft(ctypes.byref(pos), depth, ctypes.byref(out), ctypes.byref(o)))
    return out.value


def perft_divide(pos: HexaBitBoardPosition, depth: int, **kw) -> list[tuple[int, int]]:
    mv = (ctypes.c_uint16 * 256)()
    cnt = (ctypes.c_uint64 * 256)()
    n = ctypes.c_uint32()
    o = _opts(**kw)
    _check(load_library().pg_perft_divide(ctypes.byref(pos), depth, mv, cnt, ctypes.byref(n),
                                          ctypes.byref(o)))
    return [(mv[i], cnt[i]) for i in range(n.value)]


def perft_split(pos: HexaBitBoardPosition, depth: int, split_plies: int = 3, **kw) -> list[tuple[int, int]]:
    """Divided perft at deep roots with the host-side complete TT."""
    mv = (ctypes.c_uint16 * 256)()
    cnt = (ctypes.c_uint64 * 256)()
    n = ctypes.c_uint32()
    o = _opts(**kw)
    _check(load_library().pg_perft_split(ctypes.byref(pos), depth, split_plies, mv, cnt, ctypes.byref(n),
                                         ctypes.byref(o)))
    return [(mv[i], cnt[i]) for i in range(n.value)]


SELFTEST_BOUNDED_WAIT, SELFTEST_FAIL_NEXT_ALLOC = 1, 2


def selftest(which: int) -> int:
    """Returns the status code of a failure-detection self test."""
    return load_library().pg_selftest(which)


def perft_batch(boards: np.ndarray, depths: Iterable[int] | np.ndarray, **kw) -> np.ndarray:
    boards = np.ascontiguousarray(boards, dtype=BOARD_DTYPE)
    depths = np.ascontiguousarray(depths, dtype=np.uint8)
    if len(depths) != len(boards):
        raise ValueError("one depth per board")
    out = np.zeros(len(boards), dtype=np.uint64)
    o = _opts(**kw)
    _check(load_library().pg_perft_batch(boards.ctypes.data_as(_BP), depths.ctypes.data_as(_U8P),
                                         len(boards), out.ctypes.data_as(_U64P), ctypes.byref(o)))
    return out


def perft_batch_device(d_boards: int, d_depths: int, n: int, d_out: int, **kw):
    """Device-pointer variant: arguments are CUDA device addresses."""
    o = _opts(**kw)
    _check(load_library().pg_perft_batch_device(ctypes.c_void_p(d_boards), ctypes.c_void_p(d_depths),
                                                n, ctypes.c_void_p(d_out), ctypes.byref(o)))


def random_playouts(seed: int, n: int, min_plies: int, max_plies: int, min_moves: int = 1,
                    depth_lo: int = 0, depth_hi: int = 0, with_depths: bool = False):
    out = np.zeros(n, dtype=BOARD_DTYPE)
    depths = np.zeros(n, dtype=np.uint8) if with_depths else None
    _check(load_library().pg_random_playouts(seed, n, min_plies, max_plies, min_moves, depth_lo,
                                             depth_hi, out.ctypes.data_as(_BP),
                                             depths.ctypes.data_as(_U8P) if with_depths else None))
    return (out, depths) if with_depths else out


def autotune() -> dict:
    """Run (once) and report the autotuner's per-depth choices."""
    t = PgTuning()
    _check(load_library().pg_autotune(ctypes.byref(t)))
    return t.as_dict()


def tt_clear():
    """Empty the transposition tables."""
    _check(load_library().pg_tt_clear())


def tt_save(path: str):
    """Write the transposition tables to a snapshot file."""
    _check(load_library().pg_tt_save(os.fsencode(path)))


def tt_load(path: str):
    """Read a snapshot written by tt_save back into the tables."""
    _check(load_library().pg_tt_load(os.fsencode(path)))


def zobrist_key(pos: HexaBitBoardPosition) -> tuple[int, int]:
    """The 128-bit Zobrist key (low word, high word) the device tables use."""
    k = (ctypes.c_uint64 * 2)()
    _check(load_library().pg_zobrist_key(ctypes.byref(pos), k))
    return k[0], k[1]


def zobrist_key_from(src: HexaBitBoardPosition, src_key: tuple[int, int],
                     pos: HexaBitBoardPosition) -> tuple[int, int]:
    """The key of `pos` updated from the key of `src` by the features the two
    boards differ in (the incremental update the probe kernel makes from a
    parent to its child)."""
    k = (ctypes.c_uint64 * 2)(*src_key)
    out = (ctypes.c_uint64 * 2)()
    _check(load_library().pg_zobrist_key_from(ctypes.byref(src), k, ctypes.byref(pos), out))
    return out[0], out[1]


def tt_entry_pack(key: tuple[int, int], count: int) -> tuple[int, int, int, int]:
    """The four 64-bit words of a table entry holding `count` for `key`."""
    k = (ctypes.c_uint64 * 2)(*key)
    e = (ctypes.c_uint64 * 4)()
    _check(load_library().pg_tt_entry_pack(k, count, e))
    return tuple(e)


def tt_entry_match(entry, key: tuple[int, int]):
    """The count a probe for `key` reads from `entry`, or None (a miss)."""
    e = (ctypes.c_uint64 * 4)(*entry)
    k = (ctypes.c_uint64 * 2)(*key)
    acc = ctypes.c_int()
    v = ctypes.c_uint64()
    _check(load_library().pg_tt_entry_match(e, k, ctypes.byref(acc), ctypes.byref(v)))
    return v.value if acc.value else None


def board_of(row) -> HexaBitBoardPosition:
    return HexaBitBoardPosition(*(int(row[k]) for k in BOARD_DTYPE.names))


def boards_array(boards: Iterable[HexaBitBoardPosition]) -> np.ndarray:
    return np.array([b.words() for b in boards], dtype=np.uint64).view(BOARD_DTYPE).reshape(-1)


# ---------------------------------------------------------------------------
# serving
# ---------------------------------------------------------------------------

class Server:
    """Continuous-batching perft server (pg_server_*)."""

    def __init__(self, hbm_budget_bytes: int = 0, max_inflight: int = 0, slider: int | str = 0,
                 max_wave_nodes: int = 0, use_tt: bool | int | str = False, tt_bytes: int = 0,
                 persistent: bool = False):
        cfg = PgServerConfig(hbm_budget_bytes, max_inflight,
                             SLIDERS[slider] if isinstance(slider, str) else slider, max_wave_nodes,
                             _tt_mode(use_tt), tt_bytes, 1 if persistent else 0)
        _check(load_library().pg_server_start(ctypes.byref(cfg)))

    def submit(self, pos: HexaBitBoardPosition, depth: int) -> int:
        rid = ctypes.c_uint64()
        _check(load_library().pg_server_submit(ctypes.byref(pos), depth, ctypes.byref(rid)))
        return rid.value

    def poll(self, rid: int):
        res = ctypes.c_uint64()
        done = ctypes.c_int()
        lat = ctypes.c_double()
        _check(load_library().pg_server_poll(rid, ctypes.byref(res), ctypes.byref(done),
                                             ctypes.byref(lat)))
        return (res.value if done.value else None), lat.value

    def wait(self, rid: int, timeout: float = 600.0):
        t0 = time.time()
        while True:
            r, lat = self.poll(rid)
            if r is not None:
                return r, lat
            if time.time() - t0 > timeout:
                raise TimeoutError("request %d not done after %.0f s" % (rid, timeout))
            time.sleep(0.0005)

    def stats(self) -> dict:
        s = PgServerStats()
        _check(load_library().pg_server_get_stats(ctypes.byref(s)))
        return s.as_dict()

    def stop(self):
        _check(load_library().pg_server_stop())


# ---------------------------------------------------------------------------
# the reference's names (operator surface of the perft path)
# ---------------------------------------------------------------------------

class MoveGeneratorBitboard:
    """Static methods with the reference's names and argument meaning."""

    @staticmethod
    def init():
        init()

    @staticmethod
    def countMoves(pos: HexaBitBoardPosition) -> int:
        return count_moves(pos)

    @staticmethod
    def generateMoves(pos: HexaBitBoardPosition, genMoves: list | None = None) -> int:
        mv = generate_moves(pos)
        if genMoves is not None:
            genMoves[:] = mv
        return len(mv)

    @staticmethod
    def generateBoards(pos: HexaBitBoardPosition, newPositions: list | None = None) -> int:
        bd = generate_boards(pos)
        if newPositions is not None:
            newPositions[:] = bd
        return len(bd)

    @staticmethod
    def makeMove(pos: HexaBitBoardPosition, move: int) -> None:
        """In place, as the reference's makeMove<chance, false>."""
        _check(load_library().pg_make_move(ctypes.byref(pos), move))


class Utils:
    @staticmethod
    def readFENString(fen: str) -> HexaBitBoardPosition:
        return board_from_fen(fen)

    @staticmethod
    def getCompactMoveString(move: int) -> str:
        """utils.h:251-258: "e2-e4" / "e4*d5" (capture flag)."""
        frm, to = move & 63, (move >> 6) & 63
        sep = "*" if (move >> 12) & CM_FLAG_CAPTURE else "-"
        return "%s%d%s%s%d" % ("abcdefgh"[frm & 7], (frm >> 3) + 1, sep, "abcdefgh"[to & 7],
                               (to >> 3) + 1)


def perft_bb(pos: HexaBitBoardPosition, depth: int) -> int:
    """perft_bb (perft_bb.h:79-101), computed on the GPU."""
    return perft(pos, depth)


def perftLauncher(pos: HexaBitBoardPosition, depth: int, launchDepth: int = 0, **kw) -> int:
    """launcher.h:1467-1503: prints "GPU Perft d: n,   Time taken: t seconds,
    nps: r" and returns the count (the reference returns nothing)."""
    stats = PgStats()
    t0 = time.perf_counter()
    res = perft(pos, depth, stats=stats, **kw)
    dt = time.perf_counter() - t0
    print("\nGPU Perft %d: %d,   Time taken: %g seconds, nps: %d" % (depth, res, dt, int(res / dt) if dt else 0))
    return res
