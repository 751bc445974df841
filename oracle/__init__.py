"""ctypes bindings for the CPU oracle (oracle.c) and, where it was built, the
reference's own host move generator (oracle/_ref/libperft_ref.so).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by __graft_entry__.smoke() and
by the CPU-baseline / reference leg of bench.py.  The product package
(perft_gpu_gb300) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libperft_ref.so")
# the reference tree is looked for beside this repository unless REF_DIR names it
REF_DIR_DEFAULT = os.environ.get("REF_DIR") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))

BOARD_DTYPE = np.dtype([("white", "<u8"), ("pawns", "<u8"), ("knights", "<u8"),
                        ("bishop_queens", "<u8"), ("rook_queens", "<u8"), ("kings", "<u8")])
assert BOARD_DTYPE.itemsize == 48


class Board(ctypes.Structure):
    _fields_ = [("white", ctypes.c_uint64), ("pawns", ctypes.c_uint64),
                ("knights", ctypes.c_uint64), ("bishop_queens", ctypes.c_uint64),
                ("rook_queens", ctypes.c_uint64), ("kings", ctypes.c_uint64)]

    def as_tuple(self):
        return (self.white, self.pawns, self.knights, self.bishop_queens,
                self.rook_queens, self.kings)


def build(force: bool = False) -> str:
    """Compile oracle.c into liboracle.so (portable C11, any host)."""
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "oracle.h"))):
        tmp = LIB_PATH + ".tmp"
        subprocess.check_call(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-Wall",
                               "-o", tmp, src, "-lpthread"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_ref(ref_dir: str = REF_DIR_DEFAULT) -> str | None:
    """Build oracle/_ref from the reference sources when they are present."""
    if not os.path.isfile(os.path.join(ref_dir, "MoveGeneratorBitboard.h")):
        return None
    env = dict(os.environ, REF_DIR=ref_dir)
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], env=env,
                       capture_output=True, text=True)
    if r.returncode != 0:
        return None
    return REF_LIB_PATH


_BP = ctypes.POINTER(Board)
_U16P = ctypes.POINTER(ctypes.c_uint16)
_U64P = ctypes.POINTER(ctypes.c_uint64)
_U8P = ctypes.POINTER(ctypes.c_uint8)


class _Impl:
    """Common Python surface over oracle.c or the reference shim."""

    def __init__(self, lib, prefix):
        self.lib = lib
        self.p = prefix
        f = self._fn
        f("board_from_fen", ctypes.c_int, [ctypes.c_char_p, _BP])
        f("count_moves", ctypes.c_uint32, [_BP])
        f("generate_moves", ctypes.c_uint32, [_BP, _U16P])
        f("generate_boards", ctypes.c_uint32, [_BP, _BP])
        f("make_move", None, [_BP, ctypes.c_uint16])
        f("perft", ctypes.c_uint64, [_BP, ctypes.c_int])
        f("perft_batch", ctypes.c_double, [_BP, _U8P, ctypes.c_uint32, _U64P, ctypes.c_int])

    def _fn(self, name, res, args):
        fn = getattr(self.lib, self.p + name)
        fn.restype = res
        fn.argtypes = args
        setattr(self, "_" + name, fn)

    def fen(self, fen: str) -> Board:
        b = Board()
        self._board_from_fen(fen.encode(), ctypes.byref(b))
        return b

    def count_moves(self, b: Board) -> int:
        return self._count_moves(ctypes.byref(b))

    def generate_moves(self, b: Board) -> list[int]:
        buf = (ctypes.c_uint16 * 256)()
        n = self._generate_moves(ctypes.byref(b), buf)
        return list(buf[:n])

    def generate_boards(self, b: Board) -> list[tuple]:
        buf = (Board * 256)()
        n = self._generate_boards(ctypes.byref(b), buf)
        return [buf[i].as_tuple() for i in range(n)]

    def make_move(self, b: Board, move: int) -> Board:
        c = Board(*b.as_tuple())
        self._make_move(ctypes.byref(c), move)
        return c

    def perft(self, b: Board, depth: int) -> int:
        return self._perft(ctypes.byref(b), depth)

    def perft_batch(self, boards: np.ndarray, depths: np.ndarray, threads: int):
        boards = np.ascontiguousarray(boards, dtype=BOARD_DTYPE)
        depths = np.ascontiguousarray(depths, dtype=np.uint8)
        out = np.zeros(len(boards), dtype=np.uint64)
        secs = self._perft_batch(boards.ctypes.data_as(_BP), depths.ctypes.data_as(_U8P),
                                 len(boards), out.ctypes.data_as(_U64P), threads)
        return out, secs


class Oracle(_Impl):
    def __init__(self, slider_mode: int = 1):
        lib = ctypes.CDLL(build())
        super().__init__(lib, "or_")
        lib.or_init.argtypes = [ctypes.c_int]
        lib.or_init(slider_mode)
        f = self._fn
        f("perft_moves", ctypes.c_uint64, [_BP, ctypes.c_int])
        f("perft_divide", ctypes.c_uint32, [_BP, ctypes.c_int, _U16P, _U64P])
        f("playouts", None, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                             ctypes.c_int, ctypes.c_int, ctypes.c_int, _BP, _U8P])
        f("board_hash", ctypes.c_uint64, [_BP])

    def set_sliders(self, slider_mode: int):
        self.lib.or_init(slider_mode)

    def perft_moves(self, b: Board, depth: int) -> int:
        return self._perft_moves(ctypes.byref(b), depth)

    def perft_divide(self, b: Board, depth: int) -> dict[int, int]:
        mv = (ctypes.c_uint16 * 256)()
        cnt = (ctypes.c_uint64 * 256)()
        n = self._perft_divide(ctypes.byref(b), depth, mv, cnt)
        return {mv[i]: cnt[i] for i in range(n)}

    def playouts(self, seed, n, min_plies, max_plies, min_moves=1, depth_lo=0, depth_hi=0,
                 with_depths=False):
        out = np.zeros(n, dtype=BOARD_DTYPE)
        depths = np.zeros(n, dtype=np.uint8) if with_depths else None
        self._playouts(seed, n, min_plies, max_plies, min_moves, depth_lo, depth_hi,
                       out.ctypes.data_as(_BP),
                       depths.ctypes.data_as(_U8P) if with_depths else None)
        return (out, depths) if with_depths else out


class Reference(_Impl):
    def __init__(self, path: str = REF_LIB_PATH):
        lib = ctypes.CDLL(path)
        super().__init__(lib, "ref_")
        lib.ref_init()


def reference_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def board_from_array(row) -> Board:
    return Board(*(int(row[k]) for k in BOARD_DTYPE.names))
