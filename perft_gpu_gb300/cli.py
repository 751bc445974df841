"""Command line entry, the GB300 counterpart of the reference's perft_gpu
binary (perft.cu:14-164):

    python -m perft_gpu_gb300 [<fen>] [<depth>] [<numGPUs>] [<launchDepth>]
                              [--min-depth D] [--divide] [--slider ks|fancy|byte|hybrid]
                              [--tt] [--tt-mib N] [--hbm-budget-mib N] [--stats]

Like perft.cu it runs perft for every depth from the minimum (3) to <depth>
and prints one "GPU Perft" line per depth (perftLauncher, launcher.h:1488-1498).
<numGPUs> must be 1 (one GPU per process); <launchDepth> is accepted for
compatibility and ignored: the engine plans its own breadth-first split from
the HBM budget.  --divide prints the per-move counts of the last depth with
the reference's move strings (Utils::getCompactMoveString, utils.h:251-258).
--tt-mib sizes the transposition tables (default: from the HBM budget),
--hbm-budget-mib caps the engine's device memory, --stats prints the engine's
counters (launches, TT probes/hits/stores) after each depth.
"""
from __future__ import annotations

import argparse
import sys
import time

from . import PgStats, Utils, board_from_fen, init, perft, perft_divide, shutdown

START_FEN = "rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1"


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="perft_gpu_gb300")
    ap.add_argument("fen", nargs="?", default=START_FEN)
    ap.add_argument("depth", nargs="?", type=int, default=3)
    ap.add_argument("num_gpus", nargs="?", type=int, default=1)
    ap.add_argument("launch_depth", nargs="?", type=int, default=0)
    ap.add_argument("--min-depth", type=int, default=3)
    ap.add_argument("--divide", action="store_true")
    ap.add_argument("--slider", default="auto", choices=["auto", "ks", "fancy", "byte", "hybrid"])
    ap.add_argument("--tt", action="store_true", help="use the transposition tables")
    ap.add_argument("--tt-mib", type=int, default=0, help="transposition-table MiB (0 = from the budget)")
    ap.add_argument("--hbm-budget-mib", type=int, default=0, help="engine device-memory budget (0 = default)")
    ap.add_argument("--stats", action="store_true", help="print the engine's counters per depth")
    a = ap.parse_args(argv)
    if a.num_gpus != 1:
        print("numGPUs %d requested; this engine drives one GPU per process" % a.num_gpus,
              file=sys.stderr)
    fen = a.fen if len(a.fen) > 5 else START_FEN
    init(hbm_budget_bytes=a.hbm_budget_mib << 20)
    pos = board_from_fen(fen)
    for d in range(min(a.min_depth, a.depth), a.depth + 1):
        st = PgStats()
        t0 = time.perf_counter()
        res = perft(pos, d, slider=a.slider, use_tt=a.tt, tt_bytes=a.tt_mib << 20, stats=st)
        dt = time.perf_counter() - t0
        print("GPU Perft %d: %d,   Time taken: %g seconds, nps: %d" % (d, res, dt, int(res / dt) if dt else 0))
        if a.stats:
            print("  stats: " + ", ".join("%s=%s" % kv for kv in st.as_dict().items()))
        sys.stdout.flush()
    if a.divide and a.depth >= 1:
        for m, c in perft_divide(pos, a.depth, slider=a.slider, use_tt=a.tt, tt_bytes=a.tt_mib << 20):
            print("%s %d" % (Utils.getCompactMoveString(m), c))
    shutdown()
    return 0
