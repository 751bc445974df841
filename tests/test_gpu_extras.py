"""Deep divided perft with the host complete TT, the command-line binary and
its records mode, and failure detection (a bounded device wait that is made
to run out, an injected host allocation failure, a request the server cannot
admit) -- none of which faults or hangs the GPU."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_json

pytestmark = pytest.mark.gpu
CLI = os.path.join(ROOT, "perft_gpu_gb300", "perft_gpu")


def test_split_perft_matches_divide_and_reference(pg):
    fens = {f["name"]: f for f in golden_json("fens.json")}
    start = pg.board_from_fen(fens["start"]["fen"])
    st = pg.PgStats()
    split = pg.perft_split(start, 6, split_plies=3, stats=st)
    assert sum(c for _, c in split) == fens["start"]["perft"]["6"]
    assert split == pg.perft_divide(start, 6)
    assert st.tt_probes > st.tt_hits > 0  # transpositions merged at ply 3
    p2 = pg.board_from_fen(fens["position2"]["fen"])
    assert [[m, c] for m, c in pg.perft_split(p2, 4, split_plies=2)] == fens["position2"]["divide3"] or \
        sum(c for _, c in pg.perft_split(p2, 4, split_plies=2)) == fens["position2"]["perft"]["4"]
    assert sum(c for _, c in pg.perft_split(p2, 5, split_plies=2, use_tt=True)) == fens["position2"]["perft"]["5"]


def test_bounded_wait_gives_up_and_engine_stays_usable(pg):
    assert pg.selftest(pg.SELFTEST_BOUNDED_WAIT) == 6  # PG_ERR_DEVICE_TIMEOUT
    b = pg.board_from_fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    assert pg.perft(b, 4) == 197281


def test_injected_allocation_failure_is_reported_then_recovers(pg):
    b = pg.board_from_fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    assert pg.selftest(pg.SELFTEST_FAIL_NEXT_ALLOC) == 0
    with pytest.raises(pg.PerftError) as e:
        pg.perft(b, 5)
    assert e.value.status == 5  # PG_ERR_OUT_OF_MEMORY
    assert pg.perft(b, 5) == 4865609


def test_server_rejects_request_larger_than_its_pool(pg):
    srv = pg.Server(hbm_budget_bytes=4096, max_inflight=4)
    try:
        b = pg.board_from_fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
        rid = srv.submit(b, 8)
        with pytest.raises(pg.PerftError) as e:
            srv.wait(rid, timeout=60)
        assert e.value.status == 8  # PG_ERR_CAPACITY
        ok = srv.submit(b, 3)
        assert srv.wait(ok)[0] == 8902
    finally:
        srv.stop()


def test_cli_matches_reference_lines(tmp_path):
    fens = {f["name"]: f for f in golden_json("fens.json")}
    out = subprocess.run([CLI, fens["position2"]["fen"], "4"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert "GPU Perft 3: 97862," in out.stdout and "GPU Perft 4: 4085603," in out.stdout
    out = subprocess.run([CLI, fens["start"]["fen"], "4", "-divide"], capture_output=True, text=True, timeout=300)
    assert "Perft(04):              197281" in out.stdout and "..e2-e4 " in out.stdout


def test_cli_records_mode_resumes(tmp_path):
    fens = {f["name"]: f for f in golden_json("fens.json")}
    rec = tmp_path / "records.txt"
    names = ["start", "position2", "position3", "position4"]
    rec.write_text("".join("%s %d\n" % (fens[n]["fen"].strip(), k + 1) for k, n in enumerate(names[:2])))
    r = subprocess.run([CLI, "-records", str(rec), "4"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    with open(str(rec) + ".op", "a"):
        pass
    rec.write_text(rec.read_text() + "".join("%s %d\n" % (fens[n]["fen"].strip(), k + 3)
                                            for k, n in enumerate(names[2:])))
    r = subprocess.run([CLI, "-records", str(rec), "4"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = open(str(rec) + ".op").read().splitlines()
    assert len(lines) == 4
    for k, (n, line) in enumerate(zip(names, lines)):
        res, weighted = line.split()[-2:]
        assert int(res) == fens[n]["perft"]["4"] and int(weighted) == fens[n]["perft"]["4"] * (k + 1)


def test_python_cli_tt_options(tmp_path):
    """python -m perft_gpu_gb300 with a small TT, a capped HBM budget and the
    engine counters: same counts as the reference, counters printed."""
    import sys
    fens = {f["name"]: f for f in golden_json("fens.json")}
    cmd = [sys.executable, "-m", "perft_gpu_gb300", fens["position3"]["fen"], "5", "--min-depth", "4",
           "--tt", "--tt-mib", "64", "--hbm-budget-mib", "1024", "--stats"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    assert "GPU Perft 4: %d," % fens["position3"]["perft"]["4"] in out.stdout
    assert "GPU Perft 5: %d," % fens["position3"]["perft"]["5"] in out.stdout
    assert "tt_probes=" in out.stdout and "tt_stores=" in out.stdout


def test_cli_tt_snapshot_between_runs(tmp_path):
    """perft_gpu -ttsave writes the tables at exit; a second run with -ttload
    starts from them and prints the same counts."""
    fens = {f["name"]: f for f in golden_json("fens.json")}
    snap = str(tmp_path / "tt.snap")
    fen = fens["position4"]["fen"]
    r1 = subprocess.run([CLI, fen, "5", "-ttmib", "64", "-ttsave", snap], capture_output=True, text=True,
                        timeout=300)
    assert r1.returncode == 0, r1.stderr
    assert 0 < os.path.getsize(snap) <= (64 << 20) + 4096
    r2 = subprocess.run([CLI, fen, "5", "-ttmib", "64", "-ttload", snap], capture_output=True, text=True,
                        timeout=300)
    assert r2.returncode == 0, r2.stderr
    for d in (3, 4, 5):
        line = "GPU Perft %d: %d," % (d, fens["position4"]["perft"][str(d)])
        assert line in r1.stdout and line in r2.stdout
