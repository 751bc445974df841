#!/usr/bin/env python
"""bench.py -- batched uneven perft on one GB300 (and N replicas under torchrun).

Workload (one step): 4096 positions from seeded random legal playouts of 0-60
plies from the initial position, each with a depth drawn uniformly from 3..6
(seed 3), counted exactly with no transposition table.  The positions are made
on the GPU by the engine's own playout generator; their counts are checked
against tests/golden/config3.npz (the reference's own CPU counts).

  value   leaf nodes/s of pg_perft_batch_device with inputs resident in HBM,
          K steps bracketed by barrier + synchronize, CUDA events on the
          engine's stream, max over ranks; an L2-sized buffer is rewritten
          before every step (inside the timed region)
  e2e     the same metric through pg_perft_batch with host arrays (the call a
          user makes): H2D of boards + depths and D2H of the counts every step
  plain   the one-position-per-call GPU path (pg_perft per position) over the
          same workload, for the batched-vs-plain ratio of the metric

--impl reference times the reference's CPU perft on the host cores instead:
oracle/_ref (the reference compiled from its sources) where it was built,
else the oracle's C restatement of it, on the same fixed sample of the
workload every step (every 16th position, the sample of the cpu_baseline leg).

--profile-case N runs every (4096/N)-th position of the workload once
(Kogge-Stone sliders, 128-thread CTAs, two-ply leaf: the autotuner's choice
for the depths that hold most leaves; with --persistent as one persistent
launch), checks the counts and prints one JSON line: the small case of the
same kernels for ncu captures.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "bit-exact leaf nodes/s on 1 GB300 (batched vs plain); served perft p50/p99 latency"
WORKLOAD = dict(seed=3, n=4096, min_plies=0, max_plies=60, min_moves=1, depth_lo=3, depth_hi=6)
WORKLOAD_NAME = ("batched uneven perft: 4096 seeded random-playout positions (0-60 plies), "
                 "depth uniform 3..6, no TT")
LEAF_PARENT_BYTES = 48 + 4 + 1  # board + group id + remaining depth read per leaf-parent node
FALLBACK_HBM_GBS = 6800.0


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", FALLBACK_HBM_GBS)), "measured", d
    return FALLBACK_HBM_GBS, "fallback", {}


def golden_totals():
    p = os.path.join(ROOT, "tests", "golden", "config3.npz")
    if not os.path.exists(p):
        return None
    with np.load(p) as z:
        return z["totals"].copy(), z["boards"].copy(), z["depths"].copy()


class ClockSampler:
    """nvidia-smi clocks during the timed region (200 ms period)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile(prefix="clocks", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.close()
        rows = []
        with open(self.tmp.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        power = [num(r[3]) for r in rows if num(r[3]) is not None]
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(power) if power else None}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pgroup = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if _cuda_available() else "gloo"
        dist.init_process_group(backend=backend)
        pgroup = dist
    return world, rank, local, pgroup


def _cuda_available():
    import torch
    return torch.cuda.is_available()


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_model() -> str:
    """The host CPU's model name (lscpu), recorded beside every CPU number."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_leaves_per_s(boards, depths, threads, prefer_reference=True):
    """The reference's CPU perft over a sample of the workload: oracle/_ref when
    it was built here (the reference compiled from its sources), else the
    oracle's C restatement."""
    import oracle as O
    if prefer_reference and O.reference_available():
        impl, kind = O.Reference(), "reference"
    else:
        impl, kind = O.Oracle(1), "port"
    out, secs = impl.perft_batch(boards, depths, threads)
    return out, secs, kind


def config_of(n, leaves_per_step, slider, world):
    """The workload description shared by both arms' JSON lines."""
    return {"workload": WORKLOAD_NAME, "positions": n, "leaves_per_step": leaves_per_step, "slider": slider,
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "256 MiB buffer rewritten before every step (inside the timed region)"}


def run_reference(args):
    world, rank, local, dist = dist_setup()
    if rank != 0:
        return 0
    import oracle as O
    O.build()
    g = golden_totals()
    if g is None:
        boards, depths = O.Oracle(1).playouts(**{k: WORKLOAD[k] for k in ("seed", "n", "min_plies",
                                                                             "max_plies", "min_moves",
                                                                             "depth_lo", "depth_hi")},
                                               with_depths=True)
        totals = None
    else:
        totals, bw, depths = g
        boards = bw.view(O.BOARD_DTYPE).reshape(-1)
    threads = os.cpu_count() or 1
    stride = args.cpu_stride
    leaves = 0
    secs = 0.0
    kind = None
    idx = np.arange(0, len(boards), stride)  # the same sample every step
    for step in range(args.warmup + args.steps):
        out, s, kind = cpu_leaves_per_s(boards[idx], depths[idx], threads)
        if totals is not None and not np.array_equal(out, totals[idx]):
            print(json.dumps({"impl": "reference", "error": "CPU counts differ from golden"}))
            return 1
        if step >= args.warmup:
            leaves += int(out.sum())
            secs += s
    value = leaves / secs
    line = {
        "metric": METRIC, "value": value, "unit": "leaf nodes/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded playouts, same positions as the GPU arm)",
        "config": config_of(len(boards), int(totals.sum()) if totals is not None else None, args.slider, world),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "leaf nodes/s", "cores": threads, "kind": kind,
                         "cpu_model": cpu_model(),
                         "sample": "every %dth of the 4096 positions, the same %d positions (%d leaves) every "
                                   "step, each timed whole" % (stride, len(idx), int(out.sum()))},
        "e2e": {"value": value, "unit": "leaf nodes/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


SERVE_SEED = 5


def serve_requests(pg, n, seed=SERVE_SEED):
    """Request stream: playout positions (0-60 plies) and depths drawn from a
    lognormal (median 4, sigma 0.25) rounded and clipped to 3..8."""
    boards = pg.random_playouts(seed, n, 0, 60, 1)
    rng = np.random.default_rng(seed)
    depths = np.clip(np.rint(np.exp(rng.normal(np.log(4.0), 0.25, n))), 3, 8).astype(np.uint8)
    return boards, depths, rng


def pct(xs, q):
    return float(np.percentile(np.asarray(xs), q)) if len(xs) else None


def serve_leg(pg, rates, seconds, plain_rate):
    """Poisson arrivals at each rate for `seconds`; the server admits, batches
    and completes them; latency is measured by the server from submit to
    completion.  The plain path serves the same stream one pg_perft call per
    request, in arrival order."""
    import threading
    max_n = int(max(rates + [plain_rate]) * seconds * 1.5) + 64
    boards, depths, rng = serve_requests(pg, max_n)
    out = {"requests": "seeded playout positions (0-60 plies), depth lognormal(median 4, sigma 0.25) "
                       "clipped to 3..8; Poisson arrivals", "rates": [],
           "stable_def": "offered load (leaves of the requests / arrival window) at most 90% of the "
                         "saturated throughput (served leaves/s at the highest swept rate)"}
    check_n = 0
    for rate in rates:
        arrivals = np.cumsum(rng.exponential(1.0 / rate, max_n))
        n = int(np.searchsorted(arrivals, seconds))
        srv = pg.Server(hbm_budget_bytes=8 << 30)
        ids = []
        t0 = time.perf_counter()
        for i in range(n):
            dt = t0 + arrivals[i] - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            ids.append(srv.submit(pg.board_of(boards[i]), int(depths[i])))
        res = [srv.wait(r, timeout=900) for r in ids]
        wall = time.perf_counter() - t0
        srv.stop()
        lat = [l for _, l in res]
        leaves = sum(int(r) for r, _ in res)
        # every served count equals the batch engine's count for that request
        ref = pg.perft_batch(boards[:n], depths[:n])
        assert [int(r) for r, _ in res] == [int(x) for x in ref], "served counts differ"
        check_n += n
        out["rates"].append({"rate_req_s": rate, "requests": n, "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
                             "max_ms": max(lat) if lat else None, "leaves_per_s": leaves / wall,
                             "offered_leaves_per_s": leaves / float(arrivals[n - 1]) if n else 0.0,
                             "completed_per_s": n / wall})
    saturated = max(r["leaves_per_s"] for r in out["rates"])
    for r in out["rates"]:
        r["utilization"] = r["offered_leaves_per_s"] / saturated
        r["stable"] = r["utilization"] <= 0.9
    stable = [r for r in out["rates"] if r["stable"]]
    if stable:
        top = max(stable, key=lambda r: r["rate_req_s"])
        out["highest_sustained"] = {"rate_req_s": top["rate_req_s"], "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"]}
    # the same kind of stream at the middle rate with each wave as one
    # persistent launch (no per-level host round trips)
    arrivals = np.cumsum(rng.exponential(1.0 / plain_rate, max_n))
    n = int(np.searchsorted(arrivals, seconds))
    srv = pg.Server(hbm_budget_bytes=8 << 30, persistent=True)
    ids = []
    t0 = time.perf_counter()
    for i in range(n):
        dt = t0 + arrivals[i] - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        ids.append(srv.submit(pg.board_of(boards[i]), int(depths[i])))
    res = [srv.wait(r, timeout=900) for r in ids]
    wall = time.perf_counter() - t0
    srv.stop()
    lat = [l for _, l in res]
    ref = pg.perft_batch(boards[:n], depths[:n])
    assert [int(r) for r, _ in res] == [int(x) for x in ref], "persistent-wave counts differ"
    check_n += n
    out["persistent_waves"] = {"rate_req_s": plain_rate, "requests": n, "p50_ms": pct(lat, 50),
                               "p99_ms": pct(lat, 99), "max_ms": max(lat) if lat else None,
                               "leaves_per_s": sum(int(r) for r, _ in res) / wall,
                               "path": "server with each wave as one persistent launch"}
    # the same kind of stream at the middle rate, served through the
    # transposition tables (they persist across requests)
    arrivals = np.cumsum(rng.exponential(1.0 / plain_rate, max_n))
    n = int(np.searchsorted(arrivals, seconds))
    pg.tt_clear()
    srv = pg.Server(hbm_budget_bytes=8 << 30, use_tt=True)
    ids = []
    t0 = time.perf_counter()
    for i in range(n):
        dt = t0 + arrivals[i] - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        ids.append(srv.submit(pg.board_of(boards[i]), int(depths[i])))
    res = [srv.wait(r, timeout=900) for r in ids]
    wall = time.perf_counter() - t0
    srv.stop()
    lat = [l for _, l in res]
    ref = pg.perft_batch(boards[:n], depths[:n])
    assert [int(r) for r, _ in res] == [int(x) for x in ref], "TT-served counts differ"
    check_n += n
    out["tt"] = {"rate_req_s": plain_rate, "requests": n, "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
                 "max_ms": max(lat) if lat else None, "leaves_per_s": sum(int(r) for r, _ in res) / wall,
                 "path": "server with use_tt (tables persist across requests)"}
    # plain: one engine call per request, FIFO, same kind of stream
    arrivals = np.cumsum(rng.exponential(1.0 / plain_rate, max_n))
    n = int(np.searchsorted(arrivals, seconds))
    lat = []
    leaves = 0
    t0 = time.perf_counter()
    for i in range(n):
        dt = t0 + arrivals[i] - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        leaves += pg.perft(pg.board_of(boards[i]), int(depths[i]))
        lat.append(1e3 * (time.perf_counter() - (t0 + arrivals[i])))
    wall = time.perf_counter() - t0
    out["plain"] = {"rate_req_s": plain_rate, "requests": n, "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
                    "leaves_per_s": leaves / wall, "path": "one pg_perft call per request, arrival order"}
    out["verified_requests"] = check_n
    return out


def _golden_json(name):
    with open(os.path.join(ROOT, "tests", "golden", name)) as f:
        return json.load(f)


def _timed(fn):
    t0 = time.perf_counter()
    r = fn()
    return r, time.perf_counter() - t0


def workloads_leg(pg, threads):
    """One timed pass of each of the other workloads, every count checked:
    the 64-position depth-5 set (GPU batch, and the reference's CPU perft on
    all host threads and on one), the single deep position at depth 7 under
    every slider policy and with the TT, and the transposition-table workload
    (that position at depth 8 and 256 playout positions at depth 7, TT against
    no TT)."""
    out = {}
    # 64 positions at depth 5
    c1 = _golden_json("config1.json")
    b1 = pg.boards_array([pg.HexaBitBoardPosition(*(int(h, 16) for h in p["board"])) for p in c1["positions"]])
    d1 = np.array([p["depth"] for p in c1["positions"]], dtype=np.uint8)
    pg.perft_batch(b1, d1)
    st = pg.PgStats()
    r1, s1 = _timed(lambda: pg.perft_batch(b1, d1, stats=st))
    assert int(r1.sum()) == c1["total"]
    cpu_all = cpu_leaves_per_s(b1, d1, threads)
    cpu_one = cpu_leaves_per_s(b1, d1, 1)
    import oracle as O
    ks_out, ks_secs = O.Oracle(0).perft_batch(b1, d1, threads)  # the C restatement with Kogge-Stone sliders
    assert int(cpu_all[0].sum()) == c1["total"] and int(cpu_one[0].sum()) == c1["total"]
    assert int(ks_out.sum()) == c1["total"]
    out["64_positions_depth5"] = {
        "leaves": c1["total"], "gpu_leaves_per_s": c1["total"] / s1, "gpu_wall_s": s1,
        "gpu_device_ms": st.device_ms,
        "cpu": {"kind": cpu_all[2], "threads": threads, "cpu_model": cpu_model(),
                "leaves_per_s": c1["total"] / cpu_all[1],
                "kogge_stone_port_leaves_per_s": c1["total"] / ks_secs,
                "one_thread_leaves_per_s": c1["total"] / cpu_one[1]}}

    # one deep position (seed 2, 30 plies, >= 35 moves) at depth 7
    c2 = _golden_json("config2.json")
    b2 = pg.HexaBitBoardPosition(*(int(h, 16) for h in c2["board"]))
    rows = {}
    for sl in ("ks", "fancy", "byte", "hybrid", "auto"):
        pg.perft(b2, 6, slider=sl)
        st = pg.PgStats()
        r, s = _timed(lambda: pg.perft(b2, 7, slider=sl, stats=st))
        assert r == c2["perft7"], (sl, r)
        rows[sl] = {"leaves_per_s": r / s, "wall_s": s, "device_ms": st.device_ms,
                    "leaf_kernel_ms": st.leaf_kernel_ms, "launches": st.launches}
    pg.tt_clear()
    st = pg.PgStats()
    r, s = _timed(lambda: pg.perft(b2, 7, use_tt=True, stats=st))
    assert r == c2["perft7"]
    rows["tt"] = {"leaves_per_s": r / s, "wall_s": s, "device_ms": st.device_ms, "tt_probes": st.tt_probes,
                  "tt_hits": st.tt_hits, "tt_stores": st.tt_stores}
    out["single_position_depth7"] = {"leaves": c2["perft7"], "by_slider": rows}

    # the README's own figure: "position 2" (perft.cu:64) without TT, 27 G
    # leaf nodes/s on an overclocked GTX 780; depth 7 here, the count checked
    # by agreement of the engine's slider policies (depth 5 is in the goldens)
    fen2 = [f for f in _golden_json("fens.json") if f["name"] == "position2"][0]
    p2 = pg.board_from_fen(fen2["fen"])
    assert pg.perft(p2, 5) == fen2["perft"]["5"]
    pg.perft(p2, 6)
    st = pg.PgStats()
    r7, s7 = _timed(lambda: pg.perft(p2, 7, stats=st))
    assert r7 == pg.perft(p2, 7, slider="fancy")
    out["position2_depth7"] = {"leaves": r7, "leaves_per_s": r7 / s7, "wall_s": s7, "device_ms": st.device_ms,
                               "readme_gtx780_leaves_per_s": 27e9,
                               "note": "README figure is one overclocked GTX 780 (Kepler); not the same hardware"}

    # transposition-table workload: TT counts equal the no-TT counts.  Modes:
    # tables + in-level duplicate pass (use_tt=True), the duplicate pass alone
    # (use_tt="dedup"), no TT; and the tables' second call on the same
    # positions (warm tables: what they buy across calls and requests)
    def tt_row(run, leaves_of):
        rows = {}
        pg.tt_clear()
        for mode, kw in (("tables", {"use_tt": True}), ("tables_warm", {"use_tt": True}),
                         ("dedup_only", {"use_tt": "dedup"}), ("no_tt", {})):
            st = pg.PgStats()
            r, secs = _timed(lambda: run(stats=st, **kw))
            rows[mode] = {"seconds": secs, "device_ms": st.device_ms, "leaves": leaves_of(r)}
            if kw.get("use_tt") is True:
                rows[mode].update({"tt_probes": st.tt_probes, "tt_hits": st.tt_hits, "tt_stores": st.tt_stores,
                                   "hit_rate": st.tt_hits / st.tt_probes if st.tt_probes else None,
                                   "tt_entry_gb_per_s": (st.tt_probes + st.tt_stores) * 32 / (st.device_ms / 1e3)
                                   / 1e9 if st.device_ms else None})
        assert len({v["leaves"] for v in rows.values()}) == 1, rows
        for v in rows.values():
            v["speedup_vs_no_tt"] = rows["no_tt"]["seconds"] / v["seconds"]
        pg.tt_clear()
        return rows

    tt = {}
    tt["position_depth8"] = tt_row(lambda **kw: pg.perft(b2, 8, **kw), lambda r: int(r))
    c4 = np.load(os.path.join(ROOT, "tests", "golden", "config4_d5.npz"))
    b4 = c4["boards"].copy().view(pg.BOARD_DTYPE).reshape(-1)
    d4 = np.full(len(b4), 7, dtype=np.uint8)
    tt["256_positions_depth7"] = tt_row(lambda **kw: pg.perft_batch(b4, d4, **kw), lambda r: int(r.sum()))
    tt["note"] = ("128-bit Zobrist keys (two seeded 64-bit sets), per-depth tables of 32-byte entries with every "
                  "key bit verified (32 GiB in total); every mode's count equals the no-TT count")
    out["transposition_table"] = tt
    return out


def run_ours(args):
    import torch
    world, rank, local, dist = dist_setup()
    torch.cuda.set_device(local)
    import perft_gpu_gb300 as pg
    pg.load_library(build_if_missing=True)
    pg.init(device=local)
    slider = args.slider

    boards, depths = pg.random_playouts(WORKLOAD["seed"], WORKLOAD["n"], WORKLOAD["min_plies"],
                                        WORKLOAD["max_plies"], WORKLOAD["min_moves"],
                                        WORKLOAD["depth_lo"], WORKLOAD["depth_hi"], with_depths=True)
    n = len(boards)
    g = golden_totals()
    dev = torch.device("cuda", local)
    d_boards = torch.from_numpy(boards.view(np.uint8).copy()).to(dev)
    d_depths = torch.from_numpy(depths.copy()).to(dev)
    d_out = torch.zeros(n, dtype=torch.int64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.ExternalStream(pg.get_stream(), device=dev)

    def step_device(stats=None):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        kw = {"slider": slider}
        if stats is not None:
            kw["stats"] = stats
        pg.perft_batch_device(d_boards.data_ptr(), d_depths.data_ptr(), n, d_out.data_ptr(), **kw)

    # warm-up (also verifies the counts)
    for _ in range(args.warmup):
        step_device()
    out = d_out.cpu().numpy().view(np.uint64)
    leaves_per_step = int(out.sum())
    verified = None
    if g is not None:
        verified = bool(np.array_equal(out, g[0]) and np.array_equal(boards.view(np.uint64).reshape(-1, 6), g[1]))
        if not verified:
            print(json.dumps({"error": "batched counts differ from the reference's golden counts"}))
            return 1

    # timed region: K steps, inputs resident in HBM
    clocks = ClockSampler(local)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    launches = 0
    leaf_ms = 0.0
    leaf_launches = 0
    leaf_nodes = 0
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        st = pg.PgStats()
        step_device(st)
        launches += st.launches
        leaf_ms += st.leaf_kernel_ms
        leaf_launches += st.leaf_kernel_launches
        leaf_nodes += st.leaf_parent_nodes
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    clk = clocks.stop()
    elapsed = ev0.elapsed_time(ev1) / 1e3
    elapsed_max = max_over_ranks(dist, elapsed)
    value = leaves_per_step * args.steps * world / elapsed_max

    # the same steps replayed from a captured CUDA graph (first call captures)
    def step_graph():
        with torch.cuda.stream(stream):
            flush.fill_(1)
        pg.perft_batch_device(d_boards.data_ptr(), d_depths.data_ptr(), n, d_out.data_ptr(), slider=slider,
                              graph=True)
    step_graph()
    assert int(d_out.cpu().numpy().view(np.uint64).sum()) == leaves_per_step
    barrier(dist)
    torch.cuda.synchronize()
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(args.steps):
        step_graph()
    g1.record(stream)
    torch.cuda.synchronize()
    graph_el = max_over_ranks(dist, g0.elapsed_time(g1) / 1e3)
    graph_value = leaves_per_step * args.steps * world / graph_el
    assert int(d_out.cpu().numpy().view(np.uint64).sum()) == leaves_per_step

    # the same steps as one persistent cooperative launch per step (levels
    # and chunks walked on the device), and that launch replayed from a graph
    def step_persist(graph):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        pg.perft_batch_device(d_boards.data_ptr(), d_depths.data_ptr(), n, d_out.data_ptr(), persistent=True,
                              graph=graph)

    persist = {}
    psteps = min(args.steps, 5)
    for name, graph in (("launch", False), ("graph", True)):
        step_persist(graph)
        assert int(d_out.cpu().numpy().view(np.uint64).sum()) == leaves_per_step
        barrier(dist)
        torch.cuda.synchronize()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(psteps):
            step_persist(graph)
        p1.record(stream)
        torch.cuda.synchronize()
        el = max_over_ranks(dist, p0.elapsed_time(p1) / 1e3)
        assert int(d_out.cpu().numpy().view(np.uint64).sum()) == leaves_per_step
        persist[name] = {"value": leaves_per_step * psteps * world / el, "unit": "leaf nodes/s",
                         "ms_per_step": 1e3 * el / psteps, "steps": psteps}
    persist["note"] = ("one cooperative persistent launch per step (Kogge-Stone, 128-thread CTAs, two-ply leaf); "
                       "'graph': that launch replayed from a captured graph (valid for any contents)")

    # the same steps with the in-level duplicate pass (use_tt="dedup": no
    # tables, nothing kept between steps; every step recomputes its counts)
    def step_dedup():
        with torch.cuda.stream(stream):
            flush.fill_(1)
        pg.perft_batch_device(d_boards.data_ptr(), d_depths.data_ptr(), n, d_out.data_ptr(), use_tt="dedup")

    step_dedup()
    assert int(d_out.cpu().numpy().view(np.uint64).sum()) == leaves_per_step
    if g is not None:
        assert np.array_equal(d_out.cpu().numpy().view(np.uint64), g[0])
    barrier(dist)
    torch.cuda.synchronize()
    q0 = torch.cuda.Event(enable_timing=True)
    q1 = torch.cuda.Event(enable_timing=True)
    q0.record(stream)
    for _ in range(psteps):
        step_dedup()
    q1.record(stream)
    torch.cuda.synchronize()
    dedup_el = max_over_ranks(dist, q0.elapsed_time(q1) / 1e3)
    dedup = {"value": leaves_per_step * psteps * world / dedup_el, "unit": "leaf nodes/s",
             "ms_per_step": 1e3 * dedup_el / psteps, "steps": psteps,
             "note": "same workload and counts with the in-level duplicate pass (128-bit keys, no tables kept "
                     "between steps); not the headline, which counts every node"}

    # end to end through the public API with host buffers
    pin_b = torch.from_numpy(boards.view(np.uint8).copy()).pin_memory()
    pin_d = torch.from_numpy(depths.copy()).pin_memory()
    host_boards = pin_b.numpy().view(pg.BOARD_DTYPE)
    host_depths = pin_d.numpy()
    e2e_t0 = torch.cuda.Event(enable_timing=True)
    e2e_t1 = torch.cuda.Event(enable_timing=True)
    barrier(dist)
    torch.cuda.synchronize()
    e2e_t0.record(stream)
    for _ in range(args.steps):
        res = pg.perft_batch(host_boards, host_depths, slider=slider)
        assert int(res.sum()) == leaves_per_step
    e2e_t1.record(stream)
    torch.cuda.synchronize()
    e2e_el = max_over_ranks(dist, e2e_t0.elapsed_time(e2e_t1) / 1e3)
    e2e_value = leaves_per_step * args.steps * world / e2e_el

    line = None
    if rank == 0:
        # plain: one position per engine call, same workload (one pass)
        plain = None
        if not args.no_plain:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            tot = 0
            for i in range(n):
                tot += pg.perft(pg.board_of(boards[i]), int(depths[i]), slider=slider)
            plain_s = time.perf_counter() - t0
            assert tot == leaves_per_step
            plain = {"value": tot / plain_s, "unit": "leaf nodes/s", "seconds": plain_s,
                     "calls": n, "timing": "host wall clock around the per-position calls"}

        # roofline of the dominant kernel (k_leaf): integer-ALU issue, with the
        # ALU warp instructions per leaf and the DRAM bytes per leaf-parent
        # node of the ncu capture of this workload (every 16th position,
        # profiles/k_leaf_batched_uneven_256.md) applied to the live leaf
        # time of the timed steps; HBM as the secondary roofline
        peak, peak_kind, peaks = measured_peaks()
        per_launch_ms = leaf_ms / max(leaf_launches, 1)
        bytes_per_launch = leaf_nodes * LEAF_PARENT_BYTES / max(leaf_launches, 1)
        achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9 if per_launch_ms else 0.0
        traffic = None
        alu = None
        tfile = os.path.join(ROOT, "profiles", "k_leaf_batched_uneven_256.json")
        if os.path.exists(tfile):
            with open(tfile) as f:
                tj = json.load(f)
            traffic = tj["dram_bytes_per_leaf_parent"] * leaf_nodes / max(leaf_launches, 1)
            sms = torch.cuda.get_device_properties(dev).multi_processor_count
            mhz = float(peaks.get("sm_max_mhz") or clk.get("sm_max_mhz") or 2070.0)
            alu_peak = tj["alu_peak_warp_inst_per_clk_per_sm"] * sms * mhz * 1e6
            ach = tj["alu_warp_inst_per_leaf"] * leaves_per_step * args.steps / (leaf_ms / 1e3) if leaf_ms else 0.0
            alu = {"bound": "alu", "kernel": "k_leaf", "achieved": ach / 1e9, "peak": alu_peak / 1e9,
                   "unit": "G warp-inst/s", "frac": ach / alu_peak,
                   "traffic": traffic,
                   "alu_warp_inst_per_leaf": tj["alu_warp_inst_per_leaf"],
                   "achieved_def": "ALU warp-instructions per leaf (ncu, this workload) x leaves of the "
                                   "timed steps / live k_leaf time (CUDA events)",
                   "peak_source": "ncu sm__inst_executed_pipe_alu.avg.peak_sustained (%d/clk/SM) x %d SMs x "
                                  "%.0f MHz (sm_max_mhz of MEASURED_PEAKS.json)"
                                  % (tj["alu_peak_warp_inst_per_clk_per_sm"], sms, mhz),
                   "source": tj["source"]}
        hbm = {"bound": "hbm", "kernel": "k_leaf", "achieved": achieved, "peak": peak, "unit": "GB/s",
               "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
               "note": "algorithmic bytes: the leaf-parent boards read (53 B/node); leaves are counted, "
                       "never stored"}

        workloads = None
        if not args.no_workloads:
            workloads = workloads_leg(pg, os.cpu_count() or 1)

        served = None
        if not args.no_serve:
            rates = [float(x) for x in args.serve_rates.split(",")]
            served = serve_leg(pg, rates, args.serve_seconds, 50.0 if 50.0 in rates else rates[len(rates) // 2])

        cpu = None
        if not args.no_cpu:
            idx = np.arange(0, n, args.cpu_stride)
            threads = os.cpu_count() or 1
            cout, csecs, kind = cpu_leaves_per_s(boards[idx], depths[idx], threads)
            if g is not None:
                assert np.array_equal(cout, g[0][idx])
            cpu = {"value": int(cout.sum()) / csecs, "unit": "leaf nodes/s", "cores": threads,
                   "cpu_model": cpu_model(),
                   "kind": kind,
                   "sample": "every %dth of the 4096 positions (%d positions, %d leaves)"
                             % (args.cpu_stride, len(idx), int(cout.sum()))}

        line = {
            "metric": METRIC, "value": value, "unit": "leaf nodes/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * elapsed_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded random legal playouts made on the GPU; counts verified "
                    "against the reference's golden counts)" if verified else "synthetic",
            "config": config_of(n, leaves_per_step, slider, world),
            "verified_bit_exact": verified,
            "e2e": {"value": e2e_value, "unit": "leaf nodes/s",
                    "h2d_bytes_per_step": n * 48 + n, "d2h_bytes_per_step": n * 8},
            "gpu_launches": launches,
            "persistent": persist,
            "dedup": dedup,
            "graph_replay": {"value": graph_value, "unit": "leaf nodes/s",
                             "ms_per_step": 1e3 * graph_el / args.steps,
                             "note": "same steps replayed from one captured CUDA graph per step"},
            "autotune": pg.autotune(),
            "plain": plain,
            "batched_vs_plain": (value / plain["value"]) if plain else None,
            "roofline": alu if alu is not None else hbm,
            "roofline_hbm": hbm,
            "leaf_kernel": {"launches": leaf_launches, "ms_total": leaf_ms,
                            "ms_per_launch": per_launch_ms,
                            "share_of_timed": leaf_ms / (elapsed * 1e3)},
            "cpu_baseline": cpu,
            "served": served,
            "workloads": workloads,
            "clocks": clk,
        }
    barrier(dist)
    pg.shutdown()
    if line is not None:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_profile_case(args):
    """One pass over a subset of the batched workload, for ncu captures."""
    import perft_gpu_gb300 as pg
    pg.load_library(build_if_missing=True)
    pg.init()
    g = golden_totals()
    boards, depths = pg.random_playouts(WORKLOAD["seed"], WORKLOAD["n"], WORKLOAD["min_plies"],
                                        WORKLOAD["max_plies"], WORKLOAD["min_moves"],
                                        WORKLOAD["depth_lo"], WORKLOAD["depth_hi"], with_depths=True)
    idx = np.arange(0, len(boards), max(1, len(boards) // args.profile_case))
    st = pg.PgStats()
    if args.persistent:
        out = pg.perft_batch(boards[idx], depths[idx], persistent=True, stats=st)
    else:
        out = pg.perft_batch(boards[idx], depths[idx], slider="ks", block_size=128, leaf_plies=2, stats=st)
    ok = bool(np.array_equal(out, g[0][idx])) if g is not None else None
    print(json.dumps({"profile_case": len(idx), "persistent": bool(args.persistent),
                      "positions": "every %dth of the batched workload" % (len(boards) // len(idx)),
                      "leaves": int(out.sum()), "verified_bit_exact": ok,
                      "leaf_kernel_launches": st.leaf_kernel_launches, "leaf_parent_nodes": st.leaf_parent_nodes,
                      "leaf_kernel_ms": st.leaf_kernel_ms, "device_ms": st.device_ms, "launches": st.launches}))
    pg.shutdown()
    return 0 if ok is not False else 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--slider", default="auto", choices=["auto", "ks", "fancy", "byte", "hybrid"])
    ap.add_argument("--cpu-stride", type=int, default=16,
                    help="CPU legs time every k-th position (bounded sample)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-workloads", action="store_true",
                    help="skip the other workloads (64 x depth 5, one position at depth 7, TT)")
    ap.add_argument("--serve-rates", default="25,50,75,100,150,200", help="Poisson request rates (req/s)")
    ap.add_argument("--serve-seconds", type=float, default=8.0)
    ap.add_argument("--profile-case", type=int, default=0,
                    help="run N positions of the workload once and exit (small case for ncu)")
    ap.add_argument("--persistent", action="store_true",
                    help="with --profile-case: as one persistent launch")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.profile_case:
        return run_profile_case(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
