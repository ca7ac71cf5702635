#!/usr/bin/env python3
"""Benchmark of the GB300-native cuJSON parse path.

One step = one full parse (UTF-8 validation, tokenization, structural
compaction, nesting/pair recognition) of the 1 GiB standard-JSON workload
(seeded stand-in for the reference's ~1 GB datasets: depth <= 20, 1% of strings
64-128 KiB of backslash runs).

  value        device-resident parse GB/s (input already in HBM; CUDA events on
               the launching stream around K steps; whole job over all ranks)
  e2e          the same metric through the C ABI with host buffers: pinned H2D of
               the input, parse, D2H of the verdict and the result arrays
  roofline     the dominant (scan) kernel: algorithmic bytes N + 8*S per launch
               over its CUDA-event time, against the measured HBM copy bandwidth
  cpu_baseline simdjson (the copy the reference ships with its paper's related
               work, built for this machine) on the same 1 GiB document, on
               every host core (independent parsers), beside one core; the
               oracle port's figure is in cpu_baseline_port

``--impl reference`` times the reference's algorithm on the host cores (the
oracle port; the reference's own path is CUDA-only and its sources are not on
the GPU machine): every host thread parses the same 1 GiB document per step.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np
from tests import synth

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "parse GB/s (1 GiB standard JSON, device-resident)"
UNIT = "GB/s"
WORKLOAD = ("standard JSON, 1 GiB (1073741824 B), seed 0xC0DE0002, top-level array of objects "
            "(10-30 keys), nesting <= 20, 1% of strings 64-128 KiB of backslash runs")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=1 << 30, help="input bytes (default 1 GiB)")
    ap.add_argument("--cpu-sample", type=int, default=256 << 20, help="CPU-baseline sample bytes")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-documents measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-query", action="store_true", help="skip the device query measurement")
    ap.add_argument("--no-values", action="store_true", help="skip the value decoding measurement")
    ap.add_argument("--no-configs", action="store_true", help="skip configs 1 and 3")
    ap.add_argument("--query-bytes", type=int, default=0,
                    help="event-log bytes of the query measurement (default: the 2 GB JSON-Lines limit)")
    return ap.parse_args()


def workload(size: int):
    seed = synth.CONFIG_SEED_BASE + 2
    return synth.synth_document(seed, size, max_depth=20, huge_string_frac=0.01,
                             huge_string_min=64 << 10, huge_string_max=128 << 10)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_byte():
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return None
    return None


class Clocks:
    """nvidia-smi sampler running during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.rows = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def pinned_h2d_gbs(host: np.ndarray, device: int):
    """Best of 5 plain copies of the pinned input to the device (the link's
    bandwidth for this buffer), or None without torch."""
    try:
        import torch
        src = torch.from_numpy(host)
        dst = torch.empty(host.size, dtype=torch.uint8, device=f"cuda:{device}")
        best = None
        for _ in range(6):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            dst.copy_(src, non_blocking=True)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        del dst
        return host.size / best / 1e9
    except Exception:
        return None


def cpu_baseline_sample(sample_bytes: int):
    """Oracle (CPU restatement of the reference algorithm), one thread, on a
    bounded sample of the same generator; returns (GB/s, description)."""
    from oracle import cj_oracle
    d = synth.synth_document(synth.CONFIG_SEED_BASE + 2, sample_bytes, max_depth=20,
                          huge_string_frac=0.01, huge_string_min=64 << 10,
                          huge_string_max=128 << 10)
    cj_oracle.parse(d[: 1 << 20])        # load + warm
    reps, t_total = 0, 0.0
    while t_total < 10.0 and reps < 40:
        t0 = time.perf_counter()
        r = cj_oracle.parse(d)
        t_total += time.perf_counter() - t0
        reps += 1
    assert r.flags == 0
    gbs = sample_bytes * reps / t_total / 1e9
    return gbs, f"{sample_bytes} B document from the same generator, parsed {reps}x ({t_total:.1f} s)"


def workload_config(N: int, world: int) -> dict:
    """The `config` object both arms print (identical for the same workload)."""
    wl = WORKLOAD if N == 1 << 30 else WORKLOAD.replace("1 GiB (1073741824 B)", f"{N} B")
    l2 = ("input larger than the 129 MB L2, no flush between steps" if N > 129 * 10 ** 6
          else "input fits the 129 MB L2 (warm-L2 figure)")
    return {"workload": wl, "bytes": N, "parallelism": f"replicas x{world}", "l2": l2}


def run_reference(args, world, rank):
    """Reference arm: the reference's algorithm restated in C (the oracle
    port) on all host cores.  Each step, every host thread parses the whole
    1 GiB benchmark document (independent instances over the same bytes);
    value = threads x bytes / step time.  Loads only the oracle and the input
    generator, nothing of the GPU library."""
    if rank != 0:
        return
    from oracle import cj_oracle
    from concurrent.futures import ThreadPoolExecutor
    cores = os.cpu_count() or 1
    d = workload(args.size)
    N = d.size
    first = cj_oracle.parse(d)           # the counts, to size each thread's outputs
    if first.flags:
        raise SystemExit("oracle rejected the workload")
    S = first.n_structural
    L = cj_oracle.lib()
    outs = [(np.zeros(S + 1, np.int32), np.zeros(S + 1, np.int32)) for _ in range(cores)]

    def one(i):
        st = cj_oracle._Stats()
        pos, pair = outs[i]
        L.cjo_parse(d.ctypes.data, N, 0, None, 0, pos.ctypes.data, pair.ctypes.data, S + 1,
                    ctypes.byref(st))
        return st.flags == 0 and st.n_structural == S

    ex = ThreadPoolExecutor(max_workers=cores)

    def step():
        if not all(ex.map(one, range(cores))):
            raise SystemExit("oracle result differs between runs")

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    value = N * cores * args.steps / dt / 1e9
    desc = (f"{cores} host threads per step, each parsing the whole {N} B benchmark document "
            f"(independent instances over the same bytes)")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": workload_config(N, world),
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": desc},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def simdjson_baseline(data: np.ndarray):
    """simdjson 3.2.1 (the amalgamation the reference ships under
    paper_reproduced/related_works/simdjson/, built here for this machine by
    oracle/build_ref.py) on the benchmark document, timed on this machine's
    host cores: ondemand::parser::iterate (UTF-8 validation + structural
    index, cuJSON's stages 1-2) on 1 core and on every core (independent
    parsers over the same bytes), and dom::parser::parse (the full tape,
    nesting included) on every core.  None when its sources are absent."""
    import tempfile
    from oracle import build_ref
    try:
        exe = build_ref.build_simdjson()
    except Exception as e:                      # a failed build is reported, not fatal
        return {"unavailable": f"simdjson build failed: {str(e)[-200:]}"}
    if exe is None:
        return None
    cores = os.cpu_count() or 1
    res = {}
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "doc.json"
        data.tofile(path)
        for key, mode, threads, reps in (("index_1", "index", 1, 3), ("index_all", "index", cores, 2),
                                         ("dom_all", "dom", cores, 1)):
            r = subprocess.run([str(exe), str(path), mode, str(threads), str(reps)], capture_output=True,
                               text=True, timeout=900)
            if r.returncode != 0:
                res[key] = None
                continue
            f = r.stdout.split()
            res[key] = float(f[4])
    return {"cores": cores, "GBps": res}


BATCH_DOCS = 4096
BATCH_BYTES = 2 << 30


def plain_parse(cj, ctx, view, out):
    """One document through the per-document drop-in path (cj_parse_into)."""
    info = cj.ParseInfo()
    return cj.lib().cj_parse_into(ctx.handle, view.ctypes.data, view.size, 0, out.ctypes.data, out.size,
                                  ctypes.byref(info))


def run_batch(args, local):
    """Batched documents: one graph replay parses the whole batch, against a
    loop of plain per-document parses of the same documents."""
    import cujson_gb300 as cj
    seed = synth.CONFIG_SEED_BASE + 4
    pin = cj.PinnedBuffer(BATCH_BYTES + (256 << 20))
    t_gen = time.perf_counter()
    packed, sizes, kinds = synth.batch_input(seed, BATCH_DOCS, BATCH_BYTES, out=pin.array)
    t_gen = time.perf_counter() - t_gen
    n = int(sizes.size)
    N = int(sizes.sum())
    ctx = cj.Context(local)
    ctx.stage_batch_packed(packed, sizes)
    best, tried = ctx.autotune(reps=2)
    # the winner kept per GPU name and applied to a fresh context
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        tpath = os.path.join(td, "tuning.jsonl")
        ctx.save_tuning(tpath)
        tctx = cj.Context(local)
        tctx.load_tuning(tpath)
        persisted = tctx.get_tuning().as_dict()
        tctx.close()
    ctx.run_graph()
    layout, status, S, depth, off = ctx.batch_layout()
    verdicts_ok = bool(((status != 0) == (kinds > 0)).all())
    total_out = int(off[-1])

    # device-resident: graph replays of the staged batch
    for _ in range(args.warmup):
        ctx.run_graph()
    ctx.batch_info()
    launches0 = ctx.launches
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.run_graph()
    ctx.batch_info()                       # synchronises
    dev_s = (time.perf_counter() - t0) / args.steps
    launches = (ctx.launches - launches0) // args.steps

    # end to end: pinned packed input -> one H2D + scatter, graph replay,
    # per-document verdicts, one D2H of every document's layout
    out_pin = cj.PinnedBuffer(total_out * 4 + 64, dtype=np.int32)
    for _ in range(max(1, args.warmup)):
        ctx.stage_batch_packed(packed, sizes)
        ctx.run_graph()
        ctx.batch_layout(out_pin.array)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.stage_batch_packed(packed, sizes)
        ctx.run_graph()
        ctx.batch_layout(out_pin.array)
    e2e_s = (time.perf_counter() - t0) / args.steps
    same = bool(np.array_equal(out_pin.array[:total_out], layout))

    # end to end, overlapped: the batch already in the device layout (1 KiB-
    # aligned documents, cj_batch_padded_offsets) in pinned memory, copied in
    # chunks while the scan runs; verdicts and every layout back to the host
    poff, ptotal = cj.batch_padded_offsets(sizes)
    pad_pin = cj.PinnedBuffer(ptotal)
    src = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    for i in range(n):
        pad_pin.array[int(poff[i]):int(poff[i]) + int(sizes[i])] = packed[src[i]:src[i + 1]]
    for _ in range(max(1, args.warmup)):
        ctx.parse_batch_padded(pad_pin.array, sizes)
        ctx.batch_layout(out_pin.array)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.parse_batch_padded(pad_pin.array, sizes)
        ctx.batch_layout(out_pin.array)
    e2e_pad_s = (time.perf_counter() - t0) / args.steps
    same_pad = bool(np.array_equal(out_pin.array[:total_out], layout))
    pad_pin.close()

    # plain loop: one cj_parse_into per document, pinned input slices
    ctx2 = cj.Context(local)
    ctx2.reserve(int(sizes.max()), 1)
    plain_out = cj.PinnedBuffer((2 * int(sizes.max()) + 4) * 4, dtype=np.int32)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    views = [packed[offs[i]:offs[i + 1]] for i in range(n)]
    for i in range(min(n, 64)):
        plain_parse(cj, ctx2, views[i], plain_out.array)
    t0 = time.perf_counter()
    plain_bad = 0
    for i in range(n):
        plain_bad += plain_parse(cj, ctx2, views[i], plain_out.array) != 0
    plain_s = time.perf_counter() - t0
    plain_ok = plain_bad == int((kinds > 0).sum())
    out = {
        "workload": f"{n} standard documents, {N} B, lognormal sizes 1 KiB-16 MiB (seed {seed:#x}), "
                    f"{int((kinds > 0).sum())} invalid (UTF-8 overlong/surrogate, unbalanced/mismatched)",
        "docs": n, "bytes": N, "structurals": int(S.sum()),
        "docs_per_s": round(n / dev_s, 1), "ms_per_batch": round(dev_s * 1e3, 3),
        "e2e_docs_per_s": round(n / e2e_s, 1), "e2e_ms_per_batch": round(e2e_s * 1e3, 3),
        "e2e_h2d_bytes": N, "e2e_d2h_bytes": total_out * 4,
        "plain_loop_docs_per_s": round(n / plain_s, 1), "plain_loop_ms": round(plain_s * 1e3, 1),
        "e2e_overlapped_docs_per_s": round(n / e2e_pad_s, 1), "e2e_overlapped_ms_per_batch": round(e2e_pad_s * 1e3, 3),
        "e2e_overlapped_h2d_bytes": ptotal, "overlapped_results_identical": same_pad,
        "speedup_e2e_vs_plain": round(plain_s / e2e_s, 2),
        "speedup_e2e_overlapped_vs_plain": round(plain_s / e2e_pad_s, 2),
        "speedup_device_vs_plain": round(plain_s / dev_s, 2),
        "verdicts_match_generator": verdicts_ok and plain_ok, "replay_results_identical": same,
        "gpu_launches_per_batch": int(launches), "graph": True,
        "tuning": dict(best.as_dict(), pair_chunk_records=512),
        "tuning_candidates": len(tried),
        "tuning_persisted_and_reloaded": all(persisted[k] == v for k, v in best.as_dict().items() if k != "ms"),
        "generation_s": round(t_gen, 1),
    }
    ctx.close()
    ctx2.close()
    pin.close()
    out_pin.close()
    plain_out.close()
    return out


SERVE_REQUESTS = 2000
SERVE_LOADS = (0.1, 0.5, 0.8, 1.0, 1.2)


def plain_parse_any(cj, ctx, doc, lines, out):
    info = cj.ParseInfo()
    return cj.lib().cj_parse_into(ctx.handle, doc.ctypes.data, doc.size, int(lines), out.ctypes.data, out.size,
                                  ctypes.byref(info))


def run_serve(args, local):
    """Serving: Poisson arrivals replayed against the continuous-batching
    server at fractions of its measured capacity, under a fixed device-memory
    budget; beside it the plain per-document loop on the same requests."""
    import cujson_gb300 as cj
    seed = synth.CONFIG_SEED_BASE + 5
    t_gen = time.perf_counter()
    docs, lines, kinds = synth.serve_requests(seed, SERVE_REQUESTS)
    t_gen = time.perf_counter() - t_gen
    # requests live in pinned memory, as a server's receive buffers would
    offs = np.concatenate([[0], np.cumsum([d.size for d in docs])])
    arena = cj.PinnedBuffer(int(offs[-1]))
    views = []
    for i, d in enumerate(docs):
        v = arena.array[int(offs[i]):int(offs[i + 1])]
        v[:] = d
        views.append(v)
    n = len(views)
    total = sum(v.size for v in views)
    budget = 16 << 30
    srv = cj.Server(device=local, slots=2, max_batch_docs=1024, memory_budget=budget)
    zero = np.zeros(n)
    srv.replay(views, lines, zero)                        # warm the arenas
    status, lat, mk = srv.replay(views, lines, zero)      # saturated: capacity
    capacity = n / mk
    ok = int((status == 0).sum())
    rng = np.random.default_rng(seed)
    sweep = []
    for load in SERVE_LOADS:
        rate = load * capacity
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
        arrivals -= arrivals[0]
        st, lat, mk = srv.replay(views, lines, arrivals)
        sweep.append({"offered_frac": load, "offered_docs_per_s": round(rate, 1),
                      "docs_per_s": round(n / mk, 1), "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
                      "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3),
                      "all_ok": bool((st == 0).all())})
    stats = srv.stats().as_dict()
    srv.close()
    # plain loop: one cj_parse_into per request
    ctx = cj.Context(local)
    ctx.reserve(max(v.size for v in views), 1)
    out = cj.PinnedBuffer((2 * max(v.size for v in views) + 4) * 4, dtype=np.int32)
    for i in range(min(n, 32)):
        plain_parse_any(cj, ctx, views[i], lines[i], out.array)
    t0 = time.perf_counter()
    for i in range(n):
        plain_parse_any(cj, ctx, views[i], lines[i], out.array)
    plain_s = time.perf_counter() - t0
    ctx.close()
    out.close()
    arena.close()
    return {
        "workload": f"{n} requests, {total} B, lognormal sizes (median 64 KiB, up to 64 MiB), "
                    f"{int((kinds == 1).sum())} JSON Lines, {int((kinds >= 2).sum())} adversarial "
                    f"(depth-10000 nesting, 32 MiB backslash string); Poisson arrivals (seed {seed:#x})",
        "slots": 2, "max_batch_docs": 1024, "memory_budget_bytes": budget,
        "capacity_docs_per_s": round(capacity, 1), "capacity_GBps": round(total / (n / capacity) / 1e9, 2),
        "requests_ok": ok, "sweep": sweep,
        "plain_loop_docs_per_s": round(n / plain_s, 1),
        "capacity_vs_plain": round(capacity / (n / plain_s), 2),
        "stats": stats, "generation_s": round(t_gen, 1),
    }


def run_other_configs(args, local, peak):
    """Device-resident parse of the other single-input configurations (config 1:
    64 MiB standard JSON; config 3: 2 GB JSON Lines in 4 chunks), the same
    kernels and the same timing as the headline line."""
    import cujson_gb300 as cj
    out = []
    for config in (1, 3):
        data, info = synth.config_input(config)
        ctx = cj.Context(local)
        if info["kind"] == "lines":
            sizes = cj.plan_lines_count(data, 4)
            ctx.stage_lines(data, sizes)
        else:
            ctx.stage_standard(data)
        for _ in range(max(3, args.warmup)):
            ctx.run()
        inf = ctx.info()
        assert inf.status == 0
        S = int(inf.n_structural)
        ctx.timing(3)
        for _ in range(args.steps):
            ctx.run()
        span = ctx.span_ms() / args.steps
        ctx.timing(2)
        for _ in range(args.steps):
            ctx.run()
        scan_ms, _, _, runs = ctx.phase_ms()
        ctx.timing(1)
        for _ in range(args.steps):
            ctx.run()
        _, _, _, fruns = ctx.phase_ms()
        tables_ms, prefix_ms, emit_ms, _ = ctx.scan_phase_ms()
        ctx.timing(False)
        N = data.size
        B = N + 8 * S
        e2e = None
        if not args.no_e2e and info["kind"] == "lines":
            # end to end through the C ABI: pinned input (one chunk; its copy
            # overlaps the scan), parse, D2H of the reference layout
            pin_in = cj.PinnedBuffer(N)
            pin_in.array[:] = data
            pin_out = cj.PinnedBuffer((2 * S + 4) * 4, dtype=np.int32)
            ctx.parse_into(pin_in.array, pin_out.array, lines=True)
            reps = []
            for _ in range(5):
                t0 = time.perf_counter()
                inf2 = ctx.parse_into(pin_in.array, pin_out.array, lines=True)
                reps.append(time.perf_counter() - t0)
                assert inf2.status == 0 and int(inf2.n_structural) == S
            dt = statistics.median(reps)
            e2e = {"GBps": round(N / dt / 1e9, 1), "ms": round(dt * 1e3, 2), "h2d_bytes": N,
                   "d2h_bytes": (2 * S + 4) * 4}
            pin_in.close()
            pin_out.close()
        out.append({
            "config": config, "workload": f"{info['kind']} {N} B (seed {synth.CONFIG_SEED_BASE + config:#x})",
            "structurals": S, "GBps": round(N / (span / 1e3) / 1e9, 1), "ms_per_parse": round(span, 4),
            "scan_ms": round(scan_ms / runs, 4), "scan_roofline_frac": round(B / (scan_ms / runs / 1e3) / 1e9 / peak, 4),
            "scan_split_ms": {"tables": round(tables_ms / fruns, 4), "prefix": round(prefix_ms / fruns, 4),
                              "emit": round(emit_ms / fruns, 4),
                              "how": "as many runs again with an event at every kernel boundary"},
            "l2": "input larger than L2" if N > (129 << 20) else "input 64 MiB < 129 MB L2 (no flush: warm-L2 figure)",
            "e2e": e2e,
            "plan": plan_timing(cj, ctx, data, local) if info["kind"] == "lines" else None,
        })
        ctx.close()
    return out


def plan_timing(cj, ctx, data, local):
    """The 4-chunk JSON-Lines plan of the input (loadJSONLines_chunkCount's
    rule): the host planner on the host copy against the device planner on a
    device copy (median of 5 each), and whether the plans agree."""
    try:
        import torch
        d = torch.from_numpy(data).to(f"cuda:{local}")
    except Exception as e:          # the device planner needs a device copy
        return {"unavailable": str(e)[:120]}

    def median_ms(fn):
        ts = []
        for _ in range(5):
            t0 = time.perf_counter()
            r = fn()
            ts.append((time.perf_counter() - t0) * 1e3)
        return r, statistics.median(ts)

    host, host_ms = median_ms(lambda: cj.plan_lines_count(data, 4))
    dev, dev_ms = median_ms(lambda: ctx.plan_lines_count_device(d.data_ptr(), int(data.size), 4))
    del d
    return {"chunks": 4, "host_ms": round(host_ms, 3), "device_ms": round(dev_ms, 3), "same": host == dev}


QUERY_SEED = 0xC0DE5004


def run_query(args, local):
    """The reference's real-world query -- count the event records whose
    "type" is "PushEvent" -- on the device over a resident JSON-Lines result,
    end to end from a pinned file (parse + query), and the reference's host
    record loop (oracle restatement, one core) on a bounded sample."""
    import cujson_gb300 as cj
    size = args.query_bytes or cj.MAX_INPUT_BYTES
    pin = cj.PinnedBuffer(size)
    t_gen = time.perf_counter()
    doc, nrec, npush = synth.synth_events(QUERY_SEED, size)
    pin.array[:] = doc
    t_gen = time.perf_counter() - t_gen
    sizes = cj.plan_lines_count(doc, 4)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    chunks = [pin.array[offs[i]:offs[i + 1]] for i in range(len(sizes))]
    ctx = cj.Context(local)
    res = ctx.parse_json_lines(chunks)
    S = res.n_structural
    del res
    key, val = b"type", b"PushEvent"
    for _ in range(args.warmup):
        n = ctx.query_count(key, val)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        n = ctx.query_count(key, val)
    q_s = (time.perf_counter() - t0) / args.steps
    for _ in range(max(1, args.warmup)):
        ctx.stage_lines(pin.array, sizes)
        ctx.run()
        ctx.query_count(key, val)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.stage_lines(pin.array, sizes)
        ctx.run()
        n2 = ctx.query_count(key, val)
    e2e_s = (time.perf_counter() - t0) / args.steps
    ctx.close()
    pin.close()
    out = {
        "workload": f"event-log JSON Lines, {size} B in 4 chunks, {nrec} records (seed {QUERY_SEED:#x}); "
                    f"count the records whose \"type\" is \"PushEvent\"",
        "records": nrec, "structurals": S, "matches": n, "matches_generator": npush,
        "correct": n == npush and n2 == npush,
        "query_ms": round(q_s * 1e3, 4), "records_per_s": round(nrec / q_s, 1),
        "input_GBps": round(size / q_s / 1e9, 2),
        "e2e_parse_plus_query_ms": round(e2e_s * 1e3, 3),
        "e2e_GBps": round(size / e2e_s / 1e9, 2),
        "generation_s": round(t_gen, 1),
    }
    if not args.no_cpu_baseline:
        from oracle import cj_oracle
        sample = min(size, args.cpu_sample)
        sdoc, srec, _ = synth.synth_events(QUERY_SEED, sample)
        ref = cj_oracle.parse(sdoc, lines=True)
        t0 = time.perf_counter()
        reps = 0
        while True:
            cj_oracle.query_lines(sdoc, ref, key, val)
            reps += 1
            if time.perf_counter() - t0 > 2.0:
                break
        cpu_s = (time.perf_counter() - t0) / reps
        out["cpu_records_per_s"] = round(srec / cpu_s, 1)
        out["cpu_sample"] = (f"{sample} B event-log sample, {srec} records, reference record loop "
                             f"(gotoArrayIndex / checkKeyValue / gotoNextSibling) restated in C, 1 core")
        out["speedup_vs_cpu_loop"] = round(out["records_per_s"] / out["cpu_records_per_s"], 1)
    return out


def run_values(args, ctx, data, S):
    """Value decoding over the staged benchmark document: every scalar slot
    decoded on the device (strings unescaped, numbers to int64 / double,
    literals), the arrays left on the device; wall time per call, which
    includes the copy-back of the type counts."""
    ctx.stage_standard(data)
    ctx.run()
    for _ in range(max(3, args.warmup)):
        counts = ctx.decode_values_counts()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        counts = ctx.decode_values_counts()
    dt = (time.perf_counter() - t0) / args.steps
    names = ["none", "string", "int", "double", "true", "false", "null", "invalid"]
    return {"workload": f"the {data.size} B benchmark document's {S + 1} slots",
            "ms": round(dt * 1e3, 4), "input_GBps": round(data.size / dt / 1e9, 1),
            "slots_per_s": round((S + 1) / dt, 1), "by_type": dict(zip(names, counts)),
            "correct": sum(counts) == S + 1 and counts[7] == 0}


def run_ours(args, world, rank, local, pg):
    import cujson_gb300 as cj
    peak, peak_kind = measured_peaks()
    data = workload(args.size)
    N = data.size
    ctx = cj.Context(local)
    ctx.reserve(N, 1)
    ctx.stage_standard(data)
    ctx.run()
    info = ctx.info()
    if info.status != 0:
        raise SystemExit(f"parse failed: {cj.status_string(info.status)}")
    S, K = int(info.n_structural), int(info.n_brackets)

    for _ in range(args.warmup):
        ctx.run()
    ctx.info()
    clocks = Clocks(local) if rank == 0 else None
    barrier(pg)
    launches0 = ctx.launches
    ctx.timing(3)                 # events at each run's start and end only
    for _ in range(args.steps):
        ctx.run()
    span_ms = ctx.span_ms()       # synchronises the stream
    barrier(pg)
    launches = ctx.launches - launches0
    ck = clocks.stop() if clocks else None
    # the scan's time, from as many runs again with an event at the scan's end too
    ctx.timing(2)
    for _ in range(args.steps):
        ctx.run()
    scan_ms, pairing_ms, _, runs = ctx.phase_ms()
    # the split into kernels, from as many runs again with an event at every
    # kernel boundary (which keeps each kernel from starting early)
    ctx.timing(1)
    for _ in range(args.steps):
        ctx.run()
    fscan_ms, pair_ms, spine_ms, fruns = ctx.phase_ms()
    tables_ms, prefix_ms, emit_ms, _ = ctx.scan_phase_ms()
    fspan_ms = ctx.span_ms()
    ctx.timing(False)
    inf2 = ctx.info()
    assert inf2.status == 0 and inf2.n_structural == S

    span_max = allmax(pg, span_ms)
    value = N * world * args.steps / (span_max / 1e3) / 1e9
    B = N + 8 * S
    scan_avg_s = scan_ms / runs / 1e3
    achieved = B / scan_avg_s / 1e9
    tr = traffic_per_byte()
    traffic = None
    if tr and "scan_bytes_per_input_byte" in tr:
        traffic = int(tr["scan_bytes_per_input_byte"] * N)

    # end to end through the C ABI: pinned host input, H2D, parse, D2H of result
    e2e = None
    if not args.no_e2e:
        pin_in = cj.PinnedBuffer(N)
        pin_in.array[:] = data
        out_n = 2 * S + 4
        pin_out = cj.PinnedBuffer(out_n * 4, dtype=np.int32)
        for _ in range(max(1, args.warmup)):
            ctx.parse_into(pin_in.array, pin_out.array)
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.parse_into(pin_in.array, pin_out.array)
        dt = allmax(pg, time.perf_counter() - t0)
        barrier(pg)
        e2e = {"value": round(N * world * args.steps / dt / 1e9, 3), "unit": UNIT,
               "h2d_bytes_per_step": N, "d2h_bytes_per_step": out_n * 4 + 64,
               "ms_per_step": round(dt / args.steps * 1e3, 3)}
        link = pinned_h2d_gbs(pin_in.array, local)
        if link:
            e2e["pinned_h2d_GBps"] = round(link, 1)
            e2e["frac_of_pinned_h2d"] = round(e2e["value"] / world / link, 3)
        pin_in.close()
        pin_out.close()

    if rank != 0:
        return
    values = None if args.no_values else run_values(args, ctx, data, S)
    batch = None if args.no_batch else run_batch(args, local)
    serve = None if args.no_serve else run_serve(args, local)
    query = None if args.no_query else run_query(args, local)
    others = None if args.no_configs else run_other_configs(args, local, peak)
    cpu, cpu_port = None, None
    if not args.no_cpu_baseline:
        v, desc = cpu_baseline_sample(args.cpu_sample)
        cpu_port = {"value": round(v, 4), "unit": UNIT, "cores": 1, "kind": "port", "sample": desc}
        sj = simdjson_baseline(data)
        if sj and sj.get("GBps", {}).get("index_all"):
            g = sj["GBps"]
            cpu = {"value": round(g["index_all"], 3), "unit": UNIT, "cores": sj["cores"], "kind": "simdjson",
                   "sample": (f"the {N} B benchmark document, simdjson 3.2.1 ondemand::parser::iterate "
                              f"(UTF-8 validation + structural index) on {sj['cores']} host threads, "
                              f"independent parsers over the same bytes"),
                   "one_core": g.get("index_1"), "dom_parse_all_cores": g.get("dom_all")}
        else:
            cpu = dict(cpu_port)
            cpu["simdjson"] = sj
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(span_max / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": workload_config(N, world),
        "workload_stats": {"structurals": S, "brackets": K, "max_depth": int(inf2.max_depth)},
        "roofline": {"bound": "hbm", "kernel": "scan (scan_tables + prefix_reduce + prefix_apply + scan_emit)",
                     "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_kind": peak_kind, "traffic": traffic,
                     "algorithmic_bytes": B},
        "phases_ms_per_step": {"how": "as many runs again with events at the scan's and the run's ends",
                               "scan": round(scan_ms / runs, 4), "pairing": round(pairing_ms / runs, 4)},
        "kernel_split_ms_per_step": {
            "how": "as many runs again with an event at every kernel boundary",
            "parse": round(fspan_ms / fruns, 4), "scan": round(fscan_ms / fruns, 4),
            "scan_tables": round(tables_ms / fruns, 4), "scan_prefix": round(prefix_ms / fruns, 4),
            "scan_emit": round(emit_ms / fruns, 4), "pair": round(pair_ms / fruns, 4),
            "spine": round(spine_ms / fruns, 4)},
        "parse_roofline_frac": round(B / (span_max / args.steps / 1e3) / 1e9 / peak, 4),
        "e2e": e2e, "cpu_baseline": cpu, "cpu_baseline_port": cpu_port, "gpu_launches": int(launches), "clocks": ck,
        "batch": batch, "serving": serve, "query": query, "values": values, "other_configs": others,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    world, rank, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
