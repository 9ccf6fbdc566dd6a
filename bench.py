#!/usr/bin/env python3
"""MC Gbases/s on one GB300 -- the long-read abundance workload.

Workload (the configuration the headline metric is quoted on): a seeded
100 Mbp random genome with twenty 5 kbp segments present 20x each; log-normal
long reads (median 8 kbp, sigma 0.8, clipped to 500 bp..100 kbp) to 40x
(4 Gbp), 5 % errors split 60/20/20 substitution/insertion/deletion; k=63
(128-bit k-mers), m=21, x=3.  Synthetic, seeded; generated on the host.

One step = one full MC count of the whole workload: pack, minimizer scan,
superkmer partition, per-bucket counting and the `> x` threshold.
* value : Gbases/s with the FASTA bytes already resident in HBM (device time,
          CUDA events on the stream the kernels run on).
* e2e   : the same through the public C ABI with host buffers: host->device
          copy of the FASTA from pinned memory, the count, and the
          device->host read of every kept record, inside the timed region.
The inputs (4 GB) are larger than L2 (126 MB), so no L2 flush is needed.
* parity: the device digest of the timed run's result against the oracle's
          digest of the same generator output (tests/golden/digests.json).
* zi / zi_serve (N = 1): the ZI halves of the metric on the same GPU -- ZI
          subtraction of a 2 Gbp query against a 60 Mbp index, batched vs one
          pipeline per file (union checked against the oracle digest), and
          the serving sweep (p50/p99 at offered loads 0.2..1.0; the request
          count per load is stated; --workload zi-serve runs 10,000).

`--impl reference` times the CPU implementation of the same path on the host
cores: the reference is Rust and cannot be built here (no cargo/rustc), so
its C restatement (oracle/) is run on a bounded sample of the workload.
N > 1 (torchrun): independent replicas, one per GPU (the path has no
collective); value = bases of all ranks / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = {"workload": "mc_abundance_long_reads_4gbp_k63", "k": 63, "m": 21, "x": 3,
            "genome_bp": 100_000_000, "read_bases": 4_000_000_000, "reads": "lognormal median 8 kbp sigma 0.8",
            "errors": "5% (3% sub, 1% ins, 1% del)", "input": "one-line FASTA",
            "l2": "inputs (4 GB) larger than L2; no flush"}
METRIC = "MC Gbases/s"
UNIT = "Gbases/s"


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(scale: float, pinned: bool):
    """FASTA bytes of the workload in (pinned) host memory: (tensor, nbytes)."""
    import numpy as np
    import torch
    from mczi_gb300 import gen
    n = gen.c2_reads_size(scale)
    buf = torch.empty(n, dtype=torch.uint8, pin_memory=pinned)
    gen.c2_reads(scale, out=(buf.data_ptr(), n))
    return buf, n


def figure_of_record_bytes(stats, k: int, text_bytes: int):
    """Algorithmic bytes per kernel by the hot path's figure of record for the
    minimizer-filtered MC path: FASTA read once (B_fasta), the 2-bit stream
    written and read (0.5 N_b), the pass-1 re-read and minimizer table
    (0.25 N_b + 24 B per superkmer), superkmer records written and read
    (2 S_skm; payload ceil((windows + k - 1) / 4) + an 8 B header each), for
    k > 32 the k-mer key round trip (2 x 16 B per window: the keys of one
    partition do not fit on chip in a CPU-style design), and the output.
    Assigned to the kernel that stands for each step: pack (FASTA, stream
    write), scan (stream read, pass-1 terms, record write), count (record read,
    key round trip, output); partition has no term of its own."""
    nb, ns, win, nout = stats[0], stats[1], stats[6], stats[5]
    rec = 24 if k > 32 else 12
    s_skm = (win + ns * (k - 1)) / 4 + 8 * ns
    keys = 2 * 16 * win if k > 32 else 0
    return {
        "pack": text_bytes + nb / 4,
        "scan": nb / 4 + nb / 4 + 24 * ns + s_skm,
        "partition": 0.0,
        "count": s_skm + keys + rec * nout,
    }


def algorithmic_bytes(stats, k: int, text_bytes: int):
    """Bytes this design's kernels must move (inputs read once, outputs
    written once), with no credit for data the design avoids moving.

    pack     : FASTA bytes + 2-bit stream (N_b/4) + fragment bits (N_b/8)
    scan     : 2-bit stream + fragment bits + descriptors (12 B each)
    partition: two passes of read + write of the 12 B descriptors
    count    : descriptors (12 B) + each superkmer's packed bases
               ((windows + k - 1) / 4 B) + kept records (24 B for k > 32);
               the k-mers themselves are generated on chip and never
               written, so no k-mer bytes are credited.
    """
    nb, ns, win, nout = stats[0], stats[1], stats[6], stats[5]
    rec = 24 if k > 32 else 12
    return {
        "pack": text_bytes + nb / 4 + nb / 8,
        "scan": nb / 4 + nb / 8 + 12 * ns,
        "partition": 2 * 24 * ns,
        "count": 12 * ns + (win + ns * (k - 1)) / 4 + rec * nout,
    }


def run_ours(args):
    import numpy as np
    import torch
    from mczi_gb300.replicas import ReplicaGroup, env
    ws, rank, local = env()
    torch.cuda.set_device(local)
    group = ReplicaGroup("nccl")  # replicas: each rank counts its own copy of the workload
    from mczi_gb300 import build
    build.build_all()
    from mczi_gb300.mc import Context, CounterConfig

    k, m, x = WORKLOAD["k"], WORKLOAD["m"], WORKLOAD["x"]
    cfg = CounterConfig(k, m, x)
    buf, nbytes = make_workload(args.scale, pinned=True)
    stream = torch.cuda.current_stream()
    ctx = Context(local)
    ctx.set_stream(stream.cuda_stream)
    inputs = [(buf.data_ptr(), nbytes)]
    # untimed: pick the counting knobs on a 25 % sample of the workload (the
    # same generator; results never depend on the knobs; smaller samples
    # favoured other table shapes than the full workload does)
    tuning_report = None
    if not args.no_tune:
        from mczi_gb300 import autotune, gen
        sample = gen.c2_reads(min(args.scale, 1.0) * 0.25)
        _, tuning_report = autotune.tune(ctx, [sample], cfg, 0, use_cache=False)

    barrier = group.barrier
    max_over_ranks = group.max_over_ranks

    # ---- device-resident value
    ctx.stage(inputs)
    for _ in range(args.warmup):
        ctx.count_staged(cfg)
    stats = ctx.run_stats()
    phase_sum = [0.0] * 5
    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        ctx.count_staged(cfg)
        for i, t in enumerate(ctx.phase_times()[:5]):
            phase_sum[i] += t
    e1.record(stream)
    barrier()
    dev_ms_plain = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    stats = ctx.run_stats()
    nb = stats[0]
    # the same steps replayed from one captured CUDA graph (the first replay
    # request captures; results are identical, see tests)
    graph_ms = None
    if not args.no_graph:
        ctx.set_graph_replay(True)
        for _ in range(args.warmup):
            ctx.count_staged(cfg)
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            ctx.count_staged(cfg)
        e1.record(stream)
        barrier()
        graph_ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
        ctx.set_graph_replay(False)
    clk = clocks.stop()
    dev_ms = graph_ms if graph_ms else dev_ms_plain
    nb_all = group.sum_over_ranks(nb)  # bases of all ranks
    value = nb_all / (dev_ms * 1e-3) / 1e9

    # ---- end to end through the C ABI: H2D from pinned + count + D2H of every
    # record into pinned host buffers (allocated once, reused every step)
    import numpy as np
    n_records = stats[5]
    pin = [torch.empty(max(1, n_records), dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
           for _ in range(3)]
    out = (pin[0], pin[1] if k > 32 else None, pin[2])
    for _ in range(max(1, args.warmup // 2)):
        ctx.count(inputs, cfg)
        ctx.records(n_records, sorted=False, out=out)
    # host-to-device staging alone, for the record (untimed)
    barrier()
    t0 = time.perf_counter()
    ctx.stage(inputs)
    barrier()
    stage_ms = (time.perf_counter() - t0) * 1e3
    barrier()
    e2e_phase = [0.0] * 4
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        n = ctx.count(inputs, cfg)
        e2e_phase = [a + b for a, b in zip(e2e_phase, ctx.phase_times()[:4])]
        rec = ctx.records(n, sorted=False, out=out)
    e1.record(stream)
    barrier()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps)
    e2e_value = nb_all / (e2e_ms * 1e-3) / 1e9
    d2h = n_records * (8 + (8 if k > 32 else 0) + 8)
    # parity of the timed run: the digest of the last end-to-end result
    # against the oracle's digest of the same generator output
    from mczi_gb300 import gen
    parity = digest_check(WORKLOAD["workload"], args.scale, [gen.fingerprint_ptr(buf.data_ptr(), nbytes)],
                          ctx.digest())

    # ---- roofline of the dominant kernel
    names = ["pack", "scan", "partition", "count"]
    avg = {nm: phase_sum[i] / args.steps for i, nm in enumerate(names)}
    dom = max(avg, key=avg.get)
    alg = figure_of_record_bytes(stats, k, nbytes)
    own = algorithmic_bytes(stats, k, nbytes)
    peak, peak_kind = load_peaks()
    achieved = alg[dom] / (avg[dom] * 1e-3) / 1e9
    achieved_own = own[dom] / (avg[dom] * 1e-3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "ncu_traffic.json"
    if tf.exists():
        t = json.loads(tf.read_text()).get(WORKLOAD["workload"], {}).get(dom)
        if t and t.get("bytes_per_base"):
            traffic = t["bytes_per_base"] * nb

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8/u64 (2-bit bases, 128-bit k-mers)",
        "data": "synthetic (seeded generator, no dataset)",
        "config": dict(WORKLOAD, parallelism=f"replicas{ws}" if ws > 1 else "single-gpu", bases=nb,
                       superkmers=stats[1], kept_records=stats[5], scale=args.scale),
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": int(nbytes),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_ms, 3),
                "staging_ms": round(stage_ms, 3), "staging_gbs": round(nbytes / (stage_ms * 1e-3) / 1e9, 1),
                # device event times of the streamed steps: [0] spans staging + pack + scan
                "phases_ms": {nm: round(v / args.steps, 3) for nm, v in
                              zip(["staging_pack_scan", "rescan", "partition", "count"], e2e_phase)}},
        "gpu_launches": int(stats[8]) * args.steps,
        "tuning": tuning_report,
        "device_ms": {"launched": round(dev_ms_plain, 3),
                      "graph_replay": round(graph_ms, 3) if graph_ms else None},
        "phases_ms": {nm: round(v, 3) for nm, v in avg.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes": int(alg[dom]), "bytes_basis": "figure of record (key round trip credited)",
                     "traffic": int(traffic) if traffic else None},
        "roofline_onchip": {"kernel": dom, "achieved": round(achieved_own, 1), "frac": round(achieved_own / peak, 4),
                            "algorithmic_bytes": int(own[dom]),
                            "bytes_basis": "this design's own movement (k-mers never leave the chip)"},
        "pipeline_roofline": {"algorithmic_bytes": int(sum(alg.values())),
                              "achieved_gbs": round(sum(alg.values()) / (dev_ms * 1e-3) / 1e9, 1),
                              "frac": round(sum(alg.values()) / (dev_ms * 1e-3) / 1e9 / peak, 4),
                              "onchip_frac": round(sum(own.values()) / (dev_ms * 1e-3) / 1e9 / peak, 4)},
        "clocks": clk,
    }
    line["parity"] = parity
    ctx.close()
    del buf, pin, out, rec
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    if ws == 1 and not args.no_zi:
        # the ZI halves of the metric on the same GPU: batched vs plain
        # subtraction at full size (its union checked against the oracle
        # digest) and the serving sweep
        line["zi"] = zi_measure(args.scale, args.zi_files, args.line_zi_steps, 1)
        line["zi_serve"] = zi_serve_measure(args.scale, args.line_serve_requests, args.serve_workers,
                                            args.serve_max_bytes, args.serve_pool_bases)
    if ws == 1 and args.gzip_scale > 0:
        line["gzip"] = gzip_measure(args.gzip_scale, 3)
    if rank == 0:
        print(json.dumps(line), flush=True)
    group.close()


def gzip_measure(scale: float, reps: int) -> dict:
    """The same long reads as BGZF (gzip members that carry their sizes,
    compressed on the host's threads, untimed): the device decode rate
    (mczi_inflate_gzip, kernel time from CUDA events, bytes checked against
    the text), and the count through the C ABI with the input compressed (its
    compressed bytes cross the host link and are decoded in HBM) against the
    same count of the text, both from pinned host memory, digests compared."""
    import numpy as np
    import torch
    from mczi_gb300 import bgzf, gen
    from mczi_gb300.mc import Context, CounterConfig
    n = gen.c2_reads_size(scale)
    text = np.empty(n, dtype=np.uint8)
    gen.c2_reads(scale, out=(text.ctypes.data, n))
    t0 = time.perf_counter()
    gz = bgzf.compress(text, level=6)
    compress_s = time.perf_counter() - t0
    pin_gz = torch.empty(len(gz), dtype=torch.uint8, pin_memory=True)
    pin_gz.numpy()[:] = np.frombuffer(gz, dtype=np.uint8)
    pin_tx = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    pin_tx.numpy()[:] = text
    ctx = Context(0)
    ms = []
    for _ in range(reps):
        out = ctx.inflate_gzip(gz)
        ms.append(ctx.phase_times()[5])
    same = out == text.tobytes()
    del out
    dec_ms = float(np.median(ms))
    cfg = CounterConfig(63, 21, 3)
    res = {}
    for name, buf in (("bgzf", pin_gz), ("text", pin_tx)):
        ctx.count([(buf.data_ptr(), buf.numel())], cfg)  # warm-up
        ts = []
        for _ in range(reps):
            t = time.perf_counter()
            r = ctx.count([(buf.data_ptr(), buf.numel())], cfg)
            ts.append(time.perf_counter() - t)
        res[name] = {"s": round(float(np.median(ts)), 4), "gbases_per_s": round(n / float(np.median(ts)) / 1e9, 3),
                     "h2d_bytes": int(buf.numel()), "records": r, "digest": ctx.digest()}
    ctx.close()
    return {
        "workload": "mc_abundance_long_reads_bgzf_k63", "scale": scale, "text_bytes": int(n),
        "bgzf_bytes": len(gz), "members": (n + bgzf.BLOCK - 1) // bgzf.BLOCK + 1, "level": 6,
        "host_compress_s": round(compress_s, 2),
        "decode": {"kernel_ms": round(dec_ms, 3), "decoded_gb_per_s": round(n / (dec_ms * 1e-3) / 1e9, 2),
                   "bytes_match": bool(same),
                   "bound": "serial Huffman decode, one warp per member (decode rate, not HBM)"},
        "count_e2e": res, "digest_match": res["bgzf"]["digest"] == res["text"]["digest"],
    }


def digest_check(name: str, scale: float, fingerprints, got: dict) -> dict:
    """Compares a GPU result digest with the oracle's digest of the same
    input, committed in tests/golden/digests.json by
    tests/golden/make_digests.py (full-size inputs only)."""
    p = ROOT / "tests" / "golden" / "digests.json"
    entry = json.loads(p.read_text()).get(name) if p.exists() else None
    if not entry or entry["scale"] != scale:
        return {"digest_match": None, "scale": scale, "records": got["records"],
                "reason": "no committed oracle digest at this scale"}
    same_input = list(fingerprints) == entry["input_fingerprints"]
    return {"digest_match": bool(same_input and got == entry["digest"]), "input_match": same_input,
            "scale": scale, "records": got["records"], "digest": got,
            "oracle": "digest of the oracle's exact result for the same generator output, committed with the script "
                      "that made it (tests/golden/digests.json)"}


def cpu_baseline(args, sample_scale: float | None = None, data=None):
    """The C restatement (oracle/, OpenMP over all host cores) on a bounded
    sample of the same workload: the same generator at a smaller scale."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_ref
    from mczi_gb300 import gen
    from mczi_gb300._native import default_threads
    scale = sample_scale if sample_scale is not None else args.cpu_sample_scale
    if data is None:
        data = gen.c2_reads(scale)
    threads = default_threads()
    t0 = time.perf_counter()
    lo, hi, cnt = oracle_ref.count([data], WORKLOAD["k"], WORKLOAD["x"], 0, threads)
    dt = time.perf_counter() - t0
    bases = int(WORKLOAD["read_bases"] * scale)
    return {"value": round(bases / dt / 1e9, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"same generator at scale {scale} ({bases / 1e6:.0f} Mbp of the 4 Gbp workload), "
                      f"{dt:.1f} s wall, {lo.size} kept k-mers"}


def run_reference(args):
    from mczi_gb300.replicas import env
    ws, rank, _ = env()
    if rank != 0:
        return
    from mczi_gb300 import gen
    scale = args.ref_sample_scale
    data = gen.c2_reads(scale)  # one sample, counted afresh every step
    steps = []
    cb = None
    for _ in range(min(args.warmup, 1)):  # page-in; the port keeps no state between steps
        cpu_baseline(args, scale, data)
    for _ in range(args.steps):
        cb = cpu_baseline(args, scale, data)
        steps.append(cb["value"])
    value = statistics.median(steps)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "impl": "reference", "dtype": "u8/u128", "data": "synthetic (seeded generator, no dataset)",
            "config": dict(WORKLOAD, parallelism="cpu", scale=scale, bases=int(WORKLOAD["read_bases"] * scale),
                           warmup_steps_run=min(args.warmup, 1)),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cb["cores"], "kind": "port",
                             "sample": cb["sample"] + "; the Rust reference cannot be built here (no cargo/rustc)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_mc_short(args):
    """MC abundance on short reads: 1.0 M x 150 bp reads (30x of a seeded 5 Mbp
    genome, 0.5 % substitutions), k=31 m=21 x=5, KFF output as the config asks.
    Device-resident (staged once, counts timed with CUDA events) and end to end
    (each step copies the pinned FASTA in, counts, and writes the KFF file)."""
    import tempfile
    import torch
    from mczi_gb300 import build, gen
    from mczi_gb300.mc import Context, CounterConfig
    build.build_all()
    data = gen.c1_reads(args.scale)
    pinned = torch.empty(data.size, dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = data
    inputs = [(pinned.data_ptr(), data.size)]
    cfg = CounterConfig(31, 21, 5)
    ctx = Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.stage(inputs)
    for _ in range(args.warmup):
        ctx.count_staged(cfg)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    phases = [0.0] * 4
    clocks = ClockSampler(0)
    clocks.start()
    e0.record(stream)
    for _ in range(args.steps):
        ctx.count_staged(cfg)
        phases = [a + b for a, b in zip(phases, ctx.phase_times()[:4])]
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    dev_ms = e0.elapsed_time(e1) / args.steps
    st = ctx.run_stats()
    nb = st[0]
    with tempfile.TemporaryDirectory() as tmp:
        out = f"{tmp}/c1.kff"
        for _ in range(max(1, args.warmup // 2)):
            ctx.count(inputs, cfg)
            ctx.write_kff(out)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.count(inputs, cfg)
            ctx.write_kff(out)
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
        kff_bytes = os.path.getsize(out)
    line = {"metric": METRIC, "value": round(nb / (dev_ms * 1e-3) / 1e9, 3), "unit": UNIT, "impl": "ours",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u64 (2-bit bases, 64-bit k-mers)",
            "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": "mc_abundance_short_reads_150mbp_k31", "k": 31, "m": 21, "x": 5, "bases": nb,
                       "superkmers": st[1], "kept_records": st[5], "output": "KFF, u8 counts", "scale": args.scale},
            "phases_ms": dict(zip(["pack", "scan", "partition", "count"], [round(x / args.steps, 3) for x in phases])),
            "e2e": {"value": round(nb / (e2e_ms * 1e-3) / 1e9, 3), "unit": UNIT, "ms_per_step": round(e2e_ms, 3),
                    "h2d_bytes_per_step": int(data.size), "kff_bytes_written_per_step": int(kff_bytes),
                    "d2h_bytes_per_step": int(st[5] * 16), "host_memory": "pinned input"},
            "clocks": clk}
    ctx.close()
    print(json.dumps(line), flush=True)


def run_mc_fof(args):
    """MC fof dataset presence: 64 datasets drawn from one seeded 20 Mbp genome
    (0.1 % private SNPs each, 150 bp reads at coverage uniform in [5x, 30x],
    0.5 % errors), k=31 m=21 x=5 (kept if present in > 5 datasets); all
    datasets in one set of launches, in key-range passes when the superkmers
    exceed one pass's buffers.  Inputs sit in one pinned host buffer."""
    import torch
    from mczi_gb300 import build, gen
    from mczi_gb300.mc import Context, CounterConfig
    build.build_all()
    t0 = time.perf_counter()
    ds = gen.c3_datasets(64, genome_len=int(20_000_000 * args.scale))
    gen_s = time.perf_counter() - t0
    nbytes = int(sum(d.size for d in ds))
    # the datasets in one pinned host buffer (as a loader would deliver them)
    pinned = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    view, o, inputs = pinned.numpy(), 0, []
    for d in ds:
        view[o:o + d.size] = d
        inputs.append((pinned.data_ptr() + o, int(d.size)))
        o += d.size
    del ds
    cfg = CounterConfig(31, 21, 5)
    stream = torch.cuda.current_stream()
    ctx = Context(0)
    ctx.set_stream(stream.cuda_stream)
    ctx.stage(inputs)
    for _ in range(args.warmup):
        n = ctx.count_staged(cfg, 1)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    phase_sum = [0.0] * 5
    e0.record(stream)
    for _ in range(args.steps):
        n = ctx.count_staged(cfg, 1)
        phase_sum = [a + b for a, b in zip(phase_sum, ctx.phase_times())]
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    dev_ms = e0.elapsed_time(e1) / args.steps
    stats = ctx.run_stats()
    nb = stats[0]
    # end to end: staging from pinned host memory + count + records into
    # pinned buffers
    import numpy as np
    outs = [torch.empty(max(1, n), dtype=torch.int64, pin_memory=True).numpy().view(np.uint64) for _ in range(2)]
    ctx.count(inputs, cfg, 1)
    ctx.records(n, sorted=False, out=(outs[0], None, outs[1]))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        n2 = ctx.count(inputs, cfg, 1)
        rec = ctx.records(n2, sorted=False, out=(outs[0], None, outs[1]))
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    assert n2 == n
    line = {"metric": "MC Gbases/s", "value": round(nb / (dev_ms * 1e-3) / 1e9, 3), "unit": "Gbases/s",
            "impl": "ours", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dev_ms, 3), "higher_is_better": True, "scaling": "weak",
            "dtype": "u8/u64 (2-bit bases, 64-bit k-mers, 64-bit dataset masks)",
            "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": "mc_fof_64_datasets_k31", "k": 31, "m": 21, "x": 5, "mode": "presence",
                       "datasets": 64, "genome_bp": int(20_000_000 * args.scale), "bases": nb,
                       "text_bytes": nbytes, "superkmers": stats[1], "kept_records": n,
                       "launches": stats[8], "generate_s": round(gen_s, 1)},
            "phases_ms": {nm: round(v / args.steps, 3) for nm, v in
                          zip(["pack", "scan", "partition", "count", "precount"], phase_sum)},
            "e2e": {"value": round(nb / (e2e_ms * 1e-3) / 1e9, 3), "unit": "Gbases/s", "ms_per_step": round(e2e_ms, 3),
                    "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": int(n) * 16,
                    "host_memory": "pinned"},
            "clocks": clk}
    ctx.close()
    print(json.dumps(line), flush=True)


def _record_starts(buf) -> "np.ndarray":
    import numpy as np
    return np.flatnonzero(buf == ord(">"))


def zi_measure(scale: float, nfiles: int, steps: int, warmup: int, one_group: bool = False) -> dict:
    """ZI subtraction, batched vs plain: the index is the k-mer set of a 60 Mbp
    random genome (as overlapping chunks, the same set as MC's k=31 x=1 FASTA of
    that genome fed twice); the query is 2 Gbp of 150 bp reads, half from that
    genome and half from an independent one, 1 % errors, split into files.
    Batched = all files in groups of <= 64, one set of launches per group with
    a result per file; plain = one pipeline per file (its own launches and
    syncs).  The union query (the reference's one absent set over all files)
    is checked against the oracle digest committed for the full-size input."""
    import numpy as np
    import torch
    from mczi_gb300 import build, gen, zi
    from mczi_gb300.mc import Context
    build.build_all()
    k, m = 31, 19
    glen = int(60_000_000 * scale)
    qbases = int(2_000_000_000 * scale)
    t0 = time.perf_counter()
    index, query = gen.c4_index_and_query(genome_len=glen, query_bases=qbases, k=k)
    gen_s = time.perf_counter() - t0
    fps = [gen.fingerprint(index), gen.fingerprint(query)]
    # the query sits in pinned host memory, as a server's receive buffers would
    pinned = torch.empty(query.size, dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = query
    del query
    query = pinned.numpy()
    starts = _record_starts(query)
    cuts = [int(starts[int(i * len(starts) / nfiles)]) for i in range(nfiles)] + [query.size]
    files = [query[cuts[i]:cuts[i + 1]] for i in range(nfiles)]
    windows = int(qbases / 150) * (150 - k + 1)
    ctx = Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    zi.build_dictionary(index, k, m, ctx=ctx)
    info = zi.info(ctx)
    if one_group:
        # for kernel profiles: one 50-file group (every 4th file: half in-index
        # reads, half foreign, like the whole query) per input, then as a union
        group = files[::4][:50]
        out = []
        for name, run in (("per_input", zi.query_per_input), ("union", zi.query)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            n = run(ctx, group)
            torch.cuda.synchronize()
            out.append({"query": name, "files": len(group), "records": n,
                        "ms": round((time.perf_counter() - t0) * 1e3, 3),
                        "phases_ms": [round(x, 3) for x in ctx.phase_times()[:5]], "stats": ctx.run_stats()[:8]})
        ctx.close()
        return {"one_group": out}
    ngroups = -(-nfiles // 64)
    groups = [files[i * nfiles // ngroups:(i + 1) * nfiles // ngroups] for i in range(ngroups)]
    for _ in range(warmup):
        for g in groups:
            zi.query_per_input(ctx, g)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    phases = [0.0] * 5
    qsk = qbases_packed = n_rec = 0
    for _ in range(steps):
        n_rec = 0
        qsk = qbases_packed = 0
        for g in groups:
            n_rec += zi.query_per_input(ctx, g)
            phases = [a + b for a, b in zip(phases, ctx.phase_times())]
            st = ctx.run_stats()
            qbases_packed += st[0]
            qsk += st[2]
    torch.cuda.synchronize()
    batched_s = (time.perf_counter() - t0) / steps
    phases = [x / steps for x in phases]
    # per-file result lists of the last group, split on the device
    t0 = time.perf_counter()
    split = zi.batch_results(ctx, len(groups[-1]))
    split_s = time.perf_counter() - t0
    # plain: one pipeline per file, a result per file
    lat = []
    sizes = []
    t0 = time.perf_counter()
    for f in files:
        t1 = time.perf_counter()
        sizes.append(zi.query(ctx, [f]))
        lat.append(time.perf_counter() - t1)
    plain_s = time.perf_counter() - t0
    # the reference's union semantics (one absent set over all files), with
    # its digest against the oracle's
    t0 = time.perf_counter()
    n_absent = zi.query(ctx, files)
    union_s = time.perf_counter() - t0
    union_digest = ctx.digest(unit_counts=True)
    parity = digest_check("zi_subtract_2gbp_k31", scale, fps, union_digest)
    # spot-check: per-file results of the batch equal the per-file runs
    zi.query_per_input(ctx, files[:4])
    chk = zi.batch_results(ctx, 4)
    for i in range(4):
        assert len(chk[i]) == sizes[i], (i, len(chk[i]), sizes[i])
    ctx.close()
    from mczi_gb300.serve import percentile
    alg = query.size + qbases_packed / 2 + 96 * qsk + 16 * n_rec
    return {
        "metric": "ZI queries/s", "value": round(windows / batched_s, 1), "unit": "k-mer lookups/s",
        "steps": steps, "warmup": warmup,
        "config": {"workload": "zi_subtract_2gbp_k31", "k": k, "m": m, "index_genome_bp": glen,
                   "index_kmers": info["index_bases"], "query_bases": qbases, "query_files": nfiles,
                   "mphf_levels": info["mphf_levels"], "minimizers": info["minimizers"],
                   "index_build_ms": info["build_us"] / 1000.0, "records_batched": n_rec, "scale": scale,
                   "generate_s": round(gen_s, 1)},
        "batched": {"s": round(batched_s, 4), "lookups_per_s": round(windows / batched_s, 1),
                    "groups": ngroups, "split_last_group_ms": round(split_s * 1e3, 3),
                    "split_last_group_kmers": int(sum(len(x) for x in split)),
                    "phases_ms": dict(zip(["pack", "scan", "partition", "dedup_count", "probe"],
                                          [round(x, 3) for x in phases]))},
        "plain": {"s": round(plain_s, 4), "lookups_per_s": round(windows / plain_s, 1),
                  "file_p50_ms": round(percentile(lat, 50) * 1e3, 3),
                  "file_p99_ms": round(percentile(lat, 99) * 1e3, 3)},
        "batched_over_plain": round(plain_s / batched_s, 2),
        # for information (figure of record: FASTA once, 2-bit stream written and
        # read, 96 B per query superkmer for MPHF / offsets / strings, records out)
        "roofline": {"bound": "hbm", "kernel": "whole batched query", "unit": "GB/s", "algorithmic_bytes": int(alg),
                     "achieved": round(alg / batched_s / 1e9, 1), "peak": load_peaks()[0],
                     "frac": round(alg / batched_s / 1e9 / load_peaks()[0], 4)},
        "union": {"s": round(union_s, 4), "lookups_per_s": round(windows / union_s, 1), "absent_kmers": n_absent,
                  "digest": union_digest},
        "parity": parity,
    }


def run_zi(args):
    r = zi_measure(args.scale, args.zi_files, args.steps, args.warmup, args.zi_one_group)
    if "one_group" in r:
        for x in r["one_group"]:
            print(json.dumps(x), flush=True)
        return
    line = dict(r, impl="ours", n_gpus=1, higher_is_better=True, data="synthetic (seeded generator, no dataset)")
    print(json.dumps(line), flush=True)


def zi_serve_measure(scale: float, requests: int, workers: int, max_bytes: float, pool_bases: float,
                     loads=(0.2, 0.4, 0.6, 0.8, 1.0)) -> dict:
    """ZI serving through the library's native loop (mczi_serve_*): the index
    stays resident; requests of log-uniform size (10 kbp .. max_bytes, sliced
    without copying from a pool of reads) arrive as a Poisson process at
    offered loads of the measured batched peak; p50/p99 latency (submit to
    result, timed by the native server) and aggregate bases/s.  Each answered
    request's absent set is copied to the host and then dropped, so a sweep of
    10,000 requests per load holds only the requests in flight."""
    import numpy as np
    from mczi_gb300 import build, gen, zi
    from mczi_gb300.mc import Context
    from mczi_gb300.serve import ZIServer, percentile
    build.build_all()
    k, m = 31, 19
    glen = int(60_000_000 * scale)
    index, pool = gen.c4_index_and_query(genome_len=glen, query_bases=int(pool_bases), k=k)
    starts = _record_starts(pool)
    rng = np.random.default_rng(5)
    lo_b, hi_b = 10_000, int(max_bytes)

    def make_request():
        size = int(np.exp(rng.uniform(np.log(lo_b), np.log(hi_b))))
        i0 = int(rng.integers(0, max(1, len(starts) - 2)))
        a = int(starts[i0])
        j = int(np.searchsorted(starts, a + size))
        b = int(starts[j]) if j < len(starts) else pool.size
        return pool[a:b]  # a view: the server reads the pool's bytes in place

    # for information: one batch of 64 requests in one call (device work only)
    ctx = Context(0)
    zi.build_dictionary(index, k, m, ctx=ctx)
    probe = [make_request() for _ in range(64)]
    zi.query_per_input(ctx, probe)
    t0 = time.perf_counter()
    zi.query_per_input(ctx, probe)
    batch_bps = sum(len(p) for p in probe) / (time.perf_counter() - t0)
    ctx.close()
    points = []
    with ZIServer(index, k, m, workers=workers, max_batch=64, keep_results=False) as srv:
        # measured peak: the server's own throughput on a burst of requests
        # submitted at once -- bytes / the latest native completion (submit to
        # absent set in host memory) -- after one warm-up burst
        def burst(reqs):
            futs = [srv.submit(r) for r in reqs]
            for f in futs:
                f.result()
            return sum(len(r) for r in reqs) / (max(f.latency_ms for f in futs) * 1e-3)
        burst([make_request() for _ in range(128)])  # warm-up: also fills the pinned result pool
        peak_bps = burst([make_request() for _ in range(128)])
        for load in loads:
            st0 = srv.stats()
            reqs = [make_request() for _ in range(requests)]
            mean = sum(len(r) for r in reqs) / len(reqs)
            rate = load * peak_bps / mean
            arr = np.cumsum(rng.exponential(1.0 / rate, size=len(reqs)))
            lat, queue = [], []
            done = threading.Semaphore(0)

            def finished(f):
                lat.append(f.latency_ms)
                queue.append(f.queue_ms)
                done.release()  # the future (and its absent set) is dropped after this

            t_start = time.perf_counter()
            for r, at in zip(reqs, arr):
                d = t_start + at - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                srv.submit(r).add_done_callback(finished)
            for _ in reqs:
                done.acquire()
            t_end = time.perf_counter()
            st1 = srv.stats()
            nb = st1["batches"] - st0["batches"]
            points.append({"offered_load": load, "requests": len(reqs), "p50_ms": round(percentile(lat, 50), 3),
                           "p99_ms": round(percentile(lat, 99), 3), "queue_p99_ms": round(percentile(queue, 99), 3),
                           "throughput_bases_per_s": round(sum(len(r) for r in reqs) / (t_end - t_start), 1),
                           "mean_request_bytes": round(mean), "wall_s": round(t_end - t_start, 2),
                           "mean_batch": round((st1["requests"] - st0["requests"]) / max(1, nb), 2),
                           "batches": int(nb), "query_s": round(st1["query_s"] - st0["query_s"], 3),
                           "results_s": round(st1["results_s"] - st0["results_s"], 3)})
    return {"metric": "ZI-serve p99 ms", "value": points[-1]["p99_ms"], "unit": "ms", "higher_is_better": False,
            "config": {"workload": "zi_serve_k31", "index_genome_bp": glen, "workers": workers,
                       "request_bytes": [lo_b, hi_b], "requests_per_load": requests,
                       "peak_bytes_per_s": round(peak_bps, 1),
                       "peak": "server throughput on a burst of 128 requests submitted at once (native completion times)",
                       "one_batch_device_bytes_per_s": round(batch_bps, 1), "arrivals": "Poisson"},
            "sweep": points}


def run_zi_serve(args):
    r = zi_serve_measure(args.scale, args.serve_requests, args.serve_workers, args.serve_max_bytes,
                         args.serve_pool_bases)
    print(json.dumps(dict(r, impl="ours", n_gpus=1, data="synthetic (seeded generator, no dataset)")), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="workload scale (1.0 = 4 Gbp)")
    ap.add_argument("--cpu-sample-scale", type=float, default=0.05)
    ap.add_argument("--ref-sample-scale", type=float, default=0.05)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the untimed autotuning on a sample")
    ap.add_argument("--no-graph", action="store_true", help="skip the graph-replay timing")
    ap.add_argument("--workload", default="mc", choices=["mc", "mc-short", "mc-fof", "zi", "zi-serve", "gzip"])
    ap.add_argument("--zi-files", type=int, default=200)
    ap.add_argument("--zi-one-group", action="store_true",
                    help="run one 50-file group (per input, then union) and exit: the case for ZI kernel profiles")
    ap.add_argument("--serve-requests", type=int, default=10_000,
                    help="requests per offered load of --workload zi-serve (the default MC line runs "
                         "--line-serve-requests)")
    ap.add_argument("--line-serve-requests", type=int, default=500)
    ap.add_argument("--line-zi-steps", type=int, default=3)
    ap.add_argument("--no-zi", action="store_true", help="MC only: skip the ZI keys of the default line")
    ap.add_argument("--gzip-scale", type=float, default=0.25,
                    help="scale of the long reads for the default line's gzip key (BGZF decoded on the device); "
                         "0 skips it")
    ap.add_argument("--serve-workers", type=int, default=2)
    ap.add_argument("--serve-max-bytes", type=float, default=200e6)
    ap.add_argument("--serve-pool-bases", type=float, default=600e6)
    args = ap.parse_args()
    if args.workload == "zi" and args.impl == "ours":
        return run_zi(args)
    if args.workload == "zi-serve" and args.impl == "ours":
        return run_zi_serve(args)
    if args.workload == "mc-fof" and args.impl == "ours":
        return run_mc_fof(args)
    if args.workload == "mc-short" and args.impl == "ours":
        return run_mc_short(args)
    if args.workload == "gzip" and args.impl == "ours":
        # the default line's gzip key alone (BGZF long reads decoded on the device)
        print(json.dumps(gzip_measure(args.gzip_scale if args.gzip_scale > 0 else 0.25, 3)), flush=True)
        return 0
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
