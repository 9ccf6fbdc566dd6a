#!/usr/bin/env python3
"""Writes tests/golden/digests.json: oracle digests of the benchmark
workloads at their full sizes.

For each workload the seeded generator (mczi_gb300.gen) makes the input, its
fingerprint is recorded, and the CPU oracle (oracle/, the parity checker)
computes the order-independent digest (mczi_gb300.digest's definition) of
the records the path must keep -- exact canonical k-mer counts with count > x
for MC, the absent canonical k-mer set for ZI -- in hash-range passes so that
memory stays bounded.  bench.py compares the GPU result of the same input
with these digests; the tests check the digest machinery on small cases.

    python tests/golden/make_digests.py [--only NAME ...] [--threads N]

Takes minutes per workload on a few host cores (4 Gbp at k = 63 is the
largest).  Test infrastructure only.
"""
from __future__ import annotations

import argparse
import json
import platform
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

OUT = HERE / "digests.json"


def mc_long_reads():
    from mczi_gb300 import gen
    return {"name": "mc_abundance_long_reads_4gbp_k63", "scale": 1.0, "k": 63, "x": 3, "mode": 0, "passes": 32,
            "inputs": [gen.c2_reads(1.0)]}


def mc_short_reads(x):
    from mczi_gb300 import gen
    return {"name": f"mc_abundance_short_reads_150mbp_k31_x{x}", "scale": 1.0, "k": 31, "x": x, "mode": 0,
            "passes": 2, "inputs": [gen.c1_reads(1.0)]}


def zi_subtract():
    from mczi_gb300 import gen
    index, query = gen.c4_index_and_query(genome_len=60_000_000, query_bases=2_000_000_000, k=31)
    return {"name": "zi_subtract_2gbp_k31", "scale": 1.0, "k": 31, "passes": 16, "index": index,
            "inputs": [query]}


BUILDERS = {
    "mc_abundance_long_reads_4gbp_k63": mc_long_reads,
    "mc_abundance_short_reads_150mbp_k31_x5": lambda: mc_short_reads(5),
    "mc_abundance_short_reads_150mbp_k31_x0": lambda: mc_short_reads(0),
    "zi_subtract_2gbp_k31": zi_subtract,
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*", default=None)
    ap.add_argument("--threads", type=int, default=None)
    args = ap.parse_args()
    import oracle_ref
    from mczi_gb300 import gen
    data = json.loads(OUT.read_text()) if OUT.exists() else {}
    for name, make in BUILDERS.items():
        if args.only and name not in args.only:
            continue
        t0 = time.perf_counter()
        w = make()
        gen_s = time.perf_counter() - t0
        fps = [gen.fingerprint(b) for b in w["inputs"]]
        t0 = time.perf_counter()
        if "index" in w:
            d = oracle_ref.zi_absent_digest(w["index"], w["inputs"], w["k"], args.threads, w["passes"])
            fps = [gen.fingerprint(w["index"])] + fps
        else:
            d = oracle_ref.count_digest(w["inputs"], w["k"], w["x"], w["mode"], args.threads, w["passes"])
        dt = time.perf_counter() - t0
        entry = {k: v for k, v in w.items() if k not in ("inputs", "index")}
        entry.update({"input_fingerprints": fps, "input_bytes": [int(b.size) for b in w["inputs"]],
                      "digest": d, "oracle_s": round(dt, 1), "generate_s": round(gen_s, 1),
                      "host": platform.machine()})
        data[name] = entry
        OUT.write_text(json.dumps(data, indent=1, sort_keys=True) + "\n")
        print(name, json.dumps(entry), flush=True)
        del w


if __name__ == "__main__":
    main()
