"""Times the reference's own compiled sequential Dijkstra against the oracle restatement that
the benchmark's CPU baseline runs, on the same updated graph, one core each.

Test infrastructure.  Needs `oracle/_ref/ref_time`, which `make -C oracle ref` compiles from
the reference's sources (seqSSSPwithDist_undir.cpp) where they lie; on a machine without them
the benchmark's CPU baseline is the restatement alone.

    python oracle/time_ref.py [--workload rmat22|er10k|grid4096] [--reps 3]

Builds the workload's graph and batch as bench.py does, applies the batch with the reference's
semantics (the oracle's updated graph), writes the surviving edge lines as the reference's
graph text format, and runs both Dijkstras from the workload's source.  The reference's read
is not timed; its print loop (inside its djk) is.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="rmat22")
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    exe = HERE / "_ref" / "ref_time"
    if not exe.exists():
        print(f"{exe} is missing: make -C oracle ref (needs the reference's sources)", file=sys.stderr)
        return 2

    import bench
    from oracle import pyoracle as O

    n, u, v, w, src, ch = bench.make_inputs(args.workload)
    g, kept = O.updated_graph(n, u, v, w, ch, return_kept=True)
    ins = ch[ch["op"] == 1]
    m = len(u)
    lines_u = np.concatenate([u[kept[:m] == 1], ins["u"][kept[m:m + len(ins)] == 1]])
    lines_v = np.concatenate([v[kept[:m] == 1], ins["v"][kept[m:m + len(ins)] == 1]])
    lines_w = np.concatenate([w[kept[:m] == 1], ins["w"][kept[m:m + len(ins)] == 1]])

    port = []
    for _ in range(args.reps):
        t0 = time.perf_counter()
        O.dijkstra(n, g, src)
        port.append(time.perf_counter() - t0)

    ref = []
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "graph.txt")
        with open(path, "w") as f:
            step = 1 << 22
            for a in range(0, len(lines_u), step):
                b = a + step
                block = np.stack([lines_u[a:b], lines_v[a:b], lines_w[a:b]], axis=1)
                f.write("\n".join(f"{x} {y} {z}" for x, y, z in block.tolist()))
                f.write("\n")
        for _ in range(args.reps):
            out = subprocess.run([str(exe), path, str(n), str(src)], capture_output=True, text=True, check=True)
            ref.append(float(out.stdout.split()[0]))

    print(f"{args.workload}: n {n}, {len(lines_u)} edge lines after the batch, source {src}")
    print(f"  reference djk (compiled, -O3):  median {np.median(ref):.3f} s  {sorted(round(t, 3) for t in ref)}")
    print(f"  oracle restatement (C, -O2):    median {np.median(port):.3f} s  {sorted(round(t, 3) for t in port)}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
