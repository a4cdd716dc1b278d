"""Fixed device-resident workload for profiler captures: uploads one batch of
seeded uniform 4096x4096 chunk pairs (FFT 8192) and runs it a few times.

    python -m satsuma2_gb300.profile_case [--pairs 4096] [--runs 3]

Each run launches the correlation kernel, the scan kernel and two finalize
kernels once; nothing else touches the GPU, so profiler launch lists map
one-to-one onto runs.
"""
import argparse
import ctypes

import satsuma2_gb300 as sg
from satsuma2_gb300 import build, workloads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=4096)
    ap.add_argument("--runs", type=int, default=3)
    ap.add_argument("--seed", type=int, default=42)
    a = ap.parse_args()
    build.build()
    items = workloads.uniform_batch(a.pairs, seed=a.seed)
    x = sg.XCorr(target_total=4096.0 * 4096)
    b = x.upload(items)
    for _ in range(a.runs):
        b.run(ctypes.c_void_p(0))
    res = b.results()
    print("pairs %d runs %d results %d" % (a.pairs, a.runs, len(res)))
    b.free()
    x.close()


if __name__ == "__main__":
    main()
