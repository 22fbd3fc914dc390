"""Calibrates the timed CPU baseline (TEST INFRASTRUCTURE ONLY).

The benchmark's CPU baseline runs the oracle's C restatement (libvpo.so),
because the reference's own sources are not present on the machine that
runs the benchmark. This script times both on this machine, on the same
chunk sample of the benchmark world, with the same thread count and the
same compiler flags (-O2, OpenMP over chunks, cold decode), checks that they
produce the same output bytes, and writes their speed ratio to
oracle/port_vs_reference.json, which the benchmark reports beside its
baseline.

  python oracle/calibrate.py [--threads N] [--chunks N] [--reps N]
"""
import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def main():
    import bench
    from oracle import bindings as ob
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--chunks", type=int, default=1024)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    if ob.ref_lib() is None:
        sys.exit("the reference tree is not present: nothing to calibrate against")
    world = bench.make_world()
    modes = bench.mesh_modes(world)
    order = np.random.default_rng(1).permutation(world.nchunks).astype(np.uint32)[:a.chunks]
    port, ref = ob.OracleWorld(world), ob.RefWorld(world)
    times = {"port": [], "reference": []}
    out = {}
    for _ in range(a.reps):
        for name, w in (("port", port), ("reference", ref)):
            t0 = time.perf_counter()
            out[name] = w.rebuild(order, modes, bench.LOD_MAX, a.threads)
            times[name].append(time.perf_counter() - t0)
    if out["port"] != out["reference"]:
        sys.exit("port and reference produced different output sizes: %s" % out)
    rate = {k: len(order) / float(np.median(v)) for k, v in times.items()}
    res = {
        "port_vs_reference": round(rate["port"] / rate["reference"], 4),
        "port_chunks_per_s": round(rate["port"], 1),
        "reference_chunks_per_s": round(rate["reference"], 1),
        "threads": a.threads,
        "cpu": cpu_model(),
        "machine": platform.machine(),
        "sample": "%d of the %d chunks of the 2048x256x2048 benchmark world (random, seed 1), cold decode, "
                  "LOD 0..%d, %d meshed" % (len(order), world.nchunks, bench.LOD_MAX, int(modes[order].sum())),
        "flags": "gcc -O2 -fopenmp for both (the reference's -march=native is left out: this code is built for "
                 "x86-64 and Arm alike)",
        "reps": a.reps,
        "output_bytes": int(out["port"]),
    }
    with open(os.path.join(HERE, "port_vs_reference.json"), "w") as f:
        json.dump(res, f, indent=1)
        f.write("\n")
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
