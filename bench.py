"""Benchmark: full-world geometry rebuild on one GB300.

Workload (one "step"): every chunk of a 2048x256x2048 world of 64^3 chunks
(32x4x32 = 4096 chunks), terrain + caves, RLE-resident in HBM, goes through
decode -> exposure cull -> LOD 0..4 -> splat emission, or -> quad mesh for
chunks whose centre lies within 512 voxels of the camera (the reference's
near/far rule, src/game.c:612-618). Metric: 64^3 chunks per second.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]

Under torchrun (N > 1) every rank rebuilds its own replica world (the path
has no exchange step); `value` is the chunks of all ranks over the slowest
rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "64³ chunks/s (RLE→cull→LOD→emit) batched vs plain on 1 GB300; edit→mesh p99 ms"
SEED = 2024
LOD_MAX = 4
CAMERA = (1024.0, 160.0, 1024.0)
MESH_RADIUS = 512.0
L2_FLUSH_BYTES = 512 << 20
E2E_SLABS = 4
SERVE_SLOTS = 4
SERVE_MAX_BATCH = 64


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_world():
    from voxplat_gb300 import worldgen as wg
    return wg.terrain(wg.TERRAIN_CAVES, 6, (5, 2, 5), seed=SEED)


def mesh_modes(world):
    R = world.R
    n = world.nchunks
    c = np.arange(n)
    bx, by, _ = world.max_bitw
    xs = (c & ((1 << bx) - 1)) * R + R // 2
    ys = ((c >> bx) & ((1 << by) - 1)) * R + R // 2
    zs = (c >> (bx + by)) * R + R // 2
    d = np.sqrt((xs - CAMERA[0]) ** 2 + (ys - CAMERA[1]) ** 2 + (zs - CAMERA[2]) ** 2)
    return (d < MESH_RADIUS).astype(np.uint8)


def workload_config(world, modes):
    return {
        "workload": "2048x256x2048 world, 32x4x32 chunks of 64^3, terrain+caves (seed %d), RLE-resident; "
                    "decode+cull+LOD0..4+splats, near chunks (<512 voxels from camera) meshed" % SEED,
        "chunks": int(world.nchunks),
        "chunk_size": int(world.R),
        "lod_max": LOD_MAX,
        "mesh_chunks": int(modes.sum()),
        "rle_mb": round(world.rle_bytes() / 1e6, 2),
        "l2": "flushed between timed steps (512 MiB write)",
    }


_REASON_BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
                0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}


class _Nvml:
    """Read-only NVML queries through ctypes (SM clock, its maximum, power,
    the active clock-event reasons). Nothing here sets anything."""

    def __init__(self, index, pci=None):
        import ctypes
        self.c = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        ok = False
        if pci:
            for bus in ("0000" + pci, pci):
                if self.lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(self.h)) == 0:
                    ok = True
                    break
        if not ok and self.lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(self.h)) != 0:
            raise RuntimeError("no NVML handle")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        self.max_sm = self._uint(self.lib.nvmlDeviceGetMaxClockInfo, 1)

    def _uint(self, fn, *args):
        v = self.c.c_uint()
        if fn(self.h, *args, self.c.byref(v)) != 0:
            return None
        return v.value

    def sample(self):
        r = self.c.c_ulonglong()
        rs = r.value if self.reasons_fn(self.h, self.c.byref(r)) == 0 else 0
        return self._uint(self.lib.nvmlDeviceGetClockInfo, 1), self._uint(self.lib.nvmlDeviceGetPowerUsage), rs

    def close(self):
        self.lib.nvmlShutdown()


class ClockSampler:
    """SM clocks and clock-event reasons sampled during the timed region:
    NVML every 2 ms from a thread (the timed regions last tens of ms), or
    nvidia-smi every 100 ms where NVML cannot be loaded."""

    def __init__(self, index=0, pci=None, period_s=0.002):
        self.index, self.pci, self.period = index, pci, period_s
        self.proc = None
        self.nvml = None
        self.lines = []
        self.samples = []
        self.stop = threading.Event()

    def __enter__(self):
        try:
            self.nvml = _Nvml(self.index, self.pci)
            self.samples.append(self.nvml.sample())
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            return self
        except Exception:
            self.nvml = None
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _poll(self):
        while not self.stop.wait(self.period):
            self.samples.append(self.nvml.sample())

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.nvml:
            self.stop.set()
            self.t.join(timeout=5)
            self.samples.append(self.nvml.sample())
            self.nvml.close()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons, pw = [], 0.0, set(), []
        if self.nvml:
            for clk, mw, rs in self.samples:
                if clk is None:
                    continue
                sm.append(float(clk))
                if mw is not None:
                    pw.append(mw / 1e3)
                for bit, nm in _REASON_BITS.items():
                    if rs & bit:
                        reasons.add(nm)
            mx = float(self.nvml.max_sm or 0)
            src = "nvml, every %g ms" % (self.period * 1e3)
        else:
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for ln in self.lines:
                f = [x.strip() for x in ln.split(",")]
                if len(f) < 8:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = max(mx, float(f[2]))
                    pw.append(float(f[3]))
                except ValueError:
                    continue
                for k, nm in enumerate(names):
                    if f[4 + k].lower().startswith("active"):
                        reasons.add(nm)
            src = "nvidia-smi, every 100 ms"
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "sm_min_mhz": min(sm) if sm else None, "power_w": round(float(np.median(pw)), 1) if pw else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": src}


def bind_near_gpu(dev):
    """Pin this process to the CPU cores next to GPU `dev` (its PCI
    device's local_cpulist) before any pinned host buffer is allocated, so
    those pages land on the GPU's own NUMA node and host<->device copies do
    not cross the socket link. Returns what was done, for the JSON line."""
    try:
        import torch
        p = torch.cuda.get_device_properties(dev)
        bus = "%04x:%02x:%02x.0" % (getattr(p, "pci_domain_id", 0), p.pci_bus_id, p.pci_device_id)
        base = "/sys/bus/pci/devices/" + bus
        with open(base + "/local_cpulist") as f:
            spec = f.read().strip()
        cpus = set()
        for part in spec.split(","):
            a, _, b = part.partition("-")
            cpus.update(range(int(a), int(b or a) + 1))
        cpus &= os.sched_getaffinity(0)
        node = None
        try:
            with open(base + "/numa_node") as f:
                node = int(f.read().strip())
        except (OSError, ValueError):
            pass
        if cpus:
            os.sched_setaffinity(0, cpus)
        return {"pci": bus, "numa_node": node, "cpus": len(cpus)}
    except Exception as e:  # no sysfs entry (containers, other platforms): leave affinity alone
        return {"unbound": type(e).__name__}


def dist_setup():
    from voxplat_gb300 import replicas
    return replicas.init("nccl")


def port_calibration():
    """oracle/port_vs_reference.json: the port's speed over the reference's
    own C on the same chunks, threads and flags (oracle/calibrate.py)."""
    try:
        with open(os.path.join(ROOT, "oracle", "port_vs_reference.json")) as f:
            c = json.load(f)
        return {"port_vs_reference": c["port_vs_reference"], "threads": c["threads"], "cpu": c["cpu"],
                "machine": c["machine"]}
    except (OSError, ValueError, KeyError):
        return None


def cpu_baseline(world, modes, budget_s=12.0, threads=None, check=None):
    """The cpu_baseline leg: the oracle (C restatement of the reference
    mesher) timed on a bounded sample of the workload's chunks, OpenMP over
    all host cores; and, as the checker, every chunk of one GPU step's
    outputs (`check` = host svl, vbo, ibo arrays and result records)
    compared with the oracle byte for byte."""
    from oracle.bindings import OracleWorld
    threads = threads or len(os.sched_getaffinity(0))
    o = OracleWorld(world)
    parity = None
    if check is not None:
        t0 = time.perf_counter()
        bad, nbad = o.check(np.arange(world.nchunks), modes, LOD_MAX, *check, nthreads=threads)
        parity = {"checked": int(world.nchunks), "mismatches": nbad, "first_bad": bad[:8],
                  "what": "every chunk of the last end-to-end step's host outputs vs the oracle, byte for byte",
                  "s": round(time.perf_counter() - t0, 2)}
    rng = np.random.default_rng(1)
    order = rng.permutation(world.nchunks).astype(np.uint32)
    n = 256
    t0 = time.perf_counter()
    o.rebuild(order[:n], modes, LOD_MAX, threads)
    dt = time.perf_counter() - t0
    # grow the sample to fill the budget, then time it once more
    n = int(min(world.nchunks, max(n, n * budget_s / max(dt, 1e-3) / 2)))
    t0 = time.perf_counter()
    o.rebuild(order[:n], modes, LOD_MAX, threads)
    dt = time.perf_counter() - t0
    out = {"value": round(n / dt, 1), "unit": "chunks/s", "cores": threads, "kind": "port",
           "sample": "%d of the %d chunks (random, seed 1), cold decode, same modes/LOD" % (n, world.nchunks)}
    # the per-chunk pipeline on one core (the reference's single-thread view),
    # on a sample sized from the parallel rate for about two seconds
    n1 = int(min(world.nchunks, max(32, 2.0 * out["value"] / threads)))
    t0 = time.perf_counter()
    o.rebuild(order[:n1], modes, LOD_MAX, 1)
    dt1 = time.perf_counter() - t0
    out["single_thread"] = {"value": round(n1 / dt1, 1), "unit": "chunks/s", "cores": 1,
                            "voxels_per_s": round(n1 / dt1 * world.R ** 3, 1),
                            "sample": "the first %d chunks of the same sample" % n1}
    cal = port_calibration()
    if cal:
        out["calibration"] = cal
    return out, parity


def profile_value(key, name="k_geometry_world_2048x256x2048.md", cast=int):
    """A `key: value` line of a committed ncu summary under profiles/."""
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return cast(line.split(":")[1])
    except (OSError, ValueError):
        pass
    return None


def ncu_traffic(name="k_geometry_world_2048x256x2048.md"):
    """DRAM bytes per launch of k_geometry from the committed ncu summary."""
    return profile_value("traffic_bytes_per_launch", name)


def algorithmic_bytes(world, res):
    """Per rebuild: RLE read + splat/mesh output + shadow map read once."""
    rle = int(world.len.astype(np.int64).sum()) * 4
    out = int(res["svl_total"].astype(np.int64).sum()) * 2 + int(res["vbo_items"].astype(np.int64).sum()) * 2 \
        + int(res["ibo_items"].astype(np.int64).sum()) * 4
    shadow = world.shadow_w * world.shadow_z * 2
    return rle + out + shadow, rle, out, shadow


def run_ours(args):
    import torch
    from voxplat_gb300 import gpu
    rank, ws, dist = dist_setup()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    all_cpus = os.sched_getaffinity(0)
    host_binding = bind_near_gpu(dev)
    world = make_world()
    modes = mesh_modes(world)
    ctx = gpu.Context(dev)
    dw = gpu.DeviceWorld(ctx, world)
    dw.set_modes(modes)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda:%d" % dev)
    for _ in range(max(args.warmup, 3)):
        dw.rebuild(LOD_MAX, group=True)
        dw.finish()
    res = dw.results()
    assert (res["status"] == 0).all()
    ctx.set_timing(True)
    dw.kernel_ms()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev, host_binding.get("pci")) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                starts[k].record(stream)
            dw.rebuild(LOD_MAX, group=True)
            with torch.cuda.stream(stream):
                ends[k].record(stream)
        ctx.sync()
        torch.cuda.synchronize()
    step_ms = [s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)]
    shell_ms, geo_ms, grp_ms, launches = dw.kernel_ms()
    ctx.set_timing(False)
    from voxplat_gb300 import replicas
    t_ms = replicas.max_over_ranks(float(np.sum(step_ms)), dist, device="cuda")
    value = replicas.whole_job_rate(world.nchunks * args.steps, ws, t_ms)
    ab, rle_b, out_b, sh_b = algorithmic_bytes(world, res)
    geo_avg_ms = geo_ms / args.steps
    peak, peak_kind = peaks()
    achieved = ab / (geo_avg_ms / 1e3) / 1e9
    # + grouping: the splats of levels >= 1 are read and written once more
    # (a level-0 node is one chunk's level-0 segment, used where it lies)
    grouped_bytes = int(res["svl_items"][:, 1:].astype(np.int64).sum()) * 2
    step_bytes = ab + 2 * grouped_bytes
    # plain path: one launch per chunk and pass, same world and modes
    dw.rebuild(LOD_MAX, persistent=False, plain=True)
    dw.finish()
    plain_ms = []
    for _ in range(2):
        with torch.cuda.stream(stream):
            flush.zero_()
            a_ = torch.cuda.Event(enable_timing=True)
            b_ = torch.cuda.Event(enable_timing=True)
            a_.record(stream)
        dw.rebuild(LOD_MAX, persistent=False, plain=True)
        with torch.cuda.stream(stream):
            b_.record(stream)
        ctx.sync()
        torch.cuda.synchronize()
        plain_ms.append(a_.elapsed_time(b_))
    plain_value = world.nchunks / (float(np.median(plain_ms)) / 1e3)
    # the same launches spread over 16 streams, so they run side by side
    dw.rebuild(LOD_MAX, persistent=False, concurrent=True)
    dw.finish()
    conc_ms = []
    for _ in range(2):
        with torch.cuda.stream(stream):
            flush.zero_()
            a_ = torch.cuda.Event(enable_timing=True)
            b_ = torch.cuda.Event(enable_timing=True)
            a_.record(stream)
        dw.rebuild(LOD_MAX, persistent=False, concurrent=True)
        with torch.cuda.stream(stream):
            b_.record(stream)
        ctx.sync()
        torch.cuda.synchronize()
        conc_ms.append(a_.elapsed_time(b_))
    plain_conc_value = world.nchunks / (float(np.median(conc_ms)) / 1e3)
    # end to end through the C ABI with host buffers: the caller's world and
    # its output buffers live in pinned host memory; every step uploads the
    # world (H2D + device validation), rebuilds, and reads the result
    # records and all outputs back (D2H)
    keep = []

    def pinned(a, view):
        t = torch.from_numpy(np.ascontiguousarray(a).view(view)).pin_memory()
        keep.append(t)
        return t.numpy().view(a.dtype)

    pool_h = pinned(world.pool, np.int32)
    off_h = pinned(world.off, np.int64)
    len_h = pinned(world.len, np.int32)
    shadow_h = pinned(world.shadow, np.int16)
    modes_h = pinned(modes, np.int8)
    cur = [int(np.max(res[k] + res[n])) * m for k, n, m in
           (("svl_off", "svl_total", 2), ("vbo_off", "vbo_items", 2), ("ibo_off", "ibo_items", 4))]
    outs_h = [pinned(np.zeros(c // d + (64 << 10), dt), vw) for c, d, dt, vw in
              ((cur[0], 2, np.int16, np.int16), (cur[1], 2, np.int16, np.int16), (cur[2], 4, np.uint32, np.int32))]
    res_h = pinned(np.zeros(world.nchunks, gpu.RESULT_DTYPE), np.uint8)
    e2e_t = []
    h2d = pool_h.nbytes + off_h.nbytes + len_h.nbytes + shadow_h.nbytes + modes_h.nbytes
    d2h = 0
    for k in range(max(3, min(args.steps, 10))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dw.upload_arrays(pool_h, off_h, len_h, shadow_h, world.shadow_w)
        dw.set_modes(modes_h)
        used = dw.rebuild_to_host(LOD_MAX, *outs_h, res_h, group=True, slabs=E2E_SLABS)
        e2e_t.append(time.perf_counter() - t0)
        d2h = res_h.nbytes + sum(used)
    e2e_sync_value = world.nchunks / float(np.median(e2e_t[1:]))
    # the same steps pipelined: step k+1's upload and compute run while step
    # k's outputs are copied back (two pinned output sets, alternating); the
    # clock stops once the last step's outputs are in host memory
    sets = [(outs_h, res_h)]
    sets.append(([pinned(np.zeros_like(o), vw) for o, vw in zip(outs_h, (np.int16, np.int16, np.int32))],
                 pinned(np.zeros(world.nchunks, gpu.RESULT_DTYPE), np.uint8)))

    def e2e_step(k):
        o, r = sets[k % 2]
        dw.upload_arrays(pool_h, off_h, len_h, shadow_h, world.shadow_w)
        dw.set_modes(modes_h)
        return dw.rebuild_to_host_async(LOD_MAX, *o, r, group=True, slabs=E2E_SLABS)

    for k in range(3):
        e2e_step(k)
    dw.outputs_wait()
    n_e2e = max(4, args.steps)
    # three timed runs of n_e2e pipelined steps; the median run is reported
    # (the host thread's scheduling moves a single run by up to ~15 %)
    e2e_runs = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(n_e2e):
            used_p = e2e_step(k)
        dw.outputs_wait()
        e2e_runs.append(time.perf_counter() - t0)
    e2e_s = float(np.median(e2e_runs))
    e2e_value = n_e2e * world.nchunks / e2e_s
    if not (used_p == used and np.array_equal(sets[(n_e2e - 1) % 2][1]["svl_total"], res_h["svl_total"])):
        raise RuntimeError("pipelined end-to-end rebuild disagrees with the synchronous one")
    # the host link's own device->host rate for the same bytes (one pinned
    # copy): the bound of the end-to-end step
    link_dev = torch.empty(d2h, dtype=torch.uint8, device="cuda:%d" % dev)
    link_host = torch.empty(d2h, dtype=torch.uint8).pin_memory()
    link_ms = []
    for _ in range(4):
        a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_.record()
        link_host.copy_(link_dev, non_blocking=True)
        b_.record()
        torch.cuda.synchronize()
        link_ms.append(a_.elapsed_time(b_))
    link_gbs = d2h / (float(np.median(link_ms[1:])) * 1e6)
    del link_dev, link_host
    e2e_ms = e2e_s * 1e3 / n_e2e
    out = {
        "metric": METRIC,
        "value": round(value, 1),
        "unit": "chunks/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(t_ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u8",
        "data": "synthetic (seeded integer-hash terrain + caves; no dataset)",
        "config": workload_config(world, modes),
        "e2e": {"value": round(e2e_value, 1), "unit": "chunks/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_ms, 3),
                "path": "pinned host world -> vp_world_upload -> vp_world_rebuild_to_host_async -> pinned host",
                "sync_value": round(e2e_sync_value, 1),
                "link_d2h_gbs": round(link_gbs, 1),
                "link_bound_ms": round(d2h / link_gbs / 1e6, 3),
                "link_frac": round((d2h / link_gbs / 1e6) / e2e_ms, 4),
                "host": host_binding},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": ncu_traffic(), "kernel": "k_geometry<6>",
                     "peak_source": peak_kind, "algorithmic_bytes": int(ab),
                     "step_frac": round(step_bytes / (t_ms / args.steps / 1e3) / 1e9 / peak, 4)},
        "kernel_ms": {"shell": round(shell_ms / args.steps, 4), "geometry": round(geo_avg_ms, 4),
                      "group": round(grp_ms / args.steps, 4)},
        "plain_value": round(plain_value, 1),
        "plain_concurrent_value": round(plain_conc_value, 1),
        "gpu_launches": int(launches),
    }
    detail = {"detail": "bench.py sub-benchmarks; the headline is the next line",
              "voxels_per_s": round(value * world.R ** 3, 1),
              "plain": {"value": round(plain_value, 1), "unit": "chunks/s", "launches_per_step": 2 * world.nchunks,
                        "batched_over_plain": round(value / plain_value, 2),
                        "concurrent": {"value": round(plain_conc_value, 1), "streams": 16,
                                       "batched_over_plain": round(value / plain_conc_value, 2),
                                       "note": "the same launches round-robin over 16 streams"}},
              "e2e": {"steps": n_e2e, "ms_per_step": round(e2e_ms, 3),
                      "runs_ms_per_step": [round(t * 1e3 / n_e2e, 3) for t in e2e_runs],
                      "path": "pinned host world -> vp_world_upload -> vp_world_rebuild_to_host_async (group; "
                              "outputs stream back per slab, and under the next step's upload and compute) -> two "
                              "alternating pinned host buffer sets + result records; clock stops after the last "
                              "step's copies; the median of three timed runs",
                      "synchronous": {"value": round(e2e_sync_value, 1), "unit": "chunks/s",
                                      "path": "vp_world_rebuild_to_host: each step's copies end before the next"},
                      "link": {"d2h_gbs": round(link_gbs, 1), "bound_ms_per_step": round(d2h / link_gbs / 1e6, 3),
                               "note": "one pinned device->host copy of d2h_bytes_per_step, CUDA events"}},
              "roofline": {"traffic_source": "profiles/k_geometry_world_2048x256x2048.md (ncu dram__bytes_read+"
                                             "write.sum)",
                           "bytes_split": {"rle_in": rle_b, "geometry_out": out_b, "shadow_map": sh_b},
                           "step_bytes": int(step_bytes),
                           "issue_active_frac": profile_value("issue_active_frac", cast=float)}}
    if rank == 0:
        out["clocks"] = clk.summary()
        detail["picking"] = picking(dw)
        dw.rebuild(LOD_MAX, group=True)
        dw.finish()
        detail["render"] = render_frame(dw, CAMERA)
        dw.close()
        if not args.skip_edits:
            es = edit_serving(ctx)
            detail["edit_serving"] = es
            out["edit_p99_ms"] = es["p99_ms"]
        if not args.skip_uneven:
            ub = uneven_batch(ctx)
            detail["uneven_batch"] = ub
            out["uneven_batched_over_plain"] = ub["batched_over_plain"]
            out["uneven_batched_over_plain_concurrent"] = ub["batched_over_plain_concurrent"]
        if not args.skip_full_scale:
            fs = full_scale(ctx)
            res5, dw5 = fs.pop("_res"), fs.pop("_dw")
            fs["draw_cull"] = draw_cull(dw5)
            dw5.close()
            detail["full_scale"] = fs
            out["full_scale_frac"] = fs["step_frac_of_measured_hbm"]
        last = sets[(n_e2e - 1) % 2]
        os.sched_setaffinity(0, all_cpus)  # the CPU baseline gets every host core
        out["cpu_baseline"], out["parity"] = cpu_baseline(world, modes, check=(last[0][0], last[0][1], last[0][2],
                                                                                last[1]))
        print(json.dumps(detail), flush=True)
        print(json.dumps(out), flush=True)
    replicas.finish(dist)


def edit_trace(seed, n, rate, extent_xz, band=(8, 56), rmax=32):
    """Poisson arrivals at `rate`/s; spheres with r ~ U[1, rmax], centres
    uniform over the surface band, half carves and half fills (colour
    uniform 1..255)."""
    from voxplat_gb300 import gpu
    rng = np.random.default_rng(seed)
    arrival = np.cumsum(rng.exponential(1.0 / rate, n))
    rows = np.zeros((n, 5), np.int64)
    rows[:, 0] = rng.integers(0, extent_xz, n)
    rows[:, 1] = rng.integers(band[0], band[1] + 1, n)
    rows[:, 2] = rng.integers(0, extent_xz, n)
    rows[:, 3] = rng.integers(1, rmax + 1, n)
    fill = rng.random(n) < 0.5
    rows[:, 4] = np.where(fill, rng.integers(1, 256, n), 0)
    return gpu.make_edits(rows, arrival)


def uneven_batch(ctx, n=4096, seed=3, steps=5, root=None):
    """4096 standalone chunks, roots 32/64/128 in ratio 1:6:1, occupancy
    log-uniform 0.1%..100% (noise blobs + uniform random voxels), colours
    1..255; splats LOD 0..4. Batched = the autotuned configuration replayed
    as a CUDA graph (one persistent launch); plain = one launch per chunk.
    With `root` (5, 6 or 7), the first n chunks of the same sequence with
    that root only (a smaller case of one kernel, for profiling)."""
    from concurrent.futures import ThreadPoolExecutor
    from voxplat_gb300 import gpu
    from voxplat_gb300 import worldgen as wg
    t0 = time.perf_counter()
    ks = list(range(n))
    if root is not None:
        ks, k = [], 0
        while len(ks) < n:
            if wg.uneven_root_bitw(seed, k) == root:
                ks.append(k)
            k += 1
    with ThreadPoolExecutor(max(1, min(16, os.cpu_count() or 1))) as ex:
        ws = list(ex.map(lambda k: wg.uneven_chunk(seed, k), ks))
    gen_s = time.perf_counter() - t0
    b = gpu.DeviceBatch(ctx, ws)
    del ws
    b.set_modes(None)
    best, tried = b.autotune(LOD_MAX)
    ctx.set_timing(True)
    b.rebuild(LOD_MAX, mode="graph")
    b.finish()
    b.kernel_ms()
    for _ in range(steps):
        b.rebuild(LOD_MAX, mode="graph")
    b.finish()
    g_ms, g_launches = b.kernel_ms()
    g_ms /= steps
    b.rebuild(LOD_MAX, mode="plain")
    b.finish()
    p_ms, p_launches = b.kernel_ms()
    b.rebuild(LOD_MAX, mode="concurrent")
    b.finish()
    c_ms, _ = b.kernel_ms()
    ctx.set_timing(False)
    res = b.results()
    out_b = int(res["svl_total"].astype(np.int64).sum()) * 2
    step_b = b.rle_bytes + out_b
    roots = {str(1 << r): int((b.root_bitw == r).sum()) for r in (5, 6, 7)}
    eq64 = b.voxels / float(64 ** 3)
    out = {
        "workload": "%d standalone chunks, roots 32/64/128 (%s), occupancy log-uniform 0.1%%..100%%, LOD 0..4 splats"
                    % (n, ":".join(str(v) for v in roots.values())),
        "roots": roots,
        "batched_ms": round(g_ms, 3),
        "batched_chunks_per_s": round(n / (g_ms / 1e3), 1),
        "batched_chunks64_equiv_per_s": round(eq64 / (g_ms / 1e3), 1),
        "batched_launches_per_rebuild": g_launches // steps,
        "plain_ms": round(p_ms, 3),
        "plain_chunks_per_s": round(n / (p_ms / 1e3), 1),
        "plain_launches_per_rebuild": p_launches,
        "batched_over_plain": round(p_ms / g_ms, 2),
        "plain_concurrent_ms": round(c_ms, 3),
        "batched_over_plain_concurrent": round(c_ms / g_ms, 2),
        "tune": best,
        "tried": tried,
        "rle_in_mb": round(b.rle_bytes / 1e6, 1),
        "splats_out_mb": round(out_b / 1e6, 1),
        "step_gbs": round(step_b / (g_ms / 1e3) / 1e9, 1),
        "step_frac_of_measured_hbm": round(step_b / (g_ms / 1e3) / 1e9 / peaks()[0], 4),
        "gen_s": round(gen_s, 2),
    }
    b.close()
    return out


def edit_serving(ctx, seconds=2.0, rate=2000.0, seed=4):
    """8192x512x8192 world of 64^3 chunks (small terrain, heights 8..56),
    generated and kept RLE-resident on the device with all geometry; a
    Poisson trace of sphere edits replayed in real time with continuous
    batching. Latency = edit arrival -> its chunks re-encoded and remeshed."""
    import torch
    from voxplat_gb300 import gpu
    from voxplat_gb300 import worldgen as wg
    t0 = time.perf_counter()
    dw = gpu.DeviceWorld.generated(ctx, wg.TERRAIN_SMALL, 6, (7, 3, 7), seed=7)
    gen_s = time.perf_counter() - t0
    n = dw.nchunks
    c = np.arange(n)
    xs = (c & 127) * 64 + 32
    ys = ((c >> 7) & 7) * 64 + 32
    zs = (c >> 10) * 64 + 32
    modes = (np.sqrt((xs - 4096.0) ** 2 + (ys - 32.0) ** 2 + (zs - 4096.0) ** 2) < MESH_RADIUS).astype(np.uint8)
    dw.set_modes(modes)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dw.rebuild(LOD_MAX)
    dw.finish()
    rebuild_s = time.perf_counter() - t0
    edits = edit_trace(seed, int(seconds * rate), rate, 8192)
    warm = edit_trace(seed + 1, 200, rate, 8192)
    dw.serve(warm, max_batch=SERVE_MAX_BATCH, slots=SERVE_SLOTS)
    lat, st = dw.serve(edits, max_batch=SERVE_MAX_BATCH, slots=SERVE_SLOTS)
    out = {
        "workload": "8192x512x8192 world (128x8x128 chunks of 64^3), small terrain, RLE-resident; "
                    "Poisson sphere edits at %d/s, r~U[1,32], 50%% carve / 50%% fill, centres in y 8..56" % rate,
        "edits": int(st.edits),
        "p50_ms": round(float(np.percentile(lat, 50)), 4),
        "p99_ms": round(float(np.percentile(lat, 99)), 4),
        "max_ms": round(float(lat.max()), 4),
        "batches": int(st.batches),
        "mean_batch": round(st.edits / max(st.batches, 1), 2),
        "max_batch": int(st.max_batch),
        "deferred": int(st.deferred),
        "rejected": int(st.rejected),
        "slots": SERVE_SLOTS,
        "max_inflight": int(st.max_inflight),
        "mean_inflight_when_busy": round(st.inflight_s / max(st.busy_s, 1e-9), 3),
        "chunks_remeshed_per_s": round(st.chunks_remeshed / st.wall_s, 1),
        "gpu_busy_frac": round(st.busy_s / st.wall_s, 3),
        "world_gen_s": round(gen_s, 2),
        "full_rebuild_ms": round(rebuild_s * 1e3, 2),
        "full_rebuild_chunks_per_s": round(n / rebuild_s, 1),
    }
    dw.close()
    return out


def draw_cull(dw, reps=20):
    """Octree draw cull + LOD selection (src/game.c:319-395) of the grouped
    world from a camera at its centre, through the C ABI (queues to host)."""
    from voxplat_gb300.camera import perspective_view
    ext = [(1 << dw.root_bitw) << b for b in dw.max_bitw]
    eye = np.array([ext[0] / 2, 300.0, ext[2] / 2], np.float32)
    vp = perspective_view(eye, eye + np.array([0.3, -0.2, 1.0]), fov_deg=70, far=40000)
    mq, sq = dw.cull(vp, eye)
    t0 = time.perf_counter()
    for _ in range(reps):
        mq, sq = dw.cull(vp, eye)
    ms = (time.perf_counter() - t0) / reps * 1e3
    t0 = time.perf_counter()
    for _ in range(reps):
        dw.camera_modes(eye)
    mm = (time.perf_counter() - t0) / reps * 1e3
    nodes = sum((dw.nchunks >> (3 * l)) for l in range(5))
    return {"ms_per_cull": round(ms, 3), "octree_nodes": int(nodes), "mesh_queue": int(len(mq)),
            "splat_queue": int(len(sq)), "ms_per_camera_modes": round(mm, 3)}


def render_frame(dw, modes_eye, width=1920, height=1080, reps=5):
    """Draw cull + CUDA rasteriser of the splat and mesh shaders at 1080p
    from the bench camera, through the C ABI (frame back to host, into
    page-locked RGBA and depth arrays reused from frame to frame)."""
    import torch
    from voxplat_gb300.camera import camera
    eye = np.asarray(modes_eye, np.float32)
    cam = camera(eye, eye + np.array([0.6, -0.25, 1.0]), width, height, fov_deg=70.0, far=4096.0)
    mq, sq = dw.cull(cam["view_projection"], eye)
    host_rgba = torch.empty((height, width), dtype=torch.int32).pin_memory()
    host_depth = torch.empty((height, width), dtype=torch.float32).pin_memory()
    out = (host_rgba.numpy().view(np.uint32), host_depth.numpy())
    rgba, depth, stats = dw.render(cam, mq, sq, out=out)
    t0 = time.perf_counter()
    for _ in range(reps):
        rgba, depth, stats = dw.render(cam, mq, sq, out=out)
    ms = (time.perf_counter() - t0) / reps * 1e3
    return {"width": width, "height": height, "ms_per_frame": round(ms, 3), "splats": int(stats[0]),
            "triangles": int(stats[1]), "pixels_drawn": int((depth < 1.0).sum()),
            "splats_per_s": round(stats[0] / (ms / 1e3), 1), "mesh_chunks": int(len(mq)), "splat_nodes": int(len(sq))}


def picking(dw, n=65536, seed=6):
    """Picking rays (chunkset_edit_raycast_until_solid) through the C ABI:
    n rays from above the terrain, downwards at random angles."""
    rng = np.random.default_rng(seed)
    ext = [(1 << dw.root_bitw) << b for b in dw.max_bitw]
    org = np.stack([rng.uniform(0, ext[0], n), rng.uniform(200, ext[1], n), rng.uniform(0, ext[2], n)], 1)
    vec = np.stack([rng.normal(size=n), -np.abs(rng.normal(size=n)) - 0.2, rng.normal(size=n)], 1)
    org, vec = org.astype(np.float32), vec.astype(np.float32)
    vox, _, _ = dw.raycast(org, vec)
    t0 = time.perf_counter()
    for _ in range(5):
        vox, _, _ = dw.raycast(org, vec)
    s_ = (time.perf_counter() - t0) / 5
    return {"rays": n, "ms_per_batch": round(s_ * 1e3, 3), "rays_per_s": round(n / s_, 1),
            "hit_fraction": round(float((vox > 0).mean()), 3)}


def full_scale(ctx, steps=3, bits=(8, 8)):
    """16384x512x16384 world (256x8x256 = 524288 chunks of 64^3, 128 GiB of
    voxels), terrain + caves at 4x horizontal noise scale, generated and kept
    RLE-resident on the device; full rebuild with LOD 0..5, splats/meshes
    and LOD/octree grouping. `bits` (x and z chunk bit widths) give the
    corner of the same world at a smaller size, for profiling."""
    import torch
    from voxplat_gb300 import gpu
    from voxplat_gb300 import worldgen as wg
    bx, bz = bits
    t0 = time.perf_counter()
    dw = gpu.DeviceWorld.generated(ctx, wg.TERRAIN_CAVES, 6, (bx, 3, bz), seed=99, hshift=2)
    gen_s = time.perf_counter() - t0
    n = dw.nchunks
    c = np.arange(n)
    xs = (c & ((1 << bx) - 1)) * 64 + 32
    ys = ((c >> bx) & 7) * 64 + 32
    zs = (c >> (bx + 3)) * 64 + 32
    cx, cz = (1 << bx) * 32.0, (1 << bz) * 32.0
    modes = (np.sqrt((xs - cx) ** 2 + (ys - 160.0) ** 2 + (zs - cz) ** 2) < MESH_RADIUS).astype(np.uint8)
    dw.set_modes(modes)
    dw.rebuild(5, group=True)
    dw.finish()
    res = dw.results()
    ctx.set_timing(True)
    dw.kernel_ms()
    stream = torch.cuda.ExternalStream(ctx.stream)
    evs = []
    for _ in range(steps):
        a_ = torch.cuda.Event(enable_timing=True)
        b_ = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a_.record(stream)
        dw.rebuild(5, group=True)
        with torch.cuda.stream(stream):
            b_.record(stream)
        evs.append((a_, b_))
    ctx.sync()
    torch.cuda.synchronize()
    ms = float(np.median([a_.elapsed_time(b_) for a_, b_ in evs]))
    shell_ms, geo_ms, grp_ms, _ = dw.kernel_ms()
    handoff_gb = dw.handoff_bytes() / 1e9
    # the same rebuilds with the decoded-chunk handoff off (the geometry
    # pass decodes every chunk again): which of the two is faster here
    dw.set_handoff(False)
    dw.rebuild(5, group=True)
    dw.finish()
    dw.kernel_ms()
    evs_off = []
    for _ in range(steps):
        a_ = torch.cuda.Event(enable_timing=True)
        b_ = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a_.record(stream)
        dw.rebuild(5, group=True)
        with torch.cuda.stream(stream):
            b_.record(stream)
        evs_off.append((a_, b_))
    ctx.sync()
    torch.cuda.synchronize()
    ms_off = float(np.median([a_.elapsed_time(b_) for a_, b_ in evs_off]))
    shell_off, geo_off, grp_off, _ = dw.kernel_ms()
    dw.set_handoff(True)
    ctx.set_timing(False)
    splats = int(res["svl_total"].astype(np.int64).sum()) // 4
    faces = int(res["ibo_items"].astype(np.int64).sum()) // 6
    # step bytes: RLE in, splats out plus the grouped copy of levels >= 1
    # (read and written again), mesh out, the shadow map once ((X + Y) x Z
    # entries of 2 bytes)
    rle = dw.rle_bytes()
    grouped = int(res["svl_items"][:, 1:].astype(np.int64).sum()) * 2
    geo_out = int(res["svl_total"].astype(np.int64).sum()) * 2 + int(res["vbo_items"].astype(np.int64).sum()) * 2 \
        + int(res["ibo_items"].astype(np.int64).sum()) * 4
    shadow_b = ((64 << bx) + 512) * (64 << bz) * 2
    step_b = rle + geo_out + 2 * grouped + shadow_b
    out = {
        "workload": "%dx512x%d world (%dx8x%d = %d chunks of 64^3), terrain+caves at 4x horizontal "
                    "noise scale, RLE-resident; LOD 0..5, splats/meshes, LOD/octree grouping"
                    % (64 << bx, 64 << bz, 1 << bx, 1 << bz, n),
        "chunks": n,
        "ms_per_rebuild": round(ms, 3),
        "chunks_per_s": round(n / (ms / 1e3), 1),
        "voxels_per_s": round(n * 64 ** 3 / (ms / 1e3), 1),
        "kernel_ms": {"shell": round(shell_ms / steps, 3), "geometry": round(geo_ms / steps, 3),
                      "group": round(grp_ms / steps, 3)},
        "handoff_gb": round(handoff_gb, 3),
        "handoff_off": {"ms_per_rebuild": round(ms_off, 3),
                        "kernel_ms": {"shell": round(shell_off / steps, 3), "geometry": round(geo_off / steps, 3),
                                      "group": round(grp_off / steps, 3)}},
        "splats": splats,
        "faces": faces,
        "mesh_chunks": int(modes.sum()),
        "world_gen_s": round(gen_s, 2),
        "rle_gb": round(rle / 1e9, 3),
        "bytes_split": {"rle_in": rle, "geometry_out": geo_out, "grouped_copy": 2 * grouped, "shadow_map": shadow_b},
        "step_bytes": int(step_b),
        "step_gbs": round(step_b / (ms / 1e3) / 1e9, 1),
        "step_frac_of_measured_hbm": round(step_b / (ms / 1e3) / 1e9 / peaks()[0], 4),
    }
    out["_res"] = res
    out["_dw"] = dw
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.bindings import OracleWorld
    threads = len(os.sched_getaffinity(0))
    world = make_world()
    modes = mesh_modes(world)
    o = OracleWorld(world)
    rng = np.random.default_rng(1)
    order = rng.permutation(world.nchunks).astype(np.uint32)
    n = 768
    for _ in range(max(args.warmup, 1)):
        o.rebuild(order[:n], modes, LOD_MAX, threads)
    ts = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        o.rebuild(order[:n], modes, LOD_MAX, threads)
        ts.append(time.perf_counter() - t0)
    t = float(np.sum(ts))
    value = n * args.steps / t
    sample = "%d of the %d chunks per step (random, seed 1), cold decode" % (n, world.nchunks)
    out = {
        "impl": "reference",
        "metric": METRIC,
        "value": round(value, 1),
        "unit": "chunks/s",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(t * 1e3 / args.steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u8",
        "data": "synthetic (seeded integer-hash terrain + caves; no dataset)",
        "config": workload_config(world, modes),
        "cpu_baseline": dict({"value": round(value, 1), "unit": "chunks/s", "cores": threads, "kind": "port",
                              "sample": sample}, **({"calibration": port_calibration()} if port_calibration() else {})),
        "e2e": {"value": round(value, 1), "unit": "chunks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-edits", action="store_true", help="skip the edit-serving sub-benchmark")
    ap.add_argument("--skip-full-scale", action="store_true", help="skip the 524288-chunk full-scale rebuild")
    ap.add_argument("--skip-uneven", action="store_true", help="skip the mixed-root batch sub-benchmark")
    ap.add_argument("--uneven-only", type=int, nargs=2, metavar=("ROOT_BITW", "N"),
                    help="run only the mixed-root batch, restricted to its first N chunks of one root "
                         "(a small case for profiling); prints that sub-benchmark's line")
    ap.add_argument("--edits-only", action="store_true",
                    help="run only the edit-serving sub-benchmark; prints its line")
    ap.add_argument("--full-scale-only", type=int, nargs=2, metavar=("BITS_X", "BITS_Z"),
                    help="run only the full-scale rebuild, on the corner of its world 2^BITS_X x 8 x 2^BITS_Z "
                         "chunks (8 8 is the full world); prints that sub-benchmark's line")
    args = ap.parse_args()
    import __graft_entry__
    __graft_entry__.build()
    if args.uneven_only:
        from voxplat_gb300 import gpu
        root, n = args.uneven_only
        print(json.dumps(uneven_batch(gpu.Context(0), n=n, root=root)), flush=True)
        return
    if args.edits_only:
        from voxplat_gb300 import gpu
        print(json.dumps(edit_serving(gpu.Context(0))), flush=True)
        return
    if args.full_scale_only:
        from voxplat_gb300 import gpu
        fs = full_scale(gpu.Context(0), steps=2, bits=tuple(args.full_scale_only))
        fs.pop("_dw").close()
        fs.pop("_res")
        print(json.dumps(fs), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
