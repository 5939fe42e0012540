#!/usr/bin/env python3
"""Benchmark of the GB300 wave stepper on the single-grid workload.

Workload (one GPU): 3840x2160 grid, 64 seeded discs of refractive index 1.5
(TWOSPEEDS, COURANTB = COURANT/1.5) through the tcc table, absorbing boundary,
GAMMA = 1e-4, an oscillating point source of amplitude 0.05 and seeded period in
[20, 60] updates, energy reported every 100 updates (compensated sums merged in FP64).
One bench step = 100 leapfrog updates + one energy report; 100 steps = the full 10^4
updates.  `value` is the FP32 form in Gcell-updates/s (all cells count), with inputs
resident in HBM; `e2e` is the same metric through the C ABI with host buffers (the
state is copied in and out every step); the plain FP64 form is reported beside it.

--impl reference times the reference's own OpenMP CPU stepper (compiled headlessly
from its sources into oracle/_ref) on this machine's host cores.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
NX, NY, UPDATES_PER_STEP = 3840, 2160, 100
METRIC = "Gcell-updates/s"
CELLS = NX * NY
# the scene both arms step (scenes.config2, seed 0 on rank 0)
WORKLOAD = f"single grid {NX}x{NY}, 64 discs n=1.5 via tcc table, absorbing, GAMMA 1e-4, point source"


def _package():
    import importlib.util
    name = "youtube_simulations_gb300"
    if name not in sys.modules:
        d = ROOT / "youtube-simulations_gb300"
        spec = importlib.util.spec_from_file_location(name, d / "__init__.py", submodule_search_locations=[str(d)])
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def kernel_source_digest():
    """sha256 (first 16 hex digits) of the single-grid kernel sources; profiles/traffic.json
    records the digest its ncu capture was made on, so a stale capture is not reported."""
    import hashlib
    h = hashlib.sha256()
    csrc = ROOT / "youtube-simulations_gb300" / "csrc"
    for name in ("wg_tb.cu", "wg_device.cuh", "wg_cells.cuh", "wg_tma.cuh"):
        h.update((csrc / name).read_bytes())
    return h.hexdigest()[:16]


def bytes_per_cell_update(precision, coef):
    """Algorithmic bytes of one cell update (single-step compulsory traffic):
    read phi(t), psi(t-1), write phi(t+1), the 1-bit mask, and each spatially varying
    coefficient table (tcc here; tgamma is uniform, tc is read on the boundary only)."""
    s = 4 if precision == "fp32" else 8
    return 3 * s + (s if coef == "table" else 0) + 1.0 / 8.0


class Clocks:
    """nvidia-smi clock/throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.gpu = gpu_index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait(timeout=10)
        self.f.flush()
        rows = []
        for line in Path(self.f.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


class NvmlClocks:
    """SM clock and clock-event reasons read through NVML (libnvidia-ml, ctypes) every 2 ms
    from a thread while the timed region runs, so that even a region of a few tens of
    milliseconds has samples inside it.  Reads only; falls back to nvidia-smi (Clocks)
    where NVML cannot be loaded."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, gpu_index, device=None):
        import ctypes
        import threading
        self.ct, self.threading = ctypes, threading
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        bus = None
        try:
            import torch
            pr = torch.cuda.get_device_properties(device)
            bus = "%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
        except Exception:
            bus = None
        ok = bus is not None and self.lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(self.h)) == 0
        if not ok and self.lib.nvmlDeviceGetHandleByIndex_v2(gpu_index, ctypes.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        mx = ctypes.c_uint()
        self.max_mhz = float(mx.value) if self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(mx)) == 0 else None
        self.rows, self.stop_flag, self.t = [], False, None

    def _sample(self):
        ct = self.ct
        clk, rs = ct.c_uint(), ct.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(clk)) != 0:  # NVML_CLOCK_SM
            return
        fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        r = int(rs.value) if fn(self.h, ct.byref(rs)) == 0 else 0
        self.rows.append((float(clk.value), r))

    def _loop(self):
        import time as _t
        while not self.stop_flag:
            self._sample()
            _t.sleep(0.002)

    def start(self):
        self._sample()
        self.t = self.threading.Thread(target=self._loop, daemon=True)
        self.t.start()

    def stop(self):
        self.stop_flag = True
        self.t.join(timeout=5)
        self._sample()
        return self.summary(self.rows, self.max_mhz)

    @classmethod
    def summary(cls, rows, max_mhz):
        """Median SM clock of the samples, the maximum clock and the reasons seen active."""
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": max_mhz, "reasons": ["no samples"]}
        reasons = sorted({name for _, r in rows for bit, name in cls.REASONS.items() if r & bit})
        return {"sm_mhz": statistics.median(c for c, _ in rows), "sm_max_mhz": max_mhz, "reasons": reasons,
                "samples": len(rows), "source": "NVML, every 2 ms during the timed region"}


def clock_sampler(gpu_index, device=None):
    """NVML sampler where the library loads, else nvidia-smi."""
    try:
        return NvmlClocks(gpu_index, device)
    except Exception:
        return Clocks(gpu_index)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(t_ms, world, device):
    """The job's time: the slowest rank's (one all-reduce MAX; every rank gets it)."""
    if world <= 1:
        return t_ms
    import torch
    import torch.distributed as dist
    tt = torch.tensor([t_ms], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def whole_job_rate(world, cells, updates, t_ms):
    """Gcell-updates/s of the whole job: every rank advances its own replica of `cells`
    cells by `updates` updates, in the slowest rank's time t_ms."""
    return world * cells * updates / (t_ms / 1e3) / 1e9


# ---------------------------------------------------------------------------
# Reference arm: the reference's own CPU stepper
# ---------------------------------------------------------------------------
_REF_META = {}


def active_cells(params, xy):
    """Cells the bulk rule updates (wave_billiard.c:365): every cell when TWOSPEEDS, else
    the cells with xy > 0.  The metric counts all grid cells; this is the active share."""
    import numpy as np
    if params.twospeeds:
        return int(params.nx) * int(params.ny)
    return int(np.count_nonzero(np.asarray(xy) > 0))


def with_active_rate(res, active, cells):
    """Adds the active-cell rate (the same run counted over active cells only)."""
    res["active_cell_rate"] = res["value"] * active / cells
    return res


REF_BUILD_FLAGS = "gcc -O3 -fopenmp (the reference makefile's flags, default FP contraction)"


def reference_variant():
    """The timed reference build: the makefile's own flags (ref_c2_stock); the parity
    build (ref_c2, contraction off) only if that one is absent."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import refio
    if refio.available("c2_stock"):
        return "c2_stock", REF_BUILD_FLAGS
    return "c2", "gcc -O2 -fopenmp -ffp-contract=off (the parity build)"


def reference_sample(updates, threads=None):
    """Times `updates` updates of the reference's own stepper (compiled from its sources,
    OpenMP on the host cores) on the workload's grid, discs, pulse and source."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import refio
    if not _REF_META:
        _package()
        from youtube_simulations_gb300 import scenes
        _REF_META.update(scenes.config2(seed=0, nx=NX, ny=NY).meta)
    m = _REF_META
    src = (m["source"][0], m["source"][1], 0.05, m["period"])
    el, _, th = refio.time_reference(reference_variant()[0], NX, NY, updates, m["discs"], m["centre"], src=src,
                                     threads=threads)
    return el, th


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, str(ROOT / "oracle"))
    import refio
    if not (refio.available("c2") or refio.available("c2_stock")):
        print(json.dumps({"impl": "reference", "unavailable": "compiled reference (oracle/_ref) absent: "
                          "run oracle/build_ref.py where the reference sources are present"}))
        return 0
    variant, flags = reference_variant()
    threads = os.cpu_count()
    upd = args.ref_updates
    _package()
    from youtube_simulations_gb300 import scenes
    m = scenes.config2(seed=0, nx=NX, ny=NY).meta
    src = (m["source"][0], m["source"][1], 0.05, m["period"])
    # one process: the reference's own set-up once, then warm-up and timed segments
    segs, _, th = refio.time_reference(variant, NX, NY, upd, m["discs"], m["centre"], src=src, threads=threads,
                                       segments=args.warmup + args.steps + 1)
    times = segs[-args.steps:] if len(segs) > args.steps else segs
    total = sum(times)
    value = CELLS * upd * len(times) / total / 1e9
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"{WORKLOAD}; step = a {upd}-update sample of the reference's stepping loop",
                       "updates_per_step": upd, "cells": CELLS, "parallelism": f"openmp x{th}"},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": th, "kind": "reference", "build": flags,
                             "sample": f"{upd} updates of the {NX}x{NY} grid per step (stepping loop only)"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# Our arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    _package()
    from youtube_simulations_gb300 import params as P
    from youtube_simulations_gb300 import scenes
    from youtube_simulations_gb300 import wavegpu as W

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    # a stream of our own (torch's default stream has handle 0, which the library
    # would read as "no stream"); torch work and the scenes are ordered on it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    # replicas: every rank advances its own instance of the workload (seed = rank)
    sc = scenes.config2(seed=rank, nx=NX, ny=NY)
    n_act = active_cells(sc.params, sc.xy)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (126 MB)

    def make_scene(prec):
        s = W.Scene(sc.params, P.FP32 if prec == "fp32" else P.FP64, P.COEF_TABLE, stream=stream.cuda_stream)
        s.upload(sc.phi, sc.psi, sc.xy, sc.tcc, sc.tc, sc.tgamma)
        if args.block and prec == "fp32":
            s.set_blocking(*args.block)
        return s

    def timed(s, steps, warmup):
        for _ in range(warmup):
            s.step(UPDATES_PER_STEP)
            s.total_energy()
        barrier()
        l0 = s.launches()
        step_ms, energy_ms = 0.0, 0.0
        energies = []
        clocks = clock_sampler(local, dev)
        clocks.start()
        wall0 = time.perf_counter()
        for _ in range(steps):
            flush.zero_()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            s.step(UPDATES_PER_STEP)
            e1.record(stream)
            energies.append(s.total_energy())
            e2.record(stream)
            e2.synchronize()
            step_ms += e0.elapsed_time(e1)
            energy_ms += e1.elapsed_time(e2)
        barrier()
        wall = time.perf_counter() - wall0
        ck = clocks.stop()
        return step_ms, energy_ms, wall, s.launches() - l0, ck, energies

    results = {}
    for prec in (["fp32", "fp64"] if not args.fp32_only else ["fp32"]):
        s = make_scene(prec)
        step_ms, energy_ms, wall, launches, ck, energies = timed(s, args.steps, args.warmup)
        k, ti, tj = s.blocking()
        s.close()
        t_ms = max_over_ranks(step_ms + energy_ms, world, dev)
        updates = args.steps * UPDATES_PER_STEP
        main_launches = args.steps * (UPDATES_PER_STEP // k if k > 1 else UPDATES_PER_STEP)
        per_launch_s = step_ms / 1e3 / main_launches
        algo = bytes_per_cell_update(prec, "table") * CELLS * max(k, 1)
        results[prec] = dict(value=whole_job_rate(world, CELLS, updates, t_ms), ms=t_ms / args.steps,
                             step_ms=step_ms, energy_ms=energy_ms, wall=wall, launches=launches, clocks=ck,
                             blocking=(k, ti, tj), achieved_gbs=algo / per_launch_s / 1e9, per_launch_s=per_launch_s,
                             bytes_per_update=bytes_per_cell_update(prec, "table"), energies=energies)
    accuracy = run_accuracy(args, P, W, sc, stream) if (rank == 0 and not args.no_accuracy) else None

    # end to end through the C ABI with page-locked host buffers (FP32): every step moves
    # the state in and out over the host link (the library's forming kernels read and
    # write these buffers in place)
    s = make_scene("fp32")
    h_phi = torch.empty(CELLS, dtype=torch.float32).pin_memory()
    h_psi = torch.empty(CELLS, dtype=torch.float32).pin_memory()
    h_phi.copy_(torch.from_numpy(sc.phi.astype("float32")))
    h_psi.copy_(torch.from_numpy(sc.psi.astype("float32")))
    lib = W.lib()
    for _ in range(max(1, args.warmup)):
        W.check(lib.wg_scene_upload_state(s.h, h_phi.data_ptr(), h_psi.data_ptr(), P.FP32))
        s.step(UPDATES_PER_STEP)
        s.total_energy()
        W.check(lib.wg_scene_download(s.h, h_phi.data_ptr(), h_psi.data_ptr(), P.FP32))
    barrier()
    e2e_ms = 0.0
    for _ in range(args.e2e_steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        W.check(lib.wg_scene_upload_state(s.h, h_phi.data_ptr(), h_psi.data_ptr(), P.FP32))
        s.step(UPDATES_PER_STEP)
        s.total_energy()
        W.check(lib.wg_scene_download(s.h, h_phi.data_ptr(), h_psi.data_ptr(), P.FP32))
        e1.record(stream)
        e1.synchronize()
        e2e_ms += e0.elapsed_time(e1)
    s.close()
    barrier()
    e2e_ms = max_over_ranks(e2e_ms, world, dev)
    e2e_value = whole_job_rate(world, CELLS, args.e2e_steps * UPDATES_PER_STEP, e2e_ms)

    batch_res = run_batch(args, P, scenes, W, stream, rank) if not args.no_batch else None
    sweep_res = run_sweep(args, P, scenes, W, stream, rank) if not args.no_sweep else None
    serve_res = run_serving(args, P, scenes, W, stream, rank) if not args.no_serving else None
    fd_res = run_frames_domain(args, P, scenes, W, stream, rank, sc) if not args.no_frames else None
    di_res = run_dropin(args, P, W, rank, sc) if not args.no_frames else None

    if rank != 0:
        return 0
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    r32, r64 = results["fp32"], results.get("fp64")
    k32, ti32, tj32 = r32["blocking"]
    kernel = ("k_step_bulk<float, TABLE> + k_step_edge" if k32 <= 1 else
              "k_step_skew<TABLE>" if tj32 == 1 else "k_step_tb<TABLE>")
    traffic, traffic_note = None, "no capture for this blocking"
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        cap = json.loads(tf.read_text())
        if cap.get("sources") != kernel_source_digest():
            traffic_note = "stale: the kernel sources changed since the ncu capture (profiles/traffic.json)"
        elif cap.get(f"fp32_k{k32}_w{tj32}"):
            traffic = cap[f"fp32_k{k32}_w{tj32}"]
            traffic_note = "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, captured on these sources"
    cpu = None
    if not args.no_cpu_baseline:
        try:
            upd = 30
            el, th = reference_sample(upd)
            if el < 3.0:
                upd = int(min(600, max(30, upd * 10.0 / max(el, 1e-3))))
                el, th = reference_sample(upd)
            cpu = {"value": CELLS * upd / el / 1e9, "unit": METRIC, "cores": th, "kind": "reference",
                   "build": reference_variant()[1], "sample": f"{upd} updates of the {NX}x{NY} grid (reference evolve_wave_half, OpenMP, stepping loop only)"}
        except Exception as exc:  # the compiled reference is absent on this machine
            cpu = {"value": None, "unit": METRIC, "cores": 0, "kind": "reference", "sample": f"unavailable: {exc}"}
    line = {
        "metric": METRIC, "value": r32["value"], "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r32["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded discs, pulse and source)",
        "config": {"workload": f"{WORKLOAD}; step = {UPDATES_PER_STEP} updates + FP64 energy report",
                   "updates_per_step": UPDATES_PER_STEP, "cells": CELLS, "parallelism": f"replicas x{world}",
                   "l2": "flushed (256 MB write) before every timed step",
                   "temporal_block": r32["blocking"][0], "tile": list(r32["blocking"][1:])},
        "roofline": {"bound": "hbm", "achieved": r32["achieved_gbs"], "peak": hbm, "unit": "GB/s",
                     "frac": r32["achieved_gbs"] / hbm, "traffic": traffic,
                     "peak_source": f"{peak_src} hbm_gbs",
                     "algorithmic_bytes_per_cell_update": r32["bytes_per_update"],
                     "cell_updates_per_launch": CELLS * max(k32, 1),
                     "definition": "single-step algorithmic bytes x cell updates per launch / mean launch time "
                                   "(CUDA events); with temporal blocking this effective rate can pass the copy peak",
                     "dram_gbs": (traffic / r32["per_launch_s"] / 1e9) if traffic else None,
                     "traffic_source": traffic_note,
                     "kernel": kernel},
        "active_cells": {"cells": n_act, "share": n_act / CELLS, "fp32_rate": r32["value"] * n_act / CELLS,
                         "definition": "cells the bulk rule updates: all when TWOSPEEDS, else xy > 0"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": 2 * CELLS * 4,
                "d2h_bytes_per_step": 2 * CELLS * 4 + 8},
        "gpu_launches": int(r32["launches"]),
        "clocks": r32["clocks"],
    }
    if r64:
        line["fp64"] = {"value": r64["value"], "ms_per_step": r64["ms"], "achieved_gbs": r64["achieved_gbs"],
                        "frac": r64["achieved_gbs"] / hbm, "temporal_block": r64["blocking"][0],
                        "gpu_launches": int(r64["launches"]), "clocks": r64["clocks"],
                        "bytes_per_cell_update": r64["bytes_per_update"]}
    line["accuracy"] = accuracy
    if batch_res:
        line["batch"] = batch_res
    if sweep_res:
        line["sweep"] = sweep_res
    if serve_res:
        line["serving"] = serve_res
    if fd_res:
        line.update(fd_res)
    if di_res:
        line["dropin"] = di_res
    print(json.dumps(line))
    return 0


ACCURACY_UPDATES, ACCURACY_REPORT = 10000, 100
FIELD_TOL32, DRIFT_TOL32, TOL64 = 1e-5, 1e-6, 1e-12


def run_accuracy(args, P, W, sc, stream):
    """The workload's full 10^4 updates, energy every 100, against the reference's own
    FP64 OpenMP stepper (compiled from its sources, oracle/_ref/bin/ref_c2) on the same
    input bytes: FP32 field error relative to the field maximum and relative energy
    difference at every report, FP64 the same; each against its stated tolerance.
    Untimed, rank 0 only."""
    import numpy as np
    sys.path.insert(0, str(ROOT / "oracle"))
    import refio
    if not refio.available("c2"):
        return {"against": "unavailable: compiled reference (oracle/_ref/bin/ref_c2) absent"}
    p = sc.params
    updates = args.accuracy_updates
    fields = dict(phi=sc.phi, psi=sc.psi, tcc=sc.tcc, tc=sc.tc, tgamma=sc.tgamma)
    t0 = time.perf_counter()
    ref = refio.run("c2", p.nx, p.ny, refio.STEP, updates, fields=fields, xy=sc.xy,
                    src=(p.src_i, p.src_j, p.src_amp, p.src_period), report=ACCURACY_REPORT, timeout=3600)
    ref_s = time.perf_counter() - t0
    out = {"against": "the reference's own FP64 OpenMP stepper (evolve_wave_half of wave_billiard.c, compiled "
                      "from its sources with FP contraction off) on the same input bytes",
           "updates": updates, "report_every": ACCURACY_REPORT, "reference_seconds": ref_s,
           "reference_threads": ref["threads"]}
    for prec, tol_f, tol_e in (("fp32", FIELD_TOL32, DRIFT_TOL32), ("fp64", TOL64, TOL64)):
        s = W.Scene(p, P.FP32 if prec == "fp32" else P.FP64, P.COEF_TABLE, stream=stream.cuda_stream)
        s.upload(sc.phi, sc.psi, sc.xy, sc.tcc, sc.tc, sc.tgamma)
        if args.block and prec == "fp32":
            s.set_blocking(*args.block)
        energies = []
        for _ in range(updates // ACCURACY_REPORT):
            s.step(ACCURACY_REPORT)
            energies.append(s.total_energy())
        phi, psi = s.download()
        s.close()
        e = np.array(energies)
        scale = float(np.max(np.abs(ref["phi"])))
        ferr = float(np.max(np.abs(phi - ref["phi"])) / scale)
        perr = float(np.max(np.abs(psi - ref["psi"])) / float(np.max(np.abs(ref["psi"]))))
        drift = np.abs(e - ref["reports"]) / np.abs(ref["reports"])
        out[prec] = {"field_rel_err": ferr, "psi_rel_err": perr,
                     "field_max_abs_err": float(np.max(np.abs(phi - ref["phi"]))),
                     "energy_rel_drift_max": float(drift.max()), "energy_rel_drift_final": float(drift[-1]),
                     "field_tol": tol_f, "energy_tol": tol_e,
                     "pass": bool(max(ferr, perr) <= tol_f and drift.max() <= tol_e)}
    out["definition"] = ("field error = max |field - reference| / max |reference| after the run; energy drift = "
                         "|E - E_ref| / |E_ref| at each report (E = sum of compute_energy over every cell)")
    return out


def tuned_blocking(b):
    """The batch autotuner's choice per size class: skewed depth and row chunk."""
    depths, rows, _ = b.skew_tuning()
    return {f"2^{c + 10}..2^{c + 11} cells": {"depth": depths[c], "chunk_rows": rows[c] or "list-wide"}
            for c in range(16) if depths[c]}


def run_batch(args, P, scenes, W, stream, rank):
    """Uneven batch: 256 seeded instances, sizes log-uniform between 256x256 and
    1280x720, ellipse/stadium/polygon/disc-array masks, Dirichlet or periodic 50/50,
    COURANT U(0.05, 0.15), one pulse each; frames of 10 updates replayed as CUDA graphs,
    3 warm-up frames and `--batch-frames` timed frames in FP32 and in FP64.  The FP64
    energy check: every instance's energy after the run, FP32 against FP64."""
    import numpy as np
    import torch
    rng = np.random.default_rng(1000 + rank)
    members = [scenes.batch_member(rng) for _ in range(args.batch_instances)]
    active = sum(active_cells(m.params, m.xy) for m in members)
    out, prec_depths, energies = {}, {}, {}
    frames = args.batch_frames
    for prec in ("fp32", "fp64"):
        b = W.Batch(P.FP32 if prec == "fp32" else P.FP64, stream=stream.cuda_stream)
        slots = [b.add(m.params, m.phi, m.psi, m.xy) for m in members]
        n_active, cells = b.count()
        for _ in range(3):
            b.step(10)
        torch.cuda.synchronize()
        l0 = b.launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(frames):
            b.step(10)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        energies[prec] = np.array([b.energy(s) for s in slots])
        out[prec] = with_active_rate({"value": cells * 10 * frames / (ms / 1e3) / 1e9, "unit": METRIC,
                                      "ms_per_frame": ms / frames, "gpu_launches": b.launches() - l0,
                                      "frames": frames}, active, cells)
        if prec == "fp32":
            prec_depths = tuned_blocking(b)
        b.close()
    out["instances"] = n_active
    out["cells"] = cells
    out["active_cells"] = active
    out["updates"] = 10 * (frames + 3)
    out["workload"] = ("uneven batch: 256 instances log-uniform 256x256..1280x720, mixed masks, Dirichlet/periodic, "
                       "frame of 10 updates as a CUDA graph: FP32 Dirichlet scenes in skewed passes at the depth tuned "
                       "per size class, the rest one persistent kernel per update over a tile work queue")
    if prec_depths:
        out["fp32"]["blocking_per_size_class"] = prec_depths
    rel = np.abs(energies["fp32"] - energies["fp64"]) / np.maximum(np.abs(energies["fp64"]), 1e-300)
    worst = int(np.argmax(rel))
    out["energy_check"] = {"against": "FP64 batch after the same updates (compensated energy sums)",
                           "max_rel_diff": float(rel.max()), "median_rel_diff": float(np.median(rel)),
                           "p90_rel_diff": float(np.quantile(rel, 0.9)),
                           "tolerance": DRIFT_TOL32, "pass": bool(rel.max() <= DRIFT_TOL32),
                           "share_within_tolerance": float(np.mean(rel <= DRIFT_TOL32)),
                           "worst": instance_card(members[worst], worst, rel[worst])}
    return out


def instance_card(m, k, err):
    """What a batch or sweep instance is: size, boundary, coefficients, and the width of
    its Gaussian pulse in cells (variance 0.05^2, so exp(-r^2/0.0025); sigma = 0.05/sqrt(2)
    in box units, dx = 4/nx)."""
    p = m.params
    return {"index": k, "nx": int(p.nx), "ny": int(p.ny), "b_cond": int(p.b_cond), "courant": float(p.courant),
            "gamma": float(p.gamma), "pulse_sigma_cells": float(0.05 / 2 ** 0.5 / ((p.xmax - p.xmin) / p.nx)),
            "error": float(err)}


def run_sweep(args, P, scenes, W, stream, rank):
    """Parameter-sweep batch: 4096 seeded instances, nx and ny log-uniform in 128..512, a
    rectangle with 1-3 circular obstacles, absorbing, GAMMA U(0, 1e-3), COURANT
    U(0.05, 0.2).  FP32 with skewed passes at the depth the autotuner picks per size
    class, 2000 updates in frames of 10 (3 warm-up frames, the rest timed); the same
    instances in FP64 give each instance's max-abs error after the 2000 updates."""
    import numpy as np
    import torch
    rng = np.random.default_rng(3000 + rank)
    members = [scenes.sweep_member(rng) for _ in range(args.sweep_instances)]
    active = sum(active_cells(m.params, m.xy) for m in members)
    frames = max(4, args.sweep_steps // 10)
    out, fields = {}, {}
    for prec in ("fp32", "fp64"):
        b = W.Batch(P.FP32 if prec == "fp32" else P.FP64, stream=stream.cuda_stream)
        slots = [b.add(m.params, m.phi, m.psi, m.xy) for m in members]
        n_active, cells = b.count()
        for _ in range(3):
            b.step(10)
        torch.cuda.synchronize()
        l0 = b.launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(frames - 3):
            b.step(10)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[prec] = with_active_rate({"value": cells * 10 * (frames - 3) / (ms / 1e3) / 1e9, "unit": METRIC,
                                      "ms_per_frame": ms / (frames - 3), "gpu_launches": b.launches() - l0},
                                     active, cells)
        if prec == "fp32":
            out["fp32"]["blocking_per_size_class"] = tuned_blocking(b)
        fields[prec] = [b.download(s)[0] for s in slots]
        b.close()
    err = np.array([np.max(np.abs(a - b)) for a, b in zip(fields["fp32"], fields["fp64"])])
    rel = np.array([np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)
                    for a, b in zip(fields["fp32"], fields["fp64"])])
    # relative to the instance's initial field maximum (the scale of the solution: the
    # absorbing edge and GAMMA up to 1e-3 drain the field, so its final maximum can be
    # far smaller than the values whose FP32 rounding the error carries)
    rel0 = np.array([e / max(np.max(np.abs(m.phi)), 1e-300) for e, m in zip(err, members)])
    worst = int(np.argmax(rel))
    out.update({"instances": n_active, "cells": cells, "active_cells": active, "updates": 10 * frames,
                "max_abs_err_vs_fp64": {"max": float(err.max()), "p50": float(np.median(err)),
                                        "p99": float(np.quantile(err, 0.99)),
                                        "max_rel_to_initial_field_max": float(rel0.max()),
                                        "max_rel_to_final_field_max": float(rel.max()),
                                        "tolerance": FIELD_TOL32,
                                        "pass": bool(rel0.max() <= FIELD_TOL32),
                                        "worst_rel_to_final": dict(instance_card(members[worst], worst, rel[worst]),
                                                                   final_field_max=float(np.max(np.abs(fields["fp64"][worst]))),
                                                                   initial_field_max=float(np.max(np.abs(members[worst].phi))))},
                "workload": f"parameter sweep: {n_active} instances, nx, ny log-uniform 128..512, rectangle with "
                            "1-3 circular obstacles, absorbing, GAMMA U(0,1e-3), COURANT U(0.05,0.2), "
                            f"{10 * frames} updates in frames of 10 (CUDA graphs), FP32 skewed passes at the "
                            "autotuned depth per size class vs FP64 single updates"})
    return out


def serve_stream(W, srv, reqs, arrivals_s):
    """Serves the requests against the wall clock: request k is submitted once
    arrivals_s[k] seconds have passed; the server ticks while anything is resident or
    queued, and otherwise waits for the next arrival.  Returns (wall seconds, max queue
    length, max resident scenes)."""
    n = len(reqs)
    k, max_q, max_res = 0, 0, 0
    t0 = time.perf_counter()
    while True:
        now = time.perf_counter() - t0
        while k < n and arrivals_s[k] <= now:
            m, frames = reqs[k]
            srv.submit(m.params, m.phi, m.psi, m.xy, frames)
            k += 1
        st = srv.stats()
        max_q, max_res = max(max_q, st["queued"]), max(max_res, st["resident"])
        if st["resident"] or st["queued"]:
            srv.tick()
        elif k < n:
            srv.drain()
            time.sleep(max(0.0, arrivals_s[k] - (time.perf_counter() - t0)))
        else:
            srv.drain()
            if srv.stats()["completed"] + srv.stats()["cancelled"] >= n:
                break
    return time.perf_counter() - t0, max_q, max_res


def run_serving(args, P, scenes, W, stream, rank):
    """Serving loop under a wall-clock load: requests with sizes log-uniform between
    256x256 and 2560x1440 and U(50, 500) frames of 10 updates each arrive as a seeded
    Poisson process at a stated rate in requests per second; the server admits them
    under an HBM budget into the running batch (pipelined ticks) and returns a turbo RGB8
    frame per scene per tick.  FP32 at each rate of --serve-rates with a 150 GB budget,
    once more at the highest rate with a budget that binds (--serve-tight-budget-gb), and
    plain FP64 at the middle rate.  A warm-up pass over the same sizes first tunes every
    size class (the tuning is kept for the process), so no measured tick tunes."""
    import numpy as np
    rng = np.random.default_rng(2000 + rank)
    lut, palette = frame_palette()
    n_req = args.serve_requests
    gaps = rng.exponential(1.0, n_req)  # unit-rate Poisson gaps, scaled per rate
    reqs = []
    for k in range(n_req):
        m = scenes.batch_member(rng, smin=(256, 256), smax=(2560, 1440))
        frames = int(rng.integers(args.serve_frames_min, args.serve_frames_max + 1))
        reqs.append((m, frames))
    rates = [float(r) for r in args.serve_rates.split(",")]

    def one(prec, rate, budget_gb):
        srv = W.Server(lut, precision=P.FP32 if prec == "fp32" else P.FP64, steps_per_frame=10,
                       hbm_budget=int(budget_gb * (1 << 30)), stream=stream.cuda_stream, pipeline=True)
        wall, max_q, max_res = serve_stream(W, srv, reqs, np.cumsum(gaps) / rate)
        st = srv.stats()
        srv.close()
        return {"offered_rps": rate, "budget_gb": budget_gb,
                "frame_latency_p50_ms": st["frame_latency_p50_ms"], "frame_latency_p99_ms": st["frame_latency_p99_ms"],
                "frame_latency_max_ms": st["frame_latency_max_ms"],
                "tick_device_p50_ms": st["tick_device_p50_ms"], "tick_device_p99_ms": st["tick_device_p99_ms"],
                "first_frame_p50_ms": st["first_frame_p50_ms"], "first_frame_p99_ms": st["first_frame_p99_ms"],
                "frames": st["frames"], "ticks": st["ticks"], "frames_per_s": st["frames"] / wall,
                "value": st["cell_updates"] / wall / 1e9, "unit": METRIC, "wall_s": wall,
                "bytes_peak": st["bytes_peak"], "max_queued": max_q, "max_resident": max_res,
                "budget_bound": bool(max_q > 0 and st["bytes_peak"] > 0.5 * budget_gb * (1 << 30))}

    # warm-up: every request size once, a few frames, so that each size class is tuned
    for prec in ("fp32",):
        srv = W.Server(lut, precision=P.FP32, steps_per_frame=10, stream=stream.cuda_stream, pipeline=True)
        for m, _ in reqs:
            srv.submit(m.params, m.phi, m.psi, m.xy, 2)
        while srv.stats()["completed"] < n_req:
            srv.tick()
            srv.drain()
        srv.close()
    runs = [one("fp32", r, 150.0) for r in rates]
    tight = one("fp32", rates[-1], args.serve_tight_budget_gb)
    fp64 = one("fp64", rates[len(rates) // 2], 150.0)
    mid = runs[len(runs) // 2]
    out = dict(mid)
    out["dtype"] = "f32"
    out["rates"] = runs
    out["budget_bound_run"] = tight
    out["fp64"] = fp64
    out["load"] = (f"{n_req} requests, Poisson arrivals in wall-clock time at {rates} requests/s, sizes log-uniform "
                   f"256x256..2560x1440, U({args.serve_frames_min},{args.serve_frames_max}) frames of 10 updates, "
                   f"150 GB budget (and {args.serve_tight_budget_gb} GB at the highest rate), pipelined ticks, "
                   "RGB8 frames (size 2) to host each tick; top-level numbers are the middle rate")
    out["latency"] = ("per frame: host enqueue of the tick that renders it to the frame in host memory (pipelined: "
                      "includes waiting behind the previous tick); tick_device: the tick's device time")
    out["palette"] = palette
    return out


PLOT_NAMES = ["amplitude", "energy", "mixed", "mean_energy", "log_energy", "log_mean_energy", "energy_flux",
              "total_energy_flux", "average_energy", "log_average_energy"]


def run_frames_domain(args, P, scenes, W, stream, rank, sc):
    """Untimed legs on the config-2 grid (rank 0): the colour-mapped frame (size 2) in every
    plot mode into device memory, device time per frame from CUDA events over repeated
    calls, and the amplitude frame copied to host memory; and the device-side mask and
    tables builder for the config's 64 discs against the host builder (numpy)."""
    if rank != 0:
        return None
    import ctypes
    import numpy as np
    import torch
    lut, lut_name = frame_palette()
    lut = np.ascontiguousarray(lut, np.uint8)
    lib = W.lib()
    p = sc.params
    size, reps = 2, 10
    s = W.Scene(p, P.FP32, P.COEF_TABLE, stream=stream.cuda_stream)
    s.upload(sc.phi, sc.psi, sc.xy, sc.tcc, sc.tc, sc.tgamma)
    s.step(200)
    pixels = (p.nx // size) * (p.ny // size)
    d_out = torch.empty(pixels * 3, dtype=torch.uint8, device=torch.device("cuda", torch.cuda.current_device()))
    h_out = np.zeros(pixels * 3, np.uint8)
    modes = {}
    for plot, name in enumerate(PLOT_NAMES):
        fp = P.WgFrameParams(size, 0, -0.2, 1.0, 1.0, 0.8, 1.0, 1.0, 0, plot, 0.75, 0.75, 250.0, 0.95, 0.0, 0, 0)
        s.frame_reset()
        call = lambda: W.check(lib.wg_scene_frame_rgb8(s.h, ctypes.byref(fp), lut.ctypes.data, None,
                                                       ctypes.c_void_p(d_out.data_ptr())))
        for _ in range(2):
            call()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            call()
        e1.record(stream)
        e1.synchronize()
        us = 1e3 * e0.elapsed_time(e1) / reps
        modes[name] = {"us_per_call": us, "mpixel_per_s": pixels / us}
    fp = P.WgFrameParams(size, 0, -0.2, 1.0, 1.0, 0.8, 1.0, 1.0, 0, P.P_AMPLITUDE, 0.75, 0.75, 250.0, 0.95, 0.0, 0, 0)
    t0 = time.perf_counter()
    for _ in range(reps):
        W.check(lib.wg_scene_frame_rgb8(s.h, ctypes.byref(fp), lut.ctypes.data, h_out.ctypes.data, None))
    host_us = 1e6 * (time.perf_counter() - t0) / reps
    s.close()
    frames = {"grid": f"{p.nx}x{p.ny}", "size": size, "pixels": pixels, "palette": lut_name, "modes": modes,
              "amplitude_to_host_us": host_us,
              "definition": "time per wg_scene_frame_rgb8 call into device memory (CUDA events over "
                            f"{reps} back-to-back calls after 2 untimed; each call ends with its stream's "
                            "synchronisation, so the host's turnaround between calls is included), FP32 fields "
                            "after 200 updates; the amplitude frame to host memory on the host clock, copy "
                            "included"}
    # the mask and tables of the config's discs: on the device, and by the host builder
    discs = np.asarray(sc.meta["discs"], np.float64)
    s = W.Scene(p, P.FP32, P.COEF_TABLE, stream=stream.cuda_stream)
    s.build_domain(scenes.D_CIRCLES, circles=discs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        s.build_domain(scenes.D_CIRCLES, circles=discs)
    torch.cuda.synchronize()
    dev_ms = 1e3 * (time.perf_counter() - t0) / 3
    same = bool(np.array_equal(s.download_mask(), sc.xy))
    s.close()
    t0 = time.perf_counter()
    xy = scenes.mask(p, scenes.D_CIRCLES, circles=sc.meta["discs"])
    scenes.tables(p, xy)
    host_ms = 1e3 * (time.perf_counter() - t0)
    domain = {"grid": f"{p.nx}x{p.ny}", "shape": f"{len(discs)} discs, two-medium tables",
              "device_ms": dev_ms, "host_builder_ms": host_ms, "mask_equals_host": same,
              "definition": "wg_scene_build_domain (mask bit planes and init_ior_2d's tables on the device; "
                            "host clock, synchronised, mean of 3 after one untimed) against scenes.mask + "
                            "scenes.tables (numpy, one thread)"}
    return {"frames": frames, "domain_build": domain}


def run_dropin(args, P, W, rank, sc):
    """Untimed leg on the config-2 grid (rank 0): the drop-in evolve_wave of
    include/wavegpu_dropin.h (FP64, the reference's operation order, its int16 mask and three
    FP64 tables, three buffers) on the reference's row-pointer fields, in resident mode (the
    fields stay in HBM between calls) and in strict mode (every call copies the fields and
    tables in and out, as a reference program calling it unchanged would).  Host clock over
    whole calls, with a device synchronisation at the end."""
    if rank != 0:
        return None
    import numpy as np
    import torch
    p = sc.params
    cells = p.nx * p.ny
    out = {"grid": f"{p.nx}x{p.ny}", "updates_per_call": 3}
    W.configure(p)
    for mode, calls in (("resident", 30), ("strict", 3)):
        W.set_mode(mode == "resident")
        rf = W.RowFields(p, sc.phi, sc.psi, np.zeros_like(sc.phi), sc.xy, sc.tcc, sc.tc, sc.tgamma)
        W.evolve_wave(rf)  # first call: uploads (resident) / warms up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(calls):
            W.evolve_wave(rf)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[mode] = {"value": cells * 3 * calls / dt / 1e9, "unit": METRIC, "calls": calls,
                     "ms_per_call": 1e3 * dt / calls}
        W.invalidate()
    W.set_mode(False)
    out["definition"] = ("evolve_wave through the drop-in C ABI (3 updates per call), fields bit-identical to the "
                         "reference's stepper; strict mode includes the host copies of phi, psi, tmp, the mask "
                         "and the three tables every call")
    return out


def frame_palette():
    """(256x3 bytes, name): the reference's turbo palette (turbo_srgb_bytes of
    turbo_colormap.c), read as data from the snapshot of the reference's sources kept
    beside the compiled reference; a seeded byte table when that is absent (the frame
    cost does not depend on the entries)."""
    import re
    import numpy as np
    src = ROOT / "oracle" / "_ref" / "src" / "turbo_colormap.c"
    if src.exists():
        m = re.search(r"turbo_srgb_bytes\s*\[256\]\s*\[3\]\s*=\s*\{(.*?)\};", src.read_text(encoding="latin-1"), re.S)
        if m:
            vals = [int(v) for v in re.findall(r"\d+", m.group(1))]
            if len(vals) == 768:
                return np.array(vals, np.uint8).reshape(256, 3), "turbo_srgb_bytes of the reference"
    return np.random.default_rng(5).integers(0, 256, size=(256, 3), dtype=np.uint8), "seeded 256x3 byte table"


def run_probe(args):
    """Small, fixed cases for kernel captures (ncu): the config-2 scene with a given
    precision and temporal blocking, stepped `--probe-updates` times, a 64-instance
    batch (FP32 or FP64 with batch64, single updates only) stepped 4 frames of 10
    updates, or 512 parameter-sweep instances (FP32, skewed passes of depth
    `--probe-block` K) stepped 4 frames of 10 updates."""
    import numpy as np
    _package()
    from youtube_simulations_gb300 import params as P
    from youtube_simulations_gb300 import scenes
    from youtube_simulations_gb300 import wavegpu as W
    if args.probe in ("batch", "batch64"):
        rng = np.random.default_rng(1000)
        b = W.Batch(P.FP32 if args.probe == "batch" else P.FP64)
        b.set_skew(0)  # single updates only: the persistent k_batch_step
        for _ in range(64):
            m = scenes.batch_member(rng)
            b.add(m.params, m.phi, m.psi, m.xy)
        for _ in range(4):
            b.step(10)
        print(json.dumps({"probe": args.probe, "instances": b.count()[0], "energy0": b.energy(0)}))
        b.close()
        return 0
    if args.probe == "sweep":
        rng = np.random.default_rng(3000)
        b = W.Batch(P.FP32)
        b.set_skew(args.probe_block[0])
        for _ in range(512):
            m = scenes.sweep_member(rng)
            b.add(m.params, m.phi, m.psi, m.xy)
        for _ in range(4):
            b.step(10)
        print(json.dumps({"probe": "sweep", "instances": b.count()[0], "cells": b.count()[1], "energy0": b.energy(0)}))
        b.close()
        return 0
    sc = scenes.config2(seed=0, nx=NX, ny=NY)
    prec = P.FP64 if args.probe == "fp64" else P.FP32
    s = W.Scene(sc.params, prec, P.COEF_TABLE)
    s.upload(sc.phi, sc.psi, sc.xy, sc.tcc, sc.tc, sc.tgamma)
    k, L, Wd = args.probe_block
    s.set_blocking(k, L if k > 1 else 0, Wd if k > 1 else 0)
    s.step(args.probe_updates)
    print(json.dumps({"probe": args.probe, "blocking": s.blocking(), "time": s.time, "energy": s.total_energy()}))
    s.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--block", type=int, nargs=3, metavar=("K", "L", "W"),
                    help="pin the FP32 temporal blocking (depth, tile rows, tile width; width 1 = skewed strips) "
                         "instead of autotuning, e.g. for kernel captures")
    ap.add_argument("--fp32-only", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-updates", type=int, default=20, help="updates per reference step")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--probe", choices=["fp32", "fp64", "batch", "batch64", "sweep"],
                    help="run a small fixed case for kernel captures")
    ap.add_argument("--probe-block", type=int, nargs=3, default=[3, 16, 256], metavar=("K", "L", "W"))
    ap.add_argument("--probe-updates", type=int, default=24)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--no-frames", action="store_true", help="skip the frame, domain-builder and drop-in legs")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--accuracy-updates", type=int, default=ACCURACY_UPDATES,
                    help="updates of the accuracy leg against the reference (a multiple of 100)")
    ap.add_argument("--sweep-instances", type=int, default=4096)
    ap.add_argument("--sweep-steps", type=int, default=2000)
    ap.add_argument("--batch-instances", type=int, default=256)
    ap.add_argument("--batch-frames", type=int, default=497)
    ap.add_argument("--serve-requests", type=int, default=32)
    ap.add_argument("--serve-rates", default="30,60,120", help="offered loads, requests per second")
    ap.add_argument("--serve-tight-budget-gb", type=float, default=0.3)
    ap.add_argument("--serve-frames-min", type=int, default=50)
    ap.add_argument("--serve-frames-max", type=int, default=500)
    args = ap.parse_args()
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.probe:
        return run_probe(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
