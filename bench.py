#!/usr/bin/env python3
"""Benchmark of the GB300 hot path: MOM5 tracer advection + split-explicit barotropic step.

One "step" = one baroclinic step of the full hot path on the workload below:
MDFL Sweby advection of every tracer with the explicit update, then
update_ocean_barotropic (predictor-corrector subcycles + time averages).

Workload (N=1): 1440x1080x50, 0.25 degree, lat -80..80, cyclic in x, 10 tracers,
MDFL Sweby + 60 barotropic subcycles, dtts = dtuv = 600 s, dtbt = 20 s; seeded
synthetic inputs.  Metric: cell-updates/s (cells x steps / s).  The other
workloads (--config) keep their own time steps: c0 120x80x30 advection at
dt = 3600 s; c1 360x300 barotropic, 80 subcycles of 67.5 s (dtuv = 2700 s).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision fp64|mixed] [--config c2|c0|c1|c2s]

--impl reference times the reference's CPU algorithm (the C restatement in
oracle/, the reference Fortran cannot be compiled on these hosts) on all host
cores: the whole workload grid, stepped by the restatement's C loop with its
scratch held across steps and its loops spread over the cores with OpenMP
(one block per process when the compiler has no OpenMP).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "cell-updates/s (1 GB300): FP64 drop-in vs batched mixed-precision; p99 latency"


class Workload:
    """A named workload: its domain, baroclinic step and barotropic subcycle.
    nts = nint(2*dtuv/dtbt) with dtuv = dtts (ocean_barotropic.F90:1109-1115)."""

    def __init__(self, name, spec_fn, dtts, dtbt=None):
        self.name, self.spec_fn, self.dtts, self.dtbt = name, spec_fn, dtts, dtbt

    @property
    def barotropic(self):
        return self.dtbt is not None

    @property
    def nts(self):
        return int(round(2.0 * self.dtts / self.dtbt)) if self.barotropic else 0

    def spec(self):
        from mom5_gb300 import grid
        return getattr(grid, self.spec_fn)()

    def describe(self, spec):
        parts = [f"{spec.ni}x{spec.nj}x{spec.nk}"]
        if spec.ntracers:
            parts.append(f"{spec.ntracers} tracers, MDFL Sweby, dtts={self.dtts:g}s")
        if self.barotropic:
            parts.append(f"{self.nts}-subcycle B-grid barotropic, dtbt={self.dtbt:g}s (dtuv={self.dtts:g}s)")
        return ", ".join(parts)


WORKLOADS = {
    "c2": Workload("c2", "config_c2", 600.0, 20.0),
    "c2s": Workload("c2s", "config_c2_block", 600.0, 20.0),
    "c2w": Workload("c2w", "config_c2_band", 600.0, 20.0),
    "c0": Workload("c0", "config_c0", 3600.0),
    "c1": Workload("c1", "config_c1", 2700.0, 67.5),
}
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
HBM_FALLBACK = 6800.0  # GB/s


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK, "fallback"


def adv_bytes(ni, nj, nk, ntr):
    """Algorithmic bytes of one fused advection step incl. the state update:
    read T and write T(taup1) per tracer, read u, v, w, rho_dzt, rho_dztr per cell,
    seven 2-D metric columns."""
    return 8 * ni * nj * nk * (2 * ntr + 5) + 8 * ni * nj * 7


# DRAM bytes per tracer-cell of the advection launch set from ncu captures: FP64, the
# 360x270x50 block (4.740 GB for 360*270*50*10 tracer-cells); precision form, the TMA-staged
# kernel (the launch shape chosen on C2) on the 1440x360x50 band, 10.3 waves (6.099 GB for
# 1440*360*50*10 tracer-cells).
TRAFFIC_PER_TRACER_CELL = {"fp64": 4.740e9 / (360 * 270 * 50 * 10), "mixed": 6.099e9 / (1440 * 360 * 50 * 10)}
TRAFFIC_SOURCE = {"fp64": "ncu DRAM bytes of the advection launch set on a 360x270x50 block, scaled by tracer-cells",
                  "mixed": "ncu DRAM bytes of the TMA-staged kernel on a 1440x360x50 band, scaled by tracer-cells"}


# FP64 thread-instructions per tracer-cell of the exact MDFL passes (z + x + y) and per
# column of one exact barotropic subcycle (momentum 29.7 + corrector with the next
# predictor 21.0 in the steady state; 50.8 averaged over a 60-subcycle step with its
# first predictor and last corrector), counted by ncu on the 360x270x50 block; the
# FP64 instruction rate of GB300 measured with a probe kernel.
FP64_OPS_PER_TRACER_CELL = 62.4
FP64_OPS_PER_COLUMN_SUBCYCLE = 50.8
FP64_PEAK_OPS = 5.05e11


def bt_bytes(ni, nj, nts):
    """Streaming bytes of the barotropic subcycles: 28 FP64 arrays per column per subcycle."""
    return 224 * ni * nj * nts


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = []
        smax = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for name, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(name)
            except Exception:
                pass
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------- CPU side (reference algorithm)
def _oracle_inputs(spec):
    """The restatement's inputs for `spec`: grid arrays, tracers and barotropic state (numpy)."""
    import numpy as np
    import torch
    from mom5_gb300 import grid
    from oracle import oracle as O
    dom = grid.make_domain(spec)
    g = O.domain_arrays(dom)
    del dom
    if spec.ntracers > 0:
        T = g.pop("T")
    else:
        T = np.zeros((0, spec.nk, spec.nj + 2, spec.ni + 2))
    st = {k: g[k].copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    return O, g, T, st


def _ref_worker(args):
    """One host process: `spec` stepped by the restatement's C loop (orc_run_steps),
    single-threaded or with OpenMP over `threads` cores.  One untimed step sizes
    the sample: then min(steps, budget_s / its time) timed steps from there on.
    Returns (seconds, cells x timed steps, timed steps)."""
    spec, wl, steps, threads, budget_s = args
    import torch
    if threads == 1:
        torch.set_num_threads(1)
    O, g, T, st = _oracle_inputs(spec)
    d = O.dims(spec)
    kw = dict(nts=wl.nts, dtbt=wl.dtbt or 0.0, threaded=threads > 1, threads=threads)
    t1, res = O.run_steps(d, g, T, wl.dtts, warmup=0, steps=1, state=st, **kw)
    if res is not None:
        st = {"eta_t": st["eta_t"], "eta_t_bar": res["eta_t_bar"], "udrho_u": res["udrho_u"],
              "udrho_v": res["udrho_v"]}
    n = max(1, min(steps, int(budget_s / max(t1, 1e-6))))
    sec, _ = O.run_steps(d, g, T, wl.dtts, warmup=0, steps=n, state=st, **kw)
    return sec, spec.ni * spec.nj * spec.nk * n, n


def _block_proc(idx, spec, wl, steps, budget_s, barrier, t1s, q):
    """One block of the per-process split: an untimed step, then the same
    number of timed steps in every process, all started together."""
    import torch
    torch.set_num_threads(1)
    O, g, T, st = _oracle_inputs(spec)
    d = O.dims(spec)
    kw = dict(nts=wl.nts, dtbt=wl.dtbt or 0.0)
    t1, res = O.run_steps(d, g, T, wl.dtts, warmup=0, steps=1, state=st, **kw)
    if res is not None:
        st = {"eta_t": st["eta_t"], "eta_t_bar": res["eta_t_bar"], "udrho_u": res["udrho_u"],
              "udrho_v": res["udrho_v"]}
    t1s[idx] = t1
    barrier.wait()
    n = max(1, min(steps, int(budget_s / max(max(t1s[:]), 1e-6))))
    barrier.wait()
    sec, _ = O.run_steps(d, g, T, wl.dtts, warmup=0, steps=n, state=st, **kw)
    q.put((sec, spec.ni * spec.nj * spec.nk * n, n))


def _block_specs(spec, procs):
    """One walled block per process (an MPI-rank-like split of the grid)."""
    import dataclasses
    px = int(round(math.sqrt(procs)))
    while procs % px:
        px -= 1
    py = procs // px
    bi, bj = max(8, spec.ni // px), max(8, spec.nj // py)
    dlon = (spec.lon1 - spec.lon0) / spec.ni
    dlat = (spec.lat1 - spec.lat0) / spec.nj
    out = []
    for b in range(procs):
        ix, iy = b % px, b // px
        lon0 = spec.lon0 + ix * bi * dlon
        lat0 = spec.lat0 + iy * bj * dlat
        out.append(dataclasses.replace(spec, ni=bi, nj=bj, lon0=lon0, lon1=lon0 + bi * dlon, lat0=lat0,
                                       lat1=lat0 + bj * dlat, cyclic_x=False, cyclic_y=False, continent=None,
                                       seed=1000 + b))
    return out


def cpu_reference(wl, spec, steps, cores, budget_s=75.0):
    """The reference algorithm on `cores` host cores, two ways, the faster one
    reported: (1) the whole grid in one process with OpenMP over rows and
    levels (the same configuration as the GPU's); (2) one walled block per
    process, as MPI ranks hold the grid, each stepped on its own (no halo
    exchange charged, so an upper bound for the decomposed reference).  The
    C loop holds its scratch across steps; timed steps are capped so that each
    way stays within about budget_s seconds."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    runs = {}
    try:
        from oracle import oracle as O
        O.build_omp()
        with ctx.Pool(1) as pool:
            sec, cells, n = pool.apply(_ref_worker, ((spec, wl, steps, cores, budget_s),))
        runs["openmp"] = {"value": cells / sec, "grid": [spec.ni, spec.nj, spec.nk], "threads": cores,
                          "steps_timed": n, "seconds": round(sec, 3), "same_config": True}
    except Exception as e:  # a compiler without OpenMP
        runs["openmp"] = {"unavailable": str(e)[:200]}
    blocks = _block_specs(spec, cores)
    barrier, t1s, q = ctx.Barrier(len(blocks)), ctx.Array("d", len(blocks)), ctx.Queue()
    procs = [ctx.Process(target=_block_proc, args=(i, b, wl, steps, budget_s, barrier, t1s, q))
             for i, b in enumerate(blocks)]
    for p in procs:
        p.start()
    res = [q.get() for _ in procs]
    for p in procs:
        p.join()
    sec = max(r[0] for r in res)
    runs["blocks"] = {"value": sum(r[1] for r in res) / sec, "block": [blocks[0].ni, blocks[0].nj, spec.nk],
                      "procs": cores, "steps_timed": res[0][2], "seconds": round(sec, 3), "same_config": False}
    best = max((k for k in runs if "value" in runs[k]), key=lambda k: runs[k]["value"])
    info = {"reported": best, "runs": {k: {q: (round(x, 1) if isinstance(x, float) else x) for q, x in r.items()}
                                       for k, r in runs.items()}}
    return runs[best]["value"], info


# --------------------------------------------------------------------------- GPU side
def _time_domain(d, stream, wl, ntr, steps, warmup, state, clock_index=0):
    """Warm up, then time `steps` whole steps of one domain on `stream` (CUDA events)."""
    import torch

    def step():
        tau = state["tau"]
        taup1 = 3 - tau
        if ntr > 0:
            d.tracer_advection_step(tau, tau, taup1, wl.dtts)
        if wl.barotropic:
            d.update_ocean_barotropic(tau, taup1)
        state["tau"] = taup1

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    d.enable_timing(True)
    launches0 = d.launches
    clocks = ClockSampler(clock_index)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    sec = {s: d.timing(s) for s in ("mdfl", "mdfl_mixed", "tracer_update", "barotropic")}
    d.enable_timing(False)
    return {"ms": ms, "sec": sec, "launches": d.launches - launches0, "clocks": clk, "step": step}


def _fp64_roofline(prec, sec, steps, cells, ntr, ni, nj, nts):
    """The FP64-pipe roofline of the exact path (the bound of the drop-in)."""
    from mom5_gb300 import capi
    if prec != capi.PRECISION_FP64 or ntr == 0 or sec["mdfl"][0] <= 0:
        return None
    mdfl_s = sec["mdfl"][0] / steps / 1e3
    bt_s = sec["barotropic"][0] / steps / 1e3
    a = FP64_OPS_PER_TRACER_CELL * cells * ntr / mdfl_s
    b = FP64_OPS_PER_COLUMN_SUBCYCLE * (ni + 2) * (nj + 2) * nts / bt_s if bt_s > 0 else 0.0
    return {"bound": "fp64 pipe", "unit": "FP64 instructions/s", "peak": FP64_PEAK_OPS,
            "peak_source": "probe kernel on this pool (FP64 FMA rate)",
            "mdfl": {"achieved": round(a, -6), "frac": round(a / FP64_PEAK_OPS, 3),
                     "ops_per_tracer_cell": FP64_OPS_PER_TRACER_CELL},
            "barotropic": {"achieved": round(b, -6), "frac": round(b / FP64_PEAK_OPS, 3),
                           "ops_per_column_subcycle": FP64_OPS_PER_COLUMN_SUBCYCLE},
            "source": "FP64 instruction counts per tracer-cell and per column-subcycle from ncu on a "
                      "360x270x50 block"}


def max_over_ranks(ms: float, device) -> float:
    """The slowest rank's time (each rank steps its own replica of the workload)."""
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.barrier()
    return float(t.item())


def whole_job_rate(cells: int, world: int, steps: int, ms: float) -> float:
    """Cell-updates per second of the whole job: every rank advances `cells` cells
    per step (replicas, weak scaling), timed by the slowest rank."""
    return cells * world * steps / (ms / 1e3)


def _device_copy(d, fid, n, level):
    """A field of a library domain copied into a new CUDA tensor (device to device)."""
    import torch
    from mom5_gb300 import capi
    t = torch.empty(d.count(fid), dtype=torch.float64, device="cuda")
    d.check(capi.lib().mom5gpu_get_field(d.h, fid, n, level, capi.C.c_void_p(t.data_ptr()), 1))
    d.synchronize()
    return t


def _rel_err(a, b):
    """max|a - b| / max|b| (b the FP64 result)."""
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))


def run_e2e(d, stream, wl, ntr, steps, warm=3):
    """End to end through the C ABI with host buffers: every step uploads its
    inputs from pinned host memory (tracers and advection velocity; the
    barotropic forcing) and reads its results back (tracers; eta_t_bar, udrho),
    stream-ordered copies (mom5gpu_copy_field_async) ordered by events.

    Three time levels rotate, so the tracer level a step reads is the one the
    step two before wrote: its tracers are uploaded straight into that level
    (mom5gpu_copy_field_async, host to device), each as soon as that step's
    read-back of the same tracer is done, during the previous step's compute.  The velocity and the
    forcing have one copy each in the library, busy until the previous step's
    advection or barotropic step ends: they are uploaded into device staging
    buffers early and moved into their fields by a staging stream
    (mom5gpu_copy_boxes, a kernel, so the copy engines stay with the host link)
    once the field is free.  `warm` untimed steps first (first-touch
    allocations, graph captures); the timed steps are timed on the host wall
    clock and each stream's work by CUDA events."""
    import numpy as np
    import torch
    from mom5_gb300 import capi
    from mom5_gb300.capi import F
    pin = lambda n: torch.empty(n, dtype=torch.float64, pin_memory=True)
    dev = lambda n: torch.empty(n, dtype=torch.float64, device="cuda")
    n3, nw = d.count(F.TRACER), d.count(F.WRHO_BT)
    n2 = d.count(F.ETA_T_BAR)
    ups = []    # staged: (field, n, host buffer, device staging buffer, when the field is free: "adv", "step")
    direct = []  # straight into the field's time level: (field, n, host buffer)
    downs = []  # (field, n, host buffer)
    if ntr > 0:
        for n in range(1, ntr + 1):
            h = pin(n3)
            h.copy_(torch.from_numpy(d.get(F.TRACER, n=n, level=1)))
            direct.append((F.TRACER, n, h))
            downs.append((F.TRACER, n, pin(n3)))
        for fid, cnt in ((F.UHRHO_ET, n3), (F.VHRHO_NT, n3), (F.WRHO_BT, nw)):
            h = pin(cnt)
            h.copy_(torch.from_numpy(d.get(fid)))
            ups.append((fid, 0, h, dev(cnt), "adv"))
        d.set(F.RHO_DZT, d.get(F.RHO_DZT, level=1), level=3)  # the third level of the rotation
    if wl.barotropic:
        for fid in (F.FORCING_BT_U, F.FORCING_BT_V):
            h = pin(n2)
            h.copy_(torch.from_numpy(d.get(fid)))
            ups.append((fid, 0, h, dev(n2), "step"))
        for fid in (F.ETA_T_BAR, F.UDRHO_U, F.UDRHO_V):
            downs.append((fid, 0, pin(n2)))
        for fid in (F.THICKU, F.ETA_T_BAR, F.UDRHO_U, F.UDRHO_V, F.CONV_RHO_UD_T):
            d.set(fid, d.get(fid, level=1), level=3)
    h2d, stg, d2h = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    total = warm + steps
    tev = lambda: torch.cuda.Event(enable_timing=True)
    names = ("up0", "ups1", "upt0", "up1", "stg1", "c0", "adv", "c1", "d2h0", "d2h1")
    ev = {k: [tev() for _ in range(total)] for k in names}
    tr_done = []  # per step: tracer n -> event after its read-back
    torch.cuda.synchronize()
    t0 = None
    for s_ in range(total):
        if s_ == warm:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
        lin, lout = (1, 2, 3)[(2 * s_) % 3], (1, 2, 3)[(2 * s_ + 1) % 3]
        # host -> staging, once the previous step's staging copies have read the buffers
        if s_ >= 1:
            h2d.wait_event(ev["stg1"][s_ - 1])
        ev["up0"][s_].record(h2d)
        with torch.cuda.stream(h2d):
            for _, _, h, buf, _ in ups:
                buf.copy_(h, non_blocking=True)
        ev["ups1"][s_].record(h2d)
        # host -> tracer level lin, each tracer once its read-back by the step
        # that wrote the level is done (the two directions of the link overlap)
        ev["upt0"][s_].record(h2d)
        for fid, n, h in direct:
            if s_ >= 2:
                h2d.wait_event(tr_done[s_ - 2][n])
            d.copy_field_async(fid, h.data_ptr(), 1, h2d.cuda_stream, n=n, level=lin)
        ev["up1"][s_].record(h2d)
        # staging -> fields, each once its field is free, by the library's box copy
        # (a kernel: the copy engines are busy with the host link)
        for when, after in (("adv", "adv"), ("step", "c1")):
            if s_ >= 1:
                stg.wait_event(ev[after][s_ - 1])
            boxes = []
            for fid, n, _, buf, w in ups:
                if w == when:
                    boxes.append(capi.Box(buf.data_ptr(), d.device_ptr(fid), (1, buf.numel(), buf.numel()),
                                          (1, buf.numel(), buf.numel()), (buf.numel(), 1, 1)))
            if boxes:
                stg.wait_event(ev["ups1"][s_])
                capi.copy_boxes(boxes, stg.cuda_stream)
        ev["stg1"][s_].record(stg)
        stream.wait_event(ev["stg1"][s_])
        stream.wait_event(ev["up1"][s_])
        ev["c0"][s_].record(stream)
        if ntr > 0:
            d.tracer_advection_step(lin, lin, lout, wl.dtts)
        ev["adv"][s_].record(stream)
        if wl.barotropic:
            d.update_ocean_barotropic(lin, lout)
        ev["c1"][s_].record(stream)
        d2h.wait_event(ev["c1"][s_])
        ev["d2h0"][s_].record(d2h)
        tr_done.append({})
        for fid, n, h in downs:
            d.copy_field_async(fid, h.data_ptr(), 0, d2h.cuda_stream, n=n, level=lout)
            if fid == F.TRACER:
                tr_done[s_][n] = torch.cuda.Event()
                tr_done[s_][n].record(d2h)
        ev["d2h1"][s_].record(d2h)
    torch.cuda.synchronize()
    te = (time.perf_counter() - t0) / steps
    rng = range(warm, total)
    mean = lambda a, b: float(np.mean([ev[a][s].elapsed_time(ev[b][s]) for s in rng]))
    wait = float(np.mean([ev["c1"][s - 1].elapsed_time(ev["c0"][s]) for s in rng]))
    span = ev["c0"][warm].elapsed_time(ev["c1"][total - 1]) / steps
    hb = 8 * (sum(h.numel() for _, _, h, _, _ in ups) + sum(h.numel() for _, _, h in direct))
    db = 8 * sum(h.numel() for _, _, h in downs)
    up, rb = mean("up0", "ups1") + mean("upt0", "up1"), mean("d2h0", "d2h1")
    timeline = {"unit": "ms per step (means over the timed steps, CUDA events)",
                "host_wall": round(te * 1e3, 3), "compute_span": round(span, 3), "compute": round(mean("c0", "c1"), 3),
                "upload": round(up, 3), "readback": round(rb, 3), "staging_to_fields": round(mean("ups1", "stg1"), 3),
                "compute_waits_for_inputs": round(wait, 3),
                "upload_GBps": round(hb / up / 1e6, 1) if up > 0 else None,  # a lower bound: the tracer
                # uploads' span includes their waits for the read-back of each tracer
                "readback_GBps": round(db / rb / 1e6, 1) if rb > 0 else None}
    return te, hb, db, timeline


def run_ours(args, rank, world):
    import torch

    from mom5_gb300 import build, capi, grid, harness

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    build.build()
    wl = WORKLOADS[args.config]
    spec = wl.spec()
    prec = capi.PRECISION_MIXED if args.precision == "mixed" else capi.PRECISION_FP64
    headline = args.scheme == "mdfl_sweby"
    forms = (not args.no_forms) and world == 1 and prec == capi.PRECISION_FP64 and args.config == "c2" and headline
    dom = grid.make_domain(spec, device="cuda")
    opts = capi.default_options(barotropic_time_stepping_B=1, precision=prec)
    d = harness.load(dom, options=opts)
    if not headline:
        sid = getattr(capi, dict(SCHEMES)[args.scheme])
        for n in range(1, spec.ntracers + 1):
            d.set_tracer_scheme(n, sid, sid, -1.0e10, 1.0e10)
            d.set_psom_limit(n, True)
    nts = d.barotropic_init(dtuv=wl.dtts, dtbt=wl.dtbt) if wl.barotropic else 0
    assert nts == wl.nts
    ni, nj, nk, ntr = spec.ni, spec.nj, spec.nk, spec.ntracers
    cells = ni * nj * nk
    if not forms:
        del dom
    torch.cuda.empty_cache()
    # a dedicated stream: the legacy default stream's handle is 0, which the C ABI
    # reads as "the domain's own stream"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    d.set_stream(stream.cuda_stream)

    state = {"tau": 1}
    # trial steps 1 -> 2; the timed steps start at level 1
    if args.tuning:
        d.tuning = tuple(int(x) for x in args.tuning.split(","))
        tune = f"pinned {args.tuning}"
    else:
        tune = d.autotune(wl.dtts) if ntr > 0 and not args.no_autotune else None
    if world > 1:
        torch.distributed.barrier()
    r = _time_domain(d, stream, wl, ntr, args.steps, args.warmup, state, local)
    ms, sec, launches, clk = r["ms"], r["sec"], r["launches"], r["clocks"]
    if world > 1:
        ms = max_over_ranks(ms, "cuda")
    ms_step = ms / args.steps
    value = whole_job_rate(cells, world, args.steps, ms)

    # dominant kernel group: the advection step (MDFL passes + explicit update)
    adv_ms = sec["mdfl"][0] + sec["mdfl_mixed"][0] + sec["tracer_update"][0]
    adv_calls = max(1, max(sec["mdfl"][1], sec["mdfl_mixed"][1]))
    peak, peak_kind = hbm_peak()
    bt_ms = sec["barotropic"][0] / max(1, sec["barotropic"][1])
    bt_roof = None
    if wl.barotropic and bt_ms > 0:
        bt_achieved = bt_bytes(ni, nj, nts) / (bt_ms / 1e3) / 1e9
        bt_roof = {"achieved": round(bt_achieved, 1), "unit": "GB/s", "peak": peak,
                   "frac": round(bt_achieved / peak, 4), "note": "streaming model, 224 B/column/subcycle"}
    if ntr > 0:
        bytes_adv = adv_bytes(ni, nj, nk, ntr)
        per = adv_ms / adv_calls
        achieved = bytes_adv / (per / 1e3) / 1e9
        roofline = {"bound": "hbm", "kernel": f"tracer advection step ({args.scheme} + explicit update)",
                    "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                    "algorithmic_bytes_per_launch": bytes_adv, "ms_per_launch": round(per, 3),
                    "traffic": round(TRAFFIC_PER_TRACER_CELL[args.precision] * cells * ntr) if headline else None,
                    "traffic_source": TRAFFIC_SOURCE[args.precision]}
    elif bt_roof is not None:
        roofline = dict(bt_roof, bound="hbm", kernel="barotropic subcycle loop (streaming model)",
                        peak_source=peak_kind, algorithmic_bytes_per_launch=bt_bytes(ni, nj, nts),
                        ms_per_launch=round(bt_ms, 3), traffic=None)
    else:
        roofline = None

    e2e = None
    if not args.no_e2e:
        # at least 30 steps: the first step's upload and the last one's read-back, which
        # nothing can overlap, are spread over a run of steps as in a simulation
        e2e_steps = min(max(args.steps, 30), 100)
        te, hb, db, timeline = run_e2e(d, stream, wl, ntr, e2e_steps)
        e2e = {"value": round(cells / te, 1), "unit": "cell-updates/s", "h2d_bytes_per_step": hb,
               "d2h_bytes_per_step": db, "steps": e2e_steps,
               "api": "mom5gpu_copy_field_async (pinned host buffers: tracers host->time level on an upload "
                      "stream, results device->host on a read-back stream), velocity and forcing host->staging "
                      "then mom5gpu_copy_boxes (staging->fields) / mom5gpu_tracer_advection_step / "
                      "mom5gpu_update_ocean_barotropic",
               "timing": "host wall clock over the steps, every copy inside; a step's tracers go straight into "
                         "the time level it reads (three rotate) once that level's read-back is done, during the "
                         "previous step's compute; velocity and forcing land in staging buffers and are copied "
                         "into their fields once the previous step is done with them", "timeline": timeline}

    l2note = ("inputs larger than L2 (tracer state alone %.1f GB)" % (2 * ntr * cells * 8 / 1e9)
              if 2 * ntr * cells * 8 > 129e6 else "inputs smaller than L2, not flushed (launch/latency-bound case)")
    out = {"metric": METRIC, "value": round(value, 1), "unit": "cell-updates/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == capi.PRECISION_FP64 else "f32+f64",
           "data": "synthetic (seeded streamfunction flow, partial-cell bathymetry)",
           "config": {"workload": f"{args.config.upper()}: {wl.describe(spec)}"
                                  + ("" if headline else f" ({args.scheme} for every tracer)")
                                  + (", FP64 drop-in" if prec == capi.PRECISION_FP64 else ", precision form"),
                      "cells": cells, "tracers": ntr, "subcycles": nts, "dtts": wl.dtts, "dtbt": wl.dtbt,
                      "parallelism": f"replicas x{world}", "l2": l2note},
           "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "autotune": tune,
           "sections_ms_per_step": {k: round(v[0] / args.steps, 3) for k, v in sec.items()},
           "barotropic_roofline": bt_roof,
           "fp64_roofline": _fp64_roofline(prec, sec, args.steps, cells, ntr, ni, nj, nts) if headline else None,
           "clocks": clk}
    if rank == 0 and not args.no_cpu_baseline:
        # bounded sample of the same workload on one host core
        v, info = _cpu_sample(wl, spec)
        out["cpu_baseline"] = {"value": round(v, 1), "unit": "cell-updates/s", "cores": 1, "kind": "port",
                               "sample": info}
    if forms:
        out["forms"] = run_forms(args, wl, dom, d, value, stream)
    return out


# --------------------------------------------------------------------------- the three forms
FORM_DT = 400.0     # baroclinic step of the ensemble and serving domains (s)
FORM_DTBT = 20.0    # barotropic step: nts = 2 * 400 / 20 = 40 subcycles


def run_forms(args, wl, dom, d64, plain_value, stream):
    """Precision form on the same 1440x1080x50 domain, then the batched ensemble
    (64 domains) and the serving loop (256 resident domains)."""
    import torch

    from mom5_gb300 import capi, harness
    from mom5_gb300.capi import F
    spec = dom.spec
    ntr = spec.ntracers
    cells = spec.ni * spec.nj * spec.nk
    forms = {}
    # ---- precision form, same workload
    dm = harness.load(dom, options=capi.default_options(barotropic_time_stepping_B=1, precision=capi.PRECISION_MIXED))
    dm.barotropic_init(dtuv=wl.dtts, dtbt=wl.dtbt)
    dm.set_stream(stream.cuda_stream)
    tune = dm.autotune(wl.dtts)
    r = _time_domain(dm, stream, wl, ntr, args.steps, args.warmup, {"tau": 1})
    v = cells * args.steps / (r["ms"] / 1e3)
    # error against the FP64 drop-in (equal to the oracle bit for bit), one step from the same state
    errs, drift64, driftm = [], 0.0, 0.0
    for n in range(1, ntr + 1):
        d64.set(F.TRACER, dom["T"][n - 1].contiguous(), n=n, level=1)
        dm.set(F.TRACER, dom["T"][n - 1].contiguous(), n=n, level=1)
    c0 = [d64.global_tracer_content(n, 1) for n in range(1, ntr + 1)]
    d64.tracer_advection_step(1, 1, 2, wl.dtts)
    dm.tracer_advection_step(1, 1, 2, wl.dtts)
    for n in range(1, ntr + 1):
        errs.append(_rel_err(_device_copy(dm, F.TRACER, n, 2), _device_copy(d64, F.TRACER, n, 2)))
        drift64 = max(drift64, abs(d64.global_tracer_content(n, 2) - c0[n - 1]) / abs(c0[n - 1]))
        driftm = max(driftm, abs(dm.global_tracer_content(n, 2) - c0[n - 1]) / abs(c0[n - 1]))
    forms["precision"] = {
        "workload": "same as the headline, precision form (FP32 fluxes and limiters, FP64 state, subcycle, sums)",
        "value": round(v, 1), "unit": "cell-updates/s", "ms_per_step": round(r["ms"] / args.steps, 3),
        "vs_plain": round(v / plain_value, 3),
        "sections_ms_per_step": {k: round(x[0] / args.steps, 3) for k, x in r["sec"].items()},
        "max_rel_err_vs_fp64_1step": max(errs), "content_rel_change_1step": {"fp64": drift64, "precision": driftm},
        "gpu_launches": r["launches"], "clocks": r["clocks"], "autotune": tune}
    dm.close()
    forms["schemes"] = scheme_sweep(d64, stream, ntr, cells, wl.dtts)
    d64.close()
    del dom
    torch.cuda.empty_cache()
    # ---- batched ensemble and serving
    forms["batched"] = form_batched(args, stream)
    forms["serving"] = form_serving(args, stream, forms["batched"])
    return forms


SCHEMES = (("upwind", "ADVECT_UPWIND"), ("2nd_order", "ADVECT_2ND_ORDER"), ("4th_order", "ADVECT_4TH_ORDER"),
           ("6th_order", "ADVECT_6TH_ORDER"), ("quicker", "ADVECT_QUICKER"), ("mdfl_sup_b", "ADVECT_MDFL_SUP_B"),
           ("mdppm", "ADVECT_MDPPM"), ("psom", "ADVECT_PSOM"), ("mdfl_sweby", "ADVECT_MDFL_SWEBY"))


def scheme_sweep(d, stream, ntr, cells, dtts, steps=2):
    """FP64 tracer advection step (every tracer on one scheme, explicit update
    included, no barotropic) for each scheme on the headline domain."""
    import torch

    from mom5_gb300 import capi
    out = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for name, const in SCHEMES:
        sid = getattr(capi, const)
        for n in range(1, ntr + 1):
            d.set_tracer_scheme(n, sid, sid, -1.0e10, 1.0e10)
            if name == "psom":
                d.set_psom_limit(n, True)
        launches0 = d.launches
        d.tracer_advection_step(1, 1, 2, dtts)  # warm-up (allocates the scheme's fields)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            d.tracer_advection_step(1, 1, 2, dtts)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[name] = {"ms_per_step": round(ms, 3), "cell_updates_per_s": round(cells / (ms / 1e3), 1),
                     "launches_per_step": (d.launches - launches0) // (steps + 1)}
    for n in range(1, ntr + 1):
        d.set_tracer_scheme(n, capi.ADVECT_MDFL_SWEBY, capi.ADVECT_MDFL_SWEBY, -1.0e10, 1.0e10)
    return {"workload": "headline domain, every tracer on one scheme, FP64 drop-in, advection + explicit update "
                        "(no barotropic), from the same state each step; psom with the Merryfield-Holloway limiter",
            "steps": steps, "schemes": out}


def _load_set(specs, precisions):
    """Generate each domain once and load it once per precision."""
    from mom5_gb300 import capi, grid, harness
    sets = {p: [] for p in precisions}
    for s in specs:
        dom = grid.make_domain(s, device="cuda")
        for p in precisions:
            d = harness.load(dom, options=capi.default_options(barotropic_time_stepping_B=1, precision=p))
            d.barotropic_init(dtuv=FORM_DT, dtbt=FORM_DTBT)
            sets[p].append(d)
        del dom
    return sets


def form_batched(args, stream):
    import torch

    from mom5_gb300 import capi, serving
    from mom5_gb300.capi import F
    specs = serving.ensemble_specs(64)
    cells = sum(s.ni * s.nj * s.nk for s in specs)
    ntr = specs[0].ntracers
    P64, PM = capi.PRECISION_FP64, capi.PRECISION_MIXED
    sets = _load_set(specs, (P64, PM))
    for p in sets:
        for d in sets[p]:
            d.set_stream(stream.cuda_stream)
    out = {"workload": f"64 regional domains, nx,ny log-uniform in [64,512], nz in [20,50], {ntr} tracers, "
                       f"MDFL Sweby + {int(2 * FORM_DT / FORM_DTBT)}-subcycle barotropic, dt={FORM_DT:g}s",
           "cells": cells}
    batches = {p: capi.Batch(sets[p]) for p in sets}
    for b in batches.values():
        b.set_stream(stream.cuda_stream)
    # one step of both from the same state: error of the precision form
    for b in batches.values():
        b.step(FORM_DT, index=list(range(len(specs))), parity=[0] * len(specs))
    err = 0.0
    for i in range(len(specs)):
        for n in range(1, ntr + 1):
            err = max(err, _rel_err(_device_copy(sets[PM][i], F.TRACER, n, 2), _device_copy(sets[P64][i], F.TRACER, n, 2)))
    out["precision_max_rel_err_vs_fp64_1step"] = err
    for p, name in ((P64, "fp64"), (PM, "precision")):
        b = batches[p]
        report = b.autotune(FORM_DT)  # parity-0 trials: level 2 rewritten from level 1
        par = 1
        for _ in range(args.warmup):
            b.step(FORM_DT, parity=par)
            par ^= 1
        torch.cuda.synchronize()
        l0 = b.launches
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            b.step(FORM_DT, parity=par)
            par ^= 1
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        # the same step as plain per-domain launches, one domain after another
        tau = 1 + par
        per = []
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(specs) + 1)]
        ev[0].record(stream)
        for i, d in enumerate(sets[p]):
            d.tracer_advection_step(tau, tau, 3 - tau, FORM_DT)
            d.update_ocean_barotropic(tau, 3 - tau)
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
        per = [ev[i].elapsed_time(ev[i + 1]) for i in range(len(specs))]
        loop_ms = ev[0].elapsed_time(ev[-1])
        out[name] = {"value": round(cells / (ms / 1e3), 1), "unit": "cell-updates/s", "ms_per_step": round(ms, 3),
                     "launches_per_step": (b.launches - l0) // args.steps, "autotune": report,
                     "per_domain_launches": {"value": round(cells / (loop_ms / 1e3), 1), "ms_per_step": round(loop_ms, 3),
                                             "p50_ms": round(float(sorted(per)[len(per) // 2]), 3),
                                             "p99_ms": round(float(sorted(per)[min(len(per) - 1, int(0.99 * len(per)))]), 3)}}
        out[name]["tuning"] = list(b.tuning)
    out["precision_vs_fp64"] = round(out["precision"]["value"] / out["fp64"]["value"], 3)
    for b in batches.values():
        b.close()
    for p in sets:
        for d in sets[p]:
            d.close()
    torch.cuda.empty_cache()
    return out


def form_serving(args, stream, batched):
    import numpy as np
    import torch

    from mom5_gb300 import capi, grid, harness, serving
    ndom = 256
    specs = serving.ensemble_specs(ndom, seed=1)
    srv = serving.Server(FORM_DT, precision=capi.PRECISION_MIXED, slots=3, max_batch=64)

    def load(dom):
        d = harness.load(dom, options=capi.default_options(barotropic_time_stepping_B=1,
                                                           precision=capi.PRECISION_MIXED))
        d.barotropic_init(dtuv=FORM_DT, dtbt=FORM_DTBT)
        return d

    refused = 0
    for s in specs:
        try:
            srv.add_domain(grid.make_domain(s, device="cuda"), load)
        except serving.AdmissionError:
            refused += 1
    torch.cuda.empty_cache()
    srv.start()
    srv.slots[0].batch.autotune(FORM_DT)
    for s in srv.slots[1:]:
        s.batch.tuning = srv.slots[0].batch.tuning
    torch.cuda.synchronize()
    mean_cells = float(np.mean(srv.cells))
    cap = batched["precision"]["value"] / mean_cells  # requests/s the batched kernels sustain
    rng = np.random.default_rng(5)
    runs = []
    srv.run([0.0] * 64, list(rng.integers(0, len(srv.domains), 64)))  # warm-up
    for frac in (0.3, 0.6, 0.9):
        rate = frac * cap
        n = int(min(3000, max(200, rate * 2.5)))
        arr = serving.poisson_arrivals(rate, n, seed=int(frac * 100))
        res = srv.run(arr, list(rng.integers(0, len(srv.domains), n)))
        res["offered_rps"] = round(rate, 1)
        runs.append(res)
    n = 1024
    sat = srv.run([0.0] * n, list(rng.integers(0, len(srv.domains), n)))
    sat["offered_rps"] = "all at t=0"
    runs.append(sat)
    srv.close()
    for d in srv.domains:
        d.close()
    torch.cuda.empty_cache()
    plain = batched["fp64"]["per_domain_launches"]
    rnd = lambda r: {k: (round(v, 3) if isinstance(v, float) else v) for k, v in r.items()}
    return {"workload": f"{ndom} resident domains (sizes as the ensemble), step = advection + "
                        f"{int(2 * FORM_DT / FORM_DTBT)} subcycles, Poisson arrivals, precision form, "
                        f"3 overlapping batch slots, size buckets", "resident": len(srv.domains),
            "refused_by_admission": refused, "resident_cells": int(sum(srv.cells)),
            "runs": [rnd(r) for r in runs],
            "saturation_cell_updates_per_s": round(sat["cell_updates_per_s"], 1),
            "plain_fp64_per_domain": {"cell_updates_per_s": plain["value"], "p50_ms": plain["p50_ms"],
                                      "p99_ms": plain["p99_ms"],
                                      "note": "ensemble domains stepped one at a time through the one-domain "
                                              "FP64 entry points (service time, no queueing)"},
            "vs_plain_fp64": round(sat["cell_updates_per_s"] / plain["value"], 3)}


def _cpu_sample(wl, spec):
    """One host core on a bounded sample of the workload: one walled block of
    1/16 of its grid, one untimed and three timed steps of the restatement's
    C loop (about 15 s for the global config)."""
    blk = _block_specs(spec, 16)[0]
    sec, cells, _ = _ref_worker((blk, wl, 3, 1, 1e9))
    return cells / sec, (f"C restatement, 1 core, {blk.ni}x{blk.nj}x{blk.nk} block of the grid, "
                         f"{spec.ntracers} tracers, 3 steps ({wl.describe(blk)})")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--config", choices=sorted(WORKLOADS), default="c2")
    ap.add_argument("--scheme", choices=[n for n, _ in SCHEMES], default="mdfl_sweby",
                    help="advection scheme of every tracer (the headline is mdfl_sweby)")
    ap.add_argument("--metrics-jsonl", default=None, help="also append the figures to this JSON-lines file")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes (profiling runs)")
    ap.add_argument("--tuning", default=None,
                    help="pin the launch shape ROWS,PREFETCH,TJ (mom5gpu_set_tuning) instead of autotuning")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the precision, batched and serving forms reported beside the FP64 headline")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference":
        if rank != 0:
            return
        wl = WORKLOADS[args.config]
        spec = wl.spec()
        cores = os.cpu_count() or 1
        v, info = cpu_reference(wl, spec, args.steps, cores)
        r = info["runs"][info["reported"]]
        how = (f"whole grid, OpenMP on {cores} threads" if info["reported"] == "openmp"
               else f"{cores} processes x walled block {r['block']}")
        out = {"metric": METRIC, "value": round(v, 1), "unit": "cell-updates/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": round(1e3 * r["seconds"] / max(1, r["steps_timed"]), 3),
               "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
               "config": {"workload": f"{args.config.upper()}: {wl.describe(spec)}, reference algorithm on the "
                                      f"host cores (the faster of: whole grid with OpenMP; one walled block per "
                                      f"process)", "sample": info, "same_config": r["same_config"]},
               "cpu_baseline": {"value": round(v, 1), "unit": "cell-updates/s", "cores": cores, "kind": "port",
                                "sample": f"C restatement stepping loop, {how}, {r['steps_timed']} timed steps "
                                          f"after one untimed step"},
               "e2e": {"value": round(v, 1), "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                       "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    out = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(out))
        if args.metrics_jsonl:
            from mom5_gb300 import metrics
            metrics.from_bench_line(out, metrics.MetricsLog(args.metrics_jsonl))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
