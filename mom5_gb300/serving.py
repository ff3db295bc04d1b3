"""Serving form: a continuous-batching loop of step requests over resident domains.

A request asks for one baroclinic step (MDFL advection of every tracer with the
explicit update, then the barotropic subcycles) of one resident domain.  The
server keeps every domain's state on the device and never copies it back.

* Admission: a domain is admitted (created and loaded) only while the device's
  free memory minus a reserve covers its estimated footprint; otherwise
  ``add_domain`` raises ``AdmissionError`` (the C ABI's MOM5GPU_EFULL).
* Continuous batching: waiting requests are grouped by domain-size bucket
  (log2 of the cell count); whenever one of ``slots`` batch objects is free, the
  bucket with the oldest waiting request is launched as one batched step, on that
  slot's own CUDA stream, while earlier batches are still running.  A domain is
  in at most one batch at a time; requests for a busy domain wait.
* Completion is detected with CUDA events; a request's latency runs from its
  arrival to the moment the host sees its batch complete.
* Failures are contained on the host: a request for a domain that does not exist
  or is quarantined is rejected at arrival; a batched step that the library
  refuses (a non-zero status) fails the requests of that batch, quarantines their
  domains and leaves every other domain serving; with ``check_every`` > 0 the
  state of a domain is checked for non-finite values after every ``check_every``
  of its steps, and a domain that fails the check is quarantined.

All kernels come from libmom5gpu.so through the batch API
(``mom5gpu_batch_step``); this module only schedules.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import capi


class AdmissionError(RuntimeError):
    """Not enough free device memory to admit a domain."""


@dataclass
class Request:
    rid: int
    domain: int
    arrival: float
    start: float = 0.0
    done: float = 0.0
    status: str = "ok"  # ok | failed | rejected
    error: str = ""


@dataclass
class Slot:
    batch: "capi.Batch"
    stream: object
    event: object = None
    requests: List[Request] = field(default_factory=list)


def bytes_per_domain(ni, nj, nk, ntr, precision) -> int:
    """Device footprint of one domain as the library allocates it."""
    n2 = (ni + 2) * (nj + 2)
    n3 = n2 * nk
    f3 = 2 * ntr + ntr + 6  # tracers at 2 levels, th_tendency, tmask/u/v/w/rho_dzt x2/rho_dztr
    if precision == capi.PRECISION_FP64:
        f3 += 2 * ntr  # MDFL scratch
    f2 = 61  # metrics, barotropic state and scratch
    return 8 * (f3 * n3 + f2 * n2) + (ni + 4) * (nj + 4) * nk


class Server:
    def __init__(self, dtime: float, precision=capi.PRECISION_MIXED, slots: int = 3, max_batch: int = 64,
                 reserve_bytes: int = 8 << 30, memory_limit: Optional[int] = None, check_every: int = 0):
        import torch
        self.torch = torch
        self.dtime = dtime
        self.precision = precision
        self.nslots = slots
        self.max_batch = max_batch
        self.reserve = reserve_bytes
        self.memory_limit = memory_limit  # optional cap below the device's free memory (tests)
        self.domains: List[capi.Domain] = []
        self.cells: List[int] = []
        self.parity: List[int] = []
        self.busy: List[bool] = []
        self.steps_done: List[int] = []
        self.slots: List[Slot] = []
        self.used_bytes = 0
        self.check_every = check_every
        self.quarantined: Dict[int, str] = {}  # domain -> reason

    # ---- admission ----
    def free_bytes(self) -> int:
        free, _ = self.torch.cuda.mem_get_info()
        if self.memory_limit is not None:
            free = min(free, self.memory_limit - self.used_bytes)
        return free

    def add_domain(self, dom, load_fn) -> int:
        """Admit one domain (``dom`` a grid.Domain, ``load_fn(dom) -> capi.Domain``)."""
        s = dom.spec
        need = bytes_per_domain(s.ni, s.nj, s.nk, s.ntracers, self.precision)
        if self.free_bytes() - self.reserve < need:
            raise AdmissionError(f"domain {s.ni}x{s.nj}x{s.nk} needs {need / 2**30:.2f} GiB; "
                                 f"{self.free_bytes() / 2**30:.2f} GiB free with {self.reserve / 2**30:.1f} GiB reserved")
        d = load_fn(dom)
        self.domains.append(d)
        self.cells.append(s.ni * s.nj * s.nk)
        self.parity.append(0)
        self.busy.append(False)
        self.steps_done.append(0)
        self.used_bytes += need
        return len(self.domains) - 1

    def start(self):
        """Create the batch slots (after every domain is admitted)."""
        for _ in range(self.nslots):
            st = self.torch.cuda.Stream()
            b = capi.Batch(self.domains)
            b.set_stream(st.cuda_stream)
            self.slots.append(Slot(b, st))

    def close(self):
        for s in self.slots:
            s.batch.close()
        self.slots = []

    def bucket(self, i: int) -> int:
        return int(math.log2(max(1, self.cells[i])))

    # ---- the loop ----
    def run(self, arrivals: List[float], targets: List[int], timeout: float = 600.0) -> Dict:
        """Serve requests (arrival times in seconds from now, target domain ids);
        returns per-request latencies and throughput."""
        torch = self.torch
        order = np.argsort(arrivals, kind="stable")
        reqs = [Request(int(r), int(targets[r]), float(arrivals[r])) for r in order]
        t0 = time.perf_counter()
        nxt = 0
        waiting: Dict[int, deque] = {}
        free_slots = deque(range(len(self.slots)))
        inflight: List[int] = []
        done: List[Request] = []
        batches = 0
        batch_sizes = []
        while len(done) < len(reqs):
            now = time.perf_counter() - t0
            if now > timeout:
                raise TimeoutError(f"serving loop exceeded {timeout} s with {len(reqs) - len(done)} requests left")
            while nxt < len(reqs) and reqs[nxt].arrival <= now:
                r = reqs[nxt]
                nxt += 1
                if not 0 <= r.domain < len(self.domains) or r.domain in self.quarantined:
                    r.status = "rejected"
                    r.error = self.quarantined.get(r.domain, f"no domain {r.domain}")
                    r.start = r.done = now
                    done.append(r)
                    continue
                waiting.setdefault(self.bucket(r.domain), deque()).append(r)
            # completions
            for si in list(inflight):
                s = self.slots[si]
                if s.event.query():
                    t = time.perf_counter() - t0
                    for r in s.requests:
                        r.done = t
                        self.busy[r.domain] = False
                        self.parity[r.domain] ^= 1
                        self.steps_done[r.domain] += 1
                        done.append(r)
                        if self.check_every and self.steps_done[r.domain] % self.check_every == 0:
                            self.health_check(r.domain)
                    s.requests = []
                    inflight.remove(si)
                    free_slots.append(si)
            # launches: oldest bucket first, one request per idle domain
            while free_slots:
                cand = [(q[0].arrival, b) for b, q in waiting.items() if q]
                if not cand:
                    break
                launched = False
                for _, bkt in sorted(cand):
                    q = waiting[bkt]
                    take, keep, seen = [], deque(), set()
                    while q:
                        r = q.popleft()
                        if r.domain in self.quarantined:  # quarantined while the request waited
                            r.status, r.error = "rejected", self.quarantined[r.domain]
                            r.start = r.done = time.perf_counter() - t0
                            done.append(r)
                            continue
                        if (len(take) < self.max_batch and not self.busy[r.domain] and r.domain not in seen):
                            take.append(r)
                            seen.add(r.domain)
                        else:
                            keep.append(r)
                    waiting[bkt] = keep
                    if not take:
                        continue
                    si = free_slots.popleft()
                    s = self.slots[si]
                    t = time.perf_counter() - t0
                    for r in take:
                        r.start = t
                        self.busy[r.domain] = True
                    try:
                        s.batch.step(self.dtime, index=[r.domain for r in take],
                                     parity=[self.parity[r.domain] for r in take])
                    except capi.Mom5GpuError as e:
                        # the library refused the step: fail these requests, keep the others serving
                        for r in take:
                            r.status, r.error, r.done = "failed", str(e), time.perf_counter() - t0
                            self.busy[r.domain] = False
                            self.quarantined[r.domain] = f"step failed: {e}"
                            done.append(r)
                        free_slots.append(si)
                        launched = True
                        break
                    s.event = torch.cuda.Event()
                    s.event.record(s.stream)
                    s.requests = take
                    inflight.append(si)
                    batches += 1
                    batch_sizes.append(len(take))
                    launched = True
                    break
                if not launched:
                    break
            if not free_slots or (nxt < len(reqs) and not any(waiting.values())):
                time.sleep(20e-6)
        ok = [r for r in done if r.status == "ok"]
        wall = max(r.done for r in done) - min(r.arrival for r in done) if done else 0.0
        lat = np.array([r.done - r.arrival for r in ok]) if ok else np.zeros(1)
        cells = sum(self.cells[r.domain] for r in ok)
        wall = max(wall, 1e-9)
        return {"requests": len(ok), "wall_s": wall, "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
                "cell_updates_per_s": cells / wall, "requests_per_s": len(ok) / wall, "batches": batches,
                "mean_batch": float(np.mean(batch_sizes)) if batch_sizes else 0.0,
                "failed": sum(r.status == "failed" for r in done),
                "rejected": sum(r.status == "rejected" for r in done),
                "errors": {r.rid: r.error for r in done if r.status != "ok"},
                "quarantined": dict(self.quarantined)}

    def health_check(self, i: int) -> bool:
        """Quarantine domain i if any tracer at its current time level is not finite."""
        d = self.domains[i]
        level = self.parity[i] + 1
        if d.check_finite(0, level):
            return True
        self.quarantined[i] = f"non-finite tracer after {self.steps_done[i]} steps"
        return False


def poisson_arrivals(rate: float, n: int, seed: int = 0) -> List[float]:
    rng = np.random.default_rng(seed)
    return list(np.cumsum(rng.exponential(1.0 / rate, size=n)))


def ensemble_specs(n: int, seed: int = 0, ntracers: int = 4):
    """Domain sizes of the ensemble / serving configs: nx, ny log-uniform in
    [64, 512], nz uniform in 20..50, regional boxes with seeded inputs."""
    from . import grid
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        ni = int(round(math.exp(rng.uniform(math.log(64), math.log(512)))))
        nj = int(round(math.exp(rng.uniform(math.log(64), math.log(512)))))
        nk = int(rng.integers(20, 51))
        span = nj * 0.1  # 0.25 x 0.1 degree cells
        lat0 = float(rng.uniform(-70.0, 70.0 - span))
        specs.append(grid.DomainSpec(ni=ni, nj=nj, nk=nk, lon0=0.0, lon1=ni * 0.25, lat0=lat0, lat1=lat0 + span,
                                     continent=(ni // 3, nj // 3, max(2, ni // 10), max(2, nj // 10)), hmin=2000.0,
                                     ntracers=ntracers, seed=1000 + seed * 977 + i))
    return specs
