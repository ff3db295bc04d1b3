"""JSON-lines metrics log: one JSON object per line, appended as a run produces
its figures (cell-updates/s, GB/s, roofline fractions, p50/p99 latency, errors
against the FP64 path, conservation drift).  Plays the part the diagnostics
manager's time series play for the reference (diag_manager send_data), for the
library's own performance and accuracy figures."""
from __future__ import annotations

import json
import os
import time
from typing import Any, Dict, Iterator, Optional


class MetricsLog:
    def __init__(self, path: Optional[str]):
        self.path = path

    def record(self, kind: str, **fields: Any) -> Dict[str, Any]:
        """Append {"time", "kind", **fields}; a log without a path only returns it."""
        rec = {"time": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()), "kind": kind}
        rec.update(fields)
        if self.path:
            d = os.path.dirname(os.path.abspath(self.path))
            os.makedirs(d, exist_ok=True)
            with open(self.path, "a") as fh:
                fh.write(json.dumps(rec, sort_keys=True) + "\n")
        return rec


def read(path: str) -> Iterator[Dict[str, Any]]:
    with open(path) as fh:
        for line in fh:
            line = line.strip()
            if line:
                yield json.loads(line)


def from_bench_line(out: Dict[str, Any], log: MetricsLog) -> None:
    """The figures of one bench.py result line as metrics records."""
    roof = out.get("roofline") or {}
    f64 = (out.get("fp64_roofline") or {}).get("mdfl", {})
    log.record("headline", metric=out.get("metric"), value=out.get("value"), unit=out.get("unit"),
               ms_per_step=out.get("ms_per_step"), e2e=(out.get("e2e") or {}).get("value"),
               hbm_gbs=roof.get("achieved"), hbm_frac=roof.get("frac"), fp64_frac=f64.get("frac"),
               workload=(out.get("config") or {}).get("workload"), clocks=out.get("clocks"))
    forms = out.get("forms") or {}
    p = forms.get("precision")
    if p:
        log.record("precision_form", value=p.get("value"), max_rel_err_vs_fp64=p.get("max_rel_err_vs_fp64_1step"),
                   content_drift=p.get("content_rel_change_1step"))
    b = forms.get("batched")
    if b:
        log.record("batched_form", fp64=(b.get("fp64") or {}).get("value"),
                   precision=(b.get("precision") or {}).get("value"))
    s = forms.get("serving")
    if s:
        for r in s.get("runs", []):
            log.record("serving", offered_rps=r.get("offered_rps"), p50_ms=r.get("p50_ms"), p99_ms=r.get("p99_ms"),
                       cell_updates_per_s=r.get("cell_updates_per_s"))
    sw = forms.get("schemes")
    if sw:
        for name, v in sw.get("schemes", {}).items():
            log.record("scheme", scheme=name, ms_per_step=v.get("ms_per_step"),
                       cell_updates_per_s=v.get("cell_updates_per_s"))
