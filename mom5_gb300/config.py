"""Run configuration from a JSON document: the namelist groups and the per-tracer
field_table choices the reference reads, mapped onto mom5gpu_options and the
per-tracer setters of the C ABI.

    {
      "ocean_tracer_advect_nml": {"advect_sweby_all": false, "limit_with_upwind": false,
                                  "zero_tracer_advect_horz": false, "zero_tracer_advect_vert": false,
                                  "psom_limit_prather": false},
      "ocean_barotropic_nml": {"barotropic_time_stepping_A": false, "barotropic_time_stepping_B": true,
                               "pred_corr_gamma": 0.2, "initsum_with_bar": true,
                               "zero_forcing_bt": false, "zero_nonlinear_forcing_bt": false,
                               "udrho_lap": false, "udrho_bih": false, "udrho_lap_vel_micom": 0.05,
                               "udrho_bih_vel_micom": 0.01},
      "ocean_parameters": {"rho0": 1035.0, "grav": 9.8},
      "library": {"precision": "fp64"},
      "tracers": [{"name": "temp", "horiz_advect_scheme": "mdfl_sweby", "vert_advect_scheme": "mdfl_sweby",
                   "min_tracer_limit": -10.0, "max_tracer_limit": 100.0, "ppm_hlimiter": 2, "psom_limit": false,
                   "restart_file": "ocean_temp_salt.res.nc"}]
    }

Names and defaults follow ocean_tracer_advect.F90:483-495, ocean_barotropic.F90:
528-614 and the field_table keys read in ocean_tracer.F90:960-1066 (scheme
strings :982-1056, tracer defaults ocean_tpm_util.F90:76-87).  Unknown keys are
errors, as an unknown namelist entry is for the reference.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Union

from . import capi

# field_table scheme strings (ocean_tracer.F90:982-1056)
SCHEMES = {"upwind": capi.ADVECT_UPWIND, "2nd_order": capi.ADVECT_2ND_ORDER, "4th_order": capi.ADVECT_4TH_ORDER,
           "6th_order": capi.ADVECT_6TH_ORDER, "quicker": capi.ADVECT_QUICKER, "quickMOM3": capi.ADVECT_QUICKMOM3,
           "mdfl_sup_b": capi.ADVECT_MDFL_SUP_B, "mdfl_sweby": capi.ADVECT_MDFL_SWEBY,
           "dst_linear": capi.ADVECT_DST_LINEAR, "mdppm": capi.ADVECT_MDPPM, "psom": capi.ADVECT_PSOM}

_NML_KEYS = {
    "ocean_tracer_advect_nml": {"advect_sweby_all", "limit_with_upwind", "zero_tracer_advect_horz",
                                "zero_tracer_advect_vert", "psom_limit_prather"},
    "ocean_barotropic_nml": {"barotropic_time_stepping_A", "barotropic_time_stepping_B", "pred_corr_gamma",
                             "initsum_with_bar", "zero_forcing_bt", "zero_nonlinear_forcing_bt", "udrho_lap",
                             "udrho_bih", "udrho_lap_vel_micom", "udrho_bih_vel_micom"},
    "ocean_parameters": {"rho0", "grav"},
    "library": {"precision"},
}
_TRACER_KEYS = {"name", "horiz_advect_scheme", "vert_advect_scheme", "min_tracer_limit", "max_tracer_limit",
                "ppm_hlimiter", "psom_limit", "restart_file"}


@dataclass
class TracerConfig:
    name: str
    horiz_advect_scheme: str = "mdfl_sweby"
    vert_advect_scheme: str = "mdfl_sweby"
    min_tracer_limit: float = -1.0e10
    max_tracer_limit: float = 1.0e10
    ppm_hlimiter: int = 2
    psom_limit: bool = False
    restart_file: str = "ocean_tracer.res.nc"


@dataclass
class RunConfig:
    options: capi.Options
    tracers: List[TracerConfig] = field(default_factory=list)

    def apply(self, d: "capi.Domain") -> None:
        """Per-tracer choices onto a created domain (before tracer_advect_init)."""
        ntr = d.dims.num_prog_tracers
        if self.tracers and len(self.tracers) != ntr:
            raise ValueError(f"{len(self.tracers)} tracers configured, the domain has {ntr}")
        for n, t in enumerate(self.tracers, start=1):
            d.set_tracer_scheme(n, SCHEMES[t.horiz_advect_scheme], SCHEMES[t.vert_advect_scheme],
                                t.min_tracer_limit, t.max_tracer_limit)
            d.set_ppm_limiter(n, t.ppm_hlimiter)
            d.set_psom_limit(n, t.psom_limit)
            d.set_tracer_name(n, t.name, t.restart_file)


def parse(doc: Union[str, Dict[str, Any]]) -> RunConfig:
    """A RunConfig from a JSON string, a path to a JSON file or a dict."""
    if isinstance(doc, str):
        text = doc
        if not doc.lstrip().startswith("{"):
            with open(doc) as fh:
                text = fh.read()
        doc = json.loads(text)
    unknown = set(doc) - set(_NML_KEYS) - {"tracers"}
    if unknown:
        raise ValueError(f"unknown configuration groups: {sorted(unknown)}")
    kw: Dict[str, Any] = {}
    for group, keys in _NML_KEYS.items():
        vals = doc.get(group, {})
        bad = set(vals) - keys
        if bad:
            raise ValueError(f"{group}: unknown entries {sorted(bad)}")
        for k, v in vals.items():
            if k == "precision":
                if v not in ("fp64", "mixed"):
                    raise ValueError("library.precision must be 'fp64' or 'mixed'")
                kw[k] = capi.PRECISION_FP64 if v == "fp64" else capi.PRECISION_MIXED
            elif isinstance(v, bool):
                kw[k] = int(v)
            else:
                kw[k] = v
    tracers = []
    for t in doc.get("tracers", []):
        bad = set(t) - _TRACER_KEYS
        if bad:
            raise ValueError(f"tracer {t.get('name')}: unknown entries {sorted(bad)}")
        tc = TracerConfig(**t)
        for which in (tc.horiz_advect_scheme, tc.vert_advect_scheme):
            if which not in SCHEMES:
                raise ValueError(f"tracer {tc.name}: invalid advect scheme {which!r}")
        tracers.append(tc)
    return RunConfig(options=capi.default_options(**kw), tracers=tracers)


def load_domain(dom, cfg: Optional[RunConfig] = None, **load_kw) -> "capi.Domain":
    """harness.load with the configuration's options and per-tracer choices."""
    from . import harness
    cfg = cfg or parse({})
    d = harness.load(dom, options=cfg.options, **load_kw)
    if cfg.tracers:
        cfg.apply(d)
        d.tracer_advect_init()
    return d
