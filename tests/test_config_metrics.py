"""CPU tests of the run configuration layer (namelist groups and field_table
choices as JSON) and of the JSON-lines metrics log."""
import json

import pytest

capi = pytest.importorskip("mom5_gb300.capi")


@pytest.fixture(scope="module")
def cfgmod():
    from mom5_gb300 import build
    build.build()
    from mom5_gb300 import config
    return config


def test_defaults_are_the_reference_namelist_defaults(cfgmod):
    c = cfgmod.parse({})
    o = c.options
    assert (o.advect_sweby_all, o.limit_with_upwind, o.zero_tracer_advect_horz, o.zero_tracer_advect_vert) == (0, 0, 0, 0)
    assert o.pred_corr_gamma == 0.2 and o.rho0 == 1035.0 and o.grav == 9.8 and o.initsum_with_bar == 1
    assert o.psom_limit_prather == 0 and o.precision == capi.PRECISION_FP64
    assert (o.udrho_lap, o.udrho_bih, o.udrho_lap_vel_micom, o.udrho_bih_vel_micom) == (0, 0, 0.05, 0.01)
    assert c.tracers == []


def test_barotropic_friction_namelist(cfgmod):
    """ocean_barotropic_nml udrho_lap / udrho_bih and their MICOM velocities
    (ocean_barotropic.F90:599-604) reach mom5gpu_options."""
    c = cfgmod.parse({"ocean_barotropic_nml": {"udrho_lap": True, "udrho_bih": False, "udrho_lap_vel_micom": 0.1,
                                               "udrho_bih_vel_micom": 0.02}})
    o = c.options
    assert (o.udrho_lap, o.udrho_bih, o.udrho_lap_vel_micom, o.udrho_bih_vel_micom) == (1, 0, 0.1, 0.02)
    with pytest.raises(ValueError):
        cfgmod.parse({"ocean_barotropic_nml": {"udrho_lap_micom": 0.1}})


def test_namelists_and_field_table(cfgmod, tmp_path):
    doc = {"ocean_tracer_advect_nml": {"limit_with_upwind": True, "psom_limit_prather": True},
           "ocean_barotropic_nml": {"barotropic_time_stepping_B": True, "pred_corr_gamma": 0.25},
           "library": {"precision": "mixed"},
           "tracers": [{"name": "temp", "horiz_advect_scheme": "quickMOM3", "vert_advect_scheme": "quicker",
                        "restart_file": "ocean_temp_salt.res.nc"},
                       {"name": "age", "horiz_advect_scheme": "psom", "vert_advect_scheme": "psom",
                        "psom_limit": True}]}
    p = tmp_path / "run.json"
    p.write_text(json.dumps(doc))
    for src in (doc, json.dumps(doc), str(p)):
        c = cfgmod.parse(src)
        assert c.options.limit_with_upwind == 1 and c.options.psom_limit_prather == 1
        assert c.options.barotropic_time_stepping_B == 1 and c.options.pred_corr_gamma == 0.25
        assert c.options.precision == capi.PRECISION_MIXED
        assert [t.name for t in c.tracers] == ["temp", "age"]
        assert cfgmod.SCHEMES[c.tracers[0].horiz_advect_scheme] == capi.ADVECT_QUICKMOM3
        assert c.tracers[1].psom_limit and c.tracers[1].restart_file == "ocean_tracer.res.nc"


@pytest.mark.parametrize("doc", [{"ocean_tracer_advect_nml": {"advect_sweeby_all": True}},
                                 {"bogus_nml": {}},
                                 {"library": {"precision": "fp16"}},
                                 {"tracers": [{"name": "t", "horiz_advect_scheme": "mdfl_sweby_test"}]},
                                 {"tracers": [{"name": "t", "colour": "red"}]}])
def test_unknown_entries_are_errors(cfgmod, doc):
    with pytest.raises(ValueError):
        cfgmod.parse(doc)


def test_metrics_log_records_bench_figures(tmp_path):
    from mom5_gb300 import metrics
    path = str(tmp_path / "m" / "run.jsonl")
    out = {"metric": "m", "value": 4.3e8, "unit": "cell-updates/s", "ms_per_step": 180.0,
           "e2e": {"value": 4.0e8}, "roofline": {"achieved": 95.0, "frac": 0.014},
           "fp64_roofline": {"mdfl": {"frac": 0.9}}, "config": {"workload": "C2"},
           "forms": {"precision": {"value": 2.9e9, "max_rel_err_vs_fp64_1step": 3.9e-7,
                                   "content_rel_change_1step": {"fp64": 0.0, "precision": 6e-14}},
                     "serving": {"runs": [{"offered_rps": 700, "p50_ms": 2.1, "p99_ms": 4.3,
                                           "cell_updates_per_s": 1.2e9}]},
                     "schemes": {"schemes": {"psom": {"ms_per_step": 1270.0, "cell_updates_per_s": 6.1e7}}}}}
    log = metrics.MetricsLog(path)
    metrics.from_bench_line(out, log)
    log.record("note", text="second run")
    recs = list(metrics.read(path))
    kinds = [r["kind"] for r in recs]
    assert kinds == ["headline", "precision_form", "serving", "scheme", "note"]
    assert recs[0]["value"] == 4.3e8 and recs[0]["fp64_frac"] == 0.9 and recs[0]["e2e"] == 4.0e8
    assert recs[2]["p99_ms"] == 4.3 and recs[3]["scheme"] == "psom"
    assert all("time" in r for r in recs)
