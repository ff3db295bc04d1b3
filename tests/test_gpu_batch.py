"""Batching form: many uneven resident domains per launch (mom5gpu_batch_*).

A batched step must give every domain exactly the values it gets when stepped
alone through the one-domain entry points (mom5gpu_tracer_advection_step +
mom5gpu_update_ocean_barotropic): the batched kernels run the same bodies on
the same tiles.  FP64 and precision form; work lists with mixed time-level
parities; the CUDA-graph path; the autotuner.
"""
import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu

DT = 3600.0 * 3


def make_domains(capi, harness, precision, sizes, ntr=3, seed0=40):
    doms, raw = [], []
    for n, (ni, nj, nk, cx) in enumerate(sizes):
        sp = grid.DomainSpec(ni=ni, nj=nj, nk=nk, lon0=0.0, lon1=float(ni) * 0.5, lat0=-25.0, lat1=25.0,
                             cyclic_x=cx, continent=(ni // 3, nj // 3, max(2, ni // 8), max(2, nj // 8)),
                             wavelength_cells=6.0, ntracers=ntr, seed=seed0 + n)
        dom = grid.make_domain(sp)
        opts = capi.default_options(barotropic_time_stepping_B=1, precision=precision)
        d = harness.load(dom, options=opts)
        d.barotropic_init(dtuv=200.0, dtbt=20.0)
        doms.append(d)
        raw.append(dom)
    return doms, raw


SIZES = [(40, 30, 8, False), (57, 23, 11, True), (29, 41, 6, False), (64, 64, 9, False), (18, 12, 5, True)]


def snapshot(capi, d, ntr, level):
    out = [d.get(capi.F.TRACER, n=n, level=level) for n in range(1, ntr + 1)]
    for fid in (capi.F.ETA_T_BAR, capi.F.UDRHO_U, capi.F.UDRHO_V, capi.F.CONV_RHO_UD_T, capi.F.ETA_U):
        out.append(d.get(fid, level=level))
    return out


@pytest.mark.parametrize("precision,ntr,rows", [(0, 3, None), (1, 3, None), (0, 10, None), (1, 10, None), (1, 3, 24),
                                                (1, 10, 24)])
def test_batch_equals_single_domain_steps(gpu_lib, precision, ntr, rows):
    """rows 24: the precision form's TMA-staged tiles for the domains with an
    even ni (40, 64, 18 of SIZES) and the plain tiles for the others, in one
    step; every launch shape gives the same bits as the one-domain path."""
    capi = gpu_lib
    from mom5_gb300 import harness
    single, _ = make_domains(capi, harness, precision, SIZES, ntr)
    batched, _ = make_domains(capi, harness, precision, SIZES, ntr)
    b = capi.Batch(batched)
    if rows:
        b.tuning = (rows, 0, 2)
    # step 1: every domain, parity 0, through a work list
    for d in single:
        d.tracer_advection_step(1, 1, 2, DT)
        d.update_ocean_barotropic(1, 2)
    b.step(DT, index=list(range(len(SIZES))), parity=[0] * len(SIZES))
    # step 2: a subset moves on (parity 1), the rest stays
    moved = [0, 2, 3]
    for i in moved:
        single[i].tracer_advection_step(2, 2, 1, DT)
        single[i].update_ocean_barotropic(2, 1)
    b.step(DT, index=moved, parity=[1] * len(moved))
    # step 3: the others catch up (parity 1)
    rest = [1, 4]
    for i in rest:
        single[i].tracer_advection_step(2, 2, 1, DT)
        single[i].update_ocean_barotropic(2, 1)
    b.step(DT, index=rest, parity=[1] * len(rest))
    # steps 4 and 5: all domains through the CUDA graph (parity 0 then 1)
    for p in (0, 1):
        for d in single:
            d.tracer_advection_step(1 + p, 1 + p, 2 - p, DT)
            d.update_ocean_barotropic(1 + p, 2 - p)
        b.step(DT, parity=p)
    for i, (s, t) in enumerate(zip(single, batched)):
        a = snapshot(capi, s, ntr, 1)
        c = snapshot(capi, t, ntr, 1)
        for k, (x, y) in enumerate(zip(a, c)):
            assert np.all(x == y), f"domain {i} field {k}: max diff {np.abs(x - y).max()}"
    assert b.launches > 0
    b.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_autotune_keeps_results(gpu_lib, precision):
    capi = gpu_lib
    from mom5_gb300 import harness
    doms, _ = make_domains(capi, harness, precision, SIZES[:3], 2, seed0=70)
    b = capi.Batch(doms)
    report = b.autotune(DT)
    assert "chosen" in report, report
    b.step(DT, parity=0)
    t0 = [d.get(capi.F.TRACER, n=1, level=2) for d in doms]
    ref, _ = make_domains(capi, harness, precision, SIZES[:3], 2, seed0=70)
    for d, x in zip(ref, t0):
        d.tracer_advection_step(1, 1, 2, DT)
        d.update_ocean_barotropic(1, 2)
        y = d.get(capi.F.TRACER, n=1, level=2)
        if precision == 0:
            assert np.all(x == y)
        else:
            # tile height may differ from the one-domain kernel's: same method, FP32 rounding
            assert np.abs(x - y).max() <= 1e-6 * np.abs(y).max()
    b.close()


def test_batch_rejects_mixed_configurations(gpu_lib):
    capi = gpu_lib
    from mom5_gb300 import harness
    a, _ = make_domains(capi, harness, 0, SIZES[:1], 2)
    c, _ = make_domains(capi, harness, 1, SIZES[1:2], 2)
    with pytest.raises(capi.Mom5GpuError):
        capi.Batch([a[0], c[0]])


def test_batch_tuning_get_set(gpu_lib):
    capi = gpu_lib
    from mom5_gb300 import harness
    doms, _ = make_domains(capi, harness, 1, SIZES[:2], 2, seed0=90)
    b = capi.Batch(doms)
    assert b.tuning == (32, 0, 2)
    b.tuning = (16, 4, 3)
    assert b.tuning == (16, 4, 3)
    b.tuning = (24, 0, 2)
    assert b.tuning == (24, 0, 2)
    b.tuning = (16, 4, 3)
    for bad in ((20, 0, 2), (32, 3, 2), (32, 0, 0), (32, 0, 5)):
        with pytest.raises(capi.Mom5GpuError):
            b.tuning = bad
    assert b.tuning == (16, 4, 3)
    b.close()
