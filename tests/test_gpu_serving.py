"""Serving form: continuous batching of step requests over resident domains.

Each domain's state after being served in a mix of requests (batched with other
domains, on several overlapping streams) must equal its state after the same
number of steps run alone through the one-domain entry points (same precision;
the batched kernels run the same bodies on the same tiles, so the expected
agreement is exact).  Admission refuses a domain that does not fit the memory
budget.
"""
import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu

DT = 400.0


def small_specs(n, seed=3, ntr=3):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        ni, nj, nk = int(rng.integers(30, 90)), int(rng.integers(25, 80)), int(rng.integers(6, 12))
        out.append(grid.DomainSpec(ni=ni, nj=nj, nk=nk, lon0=0.0, lon1=ni * 0.25, lat0=-10.0, lat1=-10.0 + nj * 0.1,
                                   continent=(ni // 3, nj // 3, 3, 3), ntracers=ntr, seed=500 + i, wavelength_cells=6.0))
    return out


def loader(capi, precision):
    from mom5_gb300 import harness

    def load(dom):
        d = harness.load(dom, options=capi.default_options(barotropic_time_stepping_B=1, precision=precision))
        d.barotropic_init(dtuv=400.0, dtbt=20.0)
        return d
    return load


@pytest.mark.parametrize("precision", [0, 1])
def test_served_state_equals_alone(gpu_lib, precision):
    capi = gpu_lib
    from mom5_gb300 import serving
    specs = small_specs(8)
    doms = [grid.make_domain(s) for s in specs]
    srv = serving.Server(DT, precision=precision, slots=3, max_batch=4, reserve_bytes=1 << 30)
    load = loader(capi, precision)
    for dom in doms:
        srv.add_domain(dom, load)
    srv.start()
    rng = np.random.default_rng(0)
    targets = list(rng.integers(0, len(doms), size=60))
    arrivals = serving.poisson_arrivals(rate=2000.0, n=len(targets), seed=1)
    stats = srv.run(arrivals, targets)
    assert stats["requests"] == 60 and stats["batches"] >= 2
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    for i, dom in enumerate(doms):
        k = srv.steps_done[i]
        assert k == targets.count(i)
        alone = load(dom)
        tau = 1
        for _ in range(k):
            alone.tracer_advection_step(tau, tau, 3 - tau, DT)
            alone.update_ocean_barotropic(tau, 3 - tau)
            tau = 3 - tau
        assert srv.parity[i] == (k % 2)
        for n in range(1, specs[i].ntracers + 1):
            a = alone.get(capi.F.TRACER, n=n, level=tau)
            b = srv.domains[i].get(capi.F.TRACER, n=n, level=tau)
            assert np.all(a == b), f"domain {i} tracer {n}: {np.abs(a - b).max()}"
        for fid in (capi.F.ETA_T_BAR, capi.F.UDRHO_U):
            a = alone.get(fid, level=tau)
            b = srv.domains[i].get(fid, level=tau)
            assert np.all(a == b), f"domain {i} field {fid}"
        alone.close()
    srv.close()


def test_admission_by_free_memory(gpu_lib):
    capi = gpu_lib
    from mom5_gb300 import serving
    specs = small_specs(3)
    srv = serving.Server(DT, precision=1, reserve_bytes=0, memory_limit=serving.bytes_per_domain(
        specs[0].ni, specs[0].nj, specs[0].nk, specs[0].ntracers, 1) + 1000)
    load = loader(capi, 1)
    srv.add_domain(grid.make_domain(specs[0]), load)
    with pytest.raises(serving.AdmissionError):
        srv.add_domain(grid.make_domain(specs[1]), load)


def test_failures_are_contained(gpu_lib):
    """Host-side fault injection: a request for a domain that does not exist is
    rejected; a batched step the library refuses fails only the requests of that
    batch and quarantines their domains; a domain whose tracer turns non-finite is
    quarantined by the health check; every other domain keeps serving and ends
    equal to the same domain stepped alone."""
    capi = gpu_lib
    from mom5_gb300 import serving
    specs = small_specs(5, seed=9)
    doms = [grid.make_domain(s) for s in specs]
    srv = serving.Server(DT, precision=1, slots=2, max_batch=1, reserve_bytes=1 << 30, check_every=1)
    load = loader(capi, 1)
    for dom in doms:
        srv.add_domain(dom, load)
    srv.start()
    poisoned, blown = 1, 3
    # a library refusal whenever the poisoned domain is stepped
    for slot in srv.slots:
        real = slot.batch.step

        def step(dtime, index=None, parity=None, _real=real):
            if index is not None and poisoned in index:
                raise capi.Mom5GpuError(capi.EINVAL, "injected refusal")
            return _real(dtime, index=index, parity=parity)
        slot.batch.step = step
    # a non-finite value in the blown domain's tracer
    sb = specs[blown]
    T = srv.domains[blown].get(capi.F.TRACER, n=1, level=1).reshape(sb.nk, sb.nj + 2, sb.ni + 2)
    T[0, 2, 2] = np.nan  # a compute cell away from the continent
    srv.domains[blown].set(capi.F.TRACER, np.ascontiguousarray(T), n=1, level=1)
    targets = [0, 1, 2, 3, 4, 99, 0, 1, 2, 3, 4, 0, 2, 4]
    arrivals = [0.001 * i for i in range(len(targets))]
    stats = srv.run(arrivals, targets)
    assert stats["rejected"] >= 1 + 1  # the unknown domain, and later requests to a quarantined one
    assert stats["failed"] == 1 and "injected refusal" in srv.quarantined[poisoned]
    assert blown in srv.quarantined and "non-finite" in srv.quarantined[blown]
    assert srv.steps_done[poisoned] == 0 and srv.steps_done[blown] == 1
    for i in (0, 2, 4):
        k = srv.steps_done[i]
        assert k == targets.count(i)
        alone = load(doms[i])
        tau = 1
        for _ in range(k):
            alone.tracer_advection_step(tau, tau, 3 - tau, DT)
            alone.update_ocean_barotropic(tau, 3 - tau)
            tau = 3 - tau
        for n in range(1, specs[i].ntracers + 1):
            assert np.array_equal(alone.get(capi.F.TRACER, n=n, level=tau), srv.domains[i].get(capi.F.TRACER, n=n, level=tau))
        alone.close()
    srv.close()
