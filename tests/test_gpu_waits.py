"""Bounded device waits.  The cooperative barotropic launch replaces each
launch boundary of the subcycle loop with a grid barrier whose wait gives up
after a bounded number of SM clock cycles.  The self-test runs the barrier over
a full resident grid and checks after every barrier that every block arrived;
with a target one block beyond the grid no wait can succeed, so every block
gives up (after about 8 ms), the call reports MOM5GPU_ETIMEDOUT and the context
stays usable: a barotropic step afterwards still equals the restatement.  No
fault, trap or endless loop is involved."""
import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu


def test_grid_barrier_orders_blocks(gpu_lib):
    capi = gpu_lib
    from mom5_gb300 import harness
    dom = grid.make_domain(grid.DomainSpec(ni=20, nj=10, nk=1, hmin=None, ntracers=0, seed=3))
    d = harness.load(dom)
    d.grid_barrier_selftest(500)
    with pytest.raises(capi.Mom5GpuError):
        d.grid_barrier_selftest(0)
    d.close()


def test_grid_barrier_wait_gives_up_and_context_survives(gpu_lib, oracle_lib):
    capi, O = gpu_lib, oracle_lib
    from mom5_gb300 import harness
    sp = grid.DomainSpec(ni=60, nj=40, nk=1, lon0=0.0, lon1=60.0, lat0=-50.0, lat1=50.0, cyclic_x=True, hmin=None,
                         ridge_amp=1000.0, ntracers=0, seed=23)
    dom = grid.make_domain(sp)
    d = harness.load(dom, options=capi.default_options(barotropic_time_stepping_B=1))
    nts = d.barotropic_init(dtuv=300.0, dtbt=30.0)
    with pytest.raises(capi.Mom5GpuError) as e:
        d.grid_barrier_selftest(3, unreachable=True)
    assert e.value.status == capi.ETIMEDOUT
    d.synchronize()  # the error word was cleared with the report
    d.grid_barrier_selftest(20)
    # a cooperative barotropic step on the same context equals the restatement
    d.set_barotropic_fusion(2)
    d.update_ocean_barotropic(1, 2)
    g = O.domain_arrays(dom)
    st = {k: dom[k].numpy().copy() for k in ("eta_t", "eta_t_bar", "udrho_u", "udrho_v")}
    out = O.update_ocean_barotropic(O.dims(sp), g, st, nts, 30.0, time_stepping_B=True)
    for k, fid in (("eta_t_bar", capi.F.ETA_T_BAR), ("udrho_u", capi.F.UDRHO_U), ("udrho_v", capi.F.UDRHO_V)):
        assert np.array_equal(d.get(fid, level=2).reshape(out[k].shape), out[k]), k
    d.close()
