"""The reference's processor-count identity on one GPU: a domain stepped as a
2-D layout of blocks (mpp_define_domains / set_ocean_domain,
ocean_domains.F90:123-), each block a non-cyclic library domain whose halos
are exchanged between the phases of the step where the reference calls
mpp_update_domains, gives the undecomposed domain's values everywhere --
tracers after MDFL Sweby + explicit update, and every barotropic output --
value for value."""
import numpy as np
import pytest

from mom5_gb300 import decomp, grid

pytestmark = pytest.mark.gpu


def equal(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("px,py,cx,cy,sweby_all", [(2, 2, True, False, False), (3, 1, True, False, False),
                                                   (1, 2, True, False, True), (2, 3, False, False, False),
                                                   (2, 2, True, True, False)])
def test_decomposed_steps_equal_one_domain(gpu_lib, px, py, cx, cy, sweby_all):
    capi = gpu_lib
    import torch
    from mom5_gb300 import harness
    sp = grid.DomainSpec(ni=37, nj=26, nk=9, lon0=0.0, lon1=37.0, lat0=-30.0, lat1=30.0, cyclic_x=cx, cyclic_y=cy,
                         continent=(11, 8, 6, 5), wavelength_cells=6.0, ntracers=3, seed=60 + px + 3 * py)
    dom = grid.make_domain(sp)
    opts = capi.default_options(barotropic_time_stepping_B=1, advect_sweby_all=int(sweby_all))
    dt, dtuv, dtbt = 3 * 3600.0, 300.0, 30.0
    one = harness.load(dom, options=opts)
    nts = one.barotropic_init(dtuv=dtuv, dtbt=dtbt)
    layout = decomp.Layout(sp.ni, sp.nj, px, py, cx, cy)
    parts = decomp.split(dom, layout)
    stream = torch.cuda.Stream()
    blocks = []
    for r, b in enumerate(parts):
        d = harness.load(b, options=opts)
        assert d.barotropic_init(dtuv=dtuv, dtbt=dtbt) == nts
        d.set_stream(stream.cuda_stream)
        decomp.Decomposed.prepare(d, layout, r, b.mask2)
        blocks.append(d)
    dec = decomp.Decomposed(blocks, layout, decomp.LocalExchange(blocks, layout, stream.cuda_stream))
    shp = lambda d, lev: (lev, d.dims.nj + 2, d.dims.ni + 2)
    tau = 1
    for step in range(3):
        taup1 = 3 - tau
        one.tracer_advection_step(tau, tau, taup1, dt)
        one.update_ocean_barotropic(tau, taup1)
        dec.tracer_advection_step(tau, tau, taup1, dt)
        dec.update_ocean_barotropic(tau, taup1)
        torch.cuda.synchronize()
        for n in range(1, sp.ntracers + 1):
            got = decomp.join([d.get(capi.F.TRACER, n=n, level=taup1).reshape(shp(d, sp.nk)) for d in blocks], layout)
            ref = one.get(capi.F.TRACER, n=n, level=taup1).reshape(got.shape)
            assert equal(got, ref), f"step {step} tracer {n}: {np.abs(got - ref).max():.3e}"
        for fid in (capi.F.ETA_T_BAR, capi.F.UDRHO_U, capi.F.UDRHO_V, capi.F.CONV_RHO_UD_T, capi.F.ETA_U):
            got = decomp.join([d.get(fid, level=taup1).reshape(shp(d, 1)) for d in blocks], layout)
            ref = one.get(fid, level=taup1).reshape(got.shape)
            assert equal(got, ref), f"step {step} field {fid}: {np.abs(got - ref).max():.3e}"
        for fid in (capi.F.PS, capi.F.GRAD_PS_X, capi.F.GRAD_PS_Y):
            got = decomp.join([d.get(fid).reshape(shp(d, 1)) for d in blocks], layout, with_halo=False)
            ref = one.get(fid).reshape(got.shape)
            inner = (Ellipsis, slice(1, -1), slice(1, -1))
            assert equal(got[inner], ref[inner]), f"step {step} field {fid}"
        # the reproducing global sum: the same double for the blocks as for the whole domain
        for n in range(1, sp.ntracers + 1):
            whole = capi.fixed_to_double(one.tracer_content_fixed(n, taup1))
            assert dec.global_tracer_content(n, taup1) == whole
            assert abs(whole - one.global_tracer_content(n, taup1)) <= 1e-15 * abs(whole)
        tau = taup1
    for d in blocks:
        d.close()
    one.close()


def test_block_refuses_cyclic_and_wide_tracer_sets(gpu_lib):
    capi = gpu_lib
    d = capi.Domain(8, 6, 3, 2, cyclic_x=True)
    with pytest.raises(capi.Mom5GpuError) as e:
        d.set_neighbours(1, 1, 0, 0)
    assert e.value.status == capi.EINVAL
    d.close()
    d = capi.Domain(8, 6, 3, 11)
    with pytest.raises(capi.Mom5GpuError) as e:
        d.set_neighbours(1, 1, 0, 0)
    assert e.value.status == capi.EUNSUPPORTED
    d.close()


def test_fixed_content_is_the_exact_sum_of_the_columns(gpu_lib):
    """mom5gpu_tracer_content_fixed: the accumulators hold exactly the sum of
    each column's content (the reference's k-sum, total_tracer,
    ocean_tracer_diag.F90:2380-2415, formed here with numpy in the same
    order) truncated to a multiple of 2^-100."""
    from fractions import Fraction
    capi = gpu_lib
    from mom5_gb300 import harness
    sp = grid.DomainSpec(ni=45, nj=31, nk=12, lon0=0.0, lon1=45.0, lat0=-30.0, lat1=30.0, cyclic_x=True,
                         continent=(11, 8, 6, 5), wavelength_cells=6.0, ntracers=2, seed=77)
    dom = grid.make_domain(sp)
    d = harness.load(dom)
    tm, dat, rdz = dom["tmask"].numpy(), dom["dat"].numpy(), dom["rho_dzt"].numpy()
    for n in (1, 2):
        T = dom["T"][n - 1].numpy()
        col = np.zeros((sp.nj, sp.ni))
        da = dat[1:-1, 1:-1]
        for k in range(sp.nk):
            m = tm[k, 1:-1, 1:-1]
            t = np.where(m != 0.0, (1.0 * m) * da, 0.0)
            col = col + (t * rdz[k, 1:-1, 1:-1]) * T[k, 1:-1, 1:-1]
        want = sum(int(Fraction(float(c)) * (1 << 100)) for c in col.ravel())
        acc = d.tracer_content_fixed(n, 1)
        assert sum(a << (32 * i) for i, a in enumerate(acc)) == want
        assert capi.fixed_to_double(acc) == float(Fraction(want, 1 << 100))
    d.close()
