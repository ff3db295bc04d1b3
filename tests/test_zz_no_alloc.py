"""The allocation-free entry point (mom5gpu_mdfl_sweby_noalloc) against the
domain API's mom5gpu_horz_advect_tracer.

The allocation-free call exists for hosts that cannot let the library call
cudaMalloc (memory reserved by their own pool, a hard device-memory cap, or no
device-synchronising calls allowed).  It keeps its scratch in a fixed
file-scope device array that every call shares, so the test makes two calls in
a row on different tracers and checks both against the existing entry point,
with the same tolerance as the other FP64 parity tests: IEEE equality.  This
file is collected last, after every other test.
"""
import ctypes as C

import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    t = a if hasattr(a, "detach") else torch.from_numpy(np.ascontiguousarray(a))
    return t.to(device="cuda", dtype=torch.float64).contiguous()


def _call(capi, torch, C, dims, scheme, dt, f, T, th):
    return capi.lib().mom5gpu_mdfl_sweby_noalloc(
        C.byref(dims), scheme, dt, *[C.c_void_p(f[k].data_ptr()) for k in (
            "tmask", "dat", "datr", "dxte", "dyte", "dxtn", "dytn", "uhrho_et", "vhrho_nt", "wrho_bt", "rho_dzt")],
        C.c_void_p(T.data_ptr()), C.c_void_p(th.data_ptr()), None)


def _fields(torch, dom):
    return {k: _dev(torch, dom[k]) for k in ("tmask", "dat", "datr", "dxte", "dyte", "dxtn", "dytn", "uhrho_et",
                                             "vhrho_nt", "wrho_bt", "rho_dzt")}


@pytest.mark.parametrize("cyclic_x,cyclic_y,scheme", [(True, False, 9), (False, False, 9), (True, False, 10),
                                                      (True, True, 9)])
def test_noalloc_matches_domain_entry_point(gpu_lib, cyclic_x, cyclic_y, scheme):
    import torch
    capi = gpu_lib
    from mom5_gb300 import harness
    sp = grid.DomainSpec(ni=44, nj=31, nk=11, lon0=0.0, lon1=44.0, lat0=-30.0, lat1=30.0, cyclic_x=cyclic_x,
                         cyclic_y=cyclic_y, continent=(12, 9, 7, 5), wavelength_cells=6.0, ntracers=2, seed=17)
    dom = grid.make_domain(sp)
    dt = 6 * 3600.0
    # existing entry point
    d = harness.load(dom, scheme=scheme)
    ref = []
    for n in (1, 2):
        th0 = np.linspace(-1.0, 1.0, d.count(capi.F.TH_TENDENCY))  # accumulation onto a non-zero tendency
        d.set(capi.F.TH_TENDENCY, th0, n=n)
        d.horz_advect_tracer(n, 1, 1, dt)
        ref.append(d.get(capi.F.TH_TENDENCY, n=n))
    d.close()
    # a call on a larger, different domain first: whatever it leaves in the shared
    # scratch array must not reach the calls compared below
    big = grid.DomainSpec(ni=70, nj=52, nk=13, lon0=0.0, lon1=70.0, lat0=-40.0, lat1=40.0, cyclic_x=True,
                          continent=(20, 14, 9, 7), wavelength_cells=5.0, ntracers=1, seed=23)
    bd = grid.make_domain(big)
    bf = _fields(torch, bd)
    bdims = capi.Dims(big.ni, big.nj, big.nk, 1, 0, 1, capi.BGRID)
    bT = _dev(torch, bd["T"][0])
    bth = torch.zeros_like(bT)
    assert _call(capi, torch, C, bdims, 9, dt, bf, bT, bth) == capi.OK
    # allocation-free entry point: device arrays owned by the caller
    f = _fields(torch, dom)
    dims = capi.Dims(sp.ni, sp.nj, sp.nk, int(sp.cyclic_x), int(sp.cyclic_y), 2, capi.BGRID)
    for n in (1, 2):  # two calls in a row share the scratch array
        T = _dev(torch, dom["T"][n - 1])
        th = _dev(torch, np.linspace(-1.0, 1.0, T.numel()))
        st = _call(capi, torch, C, dims, scheme, dt, f, T, th)
        assert st == capi.OK, capi.lib().mom5gpu_last_error(None)
        torch.cuda.synchronize()
        got = th.cpu().numpy()
        assert np.all(got == ref[n - 1]), f"tracer {n}: {np.abs(got - ref[n - 1]).max()}"


def test_noalloc_rejects_oversized_domain(gpu_lib):
    capi = gpu_lib
    dims = capi.Dims(1440, 1080, 50, 1, 0, 1, capi.BGRID)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = capi.lib().mom5gpu_mdfl_sweby_noalloc(C.byref(dims), 9, 600.0, *([dummy] * 13), None)
    assert st == capi.EINVAL
    msg = capi.lib().mom5gpu_last_error(None).decode()
    assert "at most 2097152" in msg
