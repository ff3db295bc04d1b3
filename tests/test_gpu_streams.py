"""Stream ordering at the C ABI: a field whose first use is a copy queued on a
caller's stream (mom5gpu_copy_field_async) while the domain's own stream is
busy keeps the copied values -- the zeroing of a newly allocated field is
complete before the entry point returns, not queued behind the domain's work."""
import numpy as np
import pytest

from mom5_gb300 import grid

pytestmark = pytest.mark.gpu


def test_first_touch_copy_on_another_stream(gpu_lib):
    capi = gpu_lib
    import torch
    from mom5_gb300 import harness
    sp = grid.DomainSpec(ni=180, nj=120, nk=30, lon0=0.0, lon1=90.0, lat0=-30.0, lat1=30.0, cyclic_x=True,
                         continent=(60, 40, 10, 8), ntracers=3, seed=12)
    d = harness.load(grid.make_domain(sp), options=capi.default_options(barotropic_time_stepping_B=1))
    own = torch.cuda.Stream()
    other = torch.cuda.Stream()
    d.set_stream(own.cuda_stream)
    n3 = d.count(capi.F.TRACER)
    src = torch.empty(n3, dtype=torch.float64, pin_memory=True)
    src.copy_(torch.linspace(1.0, 2.0, n3, dtype=torch.float64))
    torch.cuda.synchronize()
    for _ in range(4):  # keep the domain's stream busy
        d.tracer_advection_step(1, 1, 2, 3600.0)
    # time level 3 of tracer 2 has never been used: this copy allocates it
    d.copy_field_async(capi.F.TRACER, src.data_ptr(), 1, other.cuda_stream, n=2, level=3)
    torch.cuda.synchronize()
    got = d.get(capi.F.TRACER, n=2, level=3)
    assert np.array_equal(got, src.numpy())
    d.close()


@pytest.mark.parametrize("count", [1, 8, 9, 300])
def test_copy_boxes_strided(gpu_lib, count):
    """mom5gpu_copy_boxes moves every box of a call, strided on both sides, in
    launches of up to 256 boxes whose descriptors travel as kernel parameters
    (8 or fewer in a small parameter block): 1, 8, 9 and 300 boxes against the
    same copies made with numpy."""
    capi = gpu_lib
    import torch
    rng = np.random.default_rng(count)
    src = torch.from_numpy(rng.standard_normal(4096 * 8)).cuda()
    dst = torch.zeros(4096 * 8, dtype=torch.float64, device="cuda")
    want = np.zeros(dst.numel())
    s_np = src.cpu().numpy()
    boxes = []
    for b in range(count):
        n = [int(rng.integers(1, 6)), int(rng.integers(1, 5)), int(rng.integers(1, 4))]
        ss = [int(rng.integers(1, 3)), 8, 40]        # source strides: elements, rows, planes
        ds = [1, n[0], n[0] * n[1]]                  # destination: packed
        so = int(rng.integers(0, src.numel() - 200))
        do = (b * 64) % (dst.numel() - 64)           # distinct 64-element slots (count <= 512)
        for z in range(n[2]):
            for y in range(n[1]):
                for x in range(n[0]):
                    want[do + x * ds[0] + y * ds[1] + z * ds[2]] = s_np[so + x * ss[0] + y * ss[1] + z * ss[2]]
        boxes.append(capi.Box(src.data_ptr() + 8 * so, dst.data_ptr() + 8 * do, tuple(ss), tuple(ds), tuple(n)))
    capi.copy_boxes(boxes)
    torch.cuda.synchronize()
    assert np.array_equal(dst.cpu().numpy(), want)
