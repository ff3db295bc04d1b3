"""Domain decomposition on the host: the block layout (mpp_compute_extent), the
neighbour map, the halo geometry the library defines (mom5gpu_halo_region,
host arithmetic) and the rank exchanger (one block per process, isend/irecv
over gloo here, NCCL between GPUs) move exactly the halo values of the whole
domain: after an exchange every block's halo regions hold what the
undecomposed domain holds there.  No GPU is used."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from mom5_gb300 import decomp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_extents_follow_mpp_compute_extent():
    # mirror-symmetric where the parities allow (the reference's own example: 18 over 4 -> 5 4 4 5);
    # the first half rounds up, so an odd split can differ by more than one point (37 over 3)
    sizes = lambda n, p: [b - a + 1 for a, b in decomp.compute_extent(n, p)]
    assert sizes(18, 4) == [5, 4, 4, 5]
    assert sizes(37, 3) == [13, 11, 13]
    assert sizes(17, 4) == [5, 4, 4, 4]  # n odd, p even: no mirror
    for n, p in ((1440, 8), (17, 4), (100, 7), (37, 3), (7, 2)):
        e = decomp.compute_extent(n, p)
        assert e[0][0] == 1 and e[-1][1] == n
        assert all(e[q][1] + 1 == e[q + 1][0] for q in range(p - 1))


def test_neighbours_wrap_only_in_periodic_directions():
    L = decomp.Layout(40, 30, 3, 2, cyclic_x=True, cyclic_y=False)
    assert L.neighbour(0, decomp.WEST) == 2 and L.neighbour(2, decomp.EAST) == 0
    assert L.neighbour(0, decomp.SOUTH) is None and L.neighbour(3, decomp.NORTH) is None
    assert L.neighbour(0, decomp.NORTHWEST) == 5 and L.neighbour(0, decomp.SOUTHWEST) is None
    assert L.faces(4) == (1, 1, 1, 0)
    one = decomp.Layout(40, 30, 1, 2, cyclic_x=True)
    assert one.neighbour(1, decomp.WEST) == 1  # its own neighbour across the periodic direction


def test_split_cuts_every_array_to_the_block():
    """Blocks carry their data domain of every array (halo from the neighbours or
    the domain's own halo) and tmask_mdfl with the two-cell halo; join puts the
    compute cells back."""
    from mom5_gb300 import grid
    sp = grid.DomainSpec(ni=23, nj=17, nk=4, lon0=0.0, lon1=23.0, lat0=-20.0, lat1=20.0, cyclic_x=True,
                         continent=(6, 5, 4, 3), ntracers=2, seed=8)
    dom = grid.make_domain(sp)
    L = decomp.Layout(23, 17, 3, 2, True, False)
    blocks = decomp.split(dom, L)
    m2 = decomp.mask_halo2(dom["tmask"].numpy(), True, False)
    for r, b in enumerate(blocks):
        s = b.spec
        is_, ie, js, je = L.extent(r)
        assert (s.ni, s.nj, s.cyclic_x) == (ie - is_ + 1, je - js + 1, False)
        assert b.mask2.shape == (sp.nk, s.nj + 4, s.ni + 4)
        assert np.array_equal(b.mask2, m2[:, js - 1:je + 4, is_ - 1:ie + 4])
        assert np.array_equal(b["T"].numpy(), dom["T"].numpy()[..., js - 1:je + 2, is_ - 1:ie + 2])
    T = decomp.join([b["T"].numpy() for b in blocks], L)
    assert np.array_equal(T, dom["T"].numpy())


def _global(ni, nj, nlev, seed):
    rng = np.random.default_rng(seed)
    g = np.zeros((nlev, nj + 2, ni + 2))
    g[:, 1:-1, 1:-1] = rng.normal(size=(nlev, nj, ni))
    return g


def _halo_image(g, i, j, cx, cy, ni, nj):
    """Value the undecomposed domain's halo point (i, j) takes (None: untouched)."""
    ii, jj = i, j
    if not 1 <= i <= ni:
        if not cx:
            return None
        ii = (i - 1) % ni + 1
    if not 1 <= j <= nj:
        if not cy:
            return None
        jj = (j - 1) % nj + 1
    return g[:, jj, ii]


def _view(flat, region):
    off, st, n = region
    return np.lib.stride_tricks.as_strided(flat[off:], shape=(n[2], n[1], n[0]),
                                           strides=(st[2] * 8, st[1] * 8, st[0] * 8))


def _rank_body(rank, world, port, layout_args, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from mom5_gb300 import capi
    ni, nj, px, py, cx, cy, nk, ntr = layout_args
    L = decomp.Layout(ni, nj, px, py, cx, cy)
    is_, ie, js, je = L.extent(rank)
    bni, bnj = ie - is_ + 1, je - js + 1
    dims = capi.Dims(bni, bnj, nk, 0, 0, ntr, capi.BGRID)
    # a field of ntr*nk levels (the tracers of one time level) ...
    G = _global(ni, nj, ntr * nk, 7)
    F = np.zeros((ntr * nk, bnj + 2, bni + 2))
    F[:, 1:-1, 1:-1] = G[:, js:je + 1, is_:ie + 1]
    # ... and tracer_mdfl after the z pass with its strip of columns -1, 0, ni+1, ni+2
    TZ = F.copy()
    HZ = np.zeros((ntr * nk, bnj, 4))
    # after the x pass with its strip of rows -1, 0, nj+1, nj+2
    HX = np.zeros((ntr * nk, 4, bni))
    arrays = {"F": (F, F), "Z": (TZ, HZ), "X": (TZ, HX)}

    def pack(key, reg, buf):
        src = arrays[key][0].reshape(-1)
        buf.copy_(torch.from_numpy(np.ascontiguousarray(_view(src, reg)).reshape(-1)))

    def unpack(key, reg, buf):
        dst = arrays[key][1].reshape(-1)
        _view(dst, reg)[...] = buf.numpy().reshape(reg[2][2], reg[2][1], reg[2][0])

    ex = decomp.RankExchange(L, rank, pack, unpack, lambda n: torch.empty(n, dtype=torch.float64))
    ex.exchange(decomp.HALO_FIELD, dims, ntr * nk, key="F")
    ex.exchange(decomp.HALO_MDFL_Z, dims, 1, key="Z")
    ex.exchange(decomp.HALO_MDFL_X, dims, 1, key="X")
    bad = []
    # every halo point of F equals the undecomposed domain's halo rule (neighbour value,
    # periodic image, or untouched = 0 beyond a wall)
    for jl in range(bnj + 2):
        for il in range(bni + 2):
            if 1 <= il <= bni and 1 <= jl <= bnj:
                continue
            gi, gj = is_ - 1 + il, js - 1 + jl
            inside = 1 <= gi <= ni and 1 <= gj <= nj
            want = G[:, gj, gi] if inside else _halo_image(G, gi, gj, cx, cy, ni, nj)
            want = np.zeros(ntr * nk) if want is None else want
            if not np.array_equal(F[:, jl, il], want):
                bad.append(("F", il, jl))
    for s, gi_of in ((0, lambda: is_ - 2), (1, lambda: is_ - 1), (2, lambda: ie + 1), (3, lambda: ie + 2)):
        gi = gi_of()
        for jl in range(bnj):
            gj = js + jl
            v = G[:, gj, gi] if 1 <= gi <= ni else _halo_image(G, gi, gj, cx, cy, ni, nj)
            v = np.zeros(ntr * nk) if v is None else v
            if not np.array_equal(HZ[:, jl, s], v):
                bad.append(("Z", s, jl))
    for s, gj in ((0, js - 2), (1, js - 1), (2, je + 1), (3, je + 2)):
        for il in range(bni):
            gi = is_ + il
            v = G[:, gj, gi] if 1 <= gj <= nj else _halo_image(G, gi, gj, cx, cy, ni, nj)
            v = np.zeros(ntr * nk) if v is None else v
            if not np.array_equal(HX[:, s, il], v):
                bad.append(("X", s, il))
    results[rank] = bad
    dist.destroy_process_group()


@pytest.mark.parametrize("layout", [(17, 11, 2, 1, True, False), (16, 12, 2, 2, True, True),
                                    (15, 10, 1, 2, True, False), (14, 13, 2, 2, False, False)])
def test_rank_exchange_fills_every_halo_of_the_whole_domain(layout):
    ni, nj, px, py, cx, cy = layout
    world = px * py
    args = (ni, nj, px, py, cx, cy, 3, 2)
    with mp.Manager() as m:
        results = m.dict()
        mp.spawn(_rank_body, args=(world, _free_port(), args, results), nprocs=world, join=True)
        res = dict(results)
    for r in range(world):
        assert res[r] == [], f"rank {r}: {res[r][:8]}"
