"""Domain decomposition: one ocean domain stepped as a 2-D layout of blocks.

The reference runs every domain this way: ``set_ocean_domain``
(ocean_domains.F90:123-) lays the global grid out over npes_x x npes_y
processor elements with ``mpp_define_domains``, each holding one block and a
one-cell halo, and ``mpp_update_domains`` fills the halos from the neighbours
wherever the path needs them: tracer_mdfl after the z and x passes of MDFL
(two cells, ocean_tracer_advect.F90:3912, :3970; all tracers together in the
all-tracer routine, :4213-4343), T(taup1) after the explicit update
(ocean_model.F90:1903-1911), the predicted eta in every barotropic subcycle
(ocean_barotropic.F90:3383) and the barotropic outputs after the loop
(:2846-2901).

Here a block is a non-cyclic ``capi.Domain`` of the block's size whose inputs
are set on its whole data domain (halo included, as after the reference's
halo updates); the library steps it phase by phase (``mdfl_pass``,
``barotropic_phase``) and an exchanger moves each halo region from the block
that owns it:

* ``LocalExchange``: every block in this process on one GPU; the exchange of a
  phase is one ``copy_boxes`` launch over all blocks (a block may be its own
  neighbour, as a one-block-wide layout of a periodic domain is);
* ``RankExchange``: one block per process of a ``torch.distributed`` group;
  each region is packed into a contiguous buffer, sent with ``isend``/``irecv``
  (NCCL between GPUs, gloo on the host) and unpacked on the other side.

The halo geometry comes from the library (``capi.halo_region``, host
arithmetic), so both exchangers and any other host move the same regions.
A decomposed step equals the undecomposed step value for value: this is the
reference's processor-count identity.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, replace
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import capi

WEST, EAST, SOUTH, NORTH, SOUTHWEST, SOUTHEAST, NORTHWEST, NORTHEAST = range(8)
FACES = (WEST, EAST, SOUTH, NORTH)
ALL_SIDES = tuple(range(8))
OPPOSITE = (EAST, WEST, NORTH, SOUTH, NORTHEAST, NORTHWEST, SOUTHEAST, SOUTHWEST)
STEP = {WEST: (-1, 0), EAST: (1, 0), SOUTH: (0, -1), NORTH: (0, 1), SOUTHWEST: (-1, -1), SOUTHEAST: (1, -1),
        NORTHWEST: (-1, 1), NORTHEAST: (1, 1)}
HALO_FIELD, HALO_MDFL_Z, HALO_MDFL_X, HALO_BT_ETA, HALO_BT_PS = 1, 2, 3, 4, 5
SEND, RECV = 0, 1
SIDES_OF = {HALO_FIELD: ALL_SIDES, HALO_MDFL_Z: (WEST, EAST), HALO_MDFL_X: (SOUTH, NORTH),
            HALO_BT_ETA: ALL_SIDES, HALO_BT_PS: ALL_SIDES}


def compute_extent(n: int, ndivs: int) -> List[Tuple[int, int]]:
    """Split points 1..n over ndivs blocks as mpp_compute_extent does
    (mpp_domains_define.inc:187-273, no explicit extents): each block takes the
    remaining points over the remaining blocks, rounded up, and the split is
    mirror-symmetric where the parities of n and ndivs allow it."""
    if ndivs < 1 or n < ndivs:
        raise ValueError(f"cannot split {n} points into {ndivs} blocks")
    even = lambda v: v % 2 == 0
    sym = (even(ndivs) and even(n)) or (not even(ndivs) and not even(n)) or \
          (not even(ndivs) and even(n) and ndivs < n // 2)
    beg, end = [0] * ndivs, [0] * ndivs
    imax, ndmax, start = n, ndivs, 1
    for nd in range(ndivs):
        if nd < (ndivs - 1) // 2 + 1:
            stop = start + math.ceil((imax - start + 1) / (ndmax - nd)) - 1
            mirror = ndivs - 1 - nd
            if mirror > nd and sym:
                beg[mirror] = max(1 + n - stop, stop + 1)
                end[mirror] = max(1 + n - start, stop + 1)
                imax = beg[mirror] - 1
                ndmax -= 1
        elif sym:
            start, stop = beg[nd], end[nd]
        else:
            stop = start + math.ceil((imax - start + 1) / (ndmax - nd)) - 1
        beg[nd], end[nd] = start, stop
        if stop < start:
            raise ValueError("block extents must be positive")
        start = stop + 1
    if end[-1] != n:
        raise ValueError("block extents do not span the domain")
    return list(zip(beg, end))


@dataclass
class Layout:
    """px x py blocks of an ni x nj domain; block rank r = ry*px + rx."""

    ni: int
    nj: int
    px: int
    py: int
    cyclic_x: bool = False
    cyclic_y: bool = False

    def __post_init__(self):
        self.xe = compute_extent(self.ni, self.px)
        self.ye = compute_extent(self.nj, self.py)

    @property
    def size(self) -> int:
        return self.px * self.py

    def coords(self, r: int) -> Tuple[int, int]:
        return r % self.px, r // self.px

    def extent(self, r: int) -> Tuple[int, int, int, int]:
        """(is, ie, js, je) of block r, 1-based global compute indices."""
        rx, ry = self.coords(r)
        return self.xe[rx][0], self.xe[rx][1], self.ye[ry][0], self.ye[ry][1]

    def neighbour(self, r: int, side: int) -> Optional[int]:
        """Rank of the block across `side`, wrapping in periodic directions; None at a wall."""
        rx, ry = self.coords(r)
        dx, dy = STEP[side]
        x, y = rx + dx, ry + dy
        if not 0 <= x < self.px:
            if not self.cyclic_x:
                return None
            x %= self.px
        if not 0 <= y < self.py:
            if not self.cyclic_y:
                return None
            y %= self.py
        return y * self.px + x

    def faces(self, r: int) -> Tuple[int, int, int, int]:
        """(west, east, south, north): 1 where a face looks at a block."""
        return tuple(int(self.neighbour(r, s) is not None) for s in FACES)


# ----------------------------------------------------------------------------- splitting a domain
def mask_halo2(tmask: np.ndarray, cyclic_x: bool, cyclic_y: bool) -> np.ndarray:
    """The whole domain's tmask_mdfl with a two-cell halo by the single-PE rule
    (periodic images, zero beyond walls, corners only when both directions are
    periodic): mdfl_init's halo update on one PE (ocean_tracer_advect.F90:1660-1668)."""
    nk, nyd, nxd = tmask.shape
    ni, nj = nxd - 2, nyd - 2
    m = np.zeros((nk, nj + 4, ni + 4))
    m[:, 2:nj + 2, 2:ni + 2] = tmask[:, 1:-1, 1:-1]
    if cyclic_x:
        m[:, 2:nj + 2, 0:2] = m[:, 2:nj + 2, ni:ni + 2]
        m[:, 2:nj + 2, ni + 2:ni + 4] = m[:, 2:nj + 2, 2:4]
    if cyclic_y:
        m[:, 0:2, 2:ni + 2] = m[:, nj:nj + 2, 2:ni + 2]
        m[:, nj + 2:nj + 4, 2:ni + 2] = m[:, 2:4, 2:ni + 2]
    if cyclic_x and cyclic_y:
        m[:, 0:2, 0:2] = m[:, nj:nj + 2, ni:ni + 2]
        m[:, 0:2, ni + 2:ni + 4] = m[:, nj:nj + 2, 2:4]
        m[:, nj + 2:nj + 4, 0:2] = m[:, 2:4, ni:ni + 2]
        m[:, nj + 2:nj + 4, ni + 2:ni + 4] = m[:, 2:4, 2:4]
    return m


def split(dom, layout: Layout) -> List:
    """The blocks of a ``grid.Domain``: every array cut to the block's data
    domain (compute block plus a one-cell halo taken from the whole domain's
    data domain, so halos hold the neighbours' values, or the domain's own
    halo at its edges), specs non-cyclic.  Each block also carries its
    ``mask2`` (tmask_mdfl with the two-cell halo)."""
    from .grid import Domain
    s = dom.spec
    tm = dom["tmask"].cpu().numpy()
    m2 = mask_halo2(tm, s.cyclic_x, s.cyclic_y)
    out = []
    for r in range(layout.size):
        is_, ie, js, je = layout.extent(r)
        sl = (slice(js - 1, je + 2), slice(is_ - 1, ie + 2))
        f = {k: v[(Ellipsis,) + sl].contiguous().clone() for k, v in dom.f.items()}
        spec = replace(s, ni=ie - is_ + 1, nj=je - js + 1, cyclic_x=False, cyclic_y=False)
        b = Domain(spec, f, dom.dzt, dom.zw)
        b.mask2 = np.ascontiguousarray(m2[:, js - 1:je + 4, is_ - 1:ie + 4])
        b.extent = (is_, ie, js, je)
        out.append(b)
    return out


def join(blocks: Sequence[np.ndarray], layout: Layout, with_halo: bool = True) -> np.ndarray:
    """Reassemble per-block data-domain arrays [..., nj_b+2, ni_b+2] into the
    whole domain's [..., nj+2, ni+2]: compute cells from their owner; halo
    cells of the whole domain from the blocks at its edges."""
    lead = blocks[0].shape[:-2]
    out = np.zeros(lead + (layout.nj + 2, layout.ni + 2))
    for r, a in enumerate(blocks):
        is_, ie, js, je = layout.extent(r)
        rx, ry = layout.coords(r)
        j0 = js - 1 if (with_halo and ry == 0) else js
        j1 = je + 1 if (with_halo and ry == layout.py - 1) else je
        i0 = is_ - 1 if (with_halo and rx == 0) else is_
        i1 = ie + 1 if (with_halo and rx == layout.px - 1) else ie
        out[..., j0:j1 + 1, i0:i1 + 1] = a[..., j0 - js + 1:j1 - js + 2, i0 - is_ + 1:i1 - is_ + 2]
    return out


# ----------------------------------------------------------------------------- exchangers
def _nlev(d: "capi.Domain", kind: int, field: int, n: int) -> int:
    if kind != HALO_FIELD:
        return 1
    cnt = d.count(field)
    n2 = (d.dims.ni + 2) * (d.dims.nj + 2)
    lev = cnt // n2
    if field == capi.F.TRACER and n == 0:
        lev *= d.dims.num_prog_tracers
    return lev


class LocalExchange:
    """Every block of the layout in this process, on one GPU: each exchange is
    one copy_boxes launch (on `stream`) over every block's halo regions."""

    def __init__(self, blocks: Sequence["capi.Domain"], layout: Layout, stream: Optional[int] = None):
        self.blocks, self.layout, self.stream = list(blocks), layout, stream

    def exchange(self, kind: int, field: int = 0, n: int = 0, level: int = 0):
        boxes = []
        for r, d in enumerate(self.blocks):
            nlev = _nlev(d, kind, field, n)
            dst_base = d.halo_base(kind, RECV, field, n, level)
            for side in SIDES_OF[kind]:
                q = self.layout.neighbour(r, side)
                if q is None:
                    continue
                src = self.blocks[q]
                s_off, s_st, s_n = capi.halo_region(src.dims, kind, nlev, OPPOSITE[side], SEND)
                d_off, d_st, d_n = capi.halo_region(d.dims, kind, nlev, side, RECV)
                if s_n != d_n:
                    raise ValueError(f"block {q} sends {s_n} to block {r}'s side {side}, which holds {d_n}")
                src_base = src.halo_base(kind, SEND, field, n, level)
                boxes.append(capi.Box(src_base + 8 * s_off, dst_base + 8 * d_off, s_st, d_st, d_n))
        capi.copy_boxes(boxes, self.stream)


def add_fixed(a, b):
    """Element-by-element sum of two fixed-point accumulator lists (exact)."""
    return [int(x) + int(y) for x, y in zip(a, b)]


class RankExchange:
    """One block per process of a torch.distributed group (rank r = block r):
    each region goes through a contiguous buffer, isend / irecv with the
    neighbour's rank, tagged by the receiving side.  ``pack``/``unpack`` move a
    region between the block's memory and a buffer (on GPU: copy_boxes; any
    host array store works the same way)."""

    def __init__(self, layout: Layout, rank: int, pack, unpack, new_buffer, group=None):
        self.layout, self.rank, self.group = layout, rank, group
        self.pack, self.unpack, self.new_buffer = pack, unpack, new_buffer

    def plan(self, kind: int, dims: "capi.Dims", nlev: int):
        """[(side, peer rank, send region, recv region)] of this rank for `kind`."""
        out = []
        for side in SIDES_OF[kind]:
            q = self.layout.neighbour(self.rank, side)
            if q is None:
                continue
            out.append((side, q, capi.halo_region(dims, kind, nlev, side, SEND),
                        capi.halo_region(dims, kind, nlev, side, RECV)))
        return out

    def exchange(self, kind: int, dims: "capi.Dims", nlev: int, key=None):
        """Send every region this block owes its neighbours and fill its halo
        regions from theirs.  What goes towards `side` arrives on the
        neighbour's OPPOSITE side; messages are tagged with the receiving
        side, so a peer on two sides (two blocks across a periodic direction)
        is matched per side."""
        import torch.distributed as dist
        plan = self.plan(kind, dims, nlev)
        recv_of = {side: recv_reg for side, _, _, recv_reg in plan}
        ops, landed = [], []
        for side, q, send_reg, recv_reg in plan:
            sbuf = self.new_buffer(int(np.prod(send_reg[2])))
            self.pack(key, send_reg, sbuf)
            if q == self.rank:  # its own neighbour (one block across a periodic direction)
                landed.append((recv_of[OPPOSITE[side]], sbuf))
                continue
            rbuf = self.new_buffer(int(np.prod(recv_reg[2])))
            ops.append(dist.P2POp(dist.isend, sbuf, q, self.group, tag=OPPOSITE[side]))
            ops.append(dist.P2POp(dist.irecv, rbuf, q, self.group, tag=side))
            landed.append((recv_reg, rbuf))
        if ops:
            for req in dist.batch_isend_irecv(ops):
                req.wait()
        for recv_reg, buf in landed:
            self.unpack(key, recv_reg, buf)

    def allreduce_fixed(self, acc):
        """Sum fixed-point accumulators over the ranks: an integer allreduce,
        exact and independent of the reduction order, so every rank gets the
        whole domain's accumulators."""
        import torch
        import torch.distributed as dist
        t = torch.tensor([int(v) for v in acc], dtype=torch.int64)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)
        return [int(v) for v in t.tolist()]


# ----------------------------------------------------------------------------- stepping
class Decomposed:
    """Steps the blocks of one domain with the reference's halo updates between
    the phases.  `exchanger.exchange(kind, field, n, level)` moves the halos."""

    def __init__(self, blocks: Sequence["capi.Domain"], layout: Layout, exchanger):
        self.blocks, self.layout, self.ex = list(blocks), layout, exchanger

    @staticmethod
    def prepare(d: "capi.Domain", layout: Layout, r: int, mask2: Optional[np.ndarray] = None):
        """Mark block r's faces and set its tmask_mdfl halo (after tracer_advect_init)."""
        d.set_neighbours(*layout.faces(r))
        if mask2 is not None and d.dims.num_prog_tracers > 0:
            d.set_mask_halo2(mask2)

    def tracer_advection_step(self, taum1: int, tau: int, taup1: int, dtime: float):
        """update_advection_only for every tracer with MDFL (FP64), decomposed."""
        for d in self.blocks:
            d.mdfl_pass(1, taum1, tau, dtime)
        self.ex.exchange(HALO_MDFL_Z)
        for d in self.blocks:
            d.mdfl_pass(2, taum1, tau, dtime)
        self.ex.exchange(HALO_MDFL_X)
        for d in self.blocks:
            d.mdfl_pass(3, taum1, tau, dtime)
            d.update_tracer(0, taum1, taup1, dtime)
        self.ex.exchange(HALO_FIELD, capi.F.TRACER, 0, taup1)

    def global_tracer_content(self, n: int, level: int) -> float:
        """Global content of tracer n over every block: the blocks' exact
        fixed-point accumulators added (and summed over the ranks when the
        exchanger has ranks), rounded once -- the same double for every
        decomposition of the domain, the undecomposed one included."""
        acc = [0] * capi.FIXED_CHUNKS
        for d in self.blocks:
            acc = add_fixed(acc, d.tracer_content_fixed(n, level))
        if hasattr(self.ex, "allreduce_fixed"):
            acc = self.ex.allreduce_fixed(acc)
        return capi.fixed_to_double(acc)

    def update_ocean_barotropic(self, tau: int, taup1: int):
        """update_ocean_barotropic (B grid, FP64), decomposed: a halo update of
        the predicted eta and pressure in every subcycle, of the averages and
        the derived fields after the loop."""
        nts = self.blocks[0].nts
        for d in self.blocks:
            d.barotropic_phase(tau, taup1, 0)
        for itime in range(1, nts + 1):
            for d in self.blocks:
                d.barotropic_phase(tau, taup1, 1, itime)
            self.ex.exchange(HALO_BT_ETA, 0, 0, (itime + 1) % 2)
            self.ex.exchange(HALO_BT_PS)
            for d in self.blocks:
                d.barotropic_phase(tau, taup1, 2, itime)
        for d in self.blocks:
            d.barotropic_phase(tau, taup1, 3)
        for f in (capi.F.ETA_T_BAR, capi.F.UDRHO_U, capi.F.UDRHO_V):
            self.ex.exchange(HALO_FIELD, f, 0, taup1)
        for d in self.blocks:
            d.barotropic_phase(tau, taup1, 4)
        for f in (capi.F.CONV_RHO_UD_T, capi.F.ETA_U):
            self.ex.exchange(HALO_FIELD, f, 0, taup1)
        for d in self.blocks:
            d.barotropic_phase(tau, taup1, 5)
