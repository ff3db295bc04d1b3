"""ctypes binding of libmom5gpu.so (the C ABI in include/mom5gpu.h).

This is the Python-side caller of the same entry points a Fortran host binds
through ISO_C_BINDING.  There is no fallback: if the compiled library is
missing or a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmom5gpu.so")
HEADER = os.path.join(HERE, "..", "include", "mom5gpu.h")

_lib: Optional[C.CDLL] = None

# ---- constants mirrored from include/mom5gpu.h ----
OK = 0
EINVAL, ENOMEM, ECUDA, ESTATE, ECFL, ENUMERIC, ETIMEDOUT, EUNSUPPORTED, EFULL = range(-1, -10, -1)
BGRID, CGRID = 1, 2
ADVECT_UPWIND, ADVECT_QUICKER, ADVECT_MDFL_SWEBY, ADVECT_DST_LINEAR = 1, 5, 9, 10
ADVECT_2ND_ORDER, ADVECT_4TH_ORDER, ADVECT_6TH_ORDER, ADVECT_MDFL_SUP_B, ADVECT_MDPPM = 2, 3, 4, 7, 8
ADVECT_PSOM = 11
ADVECT_QUICKMOM3 = 6
PRECISION_FP64, PRECISION_MIXED = 0, 1
GEOPOTENTIAL, ZSTAR, ZSIGMA, PRESSURE, PSTAR, PSIGMA = 1, 2, 3, 4, 5, 6


def _enum_values() -> dict:
    """Field ids parsed from the header's enum (single source of truth)."""
    txt = open(HEADER).read()
    body = txt[txt.index("enum mom5gpu_field"):]
    body = body[body.index("{") + 1: body.index("};")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    vals, cur = {}, 0
    for tok in body.replace("\n", " ").split(","):
        tok = tok.strip()
        if not tok:
            continue
        if "=" in tok:
            name, v = [x.strip() for x in tok.split("=")]
            cur = int(v)
        else:
            name = tok
        vals[name] = cur
        cur += 1
    return vals


FIELDS = _enum_values()
F = type("F", (), {k.replace("MOM5GPU_", ""): v for k, v in FIELDS.items()})


class Dims(C.Structure):
    _fields_ = [("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int), ("cyclic_x", C.c_int), ("cyclic_y", C.c_int),
                ("num_prog_tracers", C.c_int), ("horz_grid", C.c_int)]


class Options(C.Structure):
    _fields_ = [("advect_sweby_all", C.c_int), ("limit_with_upwind", C.c_int),
                ("zero_tracer_advect_horz", C.c_int), ("zero_tracer_advect_vert", C.c_int),
                ("barotropic_time_stepping_A", C.c_int), ("barotropic_time_stepping_B", C.c_int),
                ("initsum_with_bar", C.c_int), ("pred_corr_gamma", C.c_double), ("rho0", C.c_double),
                ("grav", C.c_double), ("precision", C.c_int), ("zero_forcing_bt", C.c_int),
                ("zero_nonlinear_forcing_bt", C.c_int), ("psom_limit_prather", C.c_int),
                ("udrho_lap", C.c_int), ("udrho_bih", C.c_int), ("udrho_lap_vel_micom", C.c_double),
                ("udrho_bih_vel_micom", C.c_double)]


class Box(C.Structure):
    """mom5gpu_box: a strided 3-D box of doubles, copied src -> dst."""
    _fields_ = [("src", C.c_void_p), ("dst", C.c_void_p), ("src_stride", C.c_long * 3),
                ("dst_stride", C.c_long * 3), ("n", C.c_int * 3)]


class Mom5GpuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with mom5_gb300.build.build() "
                              "(nvcc, sm_103a); there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        sig = {
            "mom5gpu_default_options": (None, [C.POINTER(Options)]),
            "mom5gpu_create": (C.c_int, [C.POINTER(Dims), C.POINTER(Options), C.POINTER(vp)]),
            "mom5gpu_destroy": (None, [vp]),
            "mom5gpu_last_error": (C.c_char_p, [vp]),
            "mom5gpu_strerror": (C.c_char_p, [C.c_int]),
            "mom5gpu_set_stream": (C.c_int, [vp, vp]),
            "mom5gpu_synchronize": (C.c_int, [vp]),
            "mom5gpu_device_bytes": (C.c_size_t, [vp]),
            "mom5gpu_field_count": (C.c_size_t, [vp, C.c_int]),
            "mom5gpu_set_field": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, vp, C.c_int]),
            "mom5gpu_get_field": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, vp, C.c_int]),
            "mom5gpu_field_device_ptr": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.POINTER(vp)]),
            "mom5gpu_set_vertical_grid": (C.c_int, [vp, dp, dp, ip]),
            "mom5gpu_set_tracer_scheme": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]),
            "mom5gpu_tracer_advect_init": (C.c_int, [vp]),
            "mom5gpu_barotropic_init": (C.c_int, [vp, C.c_double, C.c_double]),
            "mom5gpu_barotropic_nts": (C.c_int, [vp]),
            "mom5gpu_horz_advect_tracer": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_double]),
            "mom5gpu_vert_advect_tracer": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_double]),
            "mom5gpu_advect_tracer_sweby_all": (C.c_int, [vp, C.c_int, C.c_int, C.c_double]),
            "mom5gpu_compute_tmask_limit": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
            "mom5gpu_zero_th_tendency": (C.c_int, [vp, C.c_int]),
            "mom5gpu_update_tracer": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_double]),
            "mom5gpu_tracer_advection_step": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_double]),
            "mom5gpu_eta_and_pbot_tendency": (C.c_int, [vp, C.c_int]),
            "mom5gpu_eta_and_pbot_update": (C.c_int, [vp, C.c_int, C.c_int, C.c_double]),
            "mom5gpu_update_ocean_barotropic": (C.c_int, [vp, C.c_int, C.c_int]),
            "mom5gpu_ocean_advection_velocity": (C.c_int, [vp, C.c_int]),
            "mom5gpu_autotune": (C.c_int, [vp, C.c_double, C.c_char_p, C.c_size_t]),
            "mom5gpu_tracer_boundary_terms": (C.c_int, [vp, C.c_int]),
            "mom5gpu_set_ppm_limiter": (C.c_int, [vp, C.c_int, C.c_int]),
            "mom5gpu_set_psom_limit": (C.c_int, [vp, C.c_int, C.c_int]),
            "mom5gpu_set_itt0": (C.c_int, [vp, C.c_long]),
            "mom5gpu_set_tuning": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
            "mom5gpu_set_barotropic_fusion": (C.c_int, [vp, C.c_int]),
            "mom5gpu_grid_barrier_selftest": (C.c_int, [vp, C.c_int, C.c_int]),
            "mom5gpu_get_tuning": (C.c_int, [vp, ip, ip, ip]),
            "mom5gpu_copy_field_async": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p]),
            "mom5gpu_set_tracer_name": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_char_p]),
            "mom5gpu_write_restart": (C.c_int, [vp, C.c_char_p, C.c_int]),
            "mom5gpu_read_restart": (C.c_int, [vp, C.c_char_p, C.c_int]),
            "mom5gpu_ocean_barotropic_forcing": (C.c_int, [vp]),
            "mom5gpu_ocean_barotropic_forcing_tau": (C.c_int, [vp, C.c_int]),
            "mom5gpu_update_ucell_thickness": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
            "mom5gpu_global_tracer_content": (C.c_int, [vp, C.c_int, C.c_int, dp]),
            "mom5gpu_tracer_content_fixed": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(C.c_longlong)]),
            "mom5gpu_fixed_to_double": (C.c_int, [C.POINTER(C.c_longlong), dp]),
            "mom5gpu_global_eta_integral": (C.c_int, [vp, C.c_int, C.c_int, dp]),
            "mom5gpu_check_finite": (C.c_int, [vp, C.c_int, C.c_int, ip]),
            "mom5gpu_enable_timing": (C.c_int, [vp, C.c_int]),
            "mom5gpu_timing_query": (C.c_int, [vp, C.c_char_p, dp, C.POINTER(C.c_long)]),
            "mom5gpu_launch_count": (C.c_long, [vp]),
            "mom5gpu_mdfl_sweby_noalloc": (C.c_int, [C.POINTER(Dims), C.c_int, C.c_double] + [vp] * 14),
            "mom5gpu_set_neighbours": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
            "mom5gpu_set_mask_halo2": (C.c_int, [vp, dp]),
            "mom5gpu_halo_region": (C.c_int, [C.POINTER(Dims), C.c_int, C.c_int, C.c_int, C.c_int,
                                              C.POINTER(C.c_long), C.c_long * 3, C.c_int * 3]),
            "mom5gpu_halo_base": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(vp)]),
            "mom5gpu_copy_boxes": (C.c_int, [C.POINTER(Box), C.c_int, vp]),
            "mom5gpu_mdfl_pass": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_double]),
            "mom5gpu_barotropic_phase": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
            "mom5gpu_batch_create": (C.c_int, [C.POINTER(vp), C.c_int, C.POINTER(vp)]),
            "mom5gpu_batch_destroy": (None, [vp]),
            "mom5gpu_batch_last_error": (C.c_char_p, [vp]),
            "mom5gpu_batch_set_stream": (C.c_int, [vp, vp]),
            "mom5gpu_batch_step": (C.c_int, [vp, ip, ip, C.c_int, C.c_double]),
            "mom5gpu_batch_autotune": (C.c_int, [vp, C.c_double, C.c_char_p, C.c_size_t]),
            "mom5gpu_batch_get_tuning": (C.c_int, [vp, ip, ip, ip]),
            "mom5gpu_batch_set_tuning": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
            "mom5gpu_batch_last_ms": (C.c_double, [vp]),
            "mom5gpu_batch_launch_count": (C.c_long, [vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


FIXED_CHUNKS = 8  # MOM5GPU_FIXED_CHUNKS


def fixed_to_double(acc) -> float:
    """The double nearest to a sum of fixed-point content accumulators
    (mom5gpu_fixed_to_double; no device needed)."""
    if len(acc) != FIXED_CHUNKS:
        raise ValueError(f"{FIXED_CHUNKS} accumulators expected")
    if any(not -(1 << 63) <= int(v) < (1 << 63) for v in acc):
        raise OverflowError("an accumulator exceeds 64 bits: too many values in one sum")
    a = (C.c_longlong * FIXED_CHUNKS)(*[int(v) for v in acc])
    out = C.c_double()
    st = lib().mom5gpu_fixed_to_double(a, C.byref(out))
    if st:
        raise Mom5GpuError(st, "fixed_to_double")
    return out.value


def default_options(**kw) -> Options:
    o = Options()
    lib().mom5gpu_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _ptr(a):
    """(address, on_device) of a contiguous float64 numpy array or torch tensor."""
    if isinstance(a, np.ndarray):
        assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
        return a.ctypes.data, 0
    import torch  # device tensors (plumbing only)
    assert a.dtype == torch.float64 and a.is_contiguous()
    return a.data_ptr(), int(a.is_cuda)


class Domain:
    """One device-resident ocean domain (mom5gpu_domain)."""

    def __init__(self, ni, nj, nk, ntracers, cyclic_x=False, cyclic_y=False, horz_grid=BGRID,
                 options: Optional[Options] = None):
        self.dims = Dims(ni, nj, nk, int(cyclic_x), int(cyclic_y), ntracers, horz_grid)
        self.options = options if options is not None else default_options()
        h = C.c_void_p()
        st = lib().mom5gpu_create(C.byref(self.dims), C.byref(self.options), C.byref(h))
        if st != OK:
            raise Mom5GpuError(st, lib().mom5gpu_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().mom5gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st: int):
        if st != OK:
            raise Mom5GpuError(st, lib().mom5gpu_last_error(self.h).decode())
        return st

    # ---- data movement ----
    def count(self, field: int) -> int:
        return lib().mom5gpu_field_count(self.h, field)

    def set(self, field: int, a, n: int = 0, level: int = 0):
        addr, dev = _ptr(a)
        nbytes = a.nbytes if isinstance(a, np.ndarray) else a.numel() * 8
        assert nbytes == 8 * self.count(field), (field, nbytes, self.count(field))
        self.check(lib().mom5gpu_set_field(self.h, field, n, level, C.c_void_p(addr), dev))

    def get(self, field: int, n: int = 0, level: int = 0) -> np.ndarray:
        out = np.empty(self.count(field), dtype=np.float64)
        self.check(lib().mom5gpu_get_field(self.h, field, n, level, out.ctypes.data_as(C.c_void_p), 0))
        return out

    def device_ptr(self, field: int, n: int = 0, level: int = 0) -> int:
        p = C.c_void_p()
        self.check(lib().mom5gpu_field_device_ptr(self.h, field, n, level, C.byref(p)))
        return p.value

    def set_vertical_grid(self, dzt, zw, kmt):
        dzt = np.ascontiguousarray(dzt, dtype=np.float64)
        zw = np.ascontiguousarray(zw, dtype=np.float64)
        kmt = np.ascontiguousarray(kmt, dtype=np.int32)
        self.check(lib().mom5gpu_set_vertical_grid(self.h, dzt.ctypes.data_as(C.POINTER(C.c_double)),
                                                   zw.ctypes.data_as(C.POINTER(C.c_double)),
                                                   kmt.ctypes.data_as(C.POINTER(C.c_int))))

    def set_tracer_scheme(self, n, horz, vert=None, min_limit=-1.0e10, max_limit=1.0e10):
        self.check(lib().mom5gpu_set_tracer_scheme(self.h, n, horz, horz if vert is None else vert,
                                                   float(min_limit), float(max_limit)))

    def set_stream(self, stream_ptr: int):
        self.check(lib().mom5gpu_set_stream(self.h, C.c_void_p(stream_ptr)))

    def synchronize(self):
        self.check(lib().mom5gpu_synchronize(self.h))

    @property
    def device_bytes(self) -> int:
        return lib().mom5gpu_device_bytes(self.h)

    # ---- init ----
    def tracer_advect_init(self):
        self.check(lib().mom5gpu_tracer_advect_init(self.h))

    def barotropic_init(self, dtuv: float, dtbt: float) -> int:
        self.check(lib().mom5gpu_barotropic_init(self.h, float(dtuv), float(dtbt)))
        return lib().mom5gpu_barotropic_nts(self.h)

    @property
    def nts(self) -> int:
        """Barotropic subcycles per step (0 before barotropic_init)."""
        return lib().mom5gpu_barotropic_nts(self.h)

    # ---- hot path (reference names) ----
    def horz_advect_tracer(self, n, taum1, tau, dtime):
        self.check(lib().mom5gpu_horz_advect_tracer(self.h, n, taum1, tau, float(dtime)))

    def vert_advect_tracer(self, n, taum1, tau, dtime):
        self.check(lib().mom5gpu_vert_advect_tracer(self.h, n, taum1, tau, float(dtime)))

    def advect_tracer_sweby_all(self, taum1, tau, dtime):
        self.check(lib().mom5gpu_advect_tracer_sweby_all(self.h, taum1, tau, float(dtime)))

    def compute_tmask_limit(self, tau, index_temp=0, index_salt=0):
        self.check(lib().mom5gpu_compute_tmask_limit(self.h, tau, index_temp, index_salt))

    def zero_th_tendency(self, n=0):
        self.check(lib().mom5gpu_zero_th_tendency(self.h, n))

    def update_tracer(self, n, taum1, taup1, dtime):
        self.check(lib().mom5gpu_update_tracer(self.h, n, taum1, taup1, float(dtime)))

    def tracer_advection_step(self, taum1, tau, taup1, dtime):
        self.check(lib().mom5gpu_tracer_advection_step(self.h, taum1, tau, taup1, float(dtime)))

    def eta_and_pbot_tendency(self, tau):
        self.check(lib().mom5gpu_eta_and_pbot_tendency(self.h, tau))

    def eta_and_pbot_update(self, taum1, taup1, dtime):
        self.check(lib().mom5gpu_eta_and_pbot_update(self.h, taum1, taup1, float(dtime)))

    def update_ocean_barotropic(self, tau, taup1):
        self.check(lib().mom5gpu_update_ocean_barotropic(self.h, tau, taup1))

    # ---- diagnostics ----
    def autotune(self, dtime) -> str:
        buf = C.create_string_buffer(1024)
        self.check(lib().mom5gpu_autotune(self.h, float(dtime), buf, 1024))
        return buf.value.decode()

    def set_ppm_limiter(self, n, limiter):
        self.check(lib().mom5gpu_set_ppm_limiter(self.h, n, limiter))

    def set_psom_limit(self, n, on):
        self.check(lib().mom5gpu_set_psom_limit(self.h, n, int(bool(on))))

    @property
    def tuning(self):
        r, p, t = C.c_int(), C.c_int(), C.c_int()
        self.check(lib().mom5gpu_get_tuning(self.h, C.byref(r), C.byref(p), C.byref(t)))
        return r.value, p.value, t.value

    @tuning.setter
    def tuning(self, v):
        rows, prefetch, tj = v
        self.check(lib().mom5gpu_set_tuning(self.h, rows, int(prefetch), tj))

    def set_barotropic_fusion(self, mode: int):
        """Exact B-grid subcycles: 0 (default) three launches each, 1 one
        launch each, 2 all in one cooperative launch."""
        self.check(lib().mom5gpu_set_barotropic_fusion(self.h, int(mode)))

    def grid_barrier_selftest(self, rounds: int, unreachable: bool = False):
        """Run the cooperative grid barrier `rounds` times and check its order;
        with unreachable the waits run out and the next synchronize raises
        ETIMEDOUT."""
        self.check(lib().mom5gpu_grid_barrier_selftest(self.h, int(rounds), 1 if unreachable else 0))
        self.synchronize()

    def set_itt0(self, itt0):
        self.check(lib().mom5gpu_set_itt0(self.h, int(itt0)))

    # ---- decomposed blocks (decomp.py) ----
    def set_neighbours(self, west, east, south, north):
        self.check(lib().mom5gpu_set_neighbours(self.h, int(west), int(east), int(south), int(north)))

    def set_mask_halo2(self, mask):
        m = np.ascontiguousarray(mask, dtype=np.float64)
        dm = self.dims
        if m.size != (dm.ni + 4) * (dm.nj + 4) * dm.nk:
            raise ValueError(f"tmask with a two-cell halo has {(dm.ni + 4) * (dm.nj + 4) * dm.nk} values, got {m.size}")
        self.check(lib().mom5gpu_set_mask_halo2(self.h, m.ctypes.data_as(C.POINTER(C.c_double))))

    def halo_base(self, kind, role, field=0, n=0, level=0) -> int:
        p = C.c_void_p()
        self.check(lib().mom5gpu_halo_base(self.h, kind, field, n, level, role, C.byref(p)))
        return p.value

    def mdfl_pass(self, pass_, taum1, tau, dtime):
        self.check(lib().mom5gpu_mdfl_pass(self.h, int(pass_), taum1, tau, float(dtime)))

    def barotropic_phase(self, tau, taup1, phase, itime=0):
        self.check(lib().mom5gpu_barotropic_phase(self.h, tau, taup1, int(phase), int(itime)))

    def copy_field_async(self, field, host_ptr, to_device, stream=None, n=0, level=0):
        """Stream-ordered copy between the field and host memory at host_ptr (an
        address; pinned for overlap); stream is a cudaStream_t handle or None."""
        self.check(lib().mom5gpu_copy_field_async(self.h, field, n, level, C.c_void_p(host_ptr), int(to_device),
                                                  C.c_void_p(stream) if stream else None))

    def set_tracer_name(self, n, name, restart_file=None):
        self.check(lib().mom5gpu_set_tracer_name(self.h, n, name.encode(),
                                                 restart_file.encode() if restart_file else None))

    def write_restart(self, directory, level):
        self.check(lib().mom5gpu_write_restart(self.h, os.fsencode(directory), level))

    def read_restart(self, directory, level):
        self.check(lib().mom5gpu_read_restart(self.h, os.fsencode(directory), level))

    def tracer_boundary_terms(self, n=0):
        self.check(lib().mom5gpu_tracer_boundary_terms(self.h, n))

    def ocean_barotropic_forcing(self, tau=None):
        """ocean_barotropic_forcing; with tau (Time%tau), the barotropic friction on
        udrho(tau) too (options udrho_lap / udrho_bih)."""
        if tau is None:
            self.check(lib().mom5gpu_ocean_barotropic_forcing(self.h))
        else:
            self.check(lib().mom5gpu_ocean_barotropic_forcing_tau(self.h, tau))

    def update_ucell_thickness(self, taup1, vert_coordinate=GEOPOTENTIAL, linear_free_surface=False,
                               update_dzwu_k0=True):
        self.check(lib().mom5gpu_update_ucell_thickness(self.h, taup1, vert_coordinate, int(linear_free_surface),
                                                        int(update_dzwu_k0)))

    def ocean_advection_velocity(self, tau):
        self.check(lib().mom5gpu_ocean_advection_velocity(self.h, tau))

    def global_tracer_content(self, n, level) -> float:
        out = C.c_double()
        self.check(lib().mom5gpu_global_tracer_content(self.h, n, level, C.byref(out)))
        return out.value

    def tracer_content_fixed(self, n, level) -> list:
        """The exact fixed-point accumulators of tracer n's content (FIXED_CHUNKS
        Python ints; add them element by element across blocks, then
        fixed_to_double)."""
        acc = (C.c_longlong * FIXED_CHUNKS)()
        self.check(lib().mom5gpu_tracer_content_fixed(self.h, n, level, acc))
        return [int(v) for v in acc]

    def global_eta_integral(self, field, level) -> float:
        out = C.c_double()
        self.check(lib().mom5gpu_global_eta_integral(self.h, field, level, C.byref(out)))
        return out.value

    def enable_timing(self, on=True):
        self.check(lib().mom5gpu_enable_timing(self.h, int(on)))

    def timing(self, section: str):
        ms, calls = C.c_double(), C.c_long()
        self.check(lib().mom5gpu_timing_query(self.h, section.encode(), C.byref(ms), C.byref(calls)))
        return ms.value, calls.value

    @property
    def launches(self) -> int:
        return lib().mom5gpu_launch_count(self.h)

    def check_finite(self, n=0, level=1) -> bool:
        out = C.c_int()
        self.check(lib().mom5gpu_check_finite(self.h, n, level, C.byref(out)))
        return out.value == 0


class Batch:
    """A mom5gpu_batch over resident domains (they must outlive the batch)."""

    def __init__(self, domains):
        self.domains = list(domains)
        arr = (C.c_void_p * len(self.domains))(*[d.h.value for d in self.domains])
        h = C.c_void_p()
        st = lib().mom5gpu_batch_create(arr, len(self.domains), C.byref(h))
        if st != OK:
            raise Mom5GpuError(st, lib().mom5gpu_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().mom5gpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st):
        if st != OK:
            raise Mom5GpuError(st, lib().mom5gpu_batch_last_error(self.h).decode())

    def step(self, dtime, index=None, parity=None):
        """Step the listed domains (all with parity[0] through the CUDA graph when index is None)."""
        if index is None:
            p = (C.c_int * 1)(int(parity if parity is not None else 0))
            self.check(lib().mom5gpu_batch_step(self.h, None, p, -1, float(dtime)))
            return
        n = len(index)
        ia = (C.c_int * n)(*index)
        pa = (C.c_int * n)(*parity)
        self.check(lib().mom5gpu_batch_step(self.h, ia, pa, n, float(dtime)))

    def autotune(self, dtime) -> str:
        buf = C.create_string_buffer(1024)
        self.check(lib().mom5gpu_batch_autotune(self.h, float(dtime), buf, 1024))
        return buf.value.decode()

    def set_stream(self, stream_ptr: int):
        self.check(lib().mom5gpu_batch_set_stream(self.h, C.c_void_p(stream_ptr)))

    @property
    def tuning(self):
        r, t, b = C.c_int(), C.c_int(), C.c_int()
        self.check(lib().mom5gpu_batch_get_tuning(self.h, C.byref(r), C.byref(t), C.byref(b)))
        return (r.value, t.value, b.value)

    @tuning.setter
    def tuning(self, v):
        self.check(lib().mom5gpu_batch_set_tuning(self.h, int(v[0]), int(v[1]), int(v[2])))

    @property
    def last_ms(self) -> float:
        return lib().mom5gpu_batch_last_ms(self.h)

    @property
    def launches(self) -> int:
        return lib().mom5gpu_batch_launch_count(self.h)


def header_symbols():
    """Every function the header declares."""
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return sorted(set(re.findall(r"\b(mom5gpu_[a-z0-9_]+)\s*\(", txt)))


def halo_region(dims: Dims, kind: int, nlev: int, side: int, role: int):
    """(offset, strides, extents) of a halo region relative to its array's base
    (mom5gpu_halo_region: host arithmetic only, no device needed)."""
    off, st, n = C.c_long(), (C.c_long * 3)(), (C.c_int * 3)()
    r = lib().mom5gpu_halo_region(C.byref(dims), kind, nlev, side, role, C.byref(off), st, n)
    if r != OK:
        raise Mom5GpuError(r, f"halo_region(kind={kind}, side={side}, role={role})")
    return off.value, tuple(st), tuple(n)


def copy_boxes(boxes, stream=None):
    """One launch copying every Box in `boxes` (device memory)."""
    if not boxes:
        return
    arr = (Box * len(boxes))(*boxes)
    r = lib().mom5gpu_copy_boxes(arr, len(boxes), C.c_void_p(stream) if stream else None)
    if r != OK:
        raise Mom5GpuError(r, lib().mom5gpu_last_error(None).decode())
