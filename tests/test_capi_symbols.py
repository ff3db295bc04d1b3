"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every
entry point declared in include/mom5gpu.h (no compute calls are made)."""
import ctypes
import os
import shutil

import pytest


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not installed")
def test_library_exports_every_header_symbol():
    from mom5_gb300 import build, capi
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = capi.header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_field_ids_parse_from_header():
    from mom5_gb300 import capi
    assert capi.F.DXT == 1 and capi.F.TMASK == 40 and capi.F.TRACER == 70 and capi.F.PATM == 100
    assert len(set(capi.FIELDS.values())) == len(capi.FIELDS)


def test_error_strings_and_defaults_without_gpu():
    from mom5_gb300 import build, capi
    build.build()
    L = capi.lib()
    assert L.mom5gpu_strerror(capi.ECFL) == b"barotropic CFL violated"
    o = capi.default_options()
    assert o.pred_corr_gamma == 0.2 and o.rho0 == 1035.0 and o.initsum_with_bar == 1
    assert o.barotropic_time_stepping_A == 0 and o.barotropic_time_stepping_B == 0
