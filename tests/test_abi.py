"""The C-ABI library builds, loads and exports every entry point that
include/hystrath_gb300.h declares; without a GPU it refuses to create a
cloud instead of falling back to the CPU."""
import ctypes
import os
import re

import pytest

from hystrath_gb300 import spec as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(dsmc_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("dsmc_create", "dsmc_create_from_spec", "dsmc_initialise", "dsmc_evolve",
                     "dsmc_info", "dsmc_get_field", "dsmc_checkpoint", "dsmc_restore",
                     "dsmc_last_error", "dsmc_destroy"):
        assert required in names


def test_library_exports_every_declared_symbol(gpu_lib):
    for name in declared_functions():
        assert hasattr(gpu_lib, name), name


def test_struct_layout_matches_header(gpu_lib):
    # dsmc_spec_defaults writes the C struct; the ctypes mirror must read the defaults back
    s = S.CaseSpec()
    gpu_lib.dsmc_spec_defaults(ctypes.byref(s))
    assert s.tref == 273.0 and s.zrot == 5.0 and s.inv_zv_formulation == 2 and s.mfp_tref == 273.0
    gpu_lib.dsmc_case_spec_size.restype = ctypes.c_longlong
    assert gpu_lib.dsmc_case_spec_size() == ctypes.sizeof(S.CaseSpec)
    assert not any(bool(s.node_coords[a]) for a in range(3))


def test_no_cpu_fallback_without_gpu(gpu_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from hystrath_gb300.dsmc import DsmcCloud, DsmcError
    with pytest.raises(DsmcError) as e:
        DsmcCloud(S.config0())
    assert e.value.code == S.ERR_NO_DEVICE
