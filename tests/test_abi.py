"""The C-ABI library loads without a GPU and exports what include/sphnj.h
declares; the ctypes mirror matches the header layout."""
import ctypes as C
import re
from pathlib import Path

import sphnj_gb300 as S
from sphnj_gb300 import abi

HEADER = Path(__file__).resolve().parents[1] / "include" / "sphnj.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sphnj_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_context_api():
    names = declared_functions()
    for must in ("sphnj_create", "sphnj_upload", "sphnj_step", "sphnj_download", "sphnj_debug_cells",
                 "sphnj_last_error", "sphnj_destroy", "sphnj_params_read_ini", "sphnj_read_particles"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(S.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layout_matches_header():
    L = S.lib()
    assert L.sphnj_abi_sizeof(0) == C.sizeof(abi.Params)
    assert L.sphnj_abi_sizeof(1) == C.sizeof(abi.HostState)
    assert L.sphnj_abi_sizeof(7) == -1


def test_enum_values_match_reference_types():
    # include/types.h:4-67
    assert (abi.LIQUID, abi.GAS) == (0, 1)
    assert (abi.SLIP, abi.NO_SLIP, abi.MOVING) == (0, 1, 2)
    assert (abi.SPLASH, abi.FREE_SURFACE, abi.VICINITY, abi.INNER) == (0, 1, 2, 3)
    assert (abi.NO_PARTICLE, abi.HAS_PARTICLE, abi.HAS_NEAR_PARTICLE) == (0, 1, 2)
    assert (abi.LINEAR_ELASTIC, abi.AUXETIC, abi.UNCONSTRAINED, abi.FIXED) == (0, 1, 0, 1)


def test_no_cpu_fallback_in_the_product():
    """The product package never imports the oracle."""
    pkg = Path(S.__file__).resolve().parent
    for f in pkg.rglob("*.py"):
        assert "oracle" not in re.findall(r"^\s*(?:from|import)\s+(\w+)", f.read_text(), flags=re.M), f


def test_host_free_refuses_memory_it_did_not_allocate():
    """sphnj_host_free checks its registry before any CUDA call, so this runs
    without a GPU."""
    import numpy as np

    lib = S.lib()
    x = np.zeros(16, np.float32)
    assert lib.sphnj_host_free(C.c_void_p(x.ctypes.data)) == abi.ERR_ARG
    assert lib.sphnj_host_free(None) == 0


def test_host_alloc_without_a_gpu_fails_cleanly():
    """With no device, pinned allocation reports an error instead of
    returning memory, and the numpy state falls back to ordinary arrays."""
    import numpy as np
    import torch

    if torch.cuda.is_available():
        import pytest

        pytest.skip("a GPU is present")
    lib = S.lib()
    ptr = C.c_void_p()
    assert lib.sphnj_host_alloc(1024, C.byref(ptr)) != 0
    assert not ptr.value
    p = abi.Params()
    p.fluid_number_total = 4
    st = abi.alloc_state(p, ("fluid_position",))
    assert isinstance(st["fluid_position"], np.ndarray) and st["fluid_position"].shape == (4, 2)
