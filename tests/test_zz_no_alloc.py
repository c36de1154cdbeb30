"""sphnj_rebuild_cell_lists_noalloc: the incremental cell-list rebuild for
callers that cannot allocate device memory.

Those callers - code running while a host framework's pool allocator owns the
device memory, plugin hosts that forbid cudaMalloc after start-up, real-time
loops that must stay out of the driver's allocator - pass every input and
output buffer; the entry point keeps its scratch in a static device array.
This test allocates the buffers itself (with torch: the test may allocate,
the entry point must not) and checks, on two consecutive steps, that the
lists it builds are bit-identical to the lists that the context's own path
builds inside sphnj_step (read back with sphnj_debug_cells).  Integer lists
are compared exactly, as every cell-list test here does.
"""
import ctypes as C

import numpy as np
import pytest

import sphnj_gb300 as S
from sphnj_gb300 import abi, cases

from helpers import load

pytestmark = pytest.mark.gpu


def _entry():
    fn = S.lib().sphnj_rebuild_cell_lists_noalloc
    fn.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 6
    fn.restype = C.c_int
    return fn


def test_noalloc_rebuild_matches_context_path_on_two_steps():
    import torch

    fn = _entry()
    p, arr = load(cases.dam_break_water(dx=0.02))
    nx, ny, ncell, n = p.cell_number[0], p.cell_number[1], p.cell_number_total, p.fluid_number_total
    assert ncell <= 65536
    dev = torch.device("cuda")
    with S.Simulation(p) as g:
        g.upload(arr)
        g.step(1)  # step 1 sorts: the lists are the sorted ranges
        for call in range(2):  # steps 2 and 3 are incremental rebuilds
            prev_start, prev_count, prev_list = g.cells(0)
            g.step(1)
            g.synchronize()
            cell_id = g.download(abi.F_CELL_IDS)["fluid_cell_id"]  # the ids this step binned
            want_start, want_count, want_list = g.cells(0)

            prev_range = np.stack([prev_start, prev_count], axis=1).astype(np.int32).ravel()
            d_cell = torch.from_numpy(cell_id.astype(np.int32)).to(dev)
            d_prev_range = torch.from_numpy(prev_range).to(dev)
            d_prev_list = torch.from_numpy(np.concatenate([prev_list, [0]]).astype(np.int32)).to(dev)
            d_range = torch.full((2 * ncell,), -1, dtype=torch.int32, device=dev)
            d_list = torch.full((n,), -1, dtype=torch.int32, device=dev)
            stream = torch.cuda.current_stream(dev)
            rc = fn(nx, ny, n, d_cell.data_ptr(), d_prev_range.data_ptr(), d_prev_list.data_ptr(),
                    d_range.data_ptr(), d_list.data_ptr(), stream.cuda_stream)
            assert rc == abi.OK, rc
            torch.cuda.synchronize(dev)
            got_range = d_range.cpu().numpy().reshape(-1, 2)
            got_list = d_list.cpu().numpy()
            assert np.array_equal(got_range[:, 1], want_count), f"call {call}: counts differ"
            assert np.array_equal(got_range[:, 0], want_start), f"call {call}: starts differ"
            total = int(want_count.sum())
            assert np.array_equal(got_list[:total], want_list), f"call {call}: lists differ"


def test_noalloc_rejects_grids_beyond_its_static_scratch():
    fn = _entry()
    # 300 x 300 cells > 65536: refused before any pointer is used or work launched
    rc = fn(300, 300, 0, None, None, None, None, None, None)
    assert rc == abi.ERR_UNSUPPORTED
