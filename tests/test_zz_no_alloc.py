"""fsim_cell_sort_noalloc — the cell sort for callers that cannot allocate.

Some callers of this library must not allocate device memory once they run:
hosts that reserve all GPU memory up front under their own allocator or
budget, and real-time loops that cannot take the device synchronisation of
cudaMalloc/cudaFree.  For them the library offers a cell sort whose scratch is
one fixed device array inside the library.  This test calls it through the C
ABI on caller-owned device buffers and checks it against the cell phase of a
regular handle (fsim_run_phase + fsim_get_cells), which sorts the same way:
cell offsets and the cell-ordered ids must be identical (integer work, so the
tolerance is zero), on two calls in a row with different inputs, because the
shared scratch keeps the previous call's contents.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from fluidsim_gb300 import api, cases

pytestmark = pytest.mark.gpu


def _reference_sort(cfg, pa, species):
    sim = api.Simulation(cfg, pa, device=0)
    sim.phase(api.PHASE_CELL)
    start, ids = sim.cells(species)
    d = sim.derived()
    sim.close()
    return d, start, ids


def _noalloc_sort(lib, derived, pos):
    import torch

    dev = torch.device("cuda", 0)
    p = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).to(dev)
    start = torch.full((derived.cell_number_total + 1,), -7, dtype=torch.int32, device=dev)
    ids = torch.full((len(pos),), -7, dtype=torch.int32, device=dev)
    st = lib.fsim_cell_sort_noalloc(C.byref(derived), p.data_ptr(), len(pos), start.data_ptr(), ids.data_ptr(),
                                    None)
    assert st == api.OK, lib.fsim_last_error()
    torch.cuda.synchronize(dev)
    return start.cpu().numpy(), ids.cpu().numpy()


def test_noalloc_cell_sort_matches_cell_phase_twice():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    lib = api.load()
    cfg, pa = cases.make(cases.small_dam_break(jitter=0.01, seed=21))
    assert pa.n_fluid <= 262144
    # first call: the fluid particles; second call: the wall particles (more
    # of them, other cells), so stale scratch from call one would show
    d, ref_start, ref_ids = _reference_sort(cfg, pa, 0)
    start, ids = _noalloc_sort(lib, d, pa.fluid_pos)
    assert np.array_equal(start, ref_start)
    assert np.array_equal(ids, ref_ids)
    d2, ref_start2, ref_ids2 = _reference_sort(cfg, pa, 2)
    start2, ids2 = _noalloc_sort(lib, d2, pa.virt_pos)
    assert np.array_equal(start2, ref_start2)
    assert np.array_equal(ids2, ref_ids2)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = api.load()
    cfg, _ = cases.small_dam_break()
    d = api.derive(cfg)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = lib.fsim_cell_sort_noalloc(C.byref(d), dummy, 262145, dummy, dummy, None)
    assert st == api.EINVAL
    assert b"262144" in lib.fsim_last_error()
    big = api.derive(cases.fsi_4m()[0])  # 614,075 cells
    st = lib.fsim_cell_sort_noalloc(C.byref(big), dummy, 10, dummy, dummy, None)
    assert st == api.EINVAL
