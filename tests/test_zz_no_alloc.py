"""The entry point that allocates no device memory (nnpgpu_symm_noalloc).

It exists for callers that must not let a library allocate device memory while they run, such
as codes that divide the GPU's memory among their own pools before the first step.  Its output
must equal the regular entry point's (nnpgpu_compute with NNPGPU_SYMM) within the descriptor
tolerance of the other GPU tests, call after call, although every call reuses the same scratch
array inside the library.  After the set-up call the device's free memory must not change.
This file sorts last so that a failure here does not hide the others.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from atomnn_gb300 import workloads as W

pytestmark = pytest.mark.gpu

G_TOL = 1e-5  # relative to the largest |G| of the structure, as in test_gpu_parity.py


def test_symm_noalloc_matches_regular_entry_point(native_lib):
    import torch
    from atomnn_gb300 import engine
    eng = engine.Engine(os.path.join(GOLDEN, "mixed512.nnp"))
    stride = max(eng.ninput)
    stream = torch.cuda.current_stream().cuda_stream
    dev_before = torch.cuda.current_device()
    # set-up call: looks up the scratch array and loads the kernels before memory is measured
    eng.symm_noalloc(0, 0, 0, None, 0, stride, stream)
    # a single-image cell (900 atoms), then a small cell that needs lattice image shells (40
    # atoms), then the first again: no call may see the previous one's leftovers
    strucs = W.make_structures("mixed512", seed=44, count=2, sizes=[900, 40])
    order = [0, 1, 0]
    bufs = []
    for s in strucs:
        d_posn = torch.from_numpy(np.ascontiguousarray(s.posn, dtype=np.float64)).cuda()
        d_spec = torch.from_numpy(np.ascontiguousarray(s.species, dtype=np.int32)).cuda()
        bufs.append((d_posn, d_spec))
    outs = [torch.full((strucs[k].natoms, stride), float("nan"), dtype=torch.float32, device="cuda") for k in order]
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for k, out in zip(order, outs):
        s = strucs[k]
        eng.symm_noalloc(s.natoms, bufs[k][0].data_ptr(), bufs[k][1].data_ptr(), s.cell, out.data_ptr(), stride, stream)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after == free_before, "device memory changed by %d bytes" % (free_before - free_after)
    assert torch.cuda.current_device() == dev_before
    for k, out in zip(order, outs):
        s = strucs[k]
        _, _, Gref = eng.compute([s], engine.SYMM | engine.BATCHED)
        G = out.cpu().numpy()
        assert np.isfinite(G).all()
        assert np.abs(G - Gref).max() <= G_TOL * max(np.abs(Gref).max(), 1.0)
    # requests beyond the stated limit are refused before any device work
    with pytest.raises(engine.NNPGPUError) as ei:
        eng.symm_noalloc(1025, bufs[0][0].data_ptr(), bufs[0][1].data_ptr(), strucs[0].cell, outs[0].data_ptr(), stride, stream)
    assert ei.value.code == engine.ERR_INVALID and "limit" in str(ei.value)
    # a near-flat cell is refused by the image limit, not by an overflowing shell count
    flat = np.diag([10.0, 10.0, 1e-12])
    with pytest.raises(engine.NNPGPUError) as ei:
        eng.symm_noalloc(strucs[1].natoms, bufs[1][0].data_ptr(), bufs[1][1].data_ptr(), flat, outs[1].data_ptr(), stride, stream)
    assert ei.value.code == engine.ERR_INVALID and "lattice images" in str(ei.value)
    eng.close()
