"""The entry point that allocates no device memory (nnpgpu_symm_noalloc).

It exists for callers that must not let a library allocate device memory while they run, such
as codes that divide the GPU's memory among their own pools before the first step.  Its output
must equal the regular entry point's (nnpgpu_compute with NNPGPU_SYMM) within the descriptor
tolerance of the other GPU tests, call after call, although every call reuses the same scratch
array inside the library.  This file sorts last so that a failure here does not hide the others.
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
    # two calls in a row: the second, smaller structure must not see the first one's leftovers
    strucs = W.make_structures("mixed512", seed=44, count=2, sizes=[900, 150])
    for s in strucs:
        _, _, Gref = eng.compute([s], engine.SYMM | engine.BATCHED)
        d_posn = torch.from_numpy(np.ascontiguousarray(s.posn, dtype=np.float64)).cuda()
        d_spec = torch.from_numpy(np.ascontiguousarray(s.species, dtype=np.int32)).cuda()
        out = torch.full((s.natoms, stride), float("nan"), dtype=torch.float32, device="cuda")
        eng.symm_noalloc(s.natoms, d_posn.data_ptr(), d_spec.data_ptr(), s.cell, out.data_ptr(), stride, stream)
        torch.cuda.synchronize()
        G = out.cpu().numpy()
        assert np.isfinite(G).all()
        assert np.abs(G - Gref).max() <= G_TOL * max(np.abs(Gref).max(), 1.0)
    # requests beyond the stated limit are refused before any device work
    with pytest.raises(engine.NNPGPUError) as ei:
        eng.symm_noalloc(1025, d_posn.data_ptr(), d_spec.data_ptr(), strucs[0].cell, out.data_ptr(), stride, stream)
    assert ei.value.code == engine.ERR_INVALID and "limit" in str(ei.value)
    eng.close()
