"""The allocation-free entry point against the regular device entry point.

mlipg_compute_device_noalloc exists for callers that cannot let a library
call cudaMalloc: device memory owned by the caller's own pool or budget, or
latency-critical loops that must not enter the CUDA allocator.  It keeps the
kernel's scratch in a fixed device array inside the library instead of
buffers the handle allocates.  This file runs last (pytest collects it after
the other test files) so a failure here does not hide the rest of the suite.
"""
import numpy as np
import pytest

import mlipg
from conftest import structure
from mlipg.structures import build_system

pytestmark = pytest.mark.gpu


def _device_inputs(s, dev):
    import torch
    x4 = np.zeros((s.nall, 4))
    x4[:, :3] = s.x
    x4[:, 3] = s.type
    return dict(
        x4=torch.from_numpy(x4).to(dev),
        c=torch.arange(s.nlocal, dtype=torch.int32, device=dev),
        o=torch.from_numpy(s.nbr_off).to(dev),
        i=torch.from_numpy(s.nbr_idx).to(dev))


@pytest.mark.parametrize("prec,tol", [(mlipg.PREC_FP64, 1e-12), (mlipg.PREC_MIXED, 5e-4)])
def test_noalloc_matches_regular_entry_point(potdir, prec, tol):
    """Both entry points run the same kernel; they differ only through the order
    of the atomic additions.  In FP64 that is rounding (1e-12 of each array's
    scale).  In the mixed path a centre's adjoint is summed with FP32 atomics
    in a varying order, and a centre's per-atom virial follows its adjoint:
    two ordinary calls differ by up to ~1e-4 of the per-atom virial scale on
    this potential, so the mixed results must agree within 5e-4 of each
    array's scale (or four times the spread of two ordinary calls, if larger).
    A scratch error (stale partial sums, a wrong slot count) shows up as an
    O(1) difference in the totals, in either precision."""
    import torch
    dev = torch.device("cuda")
    g = mlipg.Potential(potdir["gtinv-820"], prec)
    s = build_system(structure("structure.lammps"), g.cutoff, skin=2.0)
    t = _device_inputs(s, dev)
    nb = int(np.diff(s.nbr_off).max())

    def run(fn):
        f = torch.zeros((s.nall, 3), dtype=torch.float64, device=dev)
        out = torch.full((8,), -1.0, dtype=torch.float64, device=dev)
        ea = torch.zeros(s.nlocal, dtype=torch.float64, device=dev)
        va = torch.zeros((s.nlocal, 6), dtype=torch.float64, device=dev)
        fn(s.nlocal, t["x4"].data_ptr(), t["c"].data_ptr(), t["o"].data_ptr(),
           t["i"].data_ptr(), f.data_ptr(), out.data_ptr(), eatom=ea.data_ptr(), nb_cap=nb,
           vatom=va.data_ptr())
        torch.cuda.synchronize()
        return f.cpu().numpy(), out.cpu().numpy(), ea.cpu().numpy(), va.cpu().numpy()

    ref = run(g.compute_device)
    ref2 = run(g.compute_device)
    spread = [np.abs(a - b).max() for a, b in zip(ref, ref2)]
    for _ in range(2):                      # two calls in a row share the scratch
        got = run(g.compute_device_noalloc)
        for a, b, sp in zip(got, ref, spread):
            scale = max(np.abs(b).max(), 1e-300)
            assert np.abs(a - b).max() <= max(4.0 * sp, tol * scale)
        assert got[1][0] == pytest.approx(got[2].sum(), rel=1e-12)
