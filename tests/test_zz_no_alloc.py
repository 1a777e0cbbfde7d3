"""The allocation-free entry point against the regular device entry point.

mlipg_compute_device_noalloc exists for callers that cannot let a library
call cudaMalloc: an MD engine or service whose device memory belongs to its
own pool or budget, or a latency-critical loop that must not enter the CUDA
allocator (which can synchronise the device).  It keeps the kernel's scratch
(per-CTA partial sums and the status word) in a fixed device array inside
the library instead of buffers the handle allocates.  This file runs last
(pytest collects it after the other test files) so that a failure here does
not hide the rest of the suite.

Both entry points run the same kernel with the same launch shape.  Total and
per-atom energies are bitwise reproducible (fixed summation orders).  Forces
and virials differ through the order of the FP64 force scatter's atomic
additions and through the scale of the adjoint's exact fixed-point sums: a
launch starts from the exponents the handle's previous launch adapted, so
two calls round the adjoint at different (equally valid) granularities.
Bounds: 1e-12 of each array's scale for MLIPG_PREC_FP64 (double-float
products, a fixed point 64 bits below the largest flush) and 1e-7 for
MLIPG_PREC_MIXED (FP32 products, 37 bits below it).  A scratch error (stale
partial sums, a wrong slot count, a missed status clear) shows up as an
O(1) difference in the totals or in d_out8[7].
"""
import numpy as np
import pytest

import mlipg
from conftest import structure
from mlipg.potential import workload_potential
from mlipg.structures import build_system, random_triclinic_cell

pytestmark = pytest.mark.gpu

TOL = {mlipg.PREC_FP64: 1e-12, mlipg.PREC_MIXED: 1e-7}


def _ghost_inputs(s, dev):
    """LAMMPS-style owned + ghost atoms, a full list, and the ghost -> owner
    force rows (d_fold)."""
    import torch
    x4 = np.zeros((s.nall, 4))
    x4[:, :3] = s.x
    x4[:, 3] = s.type
    return dict(
        n=s.nlocal, nforce=s.nlocal,
        x4=torch.from_numpy(x4).to(dev),
        c=torch.arange(s.nlocal, dtype=torch.int32, device=dev),
        o=torch.from_numpy(s.nbr_off.astype(np.int32)).to(dev),
        i=torch.from_numpy(s.nbr_idx.astype(np.int32)).to(dev),
        fold=torch.from_numpy(s.owner.astype(np.int32)).to(dev),
        nb=int(np.diff(s.nbr_off).max()), img=None)


def _image_inputs(cells, dev, rlist):
    """Several periodic cells with image-coded lists built on the device
    (no ghost atoms), and a fold map that permutes the force rows."""
    import torch
    n = np.array([c.natoms for c in cells], dtype=np.int32)
    x4 = np.concatenate([np.column_stack([c.positions, c.types]) for c in cells])
    d_x4 = torch.from_numpy(np.ascontiguousarray(x4)).to(dev)
    lat = np.stack([c.lattice for c in cells])
    nl = mlipg.DeviceNeighbourList()
    info = nl.build(n, lat, d_x4.data_ptr(), rlist)
    torch.cuda.synchronize()
    N = int(n.sum())
    perm = np.random.default_rng(3).permutation(N).astype(np.int32)
    return dict(
        n=N, nforce=N, x4=d_x4, c=torch.arange(N, dtype=torch.int32, device=dev),
        o=info["off"], i=info["idx"], img=info["img"], cell=info["cells"],
        ccell=info["center_cell"], fold=torch.from_numpy(perm).to(dev),
        nb=info["max_neigh"], keep=nl)


def _ptr(v):
    return v if isinstance(v, int) else v.data_ptr()


def _run(fn, t):
    import torch
    dev = torch.device("cuda")
    f = torch.zeros((t["nforce"], 3), dtype=torch.float64, device=dev)
    out = torch.full((8,), -1.0, dtype=torch.float64, device=dev)
    ea = torch.zeros(t["n"], dtype=torch.float64, device=dev)
    va = torch.zeros((t["n"], 6), dtype=torch.float64, device=dev)
    kw = {}
    if t["img"] is not None:
        kw = dict(img=t["img"], cell=t["cell"], center_cell=t["ccell"])
    fn(t["n"], _ptr(t["x4"]), _ptr(t["c"]), _ptr(t["o"]), _ptr(t["i"]), f.data_ptr(),
       out.data_ptr(), eatom=ea.data_ptr(), vatom=va.data_ptr(), fold=_ptr(t["fold"]),
       nb_cap=t["nb"], **kw)
    torch.cuda.synchronize()
    return f.cpu().numpy(), out.cpu().numpy(), ea.cpu().numpy(), va.cpu().numpy()


def _compare(got, ref, prec):
    f, out, ea, va = got
    fr, outr, ear, var = ref
    assert out[7] == 0.0 and outr[7] == 0.0            # status words cleared
    assert out[0] == outr[0]                           # total energy
    np.testing.assert_array_equal(ea, ear)
    for a, b in ((out[1:7], outr[1:7]), (va, var), (f, fr)):
        assert np.abs(a - b).max() <= TOL[prec] * max(np.abs(b).max(), 1e-300)
    assert out[0] == pytest.approx(ea.sum(), rel=1e-12)


@pytest.mark.parametrize("prec", [mlipg.PREC_FP64, mlipg.PREC_MIXED])
def test_noalloc_matches_regular_entry_point(potdir, prec):
    import torch
    g = mlipg.Potential(potdir["gtinv-820"], prec)
    s = build_system(structure("structure.lammps"), g.cutoff, skin=2.0)
    t = _ghost_inputs(s, torch.device("cuda"))
    ref = _run(g.compute_device, t)
    for _ in range(2):                      # two calls in a row share the scratch
        _compare(_run(g.compute_device_noalloc, t), ref, prec)


@pytest.mark.parametrize("prec", [mlipg.PREC_FP64, mlipg.PREC_MIXED])
def test_noalloc_image_coded_lists_and_fold(tmp_path, prec):
    """Device-built image-coded lists of small triclinic cells (cells narrower
    than twice the cutoff see their own images), with a fold map."""
    import torch
    p = str(tmp_path / "tric.mlip")
    workload_potential(p, "triclinic-batch", seed=4)
    rng = np.random.default_rng(8)
    cells = [random_triclinic_cell(k, 0.06, 2, rng) for k in (12, 30, 47)]
    g = mlipg.Potential(p, prec)
    t = _image_inputs(cells, torch.device("cuda"), g.cutoff + 0.5)
    ref = _run(g.compute_device, t)
    for _ in range(2):
        _compare(_run(g.compute_device_noalloc, t), ref, prec)
