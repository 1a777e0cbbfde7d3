"""Device-side status bits reach the caller on every GPU entry point.

The fused kernel never traps.  A centre with more neighbours inside the cutoff
than the launch's capacity is skipped (bit 1), a centre or neighbour whose
element index lies outside the potential is skipped (bit 2), and in the mixed
path an adjoint outside the fixed-point range is flagged (bit 4, also for
NaN or infinite values).  Each launch's status word is written to d_out8[7];
mlipg_device_status reads it back; the MD, batch, serving and host-array
entry points check it and fail with MLIPG_ECAPACITY (6), MLIPG_EINVAL (1) or
MLIPG_ENOTSUP (5).  Every case here is made on the host (a capacity below the
longest list, an element index past the last element, coefficients beyond
the FP32 range); nothing faults the GPU.
"""
import numpy as np
import pytest

import mlipg
from conftest import structure
from mlipg.potential import gaussian_params, write_potential
from mlipg.structures import build_system, random_triclinic_cell

pytestmark = pytest.mark.gpu


def _inputs(s, dev, x4_edit=None):
    import torch
    x4 = np.zeros((s.nall, 4))
    x4[:, :3] = s.x
    x4[:, 3] = s.type
    if x4_edit is not None:
        x4_edit(x4)
    return dict(x4=torch.from_numpy(x4).to(dev),
                c=torch.arange(s.nlocal, dtype=torch.int32, device=dev),
                o=torch.from_numpy(s.nbr_off.astype(np.int32)).to(dev),
                i=torch.from_numpy(s.nbr_idx.astype(np.int32)).to(dev))


def _run(g, fn, s, t, nb_cap):
    import torch
    f = torch.zeros((s.nall, 3), dtype=torch.float64, device="cuda")
    out = torch.full((8,), -1.0, dtype=torch.float64, device="cuda")
    fn(s.nlocal, t["x4"].data_ptr(), t["c"].data_ptr(), t["o"].data_ptr(), t["i"].data_ptr(),
       f.data_ptr(), out.data_ptr(), nb_cap=nb_cap)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _inside_cutoff(s, rc):
    n = 0
    for i in range(s.nlocal):
        j = s.nbr_idx[s.nbr_off[i]:s.nbr_off[i + 1]]
        d = np.linalg.norm(s.x[j] - s.x[i], axis=1)
        n = max(n, int(np.sum((d <= rc) & (d > 0))))
    return n


@pytest.mark.parametrize("prec", [mlipg.PREC_FP64, mlipg.PREC_MIXED])
@pytest.mark.parametrize("entry", ["compute_device", "compute_device_noalloc"])
def test_capacity_and_element_bits(potdir, prec, entry):
    import torch
    dev = torch.device("cuda")
    g = mlipg.Potential(potdir["gtinv-820"], prec)
    s = build_system(structure("structure.lammps"), g.cutoff, skin=2.0)
    fn = getattr(g, entry)
    nmax = _inside_cutoff(s, g.cutoff)
    assert nmax > 32
    t = _inputs(s, dev)
    out = _run(g, fn, s, t, nb_cap=int(np.diff(s.nbr_off).max()))
    assert out[7] == 0.0 and g.device_status() == 0
    e_clean = out[0]
    # capacity below the longest list inside the cutoff: bit 1, centres skipped
    out = _run(g, fn, s, t, nb_cap=32)
    assert out[7] == 1.0 and g.device_status() == 1
    assert out[0] != e_clean
    # an element index past the potential's elements on one centre: bit 2
    tb = _inputs(s, dev, lambda x4: x4.__setitem__((3, 3), 7.0))
    out = _run(g, fn, s, tb, nb_cap=int(np.diff(s.nbr_off).max()))
    assert out[7] == 2.0 and g.device_status() == 2
    # the next clean launch clears the word
    out = _run(g, fn, s, t, nb_cap=int(np.diff(s.nbr_off).max()))
    assert out[7] == 0.0 and g.device_status() == 0 and out[0] == e_clean


@pytest.fixture(scope="module")
def huge_pot(tmp_path_factory):
    """Coefficients of order 1e38: every FP32 adjoint flush overflows."""
    p = str(tmp_path_factory.mktemp("status") / "huge.mlip")
    write_potential(p, ["A", "B"], 5.0, gaussian_params(6, 5.0), 3, 2, 4, 3, [4, 4], [0, 0],
                    masses=[27.0, 58.7], seed=3, sigma=1e38)
    return p


def _cell(n, seed):
    rng = np.random.default_rng(seed)
    return random_triclinic_cell(n, 0.06, 2, rng)


def test_adjoint_range_bit_everywhere(huge_pot):
    import torch
    cell = _cell(24, 4)
    # host-array call
    g = mlipg.Potential(huge_pot, mlipg.PREC_MIXED)
    s = build_system(cell, g.cutoff, skin=1.0)
    with pytest.raises(mlipg.MlipgError) as ei:
        g.compute(s)
    assert ei.value.code == 5
    # device call: bit 4 in d_out8[7]
    t = _inputs(s, torch.device("cuda"))
    out = _run(g, g.compute_device, s, t, nb_cap=int(np.diff(s.nbr_off).max()))
    assert int(out[7]) & 4 and g.device_status() & 4
    # batch
    b = mlipg.Batch(g, [cell, _cell(16, 5)])
    with pytest.raises(mlipg.MlipgError) as ei:
        b.compute()
    assert ei.value.code == 5
    b.close()
    # MD: the first force evaluation already fails
    with pytest.raises(mlipg.MlipgError) as ei:
        mlipg.MD(g, cell)
    assert ei.value.code == 5
    g.close()
    # serving: the request fails, the server keeps running
    srv = mlipg.Server(huge_pot, budget_bytes=1 << 30, max_batch_atoms=4096)
    tk = srv.submit(cell, mlipg.PREC_MIXED)
    with pytest.raises(mlipg.MlipgError) as ei:
        srv.wait(tk, timeout_ms=60000)
    assert ei.value.code == 5
    # the FP64 path keeps FP64's range (coefficients beyond FP32's range run
    # the all-FP64 kernel): the same requests succeed
    tk = srv.submit(cell, mlipg.PREC_FP64)
    e, f, v = srv.wait(tk, timeout_ms=60000)
    assert np.isfinite(e)
    srv.close()
    g64 = mlipg.Potential(huge_pot, mlipg.PREC_FP64)
    r = g64.compute(s)
    assert np.isfinite(r["energy"]) and g64.device_status() == 0
    md = mlipg.MD(g64, cell)
    md.close()
    g64.close()


def test_md_and_batch_clean_runs_report_no_bits(tmp_path):
    from mlipg.potential import workload_potential
    p = str(tmp_path / "tric.mlip")
    workload_potential(p, "triclinic-batch", seed=2)
    g = mlipg.Potential(p, mlipg.PREC_MIXED)
    cell = _cell(32, 6)
    md = mlipg.MD(g, cell)
    md.run(5)
    assert g.device_status() == 0
    md.close()
    b = mlipg.Batch(g, [cell])
    b.compute()
    assert g.device_status() == 0
    b.close()
    g.close()
