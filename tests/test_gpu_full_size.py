"""Parity at the benchmark sizes: the full 16,000-atom binary bcc and
1,048,576-atom ternary fcc structures of the benchmark workloads.

The oracle cannot evaluate a million atoms within a test, so both sides
evaluate the same seeded random sample of 2,000 centre atoms of the full
structure (owned atoms plus ghost images, full neighbour lists) in the
owner-computes form: each sampled centre's energy, and the forces its own
adjoint puts on it and on its neighbours (summed over all centres this is
the reference's full-list result).  FP64: per-centre energies and every
force row agree with the oracle to 1e-10 relative.  Mixed: force RMS error
<= 1e-4 eV/A and the sample's energy within 1e-6 eV/atom (these potentials
have synthetic N(0, 1e-3) weights).
"""
import numpy as np
import pytest

import mlipg
from mlipg.potential import workload_potential
from mlipg.structures import bcc_cell, fcc_cell, jitter, random_types
from oracle import Oracle

pytestmark = pytest.mark.gpu

CASES = {
    # workload name: (structure, potential)
    "bcc-binary-16k": (lambda rng: random_types(jitter(bcc_cell(20, 20, 20, 3.2), 0.05, rng), 2,
                                                rng), "bcc-binary-16k"),
    "fcc-ternary-1m": (lambda rng: random_types(jitter(fcc_cell(64, 64, 64, 4.0), 0.1, rng), 3,
                                                rng), "fcc-ternary-1m"),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request, tmp_path_factory):
    make, potname = CASES[request.param]
    rng = np.random.default_rng(1)
    cell = make(rng)
    pot = str(tmp_path_factory.mktemp("full") / (potname + ".mlip"))
    workload_potential(pot, potname, seed=1)
    orc = Oracle(pot, threads=16)
    s = mlipg.native_system(cell, orc.cutoff, 0.0)
    sample = np.sort(np.random.default_rng(2).choice(s.nlocal, 2000, replace=False))
    ref = orc.compute_centers(s, sample)
    return request.param, pot, s, sample, ref


def _gpu(pot, prec, s, sample):
    import torch
    dev = torch.device("cuda")
    x4 = np.zeros((s.nall, 4))
    x4[:, :3] = s.x
    x4[:, 3] = s.type
    rows = [s.nbr_idx[s.nbr_off[i]:s.nbr_off[i + 1]] for i in sample]
    off = np.zeros(len(sample) + 1, dtype=np.int32)
    off[1:] = np.cumsum([len(r) for r in rows])
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in dict(
        x4=x4, c=sample.astype(np.int32), o=off, i=np.concatenate(rows).astype(np.int32)).items()}
    f = torch.zeros((s.nall, 3), dtype=torch.float64, device=dev)
    out = torch.zeros(8, dtype=torch.float64, device=dev)
    ea = torch.zeros(len(sample), dtype=torch.float64, device=dev)
    g = mlipg.Potential(pot, prec)
    g.compute_device(len(sample), t["x4"].data_ptr(), t["c"].data_ptr(), t["o"].data_ptr(),
                     t["i"].data_ptr(), f.data_ptr(), out.data_ptr(), eatom=ea.data_ptr(),
                     nb_cap=int(max(len(r) for r in rows)))
    torch.cuda.synchronize()
    res = dict(f=f.cpu().numpy(), out=out.cpu().numpy(), eatom=ea.cpu().numpy())
    g.close()
    return res


def test_full_size_fp64(case):
    name, pot, s, sample, ref = case
    got = _gpu(pot, mlipg.PREC_FP64, s, sample)
    assert got["out"][7] == 0.0
    e = ref["eatom"]
    assert np.abs(got["eatom"] - e).max() <= 1e-10 * np.abs(e).max()
    assert abs(got["out"][0] - ref["energy"]) <= 1e-10 * abs(ref["energy"])
    fr = ref["f_all"]
    assert np.abs(got["f"] - fr).max() <= 1e-10 * np.abs(fr).max()


def test_full_size_mixed(case):
    name, pot, s, sample, ref = case
    got = _gpu(pot, mlipg.PREC_MIXED, s, sample)
    assert got["out"][7] == 0.0
    touched = np.abs(ref["f_all"]).sum(1) > 0
    d = got["f"][touched] - ref["f_all"][touched]
    assert np.sqrt(np.mean(d ** 2)) <= 1e-4
    assert abs(got["out"][0] - ref["energy"]) / len(sample) <= 1e-6
