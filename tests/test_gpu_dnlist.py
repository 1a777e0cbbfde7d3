"""Device neighbour lists vs the host builder.

For orthogonal and triclinic cells, cells narrower than twice the list
radius (atoms see their own images) and a batch of cells of uneven size, the
device builder's list of every atom is the same set of (neighbour, image
shift) entries as the host builder's ghost-atom list, mapped through each
ghost's owner and image code; positions are wrapped into the cell like the
host builder wraps them; two builds give identical arrays.
"""
import numpy as np
import pytest

import mlipg
from mlipg.structures import (bcc_cell, fcc_cell, jitter, random_triclinic_cell, random_types,
                              read_lammps_data)

pytestmark = pytest.mark.gpu


def host_sets(cell, r):
    s = mlipg.native_system(cell, r, 0.0)
    out = []
    for i in range(s.nlocal):
        js = s.nbr_idx[s.nbr_off[i]:s.nbr_off[i + 1]]
        out.append(sorted(zip(s.owner[js].tolist(), s.image[js].tolist())))
    return out, s


def device_build(cells, r):
    import torch
    x4 = np.concatenate([np.c_[c.positions, c.types.astype(np.float64)] for c in cells])
    d = torch.from_numpy(np.ascontiguousarray(x4)).cuda()
    nl = mlipg.DeviceNeighbourList()
    info = nl.build([c.natoms for c in cells], np.stack([c.lattice for c in cells]),
                    d.data_ptr(), r)
    torch.cuda.synchronize()
    off, idx, img = nl.copy()
    xw = d.cpu().numpy()
    nl.close()
    return off, idx, img, xw, info


def cases():
    rng = np.random.default_rng(12)
    out = [
        ("fcc-4000", [random_types(jitter(fcc_cell(10, 10, 10, 4.0), 0.1, rng), 3, rng)], 7.0),
        ("bcc-small", [jitter(bcc_cell(2, 2, 2, 3.2), 0.05, rng)], 6.0),
        ("triclinic", [random_triclinic_cell(n, 0.06, 2, rng) for n in (8, 9, 17, 64, 300)], 6.0),
    ]
    return out


@pytest.mark.parametrize("name,cells,r", cases(), ids=[c[0] for c in cases()])
def test_device_lists_equal_host_lists(name, cells, r):
    off, idx, img, xw, info = device_build(cells, r)
    base = 0
    for c in cells:
        hs, s = host_sets(c, r)
        for i in range(c.natoms):
            a, b = off[base + i], off[base + i + 1]
            dev = sorted(zip((idx[a:b] - base).tolist(), img[a:b].tolist()))
            assert dev == hs[i], (name, i)
        np.testing.assert_allclose(xw[base:base + c.natoms, :3], s.x[:c.natoms], rtol=0,
                                   atol=1e-10)
        base += c.natoms
    assert info["npairs"] == off[-1]
    assert info["max_neigh"] == np.diff(off).max()


def test_regression_cell_and_determinism():
    import os
    from conftest import GOLDEN
    c = read_lammps_data(os.path.join(GOLDEN, "structure_00064_triclinic.lammps"))
    o1 = device_build([c], 8.0)
    o2 = device_build([c], 8.0)
    for a, b in zip(o1[:3], o2[:3]):
        np.testing.assert_array_equal(a, b)
    hs, _ = host_sets(c, 8.0)
    off, idx, img = o1[:3]
    for i in range(c.natoms):
        assert sorted(zip(idx[off[i]:off[i + 1]].tolist(), img[off[i]:off[i + 1]].tolist())) == hs[i]
