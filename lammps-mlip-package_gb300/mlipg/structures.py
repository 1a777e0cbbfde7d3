"""Periodic structures and LAMMPS-style neighbour data for the MLIP path.

LAMMPS hands a pair style its owned atoms followed by ghost atoms (periodic
images within the ghost cutoff), plus a full neighbour list of the owned atoms
whose entries index both owned and ghost atoms.  The reference pair style
consumes exactly that (``pair_mlip_gtinv_kokkos_impl.h:411-599``).  This module
builds the same data from a periodic cell so the library can be driven without
LAMMPS: `System.from_cell` creates owned + ghost coordinates, the ghost ->
owner map (LAMMPS reverse-communicates ghost forces onto owners) and the full
list in CSR form.

Structure generators cover the workloads named for this path: fcc / bcc
supercells with Gaussian jitter and random species, LAMMPS data files
(orthogonal and triclinic), and random triclinic cells with a minimum-distance
rejection.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

NKTV2P_METAL = 1.6021765e6  # bar per eV/A^3 (LAMMPS metal units)


@dataclasses.dataclass
class Cell:
    lattice: np.ndarray        # (3, 3) rows are the cell vectors a1, a2, a3
    positions: np.ndarray      # (N, 3) Cartesian
    types: np.ndarray          # (N,) element index (0-based)

    @property
    def volume(self) -> float:
        return float(abs(np.linalg.det(self.lattice)))

    @property
    def natoms(self) -> int:
        return int(self.positions.shape[0])


@dataclasses.dataclass
class System:
    """Owned atoms first, then ghosts; full neighbour list of the owned atoms."""
    cell: Cell
    x: np.ndarray              # (nall, 3) float64
    type: np.ndarray           # (nall,) int32 element index
    owner: np.ndarray          # (nall,) int64 owned index of every atom
    nbr_off: np.ndarray        # (nlocal + 1,) int32
    nbr_idx: np.ndarray        # (P,) int32 into [0, nall)
    nlocal: int
    cutoff: float

    @property
    def nall(self) -> int:
        return int(self.x.shape[0])

    @property
    def npairs(self) -> int:
        return int(self.nbr_idx.shape[0])

    def fold_forces(self, f_all: np.ndarray) -> np.ndarray:
        """Reverse-communicate ghost forces onto their owners (LAMMPS newton on)."""
        out = np.zeros((self.nlocal, 3))
        np.add.at(out, self.owner, f_all.reshape(-1, 3))
        return out

    def pressure_tensor(self, virial6: np.ndarray) -> np.ndarray:
        """Pxx, Pyy, Pzz, Pxy, Pxz, Pyz in bar from a LAMMPS-order virial (T = 0)."""
        return np.asarray(virial6) / self.cell.volume * NKTV2P_METAL

    def pressure(self, virial6: np.ndarray) -> float:
        v = np.asarray(virial6)
        return float((v[0] + v[1] + v[2]) / (3.0 * self.cell.volume) * NKTV2P_METAL)

    @staticmethod
    def from_cell(cell: Cell, cutoff: float, skin: float = 0.0) -> "System":
        return build_system(cell, cutoff, skin)


def _perp_widths(lat: np.ndarray) -> np.ndarray:
    vol = abs(np.linalg.det(lat))
    w = np.empty(3)
    for k in range(3):
        c = np.cross(lat[(k + 1) % 3], lat[(k + 2) % 3])
        w[k] = vol / np.linalg.norm(c)
    return w


def build_system(cell: Cell, cutoff: float, skin: float = 0.0) -> System:
    """Owned atoms + ghost images + full neighbour list (distance < cutoff + skin).

    Ghosts are images whose fractional coordinates fall within the ghost
    cutoff of the cell in every direction, as LAMMPS selects them for a
    triclinic box.  Self images are ordinary ghosts.
    """
    from scipy.spatial import cKDTree

    lat = np.asarray(cell.lattice, dtype=np.float64)
    inv = np.linalg.inv(lat)
    pos = np.asarray(cell.positions, dtype=np.float64)
    frac = pos @ inv
    frac -= np.floor(frac)
    frac[frac >= 1.0] = 0.0
    pos = frac @ lat
    n = pos.shape[0]
    rg = cutoff + skin
    w = _perp_widths(lat)
    delta = rg / w
    nmax = np.ceil(delta).astype(int)
    xs = [pos]
    ts = [np.asarray(cell.types, dtype=np.int32)]
    owners = [np.arange(n, dtype=np.int64)]
    for i in range(-nmax[0], nmax[0] + 1):
        for j in range(-nmax[1], nmax[1] + 1):
            for k in range(-nmax[2], nmax[2] + 1):
                if i == 0 and j == 0 and k == 0:
                    continue
                fs = frac + np.array([i, j, k], dtype=np.float64)
                keep = np.all((fs >= -delta) & (fs < 1.0 + delta), axis=1)
                if not keep.any():
                    continue
                idx = np.nonzero(keep)[0]
                xs.append(fs[idx] @ lat)
                ts.append(ts[0][idx])
                owners.append(idx.astype(np.int64))
    x = np.concatenate(xs)
    typ = np.concatenate(ts)
    owner = np.concatenate(owners)
    tree = cKDTree(x)
    pairs = tree.query_pairs(rg, output_type="ndarray")
    if pairs.size == 0:
        pairs = np.zeros((0, 2), dtype=np.int64)
    a, b = pairs[:, 0], pairs[:, 1]
    # directed entries whose centre is owned
    ca = a < n
    cb = b < n
    centers = np.concatenate([a[ca], b[cb]])
    nbrs = np.concatenate([b[ca], a[cb]])
    order = np.lexsort((nbrs, centers))
    centers = centers[order]
    nbrs = nbrs[order]
    counts = np.bincount(centers, minlength=n)
    off = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(counts, out=off[1:])
    return System(cell=Cell(lat, pos, ts[0]), x=x, type=typ, owner=owner,
                  nbr_off=off, nbr_idx=nbrs.astype(np.int32), nlocal=n,
                  cutoff=cutoff)


# ------------------------------------------------------------------ generators

def fcc_cell(nx: int, ny: int, nz: int, a: float) -> Cell:
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    return _supercell(base, nx, ny, nz, a)


def bcc_cell(nx: int, ny: int, nz: int, a: float) -> Cell:
    base = np.array([[0, 0, 0], [0.5, 0.5, 0.5]])
    return _supercell(base, nx, ny, nz, a)


def _supercell(base, nx, ny, nz, a) -> Cell:
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                             indexing="ij"), axis=-1).reshape(-1, 3)
    frac = (g[:, None, :] + base[None, :, :]).reshape(-1, 3)
    pos = frac * a
    lat = np.diag([nx * a, ny * a, nz * a]).astype(np.float64)
    return Cell(lat, pos.astype(np.float64), np.zeros(len(pos), dtype=np.int32))


def jitter(cell: Cell, sigma: float, rng: np.random.Generator) -> Cell:
    return Cell(cell.lattice, cell.positions + rng.normal(0.0, sigma, cell.positions.shape),
                cell.types.copy())


def random_types(cell: Cell, ntypes: int, rng: np.random.Generator) -> Cell:
    """Types assigned in equal shares (to within one atom), randomly permuted."""
    n = cell.natoms
    t = np.arange(n) % ntypes
    rng.shuffle(t)
    return Cell(cell.lattice, cell.positions, t.astype(np.int32))


def random_triclinic_cell(natoms: int, density: float, ntypes: int,
                          rng: np.random.Generator, min_dist: float = 1.8,
                          max_rounds: int = 2000) -> Cell:
    """Random cell matrix with angles U(60, 120) deg at the given number density.

    Atoms are uniform in the cell, then every atom closer than `min_dist`
    (minimum image) to an earlier atom is redrawn until no pair violates the
    distance.  Cells whose matrix is nearly degenerate are redrawn.
    """
    vol = natoms / density
    while True:
        al, be, ga = np.radians(rng.uniform(60.0, 120.0, 3))
        cx = math.cos(be)
        cy = (math.cos(al) - math.cos(be) * math.cos(ga)) / math.sin(ga)
        cz2 = 1.0 - cx * cx - cy * cy
        if cz2 < 0.05:
            continue
        m = np.array([[1.0, 0.0, 0.0],
                      [math.cos(ga), math.sin(ga), 0.0],
                      [cx, cy, math.sqrt(cz2)]])
        s = (vol / abs(np.linalg.det(m))) ** (1.0 / 3.0)
        lat = m * s
        if np.min(_perp_widths(lat)) < 0.35 * s:
            continue
        break
    frac = rng.random((natoms, 3))
    md2 = min_dist * min_dist
    if natoms > 512:
        return Cell(lat, _place_kdtree(frac, lat, min_dist, rng, max_rounds) @ lat,
                    np.asarray(rng.integers(0, ntypes, natoms), dtype=np.int32))

    def min_r2(ids):
        d = frac[ids][:, None, :] - frac[None, :, :]
        d -= np.round(d)
        dc = d @ lat
        r2 = np.einsum("ijk,ijk->ij", dc, dc)
        r2[np.arange(len(ids)), ids] = np.inf
        return r2

    r2 = min_r2(np.arange(natoms))
    bad = np.nonzero(np.triu(r2 < md2, k=1).any(axis=0))[0]   # clashes with an earlier atom
    for _ in range(max_rounds):
        if bad.size == 0:
            break
        frac[bad] = rng.random((bad.size, 3))
        bad = bad[(min_r2(bad) < md2).any(axis=1)]
    else:
        raise RuntimeError("could not place atoms with the minimum distance")
    types = np.asarray(rng.integers(0, ntypes, natoms), dtype=np.int32)
    return Cell(lat, frac @ lat, types)


def _place_kdtree(frac, lat, min_dist, rng, max_rounds):
    """Minimum-distance rejection for large cells with k-d trees over atoms
    and their 26 neighbouring images (every cell width exceeds `min_dist`).
    Atoms closer than `min_dist` to an earlier atom are redrawn; each redraw
    round tries 16 candidate positions per atom against the placed atoms and
    keeps the first free one that also clears the atoms placed before it in
    the same round."""
    import itertools

    from scipy.spatial import cKDTree

    n = frac.shape[0]
    img = np.array(list(itertools.product((-1, 0, 1), repeat=3)), dtype=np.float64) @ lat

    def tree_of(f):
        pos = f @ lat
        return cKDTree((pos[None, :, :] + img[:, None, :]).reshape(-1, 3))

    def earlier_clash(f):
        """Indices (into f) of points within min_dist of an earlier point."""
        m = f.shape[0]
        pos = f @ lat
        tree = tree_of(f)
        cnt = tree.query_ball_point(pos, min_dist, return_length=True)
        near = np.nonzero(cnt > 1)[0]
        hits = tree.query_ball_point(pos[near], min_dist) if near.size else []
        return np.asarray([i for i, h in zip(near, hits) if (np.asarray(h) % m).min() < i],
                          dtype=np.int64)

    bad = earlier_clash(frac)
    keep = np.ones(n, dtype=bool)
    keep[bad] = False
    tree = tree_of(frac[keep])
    extra = np.zeros((0, 3))
    for _ in range(max_rounds):
        if bad.size == 0:
            return frac
        cand = rng.random((bad.size, 16, 3))
        flat = (cand @ lat).reshape(-1, 3)
        free = tree.query(flat, k=1, distance_upper_bound=min_dist)[0] > min_dist
        if extra.shape[0]:
            free &= tree_of(extra).query(flat, k=1, distance_upper_bound=min_dist)[0] > min_dist
        free = free.reshape(bad.size, 16)
        has = free.any(axis=1)
        placed = bad[has]
        newf = cand[has, np.argmax(free[has], axis=1)]
        clash = np.zeros(placed.size, dtype=bool)
        clash[earlier_clash(newf)] = True
        frac[placed[~clash]] = newf[~clash]
        keep[placed[~clash]] = True
        bad = np.concatenate([bad[~has], placed[clash]])
        extra = np.concatenate([extra, newf[~clash]])
        if extra.shape[0] > 1024:
            tree = tree_of(frac[keep])
            extra = np.zeros((0, 3))
    raise RuntimeError("could not place atoms with the minimum distance")


def read_lammps_data(path: str) -> Cell:
    """Atomic-style LAMMPS data file (orthogonal or triclinic); types -> 0-based."""
    lines = open(path).read().splitlines()
    natoms = 0
    lo = np.zeros(3)
    hi = np.zeros(3)
    tilt = np.zeros(3)
    i = 0
    atoms = []
    while i < len(lines):
        s = lines[i].split("#")[0].split()
        if len(s) >= 2 and s[-1] == "atoms":
            natoms = int(s[0])
        elif len(s) >= 4 and s[-2:] == ["xlo", "xhi"]:
            lo[0], hi[0] = float(s[0]), float(s[1])
        elif len(s) >= 4 and s[-2:] == ["ylo", "yhi"]:
            lo[1], hi[1] = float(s[0]), float(s[1])
        elif len(s) >= 4 and s[-2:] == ["zlo", "zhi"]:
            lo[2], hi[2] = float(s[0]), float(s[1])
        elif len(s) >= 6 and s[-3:] == ["xy", "xz", "yz"]:
            tilt = np.array([float(s[0]), float(s[1]), float(s[2])])
        elif len(s) == 1 and s[0] == "Atoms":
            i += 1
            while len(atoms) < natoms:
                i += 1
                t = lines[i].split("#")[0].split()
                if t:
                    atoms.append([int(t[0]), int(t[1]), float(t[2]), float(t[3]), float(t[4])])
            break
        i += 1
    atoms.sort(key=lambda r: r[0])
    arr = np.array(atoms)
    lx, ly, lz = hi - lo
    xy, xz, yz = tilt
    lat = np.array([[lx, 0, 0], [xy, ly, 0], [xz, yz, lz]], dtype=np.float64)
    pos = arr[:, 2:5] - lo
    return Cell(lat, pos, (arr[:, 1].astype(np.int32) - 1))
