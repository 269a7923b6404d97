"""Seeded synthetic inputs with the shapes of the benchmark configurations (no dataset is involved).

* water_cluster(n, seed): n rigid waters (O-H 0.9572 A, H-O-H 104.52 deg), oxygens uniform in a cube of
  edge 8 (n/16)^(1/3) A by rejection until all O-O >= 2.6 A, orientations uniform on SO(3).
  n = 16, seed 0 is the 48-atom full-QC AM1 configuration.
* qcmm_water_box(seed): QC region = 21 waters + one hydroxide (O-H 0.97 A; 65 atoms, charge -1)
  placed as above at the centre of a 50 A cube holding 4000 TIP3P waters (charges O -0.834, H +0.417) by
  rejection with O-O >= 2.6 A to every oxygen already placed.  Non-periodic.
* perturbed_frames(xyz, n, sigma, seed): n copies with independent Gaussian displacements, a stand-in for
  molecular-dynamics frames of one system.
* qcmm_water_box_frames(n): the QC/MM water box (seed 1) and n of its perturbed frames (0.02 A, seed 11), the
  benchmark's input.
* large_qcmm(seed): 200 QC waters (600 atoms, N = 1200, neutral) in 20000 TIP3P waters in an 85 A cube, seed 4.
"""

import math

import numpy as np

OH = 0.9572
HOH = math.radians(104.52)
OH_HYDROXIDE = 0.97
TIP3P_O, TIP3P_H = -0.834, 0.417


def _water_local():
    h = OH * math.sin(HOH / 2.0)
    z = OH * math.cos(HOH / 2.0)
    return np.array([[0.0, 0.0, 0.0], [h, 0.0, z], [-h, 0.0, z]])


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


class _Grid:
    """Cell grid over oxygen positions for the O-O rejection test."""

    def __init__(self, lo, edge, rmin):
        self.lo, self.cell, self.rmin2 = np.asarray(lo, float), rmin, rmin * rmin
        self.n = max(1, int(edge / rmin))
        self.cells = {}

    def key(self, p):
        return tuple(np.floor((p - self.lo) / self.cell).astype(int))

    def ok(self, p):
        k = self.key(p)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for q in self.cells.get((k[0] + dx, k[1] + dy, k[2] + dz), ()):
                        d = p - q
                        if d @ d < self.rmin2:
                            return False
        return True

    def add(self, p):
        self.cells.setdefault(self.key(p), []).append(np.array(p))


def _place(rng, n, lo, edge, grid, max_tries=2000000):
    out, tries = [], 0
    while len(out) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place %d molecules in a %.1f A cube" % (n, edge))
        p = lo + rng.uniform(0.0, edge, size=3)
        if grid.ok(p):
            grid.add(p)
            out.append(p)
    return out


def water_cluster(n, seed=0, centre=None, min_oo=2.6):
    """(atomic numbers, coordinates [3n, 3]) of an n-water cluster."""
    rng = np.random.default_rng(seed)
    edge = 8.0 * (n / 16.0) ** (1.0 / 3.0)
    c = np.zeros(3) if centre is None else np.asarray(centre, float)
    lo = c - 0.5 * edge
    grid = _Grid(lo - 10.0, edge + 20.0, min_oo)
    loc = _water_local()
    Z, X = [], []
    for o in _place(rng, n, lo, edge, grid):
        R = _random_rotation(rng)
        X.extend(o + loc @ R.T)
        Z.extend([8, 1, 1])
    return np.array(Z), np.array(X)


def qcmm_water_box(seed=1, n_qc_waters=21, n_mm_waters=4000, box=50.0, min_oo=2.6, hydroxide=True):
    """Returns (atomic numbers, coordinates, MM charges (0 on QC atoms), QC atom indices, QC charge)."""
    rng = np.random.default_rng(seed)
    n_qc_mol = n_qc_waters + (1 if hydroxide else 0)
    edge = 8.0 * (n_qc_mol / 16.0) ** (1.0 / 3.0)
    centre = np.full(3, 0.5 * box)
    grid = _Grid(np.zeros(3) - 5.0, box + 10.0, min_oo)
    loc = _water_local()
    Z, X, Q = [], [], []
    qc_o = _place(rng, n_qc_mol, centre - 0.5 * edge, edge, grid)
    for k, o in enumerate(qc_o):
        R = _random_rotation(rng)
        if k < n_qc_waters:
            X.extend(o + loc @ R.T); Z.extend([8, 1, 1])
        else:   # hydroxide
            X.extend([o, o + OH_HYDROXIDE * (R @ np.array([0.0, 0.0, 1.0]))]); Z.extend([8, 1])
    Q.extend([0.0] * len(Z))
    n_qc = len(Z)
    for o in _place(rng, n_mm_waters, np.zeros(3), box, grid):
        R = _random_rotation(rng)
        X.extend(o + loc @ R.T); Z.extend([8, 1, 1]); Q.extend([TIP3P_O, TIP3P_H, TIP3P_H])
    return np.array(Z), np.array(X), np.array(Q), list(range(n_qc)), (-1 if hydroxide else 0)


def large_qcmm(seed=4, n_qc_waters=200, n_mm_waters=20000, box=85.0):
    """The large QC/MM system: a 200-water QC region (600 atoms, 1200 basis functions, neutral) at the centre of an
    85 A cube holding 20000 TIP3P waters, placed as qcmm_water_box.  Returns the same tuple."""
    return qcmm_water_box(seed=seed, n_qc_waters=n_qc_waters, n_mm_waters=n_mm_waters, box=box, hydroxide=False)


def perturbed_frames(xyz, n, sigma=0.02, seed=7):
    rng = np.random.default_rng(seed)
    xyz = np.asarray(xyz, float)
    return xyz[None] + rng.normal(scale=sigma, size=(n,) + xyz.shape)


def water_clusters(n_clusters=512, smallest=4, largest=64, seed=2):
    """n_clusters independent water clusters of seeded uniform size (smallest..largest molecules), each placed
    as water_cluster (O positions uniform in a cube of edge 8 (w/16)^(1/3) A, O-O >= 2.6 A, random
    orientations).  Returns a list of (atomic numbers, coordinates)."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(smallest, largest + 1, size=n_clusters)
    return [water_cluster(int(w), seed=seed * 1000003 + k) for k, w in enumerate(sizes)]


def qcmm_water_box_frames(n_frames, seed=1, frame_seed=11, sigma=0.02):
    """The QC/MM water box and n_frames perturbed copies of it: (Z, X, charges, qc_selection, qc_charge, frames)."""
    Z, X, Q, sel, charge = qcmm_water_box(seed=seed)
    return Z, X, Q, sel, charge, perturbed_frames(X, n_frames, sigma=sigma, seed=frame_seed)
