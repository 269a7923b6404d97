"""Properties of a converged density on the host: dipole moments and Mayer bond orders.

Restated from pMolecule-1.9.0/extensions/csource:
* qc_dipole      QCModelMNDO_DipoleMoment (QCModelMNDO.c, constants :601-602): Debye, about `center`;
                 4.8030 q_A (r_A - c) over the QC atoms (Lowdin charges of the density, coordinates in A) minus
                 5.0832 ddp[1] P(s, p_x/y/z) on every atom with p orbitals (basis order s, p_z, p_x, p_y).
* mm_dipole      MMAtomContainer_DipoleMoment (MMAtomContainer.c:77-118): the point charges times
                 (A -> Bohr) x 2.54176568 Debye per e Bohr.
* mayer          QCModelMNDO_MayerBondOrders (QCModelMNDO.c): B_AB = sum over the two atoms' orbitals of P_mn^2 (plus the
                 spin density's squares for open shells); charges 1/2 sum_B B_AB, total valence sum_B B_AB minus the
                 total density's B_AA, free valence the spin density's B_AA (zero for closed shells).
These run on a host copy of one frame's density (N x N); they are not on the hot path.
"""

import numpy as np

DIPFC1, DIPFC2 = 4.8030, 5.0832                           # QCModelMNDO.c:601-602
ANGSTROMS_TO_BOHRS = 1.0e-10 / 5.291772083e-11            # pCore Units.h
DEBYES_PER_E_BOHR = 2.54176568                            # UNITS_DIPOLE_ATOMIC_UNITS_TO_DEBYES
PZ, PX, PY = 1, 2, 3                                      # cinclude/MNDODefinitions.h:17-19


def _blocks(norbitals):
    starts = np.concatenate([[0], np.cumsum(norbitals)[:-1]]).astype(int)
    return starts, np.asarray(norbitals, dtype=int)


def lowdin_charges(zcore, norbitals, density):
    """q_A = Z_A - sum over A's orbitals of P_mm (QCModelMNDO_LowdinCharges; the NDDO basis is orthonormal)."""
    starts, norb = _blocks(norbitals)
    d = np.diag(np.asarray(density))
    return np.array([z - d[s:s + n].sum() for z, s, n in zip(zcore, starts, norb)])


def qc_dipole(zcore, norbitals, ddp1, xyz_angstrom, density, center=None):
    """Dipole moment (Debye) of the QC atoms' charge distribution."""
    P = np.asarray(density)
    X = np.asarray(xyz_angstrom, dtype=np.float64).reshape(-1, 3)
    c = np.zeros(3) if center is None else np.asarray(center, dtype=np.float64)
    q = lowdin_charges(zcore, norbitals, P)
    dip = DIPFC1 * (q[:, None] * (X - c)).sum(0)
    starts, norb = _blocks(norbitals)
    for s, n, d in zip(starts, norb, ddp1):
        if n >= 4:
            h = DIPFC2 * d
            dip = dip - h * np.array([P[s + PX, s], P[s + PY, s], P[s + PZ, s]])
    return dip


def mm_dipole(charges, xyz_angstrom, center=None):
    """Dipole moment (Debye) of point charges (e) at A positions."""
    X = np.asarray(xyz_angstrom, dtype=np.float64).reshape(-1, 3)
    c = np.zeros(3) if center is None else np.asarray(center, dtype=np.float64)
    return (np.asarray(charges, dtype=np.float64)[:, None] * (X - c)).sum(0) * (ANGSTROMS_TO_BOHRS * DEBYES_PER_E_BOHR)


def mayer(norbitals, density, spin_density=None):
    """(bond orders [n, n], charges, free valences, total valences) of a total density (and a spin density)."""
    starts, norb = _blocks(norbitals)

    def blocks(P2):
        n = len(starts)
        B = np.empty((n, n))
        for a in range(n):
            for b in range(n):
                B[a, b] = P2[starts[a]:starts[a] + norb[a], starts[b]:starts[b] + norb[b]].sum()
        return B

    Bt = blocks(np.asarray(density) ** 2)
    B = Bt + (blocks(np.asarray(spin_density) ** 2) if spin_density is not None else 0.0)
    rows = B.sum(1)
    total = rows - np.diag(Bt)          # the first contribution takes the total density's diagonal only
    free = np.diag(B) - np.diag(Bt)     # = the spin density's diagonal blocks (zero for closed shells)
    return B, 0.5 * rows, free, total


class QCState:
    """The QC state an energy leaves on the configuration (the reference's configuration.qcState): one frame's final
    density (kept on the device; copied to the host when a property needs it) with the QC atoms' coordinates (A)
    and element data."""

    def __init__(self, density, hamiltonian, atomic_numbers, xyz_angstrom):
        from .parameters import ElementParameters
        self._density, self._host = density, None
        el = {z: ElementParameters(hamiltonian, z) for z in set(int(z) for z in atomic_numbers)}
        self.atomicNumbers = [int(z) for z in atomic_numbers]
        self.norbitals = [el[z].norbitals for z in self.atomicNumbers]
        self.zcore = [el[z].zcore for z in self.atomicNumbers]
        self.ddp1 = [el[z].ddp[1] for z in self.atomicNumbers]
        self.coordinates3 = np.array(xyz_angstrom, dtype=np.float64).reshape(-1, 3)

    def density(self):
        if self._host is None:
            d = self._density
            self._host = d.cpu().numpy() if hasattr(d, "cpu") else np.asarray(d, dtype=np.float64)
        return self._host

    def __len__(self):
        return len(self.atomicNumbers)
