"""Test infrastructure: ctypes wrapper for the plain-C CPU restatement (``_build/liboracle.so``).

The library is compiled from ``mndo_oracle.c`` by ``make -C oracle oracle`` (``__graft_entry__.build()``
runs this on every machine).  Only tests, ``smoke()`` and the CPU-baseline leg of ``bench.py`` use it.
Energies are in Hartree, gradients in Hartree/Bohr, coordinates in Angstrom.
"""

import ctypes, os, subprocess

import numpy as np

from .rawtables import raw_arrays

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


class _Options(ctypes.Structure):
    _fields_ = [("densityTolerance", ctypes.c_double), ("diisOnset", ctypes.c_double),
                ("energyTolerance", ctypes.c_double), ("maximumSCFCycles", ctypes.c_int),
                ("history", ctypes.c_int), ("useRCA", ctypes.c_int)]


def build():
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        pd = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        pi = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.oracle_hamiltonian_create.restype = P
        L.oracle_hamiltonian_create.argtypes = [I, pi, pi, pd, pi, pd, pi, pd, pi, pi, pi, pd, pd, pi, pd]
        L.oracle_hamiltonian_free.argtypes = [P]
        L.oracle_element_derived.argtypes = [P, I, pd]
        L.oracle_energy.argtypes = [P, I, pi, pd, I, P, ctypes.POINTER(_Options), pd, I, pd, P, P,
                                    ctypes.POINTER(I), P]
        L.oracle_energy_open.argtypes = [P, I, pi, pd, D, D, I, I, pi, D, P, ctypes.POINTER(_Options), pd, P, P, pd, P,
                                         ctypes.POINTER(I), P, P]
        L.oracle_fock.argtypes = [P, I, pi, pd, P, pd, pd, pd]
        L.oracle_gradients.argtypes = [P, I, pi, pd, pd, pd]
        L.oracle_abfs_knots.argtypes = [D, D, D, I, I, pd, pd]
        L.oracle_qcmm.argtypes = [I, D, D, I, P, P, I, pd, I, pd, pd, P, pd, P, P]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Hamiltonian:
    def __init__(self, hamiltonian, atomic_numbers):
        self.name = hamiltonian
        self.elements = sorted(set(int(z) for z in atomic_numbers))
        self._keep = raw_arrays(hamiltonian, self.elements)
        self.handle = lib().oracle_hamiltonian_create(len(self.elements), *self._keep)
        if not self.handle:
            raise ValueError("oracle covers s and sp elements only")

    def __del__(self):
        try:
            lib().oracle_hamiltonian_free(self.handle)
        except Exception:
            pass

    def derived(self, z):
        out = np.zeros(9 + 6 + 15 + 8 + 20 + 16 + 16)
        lib().oracle_element_derived(self.handle, self.elements.index(z), out)
        names, o = {}, 0
        for key, n in (("po", 9), ("ddp", 6), ("dd", 1), ("qq", 1), ("am", 1), ("ad", 1), ("aq", 1), ("alp", 1),
                       ("zcore", 1), ("eheat", 1), ("eisol", 1), ("gss", 1), ("gsp", 1), ("gpp", 1), ("gp2", 1),
                       ("hsp", 1), ("hpp", 1), ("beta", 4), ("uspd", 4), ("fn1", 4), ("fn2", 4), ("fn3", 4),
                       ("pddgc", 4), ("pddge", 4), ("octei", 16), ("c2o", 16)):
            names[key] = out[o:o + n].copy() if n > 1 else float(out[o]); o += n
        return names


class System:
    """One QC region (closed-shell RHF) under the oracle."""

    def __init__(self, ham, atomic_numbers, charge=0, densityTolerance=1.0e-8, maximumSCFCycles=100, history=10,
                 diisOnset=0.2, energyTolerance=2.0e-4, useRCA=True):
        self.ham = ham
        self.Z = [int(z) for z in atomic_numbers]
        self.idx = np.array([ham.elements.index(z) for z in self.Z], dtype=np.int32)
        self.n = len(self.Z)
        norb = {z: int(o) for z, o in zip(ham.elements, ham._keep[1])}
        self.nbasis = sum(norb[z] for z in self.Z)
        self.charge = int(charge)
        self.options = _Options(densityTolerance, diisOnset, energyTolerance, maximumSCFCycles, history, int(useRCA))
        self.density = None   # warm start across calls, as the reference keeps its state on the configuration

    def energy(self, xyz_angstrom, phi=None, gradients=True, density=None):
        xyz = np.ascontiguousarray(xyz_angstrom, dtype=np.float64).ravel()
        nb = self.nbasis * (self.nbasis + 1) // 2
        use = density is not None or self.density is not None
        P = np.array(density if density is not None else (self.density if self.density is not None else np.zeros(nb)),
                     dtype=np.float64)
        en = np.zeros(8); g = np.zeros(3 * self.n) if gradients else None; q = np.zeros(self.n); h = np.zeros(nb)
        nc = ctypes.c_int(0)
        ph = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
        rc = lib().oracle_energy(self.ham.handle, self.n, self.idx, xyz, self.charge, _ptr(ph), ctypes.byref(self.options),
                                 P, int(use), en, _ptr(g), _ptr(q), ctypes.byref(nc), _ptr(h))
        self.density = P.copy()
        return {"total_electronic": en[0], "eelectronic": en[1], "enuclear": en[2], "baseline": en[3], "eqcmm": en[4],
                "eoei": en[6], "etei": en[7], "pure_qc_kj": 2625.5 * (en[1] + en[2] + en[3]),
                "gradients": None if g is None else g.reshape(self.n, 3), "density": P, "H": h, "charges": q,
                "ncycles": nc.value, "converged": rc == 0}

    def fock(self, xyz_angstrom, P, phi=None):
        xyz = np.ascontiguousarray(xyz_angstrom, dtype=np.float64).ravel()
        F = np.zeros(self.nbasis * (self.nbasis + 1) // 2); en = np.zeros(3)
        ph = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
        lib().oracle_fock(self.ham.handle, self.n, self.idx, xyz, _ptr(ph), np.ascontiguousarray(P, dtype=np.float64), F, en)
        return F, en

    def gradients(self, xyz_angstrom, P):
        xyz = np.ascontiguousarray(xyz_angstrom, dtype=np.float64).ravel()
        g = np.zeros(3 * self.n)
        lib().oracle_gradients(self.ham.handle, self.n, self.idx, xyz, np.ascontiguousarray(P, dtype=np.float64), g)
        return g.reshape(self.n, 3)


def abfs_knots(inner=8.0, outer=12.0, width2=None, point_density=50):
    """QC/MM Delta/Gaussian ABFS spline knots: x = r^2 (A^2), y (a.u.)."""
    if width2 is None:
        width2 = 2.0 * 5.291772083e-11 / 1.0e-10
    x = np.zeros(4096); y = np.zeros(4096)
    n = lib().oracle_abfs_knots(inner, outer, width2, point_density, 4096, x, y)
    return x[:n].copy(), y[:n].copy()


def qcmm(model, qcxyz, mmxyz, mmq, qcq=None, knots=None, inner=8.0, outer=12.0):
    """Potentials (a.u.) at QC atoms and, with charges, gradients (Eh/Bohr) on QC and MM atoms.
    model "full" is NBModelFull (1/r), "abfs" the ABFS spline."""
    qcxyz = np.ascontiguousarray(qcxyz, dtype=np.float64).ravel(); mmxyz = np.ascontiguousarray(mmxyz, dtype=np.float64).ravel()
    mmq = np.ascontiguousarray(mmq, dtype=np.float64)
    n, m = len(qcxyz) // 3, len(mmq)
    phi = np.zeros(n)
    gq = np.zeros(3 * n) if qcq is not None else None
    gm = np.zeros(3 * m) if qcq is not None else None
    qq = None if qcq is None else np.ascontiguousarray(qcq, dtype=np.float64)
    x, y = (None, None) if knots is None else (np.ascontiguousarray(knots[0]), np.ascontiguousarray(knots[1]))
    lib().oracle_qcmm(1 if model == "abfs" else 0, inner, outer, 0 if x is None else len(x), _ptr(x), _ptr(y),
                      n, qcxyz, m, mmxyz, mmq, _ptr(qq), phi, _ptr(gq), _ptr(gm))
    return phi, (None if gq is None else gq.reshape(n, 3)), (None if gm is None else gm.reshape(m, 3))


OCCUPANCY_TYPES = {"Cardinal": 0, "Fixed Fractional": 1, "Variable Fractional": 2}


def energy_open(ham, atomic_numbers, xyz_angstrom, charge=0, multiplicity=1, isSpinRestricted=True, occupancyType="Cardinal",
                numberFractional=(1, 0, 1, 0, 1, 0), fermiBroadening=1.0e3, densityTolerance=1.0e-8, maximumSCFCycles=500,
                history=10, diisOnset=0.2, energyTolerance=2.0e-4, useRCA=True, gradients=True, phi=None, start=None):
    """Open-shell / fractional-occupancy QC energy (pMolecule.QCModelMNDO keywords isSpinRestricted, occupancyType),
    alpha and beta charges as QCModel.CrossCheckModelAndState (pMolecule.QCModel.pyx:91-140) forms them.  start: packed
    start densities, (alpha, beta) when unrestricted or the total density when restricted, in place of the diagonal
    guess."""
    Z = [int(z) for z in atomic_numbers]
    idx = np.array([ham.elements.index(z) for z in Z], dtype=np.int32)
    n = len(Z)
    norb = {z: int(o) for z, o in zip(ham.elements, ham._keep[1])}
    nb = sum(norb[z] for z in Z)
    ne = float(sum(int(round(ham.derived(z)["zcore"])) for z in Z)) - float(charge)
    a, b = (ne + (multiplicity - 1.0)) / 2.0, (ne - (multiplicity - 1.0)) / 2.0
    if occupancyType == "Cardinal" and isSpinRestricted and multiplicity > 1:
        raise ValueError("A spin-unrestricted calculation is required for non-singlet states with cardinal occupancy.")
    if occupancyType != "Cardinal" and isSpinRestricted and multiplicity > 1:
        raise ValueError("A spin-unrestricted calculation is required for non-singlet states with fractional occupancy.")
    opts = _Options(densityTolerance, diisOnset, energyTolerance, maximumSCFCycles, history, int(useRCA))
    en = np.zeros(8); g = np.zeros(3 * n) if gradients else None
    PA, PB = np.zeros(nb * (nb + 1) // 2), np.zeros(nb * (nb + 1) // 2)
    nc = ctypes.c_int(0)
    ph = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
    q = np.zeros(n)
    if start is None:
        sa = sb = None
    elif isSpinRestricted:
        sa, sb = np.ascontiguousarray(start, dtype=np.float64), None
    else:
        sa, sb = (np.ascontiguousarray(x, dtype=np.float64) for x in start)
    for x in (sa, sb):
        if x is not None and x.shape != (nb * (nb + 1) // 2,):
            raise ValueError("start densities must be packed lower triangles of %d elements" % (nb * (nb + 1) // 2))
    rc = lib().oracle_energy_open(ham.handle, n, idx, np.ascontiguousarray(xyz_angstrom, dtype=np.float64).ravel(), a, b,
                                  int(bool(isSpinRestricted)), OCCUPANCY_TYPES[occupancyType],
                                  np.ascontiguousarray(numberFractional, dtype=np.int32), fermiBroadening, _ptr(ph),
                                  ctypes.byref(opts), en, _ptr(g), _ptr(q), PA, _ptr(PB), ctypes.byref(nc), _ptr(sa), _ptr(sb))
    if rc == 4:
        raise ValueError("invalid occupancy settings")
    out = {"total_electronic": en[0], "eelectronic": en[1], "enuclear": en[2], "baseline": en[3], "eqcmm": en[4],
           "eocc": en[5], "eoei": en[6], "etei": en[7], "charges": q,
           "pure_qc_kj": 2625.5 * (en[1] + en[2] + en[3]), "gradients": None if g is None else g.reshape(n, 3),
           "ncycles": nc.value, "converged": rc == 0}
    if isSpinRestricted:
        out["density"] = PA
    else:
        out["density_alpha"], out["density_beta"], out["density"] = PA, PB, PA + PB
    return out
