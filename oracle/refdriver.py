"""Test infrastructure: ctypes driver for pDynamo's own compiled C core (``_ref/libpdynref.so``).

The shared library is built by ``make -C oracle ref`` from the unmodified reference sources plus
``ref_shim.c`` (a C restatement of the Pyrex glue).  It exists only where the reference tree is
present; everything here raises ``RefUnavailable`` otherwise.  Only tests, fixture generators
and the CPU-baseline leg of ``bench.py`` use this module.
"""

import ctypes, os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libpdynref.so")

from .rawtables import MAXPRIM, PARAM_PATH, raw_arrays  # noqa: F401


class RefUnavailable(RuntimeError):
    pass


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RefUnavailable("reference library not built: " + LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        pd = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        pi = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.ref_hamiltonian_create.restype = P
        L.ref_hamiltonian_create.argtypes = [I, pi, pi, pd, pi, pd, pi, pd, pi, pi, pi, pd, pd, pi, pd]
        L.ref_element_derived.argtypes = [P, I, pd]
        L.ref_element_basis.argtypes = [P, I, pd, pd]
        L.ref_system_create.restype = P
        L.ref_system_create.argtypes = [P, I, pi, I, I, D, I, I, D, D, I]
        L.ref_system_nbasis.argtypes = [P]
        L.ref_system_energy.argtypes = [P, pd, P, I, pd, pd, P, P, ctypes.POINTER(I)]
        L.ref_system_fock.argtypes = [P, pd, P, pd, pd, pd]
        L.ref_system_gradients.argtypes = [P, pd, pd, pd]
        L.ref_system_get_density.argtypes = [P, pd]
        L.ref_system_set_density.argtypes = [P, pd]
        L.ref_system_free.argtypes = [P]
        L.ref_abfs_create.restype = P
        L.ref_abfs_create.argtypes = [D, D, I, pd, pd]
        L.ref_abfs_spline.argtypes = [P, I, pd, pd, pd]
        L.ref_abfs_qcmm.argtypes = [P, P, pd, I, pd, pd, pd, pd, pd, pd]
        L.ref_system_create_open.restype = P
        L.ref_system_create_open.argtypes = [P, I, pi, D, D, I, I, pi, D, I, D, I, I, D, D, I]
        L.ref_system_get_densities.argtypes = [P, pd, P]
        L.ref_system_properties.argtypes = [P, pd, pd, pd, pd, pd]
        L.ref_mmmm_energy.argtypes = [I, pd, pd, pi, pi, I, pd, pd, pd, pd, I, I, pi, I, pi, D, D, D, D, D, D, pd, pd]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class RefHamiltonian:
    """The reference's parameter set for one Hamiltonian restricted to the given elements."""

    def __init__(self, hamiltonian, atomic_numbers):
        self.name = hamiltonian
        self.elements = sorted(set(int(z) for z in atomic_numbers))
        self._keep = raw_arrays(hamiltonian, self.elements)
        self.handle = lib().ref_hamiltonian_create(len(self.elements), *self._keep)

    def derived(self, z):
        out = np.zeros(9 + 6 + 15 + 8 + 20 + 16 + 16)
        lib().ref_element_derived(self.handle, self.elements.index(z), out)
        names = {}
        o = 0
        for key, n in (("po", 9), ("ddp", 6), ("dd", 1), ("qq", 1), ("am", 1), ("ad", 1), ("aq", 1), ("alp", 1),
                       ("zcore", 1), ("eheat", 1), ("eisol", 1), ("gss", 1), ("gsp", 1), ("gpp", 1), ("gp2", 1),
                       ("hsp", 1), ("hpp", 1), ("beta", 4), ("uspd", 4), ("fn1", 4), ("fn2", 4), ("fn3", 4),
                       ("pddgc", 4), ("pddge", 4), ("octei", 16), ("c2o", 16)):
            names[key] = out[o:o + n].copy() if n > 1 else float(out[o]); o += n
        return names

    def nuclear_charge(self, z):
        """The element's core charge (zcore), as the QC atom container sums it."""
        return int(round(self.derived(z)["zcore"]))

    def basis(self, z):
        e = np.zeros(2 * MAXPRIM); c = np.zeros(2 * MAXPRIM)
        lib().ref_element_basis(self.handle, self.elements.index(z), e, c)
        return e.reshape(2, MAXPRIM), c.reshape(2, MAXPRIM)


class RefSystem:
    """One QC region under the reference model: energies in Hartree, gradients returned in Hartree/Bohr."""

    KJ_PER_HARTREE = 2625.5
    ANGSTROMS_TO_BOHRS = 1.0e-10 / 5.291772083e-11

    OCCUPANCY_TYPES = {"Cardinal": 0, "Fixed Fractional": 1, "Variable Fractional": 2}

    def __init__(self, ham, atomic_numbers, charge=0, qcmm=False, densityTolerance=1.0e-8, maximumSCFCycles=100,
                 history=10, diisOnset=0.2, energyTolerance=2.0e-4, useRCA=True, multiplicity=None, isSpinRestricted=True,
                 occupancyType="Cardinal", numberFractional=(1, 0, 1, 0, 1, 0), fermiBroadening=1.0e3):
        """multiplicity None: the closed-shell set-up.  Otherwise the open-shell and fractional-occupancy state of
        QCModelMNDO's keywords, with the alpha and beta electron counts of QCModel.CrossCheckModelAndState
        (pMolecule.QCModel.pyx:91-140); numberFractional = (HOOs, LUOs, alpha HOOs, alpha LUOs, beta HOOs, beta LUOs)."""
        self.ham = ham
        self.atomic_numbers = [int(z) for z in atomic_numbers]
        idx = np.array([ham.elements.index(z) for z in self.atomic_numbers], dtype=np.int32)
        self.n = len(idx)
        self.restricted = True
        if multiplicity is None:
            self.handle = lib().ref_system_create(ham.handle, self.n, idx, int(charge), int(qcmm), densityTolerance,
                                                  maximumSCFCycles, history, diisOnset, energyTolerance, int(useRCA))
        else:
            ne = float(sum(ham.nuclear_charge(z) for z in self.atomic_numbers)) - float(charge)
            a, b = (ne + (multiplicity - 1.0)) / 2.0, (ne - (multiplicity - 1.0)) / 2.0
            if occupancyType == "Cardinal":
                if abs(round(ne) - ne) > 1e-6:
                    raise ValueError("Cardinal occupancy requires integral charge.")
                if isSpinRestricted and multiplicity > 1:
                    raise ValueError("A spin-unrestricted calculation is required for non-singlet states with cardinal occupancy.")
            elif isSpinRestricted and multiplicity > 1:
                raise ValueError("A spin-unrestricted calculation is required for non-singlet states with fractional occupancy.")
            nf = np.ascontiguousarray(numberFractional, dtype=np.int32)
            self.handle = lib().ref_system_create_open(ham.handle, self.n, idx, a, b, int(bool(isSpinRestricted)),
                                                       self.OCCUPANCY_TYPES[occupancyType], nf, fermiBroadening, int(qcmm), densityTolerance,
                                                       maximumSCFCycles, history, diisOnset, energyTolerance, int(useRCA))
            self.restricted = bool(isSpinRestricted)
        self.nbasis = lib().ref_system_nbasis(self.handle)

    def __del__(self):
        try:
            lib().ref_system_free(self.handle)
        except Exception:
            pass

    def energy(self, xyz_angstrom, phi=None, gradients=True):
        """Returns dict: energies (Eh), gradients (Eh/Bohr), density (packed), H (packed), charges, ncycles, converged."""
        xyz = np.ascontiguousarray(xyz_angstrom, dtype=np.float64).ravel()
        en = np.zeros(8); g = np.zeros(3 * self.n); h = np.zeros(self.nbasis * (self.nbasis + 1) // 2)
        q = np.zeros(self.n); nc = ctypes.c_int(0)
        ph = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
        rc = lib().ref_system_energy(self.handle, xyz, _ptr(ph), int(gradients), en, g, _ptr(q), _ptr(h), ctypes.byref(nc))
        P = np.zeros_like(h)
        Q = np.zeros_like(h)
        lib().ref_system_get_densities(self.handle, P, Q.ctypes.data_as(ctypes.c_void_p))
        conv = 1.0 / (self.ANGSTROMS_TO_BOHRS * self.KJ_PER_HARTREE)
        out = {"total_electronic": en[0], "eelectronic": en[1], "enuclear": en[2], "baseline": en[3], "eqcmm": en[4],
               "eocc": en[5], "eoei": en[6], "etei": en[7],
               "pure_qc_kj": self.KJ_PER_HARTREE * (en[1] + en[2] + en[3]),
               "gradients": (g * conv).reshape(self.n, 3), "density": P, "H": h, "charges": q,
               "ncycles": nc.value, "converged": rc == 0}
        if not self.restricted:
            out["density"], out["density_alpha"], out["density_beta"] = P + Q, P, Q
        return out

    def properties(self):
        """Dipole (Debye) and Mayer bond orders, charges, free and total valences of the last energy's density."""
        n = self.n
        d, b, c, f, t = np.zeros(3), np.zeros(n * n), np.zeros(n), np.zeros(n), np.zeros(n)
        lib().ref_system_properties(self.handle, d, b, c, f, t)
        return {"dipole": d, "bond_orders": b.reshape(n, n), "charges": c, "free_valence": f, "total_valence": t}

    def set_density(self, P):
        lib().ref_system_set_density(self.handle, np.ascontiguousarray(P, dtype=np.float64))

    def fock(self, xyz_angstrom, P, phi=None):
        xyz = np.ascontiguousarray(xyz_angstrom, dtype=np.float64).ravel()
        F = np.zeros(self.nbasis * (self.nbasis + 1) // 2); en = np.zeros(3)
        ph = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
        lib().ref_system_fock(self.handle, xyz, _ptr(ph), np.ascontiguousarray(P, dtype=np.float64), F, en)
        return F, en

    def gradients(self, xyz_angstrom, P):
        xyz = np.ascontiguousarray(xyz_angstrom, dtype=np.float64).ravel()
        g = np.zeros(3 * self.n)
        lib().ref_system_gradients(self.handle, xyz, np.ascontiguousarray(P, dtype=np.float64), g)
        return (g / (self.ANGSTROMS_TO_BOHRS * self.KJ_PER_HARTREE)).reshape(self.n, 3)


class RefABFS:
    """The reference ABFS QC/MM pair routines over caller-supplied spline knots."""

    def __init__(self, inner, outer, x, y):
        self.x = np.ascontiguousarray(x, dtype=np.float64); self.y = np.ascontiguousarray(y, dtype=np.float64)
        self.handle = lib().ref_abfs_create(inner, outer, len(self.x), self.x, self.y)

    def spline(self, r2):
        r2 = np.ascontiguousarray(r2, dtype=np.float64); f = np.zeros_like(r2); g = np.zeros_like(r2)
        lib().ref_abfs_spline(self.handle, len(r2), r2, f, g)
        return f, g

    def qcmm(self, system, qcxyz, mmxyz, mmq, qcq):
        n, m = system.n, len(mmq)
        phi = np.zeros(n); gq = np.zeros(3 * n); gm = np.zeros(3 * m)
        lib().ref_abfs_qcmm(self.handle, system.handle, np.ascontiguousarray(qcxyz, dtype=np.float64).ravel(), m,
                            np.ascontiguousarray(mmxyz, dtype=np.float64).ravel(), np.ascontiguousarray(mmq, dtype=np.float64),
                            np.ascontiguousarray(qcq, dtype=np.float64), phi, gq, gm)
        return phi, gq.reshape(n, 3), gm.reshape(m, 3)


def mmmm_energy(xyz, charges, lj_types, flags, epsilon, sigma, epsilon14, sigma14, opls, exclusions, pairs14,
                inner=8.0, outer=12.0, damp=0.5, listCutoff=13.5, dielectric=1.0, scale14=1.0):
    """NBModelABFS MM/MM and QC/MM LJ energies (kJ/mol, the order of oracle.mmmm.TERMS) and gradients (kJ/mol/A)
    from the reference's pair-list generator and pair routine (ref_mmmm_energy in ref_shim.c)."""
    X = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(X)
    i32 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.int32).ravel())
    f64 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())
    ex, p14 = i32(np.asarray(exclusions).reshape(-1, 2)), i32(np.asarray(pairs14).reshape(-1, 2))
    if len(ex) == 0:
        ex = np.zeros(2, np.int32)
    n_ex = len(np.asarray(exclusions).reshape(-1, 2))
    n14 = len(np.asarray(pairs14).reshape(-1, 2))
    if len(p14) == 0:
        p14 = np.zeros(2, np.int32)
    E = np.zeros(6)
    G = np.zeros(3 * n)
    lib().ref_mmmm_energy(n, X.ravel(), f64(charges), i32(lj_types), i32(flags), len(epsilon), f64(epsilon), f64(sigma),
                          f64(epsilon14), f64(sigma14), 1 if opls else 0, n_ex, ex, n14, p14, inner, outer, damp, listCutoff,
                          dielectric, scale14, E, G)
    return E, G.reshape(n, 3)
