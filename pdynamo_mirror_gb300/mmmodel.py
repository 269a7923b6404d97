"""MM side of a QC/MM system for NBModelABFS's MM/MM and QC/MM Lennard-Jones energies.

The reference builds these from an MM force field (MMModelOPLS / MMModelCHARMM with parameter files and
connectivity); here the caller supplies what the energy needs, in the reference's terms:

* ``LJParameterContainer``  per-type epsilon (kJ/mol) and sigma (A) and the table rule of
  LJParameterContainer_MakeTableOPLS / _MakeTableAMBER (pMolecule-1.9.0/extensions/csource/LJParameterContainer.c:
  100-103, 185-210): OPLS A = 4 e s^12, B = 4 e s^6 with s = sqrt(s_i s_j); AMBER A = e s^12, B = 2 e s^6 with
  s = (s_i + s_j) / 2; e = sqrt(e_i e_j).  ``Scale`` multiplies epsilon, as LJParameterContainer_Scale does (:130-143).
* ``MMModel``  per-atom charges and LJ types, the LJ parameters and the 1-4 LJ parameters, the exclusion pairs and
  the 1-4 pairs (the reference's MMAtomContainer, ljParameters, ljParameters14, exclusions, interactions14 handed to
  NBModelABFS.SetUp, pMolecule.NBModelABFS.pyx:181).  ``MMModel.TIP3PWater`` builds one for systems of waters.
* ``MMInteractions``  the device evaluation through pdg_mm_create / pdg_mm_energy_gradients (MM/MM Elect., MM/MM LJ,
  their 1-4 terms, QC/MM LJ and its 1-4 term, labelled as NBModelABFSState.GetEnergies does) and, when the model has
  them, the harmonic bond and angle terms through pdg_mm_bonded_* (HarmonicBondContainer_Energy,
  HarmonicAngleContainer_Energy; "Harmonic Bond", "Harmonic Angle"), with the terms among QC atoms only or fixed atoms
  only left out as the reference deactivates them (pMolecule-1.9.0/pMolecule/EnergyModel.py:118-143).
"""

import ctypes

import numpy as np
import torch

from . import _native

# TIP3P (Jorgensen, Chandrasekhar, Madura, Impey, Klein, J. Chem. Phys. 79, 926 (1983)): charges and the oxygen's
# LJ parameters (epsilon 0.1521 kcal/mol, sigma 3.15061 A); hydrogens carry no LJ term.
TIP3P_CHARGE_O, TIP3P_CHARGE_H = -0.834, 0.417
TIP3P_EPSILON_O, TIP3P_SIGMA_O = 0.1521 * 4.184, 3.15061
# The flexible water of the reference's OPLS files (parameters/forceFields/opls/protein/harmonicBondParameters.yaml:359,
# harmonicAngleParameters.yaml:988): HW-OW 0.9572 A with 529.60 kcal/mol/A^2, HW-OW-HW 104.52 deg with 34.05
# kcal/mol/rad^2, E = k (x - x0)^2, converted to kJ/mol and radians as HarmonicBondParameterContainer /
# HarmonicAngleParameterContainer.ProcessRawItems do (1 kcal = 4.184 kJ).
WATER_OH_R0, WATER_OH_K = 0.9572, 529.60 * 4.184
WATER_HOH_THETA0, WATER_HOH_K = np.radians(104.52), 34.05 * 4.184


class LJParameterContainer:
    """LJ types with epsilon (kJ/mol) and sigma (A); rule "OPLS" (geometric sigma) or "AMBER" (arithmetic)."""

    def __init__(self, epsilon, sigma, rule="OPLS"):
        self.epsilon = np.array(epsilon, dtype=np.float64).ravel()
        self.sigma = np.array(sigma, dtype=np.float64).ravel()
        if self.epsilon.shape != self.sigma.shape or len(self.epsilon) == 0:
            raise ValueError("epsilon and sigma must have one entry per LJ type.")
        if rule not in ("OPLS", "AMBER"):
            raise ValueError("Invalid LJ combining rule: " + str(rule) + ".")
        self.rule = rule

    @property
    def ntypes(self):
        return len(self.epsilon)

    def Scale(self, scale):
        """A copy with epsilon times scale (the tables scale with it)."""
        return LJParameterContainer(self.epsilon * float(scale), self.sigma, self.rule)

    def tables(self):
        """Full (ntypes x ntypes) tables A (kJ/mol A^12) and B (kJ/mol A^6): E = A / r^12 - B / r^6."""
        e = np.sqrt(np.outer(self.epsilon, self.epsilon))
        if self.rule == "OPLS":
            s = np.sqrt(np.outer(self.sigma, self.sigma))
        else:
            s = 0.5 * np.add.outer(self.sigma, self.sigma)
        s6 = s ** 6
        s12 = s6 * s6
        if self.rule == "OPLS":
            e = 4.0 * e
        else:
            s6 = 2.0 * s6
        return e * s12, e * s6


def _pairs(p, n):
    a = np.array(p if p is not None else [], dtype=np.int64).reshape(-1, 2)
    if len(a) and (a.min() < 0 or a.max() >= n or (a[:, 0] == a[:, 1]).any()):
        raise ValueError("Pair indices out of range or self pairs.")
    return a


class MMModel:
    """Charges (e) and LJ types of every atom, LJ parameters, exclusions and 1-4 pairs."""

    def __init__(self, charges, ljTypes, ljParameters, ljParameters14=None, exclusions=None, interactions14=None, bonds=None,
                 angles=None):
        self.charges = np.array(charges, dtype=np.float64).ravel()
        self.ljTypes = np.array(ljTypes, dtype=np.int64).ravel()
        n = len(self.charges)
        if self.ljTypes.shape != (n,):
            raise ValueError("One LJ type per atom.")
        self.ljParameters = ljParameters
        self.ljParameters14 = ljParameters if ljParameters14 is None else ljParameters14
        if self.ljParameters14.ntypes != ljParameters.ntypes or self.ljParameters14.rule != ljParameters.rule:
            raise ValueError("The 1-4 LJ parameters must have the same types and rule.")
        if n and (self.ljTypes.min() < 0 or self.ljTypes.max() >= ljParameters.ntypes):
            raise ValueError("LJ type out of range.")
        self.exclusions = _pairs(exclusions, n)
        self.interactions14 = _pairs(interactions14, n)
        # harmonic terms: bonds (i, j, r0 A, k kJ/mol/A^2), angles (i, j apex, k, theta0 rad, k kJ/mol/rad^2)
        b = np.array(bonds if bonds is not None else [], dtype=np.float64).reshape(-1, 4)
        a = np.array(angles if angles is not None else [], dtype=np.float64).reshape(-1, 5)
        self.bonds, self.bondParameters = b[:, :2].astype(np.int64), b[:, 2:].copy()
        self.angles, self.angleParameters = a[:, :3].astype(np.int64), a[:, 3:].copy()
        for idx in (self.bonds, self.angles):
            if idx.size and (idx.min() < 0 or idx.max() >= n):
                raise ValueError("Bond or angle atom out of range.")

    @property
    def natoms(self):
        return len(self.charges)

    @classmethod
    def TIP3PWater(cls, atomicNumbers, coordinates3, bondCutoff=1.25, flexible=False):
        """Waters (and hydroxides): each hydrogen bonds to the nearest oxygen within bondCutoff (A); TIP3P charges
        and oxygen LJ (hydroxide O-H pairs take the water charges of their atoms); exclusions within each
        molecule (O-H and H-H); no 1-4 pairs.  flexible adds the O-H bonds and H-O-H angles of the reference's OPLS
        water, so that MM waters can move in dynamics."""
        Z = np.asarray(atomicNumbers)
        X = np.asarray(coordinates3, dtype=np.float64).reshape(len(Z), 3)
        if not set(np.unique(Z)) <= {1, 8}:
            raise ValueError("TIP3PWater takes oxygen and hydrogen atoms only.")
        oxy = np.nonzero(Z == 8)[0]
        owner = {}
        for h in np.nonzero(Z == 1)[0]:
            d = np.linalg.norm(X[oxy] - X[h], axis=1)
            k = int(np.argmin(d))
            if d[k] > bondCutoff:
                raise ValueError("Hydrogen %d is bonded to no oxygen." % h)
            owner.setdefault(int(oxy[k]), []).append(int(h))
        excl = []
        for o, hs in owner.items():
            excl += [(o, h) for h in hs]
            excl += [(hs[a], hs[b]) for a in range(len(hs)) for b in range(a + 1, len(hs))]
        charges = np.where(Z == 8, TIP3P_CHARGE_O, TIP3P_CHARGE_H)
        lj = LJParameterContainer([TIP3P_EPSILON_O, 0.0], [TIP3P_SIGMA_O, 0.0], rule="OPLS")
        bonds, angles = [], []
        if flexible:
            for o in sorted(owner):
                hs = owner[o]
                bonds += [(o, h, WATER_OH_R0, WATER_OH_K) for h in hs]
                if len(hs) == 2:
                    angles.append((hs[0], o, hs[1], WATER_HOH_THETA0, WATER_HOH_K))
        return cls(charges, np.where(Z == 8, 0, 1), lj, exclusions=excl, bonds=bonds, angles=angles)


class MMInteractions:
    """Device evaluation of the MM/MM and QC/MM LJ energies of an MMModel under an NBModelABFS.

    flags: the QC atoms (qcSelection) interact with the MM atoms through LJ only; fixedAtoms leave out pairs of two
    fixed atoms."""

    def __init__(self, mmModel, nbModel, qcSelection, fixedAtoms, device):
        n = mmModel.natoms
        flags = np.full(n, _native.MM_FLAG_MM, dtype=np.uint8)
        qc = np.asarray(qcSelection or [], dtype=np.int64)
        flags[qc] = _native.MM_FLAG_QC_LJ
        if fixedAtoms:
            flags[np.asarray(fixedAtoms, dtype=np.int64)] |= _native.MM_FLAG_FIXED
        self.flags = flags
        self.has14 = len(mmModel.interactions14) > 0
        self.has_qc = len(qc) > 0
        A, B = mmModel.ljParameters.tables()
        A14, B14 = mmModel.ljParameters14.tables()
        c = lambda a, t: np.ascontiguousarray(a, dtype=t)
        arrays = dict(q=c(mmModel.charges, np.float64), t=c(mmModel.ljTypes, np.int32), f=c(flags, np.uint8), A=c(A, np.float64),
                      B=c(B, np.float64), A14=c(A14, np.float64), B14=c(B14, np.float64),
                      ex=c(mmModel.exclusions.ravel(), np.int32), p14=c(mmModel.interactions14.ravel(), np.int32))
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p) if a.size else None
        L = _native.load()
        h = ctypes.c_void_p()
        _native.check(L.pdg_mm_create(n, p(arrays["q"]), p(arrays["t"]), p(arrays["f"]), mmModel.ljParameters.ntypes,
                                      p(arrays["A"]), p(arrays["B"]), p(arrays["A14"]), p(arrays["B14"]),
                                      len(mmModel.exclusions), p(arrays["ex"]), len(mmModel.interactions14), p(arrays["p14"]),
                                      nbModel.innerCutoff, nbModel.outerCutoff, nbModel.dampingCutoff, nbModel.dielectric,
                                      nbModel.electrostaticScale14, ctypes.byref(h)), "pdg_mm_create")
        self.handle, self.n, self.device = h, n, device
        self._ws = None
        # harmonic terms, those among QC atoms only or among fixed atoms only left out (EnergyModel.py:118-143)
        qcset, fixset = set(qc.tolist()), set(fixedAtoms or [])

        def active(atoms):
            return not (all(a in qcset for a in atoms) or all(a in fixset for a in atoms))
        kb = [t for t in range(len(mmModel.bonds)) if active(mmModel.bonds[t].tolist())]
        ka = [t for t in range(len(mmModel.angles)) if active(mmModel.angles[t].tolist())]
        self.has_bonds, self.has_angles = len(kb) > 0, len(ka) > 0
        self.bonded = None
        if kb or ka:
            bi = c(mmModel.bonds[kb].ravel(), np.int32); bp = c(mmModel.bondParameters[kb][:, [0, 1]].ravel(), np.float64)
            ai = c(mmModel.angles[ka].ravel(), np.int32); ap = c(mmModel.angleParameters[ka][:, [0, 1]].ravel(), np.float64)
            hb = ctypes.c_void_p()
            _native.check(L.pdg_mm_bonded_create(n, len(kb), p(bi), p(bp), len(ka), p(ai), p(ap), ctypes.byref(hb)), "pdg_mm_bonded_create")
            self.bonded = hb

    def __del__(self):
        if getattr(self, "handle", None):
            try:
                _native.load().pdg_mm_destroy(self.handle)
            except Exception:
                pass
            self.handle = None
        if getattr(self, "bonded", None):
            try:
                _native.load().pdg_mm_bonded_destroy(self.bonded)
            except Exception:
                pass
            self.bonded = None

    def run(self, frames, gradients=True):
        """frames: device tensor [F, n, 3] (A).  Returns (energies [F, 8] kJ/mol in the order of _native.MM_TERMS,
        gradients [F, n, 3] kJ/mol/A or None)."""
        F = frames.shape[0]
        L = _native.load()
        need = L.pdg_mm_workspace_bytes(self.handle, F)
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        X = frames.contiguous()
        E = torch.zeros((F, len(_native.MM_TERMS)), dtype=torch.float64, device=self.device)
        G = torch.empty((F, self.n, 3), dtype=torch.float64, device=self.device) if gradients else None
        st = _native.stream_handle(torch.cuda.current_stream(self.device))
        E6 = torch.empty((F, 6), dtype=torch.float64, device=self.device)
        _native.check(L.pdg_mm_energy_gradients(self.handle, F, _native.ptr(X), _native.ptr(E6), _native.ptr(G), _native.ptr(self._ws),
                                                self._ws.numel(), st), "pdg_mm_energy_gradients")
        E[:, :6] = E6
        if self.bonded is not None:
            Eb = torch.empty((F, 2), dtype=torch.float64, device=self.device)
            _native.check(L.pdg_mm_bonded_energy_gradients(self.bonded, F, _native.ptr(X), _native.ptr(Eb), _native.ptr(G), st),
                          "pdg_mm_bonded_energy_gradients")
            E[:, 6:] = Eb
        return E, G

    def term_names(self):
        """The labels the reference reports for this model (NBModelABFSState.GetEnergies)."""
        names = ["MM/MM Elect.", "MM/MM LJ"]
        if self.has14:
            names += ["MM/MM 1-4 Elect.", "MM/MM 1-4 LJ"]
        if self.has_qc:
            names += ["QC/MM LJ"] + (["QC/MM 1-4 LJ"] if self.has14 else [])
        names += (["Harmonic Bond"] if self.has_bonds else []) + (["Harmonic Angle"] if self.has_angles else [])
        return names
