"""MNDO-family parameters: pDynamo's parameter files -> per-element records for the device.

The numbers come from ``mndo_parameters.json`` (generated from pDynamo's YAML files by
``make_tables.py``).  Processing restates, in Python, what pDynamo does when it loads them:

* unit conversion to atomic units (``pMolecule.MNDOParameters.pyx:309-370``),
* one-centre two-electron integrals and hpp (``MNDOParameters.c:155-240``),
* multipole charge separations ``ddp`` and additive terms ``po`` (``MNDOParameters_FillDDPPO``,
  ``MNDOParameters.c:762-875``, with ``AIJL`` :726 and ``POIJ`` :880),
* STO-6G orbital shells: primitive unnormalisation, exponent scaling by zeta^2 and renormalisation of
  the contracted function (``GaussianBasis_UnnormalizePrimitives`` / ``_ScaleExponents`` /
  ``_Normalize``, ``GaussianBasisCore.c:221,280,309``; ``pMolecule.QCParameters.pyx:131-140``),
* PM6's diatomic core-core pairs (``pMolecule.MNDOParameters.pyx:259-276``, exponents to bohr^-1 :358-363),
  stored per partner by the partner's index in the system's element list (``element_table``).

The output record layout is ``PDG_ELEMENT_STRIDE`` doubles per element as declared in ``include/pdg.h``.
"""

import json, math, os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_PATH = os.path.join(HERE, "mndo_parameters.json")

HAMILTONIANS = ("am1", "mndo", "pm3", "pddgmndo", "pddgpm3", "rm1", "pm6")

# pCore Units (pCore/Units.py:43-44) and pMolecule.MNDOParameters.pyx:18-21.
BOHRS_TO_ANGSTROMS = 5.291772083e-11 / 1.0e-10
ANGSTROMS_TO_BOHRS = 1.0e-10 / 5.291772083e-11
HARTREES_TO_EV = 27.2113834
HARTREES_TO_KCAL = 27.2113834 * 23.060529
HARTREES_TO_KJ = 2625.5

# Record offsets (include/pdg.h).
STRIDE = 128
E_Z, E_NORB, E_ZCORE, E_ALP, E_GPHOT, E_NG, E_NPDDG, E_DD, E_QQ, E_PO = 0, 1, 2, 3, 4, 5, 6, 7, 8, 9
E_GSS, E_GSP, E_GPP, E_GP2, E_HSP, E_HPP = 18, 19, 20, 21, 22, 23
E_BETA, E_USPD, E_FN1, E_FN2, E_FN3, E_PDDGC, E_PDDGE = 24, 28, 32, 36, 40, 44, 48
E_EHEAT, E_EISOL, E_NSHELL, E_NPRIM_S, E_NPRIM_P, E_EXP_S, E_CCBF_S, E_EXP_P, E_CCBF_P = 52, 53, 54, 55, 56, 57, 63, 69, 75
E_DIAT, E_INDEX, E_DIAT_A, E_DIAT_X = 81, 82, 84, 100
MAX_ELEMENTS = 16

_TABLE = None


def table():
    global _TABLE
    if _TABLE is None:
        with open(TABLE_PATH) as f:
            _TABLE = json.load(f)
    return _TABLE


def atomic_mass(atomic_number):
    """Mass (amu) of an element, from pDynamo's element files (parameters/elements/<El>.yaml, "Mass")."""
    m = table().get("masses", {}).get(str(int(atomic_number)))
    if m is None or m <= 0.0:
        raise ValueError("No mass for atomic number %d." % int(atomic_number))
    return float(m)


def available_elements(hamiltonian):
    return sorted(int(z) for z in table()["hamiltonians"][hamiltonian.lower()])


def _factorial(n):
    return float(math.factorial(n))


def _aijl(z1, z2, n1, n2, l):
    """MNDOParameters.c:726 (with the reference's extra factor 2^l)."""
    return (_factorial(n1 + n2 + l) / math.sqrt(_factorial(2 * n1) * _factorial(2 * n2)) *
            (2.0 * z1 / (z1 + z2)) ** n1 * math.sqrt(2.0 * z1 / (z1 + z2)) *
            (2.0 * z2 / (z1 + z2)) ** n2 * math.sqrt(2.0 * z2 / (z1 + z2)) * 2.0 ** l / (z1 + z2) ** l)


def _poij(l, d, fg):
    """Golden-section fit of the additive term (MNDOParameters.c:880-930)."""
    if l == 0:
        return 0.5 / fg
    dsq, a1, a2, f1, f2 = d * d, 0.1, 5.0, 0.0, 0.0
    for _ in range(100):
        delta = a2 - a1
        if delta < 1.0e-8:
            break
        y1, y2 = a1 + delta * 0.382, a1 + delta * 0.618
        if l == 1:
            f1 = (0.25 * (1.0 / y1 - 1.0 / math.sqrt(y1 * y1 + dsq)) - fg) ** 2
            f2 = (0.25 * (1.0 / y2 - 1.0 / math.sqrt(y2 * y2 + dsq)) - fg) ** 2
        else:
            f1 = (0.125 * (1.0 / y1 - 2.0 / math.sqrt(y1 * y1 + 0.5 * dsq) + 1.0 / math.sqrt(y1 * y1 + dsq)) - fg) ** 2
            f2 = (0.125 * (1.0 / y2 - 2.0 / math.sqrt(y2 * y2 + 0.5 * dsq) + 1.0 / math.sqrt(y2 * y2 + dsq)) - fg) ** 2
        if f1 < f2:
            a2 = y2
        else:
            a1 = y1
    return a2 if f1 >= f2 else a1


class ElementParameters:
    """One element of one Hamiltonian in atomic units."""

    def __init__(self, hamiltonian, atomic_number):
        t = table()
        h = hamiltonian.lower()
        try:
            raw = t["hamiltonians"][h][str(int(atomic_number))]
        except KeyError:
            raise ValueError("No %s parameters for atomic number %d." % (hamiltonian, atomic_number))
        self.hamiltonian, self.Z = h, int(atomic_number)
        self.norbitals = int(raw["orbitals"])
        if self.norbitals not in (1, 4):
            raise ValueError("Only s and sp elements are on this path.")
        g = lambda k: float(raw[k])
        self.iii = int(raw["iii"])
        self.ad, self.am, self.aq = g("ad"), g("am"), g("aq")
        self.alp = g("alp") * BOHRS_TO_ANGSTROMS
        self.dd, self.qq, self.zcore, self.gphot, self.pcore = g("dd"), g("qq"), g("zcore"), g("gphot"), g("pcore")
        self.eheat = g("eheat") / HARTREES_TO_KCAL
        self.eisol = g("eisol") / HARTREES_TO_EV
        self.gss, self.gsp, self.gpp, self.gp2, self.hsp = (g(k) / HARTREES_TO_EV for k in ("gss", "gsp", "gpp", "gp2", "hsp"))
        self.hpp = 0.5 * (self.gpp - self.gp2) if self.norbitals >= 4 else 0.0
        self.zetas, self.zetap = g("zetas"), g("zetap")
        self.beta = [g("betas") / HARTREES_TO_EV] + [g("betap") / HARTREES_TO_EV] * (self.norbitals - 1)
        self.uspd = [g("uss") / HARTREES_TO_EV] + [g("upp") / HARTREES_TO_EV] * (self.norbitals - 1)
        self.fn1 = [x[0] / (BOHRS_TO_ANGSTROMS * HARTREES_TO_EV) for x in raw["gaussians"]]
        self.fn2 = [x[1] * BOHRS_TO_ANGSTROMS * BOHRS_TO_ANGSTROMS for x in raw["gaussians"]]
        self.fn3 = [x[2] / BOHRS_TO_ANGSTROMS for x in raw["gaussians"]]
        self.pddgc = [x[0] / HARTREES_TO_EV for x in raw["pddg"]]
        self.pddge = [x[1] / BOHRS_TO_ANGSTROMS for x in raw["pddg"]]
        # PM6 diatomic pairs: partner atomic number -> (coefficient x, exponent a in bohr^-1)
        self.diatomic = {int(d[0]): (float(d[1]), float(d[2]) * BOHRS_TO_ANGSTROMS) for d in raw.get("diatomic", [])}
        self._fill_ddp_po()
        label = ("%ds" % raw["qns"] if raw["qns"] else "") + ("%dp" % raw["qnp"] if raw["qnp"] else "")
        if label not in t["bases"]:
            raise ValueError("No STO-6G orbital basis %s for atomic number %d." % (label, self.Z))
        self._basis(t["bases"][label][: (1 if self.norbitals == 1 else 2)])

    def _fill_ddp_po(self):
        po, ddp, aij = [0.0] * 9, [0.0] * 6, [0.0] * 6
        if self.Z > 2 and self.zetas * self.zetap >= 1.0e-2:
            aij[1] = _aijl(self.zetas, self.zetap, self.iii, self.iii, 1)
            aij[2] = _aijl(self.zetap, self.zetap, self.iii, self.iii, 2)
        po[0] = _poij(0, 1.0, self.gss)
        po[8] = po[0]
        if self.Z > 2:
            d = aij[1] / math.sqrt(12.0)
            ddp[1], po[1] = d, _poij(1, d, self.hsp)
            po[6] = po[0]
            d = math.sqrt(aij[2] / 10.0)
            ddp[2], po[2] = d, _poij(2, d, self.hpp)
        if self.am < 1.0e-4:
            self.am = 1.0
        po[0] = 0.5 / self.am
        if self.ad > 1.0e-5: po[1] = 0.5 / self.ad
        if self.aq > 1.0e-5: po[2] = 0.5 / self.aq
        po[6] = po[0]
        po[8] = po[0]
        ddp[1] = self.dd
        ddp[2] = self.qq * math.sqrt(2.0)
        if self.pcore > 1.0e-5:
            po[8] = self.pcore
        self.po, self.ddp = po, ddp

    def _basis(self, shells):
        zeta = (self.zetas, self.zetap)
        self.shells = []
        for s, sh in enumerate(shells):
            l = {"S": 0, "P": 1}[sh["type"]]
            e0 = np.array(sh["exponents"], dtype=np.float64)
            c0 = np.array(sh["coefficients"], dtype=np.float64)
            ex = 2.0 * e0
            fac = math.pi ** 1.5 / (ex * np.sqrt(ex))
            if l == 1:
                fac = fac / (2.0 * ex)
            c = c0 / np.sqrt(fac)
            e = e0 * zeta[s] * zeta[s]
            a = e[:, None] + e[None, :]
            ov = (math.pi / a) ** 1.5 * (0.5 / a if l == 1 else 1.0)
            c = c / math.sqrt(float(c @ ov @ c))
            self.shells.append((l, e, c))

    def record(self, elements=None):
        """The device record; elements (the system's sorted element list) places the element's own index and its
        PM6 diatomic pairs by partner index."""
        r = np.zeros(STRIDE, dtype=np.float64)
        r[E_Z], r[E_NORB], r[E_ZCORE], r[E_ALP], r[E_GPHOT] = self.Z, self.norbitals, self.zcore, self.alp, self.gphot
        r[E_NG], r[E_NPDDG], r[E_DD], r[E_QQ] = len(self.fn1), len(self.pddgc), self.dd, self.qq
        r[E_PO:E_PO + 9] = self.po
        r[E_GSS], r[E_GSP], r[E_GPP], r[E_GP2], r[E_HSP], r[E_HPP] = self.gss, self.gsp, self.gpp, self.gp2, self.hsp, self.hpp
        r[E_BETA:E_BETA + self.norbitals] = self.beta
        r[E_USPD:E_USPD + self.norbitals] = self.uspd
        for k, (a, b) in enumerate(((E_FN1, self.fn1), (E_FN2, self.fn2), (E_FN3, self.fn3), (E_PDDGC, self.pddgc), (E_PDDGE, self.pddge))):
            if len(b) > 4:
                raise ValueError("more than four core-core Gaussians")
            r[a:a + len(b)] = b
        r[E_EHEAT], r[E_EISOL], r[E_NSHELL] = self.eheat, self.eisol, len(self.shells)
        for l, e, c in self.shells:
            n, oe, oc, on = (len(e), E_EXP_S, E_CCBF_S, E_NPRIM_S) if l == 0 else (len(e), E_EXP_P, E_CCBF_P, E_NPRIM_P)
            r[on] = n
            r[oe:oe + n] = e
            r[oc:oc + n] = c
        if elements is not None:
            if len(elements) > MAX_ELEMENTS:
                raise ValueError("more than %d elements in one QC region" % MAX_ELEMENTS)
            r[E_INDEX] = elements.index(self.Z)
            r[E_DIAT] = 1.0 if self.diatomic else 0.0
            for k, z in enumerate(elements):
                x, a = self.diatomic.get(int(z), (0.0, 0.0))
                r[E_DIAT_X + k], r[E_DIAT_A + k] = x, a
        return r


def element_table(hamiltonian, atomic_numbers):
    """Sorted distinct elements, their stacked records, and the per-atom element index."""
    elements = sorted(set(int(z) for z in atomic_numbers))
    records = np.stack([ElementParameters(hamiltonian, z).record(elements) for z in elements])
    index = np.array([elements.index(int(z)) for z in atomic_numbers], dtype=np.int32)
    return elements, records, index
