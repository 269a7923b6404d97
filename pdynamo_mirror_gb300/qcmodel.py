"""QCModelMNDO: the MNDO-family QC model on the GB300 path.

Mirrors the keyword surface of pDynamo's QCModelMNDO (pMolecule.QCModelMNDO.pyx:511-621): the first
positional argument or ``mndoModel`` names the Hamiltonian; ``converger`` takes a DIISSCFConverger.
Spin-restricted closed shells (RHF), spin-unrestricted states (UHF, ``isSpinRestricted=False``; with the
ElectronicState's multiplicity) and the fractional occupancies (``occupancyType`` "Fixed Fractional" with the
``numberFractional*HOOs`` / ``LUOs`` options, "Variable Fractional" with ``fermiBroadening``) are on this path;
unknown options raise ValueError, as in the reference.
"""

import numpy as np

from .converger import DIISSCFConverger
from .parameters import HAMILTONIANS, available_elements


class QCModelMNDO:
    def __init__(self, *arguments, **options):
        self.mndoModel = "am1"
        self.converger = None
        self.label = None
        self.isSpinRestricted = True
        self.keepOrbitalData = False
        # occupancy options and their defaults (QCModelMNDO_Allocate in the reference's C core)
        self.occupancyType = "Cardinal"
        self.fermiBroadening = 1.0e3
        self.numberFractional = {"numberFractionalHOOs": 1, "numberFractionalLUOs": 0, "numberFractionalAlphaHOOs": 1,
                                 "numberFractionalAlphaLUOs": 0, "numberFractionalBetaHOOs": 1, "numberFractionalBetaLUOs": 0}
        if len(arguments) > 1:
            raise ValueError("QCModelMNDO takes at most one positional argument.")
        if arguments:
            self.mndoModel = arguments[0]
        self.SetOptions(**options)

    def SetOptions(self, **options):
        if "converger" in options: self.converger = options.pop("converger")
        if "mndoModel" in options: self.mndoModel = options.pop("mndoModel")
        if "label" in options: self.label = options.pop("label")
        if "keepOrbitalData" in options: self.keepOrbitalData = bool(options.pop("keepOrbitalData"))
        if "isSpinRestricted" in options: self.isSpinRestricted = bool(options.pop("isSpinRestricted"))
        if "occupancyType" in options:
            t = options.pop("occupancyType")
            if t not in ("Cardinal", "Fixed Fractional", "Variable Fractional"):
                raise ValueError("Unknown occupancy type: " + str(t) + ".")
            self.occupancyType = t
        if "fermiBroadening" in options: self.fermiBroadening = float(options.pop("fermiBroadening"))
        for k in list(self.numberFractional):
            if k in options: self.numberFractional[k] = int(options.pop(k))
        if options:
            raise ValueError("Invalid options: " + ", ".join(sorted(options)) + ".")
        self.mndoModel = str(self.mndoModel).lower()
        if self.mndoModel not in HAMILTONIANS:
            raise ValueError("Unknown MNDO Hamiltonian: %s." % self.mndoModel)
        if self.converger is None:
            self.converger = DIISSCFConverger()
        if self.label is None:
            self.label = self.mndoModel.upper()

    def GetOption(self, optionName):
        """An option of the model (QCModelMNDO.GetOption, pMolecule.QCModelMNDO.pyx:306-318): the occupancy options;
        AttributeError for unknown names."""
        values = dict(self.numberFractional, isSpinRestricted=self.isSpinRestricted, occupancyType=self.occupancyType,
                      fermiBroadening=self.fermiBroadening)
        if optionName not in values:
            raise AttributeError("Unknown option: " + str(optionName) + ".")
        return values[optionName]

    def IsSpinRestricted(self):
        """Whether the model is spin-restricted (pMolecule.QCModel.pyx:298)."""
        return self.isSpinRestricted

    def AtomicCharges(self, configuration, chargeModel=None, spinDensities=False):
        """Lowdin charges of the QC atoms from the last energy on configuration (QCModelMNDO.AtomicCharges; the
        NDDO basis is orthonormal, so Mulliken charges are the same); with spinDensities their Lowdin spin populations
        (sum over each atom's orbitals of P_alpha - P_beta; zeros for closed shells and spin-restricted states)."""
        if chargeModel not in (None, "Lowdin", "Mulliken"):
            raise ValueError("Unknown QC charge model: " + str(chargeModel) + ".")
        q = getattr(configuration, "qcCharges", None)
        if q is None:
            return None
        if spinDensities:
            sp = getattr(configuration, "qcSpinDensities", None)
            return np.zeros(len(q)) if sp is None else np.array(sp, dtype=np.float64)
        return np.array(q, dtype=np.float64)

    def DipoleMoment(self, configuration, center=None):
        """Dipole moment (Debye) of the QC atoms from the last energy's density (QCModelMNDO_DipoleMoment)."""
        from .properties import qc_dipole
        st = getattr(configuration, "qcState", None)
        if st is None:
            return None
        return qc_dipole(st.zcore, st.norbitals, st.ddp1, st.coordinates3, st.density(), center)

    def BondOrders(self, configuration, chargeModel=None):
        """(Mayer bond orders [n, n], charges, free valences, total valences) of the last energy's density
        (QCModelMNDO.BondOrders, QCModelMNDO_MayerBondOrders)."""
        from .properties import mayer
        st = getattr(configuration, "qcState", None)
        if st is None:
            return None
        return mayer(st.norbitals, st.density())

    def CheckElements(self, atomic_numbers):
        have = set(available_elements(self.mndoModel))
        missing = sorted(set(int(z) for z in atomic_numbers) - have)
        if missing:
            raise ValueError("Error processing some QC parameter files: %s has no parameters for %s." % (self.mndoModel, missing))
