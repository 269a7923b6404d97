"""System: the drop-in surface of pDynamo's System for the QC and QC/MM energy + gradient.

``System.DefineQCModel``, ``System.DefineNBModel`` and ``System.Energy(doGradients=True)`` follow
pMolecule/System.py:182-318: energies are returned in kJ/mol, gradients are left on
``system.configuration.gradients3`` in kJ/mol/A, and the energy terms ("Pure QC", "QC/MM Elect.") on
``system.configuration.energyTerms``.  Atoms outside the QC selection are MM point charges.

``System.EnergyBatch`` evaluates many frames (coordinate sets of the same system) in one device call; it
is the throughput form of the same computation.
"""

import numpy as np
import torch

from . import _native
from .engine import GRADIENT_TO_KJ_PER_A, HARTREES_TO_KJ, QCEngine


class ElectronicState:
    def __init__(self, charge=0, multiplicity=1):
        if multiplicity != 1:
            raise ValueError("Only singlet (closed-shell) states are on this path.")
        self.charge, self.multiplicity = int(charge), int(multiplicity)


class Configuration:
    def __init__(self):
        self.energyTerms = {}
        self.gradients3 = None
        self.qcState = None


class SCFNotConverged(ValueError):
    pass


class System:
    """Atoms (atomic numbers), Cartesian coordinates in Angstrom and optional MM point charges."""

    def __init__(self, atomicNumbers, coordinates3, mmCharges=None, label=None):
        self.atomicNumbers = [int(z) for z in atomicNumbers]
        self.coordinates3 = np.array(coordinates3, dtype=np.float64).reshape(len(self.atomicNumbers), 3)
        self.mmCharges = None if mmCharges is None else np.array(mmCharges, dtype=np.float64)
        self.label = label
        self.electronicState = ElectronicState()
        self.qcModel = self.nbModel = None
        self.qcSelection = None
        self.configuration = Configuration()
        self._engine = None

    # -- model definition (System.py:182-230)
    def DefineQCModel(self, qcModel, qcSelection=None):
        n = len(self.atomicNumbers)
        sel = list(range(n)) if qcSelection is None else sorted(set(int(i) for i in qcSelection))
        if not sel or sel[0] < 0 or sel[-1] >= n:
            raise ValueError("Invalid QC selection.")
        qcModel.CheckElements([self.atomicNumbers[i] for i in sel])
        self.qcModel, self.qcSelection = qcModel, sel
        self._engine = None
        self.configuration = Configuration()

    def DefineNBModel(self, nbModel):
        if self.qcModel is None:
            raise ValueError("Define the QC model before the NB model.")
        mm = self.mm_indices()
        if mm and self.mmCharges is None:
            raise ValueError("MM atoms need point charges.")
        self.nbModel = nbModel

    def mm_indices(self):
        qc = set(self.qcSelection or [])
        return [i for i in range(len(self.atomicNumbers)) if i not in qc]

    def engine(self):
        if self._engine is None:
            qcZ = [self.atomicNumbers[i] for i in self.qcSelection]
            self._engine = QCEngine(self.qcModel.mndoModel, qcZ, self.electronicState.charge)
        return self._engine

    def _device_inputs(self, frames):
        dev = self.engine().device
        qc = torch.as_tensor(frames[:, self.qcSelection, :], dtype=torch.float64).to(dev, non_blocking=True).contiguous()
        mm_idx = self.mm_indices() if self.nbModel is not None else []
        if mm_idx:
            mm = torch.as_tensor(frames[:, mm_idx, :], dtype=torch.float64).to(dev, non_blocking=True).contiguous()
            q = torch.as_tensor(self.mmCharges[mm_idx], dtype=torch.float64).to(dev).contiguous()
        else:
            mm = q = None
        return qc, mm, q, mm_idx

    def EnergyBatch(self, frames, doGradients=True, warmStart=True):
        """frames [F, n_atoms, 3] (Angstrom).  Returns (energies kJ/mol [F], gradients kJ/mol/A [F, n, 3] or None,
        terms dict of [F] arrays).  Raises SCFNotConverged if any frame fails to converge."""
        if self.qcModel is None:
            raise ValueError("No QC model defined.")
        frames = np.asarray(frames, dtype=np.float64)
        if frames.ndim == 2:
            frames = frames[None]
        eng = self.engine()
        qc, mm, q, mm_idx = self._device_inputs(frames)
        r = eng.run(qc, self.qcModel.converger, mm, q, self.nbModel if mm is not None else None, gradients=doGradients,
                    warm_start=warmStart)
        E = r["energies"].cpu().numpy()
        st = r["status"].cpu().numpy()
        pure = HARTREES_TO_KJ * (E[:, _native.EN_ELECTRONIC] + E[:, _native.EN_NUCLEAR] + E[:, _native.EN_BASELINE])
        qcmm = HARTREES_TO_KJ * E[:, _native.EN_QCMM]
        terms = {"Pure QC": pure, "QC/MM Elect.": qcmm, "SCF Cycles": r["ncycles"].cpu().numpy(), "Status": st}
        if (st != _native.PDG_OK).any():
            self._engine.density = None
            raise SCFNotConverged("SCF procedure not converged.")
        total = pure + (qcmm if mm is not None else 0.0)
        G = None
        if doGradients:
            G = np.zeros(frames.shape)
            gq = r["qc_gradients"]
            if "qcmm_qc_gradients" in r:
                gq = gq + r["qcmm_qc_gradients"]
                G[:, mm_idx, :] = (r["qcmm_mm_gradients"] * GRADIENT_TO_KJ_PER_A).cpu().numpy()
            G[:, self.qcSelection, :] = (gq * GRADIENT_TO_KJ_PER_A).cpu().numpy()
        return total, G, terms

    def Energy(self, doGradients=False, log=None):
        """Energy (kJ/mol) of the current coordinates; gradients3 in kJ/mol/A when doGradients."""
        total, G, terms = self.EnergyBatch(self.coordinates3[None], doGradients=doGradients)
        self.configuration.energyTerms = {k: (float(v[0]) if k not in ("SCF Cycles", "Status") else int(v[0])) for k, v in terms.items()}
        if self.nbModel is None or not self.mm_indices():
            self.configuration.energyTerms.pop("QC/MM Elect.", None)
        self.configuration.gradients3 = None if G is None else G[0]
        return float(total[0])
