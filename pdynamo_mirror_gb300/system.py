"""System: the drop-in surface of pDynamo's System for the QC and QC/MM energy + gradient.

``System.DefineQCModel``, ``System.DefineNBModel`` and ``System.Energy(doGradients=True)`` follow
pMolecule/System.py:182-318: energies are returned in kJ/mol, gradients are left on
``system.configuration.gradients3`` in kJ/mol/A, and the energy terms ("Pure QC", "QC/MM Elect.") on
``system.configuration.energyTerms``.  Atoms outside the QC selection are MM point charges.

``System.EnergyBatch`` evaluates many frames (coordinate sets of the same system) in one device call; it
is the throughput form of the same computation.
"""

import math

import numpy as np
import torch

from . import _native
from .engine import GRADIENT_TO_KJ_PER_A, HARTREES_TO_KJ, QCEngine


class ElectronicState:
    def __init__(self, charge=0, multiplicity=1):
        if int(multiplicity) < 1:
            raise ValueError("Invalid multiplicity.")
        self.charge, self.multiplicity = int(charge), int(multiplicity)


class Configuration:
    def __init__(self):
        self.energyTerms = {}
        self.gradients3 = None
        self.qcState = None
        self.qcCharges = None   # Lowdin charges of the QC atoms after Energy


class SCFNotConverged(ValueError):
    """The reference raises ValueError when the SCF does not converge (pMolecule.QCModel.pyx:177); here also when a
    frame's SCF stopped on a non-finite energy or a tensor-core wait that ran out."""


def scf_failure_message(status):
    """The message for the per-frame statuses of a batch that did not all converge."""
    status = np.asarray(status)
    parts = []
    for code, what in ((_native.PDG_NOT_CONVERGED, "not converged"), (_native.PDG_NAN, "non-finite energy"),
                       (_native.PDG_TENSOR_TIMEOUT, "tensor-core completion wait ran out")):
        frames = np.nonzero(status == code)[0]
        if len(frames):
            parts.append("%s in frame%s %s" % (what, "s" if len(frames) > 1 else "", ", ".join(str(int(f)) for f in frames[:8])
                                                + (", ..." if len(frames) > 8 else "")))
    other = np.nonzero(~np.isin(status, [_native.PDG_OK, _native.PDG_NOT_CONVERGED, _native.PDG_NAN, _native.PDG_TENSOR_TIMEOUT]))[0]
    if len(other):
        parts.append("status %d in frame %d" % (int(status[other[0]]), int(other[0])))
    return "SCF procedure not converged: " + "; ".join(parts) + "."


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
        self.densityGuess = None
        self.fixedAtoms = None
        self.mmModel = None
        self._mm = None

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

    def DefineFixedAtoms(self, selection):
        """Atoms that dynamics leaves in place (System.py:142-160; None clears them)."""
        if selection is None:
            self.fixedAtoms = None
            return
        sel = sorted(set(int(i) for i in selection))
        if sel and (sel[0] < 0 or sel[-1] >= len(self.atomicNumbers)):
            raise ValueError("Invalid fixed-atom selection.")
        self.fixedAtoms = sel

    def DefineMMModel(self, mmModel):
        """The MM side of the system (mmmodel.MMModel: charges, LJ types and parameters, exclusions, 1-4 pairs):
        with an NBModelABFS, the energy then includes the MM/MM electrostatic and LJ terms and the QC/MM LJ terms
        (NBModelABFS.pyx:108-122).  The model's charges become the MM point charges.  None removes it."""
        if mmModel is not None:
            if mmModel.natoms != len(self.atomicNumbers):
                raise ValueError("The MM model must cover every atom of the system.")
            self.mmCharges = np.array(mmModel.charges, dtype=np.float64)
            if self.qcSelection is not None:
                self.mmCharges[self.qcSelection] = 0.0
        self.mmModel = mmModel
        self._mm = None
        self._sel_key = None

    def _mm_interactions(self):
        from .mmmodel import MMInteractions
        from .nbmodel import NBModelABFS
        if not isinstance(self.nbModel, NBModelABFS):
            raise ValueError("MM/MM energies need an NBModelABFS.")
        key = (id(self.mmModel), id(self.nbModel), tuple(self.qcSelection or []), tuple(self.fixedAtoms or []))
        if self._mm is None or self._mm[0] != key:
            self._mm = (key, MMInteractions(self.mmModel, self.nbModel, self.qcSelection, self.fixedAtoms, self.engine().device))
        return self._mm[1]

    def DefineDensityGuess(self, guess):
        """Start cold SCFs from a LearnedDensityGuess (None: the diagonal guess).  Not in the reference."""
        self.densityGuess = guess

    def mm_indices(self):
        qc = set(self.qcSelection or [])
        return [i for i in range(len(self.atomicNumbers)) if i not in qc]

    def spin_occupancies(self):
        """(alpha, beta) electron counts of an open-shell or fractional-occupancy model, None for the closed-shell
        cardinal (RHF) path: QCModel.CrossCheckModelAndState (pMolecule.QCModel.pyx:91-140).  Cardinal counts are
        whole numbers (ints); fractional ones are the floats (n +- (multiplicity - 1)) / 2."""
        mult = int(self.electronicState.multiplicity)
        m = self.qcModel
        fractional = m.occupancyType != "Cardinal"
        if m.isSpinRestricted and mult != 1:
            raise ValueError("A spin-unrestricted calculation is required for non-singlet states with %s occupancy."
                             % ("fractional" if fractional else "cardinal"))
        if m.isSpinRestricted and not fractional:
            return None
        eng = self.engine()
        ne = eng.n_electrons
        if not fractional:
            if (ne + mult - 1) % 2 or mult - 1 > ne:
                raise ValueError("The multiplicity is incompatible with the number of electrons.")
            return (ne + mult - 1) // 2, (ne - mult + 1) // 2
        N = eng.n_basis
        a, b = (ne + (mult - 1.0)) / 2.0, (ne - (mult - 1.0)) / 2.0
        na, nb = int(math.ceil(a)), int(math.ceil(b))
        if a < 0.0 or b < 0.0 or na > N or nb > N:
            raise ValueError("Invalid alpha or beta electronic charge (< 0 or > number of available orbitals).")
        if m.occupancyType == "Fixed Fractional":
            f = m.numberFractional
            sets = [("", na)] if m.isSpinRestricted else [("Alpha", na), ("Beta", nb)]
            for tag, nocc in sets:
                hoo, luo = f["numberFractional%sHOOs" % tag], f["numberFractional%sLUOs" % tag]
                if not (1 <= hoo <= nocc and 0 <= luo <= N - nocc):
                    raise ValueError("Invalid fixed fractional occupancy orbital specification.")
        return a, b

    def occupancy(self):
        """The pdg_occupancy of an open-shell or fractional-occupancy model (None for the RHF path)."""
        spins = self.spin_occupancies()
        if spins is None:
            return None
        m = self.qcModel
        f = m.numberFractional
        occ = _native.Occupancy(spin_restricted=1 if m.isSpinRestricted else 0, occupancy_type=_native.OCC_TYPES[m.occupancyType],
                                alpha_charge=float(spins[0]), beta_charge=float(spins[1]), fermi_broadening=float(m.fermiBroadening))
        for k, name in enumerate(("", "Alpha", "Beta")):
            occ.n_fractional[2 * k] = f["numberFractional%sHOOs" % name]
            occ.n_fractional[2 * k + 1] = f["numberFractional%sLUOs" % name]
        return occ

    def engine(self):
        """The device engine of the QC region, rebuilt when the electronic state's charge changes."""
        charge = int(self.electronicState.charge)
        if self._engine is None or getattr(self, "_engine_charge", None) != charge:
            qcZ = [self.atomicNumbers[i] for i in self.qcSelection]
            self._engine = QCEngine(self.qcModel.mndoModel, qcZ, charge)
            self._engine_charge = charge
            self._sel_key = None
            self._mm = None
        return self._engine

    def _selections(self):
        """Device index data of the QC and MM atoms, cached per model definition: a slice when the atoms are
        one contiguous range (no gather), else an index tensor."""
        key = (id(self._engine), tuple(self.qcSelection), self.nbModel is not None)
        if getattr(self, "_sel_key", None) != key:
            dev = self.engine().device

            def sel(idx):
                if not idx:
                    return None
                if idx == list(range(idx[0], idx[-1] + 1)):
                    return slice(idx[0], idx[-1] + 1)
                return torch.as_tensor(idx, dtype=torch.long, device=dev)

            mm_idx = self.mm_indices() if self.nbModel is not None else []
            q = torch.as_tensor(self.mmCharges[mm_idx], dtype=torch.float64, device=dev).contiguous() if mm_idx else None
            self._sel = (sel(self.qcSelection), sel(mm_idx), q, mm_idx)
            self._sel_key = key
        return self._sel

    @staticmethod
    def _take(X, s):
        return X[:, s].contiguous() if isinstance(s, slice) else X.index_select(1, s)

    def _device_frames(self, frames):
        """frames: [F, n, 3] host (numpy or torch, ideally pinned) or device tensor -> one copy on the device."""
        dev = self.engine().device
        X = frames if isinstance(frames, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(frames, dtype=np.float64))
        return X.to(device=dev, dtype=torch.float64, non_blocking=True)

    def _device_inputs(self, frames, X=None):
        """QC and MM coordinates of the frames, split on the device (X: the frames already on the device)."""
        if X is None:
            X = self._device_frames(frames)
        qs, ms, q, mm_idx = self._selections()
        qc = self._take(X, qs)
        mm = self._take(X, ms) if ms is not None else None
        return qc, mm, q, mm_idx

    def EnergyBatch(self, frames, doGradients=True, warmStart=True):
        """frames [F, n_atoms, 3] (Angstrom; numpy array or torch tensor, host or device).  Returns (energies
        kJ/mol [F], gradients kJ/mol/A [F, n, 3] or None, terms dict of [F] arrays).  Raises SCFNotConverged
        if any frame fails to converge."""
        if self.qcModel is None:
            raise ValueError("No QC model defined.")
        if not isinstance(frames, torch.Tensor):
            frames = np.asarray(frames, dtype=np.float64)
        if frames.ndim == 2:
            frames = frames[None]
        eng = self.engine()
        X = self._device_frames(frames)
        qc, mm, q, mm_idx = self._device_inputs(None, X)
        mmi = self._mm_interactions() if self.mmModel is not None else None
        occ = self.occupancy()
        if occ is None:
            r = eng.run(qc, self.qcModel.converger, mm, q, self.nbModel if mm is not None else None, gradients=doGradients,
                        warm_start=warmStart, guess=self.densityGuess)
        else:
            r = eng.run_open(qc, self.qcModel.converger, occ, mm, q, self.nbModel if mm is not None else None,
                             gradients=doGradients, warm_start=warmStart)
        F = qc.shape[0]
        on_gpu = torch.device(eng.device).type == "cuda"
        # one device -> host copy of the small per-frame results
        small = torch.cat([r["energies"], r["status"].to(torch.float64)[:, None], r["ncycles"].to(torch.float64)[:, None]], 1)
        if mmi is not None:
            Emm, Gmm = mmi.run(X, gradients=doGradients)
            small = torch.cat([small, Emm], 1)
        nq = r["charges"].shape[1]
        small = torch.cat([small, r["charges"]], 1)   # Lowdin charges of the QC atoms (QCModelMNDO_LowdinCharges)
        if "spin_populations" in r:                   # and, for open-shell states, their Lowdin spin populations
            small = torch.cat([small, r["spin_populations"]], 1)
        G = None
        if doGradients:
            qs, ms, _, _ = self._selections()
            Gd = torch.zeros((F, len(self.atomicNumbers), 3), dtype=torch.float64, device=eng.device)
            gq = r["qc_gradients"]
            if "qcmm_qc_gradients" in r:
                gq = gq + r["qcmm_qc_gradients"]
                Gd[:, ms] = r["qcmm_mm_gradients"]
            Gd[:, qs] = gq
            Gd *= GRADIENT_TO_KJ_PER_A
            if mmi is not None:
                Gd += Gmm
            Gh = torch.empty(Gd.shape, dtype=torch.float64, pin_memory=on_gpu)
            Gh.copy_(Gd, non_blocking=on_gpu)
        # both results come back on the stream with one host wait
        small_h = torch.empty(small.shape, dtype=torch.float64, pin_memory=on_gpu)
        small_h.copy_(small, non_blocking=on_gpu)
        if on_gpu:
            torch.cuda.current_stream(eng.device).synchronize()
        small = small_h.numpy()
        if doGradients:
            G = Gh.numpy()
        E = small[:, :_native.NENERGY]
        st = small[:, _native.NENERGY].astype(np.int32)
        if "spin_populations" in r:
            self.qcSpinBatch = small[:, small.shape[1] - nq:].copy()
            self.qcChargesBatch = small[:, small.shape[1] - 2 * nq:small.shape[1] - nq].copy()
        else:
            self.qcSpinBatch = None
            self.qcChargesBatch = small[:, small.shape[1] - nq:].copy()
        pure = HARTREES_TO_KJ * (E[:, _native.EN_ELECTRONIC] + E[:, _native.EN_NUCLEAR] + E[:, _native.EN_BASELINE])
        qcmm = HARTREES_TO_KJ * E[:, _native.EN_QCMM]
        terms = {"Pure QC": pure, "QC/MM Elect.": qcmm, "SCF Cycles": small[:, _native.NENERGY + 1].astype(np.int32), "Status": st}
        if (st != _native.PDG_OK).any():
            self._engine.density = None
            self._engine.density_open = None
            raise SCFNotConverged(scf_failure_message(st))
        # the QC density of each frame (the total density of an open-shell state) for the properties
        self._qc_density = r["density"] if occ is not None else self._engine.density
        total = pure + (qcmm if mm is not None else 0.0)
        if mmi is not None:
            Emm = small[:, _native.NENERGY + 2:_native.NENERGY + 2 + len(_native.MM_TERMS)]
            for k, name in enumerate(_native.MM_TERMS):
                if name in mmi.term_names():
                    terms[name] = Emm[:, k]
            total = total + Emm.sum(1)
        return total, G, terms

    def Energy(self, doGradients=False, log=None):
        """Energy (kJ/mol) of the current coordinates; gradients3 in kJ/mol/A when doGradients."""
        total, G, terms = self.EnergyBatch(self.coordinates3[None], doGradients=doGradients)
        self.configuration.energyTerms = {k: (float(v[0]) if k not in ("SCF Cycles", "Status") else int(v[0])) for k, v in terms.items()}
        if self.nbModel is None or not self.mm_indices():
            self.configuration.energyTerms.pop("QC/MM Elect.", None)
        self.configuration.gradients3 = None if G is None else G[0]
        self.configuration.qcCharges = self.qcChargesBatch[0].copy()
        self.configuration.qcSpinDensities = None if self.qcSpinBatch is None else self.qcSpinBatch[0].copy()
        from .properties import QCState
        self.configuration.qcState = QCState(self._qc_density[0].clone(), self.qcModel.mndoModel,
                                             [self.atomicNumbers[i] for i in self.qcSelection], self.coordinates3[self.qcSelection])
        return float(total[0])

    def DipoleMoment(self, center=None):
        """Dipole moment (Debye) after Energy (System.py:260-268): the MM point charges' part plus the QC model's."""
        from .properties import mm_dipole
        dipole = np.zeros(3)
        mm = self.mm_indices() if self.qcModel is not None else list(range(len(self.atomicNumbers)))
        if self.mmCharges is not None and mm:
            dipole = dipole + mm_dipole(self.mmCharges[mm], self.coordinates3[mm], center)
        if self.qcModel is not None:
            qc = self.qcModel.DipoleMoment(self.configuration, center)
            if qc is None:
                raise ValueError("No QC density: calculate an energy first.")
            dipole = dipole + qc
        return dipole

    def AtomicCharges(self, qcChargeModel=None, qcAtomsOnly=False, spinDensities=False):
        """Partial charges of the atoms after Energy (System.py:96-113): the MM point charges with the QC model's
        Lowdin charges added at the QC atoms, or the QC atoms' charges alone (qcAtomsOnly, or no MM charges).
        spinDensities: the QC atoms' Lowdin spin populations (zero for closed shells and spin-restricted states),
        zero at the MM atoms.  Mulliken charges equal Lowdin ones in the NDDO basis, which is orthonormal."""
        if qcChargeModel not in (None, "Lowdin", "Mulliken"):
            raise ValueError("Unknown QC charge model: " + str(qcChargeModel) + ".")
        if self.qcModel is None:
            return None
        q = getattr(self.configuration, "qcCharges", None)
        if q is None:
            raise ValueError("No QC density: calculate an energy first.")
        if spinDensities:
            sp = getattr(self.configuration, "qcSpinDensities", None)
            q = np.zeros_like(q) if sp is None else np.array(sp, dtype=np.float64)
        else:
            q = np.array(q, dtype=np.float64)
        if qcAtomsOnly or self.mmCharges is None:
            return q
        # The QC atoms carry their QC charge only, as MMAtomContainer.AtomicCharges gives 0 for the atoms that
        # DefineQCModel deactivated: whatever the order of DefineMMModel and DefineQCModel, and whatever the
        # constructor's mmCharges held at those atoms.
        charges = np.zeros(len(self.atomicNumbers)) if spinDensities else np.array(self.mmCharges, dtype=np.float64)
        charges[self.qcSelection] = q
        return charges
