"""The host side of System.Energy without a GPU: a stand-in engine returns, in the CUDA engine's shapes and units, what
the oracle computes (energies, Lowdin charges, the converged density), so that the result assembly, the energy terms,
AtomicCharges, DipoleMoment and BondOrders run as they do on the GPU path and are checked against the reference
core's fixture (tests/golden/properties_reference.json).  The stand-in is test scaffolding; the product refuses to run
without the CUDA library."""

import json, os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pdynamo_mirror_gb300 import _native

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = [c for c in json.load(open(os.path.join(HERE, "golden", "properties_reference.json")))["cases"] if c["isSpinRestricted"]]
BOHR = 1.0e-10 / 5.291772083e-11


class _OracleEngine:
    """Answers run() from the oracle for each frame (QC only)."""

    def __init__(self, hamiltonian, atomic_numbers, charge):
        self.Z, self.charge = [int(z) for z in atomic_numbers], charge
        self.ham = O.Hamiltonian(hamiltonian, self.Z)
        self.device = torch.device("cpu")
        self.density = None

    def run(self, qc_xyz, converger, mm_xyz=None, mm_charges=None, nbmodel=None, gradients=True, warm_start=True, guess=None,
            mm_gradients=True):
        assert not gradients or nbmodel is None
        F, n = qc_xyz.shape[0], qc_xyz.shape[1]
        E, Q, G, D = [], [], [], []
        for f in range(F):
            phi = None
            if nbmodel is not None:
                phi, _, _ = O.qcmm("abfs", qc_xyz[f].numpy(), mm_xyz[f].numpy(), mm_charges.numpy(),
                                   knots=O.abfs_knots(nbmodel.innerCutoff, nbmodel.outerCutoff))
            r = O.System(self.ham, self.Z, self.charge).energy(qc_xyz[f].numpy(), phi=phi, gradients=gradients)
            en = np.zeros(_native.NENERGY)
            en[_native.EN_ELECTRONIC], en[_native.EN_NUCLEAR], en[_native.EN_BASELINE] = r["eelectronic"], r["enuclear"], r["baseline"]
            en[_native.EN_QCMM] = r["eqcmm"]
            E.append(en); Q.append(r["charges"])
            if gradients:
                G.append(r["gradients"])   # Eh/Bohr, as the CUDA engine returns them
            N = int(round((np.sqrt(8 * len(r["density"]) + 1) - 1) / 2))
            P = np.zeros((N, N)); P[np.tril_indices(N)] = r["density"]
            D.append(P + P.T - np.diag(np.diag(P)))
        self.density = torch.tensor(np.array(D))
        t = lambda a: torch.tensor(np.array(a), dtype=torch.float64)
        return {"energies": t(E), "charges": t(Q), "status": torch.zeros(F, dtype=torch.int32), "ncycles": torch.full((F,), 10, dtype=torch.int32),
                "qc_gradients": t(G) if gradients else None}


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_energy_path_host_side(case, monkeypatch):
    import pdynamo_mirror_gb300.system as S
    from pdynamo_mirror_gb300 import QCModelMNDO
    monkeypatch.setattr(S, "QCEngine", _OracleEngine)
    X = np.array(case["xyz"])
    s = S.System(case["Z"], X)
    s.electronicState.charge = case["charge"]
    s.DefineQCModel(QCModelMNDO(case["hamiltonian"]))
    e = s.Energy()
    r = O.System(O.Hamiltonian(case["hamiltonian"], case["Z"]), case["Z"], case["charge"]).energy(X, gradients=False)
    assert abs(e - r["pure_qc_kj"]) < 1e-9
    assert set(s.configuration.energyTerms) == {"Pure QC", "SCF Cycles", "Status"}
    np.testing.assert_allclose(s.AtomicCharges(), r["charges"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(s.DipoleMoment(), case["dipole_debye"], rtol=0, atol=1e-5)
    B, ch, fv, tv = s.qcModel.BondOrders(s.configuration)
    np.testing.assert_allclose(B, case["bond_orders"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(tv, case["total_valence"], rtol=0, atol=1e-6)
    # a batch of frames: energies per frame and the charges of every frame
    frames = np.stack([X, X + 0.01])
    tot, G, terms = s.EnergyBatch(frames, doGradients=False)
    assert tot.shape == (2,) and s.qcChargesBatch.shape == (2, len(case["Z"])) and abs(tot[0] - e) < 1e-9


class _OracleMM:
    """Answers MMInteractions.run from oracle/mmmm.py."""

    def __init__(self, mmModel, nbModel, qcSelection, fixedAtoms, device):
        from oracle import mmmm
        self.m, self.nb, self.mmmm = mmModel, nbModel, mmmm
        self.flags = np.full(mmModel.natoms, mmmm.FLAG_MM)
        self.flags[list(qcSelection)] = mmmm.FLAG_QC_LJ
        self.has_qc, self.has14 = True, len(mmModel.interactions14) > 0

    def run(self, frames, gradients=True):
        m, lj = self.m, self.m.ljParameters
        out = [self.mmmm.energies(x.numpy(), m.charges, m.ljTypes, self.flags, lj.epsilon, lj.sigma, lj.epsilon, lj.sigma, True,
                                  m.exclusions, m.interactions14, self.nb.innerCutoff, self.nb.outerCutoff, self.nb.dampingCutoff)
               for x in frames]
        E = np.array([o[0] for o in out])
        # the MMInteractions contract: one column per _native.MM_TERMS entry (no bonded terms in this model)
        E = np.concatenate([E, np.zeros((len(out), 2))], axis=1)
        return torch.tensor(E), (torch.tensor(np.array([o[1] for o in out])) if gradients else None)

    def term_names(self):
        return ["MM/MM Elect.", "MM/MM LJ", "QC/MM LJ"]


def test_energy_path_with_mm_model_host_side(monkeypatch):
    """The MM model's terms sit after the SCF results and before the QC charges in the single device-to-host copy."""
    import pdynamo_mirror_gb300.mmmodel as M
    import pdynamo_mirror_gb300.system as S
    from pdynamo_mirror_gb300 import MMModel, NBModelABFS, QCModelMNDO, workloads
    from oracle import mmmm
    monkeypatch.setattr(S, "QCEngine", _OracleEngine)
    monkeypatch.setattr(M, "MMInteractions", _OracleMM)
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=4, n_qc_waters=2, n_mm_waters=20, box=12.0)
    s = S.System(Z, X, mmCharges=Q)
    s.electronicState.charge = charge
    s.DefineQCModel(QCModelMNDO("am1"), qcSelection=sel)
    s.DefineNBModel(NBModelABFS())
    s.DefineMMModel(MMModel.TIP3PWater(Z, X))
    e = s.Energy()
    t = s.configuration.energyTerms
    Emm = _OracleMM(s.mmModel, s.nbModel, sel, None, None).run(torch.tensor(X[None]), gradients=False)[0].numpy()[0]
    for k, name in enumerate(mmmm.TERMS):
        if name in ("MM/MM Elect.", "MM/MM LJ", "QC/MM LJ"):
            assert abs(t[name] - Emm[k]) < 1e-9
    assert abs(e - (t["Pure QC"] + t["QC/MM Elect."] + Emm.sum())) < 1e-9
    assert s.configuration.qcCharges.shape == (len(sel),) and abs(s.configuration.qcCharges.sum() - charge) < 1e-8


def test_scf_failure_message_names_each_status():
    from pdynamo_mirror_gb300 import _native
    from pdynamo_mirror_gb300.system import SCFNotConverged, scf_failure_message
    assert issubclass(SCFNotConverged, ValueError)
    m = scf_failure_message([_native.PDG_OK, _native.PDG_NAN, _native.PDG_NOT_CONVERGED, _native.PDG_TENSOR_TIMEOUT, _native.PDG_NAN])
    assert "non-finite energy in frames 1, 4" in m
    assert "not converged in frame 2" in m
    assert "tensor-core completion wait ran out in frame 3" in m
