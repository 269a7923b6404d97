"""Analytic gradients against central finite differences of the energy, as the reference's own tests check them
(pMolecule-1.9.0/tests/MNDORHFEnergies.py:20, :60-70: molecules below 10 atoms, delta 1e-4 A, max |dg| <= 2e-2 kJ/mol/A;
tests/MNDOQCMMEnergies.py:15, :66: QC/MM with NBModelFull, <= 1e-3 kJ/mol/A).  All displaced geometries of a
molecule are frames of one EnergyBatch call; every frame starts from the diagonal guess."""

import json, os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
DELTA = 1.0e-4


def _fd(system, X):
    n = len(X)
    frames = np.repeat(X[None], 6 * n, axis=0)
    for a in range(n):
        for d in range(3):
            frames[6 * a + 2 * d, a, d] += DELTA
            frames[6 * a + 2 * d + 1, a, d] -= DELTA
    E, _, _ = system.EnergyBatch(frames, doGradients=False, warmStart=False)
    return ((E[0::2] - E[1::2]) / (2.0 * DELTA)).reshape(n, 3)


@pytest.mark.parametrize("hamiltonian", ["am1", "mndo", "pm3", "rm1", "pddgmndo", "pddgpm3"])
def test_gradients_match_finite_differences(hamiltonian):
    from pdynamo_mirror_gb300 import DIISSCFConverger, QCModelMNDO, System
    mols = json.load(open(os.path.join(HERE, "golden", "molecules.json")))
    ref = json.load(open(os.path.join(HERE, "golden", "mndo_rhf_reference.json")))[hamiltonian]
    # the molecules the reference core converged for this Hamiltonian (the parity tests' set), below 10 atoms
    names = [k for k in sorted(ref) if ref[k]["converged"] and len(mols[k]["Z"]) < 10][:8]
    assert names
    for name in names:
        m = mols[name]
        X = np.array(m["xyz"])
        s = System(m["Z"], X)
        s.electronicState.charge = m["charge"]
        s.DefineQCModel(QCModelMNDO(hamiltonian, converger=DIISSCFConverger(densityTolerance=1.0e-8, maximumSCFCycles=500)))
        s.Energy(doGradients=True)
        g = s.configuration.gradients3
        np.testing.assert_allclose(g, _fd(s, X), rtol=0, atol=2.0e-2, err_msg=name)


def test_qcmm_gradients_match_finite_differences():
    from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelFull, QCModelMNDO, System, workloads
    Z, X = workloads.water_cluster(2, seed=5)
    mmX = X[:3] + np.array([5.0, 1.0, 0.0])
    allZ, allX = np.concatenate([Z, [8, 1, 1]]), np.concatenate([X, mmX])
    q = np.array([0.0] * len(Z) + [workloads.TIP3P_O, workloads.TIP3P_H, workloads.TIP3P_H])
    s = System(allZ, allX, mmCharges=q)
    # converger as MNDOQCMMEnergies.py:46-47
    s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(densityTolerance=1.0e-10, maximumSCFCycles=250)),
                    qcSelection=range(len(Z)))
    s.DefineNBModel(NBModelFull())
    s.Energy(doGradients=True)
    np.testing.assert_allclose(s.configuration.gradients3, _fd(s, allX), rtol=0, atol=1.0e-3)


def test_mixed_method_gradients_match_its_finite_differences():
    """The mixed method converges to the FP64 density, so its gradients match differences of its own energies."""
    from pdynamo_mirror_gb300 import DIISSCFConverger, QCModelMNDO, System, workloads
    Z, X = workloads.water_cluster(3, seed=2)
    s = System(Z, X)
    s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(densityStep="purification")))
    s.Energy(doGradients=True)
    np.testing.assert_allclose(s.configuration.gradients3, _fd(s, X), rtol=0, atol=2.0e-2)
