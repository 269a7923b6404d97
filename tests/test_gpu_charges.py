"""Atomic charges after an energy (System.AtomicCharges, QCModelMNDO.AtomicCharges): the Lowdin charges of the
converged density on the GPU against the oracle's, QC only and with MM point charges (NBModelFull).  Tolerance
1e-6 e (two SCFs each stopping at the 1e-8 RMS density tolerance)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _water_trimer_with_mm():
    from pdynamo_mirror_gb300 import workloads
    Z, X = workloads.water_cluster(3, seed=3)
    mmZ, mmX = np.array([8, 1, 1]), X[:3] + np.array([6.0, 0.0, 0.0])
    q = np.array([0.0] * len(Z) + [workloads.TIP3P_O, workloads.TIP3P_H, workloads.TIP3P_H])
    return Z, X, np.concatenate([Z, mmZ]), np.concatenate([X, mmX]), q


def test_qc_only_charges_match_oracle():
    from oracle import oracle as O
    from pdynamo_mirror_gb300 import QCModelMNDO, System
    Z, X, _, _, _ = _water_trimer_with_mm()
    s = System(Z, X)
    s.DefineQCModel(QCModelMNDO("am1"))
    s.Energy()
    r = O.System(O.Hamiltonian("am1", Z), Z).energy(X)
    q = s.AtomicCharges()
    assert q.shape == (len(Z),) and abs(q.sum()) < 1e-8
    np.testing.assert_allclose(q, r["charges"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(s.qcModel.AtomicCharges(s.configuration), q)


def test_qcmm_charges_match_oracle():
    from oracle import oracle as O
    from pdynamo_mirror_gb300 import NBModelFull, QCModelMNDO, System
    Z, X, allZ, allX, mmq = _water_trimer_with_mm()
    s = System(allZ, allX, mmCharges=mmq)
    s.DefineQCModel(QCModelMNDO("am1"), qcSelection=range(len(Z)))
    s.DefineNBModel(NBModelFull())
    s.Energy(doGradients=True)
    phi, _, _ = O.qcmm("full", X, allX[len(Z):], mmq[len(Z):])
    r = O.System(O.Hamiltonian("am1", Z), Z).energy(X, phi=phi)
    q = s.AtomicCharges()
    np.testing.assert_allclose(q[:len(Z)], r["charges"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(q[len(Z):], mmq[len(Z):])
    np.testing.assert_allclose(s.AtomicCharges(qcAtomsOnly=True), q[:len(Z)])
