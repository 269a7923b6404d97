"""Properties after an energy on the GPU: atomic charges (System.AtomicCharges, QCModelMNDO.AtomicCharges) against the
oracle's Lowdin charges, QC only and with MM point charges (NBModelFull), 1e-6 e; dipole moments and Mayer bond orders
against the reference core's.  The tolerances allow for two SCFs that each stop at the 1e-8 RMS density tolerance."""

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


@pytest.mark.parametrize("order", ["mm_first", "qc_first"])
def test_qcmm_charges_ignore_mm_charges_at_qc_atoms(order):
    """A TIP3P MM model puts non-zero charges on the QC atoms too.  Whichever of DefineMMModel and DefineQCModel
    comes first, the QC atoms' charges are their Lowdin charges alone (MMAtomContainer.AtomicCharges gives 0 for
    atoms that DefineQCModel deactivated) and the MM atoms keep their TIP3P charges."""
    from oracle import oracle as O
    from pdynamo_mirror_gb300 import MMModel, NBModelABFS, QCModelMNDO, System, workloads
    Z, X, allZ, allX, _ = _water_trimer_with_mm()
    nq = len(Z)
    s = System(allZ, allX)
    mm = MMModel.TIP3PWater(allZ, allX)
    assert np.abs(np.asarray(mm.charges)[:nq]).min() > 0.4
    if order == "mm_first":
        s.DefineMMModel(mm)
        s.DefineQCModel(QCModelMNDO("am1"), qcSelection=range(nq))
    else:
        s.DefineQCModel(QCModelMNDO("am1"), qcSelection=range(nq))
        s.DefineMMModel(mm)
    s.DefineNBModel(NBModelABFS())
    s.Energy(doGradients=True)
    mmq = np.asarray(mm.charges, dtype=np.float64)
    phi, _, _ = O.qcmm("abfs", X, allX[nq:], mmq[nq:], knots=O.abfs_knots(8.0, 12.0))
    r = O.System(O.Hamiltonian("am1", Z), Z).energy(X, phi=phi)
    q = s.AtomicCharges()
    np.testing.assert_allclose(q[:nq], r["charges"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(q[nq:], mmq[nq:])


def test_dipoles_and_bond_orders_match_reference():
    """System.DipoleMoment and QCModelMNDO.BondOrders after Energy against the reference core's
    QCModelMNDO_DipoleMoment / QCModelMNDO_MayerBondOrders (tests/golden/properties_reference.json, closed-shell
    cases): dipoles 1e-5 Debye, bond orders and valences 1e-6."""
    import json, os
    from pdynamo_mirror_gb300 import QCModelMNDO, System
    cases = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "properties_reference.json")))["cases"]
    n = 0
    for c in cases:
        if not c["isSpinRestricted"]:
            continue
        s = System(c["Z"], np.array(c["xyz"]))
        s.electronicState.charge = c["charge"]
        s.DefineQCModel(QCModelMNDO(c["hamiltonian"]))
        s.Energy()
        np.testing.assert_allclose(s.DipoleMoment(), c["dipole_debye"], rtol=0, atol=1e-5, err_msg=c["name"])
        B, ch, fv, tv = s.qcModel.BondOrders(s.configuration)
        np.testing.assert_allclose(B, c["bond_orders"], rtol=0, atol=1e-6, err_msg=c["name"])
        np.testing.assert_allclose(ch, c["mayer_charges"], rtol=0, atol=1e-6, err_msg=c["name"])
        np.testing.assert_allclose(tv, c["total_valence"], rtol=0, atol=1e-6, err_msg=c["name"])
        n += 1
    assert n == 5
