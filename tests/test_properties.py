"""Dipole moments and Mayer bond orders (pdynamo_mirror_gb300/properties.py) against the reference core's
QCModelMNDO_DipoleMoment / QCModelMNDO_MayerBondOrders (tests/golden/properties_reference.json), evaluated on the
oracle's converged densities; and the System / QCModelMNDO surface that assembles them.  No GPU."""

import json, os

import numpy as np
import pytest

from oracle import oracle as O
from pdynamo_mirror_gb300 import properties as PR
from pdynamo_mirror_gb300.parameters import ElementParameters

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "properties_reference.json")))["cases"]


def _unpack(p, n):
    P = np.zeros((n, n))
    P[np.tril_indices(n)] = p
    return P + P.T - np.diag(np.diag(P))


@pytest.mark.parametrize("case", CASES, ids=[c["name"] + "-" + c["hamiltonian"] for c in CASES])
def test_properties_match_reference(case):
    Z, X = case["Z"], np.array(case["xyz"])
    el = [ElementParameters(case["hamiltonian"], z) for z in Z]
    nb = [e.norbitals for e in el]
    N = sum(nb)
    ham = O.Hamiltonian(case["hamiltonian"], Z)
    if case["isSpinRestricted"]:
        r = O.System(ham, Z, case["charge"]).energy(X, gradients=False)
        P, S = _unpack(r["density"], N), None
    else:
        r = O.energy_open(ham, Z, X, case["charge"], 2, False, "Cardinal", gradients=False)
        Pa, Pb = _unpack(r["density_alpha"], N), _unpack(r["density_beta"], N)
        P, S = Pa + Pb, Pa - Pb
    assert r["converged"]
    d = PR.qc_dipole([e.zcore for e in el], nb, [e.ddp[1] for e in el], X, P)
    np.testing.assert_allclose(d, case["dipole_debye"], rtol=0, atol=1e-5)
    B, c, f, t = PR.mayer(nb, P, S)
    np.testing.assert_allclose(B, case["bond_orders"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(c, case["mayer_charges"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(f, case["free_valence"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(t, case["total_valence"], rtol=0, atol=1e-6)


def test_system_dipole_and_bond_order_assembly():
    """System.DipoleMoment = MM point-charge dipole + QC dipole; QCModelMNDO.BondOrders from the stored state."""
    from pdynamo_mirror_gb300 import QCModelMNDO, System
    c = CASES[0]   # water, AM1
    Z, X = c["Z"], np.array(c["xyz"])
    mmX = X + np.array([5.0, 0.0, 0.0])
    mmq = np.array([-0.834, 0.417, 0.417])
    s = System(list(Z) + list(Z), np.concatenate([X, mmX]), mmCharges=np.concatenate([np.zeros(3), mmq]))
    s.DefineQCModel(QCModelMNDO("am1"), qcSelection=[0, 1, 2])
    with pytest.raises(ValueError):
        s.DipoleMoment()
    r = O.System(O.Hamiltonian("am1", Z), Z).energy(X, gradients=False)
    s.configuration.qcState = PR.QCState(_unpack(r["density"], 6), "am1", Z, X)   # O 4 + 2 x H 1 basis functions
    qc = np.array(c["dipole_debye"])
    mm = (mmq[:, None] * mmX).sum(0) * PR.ANGSTROMS_TO_BOHRS * PR.DEBYES_PER_E_BOHR
    np.testing.assert_allclose(s.DipoleMoment(), qc + mm, rtol=0, atol=1e-5)
    B, ch, fv, tv = s.qcModel.BondOrders(s.configuration)
    np.testing.assert_allclose(B, c["bond_orders"], rtol=0, atol=1e-6)
