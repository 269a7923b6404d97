"""Host-side logic without a GPU: parameter processing, ABFS spline tabulation, the C ABI's exports."""
import os, re

import numpy as np
import pytest

from oracle import oracle as O
from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelABFS, QCModelMNDO, nbmodel, parameters

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("h", parameters.HAMILTONIANS)
def test_parameters_match_oracle(h):
    for z in parameters.available_elements(h):
        try:
            p = parameters.ElementParameters(h, z)
        except ValueError:
            continue   # no STO-6G basis for this element in the reference either
        d = O.Hamiltonian(h, [z]).derived(z)
        np.testing.assert_allclose(p.po, d["po"], rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(p.ddp, d["ddp"], rtol=1e-13, atol=1e-15)
        for k in ("am", "ad", "aq", "alp", "zcore", "eheat", "eisol", "gss", "gsp", "gpp", "gp2", "hsp", "hpp"):
            assert abs(getattr(p, k) - d[k]) <= 1e-13 * max(1.0, abs(d[k])), (h, z, k)
        np.testing.assert_allclose(p.beta + [0.0] * (4 - len(p.beta)), d["beta"], rtol=1e-13)
        np.testing.assert_allclose(p.uspd + [0.0] * (4 - len(p.uspd)), d["uspd"], rtol=1e-13)


def test_parameters_match_reference_core():
    R = pytest.importorskip("oracle.refdriver")
    try:
        R.lib()
    except R.RefUnavailable:
        pytest.skip("reference core not built here")
    for h in parameters.HAMILTONIANS:
        for z in (1, 6, 7, 8):
            if z not in parameters.available_elements(h):
                continue
            p = parameters.ElementParameters(h, z)
            d = R.RefHamiltonian(h, [z]).derived(z)
            np.testing.assert_allclose(p.po, d["po"], rtol=1e-14)
            ex, cc = R.RefHamiltonian(h, [z]).basis(z)
            for s, (l, e, c) in enumerate(p.shells):
                np.testing.assert_allclose(e, ex[s, :len(e)], rtol=1e-15)
                np.testing.assert_allclose(c, cc[s, :len(c)], rtol=1e-12)


def test_pm6_records_carry_the_diatomic_pairs_by_partner_index():
    """PM6 element records (pMolecule.MNDOParameters.pyx:259-276): each record knows its place in the system's element
    list and holds the diatomic pairs' coefficient x and exponent a (bohr^-1) by partner index; the other
    Hamiltonians have none."""
    els, rec, idx = parameters.element_table("pm6", [8, 1, 1, 6, 9])
    assert els == [1, 6, 8, 9] and list(idx) == [2, 0, 0, 1, 3]
    P = parameters
    for k, z in enumerate(els):
        r = rec[k]
        assert r[P.E_INDEX] == k and r[P.E_DIAT] == 1.0
        d = parameters.table()["hamiltonians"]["pm6"][str(z)]["diatomic"]
        pairs = {int(p[0]): (p[1], p[2] * P.BOHRS_TO_ANGSTROMS) for p in d}
        for j, zj in enumerate(els):
            assert (r[P.E_DIAT_X + j], r[P.E_DIAT_A + j]) == pytest.approx(pairs[zj], rel=1e-15)
        assert not r[P.E_DIAT_X + len(els):P.E_DIAT_X + P.MAX_ELEMENTS].any()
    _, rec, _ = parameters.element_table("am1", [8, 1, 1])
    assert not rec[:, P.E_DIAT].any() and not rec[:, P.E_DIAT_X:P.E_DIAT_X + P.MAX_ELEMENTS].any()


def test_abfs_knots_match_oracle():
    x, y = nbmodel.abfs_knots(8.0, 12.0)
    ox, oy = O.abfs_knots(8.0, 12.0)
    assert len(x) == len(ox) == 601
    np.testing.assert_array_equal(x, ox)
    np.testing.assert_allclose(y, oy, rtol=0, atol=1e-15)
    assert y[-1] == 0.0 and abs(y[0] - y[1]) < 1e-3


def test_option_errors_match_reference_behaviour():
    with pytest.raises(ValueError):
        DIISSCFConverger(notAnOption=1)
    with pytest.raises(ValueError):
        QCModelMNDO("am1", occupancyType="Partial")
    m = QCModelMNDO("am1", occupancyType="Variable Fractional", fermiBroadening=500.0, numberFractionalBetaLUOs=2)
    assert m.GetOption("occupancyType") == "Variable Fractional" and m.GetOption("fermiBroadening") == 500.0
    assert m.GetOption("numberFractionalBetaLUOs") == 2 and m.GetOption("numberFractionalHOOs") == 1
    assert not QCModelMNDO("am1", isSpinRestricted=False).IsSpinRestricted()
    with pytest.raises(ValueError):
        QCModelMNDO("pm7")
    with pytest.raises(ValueError):
        NBModelABFS(innerCutoff=12.0, outerCutoff=8.0)


def test_library_exports_every_declared_symbol():
    from pdynamo_mirror_gb300 import _native
    header = open(os.path.join(ROOT, "include", "pdg.h")).read()
    declared = set(re.findall(r"\b(pdg_[a-z_0-9]+)\s*\(", header))
    assert declared == set(_native.EXPORTS)
    lib = _native.load()
    for name in declared:
        assert hasattr(lib, name), name
    assert lib.pdg_version() == 100


def test_system_engine_follows_the_electronic_state(monkeypatch):
    """The device engine is rebuilt when the charge changes; non-singlet states need a spin-unrestricted model, whose
    alpha and beta electron counts follow from the multiplicity (QCModel.CrossCheckModelAndState; host logic, the
    engine itself is replaced by a stand-in, as it needs a GPU)."""
    import pdynamo_mirror_gb300.system as S
    made = []

    class Stand:
        def __init__(self, hamiltonian, atomic_numbers, charge):
            made.append(charge)
            self.device = "cpu"
            self.n_electrons = 8 - charge
            self.n_basis = 6

    monkeypatch.setattr(S, "QCEngine", Stand)
    s = S.System([8, 1, 1], [[0.0, 0.0, 0.0], [0.96, 0.0, 0.0], [-0.24, 0.93, 0.0]])
    s.DefineQCModel(QCModelMNDO("am1"))
    e1 = s.engine()
    assert s.engine() is e1
    s.electronicState.charge = 2
    e2 = s.engine()
    assert e2 is not e1 and made == [0, 2]
    s.electronicState.multiplicity = 3
    with pytest.raises(ValueError, match="spin-unrestricted"):
        s.spin_occupancies()
    s.DefineQCModel(QCModelMNDO("am1", isSpinRestricted=False))
    assert s.spin_occupancies() == (4, 2)
    s.electronicState.multiplicity = 2
    with pytest.raises(ValueError, match="incompatible"):
        s.spin_occupancies()
    s.electronicState.multiplicity = 1
    assert s.spin_occupancies() == (3, 3)
    # fractional occupancies (QCModel.CrossCheckModelAndState): restricted needs a singlet; counts as floats; the
    # fixed fractional orbitals within 1..occupied and 0..virtual
    s.DefineQCModel(QCModelMNDO("am1", occupancyType="Fixed Fractional", numberFractionalLUOs=1))
    assert s.spin_occupancies() == (3.0, 3.0) and s.occupancy() is not None
    o = s.occupancy()
    assert o.spin_restricted == 1 and o.occupancy_type == 1 and list(o.n_fractional) == [1, 1, 1, 0, 1, 0]
    s.electronicState.multiplicity = 3
    with pytest.raises(ValueError, match="fractional occupancy"):
        s.spin_occupancies()
    s.DefineQCModel(QCModelMNDO("am1", isSpinRestricted=False, occupancyType="Fixed Fractional", numberFractionalBetaHOOs=3))
    with pytest.raises(ValueError, match="fixed fractional"):
        s.spin_occupancies()
    s.DefineQCModel(QCModelMNDO("am1", isSpinRestricted=False, occupancyType="Variable Fractional"))
    assert s.spin_occupancies() == (4.0, 2.0)
    s.electronicState.multiplicity = 1
    s.DefineQCModel(QCModelMNDO("am1"))
    assert s.occupancy() is None


def test_atomic_charges_assembly():
    """System.AtomicCharges / QCModelMNDO.AtomicCharges from the charges an energy leaves on the configuration
    (System.py:96-113): MM point charges plus the QC atoms' Lowdin charges; QC atoms only; spin densities zero."""
    import numpy as np
    from pdynamo_mirror_gb300 import System
    Z = [8, 1, 1, 8, 1, 1]
    X = np.zeros((6, 3)); X[:, 0] = np.arange(6)
    s = System(Z, X, mmCharges=[0.0, 0.0, 0.0, -0.834, 0.417, 0.417])
    s.DefineQCModel(QCModelMNDO("am1"), qcSelection=[0, 1, 2])
    with pytest.raises(ValueError):
        s.AtomicCharges()
    q = np.array([-0.4, 0.2, 0.2])
    s.configuration.qcCharges = q
    np.testing.assert_allclose(s.AtomicCharges(), [-0.4, 0.2, 0.2, -0.834, 0.417, 0.417])
    np.testing.assert_allclose(s.AtomicCharges(qcAtomsOnly=True), q)
    np.testing.assert_allclose(s.AtomicCharges(spinDensities=True), np.zeros(6))
    s.configuration.qcSpinDensities = np.array([0.1, 0.45, 0.45])   # an open-shell state's Lowdin spin populations
    np.testing.assert_allclose(s.AtomicCharges(spinDensities=True), [0.1, 0.45, 0.45, 0.0, 0.0, 0.0])
    np.testing.assert_allclose(s.AtomicCharges(qcAtomsOnly=True, spinDensities=True), [0.1, 0.45, 0.45])
    np.testing.assert_allclose(s.qcModel.AtomicCharges(s.configuration, spinDensities=True), [0.1, 0.45, 0.45])
    s.configuration.qcSpinDensities = None
    np.testing.assert_allclose(s.qcModel.AtomicCharges(s.configuration, chargeModel="Mulliken"), q)
    assert s.qcModel.IsSpinRestricted() and s.qcModel.GetOption("occupancyType") == "Cardinal"
    with pytest.raises(AttributeError):
        s.qcModel.GetOption("notAnOption")
    with pytest.raises(ValueError):
        s.AtomicCharges(qcChargeModel="CM5")
