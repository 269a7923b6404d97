"""MM/MM electrostatic and LJ energies and QC/MM LJ energies of NBModelABFS on the GPU (pdg_mm_energy_gradients)
against the reference core's fixture and the oracle.

Tolerances: energies 1e-8 kJ/mol absolute (FP64; each pair's energy is summed from both atoms here and once in the
reference, so the sums differ in order), gradients 1e-9 kJ/mol/A."""

import json, os
from types import SimpleNamespace

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import mmmm  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "mmmm_reference.json")))


def _model(c):
    from pdynamo_mirror_gb300.mmmodel import LJParameterContainer, MMModel
    rule = "OPLS" if c["opls"] else "AMBER"
    return MMModel(c["charges"], c["lj_types"], LJParameterContainer(c["epsilon"], c["sigma"], rule),
                   LJParameterContainer(c["epsilon14"], c["sigma14"], rule), c["exclusions"], c["pairs14"])


def _interactions(c):
    from pdynamo_mirror_gb300.mmmodel import MMInteractions
    fl = np.array(c["flags"])
    nb = SimpleNamespace(innerCutoff=c["inner"], outerCutoff=c["outer"], dampingCutoff=c["damping"], dielectric=c["dielectric"],
                         electrostaticScale14=c["scale14"])
    qc = [int(i) for i in np.nonzero(fl & mmmm.FLAG_QC_LJ)[0]]
    fixed = [int(i) for i in np.nonzero(fl & mmmm.FLAG_FIXED)[0]]
    return MMInteractions(_model(c), nb, qc, fixed, torch.device("cuda:0"))


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=[c["name"] for c in GOLDEN["cases"]])
def test_reference_fixture(case):
    from pdynamo_mirror_gb300 import _native
    m = _interactions(case)
    X = torch.tensor(np.array(case["xyz"])[None], dtype=torch.float64, device="cuda:0")
    E, G = m.run(X)
    assert E.shape[1] == len(_native.MM_TERMS) and not E[:, 6:].any().item()   # no harmonic terms in these models
    np.testing.assert_allclose(E.cpu().numpy()[0, :6], case["energies_kj"], rtol=0, atol=1e-8)
    np.testing.assert_allclose(G.cpu().numpy()[0], case["gradients_kj_per_a"], rtol=0, atol=1e-9)


def test_frames_against_oracle():
    c = GOLDEN["cases"][1]
    m = _interactions(c)
    rng = np.random.default_rng(8)
    X0 = np.array(c["xyz"])
    frames = X0[None] + rng.normal(scale=0.1, size=(5,) + X0.shape)
    frames[3] += np.array([40.0, -13.0, 7.5])   # a translated frame: another grid origin
    E, G = m.run(torch.tensor(frames, device="cuda:0"))
    E, G = E.cpu().numpy(), G.cpu().numpy()
    for f in range(len(frames)):
        Eo, Go = mmmm.energies(frames[f], c["charges"], c["lj_types"], c["flags"], c["epsilon"], c["sigma"], c["epsilon14"],
                               c["sigma14"], c["opls"], c["exclusions"], c["pairs14"], c["inner"], c["outer"], c["damping"],
                               c["dielectric"], c["scale14"])
        np.testing.assert_allclose(E[f, :6], Eo, rtol=0, atol=1e-8)
        np.testing.assert_allclose(G[f], Go, rtol=0, atol=1e-9)


def test_larger_box_against_oracle():
    """A 30 A box of 800 waters (several cells per dimension), fixed atoms and QC LJ partners."""
    from pdynamo_mirror_gb300 import workloads
    from pdynamo_mirror_gb300.mmmodel import MMInteractions, MMModel
    Z, X, Q, sel, _ = workloads.qcmm_water_box(seed=3, n_qc_waters=6, n_mm_waters=800, box=30.0)
    model = MMModel.TIP3PWater(Z, X)
    fixed = list(range(len(sel) + 600, len(Z)))
    nb = SimpleNamespace(innerCutoff=8.0, outerCutoff=12.0, dampingCutoff=0.5, dielectric=1.0, electrostaticScale14=1.0)
    m = MMInteractions(model, nb, sel, fixed, torch.device("cuda:0"))
    E, G = m.run(torch.tensor(X[None], device="cuda:0"))
    flags = np.full(len(Z), mmmm.FLAG_MM)
    flags[sel] = mmmm.FLAG_QC_LJ
    flags[fixed] |= mmmm.FLAG_FIXED
    lj = model.ljParameters
    Eo, Go = mmmm.energies(X, model.charges, model.ljTypes, flags, lj.epsilon, lj.sigma, lj.epsilon, lj.sigma, True,
                           model.exclusions, model.interactions14)
    np.testing.assert_allclose(E.cpu().numpy()[0, :6], Eo, rtol=0, atol=1e-8)
    np.testing.assert_allclose(G.cpu().numpy()[0], Go, rtol=0, atol=1e-9)


def test_system_energy_includes_mm_terms():
    from pdynamo_mirror_gb300 import DIISSCFConverger, MMModel, NBModelABFS, QCModelMNDO, System, workloads
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=2, n_qc_waters=4, n_mm_waters=300, box=22.0)

    def make(with_mm):
        s = System(Z, X, mmCharges=Q)
        s.electronicState.charge = charge
        s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger()), qcSelection=sel)
        s.DefineNBModel(NBModelABFS())
        if with_mm:
            s.DefineMMModel(MMModel.TIP3PWater(Z, X))
        return s

    a, b = make(False), make(True)
    ea, eb = a.Energy(doGradients=True), b.Energy(doGradients=True)
    m = b.mmModel
    flags = np.full(len(Z), mmmm.FLAG_MM)
    flags[sel] = mmmm.FLAG_QC_LJ
    lj = m.ljParameters
    Eo, Go = mmmm.energies(X, m.charges, m.ljTypes, flags, lj.epsilon, lj.sigma, lj.epsilon, lj.sigma, True, m.exclusions, [])
    t = b.configuration.energyTerms
    for k, name in enumerate(mmmm.TERMS):
        if name in ("MM/MM 1-4 Elect.", "MM/MM 1-4 LJ", "QC/MM 1-4 LJ"):
            assert name not in t
        else:
            assert abs(t[name] - Eo[k]) < 1e-8
    assert abs(eb - (ea + Eo.sum())) < 1e-7
    np.testing.assert_allclose(b.configuration.gradients3, a.configuration.gradients3 + Go, rtol=0, atol=1e-7)


def test_bench_box_properties():
    """The 12065-atom QC/MM water box at full size (no oracle): pair forces sum to zero, and translating a frame
    changes nothing."""
    from pdynamo_mirror_gb300 import workloads
    from pdynamo_mirror_gb300.mmmodel import MMInteractions, MMModel
    Z, X, Q, sel, _ = workloads.qcmm_water_box(seed=1)
    model = MMModel.TIP3PWater(Z, X)
    nb = SimpleNamespace(innerCutoff=8.0, outerCutoff=12.0, dampingCutoff=0.5, dielectric=1.0, electrostaticScale14=1.0)
    m = MMInteractions(model, nb, sel, None, torch.device("cuda:0"))
    frames = workloads.perturbed_frames(X, 3, sigma=0.02, seed=5)
    frames = np.concatenate([frames, frames[:1] + np.array([-17.0, 3.25, 101.0])])
    E, G = m.run(torch.tensor(frames, device="cuda:0"))
    E, G = E.cpu().numpy(), G.cpu().numpy()
    assert np.isfinite(E).all() and np.isfinite(G).all()
    assert np.abs(G.sum(1)).max() < 1e-8 * np.abs(G).max() * len(Z)
    np.testing.assert_allclose(E[3], E[0], rtol=1e-11, atol=1e-7)
    np.testing.assert_allclose(G[3], G[0], rtol=0, atol=1e-8)


def test_water_dimer_binding_energies():
    """Water dimer binding energies, the check of the reference's QCMMWaterDimerBinding.py (:11-12: within [-35, 5]
    kJ/mol), for the models on this path: QC/QC (AM1) and QC/MM (AM1 water with a TIP3P water: NBModelABFS
    electrostatics and the MM model's QC/MM LJ; the lone MM water has no MM/MM term).  Also against the oracle."""
    from oracle import oracle as O
    from pdynamo_mirror_gb300 import MMModel, NBModelABFS, QCModelMNDO, System
    m = json.load(open(os.path.join(HERE, "golden", "molecules.json")))["waterDimer_Cs"]
    Z, X = m["Z"], np.array(m["xyz"])

    def qc(Zs, Xs):
        s = System(Zs, Xs)
        s.DefineQCModel(QCModelMNDO("am1"))
        return s.Energy()

    e1, e2, e12 = qc(Z[:3], X[:3]), qc(Z[3:], X[3:]), qc(Z, X)
    qcqc = e12 - e1 - e2
    s = System(Z, X)
    s.DefineMMModel(MMModel.TIP3PWater(Z, X))
    s.DefineQCModel(QCModelMNDO("am1"), qcSelection=[0, 1, 2])
    s.DefineNBModel(NBModelABFS())
    qcmm = s.Energy() - e1
    assert -35.0 <= qcqc <= 5.0 and -35.0 <= qcmm <= 5.0
    # the oracle: QC energies, ABFS QC/MM potentials and the QC/MM LJ term
    ham, kj = O.Hamiltonian("am1", [1, 8]), 2625.5

    def eo(Zs, Xs, phi=None):
        r = O.System(ham, Zs, 0).energy(Xs, phi=phi, gradients=False)
        return kj * (r["eelectronic"] + r["enuclear"] + r["baseline"] + r["eqcmm"])

    q = s.mmModel.charges[3:]
    phi, _, _ = O.qcmm("abfs", X[:3], X[3:], q, knots=O.abfs_knots(8.0, 12.0))
    lj = s.mmModel.ljParameters
    flags = np.array([mmmm.FLAG_QC_LJ] * 3 + [mmmm.FLAG_MM] * 3)
    E, _ = mmmm.energies(X, s.mmModel.charges, s.mmModel.ljTypes, flags, lj.epsilon, lj.sigma, lj.epsilon, lj.sigma, True,
                         s.mmModel.exclusions, [])
    o1 = eo(Z[:3], X[:3])
    assert abs(qcqc - (eo(Z, X) - o1 - eo(Z[3:], X[3:]))) < 1e-3
    assert abs(qcmm - (eo(Z[:3], X[:3], phi) + E.sum() - o1)) < 1e-3
