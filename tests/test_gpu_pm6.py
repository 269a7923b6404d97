"""PM6 for elements with s and p orbitals on the GPU (QCModelMNDO("pm6"): the diatomic core-core term in the pair
integral and gradient kernels) against the reference core's fixtures: the 42 closed-shell molecules of
tests/golden/pm6_reference.json (H, C, N, O, F; the reference's test set run with PM6) and the two open-shell radicals
of open_shell_reference.json's PM6 cases, energies 1e-6 Hartree and gradients 1e-5 Hartree/Bohr; the matrices for a
fixed density against the oracle at round-off; and the reference's own stored PM6 energies (MNDORHFEnergies.pkl,
tests/golden/pm6_pickle.json) within the 1 kJ/mol its test allows."""
import json, os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PM6 = json.load(open(os.path.join(GOLD, "pm6_reference.json")))
OPEN = json.load(open(os.path.join(GOLD, "open_shell_reference.json")))["pm6_cases"]
KJ = 2625.5
A2B = 1.0e-10 / 5.291772083e-11


def _converger():
    from pdynamo_mirror_gb300 import DIISSCFConverger
    return DIISSCFConverger(densityTolerance=1.0e-8, maximumSCFCycles=500)


@pytest.mark.parametrize("label", sorted(PM6["molecules"]))
def test_closed_shell_matches_reference_core(label):
    from pdynamo_mirror_gb300 import QCModelMNDO, System
    m = PM6["molecules"][label]
    s = System(m["Z"], m["xyz"])
    s.electronicState.charge = m["charge"]
    s.DefineQCModel(QCModelMNDO("pm6", converger=_converger()))
    e = s.Energy(doGradients=True)
    assert abs(e - m["pure_qc_kj"]) / KJ < 1e-6
    np.testing.assert_allclose(s.configuration.gradients3 / (KJ * A2B), m["gradients_hartree_per_bohr"], rtol=0, atol=1e-5)


@pytest.mark.parametrize("case", OPEN, ids=[c["label"].replace(" ", "") for c in OPEN])
def test_open_shell_matches_reference_core(case):
    from pdynamo_mirror_gb300 import QCModelMNDO, System
    s = System(case["atomic_numbers"], np.array(case["xyz"]))
    s.electronicState.charge = case["charge"]
    s.electronicState.multiplicity = case["multiplicity"]
    s.DefineQCModel(QCModelMNDO("pm6", isSpinRestricted=False, converger=_converger()))
    s.Energy(doGradients=True)
    assert abs(s.configuration.energyTerms["Pure QC"] - case["pure_qc_kj"]) / KJ < 1e-6
    np.testing.assert_allclose(s.configuration.gradients3 / (KJ * A2B), case["gradients_hartree_per_bohr"], rtol=0, atol=1e-5)


def test_fixed_density_matrices_and_gradients_match_oracle():
    """The core-core energy, the Fock matrix and the gradients for the oracle's converged density (round-off level):
    every PM6 pair type of the set (X-H, C-C, the other heavy pairs, H-H, F)."""
    import torch
    from pdynamo_mirror_gb300.engine import QCEngine
    for label in ("caffeine", "trifluorobenzene", "dihydrogen", "hydrazine", "ethanol"):
        m = PM6["molecules"][label]
        Z, X = m["Z"], np.array(m["xyz"])
        eng = QCEngine("pm6", Z, m["charge"])
        os_ = O.System(O.Hamiltonian("pm6", Z), Z, charge=m["charge"])
        r = os_.energy(X, gradients=False)
        N = eng.n_basis
        P = np.zeros((N, N))
        i, j = np.tril_indices(N)
        P[i, j] = r["density"]
        P[j, i] = r["density"]
        dev = lambda x: torch.as_tensor(np.asarray(x, dtype=np.float64), device="cuda")
        Fg, eg = eng.fock(dev(X[None]), dev(P[None]))
        Fo, eo = os_.fock(X, r["density"])
        Fo_full = np.zeros((N, N))
        Fo_full[i, j] = Fo
        Fo_full[j, i] = Fo
        np.testing.assert_allclose(Fg[0].cpu().numpy(), Fo_full, rtol=0, atol=1e-10, err_msg=label)
        eg = eg[0].cpu().numpy()
        assert abs(eg[2] - eo[2]) < 1e-10, label   # core-core
        gg = eng.gradients(dev(X[None]), dev(P[None]))[0].cpu().numpy()
        np.testing.assert_allclose(gg, os_.gradients(X, r["density"]), rtol=0, atol=1e-10, err_msg=label)


def test_matches_the_references_stored_energies():
    from pdynamo_mirror_gb300 import QCModelMNDO, System
    stored = json.load(open(os.path.join(GOLD, "pm6_pickle.json")))["pm6"]
    for label in ("water", "benzene", "glycine", "caffeine"):
        m = PM6["molecules"][label]
        s = System(m["Z"], m["xyz"])
        s.electronicState.charge = m["charge"]
        s.DefineQCModel(QCModelMNDO("pm6", converger=_converger()))
        assert abs(s.Energy() - stored[label]["value"]) <= stored[label]["tolerance"], label
