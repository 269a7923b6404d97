"""MM/MM and QC/MM Lennard-Jones energies of NBModelABFS, CPU side: the oracle's restatement pinned to the reference
core's outputs (golden fixture, and the live reference library where it is built), its gradients, the ABFS terms'
continuity, the LJ tables, the MM model builder, and the host-side argument checks of the C ABI."""

import json, os

import numpy as np
import pytest

from oracle import mmmm

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "mmmm_reference.json")))


def _run_oracle(c, xyz=None):
    return mmmm.energies(c["xyz"] if xyz is None else xyz, c["charges"], c["lj_types"], c["flags"], c["epsilon"], c["sigma"],
                         c["epsilon14"], c["sigma14"], c["opls"], c["exclusions"], c["pairs14"], c["inner"], c["outer"],
                         c["damping"], c["dielectric"], c["scale14"])


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=[c["name"] for c in GOLDEN["cases"]])
def test_oracle_matches_reference_fixture(case):
    E, G = _run_oracle(case)
    Er, Gr = np.array(case["energies_kj"]), np.array(case["gradients_kj_per_a"])
    assert (np.abs(Er) > 0).all()   # every term occurs in the fixture
    np.testing.assert_allclose(E, Er, rtol=0, atol=1e-9)
    np.testing.assert_allclose(G, Gr, rtol=0, atol=1e-10)


def test_oracle_matches_reference_library():
    R = pytest.importorskip("oracle.refdriver")
    try:
        R.lib()
    except R.RefUnavailable:
        pytest.skip("reference core not built")
    c = GOLDEN["cases"][0]
    rng = np.random.default_rng(4)
    X = np.array(c["xyz"]) + rng.normal(scale=0.05, size=(len(c["xyz"]), 3))
    flags = np.array(c["flags"])
    flags[100:180] |= mmmm.FLAG_FIXED
    args = (X, c["charges"], c["lj_types"], flags, c["epsilon"], c["sigma"], c["epsilon14"], c["sigma14"], False,
            c["exclusions"], c["pairs14"])
    E, G = mmmm.energies(*args, inner=7.0, outer=10.0, damp=0.8, dielectric=1.5, scale14=0.5)
    Er, Gr = R.mmmm_energy(*args, inner=7.0, outer=10.0, damp=0.8, listCutoff=11.0, dielectric=1.5, scale14=0.5)
    np.testing.assert_allclose(E, Er, rtol=0, atol=1e-9)
    np.testing.assert_allclose(G, Gr, rtol=0, atol=1e-10)


def test_oracle_gradients_by_finite_differences():
    c = GOLDEN["cases"][0]
    X = np.array(c["xyz"])
    _, G = _run_oracle(c)
    h = 1e-5
    for a in (0, 11, 12, 200):
        for d in range(3):
            Xp, Xm = X.copy(), X.copy()
            Xp[a, d] += h
            Xm[a, d] -= h
            num = (_run_oracle(c, Xp)[0].sum() - _run_oracle(c, Xm)[0].sum()) / (2 * h)
            assert abs(num - G[a, d]) < 2e-5 * max(1.0, abs(G[a, d]))


def test_abfs_terms_at_the_switching_radii():
    f = mmmm.abfs_factors(8.0, 12.0, 0.5)
    lo, hi = 8.0 - 1e-9, 8.0 + 1e-9
    a = mmmm.pair_terms(f, np.array([lo * lo, hi * hi]), 1.0, 1.0e5, 1.0e2)
    assert abs(a[0][0] - a[0][1]) < 1e-9 and abs(a[1][0] - a[1][1]) < 1e-9
    z = mmmm.pair_terms(f, np.array([144.0]), 1.0, 1.0e5, 1.0e2)
    assert abs(z[0][0]) < 1e-12 and abs(z[1][0]) < 1e-12
    # damping radius: electrostatics and the r^-12 part join continuously; the r^-6 part changes sign there, as in the
    # reference (PairwiseInteraction.c:132-137 builds its damped branch from -s^6 + bShift6 while
    # PairwiseInteraction.h:115 subtracts B times it), so the oracle keeps that
    lo, hi = (0.5 - 1e-12) ** 2, (0.5 + 1e-12) ** 2
    a = mmmm.pair_terms(f, np.array([lo, hi]), 1.0, 1.0e5, 0.0)
    assert abs(a[0][0] - a[0][1]) < 1e-9 and abs(a[1][0] - a[1][1]) < 1e-6 * abs(a[1][0])
    b = mmmm.pair_terms(f, np.array([lo, hi]), 0.0, 0.0, 1.0)
    np.testing.assert_allclose(b[1][0], -b[1][1], rtol=1e-9)


@pytest.mark.parametrize("rule", ["OPLS", "AMBER"])
def test_lj_tables(rule):
    from pdynamo_mirror_gb300.mmmodel import LJParameterContainer
    eps, sig = [0.6364, 0.3, 0.0], [3.15, 2.5, 0.0]
    lj = LJParameterContainer(eps, sig, rule)
    A, B = lj.tables()
    Ao, Bo = mmmm.lj_tables(np.array(eps), np.array(sig), rule == "OPLS")
    np.testing.assert_allclose(A, Ao, rtol=1e-15)
    np.testing.assert_allclose(B, Bo, rtol=1e-15)
    A2, _ = lj.Scale(0.5).tables()
    np.testing.assert_allclose(A2, 0.5 * A, rtol=1e-14)


def test_tip3p_model_of_the_water_box():
    from pdynamo_mirror_gb300 import workloads
    from pdynamo_mirror_gb300.mmmodel import MMModel
    Z, X, Q, sel, _ = workloads.qcmm_water_box(seed=1, n_qc_waters=3, n_mm_waters=50, box=14.0)
    m = MMModel.TIP3PWater(Z, X)
    n_water = int((Z == 8).sum()) - 1
    assert len(m.exclusions) == 3 * n_water + 1   # O-H, O-H, H-H per water; O-H of the hydroxide
    np.testing.assert_allclose(m.charges[len(sel):], Q[len(sel):])
    with pytest.raises(ValueError):
        MMModel(m.charges, m.ljTypes, m.ljParameters, exclusions=[(0, 0)])


def test_c_abi_rejects_bad_arguments():
    from pdynamo_mirror_gb300 import _native
    import ctypes
    L = _native.load()
    q = np.zeros(2); t = np.zeros(2, np.int32); fl = np.array([1, 1], np.uint8); tab = np.zeros(1)
    ex = np.array([0, 0], np.int32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    h = ctypes.c_void_p()
    rc = L.pdg_mm_create(2, p(q), p(t), p(fl), 1, p(tab), p(tab), p(tab), p(tab), 1, p(ex), 0, None, 8.0, 12.0, 0.5, 1.0, 1.0,
                         ctypes.byref(h))
    assert rc == _native.PDG_BAD_ARGUMENT and b"self pair" in L.pdg_last_error()
    rc = L.pdg_mm_create(2, p(q), p(t), p(fl), 1, p(tab), p(tab), p(tab), p(tab), 0, None, 0, None, 12.0, 8.0, 0.5, 1.0, 1.0,
                         ctypes.byref(h))
    assert rc == _native.PDG_BAD_ARGUMENT


def test_harmonic_terms_match_finite_differences_and_tip3p_geometry():
    """The oracle's harmonic bond and angle terms: zero at the TIP3P geometry, analytic gradients against central
    differences on a distorted water pair, and the flexible TIP3P model's terms (two bonds and one angle per water)."""
    import numpy as np
    from oracle import mmmm
    from pdynamo_mirror_gb300 import MMModel, workloads
    Z, X = workloads.water_cluster(2, seed=5)
    m = MMModel.TIP3PWater(Z, X, flexible=True)
    assert len(m.bonds) == 4 and len(m.angles) == 2
    eb, ea, G = mmmm.harmonic_terms(X, m.bonds, m.bondParameters, m.angles, m.angleParameters)
    assert abs(eb) < 1e-10 and abs(ea) < 1e-10
    Xd = X + np.random.default_rng(2).normal(scale=0.05, size=X.shape)
    eb, ea, G = mmmm.harmonic_terms(Xd, m.bonds, m.bondParameters, m.angles, m.angleParameters)
    assert eb > 0 and ea > 0
    h = 1e-6
    for a in range(len(Z)):
        for c in range(3):
            Xp, Xm = Xd.copy(), Xd.copy()
            Xp[a, c] += h; Xm[a, c] -= h
            ep = sum(mmmm.harmonic_terms(Xp, m.bonds, m.bondParameters, m.angles, m.angleParameters)[:2])
            em = sum(mmmm.harmonic_terms(Xm, m.bonds, m.bondParameters, m.angles, m.angleParameters)[:2])
            assert abs((ep - em) / (2 * h) - G[a, c]) < 1e-5 * max(1.0, abs(G[a, c]))
    assert len(MMModel.TIP3PWater(Z, X).bonds) == 0
