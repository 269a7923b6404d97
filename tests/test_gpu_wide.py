"""One QC region's SCF over the whole GPU (pdg_wide_energy_gradients) against the oracle and against the one-CTA path.

* the QC/MM water box (65 QC atoms, N = 131, ABFS) and a 60-water AM1 cluster (N = 360), with the wide engine forced,
  against the oracle at the accuracy gate (|dE| < 1e-6 Hartree, max |dF| < 1e-5 Hartree/Bohr) and against the
  one-CTA path (both converge the same FP64 SCF to the 1e-8 density tolerance: total energies within 1e-8 Hartree,
  SCF cycle counts within two);
* a warm start from the converged density converges again in at most two cycles to the same energy;
* the large QC/MM system (200 QC waters, 600 atoms, N = 1200, in 20000 TIP3P waters; the engine picks the wide path
  by size) through System.Energy against the oracle's fixture (tests/golden/large_qcmm_reference.json): energy terms,
  QC gradients, the MM gradients of the 400 MM atoms nearest the QC region and the sum of all MM gradients; with the
  plain FP64 method and with the mixed method (perturbative density steps around an FP64 base, FP32 DIIS errors and
  pair-gradient terms), and the mixed method again on a displaced geometry warm-started from the first (an MD step:
  its density steps are all perturbative ones around the kept base) against the plain method on that geometry.
"""
import json, os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

KJ = 2625.5
A2B = 1.0e-10 / 5.291772083e-11
E_TOL, G_TOL = 1.0e-6, 1.0e-5
HERE = os.path.dirname(os.path.abspath(__file__))


def _engine(h, Z, charge, wide):
    from pdynamo_mirror_gb300.engine import QCEngine
    return QCEngine(h, Z, charge, wide=wide)


def test_wide_water_box_matches_oracle_and_one_cta_path():
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelABFS, workloads
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=1)
    nq = len(sel)
    nb = NBModelABFS(innerCutoff=8.0, outerCutoff=12.0)
    qc = torch.as_tensor(X[None, :nq], device="cuda").contiguous()
    mm = torch.as_tensor(X[None, nq:], device="cuda").contiguous()
    q = torch.as_tensor(Q[nq:], device="cuda")
    out = {}
    for wide in (True, False):
        eng = _engine("am1", Z[:nq], charge, wide)
        assert eng.wide == wide
        r = eng.run(qc, DIISSCFConverger(), mm, q, nb, gradients=True, warm_start=False)
        assert int(r["status"][0]) == 0
        out[wide] = (r["energies"][0].cpu().numpy(), (r["qc_gradients"] + r["qcmm_qc_gradients"])[0].cpu().numpy(),
                     r["charges"][0].cpu().numpy(), int(r["ncycles"][0]))
    (Ew, Gw, Cw, nw), (Ec, Gc, Cc, nc) = out[True], out[False]
    knots = O.abfs_knots(8.0, 12.0)
    phi, _, _ = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], knots=knots)
    ref = O.System(O.Hamiltonian("am1", list(Z[:nq])), list(Z[:nq]), charge=charge).energy(X[:nq], phi=phi)
    _, gq, _ = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], qcq=ref["charges"], knots=knots)
    assert abs(Ew[1] + Ew[2] + Ew[3] - (ref["eelectronic"] + ref["enuclear"] + ref["baseline"])) < E_TOL
    assert abs(Ew[4] - ref["eqcmm"]) < E_TOL
    assert np.abs(Gw - (ref["gradients"] + gq)).max() < G_TOL
    # two SCFs, each stopped at the 1e-8 RMS density tolerance: the total energy is variational and agrees to 1e-8,
    # its one- and two-electron parts (first order in the density) to 1e-6, gradients and charges to 1e-6
    assert abs(Ew[0] - Ec[0]) < 1e-8
    np.testing.assert_allclose(Ew[:7], Ec[:7], rtol=0, atol=1e-6)
    np.testing.assert_allclose(Gw, Gc, rtol=0, atol=1e-6)
    np.testing.assert_allclose(Cw, Cc, rtol=0, atol=1e-6)
    assert abs(nw - nc) <= 2


def test_wide_cluster_matches_oracle_and_warm_start():
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, workloads
    Z, X = workloads.water_cluster(60, seed=61)
    eng = _engine("am1", Z, 0, True)
    xyz = torch.as_tensor(X[None], device="cuda").contiguous()
    r = eng.run(xyz, DIISSCFConverger(), gradients=True, warm_start=False)
    assert int(r["status"][0]) == 0
    E, G = r["energies"][0].cpu().numpy(), r["qc_gradients"][0].cpu().numpy()
    ref = O.System(O.Hamiltonian("am1", list(Z)), list(Z)).energy(X)
    assert abs(E[1] + E[2] + E[3] - (ref["eelectronic"] + ref["enuclear"] + ref["baseline"])) < E_TOL
    assert np.abs(G - ref["gradients"]).max() < G_TOL
    r2 = eng.run(xyz, DIISSCFConverger(), gradients=True, warm_start=True)
    assert int(r2["status"][0]) == 0 and int(r2["ncycles"][0]) <= 2
    assert abs(float(r2["energies"][0, 0]) - float(E[0])) < 1e-9


@pytest.mark.parametrize("method", ["fp64", "mixed"])
def test_wide_mixed_water_box_matches_oracle(method):
    from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelABFS, QCModelMNDO, System, workloads
    from pdynamo_mirror_gb300.converger import MIXED_METHOD
    from pdynamo_mirror_gb300.engine import QCEngine
    Z, X, Q, sel, charge, frames = workloads.qcmm_water_box_frames(2)
    nq = len(sel)
    s = System(Z, X, mmCharges=Q)
    s.electronicState.charge = charge
    s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(**(MIXED_METHOD if method == "mixed" else {}))), qcSelection=sel)
    s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
    s._engine, s._engine_charge = QCEngine("am1", list(Z[:nq]), charge, wide=True), charge
    E, G, terms = s.EnergyBatch(frames, doGradients=True, warmStart=False)
    knots = O.abfs_knots(8.0, 12.0)
    for f in range(2):
        X_ = frames[f]
        phi, _, _ = O.qcmm("abfs", X_[:nq], X_[nq:], Q[nq:], knots=knots)
        r = O.System(O.Hamiltonian("am1", list(Z[:nq])), list(Z[:nq]), charge=charge).energy(X_[:nq], phi=phi)
        _, gq, gm = O.qcmm("abfs", X_[:nq], X_[nq:], Q[nq:], qcq=r["charges"], knots=knots)
        assert abs(terms["Pure QC"][f] / KJ - (r["eelectronic"] + r["enuclear"] + r["baseline"])) < E_TOL
        assert abs(terms["QC/MM Elect."][f] / KJ - r["eqcmm"]) < E_TOL
        g = G[f] / (A2B * KJ)
        assert np.abs(g[:nq] - (r["gradients"] + gq)).max() < G_TOL
        assert np.abs(g[nq:] - gm).max() < G_TOL


@pytest.mark.parametrize("method", ["fp64", "mixed"])
def test_large_qcmm_system_matches_oracle_fixture(method):
    from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelABFS, QCModelMNDO, System, workloads
    from pdynamo_mirror_gb300.converger import MIXED_METHOD
    ref = json.load(open(os.path.join(HERE, "golden", "large_qcmm_reference.json")))
    Z, X, Q, sel, charge = workloads.large_qcmm()
    nq = len(sel)
    s = System(Z, X, mmCharges=Q)
    s.electronicState.charge = charge
    s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(**(MIXED_METHOD if method == "mixed" else {}))), qcSelection=sel)
    s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
    assert s.engine().wide and s.engine().n_basis == 1200
    s.Energy(doGradients=True)
    t = s.configuration.energyTerms
    assert abs(t["Pure QC"] / KJ - (ref["eelectronic"] + ref["enuclear"] + ref["baseline"])) < E_TOL
    assert abs(t["QC/MM Elect."] / KJ - ref["eqcmm"]) < E_TOL
    g = s.configuration.gradients3 / (A2B * KJ)
    assert np.abs(g[:nq] - np.array(ref["qc_gradients"])).max() < G_TOL
    mm = np.array(ref["mm_sample"]) + nq
    assert np.abs(g[mm] - np.array(ref["mm_gradients_sample"])).max() < G_TOL
    assert np.abs(g[nq:].sum(axis=0) - np.array(ref["mm_gradient_sum"])).max() < G_TOL
    if method == "mixed":
        # an MD-like step: every atom displaced by up to 0.005 A, warm start from the converged density; the kept base
        # carries every density step, and the result agrees with the plain method on the new geometry
        eng = s.engine()
        eng.wide_phase_events(True)
        X2 = X + np.random.default_rng(7).uniform(-0.005, 0.005, size=X.shape)
        s.coordinates3 = X2
        e_mixed = s.Energy(doGradients=True)
        g_mixed = s.configuration.gradients3.copy()
        steps = eng.wide_phase_times()
        assert steps["fp64_steps"] == 0 and steps["perturbative_steps"] >= 1
        p = System(Z, X2, mmCharges=Q)
        p.electronicState.charge = charge
        p.DefineQCModel(QCModelMNDO("am1"), qcSelection=sel)
        p.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
        e_plain = p.Energy(doGradients=True)
        assert abs(e_mixed - e_plain) / KJ < E_TOL
        assert np.abs(g_mixed - p.configuration.gradients3).max() / (A2B * KJ) < G_TOL
