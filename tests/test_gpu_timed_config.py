"""The configurations the benchmark times, each frame against the oracle.

* The QC/MM water box (65 QC atoms, charge -1, AM1, in 4000 TIP3P waters, NBModelABFS 8/12 A) on the benchmark's
  own perturbed frames, through System.EnergyBatch with the mixed method exactly as timed (MIXED_METHOD: six BF16
  partial products, purification until the RMS density change is below 1e-5, then FP64 and perturbative steps;
  with it the FP32 DIIS history and commutators, the FP32 sp-sp and sp-s pair-gradient terms and the FP32 QC/MM
  gradient pair terms), and with the plain FP64 method.
* PM3 water clusters of 30, 48 and 64 waters (N = 180-384: beyond the one-tile purification step, so their
  mixed method is FP64 + perturbative steps) computed together by MoleculeBatch, as the cluster benchmark runs them.

Every frame is checked against the oracle (QCModel.Energy's SCF to the 1e-8 density tolerance, the reference's
defaults) at the accuracy gate of this path: |dE| < 1e-6 Hartree and max |dF| < 1e-5 Hartree/Bohr, QC and MM sides.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

KJ = 2625.5
A2B = 1.0e-10 / 5.291772083e-11
E_TOL, G_TOL = 1.0e-6, 1.0e-5
N_FRAMES = 8


def _oracle_qcmm(Z, Q, sel, charge, X, knots):
    nq = len(sel)
    phi, _, _ = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], knots=knots)
    r = O.System(O.Hamiltonian("am1", list(Z[:nq])), list(Z[:nq]), charge=charge).energy(X[:nq], phi=phi)
    _, gq, gm = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], qcq=r["charges"], knots=knots)
    return r, gq, gm


@pytest.mark.parametrize("method", ["mixed", "fp64"])
def test_benchmark_water_box_frames_match_oracle(method):
    from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelABFS, QCModelMNDO, System, workloads
    from pdynamo_mirror_gb300.converger import MIXED_METHOD
    Z, X, Q, sel, charge, frames = workloads.qcmm_water_box_frames(N_FRAMES)
    s = System(Z, X, mmCharges=Q)
    s.electronicState.charge = charge
    conv = DIISSCFConverger(**(MIXED_METHOD if method == "mixed" else {}))
    s.DefineQCModel(QCModelMNDO("am1", converger=conv), qcSelection=sel)
    s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
    E, G, terms = s.EnergyBatch(frames, doGradients=True, warmStart=False)
    assert (terms["Status"] == 0).all()
    nq = len(sel)
    knots = O.abfs_knots(8.0, 12.0)
    for f in range(N_FRAMES):
        r, gq, gm = _oracle_qcmm(Z, Q, sel, charge, frames[f], knots)
        assert abs(terms["Pure QC"][f] / KJ - (r["eelectronic"] + r["enuclear"] + r["baseline"])) < E_TOL, f
        assert abs(terms["QC/MM Elect."][f] / KJ - r["eqcmm"]) < E_TOL, f
        g = G[f] / (A2B * KJ)
        assert np.abs(g[:nq] - (r["gradients"] + gq)).max() < G_TOL, f
        assert np.abs(g[nq:] - gm).max() < G_TOL, f
        np.testing.assert_allclose(s.qcChargesBatch[f], r["charges"], rtol=0, atol=1e-6)


@pytest.mark.parametrize("method", ["mixed", "fp64"])
def test_large_water_clusters_batch_match_oracle(method):
    from pdynamo_mirror_gb300 import DIISSCFConverger, MoleculeBatch, workloads
    from pdynamo_mirror_gb300.converger import MIXED_METHOD
    mols = [workloads.water_cluster(w, seed=500 + w) for w in (30, 48, 64)]
    b = MoleculeBatch("pm3", mols)
    assert max(b.n_basis) == 384
    r = b.run(b.coordinates(mols), DIISSCFConverger(**(MIXED_METHOD if method == "mixed" else {})))
    assert (r["status"].cpu().numpy() == 0).all()
    E, G = r["energies"].cpu().numpy(), r["gradients"].cpu().numpy()
    for k, (Z, X) in enumerate(mols):
        ref = O.System(O.Hamiltonian("pm3", list(Z)), list(Z)).energy(X)
        e = E[k, 1] + E[k, 2] + E[k, 3]
        assert abs(e - (ref["eelectronic"] + ref["enuclear"] + ref["baseline"])) < E_TOL, k
        assert np.abs(G[b.atom_offsets[k]:b.atom_offsets[k + 1]] - ref["gradients"]).max() < G_TOL, k


def test_shared_base_water_box_frames_match_oracle():
    """The mixed method with a shared base, as timed: a first batch of frames (their own seed) leaves the base of
    frame 0's FP64 step; the benchmark's frames then start from its density and converge by perturbative density
    steps around it alone.  Every frame against the oracle at the gate; the per-frame SCF timers show that no frame
    needed purification and (nearly) none an FP64 step."""
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelABFS, QCModelMNDO, System, workloads
    from pdynamo_mirror_gb300.converger import SHARED_BASE_METHOD
    Z, X, Q, sel, charge, frames = workloads.qcmm_water_box_frames(N_FRAMES)
    s = System(Z, X, mmCharges=Q)
    s.electronicState.charge = charge
    s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(**SHARED_BASE_METHOD)), qcSelection=sel)
    s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
    first = workloads.perturbed_frames(X, N_FRAMES, sigma=0.02, seed=99)
    s.EnergyBatch(first, doGradients=True, warmStart=False)
    eng = s.engine()
    assert eng._base is not None
    E, G, terms = s.EnergyBatch(frames, doGradients=True, warmStart=False)
    assert (terms["Status"] == 0).all()
    T = eng.timings(N_FRAMES)
    assert T["QC Densities Purification Steps"].max() == 0
    assert T["QC Densities Perturbative Steps"].min() >= 3
    assert T["QC Densities Steps"].mean() <= 0.25
    nq = len(sel)
    knots = O.abfs_knots(8.0, 12.0)
    for f in range(N_FRAMES):
        r, gq, gm = _oracle_qcmm(Z, Q, sel, charge, frames[f], knots)
        assert abs(terms["Pure QC"][f] / KJ - (r["eelectronic"] + r["enuclear"] + r["baseline"])) < E_TOL, f
        assert abs(terms["QC/MM Elect."][f] / KJ - r["eqcmm"]) < E_TOL, f
        g = G[f] / (A2B * KJ)
        assert np.abs(g[:nq] - (r["gradients"] + gq)).max() < G_TOL, f
        assert np.abs(g[nq:] - gm).max() < G_TOL, f


def test_shared_base_from_a_distant_geometry_falls_back_and_converges():
    """A base from frames 0.08 A (RMS per coordinate) away cannot carry the first step for most frames (K is not
    small): those frames start again cold (the diagonal guess and the per-frame mixed path: purification, an FP64 step, perturbative steps
    around their own base) and still converge to the plain FP64 results."""
    from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelABFS, QCModelMNDO, System, workloads
    from pdynamo_mirror_gb300.converger import SHARED_BASE_METHOD
    Z, X, Q, sel, charge, frames = workloads.qcmm_water_box_frames(4)
    res = {}
    for method in ("shared", "fp64"):
        s = System(Z, X, mmCharges=Q)
        s.electronicState.charge = charge
        s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(**(SHARED_BASE_METHOD if method == "shared" else {}))),
                        qcSelection=sel)
        s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
        if method == "shared":
            s.EnergyBatch(workloads.perturbed_frames(X, 4, sigma=0.08, seed=98), doGradients=True, warmStart=False)
        res[method] = s.EnergyBatch(frames, doGradients=True, warmStart=False)
        if method == "shared":
            T = s.engine().timings(4)
            assert (T["QC Densities Steps"] >= 1).any() and (T["QC Densities Purification Steps"] >= 1).any()
    (Es, Gs, ts), (Ep, Gp, tp) = res["shared"], res["fp64"]
    assert (ts["Status"] == 0).all()
    assert np.abs(Es - Ep).max() / KJ < E_TOL
    assert np.abs(Gs - Gp).max() / (A2B * KJ) < G_TOL


def test_linear_response_guess_with_shared_base_matches_oracle_and_saves_cycles():
    """The headline configuration: the shared base plus the learned linear-response start density, fitted to the
    densities converged on 1024 frames of another seed.  On 128 held-out frames it starts closer to the converged
    density than the shared base's density and saves SCF cycles; the benchmark's frames converge from it to the
    oracle's energies and gradients at the gate."""
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, LinearResponseGuess, NBModelABFS, QCModelMNDO, System, workloads
    from pdynamo_mirror_gb300.converger import SHARED_BASE_METHOD
    Z, X, Q, sel, charge, frames = workloads.qcmm_water_box_frames(N_FRAMES)
    s = System(Z, X, mmCharges=Q)
    s.electronicState.charge = charge
    s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(**SHARED_BASE_METHOD)), qcSelection=sel)
    s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
    eng, conv, nb = s.engine(), s.qcModel.converger, s.nbModel
    g = LinearResponseGuess(eng)
    tr = workloads.perturbed_frames(X, 1024, sigma=0.02, seed=101)
    for s0 in range(0, 1024, 256):
        qc_t, mm_t, q_t, _ = s._device_inputs(tr[s0:s0 + 256])
        r = eng.run(qc_t, conv, mm_t, q_t, nb, gradients=False, warm_start=False)
        assert (r["status"] == 0).all()
        g.fit(qc_t, r["phi"], eng.density)
    qc_v, mm_v, q_v, _ = s._device_inputs(workloads.perturbed_frames(X, 128, sigma=0.02, seed=201))
    v = g.validate(qc_v, conv, mm_v, q_v, nb)
    assert v["enabled"] and v["iterations_saved"] >= 0.5 and v["rms_error_learned"] < 5e-4, v
    s.DefineDensityGuess(g)
    E, G, terms = s.EnergyBatch(frames, doGradients=True, warmStart=False)
    assert (terms["Status"] == 0).all()
    nq = len(sel)
    knots = O.abfs_knots(8.0, 12.0)
    for f in range(N_FRAMES):
        r, gq, gm = _oracle_qcmm(Z, Q, sel, charge, frames[f], knots)
        assert abs(terms["Pure QC"][f] / KJ - (r["eelectronic"] + r["enuclear"] + r["baseline"])) < E_TOL, f
        assert abs(terms["QC/MM Elect."][f] / KJ - r["eqcmm"]) < E_TOL, f
        gg = G[f] / (A2B * KJ)
        assert np.abs(gg[:nq] - (r["gradients"] + gq)).max() < G_TOL, f
        assert np.abs(gg[nq:] - gm).max() < G_TOL, f
