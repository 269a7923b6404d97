"""GPU parity: the CUDA path (through libpdg.so's C ABI) against the oracle and the reference fixtures.

Tolerances are the accuracy gate of this path: |dE| < 1e-6 Hartree and max |dG| < 1e-5 Hartree/Bohr for
converged energies and gradients; intermediate matrices (H, F for a fixed density, gradients for a fixed
density) are compared at 1e-10 (round-off level).
"""
import json, os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
REF = json.load(open(os.path.join(GOLD, "mndo_rhf_reference.json")))
MOLS = json.load(open(os.path.join(GOLD, "molecules.json")))
QCMM = json.load(open(os.path.join(GOLD, "qcmm_reference.json")))
KJ = 2625.5
A2B = 1.0e-10 / 5.291772083e-11
E_TOL, G_TOL = 1.0e-6, 1.0e-5


def _engine(h, Z, charge=0):
    from pdynamo_mirror_gb300.engine import QCEngine
    return QCEngine(h, Z, charge)


def _dev(x):
    import torch
    return torch.as_tensor(np.asarray(x, dtype=np.float64), device="cuda")


def _unpack(p, n):
    P = np.zeros((n, n))
    k = 0
    for i in range(n):
        for j in range(i + 1):
            P[i, j] = P[j, i] = p[k]; k += 1
    return P


SMALL = ["water", "waterDimer_Cs", "methane", "formaldehyde", "glycine", "fch3cl", "dihydrogen", "hydrogenFluoride",
         "ammonia", "benzene", "acetone", "nitromethane"]


@pytest.mark.parametrize("h", ["am1", "pm3", "mndo", "rm1", "pddgmndo", "pddgpm3"])
def test_one_electron_and_fock_match_oracle(h):
    for label in SMALL:
        if label not in REF[h]:
            continue
        m = MOLS[label]
        Z, X = m["Z"], np.array(m["xyz"])
        eng = _engine(h, Z, m["charge"])
        os_ = O.System(O.Hamiltonian(h, Z), Z, charge=m["charge"])
        r = os_.energy(X, gradients=False)
        N = eng.n_basis
        Hg = eng.one_electron(_dev(X[None]))[0].cpu().numpy()
        np.testing.assert_allclose(Hg, _unpack(r["H"], N), rtol=0, atol=1e-10, err_msg=label)
        P = _unpack(r["density"], N)
        phi = np.linspace(-0.05, 0.05, len(Z))
        Fo, eo = os_.fock(X, r["density"], phi=phi)
        Fg, eg = eng.fock(_dev(X[None]), _dev(P[None]), phi=_dev(phi[None]))
        np.testing.assert_allclose(Fg[0].cpu().numpy(), _unpack(Fo, N), rtol=0, atol=1e-10, err_msg=label)
        eg = eg[0].cpu().numpy()
        assert abs(eg[0] - eo[0]) < 1e-10 and abs(eg[2] - eo[2]) < 1e-10, label
        go = os_.gradients(X, r["density"])
        gg = eng.gradients(_dev(X[None]), _dev(P[None]))[0].cpu().numpy()
        np.testing.assert_allclose(gg, go, rtol=0, atol=1e-10, err_msg=label)


def _cases():
    out = []
    for h in sorted(REF):
        for label in sorted(REF[h]):
            if len(MOLS[label]["Z"]) <= 16 or label in ("glycine", "benzene", "caffeine", "napthalene"):
                out.append((h, label))
    return out


@pytest.mark.parametrize("h,label", _cases())
def test_energy_gradients_match_reference_fixture(h, label):
    from pdynamo_mirror_gb300 import DIISSCFConverger, QCModelMNDO, System
    m, e = MOLS[label], REF[h][label]
    s = System(m["Z"], m["xyz"])
    s.electronicState.charge = m["charge"]
    s.DefineQCModel(QCModelMNDO(h, converger=DIISSCFConverger(densityTolerance=1.0e-8, maximumSCFCycles=500)))
    energy = s.Energy(doGradients=True)
    assert abs(energy - e["pure_qc_kj"]) / KJ < E_TOL
    g = s.configuration.gradients3 / (A2B * KJ)
    assert np.abs(g - np.array(e["gradients"])).max() < G_TOL
    assert abs(s.configuration.energyTerms["SCF Cycles"] - e["ncycles"]) <= 10


def test_batched_water_frames_match_oracle():
    from pdynamo_mirror_gb300 import QCModelMNDO, System, workloads
    Z, X = workloads.water_cluster(16, seed=0)
    frames = workloads.perturbed_frames(X, 6, sigma=0.03, seed=3)
    s = System(Z, X)
    s.DefineQCModel(QCModelMNDO("am1"))
    E, G, terms = s.EnergyBatch(frames, doGradients=True)
    ham = O.Hamiltonian("am1", Z)
    for f in range(len(frames)):
        r = O.System(ham, list(Z)).energy(frames[f])
        e_ref = KJ * (r["eelectronic"] + r["enuclear"] + r["baseline"])
        assert abs(E[f] - e_ref) / KJ < E_TOL
        assert np.abs(G[f] / (A2B * KJ) - r["gradients"]).max() < G_TOL


def test_warm_start_reuses_density():
    from pdynamo_mirror_gb300 import QCModelMNDO, System, workloads
    Z, X = workloads.water_cluster(8, seed=4)
    s = System(Z, X)
    s.DefineQCModel(QCModelMNDO("pm3"))
    e1 = s.Energy(doGradients=True)
    c1 = s.configuration.energyTerms["SCF Cycles"]
    e2 = s.Energy(doGradients=True)
    c2 = s.configuration.energyTerms["SCF Cycles"]
    assert abs(e1 - e2) / KJ < 1e-8 and c2 < c1


def test_not_converged_raises():
    from pdynamo_mirror_gb300 import DIISSCFConverger, QCModelMNDO, SCFNotConverged, System, workloads
    Z, X = workloads.water_cluster(4, seed=5)
    s = System(Z, X)
    s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(maximumSCFCycles=2)))
    with pytest.raises(SCFNotConverged):
        s.Energy()


def _qcmm_system(c, nb):
    from pdynamo_mirror_gb300 import QCModelMNDO, System
    s = System(c["Z"], c["xyz"], mmCharges=c["mm_charges"])
    s.DefineQCModel(QCModelMNDO("am1"), qcSelection=c["qc"])
    s.DefineNBModel(nb)
    return s


def test_book_example8_qcmm():
    from pdynamo_mirror_gb300 import NBModelFull
    c = QCMM["example8"]
    s = _qcmm_system(c, NBModelFull())
    s.Energy(doGradients=True)
    t = s.configuration.energyTerms
    b = c["book"]
    assert abs(t["Pure QC"] - b["pure_qc_kj"]) < 5e-5 and abs(t["QC/MM Elect."] - b["qcmm_kj"]) < 5e-5
    assert abs(t["Pure QC"] - c["pure_qc_kj"]) / KJ < E_TOL
    g = s.configuration.gradients3 / (A2B * KJ)
    assert np.abs(g[:3] - np.array(c["qc_gradients"])).max() < G_TOL
    assert np.abs(g[3:] - np.array(c["mm_gradients"])).max() < G_TOL


def test_abfs_qcmm_matches_reference_fixture():
    from pdynamo_mirror_gb300 import NBModelABFS
    c = QCMM["abfs"]
    s = _qcmm_system(c, NBModelABFS(innerCutoff=c["inner"], outerCutoff=c["outer"]))
    s.Energy(doGradients=True)
    t = s.configuration.energyTerms
    assert abs(t["Pure QC"] - c["pure_qc_kj"]) / KJ < E_TOL
    assert abs(t["QC/MM Elect."] - c["qcmm_kj"]) / KJ < E_TOL
    nq = len(c["qc"])
    g = s.configuration.gradients3 / (A2B * KJ)
    assert np.abs(g[:nq] - np.array(c["qc_gradients"])).max() < G_TOL
    assert np.abs(g[nq:] - np.array(c["mm_gradients"])).max() < G_TOL


@pytest.mark.parametrize("model", ["abfs", "full"])
def test_qcmm_potentials_and_gradients_match_oracle(model):
    import torch
    from pdynamo_mirror_gb300 import NBModelABFS, NBModelFull, _native, workloads
    from pdynamo_mirror_gb300.engine import QCEngine
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=1, n_mm_waters=800, box=30.0)
    nq = len(sel)
    nb = NBModelABFS() if model == "abfs" else NBModelFull()
    qcq = np.random.default_rng(0).uniform(-0.5, 0.5, nq)
    knots = O.abfs_knots(8.0, 12.0) if model == "abfs" else None
    phi_o, gq_o, gm_o = O.qcmm(model, X[:nq], X[nq:], Q[nq:], qcq=qcq, knots=knots)
    L = _native.load()
    dq, dm, dc = _dev(X[None, :nq]), _dev(X[None, nq:]), _dev(Q[nq:])
    kn = _dev(nb.knots()) if model == "abfs" else None
    nk = 0 if kn is None else kn.numel() // 3
    phi = torch.empty((1, nq), dtype=torch.float64, device="cuda")
    s = _native.stream_handle(torch.cuda.current_stream())
    wb = int(L.pdg_qcmm_workspace_bytes(1, len(Q) - nq))
    ws = torch.empty(wb, dtype=torch.uint8, device="cuda")
    _native.check(L.pdg_qcmm_potentials(nb.model_id, 1, nq, len(Q) - nq, _native.ptr(dq), _native.ptr(dm), _native.ptr(dc), nk,
                                        _native.ptr(kn), float(nb.outerCutoff), _native.ptr(phi), _native.ptr(ws), wb, s), "potentials")
    gq = torch.empty((1, nq, 3), dtype=torch.float64, device="cuda")
    gm = torch.empty((1, len(Q) - nq, 3), dtype=torch.float64, device="cuda")
    _native.check(L.pdg_qcmm_gradients(nb.model_id, 1, nq, len(Q) - nq, _native.ptr(dq), _native.ptr(dm), _native.ptr(dc),
                                       _native.ptr(_dev(qcq[None])), nk, _native.ptr(kn), float(nb.outerCutoff),
                                       _native.ptr(gq), _native.ptr(gm), _native.ptr(ws), wb, s), "gradients")
    np.testing.assert_allclose(phi[0].cpu().numpy(), phi_o, rtol=0, atol=1e-11)
    np.testing.assert_allclose(gq[0].cpu().numpy(), gq_o, rtol=0, atol=1e-11)
    np.testing.assert_allclose(gm[0].cpu().numpy(), gm_o, rtol=0, atol=1e-11)


def test_qcmm_water_box_energy_matches_oracle():
    """The benchmark system (65 QC atoms, charge -1, in 4000 TIP3P waters, ABFS 8/12 A) end to end."""
    from pdynamo_mirror_gb300 import NBModelABFS, QCModelMNDO, System, workloads
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=1)
    s = System(Z, X, mmCharges=Q)
    s.electronicState.charge = charge
    s.DefineQCModel(QCModelMNDO("am1"), qcSelection=sel)
    s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
    s.Energy(doGradients=True)
    t = s.configuration.energyTerms
    nq = len(sel)
    knots = O.abfs_knots(8.0, 12.0)
    phi, _, _ = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], knots=knots)
    r = O.System(O.Hamiltonian("am1", Z[:nq]), list(Z[:nq]), charge=charge).energy(X[:nq], phi=phi)
    _, gq, gm = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], qcq=r["charges"], knots=knots)
    assert abs(t["Pure QC"] / KJ - (r["eelectronic"] + r["enuclear"] + r["baseline"])) < E_TOL
    assert abs(t["QC/MM Elect."] / KJ - r["eqcmm"]) < E_TOL
    g = s.configuration.gradients3 / (A2B * KJ)
    assert np.abs(g[:nq] - (r["gradients"] + gq)).max() < G_TOL
    assert np.abs(g[nq:] - gm).max() < G_TOL


def test_scf_alone_reproduces_energy_gradients():
    """pdg_scf on the integrals left by pdg_energy_gradients gives the same converged energies."""
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, workloads
    from pdynamo_mirror_gb300.engine import QCEngine
    Z, X = workloads.water_cluster(8, seed=21)
    frames = workloads.perturbed_frames(X, 3, sigma=0.03, seed=22)
    eng = QCEngine("am1", Z, 0)
    conv = DIISSCFConverger()
    out = eng.run(_dev(frames), conv, gradients=False, warm_start=False)
    e1 = out["energies"].cpu().numpy()
    e2, st, nc = eng.scf(conv)
    assert (st.cpu().numpy() == 0).all()
    np.testing.assert_allclose(e2.cpu().numpy()[:, :7], e1[:, :7], rtol=0, atol=1e-12)
    assert (nc.cpu().numpy() == out["ncycles"].cpu().numpy()).all()


@pytest.mark.parametrize("products", [3, 6])
def test_purification_density_step_converges_to_the_fp64_result(products):
    """Split-BF16 purification cycles followed by FP64 cycles reach the plain FP64 path's converged
    energies and gradients (the last cycles are FP64, so the difference is convergence-level)."""
    from pdynamo_mirror_gb300 import DIISSCFConverger, QCModelMNDO, System, workloads
    Z, X = workloads.water_cluster(16, seed=0)
    frames = workloads.perturbed_frames(X, 4, sigma=0.03, seed=5)
    out = {}
    for step in ("fp64", "purification"):
        s = System(Z, X)
        s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(densityStep=step, purificationProducts=products)))
        out[step] = s.EnergyBatch(frames, doGradients=True, warmStart=False)
    (E0, G0, _), (E1, G1, t1) = out["fp64"], out["purification"]
    assert np.abs(E1 - E0).max() / KJ < 1e-8
    assert np.abs(G1 - G0).max() / (A2B * KJ) < 1e-6
    assert (t1["Status"] == 0).all()


def test_purification_qcmm_water_box_matches_oracle():
    """The benchmark system with the purification density step: same gate against the oracle."""
    from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelABFS, QCModelMNDO, System, workloads
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=1)
    s = System(Z, X, mmCharges=Q)
    s.electronicState.charge = charge
    s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(densityStep="purification")), qcSelection=sel)
    s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
    s.Energy(doGradients=True)
    t = s.configuration.energyTerms
    nq = len(sel)
    knots = O.abfs_knots(8.0, 12.0)
    phi, _, _ = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], knots=knots)
    r = O.System(O.Hamiltonian("am1", Z[:nq]), list(Z[:nq]), charge=charge).energy(X[:nq], phi=phi)
    _, gq, gm = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], qcq=r["charges"], knots=knots)
    assert abs(t["Pure QC"] / KJ - (r["eelectronic"] + r["enuclear"] + r["baseline"])) < E_TOL
    assert abs(t["QC/MM Elect."] / KJ - r["eqcmm"]) < E_TOL
    g = s.configuration.gradients3 / (A2B * KJ)
    assert np.abs(g[:nq] - (r["gradients"] + gq)).max() < G_TOL
    assert np.abs(g[nq:] - gm).max() < G_TOL
