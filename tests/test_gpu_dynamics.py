"""Langevin dynamics on the GPU (csrc/dynamics.cu) through the C ABI and the LangevinDynamics driver:
the counter-based normal deviates against the oracle's restatement, the two half-step kernels against the
oracle's restatement of LangevinVelocityVerletIntegrator.Iteration for given deviates, a QC/MM trajectory against
the oracle's energies and gradients step by step, the thermostat's temperature and position variance in a
harmonic well, and the invariance of trajectories under the SCF start density (the converged SCF decides)."""
import ctypes, math

import numpy as np
import pytest

from oracle import dynamics as D
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _sh():
    import torch
    from pdynamo_mirror_gb300 import _native
    return _native.stream_handle(torch.cuda.current_stream())


def _trimer(guess_seed=3):
    from pdynamo_mirror_gb300 import NBModelFull, QCModelMNDO, System, workloads
    Z, X = workloads.water_cluster(3, seed=guess_seed)
    mmX = X[:3] + np.array([6.0, 0.0, 0.0])
    q = np.array([workloads.TIP3P_O, workloads.TIP3P_H, workloads.TIP3P_H])
    s = System(np.concatenate([Z, [8, 1, 1]]), np.concatenate([X, mmX]), mmCharges=np.concatenate([np.zeros(len(Z)), q]))
    s.DefineQCModel(QCModelMNDO("am1"), qcSelection=range(len(Z)))
    s.DefineNBModel(NBModelFull())
    s.DefineFixedAtoms(range(len(Z), len(Z) + 3))
    return s, list(Z), mmX, q


def test_normal_deviates_match_oracle():
    import torch
    from pdynamo_mirror_gb300 import _native
    L = _native.load()
    for (n, seed, step, stream) in ((10001, 12345, 0, 0), (777, 2 ** 40 + 99, 31, 1)):
        out = torch.empty(2 * n, dtype=torch.float64, device="cuda")
        _native.check(L.pdg_normal_deviates(n, seed, step, stream, _native.ptr(out), _sh()), "pdg_normal_deviates")
        ref = D.normal_pairs(n, seed, step, stream).ravel()
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=0, atol=1e-13)


def test_half_step_kernels_match_oracle():
    import torch
    from pdynamo_mirror_gb300 import LangevinVelocityVerletIntegrator, _native
    L = _native.load()
    rng = np.random.default_rng(4)
    R, n_atoms, free = 3, 5, [0, 2, 3, 4]
    m = np.array([15.9994, 1.00794, 12.011, 1.00794, 14.0067])[free]
    x = rng.normal(size=(R, n_atoms, 3)); v = rng.normal(size=(R, len(free), 3)); a = rng.normal(size=(R, len(free), 3)) * 50
    integ = LangevinVelocityVerletIntegrator(25.0, 300.0, 0.0005)
    c = integ.constants
    t = lambda A, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(A), dtype=dt, device="cuda")
    dx, dv, da = t(x), t(v), t(a)
    dfree, dm, disq = t(free, torch.int32), t(m), t(1.0 / np.sqrt(m))
    dev = torch.empty((R, len(free), 3, 2), dtype=torch.float64, device="cuda")
    _native.check(L.pdg_langevin_positions(R, n_atoms, len(free), _native.ptr(dfree), _native.ptr(disq), _native.ptr(dx), _native.ptr(dv),
                                           _native.ptr(da), integ.factors(), 1, 99, 7, _native.ptr(dev), _sh()), "positions")
    w = dev.cpu().numpy()
    np.testing.assert_allclose(w.reshape(-1, 2), D.normal_pairs(R * len(free) * 3, 99, 7), rtol=0, atol=1e-13)
    for r in range(R):
        xr, vr = D.positions(x[r, free], v[r], a[r], m, c, w[r, ..., 0], w[r, ..., 1])
        np.testing.assert_allclose(dx.cpu().numpy()[r, free], xr, rtol=1e-14, atol=1e-14)
        np.testing.assert_allclose(dv.cpu().numpy()[r], vr, rtol=1e-14, atol=1e-14)
    fixed = [1]
    np.testing.assert_array_equal(dx.cpu().numpy()[:, fixed], x[:, fixed])
    # second half: gradients of two parts on n_atoms rows, scaled
    ga, gb = rng.normal(size=(R, n_atoms, 3)), rng.normal(size=(R, n_atoms, 3))
    v1 = dv.cpu().numpy()
    mv2 = torch.empty(R, dtype=torch.float64, device="cuda")
    dga, dgb = t(ga), t(gb)   # held: a temporary's memory could be reused before the kernel reads it
    _native.check(L.pdg_langevin_velocities(R, len(free), n_atoms, _native.ptr(dfree), _native.ptr(dm), _native.ptr(dga), _native.ptr(dgb),
                                            4962.0, c["facV3"], _native.ptr(dv), _native.ptr(da), _native.ptr(mv2), _sh()), "velocities")
    for r in range(R):
        vr, ar = D.velocities(v1[r], 4962.0 * (ga[r, free] + gb[r, free]), m, c)
        np.testing.assert_allclose(dv.cpu().numpy()[r], vr, rtol=1e-13, atol=1e-12)
        np.testing.assert_allclose(da.cpu().numpy()[r], ar, rtol=1e-13, atol=1e-12)
        assert math.isclose(float(mv2[r]), float((m[:, None] * vr * vr).sum()), rel_tol=1e-13)


def test_density_combine_matches_torch():
    import torch
    from pdynamo_mirror_gb300 import _native
    L = _native.load()
    for n in (1, 17, 131 * 131 * 3):
        terms = [torch.randn(n, dtype=torch.float64, device="cuda") for _ in range(5)]
        coef = [2.0, -1.0, 1.0, -2.0, 1.0]
        out = torch.empty(n, dtype=torch.float64, device="cuda")
        arr = (ctypes.c_void_p * 5)(*[x.data_ptr() for x in terms])
        _native.check(L.pdg_density_combine(n, 5, arr, (ctypes.c_double * 5)(*coef), _native.ptr(out), _sh()), "combine")
        ref = sum(c * x for c, x in zip(coef, terms))
        torch.testing.assert_close(out, ref, rtol=1e-15, atol=1e-14)
    bad = torch.empty(3, dtype=torch.float64, device="cuda")
    arr = (ctypes.c_void_p * 1)(bad.data_ptr() + 8)
    assert L.pdg_density_combine(2, 1, arr, (ctypes.c_double * 1)(1.0), _native.ptr(bad), _sh()) == _native.PDG_BAD_ARGUMENT


def _oracle_accelerations(Zq, x, mmX, q, masses, density):
    """Oracle E+grad of the QC atoms (QC + QC/MM, NBModelFull) -> accelerations A/ps^2 and the converged density."""
    from pdynamo_mirror_gb300.engine import GRADIENT_TO_KJ_PER_A
    phi, _, _ = O.qcmm("full", x, mmX, q)
    sysq = O.System(O.Hamiltonian("am1", Zq), Zq)
    r = sysq.energy(x, phi=phi, density=density)
    _, gq, _ = O.qcmm("full", x, mmX, q, qcq=r["charges"])
    g = (r["gradients"] + gq) * GRADIENT_TO_KJ_PER_A
    return -100.0 * g / masses[:, None], r["density"]


def test_qcmm_trajectory_matches_oracle():
    """Four Langevin steps of two replicas of a polarised water trimer: coordinates and velocities follow the
    oracle's integrator driven by the oracle's energies and gradients and the kernel's own deviates."""
    import torch
    from pdynamo_mirror_gb300 import LangevinDynamics
    from pdynamo_mirror_gb300.parameters import atomic_mass
    s, Zq, mmX, q = _trimer()
    md = LangevinDynamics(s, replicas=2, timeStep=0.0005, temperature=300.0, collisionFrequency=25.0, seed=11, densityGuess="previous")
    m = np.array([atomic_mass(z) for z in Zq])
    c = md.integrator.constants
    x = md.xyz.cpu().numpy().copy()
    v = md.vel.cpu().numpy().copy()
    for r in range(2):   # VelocitiesAssign: the exact temperature per replica
        assert math.isclose(D.temperature(v[r], m, 3 * len(m))[1], 300.0, rel_tol=1e-12)
    md.initialize()
    acc, dens = [], [None, None]
    for r in range(2):
        a_r, dens[r] = _oracle_accelerations(Zq, x[r], mmX, q, m, None)
        acc.append(a_r)
    np.testing.assert_allclose(md.acc.cpu().numpy(), np.array(acc), rtol=0, atol=2e-3)
    dev = torch.empty((2, len(Zq), 3, 2), dtype=torch.float64, device="cuda")
    for step in range(4):
        md.step(deviates=dev)
        w = dev.cpu().numpy()
        for r in range(2):
            x[r], v[r] = D.positions(x[r], v[r], acc[r], m, c, w[r, ..., 0], w[r, ..., 1])
            acc[r], dens[r] = _oracle_accelerations(Zq, x[r], mmX, q, m, dens[r])
            v[r], _ = D.velocities(v[r], -acc[r] * m[:, None] / 100.0, m, c)
        np.testing.assert_allclose(md.xyz.cpu().numpy(), x, rtol=0, atol=1e-8)
        np.testing.assert_allclose(md.vel.cpu().numpy(), v, rtol=0, atol=1e-5)
    ke, t = md.temperatures()
    for r in range(2):
        assert math.isclose(t[r], D.temperature(v[r], m, 3 * len(m))[1], rel_tol=1e-6)
    # the fixed MM atoms did not move and the system's coordinates are untouched until the run ends
    np.testing.assert_array_equal(md.mm_xyz.cpu().numpy()[0], mmX)


def test_thermostat_temperature_and_harmonic_variance():
    """4096 replicas of one hydrogen atom in a harmonic well (k = 100 kJ/mol/A^2) driven only by the kernels:
    after equilibration <T> = 300 K and <x^2> = kT / k per axis."""
    import torch
    from pdynamo_mirror_gb300 import LangevinVelocityVerletIntegrator, _native
    L = _native.load()
    R, k = 4096, 100.0
    integ = LangevinVelocityVerletIntegrator(25.0, 300.0, 0.001)
    c = integ.constants
    x = torch.zeros((R, 1, 3), dtype=torch.float64, device="cuda")
    v = torch.zeros_like(x); a = torch.zeros_like(x); g = torch.zeros_like(x)
    free = torch.zeros(1, dtype=torch.int32, device="cuda")
    m = torch.full((1,), 1.00794, dtype=torch.float64, device="cuda")
    isq = 1.0 / torch.sqrt(m)
    mv2 = torch.empty(R, dtype=torch.float64, device="cuda")
    temps, x2 = [], []
    for step in range(1, 1201):
        _native.check(L.pdg_langevin_positions(R, 1, 1, _native.ptr(free), _native.ptr(isq), _native.ptr(x), _native.ptr(v), _native.ptr(a),
                                               integ.factors(), 1, 5, step, None, _sh()), "positions")
        torch.mul(x, k, out=g)
        _native.check(L.pdg_langevin_velocities(R, 1, 1, _native.ptr(free), _native.ptr(m), _native.ptr(g), None, 1.0, c["facV3"],
                                                _native.ptr(v), _native.ptr(a), _native.ptr(mv2), _sh()), "velocities")
        if step > 400:
            temps.append(float(mv2.mean()) * D.AMUA2PS2_TO_K / 3.0)
            x2.append(float((x * x).mean()))
    kT = 1.3806505e-23 * 300.0 * 6.0221415e23 / 1000.0   # kJ/mol
    assert abs(np.mean(temps) - 300.0) < 6.0
    assert abs(np.mean(x2) - kT / k) < 0.03 * kT / k


def test_trajectories_do_not_depend_on_the_start_density():
    """Diagonal, previous-step and extrapolated start densities (and an untrained learned correction) give the
    same trajectory to SCF precision; the better starts take fewer SCF cycles."""
    from pdynamo_mirror_gb300 import LangevinDynamics, LearnedDensityGuess
    s, _, _, _ = _trimer()
    xs, cycles = {}, {}
    for mode in ("diagonal", "previous", "extrapolate", "learned"):
        guess = LearnedDensityGuess(s.engine(), seed=0) if mode == "learned" else mode
        md = LangevinDynamics(s, replicas=2, timeStep=0.0005, seed=5, densityGuess=guess)
        cyc = md.run(8)
        xs[mode] = md.xyz.cpu().numpy()
        cycles[mode] = float(np.mean([c.double().mean().item() for c in cyc[3:]]))
    for mode in ("previous", "extrapolate", "learned"):
        np.testing.assert_allclose(xs[mode], xs["diagonal"], rtol=0, atol=1e-7)
    assert cycles["extrapolate"] < cycles["diagonal"]
    assert cycles["previous"] < cycles["diagonal"]


def test_dynamics_writes_a_dcd_trajectory(tmp_path):
    """Frames at iteration 0 and every saveFrequency-th step of the chosen replica, fixed MM atoms once."""
    from pdynamo_mirror_gb300 import DCDTrajectoryFileReader, DCDTrajectoryFileWriter, LangevinDynamics
    s, Zq, mmX, q = _trimer()
    md = LangevinDynamics(s, replicas=2, timeStep=0.0005, seed=3)
    X0 = md.replica_coordinates(1)
    w = DCDTrajectoryFileWriter(tmp_path / "md.dcd", s, timeStep=0.0005, saveFrequency=2)
    snaps = []
    md.run(6, callback=lambda m, r: snaps.append(m.replica_coordinates(1)), trajectories=[(w, 2)], replica=1)
    w.Close()
    r = DCDTrajectoryFileReader(tmp_path / "md.dcd")
    assert len(r) == 4 and r.numberOfFixedAtoms == 3
    np.testing.assert_array_equal(r.ReadFrame(0), X0.astype(np.float32))
    for k in range(1, 4):
        np.testing.assert_array_equal(r.ReadFrame(k), snaps[2 * k - 1].astype(np.float32))
    assert not np.allclose(r.ReadFrame(3)[:len(Zq)], r.ReadFrame(0)[:len(Zq)])


def test_linear_constraints_projection_matches_oracle():
    """pdg_linear_constraints_project against the oracle's projection: velocities (weights sqrt(m)), the two deviate
    vectors (weights 1, width 2) and gradient rows of an all-atom array (weights 1/sqrt(m)); 1e-12."""
    import torch
    from pdynamo_mirror_gb300 import _native, workloads
    from pdynamo_mirror_gb300.parameters import atomic_mass
    L = _native.load()
    Z, X = workloads.water_cluster(5, seed=9)
    m = np.array([atomic_mass(z) for z in Z])
    R, n = 3, len(Z)
    rng = np.random.default_rng(4)
    Xr = X[None] + rng.normal(scale=0.1, size=(R, n, 3))
    V = np.array([D.rotation_translation_vectors(Xr[r], m) for r in range(R)])
    dV = torch.as_tensor(V, device="cuda")
    sq = torch.as_tensor(np.sqrt(m), device="cuda")
    v = rng.normal(size=(R, n, 3))
    dv = torch.as_tensor(v, device="cuda")
    _native.check(L.pdg_linear_constraints_project(R, n, n, None, 6, _native.ptr(dV), _native.ptr(sq), 1, _native.ptr(dv), _sh()), "project")
    np.testing.assert_allclose(dv.cpu().numpy(), [D.project(v[r], V[r], np.sqrt(m)) for r in range(R)], rtol=0, atol=1e-12)
    w = rng.normal(size=(R, n, 3, 2))
    dw = torch.as_tensor(w, device="cuda")
    _native.check(L.pdg_linear_constraints_project(R, n, n, None, 6, _native.ptr(dV), None, 2, _native.ptr(dw), _sh()), "project")
    for c in range(2):
        np.testing.assert_allclose(dw.cpu().numpy()[..., c], [D.project(w[r, ..., c], V[r], np.ones(n)) for r in range(R)], rtol=0, atol=1e-12)
    # rows: the free atoms are rows 2..n+1 of an array of n+3 rows
    rows = np.arange(2, n + 2)
    g = rng.normal(size=(R, n + 3, 3))
    dg = torch.as_tensor(g, device="cuda")
    drows = torch.as_tensor(rows, dtype=torch.int32, device="cuda")
    isq = 1.0 / sq
    _native.check(L.pdg_linear_constraints_project(R, n, n + 3, _native.ptr(drows), 6, _native.ptr(dV), _native.ptr(isq), 1, _native.ptr(dg),
                                                   _sh()), "project")
    ref = g.copy()
    for r in range(R):
        ref[r, rows] = D.project(g[r, rows], V[r], 1.0 / np.sqrt(m))
    np.testing.assert_allclose(dg.cpu().numpy(), ref, rtol=0, atol=1e-12)


def _free_water_box(fixed_outer, seed=4, n_qc_waters=1, n_mm_waters=6, box=10.0):
    """A hydroxide and QC waters in flexible TIP3P waters (NBModelABFS, MM model with harmonic O-H bonds and H-O-H
    angles); fixed_outer fixes the MM waters whose oxygen is farther than 4 A from the QC centre."""
    from pdynamo_mirror_gb300 import MMModel, NBModelABFS, QCModelMNDO, System, workloads
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=seed, n_qc_waters=n_qc_waters, n_mm_waters=n_mm_waters, box=box)
    s = System(Z, X, mmCharges=Q)
    s.electronicState.charge = charge
    s.DefineQCModel(QCModelMNDO("am1"), qcSelection=sel)
    s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
    s.DefineMMModel(MMModel.TIP3PWater(Z, X, flexible=True))
    if fixed_outer:
        c = X[sel].mean(0)
        far = [o for o in range(len(sel), len(Z)) if Z[o] == 8 and np.linalg.norm(X[o] - c) > 4.0]
        fixed = sorted(a for o in far for a in (o, o + 1, o + 2))
        assert 0 < len(fixed) < len(Z) - len(sel)
        s.DefineFixedAtoms(fixed)
    return s


def _oracle_system(s, x, density):
    """Oracle energy (kJ/mol) and gradients (kJ/mol/A) of every atom: QC (AM1) with ABFS QC/MM electrostatics, the
    MM model's non-bonded terms (oracle/mmmm.py) and its active harmonic terms; and the converged density."""
    from oracle import mmmm
    from pdynamo_mirror_gb300.engine import GRADIENT_TO_KJ_PER_A, HARTREES_TO_KJ
    sel, mm = list(s.qcSelection), s.mm_indices()
    Zq = [int(s.atomicNumbers[i]) for i in sel]
    nb, mod = s.nbModel, s.mmModel
    knots = O.abfs_knots(nb.innerCutoff, nb.outerCutoff)
    q = np.asarray(s.mmCharges)[mm]
    phi, _, _ = O.qcmm("abfs", x[sel], x[mm], q, knots=knots, inner=nb.innerCutoff, outer=nb.outerCutoff)
    r = O.System(O.Hamiltonian("am1", Zq), Zq, int(s.electronicState.charge)).energy(x[sel], phi=phi, density=density)
    assert r["converged"]
    _, gq, gm = O.qcmm("abfs", x[sel], x[mm], q, qcq=r["charges"], knots=knots, inner=nb.innerCutoff, outer=nb.outerCutoff)
    G = np.zeros_like(x)
    G[sel] = (r["gradients"] + gq) * GRADIENT_TO_KJ_PER_A
    G[mm] = gm * GRADIENT_TO_KJ_PER_A
    E = HARTREES_TO_KJ * (r["eelectronic"] + r["enuclear"] + r["baseline"] + r["eqcmm"])
    fixed = set(s.fixedAtoms or [])
    flags = np.where(np.isin(np.arange(len(x)), sel), mmmm.FLAG_QC_LJ, mmmm.FLAG_MM)
    flags = flags | np.where(np.isin(np.arange(len(x)), list(fixed)), mmmm.FLAG_FIXED, 0)
    lj = mod.ljParameters
    Emm, Gmm = mmmm.energies(x, mod.charges, mod.ljTypes, flags, lj.epsilon, lj.sigma, lj.epsilon, lj.sigma, True, mod.exclusions,
                             mod.interactions14, nb.innerCutoff, nb.outerCutoff, nb.dampingCutoff)
    qcs = set(sel)

    def active(t):
        return not (all(a in qcs for a in t) or all(a in fixed for a in t))
    kb = [k for k in range(len(mod.bonds)) if active(mod.bonds[k].tolist())]
    ka = [k for k in range(len(mod.angles)) if active(mod.angles[k].tolist())]
    eb, ea, Gh = mmmm.harmonic_terms(x, mod.bonds[kb], mod.bondParameters[kb], mod.angles[ka], mod.angleParameters[ka])
    return E + Emm.sum() + eb + ea, G + Gmm + Gh, r["density"]


@pytest.mark.parametrize("fixed_outer", [False, True], ids=["all_free", "outer_fixed"])
def test_free_mm_water_trajectory_matches_oracle(fixed_outer):
    """Four Langevin steps of two replicas of a hydroxide and a QC water among six flexible TIP3P waters whose atoms
    move: the MM model's LJ, electrostatic and harmonic forces and the QC/MM forces on the MM atoms drive them.
    With no atom fixed, rotation and translation are removed: the velocities carry no momentum, the applied
    deviates are the projected counter-based deviates, and the gradients are projected as the oracle does.
    Coordinates within 1e-8 A and velocities within 1e-5 A/ps of the oracle's integrator step by step, the
    potential energy within 1e-5 kJ/mol of the oracle's."""
    import torch
    from pdynamo_mirror_gb300 import LangevinDynamics
    from pdynamo_mirror_gb300.parameters import atomic_mass
    s = _free_water_box(fixed_outer)
    R = 2
    md = LangevinDynamics(s, replicas=R, timeStep=0.0005, temperature=300.0, collisionFrequency=25.0, seed=17)
    free = md.free
    m = np.array([atomic_mass(s.atomicNumbers[i]) for i in free])
    allm = np.array([atomic_mass(z) for z in s.atomicNumbers])
    c = md.integrator.constants
    X = md.X.cpu().numpy().copy()
    v = md.vel.cpu().numpy().copy()
    V = None if fixed_outer else [D.rotation_translation_vectors(X[r], allm) for r in range(R)]
    assert md.n_constraints == (0 if fixed_outer else 6) and md.dof == 3 * len(free) - md.n_constraints
    for r in range(R):
        assert math.isclose(D.temperature(v[r], m, md.dof)[1], 300.0, rel_tol=1e-12)
        if V is not None:
            np.testing.assert_allclose((m[:, None] * v[r]).sum(0), 0.0, atol=1e-10)

    def accel(r, dens):
        E, G, P = _oracle_system(s, X[r], dens)
        g = G[free]
        if V is not None:
            g = D.project(g, V[r], 1.0 / np.sqrt(m))
        return -100.0 * g / m[:, None], P, E

    md.initialize()
    acc, dens, pot = [None] * R, [None] * R, [None] * R
    for r in range(R):
        acc[r], dens[r], pot[r] = accel(r, None)
    np.testing.assert_allclose(md.acc.cpu().numpy(), np.array(acc), rtol=0, atol=2e-3)
    np.testing.assert_allclose(md.potential_energies(), pot, rtol=0, atol=1e-5)
    dev = torch.empty((R, len(free), 3, 2), dtype=torch.float64, device="cuda")
    for step in range(1, 5):
        md.step(deviates=dev)
        w = dev.cpu().numpy()
        if V is not None:
            raw = D.normal_pairs(R * len(free) * 3, 17, step).reshape(R, len(free), 3, 2)
            for r in range(R):
                for k in range(2):
                    np.testing.assert_allclose(w[r, ..., k], D.project(raw[r, ..., k], V[r], np.ones(len(free))), rtol=0, atol=1e-12)
        for r in range(R):
            xf, v[r] = D.positions(X[r][free], v[r], acc[r], m, c, w[r, ..., 0], w[r, ..., 1])
            X[r][free] = xf
            acc[r], dens[r], pot[r] = accel(r, dens[r])
            v[r], _ = D.velocities(v[r], -acc[r] * m[:, None] / 100.0, m, c)
        np.testing.assert_allclose(md.X.cpu().numpy(), X, rtol=0, atol=1e-8)
        np.testing.assert_allclose(md.vel.cpu().numpy(), v, rtol=0, atol=1e-5)
        np.testing.assert_allclose(md.potential_energies(), pot, rtol=0, atol=1e-5)
    if fixed_outer:
        fx = list(s.fixedAtoms)
        np.testing.assert_array_equal(md.X.cpu().numpy()[:, fx], np.broadcast_to(s.coordinates3[fx], (R, len(fx), 3)))


def _nve(dt, steps):
    from pdynamo_mirror_gb300 import LangevinDynamics
    from pdynamo_mirror_gb300.parameters import atomic_mass
    s = _free_water_box(False, seed=6, n_qc_waters=2, n_mm_waters=30, box=14.0)
    md = LangevinDynamics(s, replicas=4, timeStep=dt, temperature=300.0, collisionFrequency=1.0e-4, seed=23)
    allm = np.array([atomic_mass(z) for z in s.atomicNumbers])
    com0 = np.einsum("i,rij->rj", allm, md.X.cpu().numpy()) / allm.sum()
    md.initialize()
    tot, kin = [md.total_energies()], [md.temperatures()[0]]
    for _ in range(steps):
        md.step(random=False)
        tot.append(md.total_energies())
        kin.append(md.temperatures()[0])
    com = np.einsum("i,rij->rj", allm, md.X.cpu().numpy()) / allm.sum()
    return np.array(tot), np.array(kin), com - com0


def test_free_water_box_conserves_energy_without_a_bath():
    """NVE: a hydroxide and two QC waters among 30 flexible TIP3P waters, nothing fixed, no random forces and a
    collision frequency of 1e-4 ps^-1 (velocity Verlet), 0.1 ps in 4 replicas from an unrelaxed start whose kinetic
    energy then swings by more than 500 kJ/mol.  At 0.25 fs steps the total energy (potential + kinetic) stays
    within 1 kJ/mol (below 2e-3 of the kinetic swing) of its start in every replica and drifts by less than
    1 kJ/mol/ps; at 0.125 fs the largest deviation is at least 3x smaller (velocity Verlet's dt^2 error: the
    forces are the energy's gradients).  The centre of mass stays put (translation removed)."""
    res = {}
    for dt, steps in ((0.00025, 400), (0.000125, 800)):
        tot, kin, dcom = _nve(dt, steps)
        dev = np.abs(tot - tot[0]).max(0)
        slope = np.polyfit(np.arange(len(tot)) * dt, tot, 1)[0]
        swing = kin.max(0) - kin.min(0)
        print("NVE dt %.3f fs: max |E - E0| (kJ/mol) %s, drift (kJ/mol/ps) %s, kinetic swing %s" % (1e3 * dt, dev, slope, swing))
        res[dt] = dev
        np.testing.assert_allclose(dcom, 0.0, rtol=0, atol=1e-8)
        assert (swing > 100.0).all()
        assert (dev < 1.0).all() and (dev < 2e-3 * swing).all()
        assert (np.abs(slope) < 1.0).all()
    assert (res[0.000125] * 3.0 < res[0.00025]).all()
