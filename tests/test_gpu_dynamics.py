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
