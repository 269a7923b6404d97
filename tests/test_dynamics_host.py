"""Langevin dynamics, host side (no GPU): the oracle's counter-based generator against the published
Philox4x32-10 known-answer vectors, the integration constants against the oracle's restatement of
LangevinVelocityVerletIntegrator.CalculateIntegrationConstants in both of its branches, and the argument checks
of the dynamics surface."""
import math

import numpy as np
import pytest

from oracle import dynamics as D
from pdynamo_mirror_gb300 import LangevinDynamics, LangevinVelocityVerletIntegrator, NBModelFull, QCModelMNDO, System, workloads
from pdynamo_mirror_gb300.parameters import atomic_mass

# Philox4x32-10 known-answer vectors published with the generator (Salmon et al., SC 2011; Random123 kat_vectors):
# (counter, key) -> output, all 32-bit words.
PHILOX_KAT = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
              ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
              ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
               (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]


@pytest.mark.parametrize("ctr,key,expected", PHILOX_KAT)
def test_oracle_philox_matches_published_vectors(ctr, key, expected):
    out = D.philox4x32_10(np.array([ctr], dtype=np.uint64), key)[0]
    assert tuple(int(x) for x in out) == expected


def test_oracle_normal_pairs_are_standard_normal():
    w = D.normal_pairs(400000, seed=2024, step=3)
    assert np.all(np.abs(w.mean(0)) < 5e-3)
    assert np.all(np.abs(w.std(0) - 1.0) < 5e-3)
    assert abs(np.corrcoef(w[:, 0], w[:, 1])[0, 1]) < 5e-3
    # different steps and streams give different deviates
    assert not np.allclose(w[:100], D.normal_pairs(100, 2024, 4))
    assert not np.allclose(w[:100], D.normal_pairs(100, 2024, 3, stream=1))


@pytest.mark.parametrize("gamma,dt", [(25.0, 0.0005), (25.0, 0.001), (1.0, 0.001), (5.0, 0.0005), (0.5, 0.002)])
def test_integration_constants_match_oracle(gamma, dt):
    a = LangevinVelocityVerletIntegrator(gamma, 300.0, dt).constants
    b = D.integration_constants(gamma, dt, 300.0)
    for k in b:
        assert abs(a[k] - b[k]) <= 1e-14 * abs(b[k]), k


def test_integration_constant_branches_agree_at_the_switch():
    """Series (gamma dt <= 0.009) and exponential forms give the same constants on either side of the switch."""
    lo = LangevinVelocityVerletIntegrator(9.0, 300.0, 0.000999999).constants
    hi = LangevinVelocityVerletIntegrator(9.0, 300.0, 0.001000001).constants
    for k in lo:
        assert abs(lo[k] - hi[k]) <= 1e-5 * abs(hi[k]), k


def test_integration_constants_limits():
    """gamma -> 0: velocity Verlet (facR1 = dt, facR2 = dt^2/2, facV1 = 1, facV2 = facV3 = dt/2, no noise)."""
    c = LangevinVelocityVerletIntegrator(1e-6, 300.0, 0.001).constants
    assert math.isclose(c["facR1"], 0.001, rel_tol=1e-8) and math.isclose(c["facR2"], 0.5e-6, rel_tol=1e-8)
    assert math.isclose(c["facV2"], 0.0005, rel_tol=1e-8) and math.isclose(c["facV3"], 0.0005, rel_tol=1e-8)
    assert c["sdR"] < 1e-6 and c["sdV1"] < 1e-3


def test_integrator_option_errors():
    with pytest.raises(ValueError):
        LangevinVelocityVerletIntegrator(collisionFrequency=0.0)
    with pytest.raises(ValueError):
        LangevinVelocityVerletIntegrator(temperature=-1.0)


def test_masses_are_pdynamos():
    assert atomic_mass(1) == 1.00794 and atomic_mass(8) == 15.9994 and atomic_mass(6) == 12.011
    with pytest.raises(ValueError):
        atomic_mass(0)


def test_dynamics_needs_free_atoms():
    Z, X = workloads.water_cluster(2, seed=1)
    s = System(Z, X)
    s.DefineQCModel(QCModelMNDO("am1"))
    s.DefineFixedAtoms(range(len(Z)))
    with pytest.raises(ValueError, match="No free atoms"):
        LangevinDynamics(s)
    s.DefineFixedAtoms(None)
    with pytest.raises(ValueError, match="densityGuess"):
        LangevinDynamics(s, densityGuess="guess")


def test_rotation_translation_vectors_match_oracle():
    """The host vectors against the oracle's restatement of Coordinates3_RotationTranslationVectors: six for a bent
    molecule, five for a linear one, three for one atom; orthonormal; and projecting them out of a velocity field
    leaves no linear or angular momentum."""
    from pdynamo_mirror_gb300.dynamics import rotation_translation_vectors
    from pdynamo_mirror_gb300.parameters import atomic_mass
    Z, X = workloads.water_cluster(3, seed=2)
    m = np.array([atomic_mass(z) for z in Z])
    V = rotation_translation_vectors(X, m)
    Vo = D.rotation_translation_vectors(X, m)
    assert V.shape == (6, len(Z), 3)
    np.testing.assert_allclose(V, Vo, rtol=0, atol=1e-12)
    F = V.reshape(6, -1)
    np.testing.assert_allclose(F @ F.T, np.eye(6), rtol=0, atol=1e-12)
    v = np.random.default_rng(0).normal(size=X.shape)
    vp = D.project(v, V, np.sqrt(m))
    c = X - np.average(X, axis=0, weights=m)
    np.testing.assert_allclose((m[:, None] * vp).sum(0), 0.0, atol=1e-12)
    np.testing.assert_allclose((m[:, None] * np.cross(c, vp)).sum(0), 0.0, atol=1e-11)
    lin = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 1.16], [0.0, 0.0, -1.16]])
    ml = np.array([12.011, 15.9994, 15.9994])
    assert rotation_translation_vectors(lin, ml).shape == (5, 3, 3)
    np.testing.assert_allclose(rotation_translation_vectors(lin, ml), D.rotation_translation_vectors(lin, ml), atol=1e-12)
    assert rotation_translation_vectors(np.zeros((1, 3)), [1.00794]).shape == (3, 1, 3)


def test_oracle_velocity_assignment_hits_the_temperature():
    m = np.array([15.9994, 1.00794, 1.00794] * 5)
    v = D.assign_velocities(m, 300.0, np.random.default_rng(0))
    assert math.isclose(D.temperature(v, m, 3 * len(m))[1], 300.0, rel_tol=1e-12)
