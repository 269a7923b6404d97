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


def test_dynamics_requires_fixed_mm_atoms():
    Z, X = workloads.water_cluster(2, seed=1)
    allZ = np.concatenate([Z, [8, 1, 1]])
    allX = np.concatenate([X, X[:3] + 6.0])
    s = System(allZ, allX, mmCharges=[0.0] * len(Z) + [workloads.TIP3P_O, workloads.TIP3P_H, workloads.TIP3P_H])
    s.DefineQCModel(QCModelMNDO("am1"), qcSelection=range(len(Z)))
    s.DefineNBModel(NBModelFull())
    with pytest.raises(ValueError):
        LangevinDynamics(s)
    with pytest.raises(ValueError):
        s.DefineFixedAtoms([len(allZ)])
    # an MM model's LJ terms are not in the dynamics driver: refused rather than left out
    from pdynamo_mirror_gb300 import MMModel
    s.DefineFixedAtoms(range(len(Z), len(allZ)))
    s.DefineMMModel(MMModel.TIP3PWater(allZ, allX))
    with pytest.raises(ValueError, match="LJ"):
        LangevinDynamics(s)


def test_oracle_velocity_assignment_hits_the_temperature():
    m = np.array([15.9994, 1.00794, 1.00794] * 5)
    v = D.assign_velocities(m, 300.0, np.random.default_rng(0))
    assert math.isclose(D.temperature(v, m, 3 * len(m))[1], 300.0, rel_tol=1e-12)
