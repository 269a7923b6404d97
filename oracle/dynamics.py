"""Oracle (test infrastructure only): numpy restatement of pDynamo's Langevin velocity Verlet step and of the
counter-based normal generator the GPU integrator draws its random forces from.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module; the product never imports it.

* integration_constants  LangevinVelocityVerletIntegrator.CalculateIntegrationConstants
                         (pCore-1.9.0/pCore/LangevinVelocityVerletIntegrator.py:63-112), both branches.
* positions / velocities LangevinVelocityVerletIntegrator.Iteration and RandomForces (:126-157), written for
                         unweighted Cartesian variables (the reference's mass-weighted x_w = sqrt(m) x, divided
                         through by sqrt(m)); accelerations a = -100 g / m (SystemGeometryObjectiveFunction.py:57-66).
* temperature            SystemGeometryObjectiveFunction.Temperature (:255-260).
* philox4x32_10, normals Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC 2011) and the Box-Muller pair the GPU
                         kernels form from it; pinned by the published known-answer vectors in tests.
"""

import math

import numpy as np

# pCore-1.9.0/pCore/Units.py:15,17 and SystemGeometryObjectiveFunction.py:19-28
CONSTANT_ATOMIC_MASS = 1.66053886e-27
CONSTANT_BOLTZMANN = 1.3806505e-23
MS_TO_APS = 1.0e-2
AMUA2PS2_TO_K = CONSTANT_ATOMIC_MASS / (CONSTANT_BOLTZMANN * MS_TO_APS ** 2)
AMUA2PS2_TO_KJMOL = 1.0e-2
KJMOL_TO_AMUA2PS2 = 1.0e+2


def integration_constants(collision_frequency, time_step, temperature):
    """(facR1, facR2, facV1, facV2, facV3, sdR, sdV1, sdV2) as CalculateIntegrationConstants leaves them."""
    fact = collision_frequency * time_step
    if fact > 0.009:
        c0 = math.exp(-fact)
        c1 = (1.0 - c0) / fact
        c2 = (1.0 - c1) / fact
        sdR = math.sqrt(time_step ** 2 * (2.0 - (3.0 - 4.0 * c0 + c0 * c0) / fact) / fact)
        sdV = math.sqrt(1.0 - c0 * c0)
        cRV1 = time_step * (1.0 - c0) ** 2 / (fact * sdR * sdV)
        cRV2 = math.sqrt(1.0 - cRV1 * cRV1)
    else:
        f = fact
        c0 = 1.0 - f + f ** 2 / 2.0 - f ** 3 / 6.0 + f ** 4 / 24.0 - f ** 5 / 120.0
        c1 = 1.0 - f / 2.0 + f ** 2 / 6.0 - f ** 3 / 24.0 + f ** 4 / 120.0 - f ** 5 / 720.0
        c2 = 0.5 - f / 6.0 + f ** 2 / 24.0 - f ** 3 / 120.0 + f ** 4 / 720.0 - f ** 5 / 5040.0
        sdR = (2.0 - 3.0 * f / 4.0 + 67.0 * f ** 2 / 320.0 - 119.0 * f ** 3 / 2560.0) * math.sqrt(f / 6.0) * time_step
        sdV = (2.0 - f + 5.0 * f ** 2 / 12.0 - f ** 3 / 8.0 + 79.0 * f ** 4 / 2880.0) * math.sqrt(f / 2.0)
        cRV1 = (3.0 / 2.0 - 3.0 * f / 16.0 - 51.0 * f ** 2 / 1280.0 + 17.0 * f ** 3 / 2048.0 + 40967.0 * f ** 4 / 11468800.0
                - 57203.0 * f ** 5 / 91750400.0) / math.sqrt(3.0)
        cRV2 = (0.5 + 3.0 * f / 16.0 - 9.0 * f ** 2 / 1280.0 - 109.0 * f ** 3 / 10240.0 + 10077.0 * f ** 4 / 11468800.0
                + 14887.0 * f ** 5 / 18350080.0)
    t = math.sqrt(temperature / AMUA2PS2_TO_K)
    return dict(facR1=c1 * time_step, facR2=c2 * time_step ** 2, facV1=c0, facV2=(c1 - c2) * time_step, facV3=c2 * time_step,
                sdR=sdR * t, sdV1=cRV1 * sdV * t, sdV2=cRV2 * sdV * t)


M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(counter, key):
    """Vectorised Philox4x32-10: counter uint64 array [..., 4] of 32-bit words, key [2] -> four words."""
    c = [np.asarray(counter[..., i], dtype=np.uint64) & MASK for i in range(4)]
    k0 = np.uint64(key[0] & MASK)
    k1 = np.uint64(key[1] & MASK)
    for _ in range(10):
        p0 = np.uint64(M0) * c[0]
        p1 = np.uint64(M1) * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & np.uint64(MASK)
        hi1, lo1 = p1 >> np.uint64(32), p1 & np.uint64(MASK)
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
        k0 = (k0 + np.uint64(W0)) & np.uint64(MASK)
        k1 = (k1 + np.uint64(W1)) & np.uint64(MASK)
    return np.stack(c, axis=-1)


def normal_pairs(n_pairs, seed, step, stream=0):
    """(w1, w2) for pair indices 0..n_pairs-1, as the GPU generator forms them: [n_pairs, 2]."""
    g = np.arange(n_pairs, dtype=np.uint64)
    ctr = np.stack([g & np.uint64(MASK), g >> np.uint64(32), np.full_like(g, step), np.full_like(g, stream)], axis=-1)
    r = philox4x32_10(ctr, (seed & MASK, (seed >> 32) & MASK))
    u1 = (((r[:, 0] >> np.uint64(6)) << np.uint64(27)) | (r[:, 1] >> np.uint64(5))).astype(np.float64) * 2.0 ** -53
    u2 = (((r[:, 2] >> np.uint64(6)) << np.uint64(27)) | (r[:, 3] >> np.uint64(5))).astype(np.float64) * 2.0 ** -53
    rad = np.sqrt(-2.0 * np.log(1.0 - u1))
    return np.stack([rad * np.cos(2.0 * np.pi * u2), rad * np.sin(2.0 * np.pi * u2)], axis=-1)


def positions(x, v, a, masses, c, w1=None, w2=None):
    """First half of Iteration (:129-137) and RandomForces (:147-157); x [n, 3] A, v A/ps, a A/ps^2, masses amu.
    Returns new (x, v)."""
    s = 1.0 / np.sqrt(masses)[:, None]
    x = x + c["facR1"] * v + c["facR2"] * a
    v = c["facV1"] * v + c["facV2"] * a
    if w1 is not None:
        x = x + c["sdR"] * w1 * s
        v = v + c["sdV1"] * w1 * s
        v = v + c["sdV2"] * w2 * s
    return x, v


def velocities(v, gradients_kj_per_a, masses, c):
    """Second half (:139-144): a = -100 g / m, v += facV3 a.  Returns (v, a)."""
    a = -KJMOL_TO_AMUA2PS2 * gradients_kj_per_a / masses[:, None]
    return v + c["facV3"] * a, a


def temperature(v, masses, degrees_of_freedom):
    """(kinetic energy kJ/mol, temperature K) of unweighted velocities."""
    ke = float((masses[:, None] * v * v).sum())
    return 0.5 * AMUA2PS2_TO_KJMOL * ke, AMUA2PS2_TO_K * ke / float(degrees_of_freedom)


def assign_velocities(masses, temperature_k, rng):
    """VelocitiesAssign (SystemGeometryObjectiveFunction.py:317-345) for unweighted velocities: Gaussian weighted
    velocities of width sigma, then scaled to the exact temperature."""
    sigma = MS_TO_APS * math.sqrt(CONSTANT_BOLTZMANN * temperature_k / CONSTANT_ATOMIC_MASS)
    v = rng.standard_normal((len(masses), 3)) * sigma / np.sqrt(masses)[:, None]
    _, t = temperature(v, masses, 3 * len(masses))
    return v * math.sqrt(temperature_k / t)


def rotation_translation_vectors(x, masses):
    """Mass-weighted rotation and translation vectors (Coordinates3_RotationTranslationVectors,
    pCore-1.9.0/extensions/csource/Coordinates3.c:1315-1385, weights = masses): columns Tx, Ty, Tz, Rx, Ry, Rz of a
    3n x 6 matrix, sqrt(m) weights and rotations about the centre of mass, orthonormalised by one Gram-Schmidt pass
    that drops columns whose norm falls to 1e-10 sqrt(3n) or below (Real2DArray.c:487-545).  Returns [K, n, 3]."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, 3)
    m = np.asarray(masses, dtype=np.float64)
    n = len(m)
    sw = np.sqrt(m)
    c = x - np.average(x, axis=0, weights=m)
    M = np.zeros((3 * n, 6))
    for a in range(3):
        M[a::3, a] = sw
    # rotation about axis a: sqrt(m) (e_a x (x - c))
    for a in range(3):
        e = np.zeros(3); e[a] = 1.0
        M[:, 3 + a] = (sw[:, None] * np.cross(e, c)).ravel()
    kept = []
    for col in range(6):
        v = M[:, col].copy()
        for u in kept:
            v = v - np.dot(v, u) * u
        if np.linalg.norm(v) > 1.0e-10 * math.sqrt(3 * n):
            kept.append(v / np.linalg.norm(v))
    return np.array(kept).reshape(-1, n, 3)


def project(a, vectors, weights):
    """Removes the vectors (orthonormal in the weighted space) from a [n, 3] whose weighted form is weights[:, None] a
    (ProjectOutOfArray on the objective function's mass-weighted variables)."""
    aw = (np.asarray(weights, dtype=np.float64)[:, None] * a).ravel()
    V = np.asarray(vectors, dtype=np.float64).reshape(len(vectors), -1)
    aw = aw - V.T @ (V @ aw)
    return aw.reshape(-1, 3) / np.asarray(weights, dtype=np.float64)[:, None]
