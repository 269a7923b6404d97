"""Oracle (test infrastructure only): numpy restatement of NBModelABFS's MM/MM and QC/MM Lennard-Jones energies.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module; the product never imports it.
Brute force over every atom pair (small systems only), with the selections of the reference's pair lists:

* lj_tables       LJParameterContainer_MakeTable (pMolecule-1.9.0/extensions/csource/LJParameterContainer.c:185-210):
                  OPLS  A = 4 e s^12, B = 4 e s^6 with s = sqrt(s_i s_j);  AMBER  A = e s^12, B = 2 e s^6 with
                  s = (s_i + s_j) / 2;  e = sqrt(e_i e_j).
* abfs_factors    PairwiseInteractionABFS_MakeFactors (PairwiseInteraction.c:89-140).
* pair_terms      PairwiseInteractionABFS_CheckDistances / _ElectrostaticTerm / _LennardJonesTerm
                  (cinclude/PairwiseInteraction.h:72-120): damped below the damping cutoff, plain between it and the
                  inner cutoff, force-switched up to the outer cutoff; dF is the derivative with respect to r^2.
* energies        NBModelABFS_MMMMEnergy / _QCMMEnergyLJ (NBModelABFS.c:228-330) over the lists of GenerateLists and
                  GenerateLists14 (:1050-1160): MM/MM pairs of active MM atoms, not excluded, at least one atom free;
                  1-4 pairs from the 1-4 list with electrostaticScale14 and the 1-4 LJ tables; QC/MM LJ pairs of a QC
                  atom with LJ interactions and an MM atom (LJ only).  The pair lists' list cutoff only bounds the
                  search: every pair within the outer cutoff is evaluated, as here.

Energies in kJ/mol, gradients in kJ/mol/A, coordinates in A.
"""

import math

import numpy as np

# pCore-1.9.0/extensions/cinclude/Units.h:18-49
CONSTANT_AVOGADRO_NUMBER = 6.0221415e+23
CONSTANT_ELECTRON_CHARGE = 1.60217653e-19
CONSTANT_VACUUM_PERMITTIVITY = 8.854187817e-12
E2ANGSTROMS_TO_KJMOL = (1.0e+7 * CONSTANT_AVOGADRO_NUMBER * CONSTANT_ELECTRON_CHARGE ** 2) / (4.0 * math.pi * CONSTANT_VACUUM_PERMITTIVITY)

FLAG_MM, FLAG_QC_LJ, FLAG_FIXED = 1, 2, 4
TERMS = ("MM/MM Elect.", "MM/MM LJ", "MM/MM 1-4 Elect.", "MM/MM 1-4 LJ", "QC/MM LJ", "QC/MM 1-4 LJ")


def lj_tables(epsilon, sigma, opls=True):
    """Full (types x types) A and B tables."""
    e = np.sqrt(np.outer(epsilon, epsilon))
    s = np.sqrt(np.outer(sigma, sigma)) if opls else 0.5 * (np.add.outer(sigma, sigma))
    s6 = s ** 6
    s12 = s6 * s6
    if opls:
        e = 4.0 * e
    else:
        s6 = 2.0 * s6
    return e * s12, e * s6


def abfs_factors(inner, outer, damp):
    f = {}
    f["r2Damp"], f["r2Off"], f["r2On"] = damp * damp, outer * outer, inner * inner
    r2Off, r2On = f["r2Off"], f["r2On"]
    gamma = (r2Off - r2On) ** 3
    f["a"] = r2Off * r2Off * (r2Off - 3.0 * r2On) / gamma
    f["b"] = 6.0 * r2Off * r2On / gamma
    f["c"] = -(r2Off + r2On) / gamma
    f["d"] = 0.4 / gamma
    f["qShift1"] = 8.0 * (r2Off * r2On * (outer - inner) - 0.2 * (outer * r2Off * r2Off - inner * r2On * r2On)) / gamma
    f["qShift2"] = -(f["a"] / outer) + f["b"] * outer + f["c"] * outer * r2Off + f["d"] * outer * r2Off * r2Off
    g = -1.0 / f["r2Damp"] if damp > 0.0 else 0.0
    fq = (1.0 / damp + f["qShift1"]) if damp > 0.0 else 0.0
    f["qF0"] = fq - 0.5 * damp * g
    f["qAlpha"] = -0.5 * g / damp if damp > 0.0 else 0.0
    f["aF6"] = 1.0 / (r2Off ** 3)
    f["aK12"] = r2Off ** 3 / (r2Off ** 3 - r2On ** 3)
    f["aShift12"] = 1.0 / (inner * outer) ** 6
    if damp > 0.0:
        s12 = 1.0 / damp ** 12
        fa, ga = s12 - f["aShift12"], -12.0 * s12 / damp
        f["aF0"], f["aAlpha"] = fa - 0.5 * damp * ga, -0.5 * ga / damp
    else:
        f["aF0"] = f["aAlpha"] = 0.0
    f["bF3"] = 1.0 / (outer * r2Off)
    f["bK6"] = (outer * r2Off) / (outer * r2Off - inner * r2On)
    f["bShift6"] = 1.0 / (inner * outer) ** 3
    if damp > 0.0:
        s6 = 1.0 / damp ** 6
        fb, gb = -s6 + f["bShift6"], 6.0 * s6 / damp
        f["bF0"], f["bAlpha"] = fb - 0.5 * damp * gb, -0.5 * gb / damp
    else:
        f["bF0"] = f["bAlpha"] = 0.0
    return f


def pair_terms(f, r2, qij, A, B):
    """(electrostatic energy, LJ energy, dF) for arrays of pairs inside the outer cutoff."""
    r2 = np.asarray(r2, float)
    damped = r2 < f["r2Damp"]
    s2 = np.where(damped, 0.0, 1.0 / np.where(damped, 1.0, r2))
    s = np.sqrt(s2)
    on, mid = r2 > f["r2On"], (r2 <= f["r2On"]) & ~damped
    fe = np.where(on, qij * (s * (f["a"] - r2 * (f["b"] + r2 * (f["c"] + f["d"] * r2))) + f["qShift2"]),
                  np.where(mid, qij * (s + f["qShift1"]), qij * (f["qF0"] - f["qAlpha"] * r2)))
    de = np.where(on, -qij * 0.5 * s * (f["a"] + r2 * (f["b"] + r2 * (3.0 * f["c"] + 5.0 * f["d"] * r2))) / r2,
                  np.where(mid, -qij * 0.5 * s / r2, -qij * f["qAlpha"]))
    s6 = s2 * s2 * s2
    l1, l2 = s6 - f["aF6"], np.where(on, s / r2, 0.0) - f["bF3"]
    fl = np.where(on, A * f["aK12"] * l1 ** 2 - B * f["bK6"] * l2 ** 2,
                  np.where(mid, A * (s6 * s6 - f["aShift12"]) - B * (s6 - f["bShift6"]),
                           A * (f["aF0"] - f["aAlpha"] * r2) - B * (f["bF0"] - f["bAlpha"] * r2)))
    safe_s = np.where(s > 0.0, s, 1.0)
    dl = np.where(on, -3.0 * s6 * (2.0 * A * f["aK12"] * l1 / r2 - B * f["bK6"] * l2 / safe_s),
                  np.where(mid, -3.0 * s6 * (2.0 * A * s6 - B) / r2, -A * f["aAlpha"] + B * f["bAlpha"]))
    return fe, fl, de + dl, de, dl


def energies(xyz, charges, lj_types, flags, epsilon, sigma, epsilon14, sigma14, opls, exclusions, pairs14,
             inner=8.0, outer=12.0, damp=0.5, dielectric=1.0, scale14=1.0):
    """Returns (energies [6] in the order of TERMS, gradients [n, 3])."""
    X = np.asarray(xyz, float).reshape(-1, 3)
    n = len(X)
    q = np.asarray(charges, float)
    t = np.asarray(lj_types, int)
    fl = np.asarray(flags, int)
    mm, qcp, free = (fl & FLAG_MM) != 0, (fl & FLAG_QC_LJ) != 0, (fl & FLAG_FIXED) == 0
    A, B = lj_tables(np.asarray(epsilon, float), np.asarray(sigma, float), opls)
    A14, B14 = lj_tables(np.asarray(epsilon14, float), np.asarray(sigma14, float), opls)
    fac = abfs_factors(inner, outer, damp)
    escale = E2ANGSTROMS_TO_KJMOL / dielectric
    excl = np.zeros((n, n), bool)
    for i, j in np.asarray(exclusions, int).reshape(-1, 2):
        excl[i, j] = excl[j, i] = True
    E = np.zeros(6)
    G = np.zeros((n, 3))
    iu, ju = np.triu_indices(n, 1)

    def add(i, j, qq, AA, BB, k_el, k_lj, with_el):
        d = X[i] - X[j]
        r2 = (d * d).sum(1)
        keep = r2 <= fac["r2Off"]
        i, j, d, r2, qq, AA, BB = i[keep], j[keep], d[keep], r2[keep], qq[keep], AA[keep], BB[keep]
        fe, flj, dF, de, dl = pair_terms(fac, r2, qq, AA, BB)
        if with_el:
            E[k_el] += fe.sum()
        else:
            dF = dl
        E[k_lj] += flj.sum()
        gv = 2.0 * dF[:, None] * d
        np.add.at(G, i, gv)
        np.add.at(G, j, -gv)

    either_free = free[iu] | free[ju]
    sel = mm[iu] & mm[ju] & ~excl[iu, ju] & either_free
    i, j = iu[sel], ju[sel]
    add(i, j, escale * q[i] * q[j], A[t[i], t[j]], B[t[i], t[j]], 0, 1, True)
    sel = ((qcp[iu] & mm[ju]) | (mm[iu] & qcp[ju])) & ~excl[iu, ju] & either_free
    i, j = iu[sel], ju[sel]
    add(i, j, np.zeros(len(i)), A[t[i], t[j]], B[t[i], t[j]], 0, 4, False)
    p14 = np.asarray(pairs14, int).reshape(-1, 2)
    if len(p14):
        i, j = p14[:, 0], p14[:, 1]
        f2 = free[i] | free[j]
        s = mm[i] & mm[j] & f2
        add(i[s], j[s], escale * scale14 * q[i[s]] * q[j[s]], A14[t[i[s]], t[j[s]]], B14[t[i[s]], t[j[s]]], 2, 3, True)
        s = ((qcp[i] & mm[j]) | (mm[i] & qcp[j])) & f2
        add(i[s], j[s], np.zeros(int(s.sum())), A14[t[i[s]], t[j[s]]], B14[t[i[s]], t[j[s]]], 2, 5, False)
    return E, G


def harmonic_terms(X, bonds, bond_params, angles, angle_params):
    """Harmonic bonds and angles, as HarmonicBondContainer_Energy (pMolecule-1.9.0/extensions/csource/
    HarmonicBondContainer.c:149-181: E = k (r - r0)^2) and HarmonicAngleContainer_Energy (HarmonicAngleContainer.c:157-200:
    E = k (theta - theta0)^2 at the middle atom, cosine clamped to +-0.999999).  X [n, 3] (A); bonds [nb, 2] with
    (r0, k); angles [na, 3] with (theta0 rad, k).  Returns (E_bond, E_angle) in kJ/mol and the gradients [n, 3]."""
    X = np.asarray(X, dtype=np.float64)
    G = np.zeros_like(X)
    eb = ea = 0.0
    for (i, j), (r0, k) in zip(np.asarray(bonds, dtype=np.int64).reshape(-1, 2), np.asarray(bond_params, dtype=np.float64).reshape(-1, 2)):
        d = X[i] - X[j]
        r = np.sqrt(d @ d)
        df = k * (r - r0)
        eb += df * (r - r0)
        g = (2.0 * df / r) * d
        G[i] += g; G[j] -= g
    for (i, j, l), (t0, k) in zip(np.asarray(angles, dtype=np.int64).reshape(-1, 3), np.asarray(angle_params, dtype=np.float64).reshape(-1, 2)):
        a, c = X[i] - X[j], X[l] - X[j]
        ra, rc = np.sqrt(a @ a), np.sqrt(c @ c)
        a, c = a / ra, c / rc
        dot = min(0.999999, max(-0.999999, a @ c))
        theta = np.arccos(dot)
        df = k * (theta - t0)
        ea += df * (theta - t0)
        d2 = 2.0 * df * (-1.0 / np.sqrt(1.0 - dot * dot))
        gi, gk = d2 * (c - dot * a) / ra, d2 * (a - dot * c) / rc
        G[i] += gi; G[l] += gk; G[j] -= gi + gk
    return eb, ea, G
