"""Generate tests/golden/mmmm_reference.json: NBModelABFS MM/MM and QC/MM Lennard-Jones energies and gradients
computed by the pDynamo 1.9.0 reference core (pair-list generator with its cell grid, PairwiseInteractionABFS_MMMMEnergy
in analytic form), through ``ref_mmmm_energy`` of oracle/ref_shim.c.

Run where the reference tree and the compiled reference core exist (``make -C oracle ref``):

    python tests/golden/make_mmmm_golden.py

Cases (seeded water boxes: TIP3P charges and oxygen LJ parameters, exclusions within each molecule):
  opls_free   OPLS combining rule, no fixed atoms, a few 1-4 pairs (MM/MM and QC/MM) with halved 1-4 epsilon;
  amber_fixed AMBER combining rule, most MM waters fixed (pairs of two fixed atoms are left out), dielectric 2,
              electrostaticScale14 0.5.
"""

import json, os, sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import refdriver as R  # noqa: E402
from pdynamo_mirror_gb300 import workloads  # noqa: E402

# TIP3P oxygen (Jorgensen et al. 1983): epsilon 0.1521 kcal/mol, sigma 3.15061 A; hydrogens carry no LJ term
EPSILON = [0.1521 * 4.184, 0.0]
SIGMA = [3.15061, 0.0]


def water_case(seed, n_qc_waters, n_mm_waters, box):
    Z, X, Q, sel, _ = workloads.qcmm_water_box(seed=seed, n_qc_waters=n_qc_waters, n_mm_waters=n_mm_waters, box=box)
    n = len(Z)
    types = np.where(Z == 8, 0, 1)
    flags = np.where(np.arange(n) < len(sel), 2, 1)
    excl, i = [], 0
    while i < n:   # molecules are O, H, H (the hydroxide O, H)
        if i + 2 < n and Z[i] == 8 and Z[i + 1] == 1 and Z[i + 2] == 1:
            excl += [(i, i + 1), (i, i + 2), (i + 1, i + 2)]
            i += 3
        elif i + 1 < n and Z[i] == 8 and Z[i + 1] == 1:
            excl += [(i, i + 1)]
            i += 2
        else:
            i += 1
    return X, Q, types, flags, excl


def case(name, seed, opls, fixed_from, dielectric, scale14):
    X, Q, types, flags, excl = water_case(seed, 3, 150, 18.0)
    n = len(X)
    if fixed_from is not None:
        flags = flags.copy()
        flags[fixed_from:] |= 4
    mm_o = [i for i in range(n) if types[i] == 0 and flags[i] & 1]

    def nearest(a):   # the closest MM oxygen of another molecule, so that the 1-4 pair lies inside the cutoff
        d = [np.linalg.norm(X[a] - X[b]) if b != a else np.inf for b in mm_o]
        return mm_o[int(np.argmin(d))]
    # O-O MM/MM pairs, a QC O - MM O pair, an MM O - QC H pair
    pairs14 = [(mm_o[0], nearest(mm_o[0])), (mm_o[5], nearest(mm_o[5])), (0, nearest(0)), (nearest(2), 2)]
    eps14 = [0.5 * e for e in EPSILON]
    E, G = R.mmmm_energy(X, Q, types, flags, EPSILON, SIGMA, eps14, SIGMA, opls, excl, pairs14,
                         inner=8.0, outer=12.0, damp=0.5, listCutoff=13.5, dielectric=dielectric, scale14=scale14)
    return {"name": name, "xyz": X.tolist(), "charges": list(map(float, Q)), "lj_types": types.tolist(), "flags": flags.tolist(),
            "epsilon": EPSILON, "sigma": SIGMA, "epsilon14": eps14, "sigma14": SIGMA, "opls": bool(opls),
            "exclusions": [list(p) for p in excl], "pairs14": [list(p) for p in pairs14], "inner": 8.0, "outer": 12.0,
            "damping": 0.5, "list": 13.5, "dielectric": dielectric, "scale14": scale14,
            "energies_kj": E.tolist(), "gradients_kj_per_a": G.tolist()}


def main():
    out = {"terms": ["MM/MM Elect.", "MM/MM LJ", "MM/MM 1-4 Elect.", "MM/MM 1-4 LJ", "QC/MM LJ", "QC/MM 1-4 LJ"],
           "cases": [case("opls_free", 5, True, None, 1.0, 1.0), case("amber_fixed", 6, False, 200, 2.0, 0.5)]}
    json.dump(out, open(os.path.join(HERE, "mmmm_reference.json"), "w"), indent=0)


if __name__ == "__main__":
    main()
