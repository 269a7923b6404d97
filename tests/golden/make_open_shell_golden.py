"""Generate tests/golden/open_shell_reference.json: AM1 energies, gradients and SCF cycle counts of the reference's
radical test set (pMolecule-1.9.0/tests/QCTestSystems.py:34-56, as pMolecule-1.9.0/tests/MNDOUHFEnergies.py runs it:
converger densityTolerance 1e-8, maximumSCFCycles 500) for every restricted / unrestricted and occupancy-type
combination listed there, computed by the reference's compiled C core (oracle/ref_shim.c: ref_system_create_open).
Spin densities (alpha and beta, packed) are kept for the two small radicals and for the tyrosine dipeptide triplet
(unrestricted, cardinal occupancies: the start density of the converged-state test).  QC/MM cases: the three open-shell
systems in the field of seeded point charges (their potentials at the QC atoms stored with the case).  PM6 cases:
the allyl and methylene radicals, unrestricted.

Run where the reference tree and the compiled reference core exist (``make -C oracle ref``):

    PDYNAMO_REFERENCE=<reference tree> python tests/golden/make_open_shell_golden.py
"""

import json, os, sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
sys.path.insert(0, HERE)
from oracle import refdriver as R  # noqa: E402
from make_golden import read_xyz  # noqa: E402

# label, file, data directory, charge, multiplicity (QCTestSystems.py:34-38)
SYSTEMS = (("Tyrosine Dipeptide Singlet", "tyrosineDipeptide", "xyz", 0, 1),
           ("Tyrosine Dipeptide Triplet", "tyrosineDipeptide", "xyz", 0, 3),
           ("Allyl Radical", "allyl", "radicals", 0, 2),
           ("Methylene Radical", "methylene", "radicals", 0, 3))
UNRESTRICTED = [(False, "Cardinal"), (False, "Fixed Fractional"), (False, "Variable Fractional")]
KEYWORDS = {"Tyrosine Dipeptide Singlet": [(True, "Cardinal"), (False, "Cardinal"), (True, "Fixed Fractional"),
                                           (False, "Fixed Fractional"), (True, "Variable Fractional"), (False, "Variable Fractional")],
            "Tyrosine Dipeptide Triplet": UNRESTRICTED, "Allyl Radical": UNRESTRICTED, "Methylene Radical": UNRESTRICTED}
SMALL = ("Allyl Radical", "Methylene Radical")


def reference_root():
    """The pDynamo 1.9.0 tree: the first argument, else $PDYNAMO_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PDYNAMO_REFERENCE")
    if not root:
        raise SystemExit("usage: %s <reference tree>  (or set PDYNAMO_REFERENCE)" % sys.argv[0])
    return root


def main(root):
    out = {"hamiltonian": "am1", "converger": {"densityTolerance": 1.0e-8, "maximumSCFCycles": 500}, "cases": []}
    for label, name, sub, charge, mult in SYSTEMS:
        Z, X = read_xyz(os.path.join(root, "pMolecule-1.9.0", "data", sub, name + ".xyz"))
        ham = R.RefHamiltonian("am1", Z)
        for restricted, occ in KEYWORDS[label]:
            s = R.RefSystem(ham, Z, charge=charge, multiplicity=mult, isSpinRestricted=restricted, occupancyType=occ,
                            densityTolerance=1.0e-8, maximumSCFCycles=500)
            r = s.energy(np.array(X))
            case = {"label": label, "atomic_numbers": Z, "xyz": X, "charge": charge, "multiplicity": mult,
                    "isSpinRestricted": restricted, "occupancyType": occ, "converged": bool(r["converged"]),
                    "ncycles": int(r["ncycles"]), "pure_qc_kj": float(r["pure_qc_kj"]),
                    "eelectronic": float(r["eelectronic"]), "enuclear": float(r["enuclear"]),
                    "gradients_hartree_per_bohr": r["gradients"].tolist()}
            if label in SMALL or (label == "Tyrosine Dipeptide Triplet" and occ == "Cardinal"):
                if restricted:
                    case["density"] = r["density"].tolist()
                else:
                    case["density_alpha"], case["density_beta"] = r["density_alpha"].tolist(), r["density_beta"].tolist()
            out["cases"].append(case)
            print(label, "restricted" if restricted else "unrestricted", occ, case["converged"], case["ncycles"],
                  "%.6f" % case["pure_qc_kj"])
    # QC/MM: the radicals in the field of seeded point charges (potentials at the QC atoms in atomic units, the
    # form the reference's QC model receives them, QCMMInteractionState.qcmmPotentials)
    out["qcmm_cases"] = []
    rng = np.random.default_rng(17)
    bohr = 1.0e-10 / 5.291772083e-11
    for label, name, sub, charge, mult in SYSTEMS[1:]:
        Z, X = read_xyz(os.path.join(root, "pMolecule-1.9.0", "data", sub, name + ".xyz"))
        X = np.array(X)
        centre = X.mean(0)
        d = rng.normal(size=(8, 3))
        sites = centre + 5.0 * d / np.linalg.norm(d, axis=1)[:, None]
        q = rng.uniform(-0.8, 0.8, size=8)
        phi = [float(sum(qm / (np.linalg.norm(x - m) * bohr) for qm, m in zip(q, sites))) for x in X]
        ham = R.RefHamiltonian("am1", Z)
        occ = "Variable Fractional" if label == "Tyrosine Dipeptide Triplet" else "Cardinal"
        s = R.RefSystem(ham, Z, charge=charge, qcmm=True, multiplicity=mult, isSpinRestricted=False, occupancyType=occ,
                        densityTolerance=1.0e-8, maximumSCFCycles=500)
        r = s.energy(X, phi=np.array(phi))
        out["qcmm_cases"].append({"label": label, "atomic_numbers": Z, "xyz": X.tolist(), "charge": charge,
                                  "multiplicity": mult, "isSpinRestricted": False, "occupancyType": occ, "phi": phi,
                                  "converged": bool(r["converged"]), "ncycles": int(r["ncycles"]),
                                  "total_electronic": float(r["total_electronic"]), "eqcmm": float(r["eqcmm"]),
                                  "charges": r["charges"].tolist(), "gradients_hartree_per_bohr": r["gradients"].tolist()})
        print("QC/MM", label, occ, r["converged"], r["ncycles"], "%.10f" % r["total_electronic"])
    # PM6 (diatomic core-core term) for the two small radicals, unrestricted, cardinal occupancy
    out["pm6_cases"] = []
    for label, name, sub, charge, mult in SYSTEMS[2:]:
        Z, X = read_xyz(os.path.join(root, "pMolecule-1.9.0", "data", sub, name + ".xyz"))
        s = R.RefSystem(R.RefHamiltonian("pm6", Z), Z, charge=charge, multiplicity=mult, isSpinRestricted=False,
                        occupancyType="Cardinal", densityTolerance=1.0e-8, maximumSCFCycles=500)
        r = s.energy(np.array(X))
        out["pm6_cases"].append({"label": label, "atomic_numbers": Z, "xyz": X, "charge": charge, "multiplicity": mult,
                                 "converged": bool(r["converged"]), "ncycles": int(r["ncycles"]),
                                 "pure_qc_kj": float(r["pure_qc_kj"]), "gradients_hartree_per_bohr": r["gradients"].tolist()})
        print("PM6", label, r["converged"], r["ncycles"], "%.6f" % r["pure_qc_kj"])
    json.dump(out, open(os.path.join(HERE, "open_shell_reference.json"), "w"), indent=0)


if __name__ == "__main__":
    main(reference_root())
