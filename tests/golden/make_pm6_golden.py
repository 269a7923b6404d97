"""Generate tests/golden/pm6_reference.json: closed-shell PM6 energies, gradients and SCF cycle counts computed by
the reference's compiled C core (oracle/ref_shim.c with the PM6 diatomic core-core parameters,
pMolecule-1.9.0/extensions/csource/MNDOIntegralUtilities.c:35-230) for the reference's closed-shell test molecules
(tests/golden/molecules.json) whose elements all have s and p orbitals only under PM6 and that have at most 30 atoms,
converger as pMolecule-1.9.0/tests/MNDORHFEnergies.py runs it.  The reference stores PM6 energies only (below), so
the gradients and cycle counts come from the core run here; its energies equal the stored ones to 1e-8 kJ/mol.

Run where the reference tree and the compiled reference core exist (``make -C oracle ref``):

    PDYNAMO_REFERENCE=<reference tree> python tests/golden/make_pm6_golden.py

It also writes pm6_pickle.json: the reference's stored PM6 "Pure QC" energies (kJ/mol, with their tolerance) from
pMolecule-1.9.0/data/reference/MNDORHFEnergies.pkl, read as make_golden.py reads the other Hamiltonians'.
"""

import json, os, sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import refdriver as R  # noqa: E402
from oracle.rawtables import table  # noqa: E402
sys.path.insert(0, HERE)
from make_golden import load_pickle  # noqa: E402


def reference_root():
    """The pDynamo 1.9.0 tree: the first argument, else $PDYNAMO_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PDYNAMO_REFERENCE")
    if not root:
        raise SystemExit("usage: %s <reference tree>  (or set PDYNAMO_REFERENCE)" % sys.argv[0])
    return root


def main(root):
    pk = load_pickle(os.path.join(root, "pMolecule-1.9.0", "data", "reference", "MNDORHFEnergies.pkl"))
    json.dump({"pm6": pk["pm6"]}, open(os.path.join(HERE, "pm6_pickle.json"), "w"), indent=1, sort_keys=True)
    mols = json.load(open(os.path.join(HERE, "molecules.json")))
    pm6 = table()["hamiltonians"]["pm6"]
    out = {"hamiltonian": "pm6", "converger": {"densityTolerance": 1.0e-8, "maximumSCFCycles": 500}, "molecules": {}}
    for name in sorted(mols):
        m = mols[name]
        Z = [int(z) for z in m["Z"]]
        if len(Z) > 30 or any(str(z) not in pm6 for z in Z):
            continue
        ham = R.RefHamiltonian("pm6", Z)
        s = R.RefSystem(ham, Z, charge=m["charge"], densityTolerance=1.0e-8, maximumSCFCycles=500)
        r = s.energy(np.array(m["xyz"]))
        out["molecules"][name] = {"Z": Z, "charge": m["charge"], "xyz": m["xyz"], "converged": bool(r["converged"]),
                                  "ncycles": int(r["ncycles"]), "eelectronic": float(r["eelectronic"]),
                                  "enuclear": float(r["enuclear"]), "pure_qc_kj": float(r["pure_qc_kj"]),
                                  "gradients_hartree_per_bohr": r["gradients"].tolist()}
        print(name, len(Z), r["converged"], r["ncycles"], "%.6f" % r["pure_qc_kj"])
    json.dump(out, open(os.path.join(HERE, "pm6_reference.json"), "w"), indent=0)


if __name__ == "__main__":
    main(reference_root())
