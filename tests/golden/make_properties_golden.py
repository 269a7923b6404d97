"""Generate tests/golden/properties_reference.json: dipole moments (Debye) and Mayer bond orders, charges, free and total
valences of converged densities, computed by the reference's compiled C core (QCModelMNDO_DipoleMoment and
QCModelMNDO_MayerBondOrders through ref_system_properties in oracle/ref_shim.c), as pMolecule-1.9.0/tests/
MNDORHFEnergies.py and MNDOUHFEnergies.py print them: closed-shell test molecules under AM1 and PM3, and the allyl
radical (UHF, AM1).

Run where the reference tree and the compiled reference core exist (``make -C oracle ref``):

    PDYNAMO_REFERENCE=<reference tree> python tests/golden/make_properties_golden.py
"""

import json, os, sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
sys.path.insert(0, HERE)
from oracle import refdriver as R  # noqa: E402
from make_golden import read_xyz  # noqa: E402

CLOSED = (("water", "am1"), ("formaldehyde", "am1"), ("glycine", "am1"), ("pyridine", "pm3"), ("nitromethane", "pm3"))


def reference_root():
    """The pDynamo 1.9.0 tree: the first argument, else $PDYNAMO_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PDYNAMO_REFERENCE")
    if not root:
        raise SystemExit("usage: %s <reference tree>  (or set PDYNAMO_REFERENCE)" % sys.argv[0])
    return root


def main(root):
    mols = json.load(open(os.path.join(HERE, "molecules.json")))
    out = {"cases": []}

    def record(name, ham_name, Z, X, charge, restricted, r, p):
        case = {"name": name, "hamiltonian": ham_name, "Z": [int(z) for z in Z], "xyz": np.asarray(X).tolist(), "charge": charge,
                "isSpinRestricted": restricted, "dipole_debye": p["dipole"].tolist(), "bond_orders": p["bond_orders"].tolist(),
                "mayer_charges": p["charges"].tolist(), "free_valence": p["free_valence"].tolist(),
                "total_valence": p["total_valence"].tolist()}
        out["cases"].append(case)
        print(name, ham_name, r["converged"], "%.6f" % np.linalg.norm(p["dipole"]))

    for name, ham_name in CLOSED:
        m = mols[name]
        s = R.RefSystem(R.RefHamiltonian(ham_name, m["Z"]), m["Z"], m["charge"])
        r = s.energy(np.array(m["xyz"]))
        record(name, ham_name, m["Z"], m["xyz"], m["charge"], True, r, s.properties())
    Z, X = read_xyz(os.path.join(root, "pMolecule-1.9.0", "data", "radicals", "allyl.xyz"))
    s = R.RefSystem(R.RefHamiltonian("am1", Z), Z, 0, multiplicity=2, isSpinRestricted=False, maximumSCFCycles=500)
    r = s.energy(np.array(X))
    record("allyl", "am1", Z, X, 0, False, r, s.properties())
    json.dump(out, open(os.path.join(HERE, "properties_reference.json"), "w"), indent=0)


if __name__ == "__main__":
    main(reference_root())
