"""Generate the golden fixtures under tests/golden/ from the pDynamo 1.9.0 reference tree.

Run in a container that has the reference tree and the compiled reference core
(``make -C oracle ref``):

    python tests/golden/make_golden.py /root/reference

It writes
  mndo_rhf_pickle.json     the reference's stored "Pure QC" energies (kJ/mol) for every closed-shell test
                           molecule and Hamiltonian, read from pMolecule-1.9.0/data/reference/MNDORHFEnergies.pkl
                           (a Python-2 pickle of pCore.Testing.TestDataSet; loaded with a stub unpickler);
  molecules.json           the geometries of those molecules (the reference's own XYZ test inputs) with the
                           charges of pMolecule-1.9.0/tests/QCTestSystems.py:20-24;
  mndo_rhf_reference.json  energies (Eh), gradients (Eh/Bohr), SCF cycle counts and packed densities computed
                           by the reference's compiled C core on those molecules (<= 30 atoms, as
                           pMolecule-1.9.0/tests/MNDORHFEnergies.py:34 does), converger as in :39-40;
  qcmm_reference.json      QC/MM fixtures: the book's water dimer (book/examples/Example8.py, OPLS charges,
                           NBModelFull) run through the reference core, and an ABFS case.
"""

import glob, json, math, os, pickle, sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import refdriver as R  # noqa: E402

HAMILTONIANS = ("am1", "mndo", "pm3", "pddgmndo", "pddgpm3", "rm1")
CHARGES = {"cadmiumComplex": 2, "fch3cl": -1, "histamine": 1, "methylPhosphate": -2, "rhodiumComplex": -2}
SYMBOLS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
           "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm "
           "Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi").split()


def load_pickle(path):
    class Holder(dict):
        def __setstate__(self, st):
            self.update(st)

    def reconstruct(cls, base, state):
        return cls()

    class Unpickler(pickle.Unpickler):
        def find_class(self, module, name):
            if module == "copy_reg" and name == "_reconstructor":
                return reconstruct
            if module == "__builtin__" and name == "object":
                return object
            return type(name, (Holder,), {})

    data = Unpickler(open(path, "rb"), encoding="latin1").load()
    out = {}
    for h, ds in data["children"].items():
        out[h] = {label: {"value": float(v["value"]), "tolerance": float(v["absoluteErrorTolerance"])}
                  for label, v in ds["data"].items()}
    return out


def read_xyz(path):
    lines = open(path).read().splitlines()
    n = int(lines[0].split()[0])
    Z, xyz = [], []
    for line in lines[2:2 + n]:
        t = line.split()
        sym = t[0].capitalize()
        Z.append(SYMBOLS.index(sym) + 1 if not sym.isdigit() else int(sym))
        xyz.append([float(t[1]), float(t[2]), float(t[3])])
    return Z, xyz


def molecules(root):
    sources = (os.path.join(root, "pMolecule-1.9.0", "data", "xyz"),
               os.path.join(root, "molecularStructures", "difficultSCFCases", "xyz"),
               os.path.join(root, "molecularStructures", "gaussianGeometryOptimization", "xyz"))
    out = {}
    for src in sources:  # later sources replace earlier ones with the same label (QCTestSystems.py:64-72)
        for path in sorted(glob.glob(os.path.join(src, "*.xyz"))):
            label = os.path.basename(path)[:-4]
            Z, xyz = read_xyz(path)
            out[label] = {"Z": Z, "xyz": xyz, "charge": CHARGES.get(label, 0)}
    return out


def main(root):
    pk = load_pickle(os.path.join(root, "pMolecule-1.9.0", "data", "reference", "MNDORHFEnergies.pkl"))
    pk = {h: v for h, v in pk.items() if h in HAMILTONIANS}
    json.dump(pk, open(os.path.join(HERE, "mndo_rhf_pickle.json"), "w"), indent=1, sort_keys=True)
    mols = molecules(root)
    small = {k: v for k, v in mols.items() if len(v["Z"]) <= 30}
    json.dump(small, open(os.path.join(HERE, "molecules.json"), "w"), indent=0, sort_keys=True)
    table = json.load(open(R.PARAM_PATH))
    ref = {}
    for h in HAMILTONIANS:
        ref[h] = {}
        for label in sorted(pk[h]):
            if label not in small:
                continue
            m = small[label]
            if any(str(z) not in table["hamiltonians"][h] for z in m["Z"]):
                continue
            ham = R.RefHamiltonian(h, m["Z"])
            sysr = R.RefSystem(ham, m["Z"], charge=m["charge"], densityTolerance=1.0e-8, maximumSCFCycles=500)
            r = sysr.energy(np.array(m["xyz"]))
            entry = {"converged": bool(r["converged"]), "ncycles": r["ncycles"], "pure_qc_kj": r["pure_qc_kj"],
                     "eelectronic": r["eelectronic"], "enuclear": r["enuclear"], "baseline": r["baseline"],
                     "gradients": r["gradients"].tolist(), "pickle_kj": pk[h][label]["value"]}
            if len(m["Z"]) <= 6:
                entry["density"] = r["density"].tolist()
            ref[h][label] = entry
            print("%-9s %-22s conv=%d cyc=%3d E=%16.8f pickle=%16.8f d=%.2e" % (
                h, label, r["converged"], r["ncycles"], r["pure_qc_kj"], pk[h][label]["value"],
                r["pure_qc_kj"] - pk[h][label]["value"]))
    json.dump(ref, open(os.path.join(HERE, "mndo_rhf_reference.json"), "w"), indent=0, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
