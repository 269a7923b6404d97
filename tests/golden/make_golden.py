"""Generate the golden fixtures under tests/golden/ from the pDynamo 1.9.0 reference tree.

Run in a container that has the reference tree and the compiled reference core
(``make -C oracle ref``):

    PDYNAMO_REFERENCE=<reference tree> python tests/golden/make_golden.py

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


def reference_root():
    """The pDynamo 1.9.0 tree: the first argument, else $PDYNAMO_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PDYNAMO_REFERENCE")
    if not root:
        raise SystemExit("usage: %s <reference tree>  (or set PDYNAMO_REFERENCE)" % sys.argv[0])
    return root


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
    qcmm_fixtures(root)


def qcmm_fixtures(root):
    """QC/MM fixtures.  example8: the book's AM1 water dimer (QC = first water, OPLS/TIP3P charges on the
    second, NBModelFull) with its published values (book/logs/Example8.log:75-85) and the reference core's
    results.  abfs: a 4-water AM1 QC cluster in 300 TIP3P waters with NBModelABFS 8/12 A through the
    reference's ABFS pair routines; the spline knots are the C restatement's (oracle.abfs_knots) because
    the reference tabulates them in Python-2 Pyrex that cannot run here."""
    sys.path.insert(0, os.path.join(HERE, "..", ".."))
    from oracle import oracle as O
    from pdynamo_mirror_gb300 import workloads as W
    out = {}
    lines = open(os.path.join(root, "book", "data", "mol", "waterDimer_cs.mol")).read().splitlines()
    X = np.array([[float(v) for v in l.split()[:3]] for l in lines[4:10]])
    Zq, q = [8, 1, 1], np.array([-0.834, 0.417, 0.417])
    phi, _, _ = O.qcmm("full", X[:3], X[3:], q)
    rs = R.RefSystem(R.RefHamiltonian("am1", Zq), Zq, qcmm=True)
    r = rs.energy(X[:3], phi=phi)
    gfull = np.zeros((6, 3))
    _, gq, gm = O.qcmm("full", X[:3], X[3:], q, qcq=r["charges"])
    out["example8"] = {"Z": [8, 1, 1, 8, 1, 1], "xyz": X.tolist(), "mm_charges": [0, 0, 0] + q.tolist(), "qc": [0, 1, 2],
                       "model": "full", "book": {"pure_qc_kj": -244.1191, "qcmm_kj": -23.7448, "electronic_with_qcmm": -18.121115,
                                                 "nuclear": 5.3040515, "ncycles": 8},
                       "pure_qc_kj": r["pure_qc_kj"], "qcmm_kj": 2625.5 * r["eqcmm"], "ncycles": r["ncycles"],
                       "qc_gradients": (r["gradients"] + gq).tolist(), "mm_gradients": gm.tolist()}
    Zc, Xc = W.water_cluster(4, seed=11, centre=[10.0, 10.0, 10.0])
    rng = np.random.default_rng(5)
    mmX, mmZ, mmq = [], [], []
    grid = W._Grid(np.zeros(3) - 5.0, 30.0, 2.6)
    for o in Xc[Zc == 8]:
        grid.add(o)
    for o in W._place(rng, 300, np.zeros(3), 20.0, grid):
        Rm = W._random_rotation(rng)
        mmX.extend(o + W._water_local() @ Rm.T); mmZ.extend([8, 1, 1]); mmq.extend([W.TIP3P_O, W.TIP3P_H, W.TIP3P_H])
    mmX, mmq = np.array(mmX), np.array(mmq)
    kx, ky = O.abfs_knots(8.0, 12.0)
    ab = R.RefABFS(8.0, 12.0, kx, ky)
    Zl = [int(z) for z in Zc]
    rs = R.RefSystem(R.RefHamiltonian("am1", Zl), Zl, qcmm=True)
    phi, _, _ = ab.qcmm(rs, Xc, mmX, mmq, np.zeros(len(Zl)))
    r = rs.energy(Xc, phi=phi)
    _, gq, gm = ab.qcmm(rs, Xc, mmX, mmq, r["charges"])
    conv = 1.0 / ((1.0e-10 / 5.291772083e-11) * 2625.5)   # kJ/mol/A -> Eh/Bohr
    out["abfs"] = {"Z": Zl + mmZ, "xyz": np.concatenate([Xc, mmX]).tolist(), "mm_charges": [0.0] * len(Zl) + mmq.tolist(),
                   "qc": list(range(len(Zl))), "model": "abfs", "inner": 8.0, "outer": 12.0,
                   "pure_qc_kj": r["pure_qc_kj"], "qcmm_kj": 2625.5 * r["eqcmm"], "ncycles": r["ncycles"], "phi": phi.tolist(),
                   "qc_gradients": (r["gradients"] + gq * conv).tolist(), "mm_gradients": (gm * conv).tolist()}
    json.dump(out, open(os.path.join(HERE, "qcmm_reference.json"), "w"), indent=0)
    print("example8 pure %.4f qcmm %.4f cycles %d; abfs pure %.4f qcmm %.4f cycles %d" % (
        out["example8"]["pure_qc_kj"], out["example8"]["qcmm_kj"], out["example8"]["ncycles"],
        out["abfs"]["pure_qc_kj"], out["abfs"]["qcmm_kj"], out["abfs"]["ncycles"]))


if __name__ == "__main__":
    main(reference_root())
