"""Generate ``mndo_parameters.json`` from pDynamo's parameter YAML files.

The element parameter files (``parameters/mndoParameters/<hamiltonian>/<El>.yaml``) and the
STO-6G shells (``parameters/mndoParameters/mndostong/<label>.yaml``) of pDynamo 1.9.0 are
published parameter data.  This script copies their numbers, unchanged and in their original
units (eV, Angstrom, kcal/mol, atomic), into one JSON file that the package reads at run time,
so that nothing at run time needs the pDynamo tree.  Unit conversion happens in
``pdynamo_mirror_gb300.parameters`` (restating ``pMolecule.MNDOParameters.pyx:309-370``).

Usage: python make_tables.py <pDynamo root> [output.json]
"""

import json, os, re, sys

HAMILTONIANS = ("am1", "mndo", "pm3", "pddgmndo", "pddgpm3", "rm1")
# tabulated as well (the checkers use them; the product's Hamiltonians are the list above): PM6 with its
# diatomic core-core parameters, elements with s and p orbitals only
TABLE_HAMILTONIANS = HAMILTONIANS + ("pm6",)
SYMBOLS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
           "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm "
           "Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi").split()

_ROW = re.compile(r"^\s*-\s*\[(.*)\]\s*$")


def _numbers(text):
    return [float(t) for t in text.replace("[", " ").replace("]", " ").replace(",", " ").split()]


def read_element(path):
    """Parse the fixed layout of an MNDOParameters YAML file (scalars + optional tables)."""
    scalars, tables, section = {}, {}, None
    for line in open(path):
        s = line.strip()
        if s.startswith("Scalar Parameters:"): section = "scalars"; continue
        if s.startswith("AM1/PM3 Gaussian Parameters:"): section = "gaussians"; continue
        if s.startswith("PDDG Gaussian Parameters:"): section = "pddg"; continue
        if s.startswith("Diatomic Parameters:"): section = "diatomic"; continue
        m = _ROW.match(line)
        if m is None:
            if s and not s.startswith("-") and ":" in s: section = None
            continue
        if section == "scalars":
            label, value, units = [t.strip() for t in m.group(1).split(",")]
            scalars[label] = float(value) if ("." in value or "e" in value.lower()) else int(value)
        elif section in ("gaussians", "pddg", "diatomic"):
            tables.setdefault(section, []).append(_numbers(m.group(1)))
    out = dict(scalars)
    out["gaussians"] = tables.get("gaussians", [])
    out["pddg"] = tables.get("pddg", [])
    if tables.get("diatomic"):
        out["diatomic"] = tables["diatomic"]   # [partner atomic number, coefficient, exponent (A^-1)], PM6
    return out


def read_basis(path):
    """Parse an STO-nG GaussianBasis YAML file into shells of (type, exponents, coefficients)."""
    shells, current = [], None
    for line in open(path):
        s = line.strip()
        if s.startswith("- Primitives:"):
            current = {"exponents": [], "coefficients": []}
            shells.append(current)
        elif s.startswith("Type:"):
            current["type"] = s.split(":")[1].strip()
        elif current is not None and s.startswith("- ["):
            v = _numbers(s[1:])
            current["exponents"].append(v[0])
            current["coefficients"].append(v[1])
    return shells


def read_masses(folder):
    """Atomic masses (amu) by atomic number from the element files (``Atomic Number`` and ``Mass`` lines):
    the masses pDynamo's dynamics weights the coordinates with (SystemGeometryObjectiveFunction.py:106-120)."""
    masses = {}
    for fname in sorted(os.listdir(folder)):
        if not fname.endswith(".yaml"): continue
        z = m = None
        for line in open(os.path.join(folder, fname)):
            key, _, value = line.partition(":")
            if key.strip() == "Atomic Number": z = int(value)
            elif key.strip() == "Mass": m = float(value)
        if z is not None and m is not None:
            masses[str(z)] = m
    return masses


def main(root, output):
    base = os.path.join(root, "parameters", "mndoParameters")
    data = {"source": "pDynamo-1.9.0 parameters/mndoParameters", "hamiltonians": {}, "bases": {}}
    labels = set()
    for h in TABLE_HAMILTONIANS:
        table = {}
        for fname in sorted(os.listdir(os.path.join(base, h))):
            if not fname.endswith(".yaml"): continue
            el = read_element(os.path.join(base, h, fname))
            if "diatomic" in el and h not in ("pm6",):
                raise ValueError("diatomic core-core parameters outside PM6: " + fname)
            if el["orbitals"] not in (1, 4):
                continue  # d-orbital elements belong to the PM6 path
            table[str(el["atomicNumber"])] = el
            lab = ""
            if el["qns"]: lab += "%ds" % el["qns"]
            if el["qnp"]: lab += "%dp" % el["qnp"]
            labels.add(lab)
        data["hamiltonians"][h] = table
    for lab in sorted(labels):
        path = os.path.join(base, "mndostong", lab + ".yaml")
        if os.path.exists(path):  # pDynamo ships no 6s6p shells, so those elements cannot be set up there either
            data["bases"][lab] = read_basis(path)
    data["masses"] = read_masses(os.path.join(root, "parameters", "elements"))
    with open(output, "w") as f:
        json.dump(data, f, indent=0, sort_keys=True)


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    main(sys.argv[1], sys.argv[2] if len(sys.argv) > 2 else os.path.join(here, "mndo_parameters.json"))
