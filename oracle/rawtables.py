"""Test infrastructure: flat raw-parameter arrays shared by the two CPU checkers.

Both ``ref_shim.c`` (driving pDynamo's compiled core) and ``mndo_oracle.c`` (the plain-C
restatement) take per-element parameters in the units of pDynamo's YAML files, laid out as the
arrays built here from ``pdynamo_mirror_gb300/parameters/mndo_parameters.json``.
"""

import json, os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PARAM_PATH = os.path.join(HERE, "..", "pdynamo_mirror_gb300", "parameters", "mndo_parameters.json")

RAW_FIELDS = ("iii", "iiid", "ir016", "ir066", "ir244", "ir266", "ir466", "qnd", "qnp", "qns",
              "ad", "alp", "am", "aq", "betad", "betap", "betas", "dd", "eheat", "eisol", "f0sd", "gphot",
              "gpp", "gp2", "gsp", "gss", "g2sd", "hsp", "pcore", "qq", "udd", "upp", "uss", "zcore",
              "zetad", "zetap", "zetas", "zdn", "zpn", "zsn")
MAXGAUSS, MAXPDDG, MAXPRIM = 4, 4, 6
MAXDIATOMIC = 100   # PM6 diatomic core-core pairs per element (partner atomic numbers < 100)
SHELL_TYPE = {"S": 0, "P": 1}
_TABLE = None


def table():
    global _TABLE
    if _TABLE is None:
        _TABLE = json.load(open(PARAM_PATH))
    return _TABLE


def raw_arrays(hamiltonian, elements):
    """Arrays (Z, norb, raw, ng, gauss, npddg, pddg, nshell, stype, nprim, exps, coefs, ndiatomic, diatomic) for
    sorted elements; diatomic rows are (partner atomic number, coefficient x, exponent a in A^-1) as the PM6
    files list them."""
    t = table()
    ne = len(elements)
    Z = np.array(elements, dtype=np.int32)
    norb = np.zeros(ne, np.int32); raw = np.zeros((ne, len(RAW_FIELDS)))
    ng = np.zeros(ne, np.int32); gauss = np.zeros((ne, MAXGAUSS, 3))
    npd = np.zeros(ne, np.int32); pddg = np.zeros((ne, MAXPDDG, 2))
    nsh = np.zeros(ne, np.int32); stype = np.zeros((ne, 2), np.int32); nprim = np.zeros((ne, 2), np.int32)
    exps = np.zeros((ne, 2, MAXPRIM)); coefs = np.zeros((ne, 2, MAXPRIM))
    nd = np.zeros(ne, np.int32); diat = np.zeros((ne, MAXDIATOMIC, 3))
    for e, z in enumerate(elements):
        el = t["hamiltonians"][hamiltonian][str(z)]
        norb[e] = el["orbitals"]
        raw[e] = [float(el[f]) for f in RAW_FIELDS]
        ng[e] = len(el["gaussians"]); npd[e] = len(el["pddg"])
        for i, g in enumerate(el["gaussians"]): gauss[e, i] = g
        for i, g in enumerate(el["pddg"]): pddg[e, i] = g
        nd[e] = len(el.get("diatomic", []))
        for i, g in enumerate(el.get("diatomic", [])): diat[e, i] = g
        lab = ("%ds" % el["qns"] if el["qns"] else "") + ("%dp" % el["qnp"] if el["qnp"] else "")
        shells = t["bases"][lab][: (1 if el["orbitals"] == 1 else 2)]
        nsh[e] = len(shells)
        for s, sh in enumerate(shells):
            stype[e, s] = SHELL_TYPE[sh["type"]]; nprim[e, s] = len(sh["exponents"])
            exps[e, s, :nprim[e, s]] = sh["exponents"]; coefs[e, s, :nprim[e, s]] = sh["coefficients"]
    return (Z, norb, raw.ravel().copy(), ng, gauss.ravel().copy(), npd, pddg.ravel().copy(), nsh,
            stype.ravel().copy(), nprim.ravel().copy(), exps.ravel().copy(), coefs.ravel().copy(), nd, diat.ravel().copy())
