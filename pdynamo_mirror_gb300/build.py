"""In-tree build of libpdg.so (the CUDA path) for sm_103a.

Translation units are compiled in parallel with nvcc and linked with ``nvcc -shared``; the result
lands in ``pdynamo_mirror_gb300/_lib/libpdg.so`` (git-ignored).  A build is skipped when the library
is newer than every source.
"""

import os, subprocess, sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libpdg.so")
UNITS = ("api.cu", "integrals.cu", "scf.cu", "scf_wide.cu", "qcmm.cu", "tc.cu", "guess.cu", "dynamics.cu", "mmmm.cu", "wide.cu", "bonded.cu")
HEADERS = ("common.cuh", "multipole.cuh", "overlap.cuh", "tc.cuh")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-diag-suppress", "177"]


def _nvcc():
    for c in (os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc"), "nvcc"):
        if os.path.sep not in c or os.path.exists(c):
            return c
    return "nvcc"


def _defines():
    """Extra -D options from PDG_NVCC_DEFINES (space separated, e.g. "PDG_SCF_CTAS_PER_SM=2"), for trying
    compile-time configurations; empty by default."""
    return ["-D" + d for d in os.environ.get("PDG_NVCC_DEFINES", "").split()]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, u) for u in UNITS + HEADERS] + [os.path.join(HERE, "..", "include", "pdg.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    objs = [os.path.join(LIBDIR, u.replace(".cu", ".o")) for u in UNITS]

    def compile_one(args):
        src, obj = args
        cmd = [nvcc] + ARCH + FLAGS + _defines() + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(compile_one, zip(UNITS, objs)))
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lcublas"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
