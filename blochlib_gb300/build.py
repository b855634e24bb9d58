"""In-tree build of libblochlib_gb300.so (sm_103a) and of the CPU oracle.

The product library is the CUDA engine plus its host layer and C ABI.  The oracle
(oracle/gcompute_ref.cc, test infrastructure only) is built beside it so that tests and
the bench's CPU-baseline leg can load it; the product never links it.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "blochlib_gb300"
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libblochlib_gb300.so"
ORACLE_SRC = ROOT / "oracle" / "gcompute_ref.cc"
ORACLE_BUILD = ROOT / "oracle" / "_build"
ORACLE_LIB = ORACLE_BUILD / "liboracle.so"
ORACLE_BIN = ORACLE_BUILD / "gcompute_ref"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and Path(c, "bin", "nvcc").exists():
            return Path(c)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(map(str, cmd)) + "\n" + r.stdout)
    return r.stdout


def _stale(target, sources):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in sources)


def build_library(verbose=False, force=False):
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "blochlib_gb300.h"]
    units = [
        (CSRC / "bl_engine.cu", [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                 "-Xptxas", "-v" if verbose else "-O3"]),
        (CSRC / "bl_host.cc", ["g++", "-O2", "-std=c++17", "-fPIC"]),
        (CSRC / "bl_hamgen.cc", ["g++", "-O2", "-std=c++17", "-fPIC"]),
        (CSRC / "bl_capi.cc", ["g++", "-O2", "-std=c++17", "-fPIC", f"-I{cuda / 'include'}"]),
        (CSRC / "bl_server.cc", ["g++", "-O2", "-std=c++17", "-fPIC", f"-I{cuda / 'include'}"]),
    ]
    objs = []
    jobs = []
    for src, cmd in units:
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append(cmd + ["-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=4) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-cudart", "static"])
    return LIB


EXAMPLES = PKG / "examples"


def build_examples(force=False):
    """C++ programs written against include/blochlib_gb300.hpp (linked to the library)."""
    out = EXAMPLES / "_build"
    out.mkdir(exist_ok=True)
    built = []
    for src in sorted(EXAMPLES.glob("*.cc")):
        exe = out / src.stem
        deps = [src, ROOT / "include" / "blochlib_gb300.hpp", ROOT / "include" / "blochlib_gb300.h", LIB]
        if force or _stale(exe, deps):
            _run(["g++", "-O2", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(exe), f"-L{PKG}",
                  "-lblochlib_gb300", f"-Wl,-rpath,{PKG}"])
        built.append(exe)
    return built


def build_oracle(force=False):
    """Oracle (test infrastructure): shared library for ctypes and the CLI binary."""
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    if force or _stale(ORACLE_LIB, [ORACLE_SRC]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", str(ORACLE_LIB), str(ORACLE_SRC)])
    if force or _stale(ORACLE_BIN, [ORACLE_SRC]):
        _run(["g++", "-O2", "-std=c++17", "-DORACLE_MAIN", "-o", str(ORACLE_BIN), str(ORACLE_SRC)])
    return ORACLE_LIB


def reference_tree():
    """The reference tree's path as oracle/build_ref.sh resolves it (BLOCHLIB_REF or the
    recipe's default), or None where it is absent."""
    r = subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh"), "where"], stdout=subprocess.PIPE,
                       stderr=subprocess.DEVNULL, text=True)
    return Path(r.stdout.strip()) if r.returncode == 0 and r.stdout.strip() else None


def build_reference():
    """The reference's own path (oracle/_ref), when its sources are present."""
    script = ROOT / "oracle" / "build_ref.sh"
    have_src = (reference_tree() is not None) or (ROOT / "oracle" / "_ref" / "src" / ".patched").exists()
    if not have_src:
        return None
    r = subprocess.run(["bash", str(script), "all"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write("reference build failed (continuing without it):\n" + r.stdout[-2000:])
        return None
    return ROOT / "oracle" / "_ref" / "ref_fid"


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_library(verbose="-v" in sys.argv, force=force))
    print(build_oracle(force=force))
    print(build_examples(force=force))
