"""In-tree build of ``libjaxabm_gb300.so`` (CUDA kernels + C ABI) for sm_103a.

Every ``csrc/*.cu`` and ``csrc/*.cpp`` file is compiled to an object in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into one shared library next
to this file.  The library links only the CUDA runtime: no torch types cross the ABI.

``build(checked=True)`` compiles the same sources with ``-DABM_CHECKED`` into
``libjaxabm_gb300_checked.so``: the range-checked build, in which gathers indexed by caller
data report an out-of-range index as ABM_ERR_BOUNDS (slower: every checked entry point
waits for its stream).  It is built only on request.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libjaxabm_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)
CHECKED_BUILD_DIR = os.path.join(HERE, "_build_checked")
CHECKED_LIB_PATH = os.path.join(HERE, "libjaxabm_gb300_checked.so")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                "-Xcompiler", "-fvisibility=hidden", "-I", INCLUDE]


def nvcc_path():
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "bin", "nvcc")):
            return os.path.join(root, "bin", "nvcc")
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build jaxabm_gb300")


def sources():
    out = []
    for name in sorted(os.listdir(CSRC)):
        if name.endswith((".cu", ".cpp")):
            out.append(os.path.join(CSRC, name))
    return out


def _headers():
    hs = [os.path.join(CSRC, n) for n in os.listdir(CSRC) if n.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, n) for n in os.listdir(INCLUDE) if n.endswith(".h")]
    return hs


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def up_to_date(path=LIB_PATH):
    if not os.path.exists(path):
        return False
    return os.path.getmtime(path) >= _newest(sources() + _headers() + [__file__])


def _compile(nvcc, src, extra, build_dir=BUILD_DIR):
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
    cmd = [nvcc] + ARCH_FLAGS + COMMON_FLAGS + extra + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd += ["-Xcompiler", "-pthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{res.stderr}")
    return obj, res.stderr


def build(force=False, verbose=False, extra_flags=(), checked=False):
    """Compile the library (the range-checked one with ``checked``) if any source is newer
    than it; return the library path."""
    lib_path = CHECKED_LIB_PATH if checked else LIB_PATH
    build_dir = CHECKED_BUILD_DIR if checked else BUILD_DIR
    if not force and not extra_flags and up_to_date(lib_path):
        return lib_path
    nvcc = nvcc_path()
    os.makedirs(build_dir, exist_ok=True)
    srcs = sources()
    extra = list(extra_flags) + (["-DABM_CHECKED"] if checked else [])
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, extra, build_dir), srcs))
    objs = [r[0] for r in results]
    if verbose:
        for _, log in results:
            if log.strip():
                sys.stderr.write(log)
    tmp = lib_path + ".tmp"
    cmd = [nvcc] + ARCH_FLAGS + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, checked="--checked" in sys.argv))
