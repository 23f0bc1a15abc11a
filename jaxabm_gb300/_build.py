"""In-tree build of ``libjaxabm_gb300.so`` (CUDA kernels + C ABI) for sm_103a.

Every ``csrc/*.cu`` and ``csrc/*.cpp`` file is compiled to an object in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into one shared library next
to this file.  The library links only the CUDA runtime: no torch types cross the ABI.
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


def up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    return os.path.getmtime(LIB_PATH) >= _newest(sources() + _headers() + [__file__])


def _compile(nvcc, src, extra):
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc] + ARCH_FLAGS + COMMON_FLAGS + extra + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd += ["-Xcompiler", "-pthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{res.stderr}")
    return obj, res.stderr


def build(force=False, verbose=False, extra_flags=()):
    """Compile the library if any source is newer than it; return the library path."""
    if not force and not extra_flags and up_to_date():
        return LIB_PATH
    nvcc = nvcc_path()
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = sources()
    extra = list(extra_flags)
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, extra), srcs))
    objs = [r[0] for r in results]
    if verbose:
        for _, log in results:
            if log.strip():
                sys.stderr.write(log)
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc] + ARCH_FLAGS + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
