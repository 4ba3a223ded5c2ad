"""Build libhfgpu.so in-tree for sm_103a.

Generates the ERI and ERI-gradient class bodies (csrc/gen_eri.py,
csrc/gen_grad.py), compiles every translation
unit with nvcc in parallel (objects cached in csrc/_build by content hash of
the source and the local headers), and links hfsolver_gb300/libhfgpu.so
against cudart, cuBLAS and cuSOLVER.
"""
import concurrent.futures as cf
import hashlib
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(CSRC, "_build")
LIB = os.path.join(PKG, "libhfgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              *ARCH]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.exists(c) or c == "nvcc"):
            return c
    return "nvcc"


def _sources():
    for gen in ("gen_eri.py", "gen_grad.py"):
        subprocess.run([sys.executable, os.path.join(CSRC, gen)], check=True, capture_output=True)
    srcs = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cpp"))]
    gen = os.path.join(CSRC, "gen")
    srcs += [os.path.join(gen, f) for f in sorted(os.listdir(gen)) if f.endswith(".cu")]
    # largest first so the longest compiles start early
    return sorted(srcs, key=lambda p: -os.path.getsize(p))


def _headers_digest():
    h = hashlib.sha256()
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".h", ".cuh")):
            h.update(open(os.path.join(CSRC, f), "rb").read())
    h.update(open(os.path.join(PKG, "..", "include", "hfgpu.h"), "rb").read())
    h.update(" ".join(NVCC_FLAGS).encode())
    return h.hexdigest()


def _compile(src, hdr):
    key = hashlib.sha256(open(src, "rb").read() + hdr.encode()).hexdigest()[:16]
    obj = os.path.join(BUILD, os.path.basename(src) + "." + key + ".o")
    if os.path.exists(obj):
        return obj, None
    cmd = [_nvcc(), *NVCC_FLAGS, "-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return None, " ".join(cmd) + "\n" + r.stdout + r.stderr
    os.replace(obj + ".tmp", obj)
    return obj, None


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    hdr = _headers_digest()
    jobs = jobs or max(2, os.cpu_count() or 2)
    objs = []
    with cf.ThreadPoolExecutor(jobs) as ex:
        for src, (obj, err) in zip(srcs, ex.map(lambda s: _compile(s, hdr), srcs)):
            if err:
                raise RuntimeError("nvcc failed for " + src + ":\n" + err)
            objs.append(obj)
            if verbose:
                print("compiled", os.path.basename(src))
    cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcublas", "-lcusolver"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    # drop stale objects
    keep = set(objs)
    for f in os.listdir(BUILD):
        p = os.path.join(BUILD, f)
        if p not in keep and f.endswith(".o"):
            os.remove(p)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
