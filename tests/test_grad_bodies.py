"""The generated ERI-gradient class bodies, checked on the host.

gen_grad.py emits, for each of the 36 ordered quartet classes, the ket sums of
one primitive quartet (GradPrim) and the density contraction of one bra
primitive pair (GradContract).  tests/grad_host compiles exactly that
generated code with the host C++ compiler, runs it over every ket chunk and
bra primitive of one quartet of contracted shells (random exponents,
coefficients, centres and density values), and compares the derivatives with
respect to the bra's first centre and to both bra centres moved together with
central finite differences (h = 1e-4 bohr) of sum Gamma (ab|cd) computed by an
independent McMurchie-Davidson evaluation: relative agreement 1e-6.  The
device kernels (grad_kernel.cuh) wrap these same bodies; the -m gpu tests
check the assembled gradient against finite differences of the energy."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "hfsolver_gb300", "csrc")
HOST = os.path.join(HERE, "grad_host")


def _cxx():
    for c in ("g++", "c++"):
        if shutil.which(c):
            return c
    return None


@pytest.mark.skipif(_cxx() is None, reason="no host C++ compiler")
def test_generated_gradient_bodies_match_finite_differences(tmp_path):
    gen = tmp_path / "gen"
    subprocess.run([sys.executable, os.path.join(CSRC, "gen_grad.py"), str(gen)], check=True, capture_output=True)
    subprocess.run([sys.executable, os.path.join(HOST, "make_checks.py"), str(gen), str(tmp_path)], check=True)
    for f in ("common.h", "ref.cpp", "records.cpp"):
        shutil.copy(os.path.join(HOST, f), tmp_path / f)
    srcs = sorted(str(p) for p in (tmp_path / "cls").glob("*.cpp")) + [
        str(tmp_path / f) for f in ("ref.cpp", "records.cpp", "main.cpp")]
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    flags = ["-std=c++17", "-O1", "-w", "-I", str(tmp_path), "-I", CSRC, "-I", cuda_inc]

    def compile_one(src):
        obj = src[:-4] + ".o"
        r = subprocess.run([_cxx(), *flags, "-c", src, "-o", obj], capture_output=True, text=True)
        return obj, r.returncode, r.stderr[-2000:]

    with cf.ThreadPoolExecutor(max(2, os.cpu_count() or 2)) as ex:
        results = list(ex.map(compile_one, srcs))
    for obj, rc, err in results:
        assert rc == 0, err
    exe = str(tmp_path / "check")
    subprocess.run([_cxx(), "-o", exe, *[o for o, _, _ in results]], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-4000:]
    assert r.stdout.count(": ok") == 36, r.stdout
