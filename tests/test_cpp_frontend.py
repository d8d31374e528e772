"""The C++ front end (include/nabo_cuda.hpp): a program written against it the
way a libnabo user writes against Nabo::NearestNeighbourSearch compiles with
g++, raises the reference's errors, and (on the GPU) returns the oracle's
results through both knn() overloads in float and double."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    lib = os.path.join(ROOT, "libnabo_gb300", "lib")
    if not os.path.exists(os.path.join(lib, "libnabo_gb300.so")):
        pytest.skip("library not built")
    exe = str(tmp_path / "frontend_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "frontend_check.cpp"), "-L", lib, "-lnabo_gb300",
                    f"-Wl,-rpath,{lib}", "-o", exe], check=True, capture_output=True, text=True)
    return exe


def test_cpp_frontend_compiles_and_rejects_bad_arguments(tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe, "errors"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok ") == 4


@pytest.mark.gpu
def test_cpp_frontend_search_matches_oracle(tmp_path):
    from libnabo_gb300 import synthetic as S
    from oracle import oracle as O
    exe = _compile(tmp_path)
    n, nq, k, dim = 20000, 3001, 7, 3
    cloud = S.uniform(n, dim, seed=21)
    q = S.uniform(nq, dim, seed=22)
    radii = np.random.default_rng(23).uniform(0.01, 0.1, nq).astype(np.float32)
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as f:
        np.array([n, nq, k, dim], np.int32).tofile(f)
        cloud.tofile(f)
        q.tofile(f)
        radii.tofile(f)
    r = subprocess.run([exe, "search", inp, out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout and r.stdout.count("ok ") == 14, r.stdout
    raw = open(out, "rb").read()
    off = 0

    def take(dt, count):
        nonlocal off
        a = np.frombuffer(raw, dtype=dt, count=count, offset=off)
        off += a.nbytes
        return a

    for T in (np.float32, np.float64):
        c, qq, rr = cloud.astype(T), q.astype(T), radii.astype(T)
        tree = O.OracleTree(c, creation_flags=O.TOUCH_STATISTICS)
        oi, od, ot = tree.knn(qq, k, 0.0, 2, 1.0, mode=O.MODE_CANONICAL)
        gi = take(np.int32, k * nq).reshape(nq, k)
        gd = take(T, k * nq).reshape(nq, k)
        assert np.array_equal(gi, oi) and np.array_equal(gd, od), T
        oi2, od2, _ = tree.knn(qq, k, max_radii=rr, mode=O.MODE_CANONICAL)
        gi2 = take(np.int32, k * nq).reshape(nq, k)
        gd2 = take(T, k * nq).reshape(nq, k)
        assert np.array_equal(gi2, oi2) and np.array_equal(gd2, od2), T
        assert int(take(np.uint64, 1)[0]) == int(ot), T
