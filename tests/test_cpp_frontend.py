"""The C++ front end (include/nabo_cuda.hpp): a program written against it the
way a libnabo user writes against Nabo::NearestNeighbourSearch compiles with
g++, raises the reference's errors, and (on the GPU) returns the oracle's
results through both knn() overloads in float and double. A second program
is the reference's CTest validation (text cloud loader, knnvalidate's
queries and checks) over the same header, run on the reference's scans."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import helpers as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp_path, name="frontend_check"):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    lib = os.path.join(ROOT, "libnabo_gb300", "lib")
    if not os.path.exists(os.path.join(lib, "libnabo_gb300.so")):
        pytest.skip("library not built")
    exe = str(tmp_path / name)
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-Wall", "-Wextra", "-Werror", "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", f"{name}.cpp"), "-L", lib,
                    "-lnabo_gb300", f"-Wl,-rpath,{lib}", "-o", exe], check=True, capture_output=True, text=True)
    return exe


def _write_text_cloud(path, arr, sep=" "):
    """A cloud in the reference's text format: one point per line."""
    with open(path, "w") as f:
        for row in arr:
            f.write(sep.join(repr(float(v)) for v in row) + "\n")


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
    # 9 checks per scalar type, 2 of them through the Matrix3X-like and the
    # mapped cloud types
    assert "FAIL" not in r.stdout and r.stdout.count("ok ") == 18, r.stdout
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


def test_text_loader_reads_like_the_reference(tmp_path, ref_scans):
    """tests/helpers.h:46-80: any run of space, tab, comma or semicolon
    separates values; the first line fixes the dimension."""
    exe = _compile(tmp_path, "knn_validate")
    mixed = tmp_path / "mixed.txt"
    mixed.write_text("1.5,\t-2e-3 ;7\n4 5 6\n\n0.125;0.25,,0.5\n")
    r = subprocess.run([exe, "--parse", str(mixed)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.split("\n")
    assert lines[0] == "dim 3 points 3"
    assert [float(v) for v in lines[1].split()] == [1.5, -2e-3, 7.0]
    assert [float(v) for v in lines[3].split()] == [0.125, 0.25, 0.5]
    scan = ref_scans["scan_3d"]
    path = tmp_path / "scan.3d.txt"
    _write_text_cloud(path, scan, sep="   ")
    r = subprocess.run([exe, "--parse", str(path)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.split("\n")[0] == f"dim 3 points {scan.shape[0]}"
    assert [float(v) for v in r.stdout.split("\n")[1].split()] == list(scan[0])
    r = subprocess.run([exe, str(tmp_path / "missing.txt"), "10", "3", "-1"], capture_output=True, text=True)
    assert r.returncode == 2 and "Cannot open file" in r.stderr
    r = subprocess.run([exe, str(path), "10", "2", "-1"], capture_output=True, text=True)
    assert r.returncode == 2 and "requested dimensions were 2" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("case", H.KNNVALIDATE_CASES, ids=lambda c: f"{c[0]}-{c[3]}-{c[4]}")
def test_knn_validate_program_on_reference_scans(tmp_path, ref_scans, case):
    """tests/CMakeLists.txt:9-14, one CTest line each: KDTREE_CUDA against
    BRUTE_FORCE_CUDA on the reference's scans, float and double."""
    name, k, dim, method, radius = case
    exe = _compile(tmp_path, "knn_validate")
    path = tmp_path / f"{name}.txt"
    _write_text_cloud(path, ref_scans[name])
    args = [exe, str(path), str(k), str(dim), str(method)] + ([] if np.isinf(radius) else [str(radius)])
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok ") == 2, r.stdout
