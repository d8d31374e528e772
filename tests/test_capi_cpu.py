"""C-ABI checks that need no GPU: the in-tree library loads, exports every
function include/nabo_gb300.h declares, and rejects bad create() arguments
with the reference's messages before touching the device."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "nabo_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nabo_cuda_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from libnabo_gb300 import _native
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(_native.lib, n), f"{n} not exported"
        assert n in _native.SIGNATURES, f"{n} has no ctypes signature"
    assert set(_native.SIGNATURES) == set(names)


def test_params_defaults():
    from libnabo_gb300 import _native
    p = _native.nabo_cuda_params()
    _native.lib.nabo_cuda_params_init(ctypes.byref(p))
    assert p.bucketSize == 8 and p.queryOrdering == 1 and p.struct_size == ctypes.sizeof(p)
    assert p.pipelineChunks == 0 and ctypes.sizeof(p) == 32


def test_version():
    import libnabo_gb300 as nb
    assert nb.version() == "0.1.0"


@pytest.mark.parametrize("kwargs,msg,code", [
    (dict(dim=0), "Your space must have at least one dimension", 1),
    (dict(params={"bucketSize": 1}), "Requested bucket size 1, but must be larger than 2", 1),
    (dict(params={"bucketSize": 0}), "Requested bucket size 0, but must be larger than 2", 1),
    (dict(searchType=1), "only the CUDA search types", 3),
    (dict(searchType=99), "Unknown search type", 1),
    (dict(params={"pipelineChunks": 65}), "pipelineChunks must be between 0 and 64", 1),
    (dict(params={"pipelineChunks": -1}), "pipelineChunks must be between 0 and 64", 1),
])
def test_create_argument_errors(kwargs, msg, code):
    import libnabo_gb300 as nb
    cloud = np.random.default_rng(0).random((50, 3)).astype(np.float32)
    with pytest.raises(nb.NaboError) as ei:
        nb.NearestNeighbourSearch(cloud, **kwargs)
    assert msg in str(ei.value)
    assert ei.value.code == code


def test_create_empty_cloud_errors():
    import libnabo_gb300 as nb
    with pytest.raises(nb.NaboError, match="Cloud has no points"):
        nb.NearestNeighbourSearch(np.zeros((0, 3), np.float32))
    with pytest.raises(nb.NaboError, match="Cloud has 0 dimensions"):
        nb.NearestNeighbourSearch(np.zeros((5, 0), np.float32))


def test_create_messages_match_oracle():
    import libnabo_gb300 as nb
    from oracle import oracle as O
    cloud = np.random.default_rng(1).random((40, 3)).astype(np.float32)
    for bs in (0, 1):
        with pytest.raises(O.OracleError) as eo:
            O.OracleTree(cloud, bucket_size=bs)
        with pytest.raises(nb.NaboError) as eg:
            nb.NearestNeighbourSearch(cloud, params={"bucketSize": bs})
        assert str(eo.value) == str(eg.value)


def test_c_header_compiles_links_and_runs_as_c99(tmp_path):
    """include/nabo_gb300.h is a C header: a C99 program includes it with
    every warning on, links the library and calls what needs no GPU."""
    import os
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = os.path.join(root, "libnabo_gb300", "lib")
    src = tmp_path / "c_check.c"
    src.write_text(
        '#include <stdio.h>\n#include "nabo_gb300.h"\n'
        "int main(void) {\n"
        "  nabo_cuda_params p;\n  nabo_cuda_search* s = 0;\n"
        "  nabo_cuda_params_init(&p);\n"
        "  if (p.bucketSize != 8 || p.struct_size != sizeof p) return 1;\n"
        "  if (nabo_cuda_create(NABO_CUDA_FLOAT32, 0, 3, 0, 3, 0, 6, 0, &p, &s) == 0) return 2;\n"
        '  printf("%s|%s\\n", nabo_cuda_version(), nabo_cuda_last_error());\n'
        "  return 0;\n}\n")
    exe = tmp_path / "c_check"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Wpedantic", "-Werror", "-I", os.path.join(root, "include"),
                    str(src), "-L", lib, "-lnabo_gb300", f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("0.1.0|") and "Your space must have at least one dimension" in r.stdout
