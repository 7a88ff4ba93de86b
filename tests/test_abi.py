"""The C ABI: the library builds, loads and exports every function that
include/hsmu_gb.h declares; ctypes struct layouts match the C compiler's;
status strings.  No compute call (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HDR = os.path.join(ROOT, "include", "hsmu_gb.h")


def declared_functions():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(hsmu_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from hsmu_gb import build

    build.build()
    import hsmu_gb

    return hsmu_gb.load_library()


def test_exports_every_declared_symbol(lib):
    import hsmu_gb

    names = declared_functions()
    assert len(names) >= 10
    assert sorted(hsmu_gb.EXPORTS) == names
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", hsmu_gb.LIB_PATH], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(r" T %s$" % n, out, flags=re.M), n


def test_status_strings(lib):
    assert lib.hsmu_strerror(0) == b"ok"
    assert b"canonical" in lib.hsmu_strerror(5)
    assert lib.hsmu_strerror(99) == b"unknown status"
    assert lib.hsmu_abi_version() == 1


def test_struct_layouts(tmp_path):
    import hsmu_gb

    prog = tmp_path / "sizes.c"
    prog.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "hsmu_gb.h"\n'
                    'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(hsmu_csr),'
                    ' sizeof(hsmu_btiles), sizeof(hsmu_opts), sizeof(hsmu_stats), offsetof(hsmu_stats, ms_convert),'
                    ' offsetof(hsmu_stats, launches), sizeof(hsmu_csr64), offsetof(hsmu_csr64, nnz),'
                    ' offsetof(hsmu_csr64, row_ptr)); return 0;}\n')
    exe = str(tmp_path / "sizes")
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", exe])
    got = [int(x) for x in subprocess.check_output([exe]).split()]
    want = [ctypes.sizeof(hsmu_gb.c_csr), ctypes.sizeof(hsmu_gb.c_btiles), ctypes.sizeof(hsmu_gb.c_opts),
            ctypes.sizeof(hsmu_gb.c_stats), hsmu_gb.c_stats.ms_convert.offset, hsmu_gb.c_stats.launches.offset,
            ctypes.sizeof(hsmu_gb.c_csr64), hsmu_gb.c_csr64.nnz.offset, hsmu_gb.c_csr64.row_ptr.offset]
    assert got == want


def test_engine_refuses_without_gpu():
    import torch

    import hsmu_gb

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(hsmu_gb.HsmuError):
        hsmu_gb.Engine()
