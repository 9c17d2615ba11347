"""The C ABI: the library loads and exports every symbol include/covgpu.h
declares; struct layouts agree between the header and the ctypes binding.
No compute call (no GPU needed)."""
import ctypes
import os
import subprocess
import tempfile

from coldcase_gb300 import _build, lib as L


def test_exports_every_declared_symbol(covlib):
    names = L.header_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(covlib, n)]
    assert not missing, missing
    assert set(L.SIGNATURES) <= set(names)


def test_struct_layouts_match_header():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "covgpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(cov_move_rec), sizeof(cov_params), sizeof(cov_status),
         offsetof(cov_params, stall), offsetof(cov_move_rec, ncand));
  return 0; }
'''
    with tempfile.TemporaryDirectory() as td:
        c = os.path.join(td, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(td, "t")
        subprocess.run(["gcc", "-I", _build.INCLUDE, c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    got = [int(x) for x in out]
    want = [ctypes.sizeof(L.CovMoveRec), ctypes.sizeof(L.CovParams), ctypes.sizeof(L.CovStatus),
            L.CovParams.stall.offset, L.CovMoveRec.ncand.offset]
    assert got == want


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_build, "LIBDIR", str(tmp_path))
    monkeypatch.setattr(L, "_lib", None)
    try:
        L.load()
    except L.CovError as e:
        assert "not built" in str(e)
    else:
        raise AssertionError("load() must fail without the library")
