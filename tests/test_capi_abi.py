"""The C-ABI library loads and exports every symbol include/adscf.h declares
(CPU only: no compute calls)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "adscf.h").read_text()
    return sorted(set(re.findall(r"ADSCF_API[^;(]*?\b(adscf_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("adscf_ctx_create", "adscf_propagate_diblock", "adscf_mix",
                 "adscf_scf_run", "adscf_propagate_step", "adscf_mean_fields"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_binding_covers_every_declared_symbol():
    from adscf_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_struct_layout_matches_c(tmp_path):
    """sizeof of the ABI structs seen by C equals the ctypes mirror."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include "adscf.h"\nint main(){printf("%zu %zu %zu",'
                   ' sizeof(adscf_params), sizeof(adscf_chain_result), sizeof(adscf_iter_result));}')
    exe = tmp_path / "sz"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    from adscf_gb300 import _lib
    assert [int(v) for v in out] == [ctypes.sizeof(_lib.Params), ctypes.sizeof(_lib.ChainResult),
                                     ctypes.sizeof(_lib.IterResult)]


def test_status_strings_without_gpu(lib):
    assert lib.adscf_abi_version() == 2
    assert lib.adscf_status_string(3).decode() == "zero tridiagonal pivot"


def test_missing_library_fails_loudly(tmp_path):
    from adscf_gb300 import _lib
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load(tmp_path / "nope.so")
