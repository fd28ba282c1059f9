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


def _c_struct_members(name):
    """Member names, in order, of `typedef struct name {...} name;` in adscf.h."""
    text = (ROOT / "include" / "adscf.h").read_text()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        decl = re.sub(r"^(const )?(unsigned )?\w+ \*?", "", decl)
        for d in decl.split(","):
            names.append(re.sub(r"[\s*]|\[.*\]", "", d))
    return names


def _fortran_members(tname):
    text = (ROOT / "include" / "adscf.f90").read_text()
    body = re.search(r"type, bind\(C\) :: %s\n(.*?)end type" % tname, text, re.S).group(1)
    names = []
    for line in body.splitlines():
        line = line.split("!")[0]
        if "::" not in line:
            continue
        for d in line.split("::")[1].split(","):
            names.append(re.sub(r"\(.*\)", "", d).strip())
    return names


CTYPES_NAME = {"lambda": "lam"}   # `lambda` is a Python keyword


@pytest.mark.parametrize("cname,pyname", [("adscf_params", "Params"),
                                          ("adscf_chain_result", "ChainResult"),
                                          ("adscf_iter_result", "IterResult")])
def test_struct_field_offsets_match_c(tmp_path, cname, pyname):
    """offsetof of every member seen by gcc equals the ctypes mirror's offset,
    and the Fortran bind(C) type lists the same members in the same order."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    members = _c_struct_members(cname)
    prog = ['#include <stdio.h>', '#include <stddef.h>', '#include "adscf.h"', "int main(){"]
    prog += ['printf("%%zu\\n", offsetof(%s, %s));' % (cname, m) for m in members]
    prog += ["return 0;}"]
    src = tmp_path / "off.c"
    src.write_text("\n".join(prog))
    exe = tmp_path / "off"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    offs = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                           check=True).stdout.split()]
    from adscf_gb300 import _lib
    cls = getattr(_lib, pyname)
    py = [getattr(cls, CTYPES_NAME.get(m, m)).offset for m in members]
    assert offs == py, list(zip(members, offs, py))
    assert [f[0] for f in cls._fields_] == [CTYPES_NAME.get(m, m) for m in members]
    assert _fortran_members(cname) == members


SHIMS = ("adscf_shim_state.f90", "adscf_shim.f90", "adscf_shim_film.f90", "adscf_shim_brush.f90")

# Global members each driver family declares (Bulk_3D_FFT/Main_Diblock_Melt,
# Film_CK_AD/Film_*/Main_Diblock_Melt and Brush_CK_AD/Main_brush
# mod_global.f90) that the shims read; the shared state module may use only
# the members all of them declare
GLOBAL_ONLY = {
    "adscf_shim_state.f90": {"dz", "int_scheme", "dvol", "volume"},
    "adscf_shim.f90": {"dz", "int_scheme"},
    "adscf_shim_film.f90": {"dvol"},
    "adscf_shim_brush.f90": {"dvol"},
}


def _code(text):
    return "\n".join(line.split("!")[0] for line in text.splitlines())


def test_fortran_binding_names_declared_symbols():
    """Every bind(C) name of the Fortran binding is an entry point of the
    header, the shims keep the reference's module procedure names, and they
    call only bound entry points."""
    decl = set(declared_symbols())
    f90 = (ROOT / "include" / "adscf.f90").read_text()
    bound = re.findall(r'bind\(C, name="(\w+)"\)', f90)
    assert bound and set(bound) <= decl
    text = {f: (ROOT / "include" / f).read_text() for f in SHIMS}
    want_mods = {
        "adscf_shim_state.f90": ("adscf_shim_state",),
        "adscf_shim.f90": ("Propagate", "Molecule_Diblock_Copolymer", "Molecule_Solvent", "Iterate"),
        "adscf_shim_film.f90": ("RealSpace_adscf", "Molecule_Diblock_Copolymer"),
        "adscf_shim_brush.f90": ("RealSpace_adscf",),
    }
    want_procs = {
        "adscf_shim.f90": ("Calculate_Expfield", "Propagate_Step", "Initialize_Diblock", "Propagate_Diblock",
                           "Initialize_Solvent", "Update_Solvent", "Mixing_Simple", "Mixing_Lambda",
                           "Mixing_Anderson"),
        "adscf_shim_film.f90": ("Propagate_Step", "integrator", "Initialize_Diblock", "Propagate_Diblock"),
        "adscf_shim_brush.f90": ("Propagate_Step", "integrator"),
    }
    for f, mods in want_mods.items():
        for mod in mods:
            assert re.search(r"^module %s$" % mod, text[f], re.M), (f, mod)
    for f, procs in want_procs.items():
        for proc in procs:
            assert re.search(r"^\s*subroutine %s\(" % proc, text[f], re.M), (f, proc)
    for f, t in text.items():
        called = set(re.findall(r"\b(adscf_\w+)\(", _code(t))) - {"adscf_check", "adscf_error_text"}
        assert called <= set(bound), (f, called - set(bound))


def test_fortran_shims_use_only_their_drivers_globals():
    """The bulk shim compiles against the bulk Global (no dz, int_scheme),
    the film and brush shims against theirs (no dvol), and the shared state
    module against any of them."""
    for f, banned in GLOBAL_ONLY.items():
        # identifiers, not derived-type components (p%dz is a member of adscf_params)
        words = set(re.findall(r"(?<![%\w])[a-z_]\w*", _code((ROOT / "include" / f).read_text()).lower()))
        assert not (words & banned), (f, words & banned)


def test_status_strings_without_gpu(lib):
    assert lib.adscf_abi_version() == 2
    assert lib.adscf_status_string(3).decode() == "zero tridiagonal pivot"


def test_invalid_params_rejected_without_gpu(lib):
    """Parameter checks run before any CUDA call: each invalid set of
    parameters returns ADSCF_E_ARG and no context."""
    import ctypes as C
    from adscf_gb300 import _lib

    dz = (C.c_double * 2)(0.5, 0.5)

    def params(**kw):
        p = _lib.Params()
        p.geometry, p.gx, p.gy, p.gz = 0, 8, 8, 8
        p.sizex = p.sizey = p.sizez = 1.0
        p.ds, p.ensemble, p.precision, p.mixing_type, p.mixing_dim = 0.01, 1, 0, 1, 2
        p.block_length[0], p.block_length[1] = 0.5, 0.5
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    cases = [dict(geometry=7), dict(gz=0), dict(precision=5), dict(mixing_type=3, mixing_dim=17),
             dict(ensemble=3), dict(ds=0.0), dict(sizex=0.0), dict(geometry=1, gx=1, gy=1),
             dict(geometry=2, gz=1, dz=C.cast(dz, C.POINTER(C.c_double))),
             dict(geometry=1, gx=1, gy=1, gz=1, dz=C.cast(dz, C.POINTER(C.c_double)))]
    for kw in cases:
        ctx = C.c_void_p()
        p = params(**kw)
        assert lib.adscf_ctx_create(C.byref(p), C.byref(ctx)) == 1, kw
        assert not ctx.value, kw
    ctx = C.c_void_p()
    assert lib.adscf_ctx_create(None, C.byref(ctx)) == 1
    # bulk batches check every instance before any CUDA call
    for kw in [dict(precision=5), dict(gz=0), dict(ds=0.0), dict(geometry=2)]:
        arr = (_lib.Params * 2)(params(), params(**kw))
        if "precision" in kw:
            arr = (_lib.Params * 2)(params(**kw), params())
        b = C.c_void_p()
        assert lib.adscf_batch_create(arr, 2, C.byref(b)) == 1, kw
        assert not b.value, kw
    b = C.c_void_p()
    assert lib.adscf_batch_create((_lib.Params * 1)(params()), 0, C.byref(b)) == 1


def test_missing_library_fails_loudly(tmp_path):
    from adscf_gb300 import _lib
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load(tmp_path / "nope.so")
