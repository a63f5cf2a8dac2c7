"""The C-ABI library: builds, loads without a GPU, exports every entry point
declared in include/sis_gpu.h, and its structs have the layout the Python
binding assumes.  No compute call is made here."""
import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "sis_gpu.h"
FMODULE = ROOT / "include" / "sis_gpu.f90"


@pytest.fixture(scope="module")
def lib():
    from sis_gb300.build import build_lib

    build_lib()
    from sis_gb300 import _abi

    return _abi.lib()


def declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(sis_gpu_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    names = declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    from sis_gb300 import _abi

    assert set(names) == set(_abi.EXPORTS)


def test_no_oracle_symbols_in_product(lib):
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", str(ROOT / "sis_gb300" / "_lib" / "libsisgpu.so")], capture_output=True, text=True).stdout
    assert "or_force" not in out and "or_create" not in out


def test_struct_layout_matches_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from sis_gb300 import _abi

    src = tmp_path / "layout.c"
    fields = {s.__name__: [f for f, _ in s._fields_] for s in (_abi.sis_params, _abi.sis_topology, _abi.sis_stats)}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for s, fs in fields.items():
        lines.append(f'printf("{s} %zu\\n", sizeof({s}));')
        for f in fs:
            lines.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for s in (_abi.sis_params, _abi.sis_topology, _abi.sis_stats):
        assert int(got[s.__name__]) == C.sizeof(s), s.__name__
        for f, _ in s._fields_:
            assert int(got[f"{s.__name__}.{f}"]) == getattr(s, f).offset, f


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from sis_gb300 import _abi

    monkeypatch.setattr(_abi, "_lib", None)
    monkeypatch.setattr(_abi, "LIB_PATH", tmp_path / "absent.so")
    with pytest.raises(RuntimeError):
        _abi.lib()


def _c_params(text):
    """Parameter count of every sis_gpu_* declaration in the header."""
    out = {}
    decl = r"^[ \t]*(?:const[ \t]+)?\w+[ \t]*\**[ \t]*(sis_gpu_\w+)\s*\(([^;]*?)\)\s*;"
    for name, params in re.findall(decl, text, flags=re.S | re.M):
        params = params.strip()
        out[name] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_fortran_bindings_match_the_header():
    """The ISO_C_BINDING interfaces of include/sis_gpu.f90 bind names the
    header declares, with as many arguments; every entry point the module and
    INTEGRATION.md name exists."""
    c = _c_params(HEADER.read_text())
    mod = FMODULE.read_text()
    binds = re.findall(r"function\s+(\w+)\s*\(([^)]*)\)\s*&?\s*bind\(C,\s*name=\"(\w+)\"\)", mod)
    assert len(binds) >= 20
    for fname, args, cname in binds:
        assert fname == cname and cname in c, cname
        nargs = len([a for a in args.split(",") if a.strip()])
        assert nargs == c[cname], (cname, nargs, c[cname])
    doc = mod + (ROOT / "INTEGRATION.md").read_text()
    named = set(re.findall(r"\bsis_gpu_\w+", doc)) - {"sis_gpu_mod"}
    assert named <= set(c), named - set(c)


def test_header_is_plain_c_and_links(lib, tmp_path):
    """include/sis_gpu.h is plain C99 (-pedantic), and a C program that takes
    the address of every entry point links against the library (nothing is
    run)."""
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    names = declared()
    src = tmp_path / "use.c"
    src.write_text('#include "sis_gpu.h"\n#include <stdio.h>\nint main(void) {\n'
                   + "".join(f'    printf("%p\\n", (void *)&{n});\n' for n in names)
                   + "    return 0;\n}\n")
    hdr = tmp_path / "hdr.c"
    hdr.write_text('#include "sis_gpu.h"\nint sis_header_check(void) { return (int)sizeof(sis_params); }\n')
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", f"-I{ROOT / 'include'}",
                        "-fsyntax-only", str(hdr)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    libdir = ROOT / "sis_gb300" / "_lib"
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src), f"-L{libdir}",
                        "-lsisgpu", "-o", str(tmp_path / "use")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _c_struct_fields(text, name):
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", text, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    ctype = {"double": "real(c_double)", "int32_t": "integer(c_int32_t)", "uint64_t": "integer(c_int64_t)",
             "int64_t": "integer(c_int64_t)"}
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(?:const\s+)?(\w+)\s*(\**)\s*(.*)", decl, flags=re.S)
        base, star, rest = m.groups()
        for var in rest.split(","):
            var = var.strip()
            ptr_ = star or var.startswith("*")
            nm = re.match(r"\**\s*(\w+)", var).group(1)
            n = 1
            for d in re.findall(r"\[(\d+)\]", var):
                n *= int(d)
            out.append((nm.lower(), "type(c_ptr)" if ptr_ else ctype[base], n))
    return out


def _fortran_type_fields(doc, name):
    body = re.search(r"type, bind\(C\) :: " + name + r"\n(.*?)\n\s*end type", doc, flags=re.S).group(1)
    out = []
    for line in body.splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        ftype, names = (x.strip() for x in line.split("::"))
        for var in re.findall(r"(\w+)(\([^)]*\))?", names):
            n = 1
            for d in re.findall(r"\d+", var[1]):
                n *= int(d)
            out.append((var[0].lower(), ftype.replace(" ", ""), n))
    return out


@pytest.mark.parametrize("name", ["sis_params", "sis_topology", "sis_stats"])
def test_fortran_struct_types_match_the_header(name):
    """The bind(C) derived types of include/sis_gpu.f90 list the C structs'
    fields in order, with matching kinds and array sizes."""
    c = _c_struct_fields(HEADER.read_text(), name)
    f = _fortran_type_fields(FMODULE.read_text(), name)
    assert f == c


def _c_param_lists(text):
    decl = r"^[ \t]*(?:const[ \t]+)?\w+[ \t]*\**[ \t]*(sis_gpu_\w+)\s*\(([^;]*?)\)\s*;"
    out = {}
    for name, params in re.findall(decl, text, flags=re.S | re.M):
        ps = []
        for prm in params.split(","):
            prm = prm.strip()
            if not prm or prm == "void":
                continue
            m = re.match(r"(?:const\s+)?(\w+)\s*(\**)\s*(\w+)$", prm)
            base, stars, pname = m.groups()
            ps.append((pname.lower(), base, len(stars)))
        out[name] = ps
    return out


def test_fortran_argument_kinds_match_the_header():
    """Each dummy argument of the ISO_C_BINDING interfaces passes what the C
    parameter in the same position expects: scalars by value with the same
    kind, pointers as type(c_ptr) by value or as an array or scalar by
    reference of the same kind."""
    kind = {"double": "real(c_double)", "int32_t": "integer(c_int32_t)", "int64_t": "integer(c_int64_t)",
            "uint64_t": "integer(c_int64_t)", "uint8_t": "integer(c_int8_t)", "float": "real(c_float)",
            "sis_ctx": "type(c_ptr)", "sis_topology": "type(sis_topology)", "sis_params": "type(sis_params)",
            "sis_stats": "type(sis_stats)"}
    c = _c_param_lists(HEADER.read_text())
    doc = FMODULE.read_text()
    blocks = re.findall(r"(?:function|subroutine)\s+\w+\s*\(([^)]*)\)\s*&?\s*bind\(C,\s*name=\"(\w+)\"\)(.*?)end (?:function|subroutine)",
                        doc, flags=re.S)
    checked = 0
    for args, cname, body in blocks:
        f = {}
        for line in body.splitlines():
            line = line.split("!")[0].strip()
            if "::" not in line or line.startswith("import"):
                continue
            attrs, names = (x.strip() for x in line.split("::"))
            parts = [a.strip() for a in re.split(r",(?![^(]*\))", attrs)]
            ftype, by_value = parts[0].replace(" ", ""), "value" in parts[1:]
            for nm in re.findall(r"(\w+)(?:\([^)]*\))?", names):
                f[nm.lower()] = (ftype, by_value)
        fargs = [a.strip().lower() for a in args.split(",") if a.strip()]
        assert len(fargs) == len(c[cname]), cname
        for (pname, base, stars), farg in zip(c[cname], fargs):
            ftype, by_value = f[farg]
            if stars == 0:
                assert by_value and ftype == kind[base], (cname, pname)
            elif base == "sis_ctx" and stars == 1:
                assert by_value and ftype == "type(c_ptr)", (cname, pname)
            elif stars == 1:
                assert (by_value and ftype == "type(c_ptr)") or (not by_value and ftype == kind[base]), (cname, pname)
            else:  # sis_ctx **: the handle returned by reference
                assert not by_value and ftype == "type(c_ptr)", (cname, pname)
            checked += 1
    assert checked >= 60


def test_ctypes_argtypes_match_the_header():
    """sis_gb300._abi declares every entry point with the header's parameter
    count and kinds (pointers as c_void_p or a POINTER, scalars by their
    width) and an int status (or the header's return type)."""
    from sis_gb300 import _abi

    scalar = {"double": C.c_double, "int32_t": C.c_int32, "int64_t": C.c_int64, "uint64_t": C.c_uint64,
              "uint32_t": C.c_uint32, "float": C.c_float}
    text = HEADER.read_text()
    c = _c_param_lists(text)
    rets = dict((n, r.strip()) for r, n in re.findall(r"^[ \t]*((?:const[ \t]+)?\w+[ \t]*\**)[ \t]*(sis_gpu_\w+)\s*\(",
                                                      text, flags=re.M))
    ret_kind = {"int": C.c_int, "void": None, "const char *": C.c_char_p, "int64_t": C.c_int64}
    for name, (restype, argtypes) in _abi.EXPORTS.items():
        assert restype is ret_kind[" ".join(rets[name].replace("*", " *").split())], name
        params = c[name]
        assert len(argtypes) == len(params), name
        for (pname, base, stars), at in zip(params, argtypes):
            if stars:
                assert at is C.c_void_p or at is C.c_char_p or hasattr(at, "_type_") and issubclass(at, C._Pointer), \
                    (name, pname, at)
            else:
                assert at is scalar[base], (name, pname, at)
