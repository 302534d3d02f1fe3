"""The C-ABI library builds, loads, and exports every symbol include/fvm_gpu.h declares
(no compute calls: there is no GPU here)."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "fvm_gpu.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\bint\s+(fvm_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from fvmgpu import _build, _lib

    path = _build.build()
    lib = ctypes.CDLL(str(path))
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(_lib.SIGNATURES), "ctypes signatures must mirror the header"
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (fvm_\w+)", out))
    assert set(syms) <= exported


def test_version_device_count_and_last_error():
    from fvmgpu import _lib

    lib = _lib.load()
    assert lib.fvm_version() >= 10000
    n = ctypes.c_int(-1)
    assert lib.fvm_device_count(ctypes.byref(n)) == 0 and n.value >= 0
    buf = ctypes.create_string_buffer(64)
    assert lib.fvm_last_error(buf, len(buf)) == 0
    assert lib.fvm_last_error(None, 0) == _lib.FVM_ERR_INVALID_ARGUMENT


def test_null_arguments_return_status_not_crash():
    from fvmgpu import _lib

    lib = _lib.load()
    assert lib.fvm_mesh_create(None, 0, None, 0, None, None, 0, 0, 0, None) == _lib.FVM_ERR_INVALID_ARGUMENT
    assert lib.fvm_rhs(None, None, None, 0.0, 0, None) == _lib.FVM_ERR_INVALID_ARGUMENT
    assert lib.fvm_problem_create(None, None, None) == _lib.FVM_ERR_INVALID_ARGUMENT
    assert lib.fvm_template_create(None, 0, None) == _lib.FVM_ERR_INVALID_ARGUMENT
    assert "NULL" in _lib.last_error() or _lib.last_error()


def test_no_cpu_fallback_without_gpu():
    """The product path refuses to run without a device (there is no CPU fallback)."""
    from fvmgpu import _lib

    if _lib.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.require_gpu()


STRUCTS = {  # C struct in include/fvm_gpu.h -> its ctypes mirror in fvmgpu/_lib.py
    "fvm_problem_desc": "ProblemDesc",
    "fvm_system_desc": "SystemDesc",
    "fvm_ode_options": "OdeOptions",
    "fvm_ode_stats": "OdeStats",
    "fvm_solver_options": "SolverOptions",
    "fvm_solver_stats": "SolverStats",
    "fvm_adjoint_stats": "AdjointStats",
    "fvm_implicit_stats": "ImplicitStats",
    "fvm_steady_options": "SteadyOptions",
    "fvm_steady_stats": "SteadyStats",
}


def test_ctypes_structures_match_the_header_layout(tmp_path):
    """Every field of every C-ABI struct has the same name order, offset and size in the ctypes
    mirror as the C compiler gives it (a mismatch would pass arguments silently corrupted)."""
    from fvmgpu import _lib

    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        st = getattr(_lib, pyname)
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for field, _ in st._fields_:
            lines.append(f'printf("{cname} {field} %zu %zu\\n", offsetof({cname}, {field}), '
                         f'sizeof((({cname}*)0)->{field}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in filter(None, out):
        parts = line.split()
        got[(parts[0], parts[1])] = tuple(int(v) for v in parts[2:])
    for cname, pyname in STRUCTS.items():
        st = getattr(_lib, pyname)
        assert got[(cname, "sizeof")] == (ctypes.sizeof(st),), cname
        for field, _ in st._fields_:
            desc = getattr(st, field)
            assert got[(cname, field)] == (desc.offset, desc.size), (cname, field)
    # and the ctypes mirrors name every field of the C structs, in order
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    for cname, pyname in STRUCTS.items():
        body = re.search(r"typedef struct " + cname + r" \{(.*?)\}", text, flags=re.S).group(1)
        names = re.findall(r"(\w+)\s*(?:\[[^\]]*\])?\s*[;,]", body)
        assert names == [f for f, _ in getattr(_lib, pyname)._fields_], cname


JULIA = ROOT / "finitevolumemethod.jl_gb300" / "julia" / "FiniteVolumeMethodGPU" / "src" / "FiniteVolumeMethodGPU.jl"
JULIA_STRUCTS = {"ProblemDesc": "fvm_problem_desc", "SystemDesc": "fvm_system_desc", "OdeOptions": "fvm_ode_options",
                 "OdeStats": "fvm_ode_stats", "SolverOptions": "fvm_solver_options", "SolverStats": "fvm_solver_stats",
                 "AdjointStats": "fvm_adjoint_stats", "ImplicitStats": "fvm_implicit_stats",
                 "SteadyOptions": "fvm_steady_options", "SteadyStats": "fvm_steady_stats"}
JULIA_SIZES = {"Int8": 1, "Int32": 4, "Cint": 4, "Int64": 8, "Float64": 8}


def test_julia_binding_structures_match_the_header_layout():
    """The Julia binding cannot run here (no Julia), but its ccall structures can be checked: laid
    out with C rules from their field types (isbits structs are C-compatible), each must give
    the header's field names, offsets and size, the same as the ctypes mirrors do."""
    from fvmgpu import _lib

    text = JULIA.read_text()
    for jname, cname in JULIA_STRUCTS.items():
        body = re.search(r"^(?:mutable )?struct " + jname + r"\n(.*?)^end", text, flags=re.S | re.M).group(1)
        fields = re.findall(r"^\s*(\w+)::([\w{}]+)\s*$", body, flags=re.M)
        pyst = getattr(_lib, STRUCTS_BY_C[cname])
        assert [f for f, _ in fields] == [f for f, _ in pyst._fields_], jname
        off = 0
        align = 1
        for (f, ty), (_, _) in zip(fields, pyst._fields_):
            size = 8 if ty.startswith("Ptr") else JULIA_SIZES[ty]
            off = (off + size - 1) // size * size
            assert off == getattr(pyst, f).offset and size == getattr(pyst, f).size, (jname, f)
            off += size
            align = max(align, size)
        assert (off + align - 1) // align * align == ctypes.sizeof(pyst), jname


STRUCTS_BY_C = {c: p for c, p in STRUCTS.items()}


def _c_prototypes():
    """name -> list of parameter types (whitespace-normalised) of every fvm_* entry point."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for name, params in re.findall(r"\bint\s+(fvm_\w+)\s*\(([^)]*)\)\s*;", text):
        types = []
        for p in params.split(","):
            p = " ".join(p.split())
            if p in ("void", ""):
                continue
            types.append(re.sub(r"\s*\w+$", "", p).replace(" *", "*"))  # drop the parameter name
        out[name] = types
    return out


def _julia_type(c):
    """The Julia ccall type a C parameter type takes (by value or through a pointer)."""
    c = c.replace("const ", "")
    scalars = {"double": "Float64", "int32_t": "Int32", "int64_t": "Int64", "size_t": "Csize_t", "int": "Cint",
               "int8_t": "Int8", "char": "UInt8"}
    if c.endswith("**"):
        return {"Ref{Ptr{Cvoid}}"}
    if c.endswith("*"):
        base = c[:-1]
        if base in scalars:  # an array, or one value written back through a Ref
            return {f"Ptr{{{scalars[base]}}}", f"Ref{{{scalars[base]}}}"}
        if base in ("void", "fvm_mesh", "fvm_problem", "fvm_system", "fvm_template", "fvm_batch", "fvm_adjoint"):
            return {"Ptr{Cvoid}"}
        return {"Ref{" + {v: k for k, v in JULIA_STRUCTS.items()}[base] + "}"}  # a struct, passed by reference
    return {scalars[c]}


def test_julia_ccalls_match_the_header_prototypes():
    """Each ccall of the Julia binding passes as many arguments as the C prototype has, each of a
    Julia type that the C parameter type takes."""
    protos = _c_prototypes()
    text = JULIA.read_text()
    calls = re.findall(r"ccall\(\(:(fvm_\w+), libfvmgpu\), Cint,\s*\(([^()]*(?:\([^()]*\)[^()]*)*)\)", text)
    assert len(calls) >= 30
    # every entry point a user of the reference needs is bound
    bound = {name for name, _ in calls}
    for name in ("fvm_template_create", "fvm_template_tsit5_solve", "fvm_template_steady_solve", "fvm_batch_create",
                 "fvm_batch_tsit5_solve", "fvm_adjoint_forward", "fvm_adjoint_pullback", "fvm_mesh_locate",
                 "fvm_pl_interpolate", "fvm_system_tsit5_solve", "fvm_tsit5_solve", "fvm_jvp", "fvm_trbdf2_solve", "fvm_template_trbdf2_solve"):
        assert name in bound, name
    for name, types in calls:
        jt = [t.strip() for t in re.split(r",(?![^{]*\})", types) if t.strip()]
        ct = protos[name]
        assert len(jt) == len(ct), (name, jt, ct)
        for j, c in zip(jt, ct):
            assert j in _julia_type(c), (name, j, c)


def test_ctypes_signatures_match_the_header_prototypes():
    """Each ctypes signature has the C prototype's arity, an int result, and an argument type the
    C parameter type takes (pointers as typed pointers or void pointers)."""
    from fvmgpu import _lib

    scalars = {"double": ctypes.c_double, "int32_t": ctypes.c_int32, "int64_t": ctypes.c_int64,
               "size_t": ctypes.c_size_t, "int": ctypes.c_int, "int8_t": ctypes.c_int8, "char": ctypes.c_char}
    structs = {c: getattr(_lib, p) for c, p in STRUCTS.items()}
    for name, ctypes_ in _c_prototypes().items():
        res, args = _lib.SIGNATURES[name]
        assert res is ctypes.c_int, name
        assert len(args) == len(ctypes_), name
        for a, c in zip(args, ctypes_):
            c = c.replace("const ", "")
            if c.endswith("**"):
                ok = a is ctypes.c_void_p or a == ctypes.POINTER(ctypes.c_void_p)
            elif c.endswith("*"):
                base = c[:-1]
                allowed = {ctypes.c_void_p, ctypes.c_char_p}
                if base in scalars:
                    allowed.add(ctypes.POINTER(scalars[base]))
                if base in structs:
                    allowed.add(ctypes.POINTER(structs[base]))
                ok = a in allowed
            else:
                ok = a is scalars[c]
            assert ok, (name, a, c)


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "fvm_gpu.h"
/* A plain C11 caller: the header compiles as C and the library links with C linkage. */
int main(void) {
    int n = -1;
    char msg[256];
    fvm_mesh* mesh = NULL;
    fvm_system* sys = NULL;
    fvm_system_desc sd;
    memset(&sd, 0, sizeof sd);
    if (fvm_version() < 10000) return 10;
    if (fvm_device_count(&n) != FVM_OK || n < 0) return 11;
    if (fvm_mesh_create(NULL, 0, NULL, 0, NULL, NULL, 0, 0, 0, &mesh) != FVM_ERR_INVALID_ARGUMENT) return 12;
    if (fvm_last_error(msg, sizeof msg) != FVM_OK || msg[0] == 0) return 13;
    if (fvm_system_create(NULL, &sd, &sys) != FVM_ERR_INVALID_ARGUMENT || sys != NULL) return 14;
    if (fvm_system_rhs(NULL, NULL, NULL, 0.0, FVM_PTR_HOST, NULL) != FVM_ERR_INVALID_ARGUMENT) return 15;
    if (fvm_system_destroy(NULL) != FVM_OK) return 16;
    printf("ok %d\n", n);
    return 0;
}
"""


def test_plain_c_caller_compiles_links_and_gets_statuses(tmp_path):
    """A C11 program that includes only include/fvm_gpu.h links against libfvmgpu.so and gets
    status codes and messages back, without a GPU (argument checks come before device work)."""
    from fvmgpu import _build

    lib = _build.build()
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", f"-I{HEADER.parent}", str(src), str(lib),
                    f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), (r.returncode, r.stdout, r.stderr)
