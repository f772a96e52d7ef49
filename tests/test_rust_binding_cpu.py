"""The Rust binding (bindings/rust) against include/bacon_gb300.h, on CPU.

cargo is not installed here, so the crate cannot be compiled.  This test
parses its raw `extern "C"` block and `#[repr(C)]` structs and checks them
against the header: every header function is bound with the same parameter
and return types, and every struct has the header's fields, in order, with
the same types.  It also checks that the safe layer keeps the builder
spelling of bacon-sci's IVPSolver trait (src/ivp.rs:134-190), the README's
aliases and the gradient entry point.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bacon_gb300.h")
FFI = os.path.join(ROOT, "bindings", "rust", "src", "ffi.rs")
GPU = os.path.join(ROOT, "bindings", "rust", "src", "gpu.rs")

C_SCALARS = {"int": "i32", "int32_t": "i32", "int64_t": "i64", "double": "f64", "void": "void", "char": "i8",
             "unsigned long long": "u64", "uint32_t": "u32"}
R_SCALARS = {"c_int": "i32", "i32": "i32", "i64": "i64", "f64": "f64", "c_void": "void", "c_char": "i8",
             "u64": "u64", "u32": "u32"}


def _c_type(decl: str) -> str:
    """'const bacon_problem* problem' or 'int32_t' -> canonical type."""
    decl = decl.strip()
    stars = decl.count("*")
    words = decl.replace("*", " ").split()
    const = words[0] == "const"
    if const:
        words = words[1:]
    base = C_SCALARS.get(" ".join(words), C_SCALARS.get(words[0], words[0]))
    if stars == 0:
        return base
    t = ("*const " if const else "*mut ") + base
    for _ in range(stars - 1):
        t = "*mut " + t
    return t


def _r_type(t: str) -> str:
    t = " ".join(t.split())
    m = re.match(r"^(\*(?:const|mut) )(.*)$", t)
    if m:
        return m.group(1) + _r_type(m.group(2))
    return R_SCALARS.get(t, t)


def _header():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    funcs = {}
    for ret, name, args in re.findall(r"([A-Za-z_][\w\s\*]*?)\s*\b(bacon_\w+)\s*\(([^)]*)\)\s*;", text):
        ret_t = _c_type(ret.split("\n")[-1])
        params = []
        a = args.strip()
        if a and a != "void":
            for part in a.split(","):
                part = part.strip()
                toks = part.replace("*", " * ").split()
                params.append(_c_type(" ".join(toks[:-1])))
        funcs[name] = (params, ret_t)
    structs = {}
    for body, name in re.findall(r"typedef struct\s*\{(.*?)\}\s*(bacon_\w+)\s*;", text, flags=re.S):
        fields = []
        for line in body.split(";"):
            line = line.strip()
            if not line:
                continue
            head, *rest = line.split(",")
            toks = head.replace("*", " * ").split()
            ftype = " ".join(toks[:-1])
            fields.append((toks[-1], _c_type(ftype)))
            for extra in rest:
                fields.append((extra.strip(), _c_type(ftype)))
        structs[name] = fields
    return funcs, structs


def _rust():
    text = re.sub(r"//[^\n]*", "", open(FFI).read())
    block = text[text.index('extern "C" {'):]
    block = block[:block.index("\n}\n") + 3]
    funcs = {}
    for name, args, ret in re.findall(r"pub fn (\w+)\s*\(([^)]*)\)\s*(?:->\s*([^;]+))?;", block, flags=re.S):
        params = []
        for part in args.split(","):
            part = part.strip()
            if part:
                params.append(_r_type(part.split(":", 1)[1]))
        funcs[name] = (params, _r_type(ret) if ret else "void")
    structs = {}
    for name, body in re.findall(r"#\[repr\(C\)\][^{]*?pub struct (\w+)\s*\{(.*?)\}", text, flags=re.S):
        fields = []
        for line in body.split(","):
            line = line.strip()
            if line.startswith("pub "):
                fname, ftype = line[4:].split(":", 1)
                fields.append((fname.strip(), _r_type(ftype)))
        structs[name] = fields
    return funcs, structs


def test_every_header_function_bound_with_its_signature():
    hf, _ = _header()
    rf, _ = _rust()
    assert len(hf) >= 30
    assert set(hf) == set(rf), (sorted(set(hf) - set(rf)), sorted(set(rf) - set(hf)))
    for name, sig in hf.items():
        assert rf[name] == sig, (name, sig, rf[name])


def test_every_header_struct_mirrored_field_by_field():
    _, hs = _header()
    _, rs = _rust()
    assert len(hs) >= 8
    for name, fields in hs.items():
        assert name in rs, name
        assert rs[name] == fields, (name, fields, rs[name])


def test_safe_layer_keeps_the_builder_and_readme_spelling():
    src = open(GPU).read()
    for m in ["new", "new_dyn", "with_tolerance", "with_maximum_dt", "with_minimum_dt", "with_initial_time",
              "with_ending_time", "with_initial_conditions_slice", "with_derivative", "solve",
              # README.md:32-40
              "with_dt_min", "with_dt_max", "with_start", "with_end", "with_initial_conditions", "build", "solve_ivp",
              # gradients
              "solve_ivp_adjoint"]:
        assert re.search(rf"pub fn {m}\b", src), m
    # IVPError's variants in declaration order (src/ivp.rs:50-76), codes 1..12
    names = ["MissingParameters", "UserError", "ToleranceOOB", "TimeDeltaOOB", "TimeEndOOB", "TimeStartOOB",
             "FromPrimitiveFailure", "MinimumTimeDeltaExceeded", "MaximumIterationsExceeded", "SingularMatrix",
             "DynamicOnStatic", "StaticOnDynamic"]
    for code, nm in enumerate(names, start=1):
        assert re.search(rf"\b{code} => GpuError::{nm}\b", src), nm
