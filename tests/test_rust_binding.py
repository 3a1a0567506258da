"""The Rust `-sys` binding (gammaray_gb300/rust/gammaray-sys/src/lib.rs) against the C
header, read as text.  No Rust toolchain exists on the machines this repository is built
and tested on, so the crate is not compiled; instead every declaration is compared with
include/gammaray.h:
  - the same entry points, each with the same argument types in order and the same
    return type;
  - every C struct as a `#[repr(C)]` struct with the same field names, order and types;
  - every #define'd constant with the same value.
"""
from __future__ import annotations

import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gammaray.h")
SYS = os.path.join(ROOT, "gammaray_gb300", "rust", "gammaray-sys", "src", "lib.rs")

SCALARS = {"uint32_t": "u32", "int32_t": "i32", "uint64_t": "u64", "uint8_t": "u8", "float": "f32",
           "double": "f64", "int": "c_int", "char": "c_char", "void": "c_void", "gr_status": "gr_status"}


def _strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def c_to_rust(ctype: str) -> str:
    """A C declaration type (after the name is removed) as the binding's Rust type."""
    t = ctype.strip()
    const = t.startswith("const ")
    if const:
        t = t[len("const "):].strip()
    stars = t.count("*")
    base = t.replace("*", "").strip()
    rust = SCALARS.get(base, base)
    if stars == 0:
        return rust
    out = ("*const " if const else "*mut ") + rust
    for _ in range(stars - 1):
        out = "*mut " + out
    return out


def header_functions():
    src = _strip_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"^(const char\*|gr_status|void|int)\s+(gr_\w+)\s*\(([^)]*)\)\s*;", src, re.M):
        ret, name, args = m.group(1), m.group(2), m.group(3).strip()
        types = []
        if args and args != "void":
            for a in args.split(","):
                a = " ".join(a.split())
                nm = re.match(r"(.*?)([\w]+)$", a)
                types.append(c_to_rust(nm.group(1)))
        out[name] = ("" if ret == "void" else c_to_rust(ret), types)
    return out


def header_structs():
    src = _strip_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"typedef struct (gr_\w+)\s*\{(.*?)\}\s*\1\s*;", src, re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            fm = re.match(r"(.*?)(\w+)(\[(\d+)\])?$", decl)
            ty = c_to_rust(fm.group(1))
            if fm.group(4):
                ty = f"[{ty}; {fm.group(4)}]"
            fields.append((fm.group(2), ty))
        out[m.group(1)] = fields
    return out


def header_defines():
    src = open(HEADER).read()
    return {m.group(1): int(m.group(2), 0)
            for m in re.finditer(r"^#define (GR_\w+) (0x[0-9A-Fa-f]+|\d+)u?\s*$", src, re.M)}


def rust_source():
    return _strip_comments(open(SYS).read())


def rust_functions():
    src = rust_source()
    block = src[src.index('extern "C" {'):]
    out = {}
    for m in re.finditer(r"pub fn (gr_\w+)\((.*?)\)\s*(->\s*([^;]+))?;", block, re.S):
        args = " ".join(m.group(2).split())
        types = [a.split(":", 1)[1].strip() for a in args.split(",") if a.strip()]
        out[m.group(1)] = ((m.group(4) or "").strip(), types)
    return out


def rust_structs():
    src = rust_source()
    out = {}
    for m in re.finditer(r"#\[repr\(C\)\]\s*(?:#\[derive\([^)]*\)\]\s*)?pub struct (gr_\w+)\s*\{(.*?)\}", src, re.S):
        fields = []
        for decl in m.group(2).split(","):
            decl = " ".join(decl.split())
            if not decl or decl.startswith("_private"):
                continue
            name, ty = decl[len("pub "):].split(":", 1)
            fields.append((name.strip(), ty.strip()))
        out[m.group(1)] = fields
    return out


def test_every_entry_point_is_bound_with_its_signature():
    h, r = header_functions(), rust_functions()
    assert len(h) > 40
    assert set(h) == set(r), (sorted(set(h) - set(r)), sorted(set(r) - set(h)))
    for name, (ret, args) in h.items():
        assert r[name] == (ret, args), (name, (ret, args), r[name])


def test_every_struct_has_the_same_fields_in_order():
    h, r = header_structs(), rust_structs()
    assert len(h) == 17
    assert set(h) <= set(r), sorted(set(h) - set(r))
    for name, fields in h.items():
        assert r[name] == fields, (name, fields, r[name])


def test_constants_have_the_header_values():
    src = rust_source()
    consts = {m.group(1): int(m.group(2).replace("_", ""), 0)
              for m in re.finditer(r"pub const (GR_\w+): \w+ = (0x[0-9A-Fa-f_]+|\d+);", src)}
    for name, value in header_defines().items():
        assert consts.get(name) == value, (name, value, consts.get(name))
    enums = _strip_comments(open(HEADER).read())
    for m in re.finditer(r"(GR_[A-Z_]+) = (\d+)", enums):
        assert consts.get(m.group(1)) == int(m.group(2)), m.group(1)
