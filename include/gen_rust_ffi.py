"""Generate the Rust declaration of the C ABI (spectral_rbc_ffi.rs) from
spectral_rbc.h: its constants, the #[repr(C)] structs, the opaque handle
types, the callback type and one `pub fn` per entry point.

    python include/gen_rust_ffi.py > include/spectral_rbc_ffi.rs

The output is what rustpde adds as `src/gpu/ffi.rs` to bind the library;
`tests/test_rust_ffi_cpu.py` checks that the committed file is this script's
output for the current header."""
import os
import re
import sys

HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "spectral_rbc.h")
BASE = {"int": "c_int", "double": "c_double", "size_t": "usize", "uint64_t": "u64", "int64_t": "i64",
        "long long": "c_longlong", "long": "c_long", "char": "c_char", "void": "c_void", "float": "f32",
        "unsigned int": "c_uint", "unsigned": "c_uint"}
RUST_KEYWORDS = {"type", "fn", "ref", "in", "loop", "move", "match", "mod", "impl", "use", "where"}


def rust_type(t):
    t = " ".join(t.split())
    const = t.startswith("const ")
    if const:
        t = t[6:]
    stars = t.count("*")
    t = t.replace("*", "").strip()
    if t == "rbc_callback":  # nullable function pointer
        return "Option<RbcCallback>"
    base = BASE.get(t, t)
    if stars == 0:
        return base
    out = ("*const " if const else "*mut ") + base
    for _ in range(stars - 1):
        out = "*mut " + out
    return out


def parse_args(a):
    a = " ".join(a.split())
    if a in ("", "void"):
        return []
    res = []
    for part in a.split(","):
        m = re.match(r"(.*?)(\w+)\s*(\[\s*\d*\s*\])?$", part.strip())
        ty, name, arr = m.group(1), m.group(2), m.group(3)
        if arr:  # an array parameter is a pointer
            ty += "*"
        if name in RUST_KEYWORDS:
            name += "_"
        res.append((name, rust_type(ty)))
    return res


def parse(raw):
    """(constants, opaque types, structs, callback, prototypes) of the header."""
    consts = []
    for name, val in re.findall(r"^#define\s+([A-Z][A-Z_0-9]+)\s+(\(4u \* 1024u \* 1024u\)|\(?-?\d+\)?)", raw,
                                flags=re.M):
        v = val.strip("()")
        ty = "usize" if "u" in v else "c_int"
        consts.append((name, ty, v.replace("u", "").replace(" ", "")))
    src = re.sub(r"/\*.*?\*/", " ", raw, flags=re.S)
    src = re.sub(r"//[^\n]*", " ", src)
    src = re.sub(r"#[^\n]*", " ", src)
    opaque = re.findall(r"typedef\s+struct\s+(\w+)\s+\1\s*;", src)
    structs = re.findall(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*\1\s*;", src, flags=re.S)
    cb = re.search(r"typedef\s+int\s*\(\*\s*(\w+)\s*\)\s*\((.*?)\)\s*;", src, flags=re.S)
    body = re.sub(r"typedef\s+struct\s+(\w+)\s*\{.*?\}\s*\1\s*;", " ", src, flags=re.S)
    body = re.sub(r"typedef[^;]*;", " ", body)
    body = re.sub(r'extern\s+"C"\s*\{', " ", body)
    protos, seen = [], set()
    for ret, name, args in re.findall(r"([A-Za-z_][\w\s\*]*?)\b((?:rbc|fs|sv|df)_\w+)\s*\(([^)]*)\)\s*;", body):
        if name not in seen:
            seen.add(name)
            protos.append((" ".join(ret.split()), name, args))
    return consts, opaque, structs, cb, protos


def generate(raw):
    consts, opaque, structs, cb, protos = parse(raw)
    out = ["// Rust declaration of the C ABI of libspectral_rbc (generated from spectral_rbc.h by",
           "// gen_rust_ffi.py; regenerate, do not edit).  rustpde adds it as src/gpu/ffi.rs.",
           "#![allow(non_camel_case_types, dead_code)]",
           "use std::os::raw::{c_char, c_double, c_int, c_long, c_longlong, c_uint, c_void};", ""]
    out += [f"pub const {n}: {t} = {v};" for n, t, v in consts]
    out.append("")
    out += [f"#[repr(C)] pub struct {o} {{ _p: [u8; 0] }}" for o in opaque]
    for name, fields in structs:
        out += ["#[repr(C)]", "#[derive(Default, Clone, Copy, Debug)]", f"pub struct {name} {{"]
        for line in fields.split(";"):
            line = " ".join(line.split())
            if not line:
                continue
            m = re.match(r"((?:const\s+)?(?:unsigned\s+|long\s+)*\w+)\s+(.*)$", line)
            out += [f"    pub {n.strip()}: {rust_type(m.group(1))}," for n in m.group(2).split(",")]
        out.append("}")
    if cb:
        args = ", ".join(f"{n}: {t}" for n, t in parse_args(cb.group(2)))
        out.append(f'pub type RbcCallback = unsafe extern "C" fn({args}) -> c_int;')
    out += ["", '#[link(name = "spectral_rbc")]', 'extern "C" {']
    for ret, name, args in protos:
        r = rust_type(ret)
        a = ", ".join(f"{n}: {t}" for n, t in parse_args(args))
        out.append(f"    pub fn {name}({a})" + ("" if r == "c_void" else f" -> {r}") + ";")
    out.append("}")
    return "\n".join(out) + "\n"


if __name__ == "__main__":
    sys.stdout.write(generate(open(HEADER).read()))
