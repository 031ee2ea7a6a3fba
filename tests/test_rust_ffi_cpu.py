"""The Rust declaration of the C ABI (include/spectral_rbc_ffi.rs): it is the
generator's output for the current header, it declares every entry point the
header declares with the same number of parameters, and its #[repr(C)]
structs list the same fields, in the same order and of the same C types, as
the ctypes mirror the Python host uses (no GPU is used)."""
import ctypes
import importlib.util
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def load_generator():
    spec = importlib.util.spec_from_file_location("gen_rust_ffi", os.path.join(INC, "gen_rust_ffi.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def header():
    with open(os.path.join(INC, "spectral_rbc.h")) as f:
        return f.read()


def rust():
    with open(os.path.join(INC, "spectral_rbc_ffi.rs")) as f:
        return f.read()


def test_committed_file_is_generated_from_header():
    assert load_generator().generate(header()) == rust()


def test_every_entry_point_declared():
    g = load_generator()
    _, _, _, _, protos = g.parse(header())
    decl = dict(re.findall(r"pub fn (\w+)\((.*?)\)", rust()))
    assert len(protos) >= 120
    for ret, name, args in protos:
        assert name in decl, name
        n_c = len(g.parse_args(args))
        n_r = 0 if decl[name].strip() == "" else decl[name].count(":")
        assert n_c == n_r, (name, n_c, n_r)


def test_structs_match_the_ctypes_mirror():
    import rustpde_gb300 as R
    # (ctypes.c_size_t is ctypes.c_ulong, the same class as c_uint64 here: no struct field is a uint64_t)
    ctype_of = {ctypes.c_int: "c_int", ctypes.c_double: "c_double", ctypes.c_size_t: "usize",
                ctypes.c_longlong: "c_longlong"}
    body = rust()
    for name in ("RbcParams", "RbcServerConfig", "RbcRequestResult", "RbcServerStats"):
        m = re.search(r"pub struct %s \{(.*?)\}" % name, body, flags=re.S)
        assert m, name
        fields = re.findall(r"pub (\w+): (\w+),", m.group(1))
        mirror = [(f, ctype_of[t]) for f, t in getattr(R, name)._fields_]
        assert fields == mirror, (name, fields, mirror)
