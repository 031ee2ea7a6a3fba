"""The Rust binding written out in INTEGRATION.md (not compiled here: no Rust
toolchain) names only functions the header declares, with the same number of
parameters."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_params():
    decl = {}
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b((?:rbc|fs|sv|df)_[a-z0-9_]*)\s*\(([^)]*)\)\s*;", text):
            args = m.group(2).strip()
            decl[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return decl


def rust_externs():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    out = {}
    for block in re.findall(r"```rust\n(.*?)```", text, flags=re.S):
        for m in re.finditer(r"\bfn\s+((?:rbc|fs|sv|df)_[a-z0-9_]*)\s*\(([^)]*)\)\s*(?:->[^;]*)?;", block, flags=re.S):
            args = m.group(2).strip()
            out[m.group(1)] = 0 if not args else args.count(",") + 1
    return out


def test_rust_binding_matches_header():
    decl = header_params()
    rust = rust_externs()
    assert len(rust) >= 30
    missing = sorted(n for n in rust if n not in decl)
    assert not missing, f"INTEGRATION.md binds functions the header does not declare: {missing}"
    arity = sorted((n, rust[n], decl[n]) for n in rust if rust[n] != decl[n])
    assert not arity, f"parameter counts differ (name, rust, header): {arity}"
