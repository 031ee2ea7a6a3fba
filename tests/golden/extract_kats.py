"""Extract the reference's known-answer vectors into tests/golden/reference_kats.json.

rustpde (Rust) cannot be built in this environment, so its unit tests and
doctests are read as text: every expected-value array literal listed below is
parsed from the reference source at the cited file:line and stored verbatim.
The inputs of each test are rebuilt in tests/test_oracle_kats.py from the same
test code (cited there).  Run from the repository root:

    python tests/golden/extract_kats.py /path/to/rustpde
"""
from __future__ import annotations

import json
import os
import re
import sys

# (name, file relative to the reference root, 1-based line where the literal starts)
KATS = [
    ("hholtz_adi_1d", "src/solver/hholtz_adi.rs", 164),
    ("hholtz_adi_2d", "src/solver/hholtz_adi.rs", 197),
    ("poisson_1d", "src/solver/poisson.rs", 202),
    ("poisson_2d", "src/solver/poisson.rs", 228),
    ("poisson_2d_complex", "src/solver/poisson.rs", 263),
    ("tensor2d_a", "src/solver/fdma_tensor.rs", 332),
    ("tensor2d_c", "src/solver/fdma_tensor.rs", 340),
    ("cheb_diff_lane_twice", "funspace/src/chebyshev/ortho.rs", 100),
    ("cheb_diff_lane_zero", "funspace/src/chebyshev/ortho.rs", 104),
    ("cheb_forward_4", "funspace/src/chebyshev/ortho.rs", 220),
    ("cheb_backward_4", "funspace/src/chebyshev/ortho.rs", 270),
    ("cheb_differentiate_axis0", "funspace/src/chebyshev/ortho.rs", 637),
    ("cheb_differentiate_axis1", "funspace/src/chebyshev/ortho.rs", 653),
    ("cd_to_ortho_doc", "funspace/src/chebyshev/composite.rs", 134),
    ("cd_from_ortho_doc", "funspace/src/chebyshev/composite.rs", 195),
    ("cd_forward_5", "funspace/src/chebyshev/composite.rs", 361),
    ("cd_backward_5", "funspace/src/chebyshev/composite.rs", 408),
    ("cd_differentiate_5", "funspace/src/chebyshev/composite.rs", 521),
    ("cd_to_ortho_axis0", "funspace/src/chebyshev/composite.rs", 622),
    ("cd_to_ortho_axis1", "funspace/src/chebyshev/composite.rs", 638),
    ("cd_differentiate_axis0", "funspace/src/chebyshev/composite.rs", 660),
    ("cd_differentiate_axis1", "funspace/src/chebyshev/composite.rs", 678),
    ("stencil_parent_in", "funspace/src/chebyshev/composite_stencil.rs", 418),
    ("stencil_composite_out", "funspace/src/chebyshev/composite_stencil.rs", 420),
    ("stencil_composite_in", "funspace/src/chebyshev/composite_stencil.rs", 423),
    ("stencil_parent_out", "funspace/src/chebyshev/composite_stencil.rs", 425),
    ("stencil_bc_parent_in", "funspace/src/chebyshev/composite_stencil.rs", 446),
    ("stencil_bc_composite_out", "funspace/src/chebyshev/composite_stencil.rs", 448),
    ("stencil_bc_composite_in", "funspace/src/chebyshev/composite_stencil.rs", 451),
    ("stencil_bc_parent_out", "funspace/src/chebyshev/composite_stencil.rs", 453),
    ("fourier_forward_4", "funspace/src/fourier/r2c.rs", 140),
    ("fourier_backward_4", "funspace/src/fourier/r2c.rs", 191),
]

_START = re.compile(r"(ndarray::)?(array!|vec!)\[")
_NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")
_CPLX = re.compile(r"Complex::new\(\s*([^,()]+)\s*,\s*([^,()]+)\s*\)")


def _literal_at(lines, lineno):
    """Return the text of the first array!/vec! literal starting on lineno."""
    text = "\n".join(l.split("//", 1)[0] if not l.lstrip().startswith("///") else l.lstrip()[3:]
                     for l in lines[lineno - 1: lineno + 40])
    m = _START.search(text)
    if not m:
        raise ValueError(f"no array literal at line {lineno}")
    i = m.end() - 1
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "[":
            depth += 1
        elif text[j] == "]":
            depth -= 1
            if depth == 0:
                return text[i: j + 1]
    raise ValueError(f"unterminated literal at line {lineno}")


def _parse(lit: str):
    lit = _CPLX.sub(lambda m: f"[{m.group(1)}, {m.group(2)}]", lit)
    lit = re.sub(r"(\d)\.(?=[\s,\]])", r"\1.0", lit)  # Rust "2." -> "2.0"
    toks = re.findall(r"\[|\]|" + _NUM.pattern, lit)
    stack = [[]]
    for t in toks:
        if t == "[":
            stack.append([])
        elif t == "]":
            v = stack.pop()
            stack[-1].append(v)
        else:
            stack[-1].append(float(t))
    return stack[0][0]


def main(ref_root: str, out_path: str):
    result = {"_comment": "expected values parsed verbatim from the rustpde sources; see extract_kats.py"}
    for name, rel, line in KATS:
        with open(os.path.join(ref_root, rel)) as f:
            lines = f.read().split("\n")
        lit = _literal_at(lines, line)
        result[name] = {"source": f"{rel}:{line}", "values": _parse(lit)}
    with open(out_path, "w") as f:
        json.dump(result, f, indent=1)
    print(f"wrote {len(KATS)} vectors to {out_path}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/extract_kats.py /path/to/rustpde")
    root = sys.argv[1]
    here = os.path.dirname(os.path.abspath(__file__))
    main(root, os.path.join(here, "reference_kats.json"))
