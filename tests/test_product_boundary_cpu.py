"""The product (the rustpde_gb300 package and its CUDA library) never imports,
links or runs the oracle: the oracle is test infrastructure only."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "rustpde_gb300")


def product_sources():
    for d, _, files in os.walk(PKG):
        if "__pycache__" in d or os.sep + "_lib" in d:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                yield os.path.join(d, f)


def test_product_never_touches_the_oracle():
    hits = []
    for path in product_sources():
        text = open(path, encoding="utf-8").read()
        if re.search(r"\boracle\b|rbc_oracle|or_navier", text):
            hits.append(os.path.relpath(path, ROOT))
    assert not hits, f"product sources that name the oracle: {hits}"


def test_build_links_no_oracle_object():
    from rustpde_gb300 import build
    srcs = " ".join(getattr(build, "SOURCES", []))
    assert "oracle" not in srcs
