"""The C-ABI library loads without a GPU and exports every function that
include/sff.h and include/sffg.h declare (no compute calls here)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECL = re.compile(r"^\s*(?:const\s+)?(?:[A-Z_]+_T|int|long long|size_t|char|void|double|PARMSTRUCT_T)\s*\**\s*"
                  r"(\w+)\s*\(", re.M)


def declared(header):
    with open(os.path.join(ROOT, "include", header)) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)  # comments
    names = set(DECL.findall(text))
    names.discard("if")
    return names


@pytest.mark.parametrize("header", ["sff.h", "sffg.h"])
def test_every_declared_function_is_exported(lib, header):
    names = declared(header)
    assert len(names) >= (14 if header == "sff.h" else 25)
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_symbols_present(lib):
    """The entry points the reference's drivers call (src/sff/sff.h)."""
    for n in ("mm_options", "mme_init_sff", "mme", "md", "conjgrad", "mme_timer", "rdparm", "wrparm", "free_prm",
              "getxv", "putxv", "rand2", "gauss2", "setseed", "nabout", "mme_rattle", "xmin", "xminC",
              "xmin_opt_init"):
        assert hasattr(lib, n), n


def test_library_is_in_tree(lib):
    from nabc_gb300 import _build
    path = os.path.realpath(_build.library_path())
    assert path.startswith(os.path.realpath(os.path.join(ROOT, "nabc_gb300")))
    assert os.path.exists(path)
