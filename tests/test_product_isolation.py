"""The product never routes through the checker: the package's Python and
CUDA/C++ sources neither import, include nor load anything under oracle/,
and the build links only the library's own objects and the CUDA runtime."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ddc-svd_gb300")


def _sources(exts):
    for dp, _, fs in os.walk(PKG):
        if "__pycache__" in dp or "_lib" in os.path.basename(dp):
            continue
        for f in fs:
            if f.endswith(exts):
                yield os.path.join(dp, f)


def test_python_package_does_not_import_the_oracle():
    bad = []
    for p in _sources((".py",)):
        text = open(p).read()
        if re.search(r"^\s*(from\s+oracle\b|import\s+oracle\b)", text, re.M) or "ddcsvd_oracle" in text:
            bad.append(p)
    assert not bad, bad


def test_native_sources_do_not_include_or_load_the_oracle():
    bad = []
    for p in _sources((".cu", ".cuh", ".hpp", ".h", ".cpp", ".c")):
        text = open(p).read()
        if re.search(r'#\s*include\s*[<"][^>"]*oracle', text) or re.search(r"dlopen|ddcsvd_oracle|ddcsvd_ref|_ref/", text):
            bad.append(p)
    assert not bad, bad


def test_build_links_no_oracle_objects():
    from ddcsvd import build as b
    srcs = b.sources()
    assert srcs and all(os.path.abspath(s).startswith(os.path.join(PKG, "csrc")) for s in srcs), srcs
