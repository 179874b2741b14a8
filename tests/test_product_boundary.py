"""The product path never reaches the oracle: the package's Python modules,
its CUDA/C++ sources and its build recipe import, include or link nothing
under oracle/, which only tests, smoke() and bench.py's CPU arms may load."""
import ast
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pilon_gb300")


def _files(exts):
    for d, _, names in os.walk(PKG):
        for n in names:
            if n.endswith(exts):
                yield os.path.join(d, n)


def test_package_modules_do_not_import_the_oracle():
    for path in _files((".py",)):
        tree = ast.parse(open(path).read(), path)
        for node in ast.walk(tree):
            if isinstance(node, ast.Import):
                mods = [a.name for a in node.names]
            elif isinstance(node, ast.ImportFrom):
                mods = [node.module or ""]
            else:
                continue
            for m in mods:
                assert not m.split(".")[0] == "oracle", f"{path}:{node.lineno} imports {m}"


def test_native_sources_and_build_do_not_use_the_oracle():
    for path in _files((".cu", ".cuh", ".cpp", ".h")):
        src = open(path).read()
        assert not re.search(r'#\s*include\s*[<"][^>"]*oracle', src), path
    build = open(os.path.join(PKG, "build.py")).read()
    assert "oracle" not in build and "pilon_oracle" not in build
