"""The Python examples of the integration guide at the repository root compile
and name functions the package has."""
import ast
import importlib
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _blocks():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```python\n(.*?)```", text, flags=re.S)


def test_examples_compile_and_name_real_functions():
    blocks = _blocks()
    assert blocks
    for code in blocks:
        tree = ast.parse(code)
        for node in ast.walk(tree):
            if isinstance(node, ast.ImportFrom) and node.module and node.module.startswith("pilon_gb300"):
                mod = importlib.import_module(node.module)
                for a in node.names:
                    assert hasattr(mod, a.name) or importlib.util.find_spec(f"{node.module}.{a.name}"), \
                        f"{node.module}.{a.name}"
            if (isinstance(node, ast.Attribute) and isinstance(node.value, ast.Name)
                    and node.value.id in ("bam", "fasta", "synth", "_abi")):
                mod = importlib.import_module(f"pilon_gb300.{node.value.id}")
                assert hasattr(mod, node.attr), f"{node.value.id}.{node.attr}"
            if isinstance(node, ast.Attribute) and isinstance(node.value, ast.Name) and node.value.id == "e":
                from pilon_gb300.engine import Engine
                assert hasattr(Engine, node.attr), f"Engine.{node.attr}"


def test_guide_names_every_entry_point():
    """Every function include/pilon_gb300.h declares is named in the guide, and
    the guide names no pg_ function the header lacks."""
    header = open(os.path.join(ROOT, "include", "pilon_gb300.h")).read()
    header = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    declared = set(re.findall(r"^\s*(?:pg_status|void|const char\s*\*)\s*(pg_\w+)\s*\(", header, flags=re.M))
    guide = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    named = set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(|`(pg_[a-z0-9_]+)`", guide))
    named = {a or b for a, b in named}
    assert declared and not sorted(n for n in declared if n not in guide)
    types = set(re.findall(r"\b(pg_\w+)\s*[;{]|typedef\s+\w+\s+(pg_\w+)", open(os.path.join(
        ROOT, "include", "pilon_gb300.h")).read()))
    known = declared | {t for pair in types for t in pair if t} | {"pg_ctx", "pg_server"}
    assert not sorted(n for n in named if n.startswith("pg_") and n not in known and not n.startswith("pg_ERR"))
