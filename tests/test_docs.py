"""Every repository file and test the documents cite exists: a path in
backticks (``csrc/mhd_api.cu``, ``tests/test_driver.py::test_name``) must
resolve in the tree, and a cited test function must be defined there.
Reference sources and decks, run outputs and ``a_fp32/64`` shorthands are the
only names allowed not to resolve."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "mhd3d_mpi_fortran_gb300"
DOCS = ["README.md", "DESIGN.md", "INTEGRATION.md", "profiles/README.md"]
# files of the reference project and files a run writes
NOT_IN_TREE = {"mhd3d3.f90", "mhd3d2.f90", "mhd3d3.in", "mhd3d2.in", "process_mhd_2d.m", "frames.json"}
PAT = re.compile(r"`([A-Za-z0-9_./-]+\.(?:py|cu|cuh|h|cpp|md|json|f90|npz|in))(?:::(\w+))?`")


def _tree_files():
    return [p for p in ROOT.rglob("*") if p.is_file() and not {".git", "_work", "gpurun_out"} & set(p.parts)]


def _resolve(path, files):
    for base in (ROOT, PKG, ROOT / "profiles", ROOT / "oracle", ROOT / "tests"):
        if (base / path).is_file():
            return base / path
    if "/" not in path:
        hits = [p for p in files if p.name == path]
        if hits:
            return hits[0]
    return None


@pytest.mark.parametrize("doc", DOCS)
def test_cited_files_and_tests_exist(doc):
    files = _tree_files()
    missing = []
    for m in PAT.finditer((ROOT / doc).read_text()):
        path, fn = m.group(1), m.group(2)
        if Path(path).name in NOT_IN_TREE or re.search(r"fp32/64", path):
            continue
        hit = _resolve(path, files)
        if hit is None:
            missing.append(path)
        elif fn and not re.search(rf"def {fn}\(", hit.read_text()):
            missing.append(f"{path}::{fn}")
    assert not missing, missing


@pytest.mark.parametrize("doc", DOCS)
def test_cited_kernels_and_entry_points_exist(doc):
    """Every `k_*` kernel, `mhd_*` entry point and `oracle_*` function the
    document names is defined in the sources."""
    exts = {".cu", ".cuh", ".h", ".py", ".cpp", ".f90"}
    roots = [PKG, ROOT / "include", ROOT / "oracle"]
    src = "".join(p.read_text(errors="ignore") for r in roots for p in r.rglob("*")
                  if p.is_file() and p.suffix in exts)
    names = set(re.findall(r"`((?:k|mhd|oracle)_\w+)", (ROOT / doc).read_text()))
    missing = sorted(n for n in names if not re.search(r"\b" + re.escape(n) + r"\b", src))
    assert not missing, missing


@pytest.mark.parametrize("doc", ["README.md", "INTEGRATION.md"])
def test_python_examples_match_the_api(doc):
    """Each ```python block compiles, and every call to a package function or
    class it names binds to that callable's signature."""
    import ast
    import inspect
    import mhd3d_mpi_fortran_gb300 as pkg
    from mhd3d_mpi_fortran_gb300 import abi, deck, ics, learned
    modules = {"learned": learned, "ics": ics, "deck": deck, "abi": abi}
    names = {"MHDSolver": pkg.MHDSolver, "ensemble_step": pkg.ensemble_step,
             "ensemble_autotune": pkg.ensemble_autotune, "Params": abi.Params}
    blocks = re.findall(r"```python\n(.*?)```", (ROOT / doc).read_text(), re.S)
    for src in blocks:
        tree = ast.parse(src)
        for node in ast.walk(tree):
            if not isinstance(node, ast.Call):
                continue
            f = node.func
            fn = None
            if isinstance(f, ast.Attribute) and isinstance(f.value, ast.Name) and f.value.id in modules:
                fn = getattr(modules[f.value.id], f.attr, None)
                assert fn is not None, f"{f.value.id}.{f.attr} does not exist"
            elif isinstance(f, ast.Name) and f.id in names:
                fn = names[f.id]
            if fn is None:
                continue
            sig = inspect.signature(fn)
            args = [object()] * len(node.args)
            kwargs = {k.arg: object() for k in node.keywords if k.arg}
            sig.bind(*args, **kwargs)  # raises TypeError on a mismatch


def test_c_example_compiles_against_the_header(tmp_path):
    """The ```c example of INTEGRATION.md, wrapped in a function that declares
    the host arrays it uses, compiles against include/mhd_gpu.h."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    block = re.search(r"```c\n(.*?)```", (ROOT / "INTEGRATION.md").read_text(), re.S).group(1)
    body = "\n".join(line for line in block.splitlines() if not line.startswith("#include"))
    arrays = ", ".join(f"double* {v}" for v in ("rho", "vx", "vy", "vz", "pr", "bi", "bj", "bk", "bx", "by", "bz",
                                                  "dx", "dy", "dz"))
    src = tmp_path / "example.c"
    src.write_text(f'#include <stdio.h>\n#include "mhd_gpu.h"\nvoid example({arrays}) {{\n{body}\n}}\n')
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
