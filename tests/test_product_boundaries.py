"""The oracle is test infrastructure: the package never imports it, and the two entry scripts
import it only where they may (bench.py's CPU baseline and reference legs, and the build and
smoke check of __graft_entry__).  Nothing committed imports the working-files folder."""
import ast
import glob
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _imports(path):
    """(module, enclosing top-level function or None) for every import in a file."""
    tree = ast.parse(open(path).read(), filename=path)
    out = []

    def visit(node, fn):
        for child in ast.iter_child_nodes(node):
            f = fn
            if isinstance(child, (ast.FunctionDef, ast.AsyncFunctionDef)) and fn is None:
                f = child.name
            if isinstance(child, ast.Import):
                out.extend((a.name, f) for a in child.names)
            elif isinstance(child, ast.ImportFrom):
                out.append((("." * child.level) + (child.module or ""), f))
            visit(child, f)

    visit(tree, None)
    return out


def _is(mod, top):
    return mod == top or mod.startswith(top + ".")


def test_package_never_imports_the_oracle():
    files = glob.glob(os.path.join(ROOT, "scatter_gb300", "**", "*.py"), recursive=True)
    assert files
    for path in files:
        for mod, _ in _imports(path):
            assert not _is(mod, "oracle") and not _is(mod, "tests") and "_work" not in mod, (path, mod)


def test_entry_scripts_import_the_oracle_only_where_allowed():
    allowed = {"bench.py": {"cpu_baseline_run", "run_reference"}, "__graft_entry__.py": {"build", "smoke"}}
    for name, fns in allowed.items():
        for mod, fn in _imports(os.path.join(ROOT, name)):
            if _is(mod, "oracle"):
                assert fn in fns, (name, mod, fn)
            assert "_work" not in mod, (name, mod)


def test_nothing_committed_imports_working_files():
    for path in glob.glob(os.path.join(ROOT, "**", "*.py"), recursive=True):
        rel = os.path.relpath(path, ROOT)
        if rel.startswith("_work") or rel.startswith("baseline"):
            continue
        for mod, _ in _imports(path):
            assert "_work" not in mod, (rel, mod)
