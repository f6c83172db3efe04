"""Writes solver_api.json: the public methods of the reference's Solver
(src/warpmpm/core/solver.py, class Solver) with their parameter names, kinds and
default values. The file is parsed with `ast`; nothing is imported, so Warp is not
needed.

    python tests/golden/make_api.py <reference_root>
"""
import ast
import json
import sys
from pathlib import Path


def _default(node):
    try:
        return {"value": ast.literal_eval(node)}
    except ValueError:
        return {"source": ast.unparse(node)}


def _params(fn: ast.FunctionDef):
    a = fn.args
    out = []
    pos = a.posonlyargs + a.args
    defaults = [None] * (len(pos) - len(a.defaults)) + list(a.defaults)
    for arg, d in zip(pos, defaults):
        out.append({"name": arg.arg, "kind": "positional", **({} if d is None else {"default": _default(d)})})
    if a.vararg:
        out.append({"name": a.vararg.arg, "kind": "var_positional"})
    for arg, d in zip(a.kwonlyargs, a.kw_defaults):
        out.append({"name": arg.arg, "kind": "keyword_only", **({} if d is None else {"default": _default(d)})})
    if a.kwarg:
        out.append({"name": a.kwarg.arg, "kind": "var_keyword"})
    return out


def main(ref_root: str):
    src = Path(ref_root) / "src" / "warpmpm" / "core" / "solver.py"
    tree = ast.parse(src.read_text())
    cls = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == "Solver")
    methods = {}
    for n in cls.body:
        if isinstance(n, ast.FunctionDef) and not n.name.startswith("_"):
            is_prop = any(isinstance(d, ast.Name) and d.id == "property" for d in n.decorator_list)
            methods[n.name] = {"property": is_prop, "params": _params(n)[1:]}   # drop self
    fields = [n.target.id for n in cls.body if isinstance(n, ast.AnnAssign) and isinstance(n.target, ast.Name)]
    out = {"source": "src/warpmpm/core/solver.py", "fields": fields, "methods": methods}
    dest = Path(__file__).resolve().parent / "solver_api.json"
    dest.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"{dest}: {len(methods)} methods, {len(fields)} fields")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {Path(__file__).name} <reference checkout root>")
    main(sys.argv[1])
