"""The drop-in boundary, checked without a GPU: every public method and constructor
field of the reference's Solver (src/warpmpm/core/solver.py, recorded in
golden/solver_api.json by golden/make_api.py) exists on mpm_engine_gb300.Solver.
Each method must have the same parameter names in the same order, the same kinds,
and equal default values, so a caller's positional and keyword arguments mean
the same thing."""
import dataclasses
import inspect
import json
from pathlib import Path

import pytest

from mpm_engine_gb300 import Solver

API = json.loads((Path(__file__).resolve().parent / "golden" / "solver_api.json").read_text())
KIND = {"positional": (inspect.Parameter.POSITIONAL_OR_KEYWORD, inspect.Parameter.POSITIONAL_ONLY),
        "keyword_only": (inspect.Parameter.KEYWORD_ONLY,),
        "var_positional": (inspect.Parameter.VAR_POSITIONAL,),
        "var_keyword": (inspect.Parameter.VAR_KEYWORD,)}


def _same(a, b):
    if isinstance(a, (list, tuple)) and isinstance(b, (list, tuple)):
        return len(a) == len(b) and all(_same(x, y) for x, y in zip(a, b))
    return a == b


def test_constructor_fields_match():
    names = [f.name for f in dataclasses.fields(Solver) if not f.name.startswith("_")]
    ref = [f for f in API["fields"] if not f.startswith("_")]
    assert names[:len(ref)] == ref


@pytest.mark.parametrize("name", sorted(API["methods"]))
def test_method_signature_matches_reference(name):
    ref = API["methods"][name]
    assert hasattr(Solver, name), f"Solver.{name} is missing"
    attr = inspect.getattr_static(Solver, name)
    if ref["property"]:
        assert isinstance(attr, property), f"Solver.{name} should be a property"
        return
    params = list(inspect.signature(getattr(Solver, name)).parameters.values())[1:]   # drop self
    assert [p.name for p in params] == [p["name"] for p in ref["params"]], name
    for p, r in zip(params, ref["params"]):
        assert p.kind in KIND[r["kind"]], (name, p.name, p.kind)
        if "default" not in r:
            assert p.default is inspect.Parameter.empty, (name, p.name, "has a default the reference lacks")
            continue
        assert p.default is not inspect.Parameter.empty, (name, p.name, "lacks the reference's default")
        d = r["default"]
        if "value" in d:
            assert _same(p.default, d["value"]), (name, p.name, p.default, d["value"])
