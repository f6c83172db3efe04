"""The autotuner's cache and bucket keys, without a GPU."""
import json

from mpm_engine_gb300 import autotune


class _Grid:
    def __init__(self, n):
        self.n_grid = n


class _Model:
    def __init__(self, mask):
        self.material_mask = mask


class _Scene:
    def __init__(self, n, ng, mask):
        self.n_particles, self.grid, self._model = n, _Grid(ng), _Model(mask)


def test_keys_bucket_workloads():
    a = [_Scene(10_000, 48, 1 << 1), _Scene(50_000, 128, 1 << 0)]
    b = [_Scene(10_500, 48, 1 << 1), _Scene(50_500, 128, 1 << 0)]
    c = [_Scene(10_000, 48, 1 << 10), _Scene(50_000, 128, 1 << 10)]
    assert autotune.batch_key(a, 100) == autotune.batch_key(b, 100)       # same half-octave, grids, laws
    assert autotune.batch_key(a, 100) != autotune.batch_key(c, 100)       # solids against fluids
    assert autotune.batch_key(a, 100) != autotune.batch_key(a, 20)        # substeps per tick
    assert "solids" in autotune.solver_key(a[0], 10) and "fluids" in autotune.solver_key(c[0], 10)


def test_cache_round_trip(tmp_path, monkeypatch):
    monkeypatch.setenv("GBMPM_AUTOTUNE_CACHE", str(tmp_path / "sub" / "tune.json"))
    monkeypatch.setattr(autotune, "_memory", {})
    autotune._store("k1", {"tuning": [1, 64, 2, 2], "ms_per_tick": {"1,64,2,2": 1.5}})
    monkeypatch.setattr(autotune, "_memory", {})
    assert autotune._lookup("k1")["tuning"] == [1, 64, 2, 2]
    data = json.loads((tmp_path / "sub" / "tune.json").read_text())
    assert list(data) == ["k1"]
    assert autotune._lookup("missing") is None
