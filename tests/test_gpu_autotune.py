"""The autotuner runs end to end on the GPU: it times the planner's tiling and the
candidate tiles of a shape and writes a table that Ensemble applies."""
import json

import pytest

pytestmark = pytest.mark.gpu


def test_tune_writes_a_usable_table(gpu_lib, tmp_path):
    from cgenie_gb300 import autotune
    path = tmp_path / "tuning.json"
    table = autotune.tune(shapes=((18, 18, 16),), members=4, steps=3, path=str(path), verbose=False)
    stored = json.loads(path.read_text())
    assert stored == table
    for key, v in stored.items():
        # (0, 0): the planner's own tile was kept (no candidate beat it by more than the noise)
        assert key == "18x18x16" and v[2] > 0 and ((v[0], v[1]) == (0, 0) or 64 <= v[0] * v[1] <= 128)
