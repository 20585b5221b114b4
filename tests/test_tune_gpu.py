"""The tile-shape autotuner: it measures candidates on the device, keeps the
fastest per table class, persists them as JSON, and never changes results."""
import os

import numpy as np
import pytest

from fuzzyblue_gb300.params import PRECISION_MIXED, Parameters, dump_parameters, smoke_parameters

pytestmark = pytest.mark.gpu


def _build(builder, p):
    from fuzzyblue_gb300.api import Atmosphere
    pend = Atmosphere.build(builder, p)
    pend.wait()
    out = pend.atmosphere().to_host()
    pend.release()
    return out


def test_autotune_keeps_results_and_persists(tmp_path):
    from fuzzyblue_gb300.api import Builder
    classes = [dump_parameters(), smoke_parameters(precision=PRECISION_MIXED)]
    with Builder(0) as b:
        before = [_build(b, p) for p in classes]
        assert b.tuned_shape(classes[0]) is None
        b.autotune(classes, batch=2)
        shapes = [b.tuned_shape(p) for p in classes]
        for s in shapes:
            assert s is not None and s["density_ms"] > 0 and s["multiple_ms"] > 0
            # density: occupancy 0-2, + 3 for exact-size interval tables
            assert s["density_variant"] in range(6) and s["multiple_variant"] in (0, 1)
        after = [_build(b, p) for p in classes]
        for x, y in zip(before, after):
            for k in x:
                assert np.array_equal(x[k], y[k]), k
        path = os.path.join(str(tmp_path), "tuning.json")
        b.save_tuning(path)
    with Builder(0) as b2:
        b2.load_tuning(path)
        assert b2.tuned_shape(classes[0]) == shapes[0]
        assert b2.tuned_shape(classes[1]) == shapes[1]
