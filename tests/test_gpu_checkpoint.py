"""Device checkpoints and the gather block-size autotuner (GPU)."""
import numpy as np
import pytest

from tests._support import gpu_domain
from weldform_gb300 import configs, PRECISION_MIXED

pytestmark = pytest.mark.gpu


def _state(d):
    return {f: d.get_array(f) for f in ("x", "v", "Sigma", "pl_strain", "Density")} | {"t": d.Time}


def test_checkpoint_rewinds_bit_exactly():
    d = gpu_domain()
    case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    d.prepare(case.dt)
    d.step(7)
    d.checkpoint_save(3)
    d.step(13)  # crosses neighbour rebuilds
    a = _state(d)
    d.checkpoint_restore(3)
    assert d.geti("steps") == 7
    d.step(13)
    b = _state(d)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    d.checkpoint_free(3)


def test_autotune_keeps_state_and_results():
    """The autotuner restores the state it timed from, and the run it leaves
    behind is bit-identical to one launched with its choice set directly (the
    block size never changes results; the lane count sets the acceleration
    gather's summation order)."""
    res = []
    choice = None
    for tune in (True, False):
        d = gpu_domain()
        d.set("precision", PRECISION_MIXED)
        case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
        d.prepare(case.dt)
        d.step(3)
        if tune:
            before = _state(d)
            b = d.autotune(2)
            assert b in (64, 128, 256, 512)
            choice = (b, d.geti("gather_lanes"))
            assert choice[1] in (1, 2, 4)
            after = _state(d)
            for k in before:
                assert np.array_equal(before[k], after[k]), k
        else:
            d.set("gather_lanes", choice[1])
        d.step(20)
        res.append(_state(d))
    for k in res[0]:
        assert np.array_equal(res[0][k], res[1][k]), k
